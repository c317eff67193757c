// Test-infrastructure run of the reference's own main (main.cc:38-85) with
// the reference-side adapter in place, as a maintainer would change it:
// qsgAttach after initMC, qsgCycleTracking instead of cycleTracking; the
// reference's own cycleInit, cycleFinalize (whose Tallies::PrintSummary
// prints each cycle's counters and scalar-flux total), Last_Cycle_Report,
// gameOver (timer report, figure of merit, spectrum file) and CORAL2 checks.
// Built by oracle/Makefile (`make dropin_cycle`) from the UNMODIFIED
// reference's sources, the adapter (oracle/dropin_adapter.hh) and the CPU
// stand-in for libqsg's tracking calls (oracle/qsg_cpu_standin.c, answered
// by the C oracle), so it runs without a GPU; the tests compare its printout
// with the unmodified reference's.  Built with -DEXPONENTIAL_TALLY
// (`make dropin_cycle_exp`) it also prints, after each cycle's tracking, the
// cell tally the adapter handed to the reference's Tallies
// ("cell_tally_total <sum>", summed over domains, each in cell order).  Exit status 2 when
// qsgAttach fails.

#include <cstdio>

#include "initMC.hh"
#include "utilsMpi.hh"
#include "CoralBenchmark.hh"
#include "MC_Processor_Info.hh"
#include "dropin_adapter.hh"

void cycleInit(bool loadBalance);
void cycleFinalize();
void gameOver();

int main(int argc, char** argv)
{
    mpiInit(&argc, &argv);
    Parameters params = getParameters(argc, argv);
    mcco = initMC(params);
    qsgAttach(mcco);
    if (!g_qsg) return 2;
    MC_FASTTIMER_START(MC_Fast_Timer::main);
    for (int ii = 0; ii < params.simulationParams.nSteps; ++ii) {
        cycleInit(bool(params.simulationParams.loadBalance));
        qsgCycleTracking(mcco);
#ifdef EXPONENTIAL_TALLY
        double total = 0.0;
        for (int d = 0; d < mcco->_tallies->_cellTallyDomain.size(); ++d) {
            const CellTallyTask& t = mcco->_tallies->_cellTallyDomain[d]._task[0];
            for (int c = 0; c < t._cell.size(); ++c) total += t._cell[c];
        }
        printf("cell_tally_total %.17g\n", total);
#endif
        cycleFinalize();
        mcco->fast_timer->Last_Cycle_Report(params.simulationParams.cycleTimers, mcco->processor_info->rank,
                                            mcco->processor_info->num_processors,
                                            mcco->processor_info->comm_mc_world);
    }
    MC_FASTTIMER_STOP(MC_Fast_Timer::main);
    gameOver();
    coralBenchmarkCorrectness(mcco, params);
    qsg_destroy(g_qsg);
    return 0;
}
