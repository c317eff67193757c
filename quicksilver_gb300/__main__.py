"""``python -m quicksilver_gb300 DECK [--nSteps N] [--key value ...]``

Runs a Quicksilver input deck with every cycle on the GPU, the way the
reference's driver does (main.cc:38-85): the deck echoed with every default
filled in (printParameters, Parameters.cc:97-215), nSteps cycles of cycleInit /
cycleTracking / cycleFinalize, one summary line per cycle with the balance
counters, the scalar-flux total and the three phase times (the columns of
Tallies::PrintSummary, Tallies.cc:122-144, Tallies.hh:60-76), then the
figure of merit (segments per second of tracking), the census energy
spectrum file when the deck names one (EnergySpectrum.cc:38-59) and the
CORAL2 checks when the deck sets coralBenchmark (CoralBenchmark.cc:17-44).
Simulation keys may be overridden on the command line (``--nParticles 1e5``),
as the reference's flags do (Parameters.cc:230-255).  ``--exponential-tally``
runs as the reference built with -DEXPONENTIAL_TALLY (CycleTracking.cc:48-50)
and adds each cycle's exponential cell-tally total to its line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import sys
import time

from . import _native as N
from .monte_carlo import MonteCarlo
from .observe import coral_benchmark_correctness, cumulative_balance, write_cross_sections, write_energy_spectrum
from .problem import Deck

COLUMNS = ["start", "source", "rr", "split", "absorb", "scatter", "fission", "produce", "collision", "escape",
           "census", "num_segments"]
HEADER = ["start", "source", "rr", "split", "absorb", "scatter", "fission", "produce", "collisn", "escape",
          "census", "num_seg"]


def main(argv=None) -> int:
    t_main = time.perf_counter()   # MC_Fast_Timer::main covers the whole run
    ap = argparse.ArgumentParser(prog="python -m quicksilver_gb300", description=__doc__.split("\n\n")[1])
    ap.add_argument("deck")
    ap.add_argument("--exponential-tally", action="store_true",
                    help="behave as the reference built with -DEXPONENTIAL_TALLY")
    args, extra = ap.parse_known_args(argv)
    deck = Deck.from_file(args.deck)
    it = iter(extra)
    for flag in it:
        if not flag.startswith("--"):
            ap.error(f"unexpected argument {flag!r}")
        deck.set(flag[2:], next(it))
    sim = deck.simulation
    mc = MonteCarlo(deck)
    spectrum_stem = deck.energy_spectrum
    mc.observe(fluence=bool(sim.coral_benchmark), spectrum=bool(spectrum_stem))
    if args.exponential_tally:
        mc.exponential_tally(True)
    out = sys.stdout
    out.write(deck.text() + "\n")
    if deck.cross_sections_out:   # written by initMC in the reference (initMC.cc:392-490)
        write_cross_sections(deck.cross_sections_out, mc.problem, deck.material_names)
    out.write(summary_header() + (" %14s" % "cell_tally" if args.exponential_tally else "") + "\n")
    track_s = 0.0
    clock = {name: [0, 0.0] for name in TIMERS}   # calls, seconds
    for cycle in range(sim.n_steps):
        t0 = time.perf_counter()
        mc.cycle_init()
        h = mc.tracker
        mc_sync(h)
        t1 = time.perf_counter()
        mc.cycle_tracking()
        mc_sync(h)
        t2 = time.perf_counter()
        cell_total = mc.cell_tally().sum() if args.exponential_tally else None   # finalize resets it
        mc.cycle_finalize()
        row = mc.history(cycle, 1)
        t3 = time.perf_counter()
        track_s += t2 - t1
        for name, dt in (("cycleInit", t1 - t0), ("cycleTracking", t2 - t1), ("cycleTracking_Kernel", t2 - t1),
                         ("cycleFinalize", t3 - t2)):
            clock[name][0] += 1
            clock[name][1] += dt
        bal = row.balance[0]
        out.write(summary_line(cycle, bal, row.flux_total[0], (t1 - t0, t2 - t1, t3 - t2)) +
                  (" %14e" % cell_total if cell_total is not None else "") + "\n")
    flags = mc.device_status()
    if flags:
        raise N.QsgError(N.QSG_ERR_DEVICE, f"device flags 0x{flags:x} raised during the run")
    hist = mc.history(0, sim.n_steps)
    cum = cumulative_balance(hist.balance)
    clock["main"] = [1, time.perf_counter() - t_main]
    timer_report(out, clock, cum["num_segments"])
    if spectrum_stem:
        path = write_energy_spectrum(spectrum_stem, mc.problem.array("energies"), mc.energy_spectrum()[0])
        out.write(f"energy spectrum written to {path}\n")
    if sim.coral_benchmark:
        coral_benchmark_correctness(cum, mc.fluence(), sim.coral_benchmark, out)
    mc.close()
    return 0


def summary_header() -> str:
    """Tallies::PrintSummary's header (Tallies.cc:126-131, Balance::PrintHeader, Tallies.hh:60-67)."""
    return ("%-8s " % "cycle" + " ".join("%12s" % h for h in HEADER) +
            "%14s %14s %14s %14s" % ("scalar_flux", "cycleInit", "cycleTracking", "cycleFinalize"))


def summary_line(cycle: int, balance, flux_total: float, times) -> str:
    """Tallies::PrintSummary's line for one cycle (Tallies.cc:133-140,
    Balance::Print, Tallies.hh:69-76): counters, scalar-flux sum, and the
    cycleInit / cycleTracking / cycleFinalize seconds."""
    return ("%8d " % cycle + " ".join("%12d" % int(balance[N.BAL[c]]) for c in COLUMNS) +
            "%14e %14e %14e %14e" % (flux_total, times[0], times[1], times[2]))


# MC_Fast_Timer's timers (MC_Fast_Timer.hh:31-41, MC_Fast_Timer.cc:8-17); one
# process and one domain: no particle exchange, so the MPI and test-for-done
# timers are never started
TIMERS = ["main", "cycleInit", "cycleTracking", "cycleTracking_Kernel", "cycleTracking_MPI",
          "cycleTracking_Test_Done", "cycleFinalize"]


def timer_report(out, clock: dict, num_segments: int) -> None:
    """MC_Fast_Timer_Container::Cumulative_Report (MC_Fast_Timer.cc:45-104)
    for one rank: microseconds per timer (min = avg = max, no spread) and the
    figure of merit, segments per second of cycleTracking."""
    out.write("\n%-25s %12s %12s %12s %12s %12s %12s\n" % ("Timer", "Cumulative", "Cumulative", "Cumulative",
                                                          "Cumulative", "Cumulative", "Cumulative"))
    out.write("%-25s %12s %12s %12s %12s %12s %12s\n" % ("Name", "number", "microSecs", "microSecs", "microSecs",
                                                        "microSecs", "Efficiency"))
    out.write("%-25s %12s %12s %12s %12s %12s %12s\n" % ("", "of calls", "min", "avg", "max", "stddev", "Rating"))
    for name in TIMERS:
        calls, secs = clock.get(name, [0, 0.0])
        us = float(int(secs * 1e6))   # the reference keeps whole microseconds
        out.write("%-25s %12d %12.3e %12.3e %12.3e %12.3e %12.2f\n" %
                  (name, calls, us, us, us, 0.0, 100.0 * us / (us + 1.0e-80)))
    track_us = float(int(clock["cycleTracking"][1] * 1e6))
    out.write("%-25s %12.3e %-25s\n" % ("Figure Of Merit", num_segments / (track_us * 1e-6),
                                         "[Num Segments / Cycle Tracking Time]"))


def mc_sync(tracker) -> None:
    """Wait for the work enqueued so far (phase timing): qsg_sizes reads the
    stores' device counters, which waits for the device."""
    a, b = C.c_uint64(), C.c_uint64()
    N.check(N.lib().qsg_sizes(tracker.handle, C.byref(a), C.byref(b)))


if __name__ == "__main__":
    sys.exit(main())
