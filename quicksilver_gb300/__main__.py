"""``python -m quicksilver_gb300 [-i] DECK [-n 1e5 | --nParticles 1e5 ...] [--exponential-tally]``

Runs a Quicksilver input deck with every cycle on the GPU, the way the
reference's driver does (main.cc:38-85): the deck echoed with every default
filled in (printParameters, Parameters.cc:97-215), nSteps cycles of cycleInit /
cycleTracking / cycleFinalize, one summary line per cycle with the balance
counters, the scalar-flux total and the three phase times (the columns of
Tallies::PrintSummary, Tallies.cc:122-144, Tallies.hh:60-76), then the
figure of merit (segments per second of tracking) after the cumulative
timer table (MC_Fast_Timer.cc:58-104) -- with cycleTimers 1 (``-c 1``) also
the last-cycle table after every summary line (MC_Fast_Timer.cc:106-152) --,
the census energy
spectrum file when the deck names one (EnergySpectrum.cc:38-59) and the
CORAL2 checks when the deck sets coralBenchmark (CoralBenchmark.cc:17-44).
The command line takes the reference's flags (Parameters.cc:230-255: short
``-n 1e5`` or long ``--nParticles 1e5`` / ``--nParticles=1e5``, ``-i DECK`` or
the deck as the first argument, no deck for the default problem) with its
precedence (Parameters.cc:80-95): a Simulation key the deck sets wins over
the flag, except energySpectrum and crossSectionsOut.  ``--exponential-tally``
runs as the reference built with -DEXPONENTIAL_TALLY (CycleTracking.cc:48-50)
and adds each cycle's exponential cell-tally total to its line.
"""
from __future__ import annotations

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


# The reference's flags in its order (Parameters.cc:230-255): long name,
# short letter, takes a value, value type, help text.  help (-h) and
# loadBalance (-l) take no value.
ARGUMENTS = [
    ("help", "h", 0, "i", "print this message"),
    ("dt", "D", 1, "d", "time step (seconds)"),
    ("fMax", "f", 1, "d", "max random mesh node displacement"),
    ("inputFile", "i", 1, "s", "name of input file"),
    ("energySpectrum", "e", 1, "s", "name of energy spectrum output file"),
    ("crossSectionsOut", "S", 1, "s", "name of cross section output file"),
    ("loadBalance", "l", 0, "i", "enable/disable load balancing"),
    ("cycleTimers", "c", 1, "i", "enable/disable cycle timers"),
    ("debugThreads", "t", 1, "i", "set thread debug level to 1, 2, 3"),
    ("lx", "X", 1, "d", "x-size of simulation (cm)"),
    ("ly", "Y", 1, "d", "y-size of simulation (cm)"),
    ("lz", "Z", 1, "d", "z-size of simulation (cm)"),
    ("nParticles", "n", 1, "u", "number of particles"),
    ("batchSize", "g", 1, "u", "number of particles in a vault/batch"),
    ("nBatches", "b", 1, "u", "number of vault/batch to start (sets batchSize automaticaly)"),
    ("nSteps", "N", 1, "i", "number of time steps"),
    ("nx", "x", 1, "i", "number of mesh elements in x"),
    ("ny", "y", 1, "i", "number of mesh elements in y"),
    ("nz", "z", 1, "i", "number of mesh elements in z"),
    ("seed", "s", 1, "i", "random number seed"),
    ("xDom", "I", 1, "i", "number of MPI ranks in x"),
    ("yDom", "J", 1, "i", "number of MPI ranks in y"),
    ("zDom", "K", 1, "i", "number of MPI ranks in z"),
    ("bTally", "B", 1, "i", "number of balance tally replications"),
    ("fTally", "F", 1, "i", "number of scalar flux tally replications"),
    ("cTally", "C", 1, "i", "number of scalar cell tally replications"),
]
SHORT_FLAGS = {short: name for name, short, _, _, _ in ARGUMENTS if name != "help"}
COMMAND_LINE_WINS = ("energySpectrum", "crossSectionsOut")   # Parameters.cc:88-90


def help_text() -> str:
    """The reference's argument list as its -h prints it (printArgs,
    cmdLineParser.cc:123-142: long names padded to the longest), then this
    driver's own flag."""
    width = max(len(name) for name, *_ in ARGUMENTS)
    lines = ["", "  Arguments are: "]
    lines += [f"   --{name:<{width}} -{short}  arg={arg} type={kind}  {text}" for name, short, arg, kind, text in ARGUMENTS]
    lines += ["", "", "  --exponential-tally: run as the reference built with -DEXPONENTIAL_TALLY "
              "(one extra random number per segment, exp of it tallied per cell)", ""]
    return "\n".join(lines)


def parse_command_line(argv) -> tuple:
    """(deck path or None, {Simulation key: value} from the flags, exponential tally?)."""
    path, values, exp_tally = None, {}, False
    args = list(argv)
    k = 0
    while k < len(args):
        a = args[k]
        k += 1
        if a == "--exponential-tally":
            exp_tally = True
            continue
        if a.startswith("--"):
            name, eq, val = a[2:].partition("=")
        elif a.startswith("-") and len(a) == 2 and a[1] in SHORT_FLAGS:
            name, eq, val = SHORT_FLAGS[a[1]], "", ""
        elif path is None and not a.startswith("-"):
            path = a   # the deck as a positional argument
            continue
        else:
            raise SystemExit(f"unexpected argument {a!r}")
        if name == "loadBalance" and not eq:
            val = "1"
        elif not eq:
            if k >= len(args):
                raise SystemExit(f"flag {a!r} needs a value")
            val = args[k]
            k += 1
        if name == "inputFile":
            path = val
        else:
            values[name] = val
    return path, values, exp_tally


def deck_simulation_keys(text: str) -> set:
    """Keys the deck's Simulation block sets (they win over the flags)."""
    keys, block = set(), None
    for line in text.splitlines():
        stripped = line.split("//")[0].split("#")[0].rstrip()
        if not stripped:
            continue
        if not line[0].isspace():
            block = stripped.rstrip(":").strip()
        elif block == "Simulation" and ":" in stripped:
            keys.add(stripped.split(":", 1)[0].strip())
    return keys


def deck_from_command_line(argv) -> tuple:
    """getParameters (Parameters.cc:80-95): flags first, then the deck's own
    Simulation keys over them (but not over energySpectrum and
    crossSectionsOut), then the defaults.  Returns (Deck, exponential tally?)."""
    path, values, exp_tally = parse_command_line(argv)
    if path is None:
        deck, deck_keys = Deck.from_string(""), set()
    else:
        deck = Deck.from_file(path)
        with open(path) as fh:
            deck_keys = deck_simulation_keys(fh.read())
    for key, val in values.items():
        if key in COMMAND_LINE_WINS or key not in deck_keys:
            deck.set(key, val)
    return deck, exp_tally


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if "-h" in argv or "--help" in argv:   # the reference prints its list and stops (Parameters.cc:263-271)
        sys.stdout.write(help_text())
        return 2
    deck, exponential_tally = deck_from_command_line(argv)
    sim = deck.simulation
    cycle_timers = int(deck._echo_values("Simulation", "cycleTimers")[0])
    mc = MonteCarlo(deck)
    t_main = time.perf_counter()   # MC_Fast_Timer::main starts once the problem is set up (main.cc:51)
    spectrum_stem = deck.energy_spectrum
    mc.observe(fluence=bool(sim.coral_benchmark), spectrum=bool(spectrum_stem))
    if exponential_tally:
        mc.exponential_tally(True)
    out = sys.stdout
    out.write(deck.text() + "\n")
    # initMC's progress lines for the one domain tracked here (initMC.cc:295-319);
    # the mesh self-test they bracket ran in qsg_create (initMC.cc:202-234)
    out.write("Building partition 0\ndone building\nBuilding MC_Domain 0\n"
              "Starting Consistency Check\nFinished Consistency Check\nFinished initMesh\n")
    if deck.cross_sections_out:   # written by initMC in the reference (initMC.cc:392-490)
        write_cross_sections(deck.cross_sections_out, mc.problem, deck.material_names)
    out.write(summary_header() + (" %14s" % "cell_tally" if exponential_tally else "") + "\n")
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
        cell_total = mc.cell_tally().sum() if exponential_tally else None   # finalize resets it
        mc.cycle_finalize()
        row = mc.history(cycle, 1)
        t3 = time.perf_counter()
        track_s += t2 - t1
        # the reference stops its finalize timer for the summary line and
        # starts it again after (Tallies.cc:125, 143): two calls a cycle,
        # the second one empty here
        last = {"cycleInit": (1, t1 - t0), "cycleTracking": (1, t2 - t1), "cycleTracking_Kernel": (1, t2 - t1),
                "cycleFinalize": (2, t3 - t2)}
        for name, (calls, dt) in last.items():
            clock[name][0] += calls
            clock[name][1] += dt
        bal = row.balance[0]
        out.write(summary_line(cycle, bal, row.flux_total[0], (t1 - t0, t2 - t1, t3 - t2)) +
                  (" %14e" % cell_total if cell_total is not None else "") + "\n")
        if cycle_timers == 1:   # Last_Cycle_Report: cumulative calls, this cycle's time (main.cc:61-65)
            timer_table(out, "Last Cycle", {name: (clock[name][0], dt) for name, (_, dt) in last.items()})
    flags = mc.device_status()
    if flags:
        raise N.QsgError(N.QSG_ERR_DEVICE, f"device flags 0x{flags:x} raised during the run")
    hist = mc.history(0, sim.n_steps)
    cum = cumulative_balance(hist.balance)
    clock["main"] = [1, time.perf_counter() - t_main]
    timer_report(out, clock, cum["num_segments"])
    if spectrum_stem:
        # written silently, as the reference's PrintSpectrum does (EnergySpectrum.cc:38-59)
        write_energy_spectrum(spectrum_stem, mc.problem.array("energies"), mc.energy_spectrum()[0])
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


# MC_Fast_Timer's timers (MC_Fast_Timer.hh:31-41, MC_Fast_Timer.cc:8-17).
# cycleTracking_Kernel counts one call per cycle (the reference: one per
# particle vault processed); cycleTracking_MPI and cycleTracking_Test_Done
# stay at zero, as one GPU exchanges no particles (the reference times its
# vault bookkeeping under cycleTracking_MPI even on one rank, main.cc:243-292)
TIMERS = ["main", "cycleInit", "cycleTracking", "cycleTracking_Kernel", "cycleTracking_MPI",
          "cycleTracking_Test_Done", "cycleFinalize"]


def timer_table(out, kind: str, clock: dict) -> None:
    """Print_Cumulative_Heading / Print_Last_Cycle_Heading and the timer
    lines (MC_Fast_Timer.cc:31-56, 81-95, 133-146) for one rank:
    {name: (calls, seconds)}, whole microseconds, min = avg = max, no spread."""
    out.write("\n%-25s %12s %12s %12s %12s %12s %12s\n" % (("Timer",) + (kind,) * 6))
    out.write("%-25s %12s %12s %12s %12s %12s %12s\n" % ("Name", "number", "microSecs", "microSecs", "microSecs",
                                                        "microSecs", "Efficiency"))
    out.write("%-25s %12s %12s %12s %12s %12s %12s\n" % ("", "of calls", "min", "avg", "max", "stddev", "Rating"))
    for name in TIMERS:
        calls, secs = clock.get(name, (0, 0.0))
        us = float(int(secs * 1e6))   # the reference keeps whole microseconds
        out.write("%-25s %12d %12.3e %12.3e %12.3e %12.3e %12.2f\n" %
                  (name, calls, us, us, us, 0.0, 100.0 * us / (us + 1.0e-80)))


def timer_report(out, clock: dict, num_segments: int) -> None:
    """MC_Fast_Timer_Container::Cumulative_Report (MC_Fast_Timer.cc:58-104)
    for one rank: the timer table and the figure of merit, segments per
    second of cycleTracking."""
    timer_table(out, "Cumulative", clock)
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
