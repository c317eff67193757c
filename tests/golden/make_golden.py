"""Generate golden fixtures from the UNMODIFIED reference (test infrastructure).

Needs the reference sources ($QS_REF_SRC, default: a checkout beside the repository, ../reference/src) and builds
``oracle/_ref/qs_ref_harness`` with ``make -C oracle ref``.  For every deck in
quicksilver_gb300/decks it runs the reference harness and stores in
``tests/golden/<deck>.npz``:

* ``balance``        [cycles, 13] uint64, Tallies.cc:400-414 order
* ``flux``           [cycles, cells, groups] float64 (small decks only)
* ``flux_cell``      [cycles, cells]  per-cell sums, gid order (not for config2;
  config2 and config4 are stored for their first three cycles)
* ``flux_group``     [cycles, groups] per-group sums
* ``flux_proj``      [cycles, 4] projections on fixed pseudo-random weights
* ``init_sha``/``census_sha``  sha256 of the sorted 136-byte particle records
  after cycleInit and after cycleTracking, plus their counts
* ``init_head``      first 32 sorted records after cycle 0's cycleInit
* ``table_sha``      sha256 of every problem table in global-cell order
* ``rng_*``          known-answer vectors of rngSample / rngSpawn
* ``track_seconds``  reference cycleTracking wall time per cycle (8 threads here)

With ``--exponential-tally`` it builds the reference with -DEXPONENTIAL_TALLY
(``make -C oracle ref_exp``: one extra random number per segment, its exp
tallied per cell, CycleTracking.cc:48-50) and stores ``exp_<deck>.npz``:
``balance``, ``flux_cell``, ``flux_total``, ``census_sha`` / ``census_n`` and
``cell_tally`` [cycles, cells] (gid order) for t_homog and t_fission by default.

With ``--echo`` it stores the reference's start-up echo of every deck in
quicksilver_gb300/decks (printParameters, Parameters.cc:97-215) in
``deck_echo.npz`` (one string per deck stem).

With ``--xsec`` it stores the file the reference's initMC writes for
``-S <stem>`` (crossSectionsOut, initMC.cc:392-490) for a few decks in
``xsec_out.npz``.

With ``--spectrum`` it stores the census energy spectrum file the reference
prints for ``-e <stem>`` (EnergySpectrum.cc:38-59) after all cycles of a few
decks in ``spectrum_out.npz``.

With ``--coral`` it stores what the reference's coralBenchmarkCorrectness
prints (CoralBenchmark.cc:17-228) after the cycles of t_coral1 and of t_homog /
t_fission run with coralBenchmark 1 / 2 (failing checks included) in
``coral_out.npz``.

With ``--summary`` it stores the reference's per-cycle summary lines
(Tallies::PrintSummary, Tallies.cc:122-144: header and one line per cycle,
as printed to stdout) for a few decks in ``summary_out.npz``.

With ``--timers`` it stores what the reference prints from its first
summary line on for t_homog run with ``-c 1`` (cycleTimers): per cycle the
summary line and the last-cycle timer table (MC_Fast_Timer.cc:106-152), then
the cumulative table and the figure of merit (MC_Fast_Timer.cc:58-104), in
``timers_out.npz``.

With ``--transcript`` it stores, for t_coral1 run with ``-e spectrum``, what
the reference prints after its deck echo (initMC's progress lines, summary
lines, cumulative timer table, figure of merit, CORAL2 checks) and the
spectrum file it writes, and what it prints for ``-h`` (printArgs,
cmdLineParser.cc:123-142), in ``transcript_out.npz``.

With ``--portable-math`` it runs the reference linked with the portable
elementary functions (``make -C oracle ref_pm``, QS_PORTABLE_MATH=1: its
tracking path's log / sin / cos are those of
quicksilver_gb300/csrc/portable_math.h, initMC keeps libm) and stores, per
deck, ``pm_<deck>.npz``: the counters, the flux (whole when small, otherwise
per cell / per group / projections / total) and the sha256 of the sorted
particle sets after each cycleInit and cycleTracking.

With ``--config3`` it stores ``config3_pNN.npz`` for five problems of the config3
ensemble (one per mesh edge), two cycles each.

With ``--config5`` it stores ``config5_r0.npz``: the first replica of the config5
ensemble (its 64^3 slab geometry, 3e6 particles, 2 cycles).

Usage: python tests/golden/make_golden.py [--exponential-tally | --portable-math | --echo | --xsec |
                                           --spectrum | --coral | --summary | --timers | --transcript |
                                           --config3 | --config5]
"""
from __future__ import annotations

import hashlib
import os
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
DECKS = ROOT / "quicksilver_gb300" / "decks"
HARNESS = ROOT / "oracle" / "_ref" / "qs_ref_harness"
HARNESS_EXP = ROOT / "oracle" / "_ref_exp" / "qs_ref_harness"
REF_SRC = os.environ.get("QS_REF_SRC", str(Path(__file__).resolve().parents[3] / "reference" / "src"))
FULL_FLUX_LIMIT = 20000   # store the whole flux array when cells*groups is at most this

PARTICLE_DTYPE = np.dtype([
    ("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("vx", "<f8"), ("vy", "<f8"), ("vz", "<f8"),
    ("kinetic_energy", "<f8"), ("weight", "<f8"), ("time_to_census", "<f8"), ("age", "<f8"),
    ("num_mean_free_paths", "<f8"), ("num_segments", "<f8"),
    ("random_number_seed", "<u8"), ("identifier", "<u8"),
    ("last_event", "<i4"), ("num_collisions", "<i4"), ("breed", "<i4"), ("species", "<i4"),
    ("domain", "<i4"), ("cell", "<i4"),
])

TABLES = ["energies", "iso_react_off", "reaction_type", "reaction_nubar", "reaction_xs", "mat_iso_off",
          "mat_iso_gid", "mat_iso_af", "mat_mass", "cell_volume", "cell_density", "cell_material",
          "cell_nodes", "cell_planes", "facet_point_coords", "facet_event", "facet_adj_facet", "facet_adj_gid",
          "time_step"]


def read_dump(path: Path) -> dict:
    out = {}
    data = path.read_bytes()
    off = 0
    while off < len(data):
        (nlen,) = struct.unpack_from("<I", data, off)
        off += 4
        name = data[off:off + nlen].decode()
        off += nlen
        dtype = chr(data[off])
        off += 1
        (count,) = struct.unpack_from("<Q", data, off)
        off += 8
        np_dtype = {"d": "<f8", "q": "<u8", "i": "<i4"}[dtype]
        nbytes = count * np.dtype(np_dtype).itemsize
        out[name] = np.frombuffer(data, dtype=np_dtype, count=count, offset=off).copy()
        off += nbytes
    return out


def particles(d: dict, name: str) -> np.ndarray:
    f = d[name + "_f64"].reshape(-1, 12)
    q = d[name + "_u64"].reshape(-1, 2)
    i = d[name + "_i32"].reshape(-1, 6)
    recs = np.empty(len(f), dtype=PARTICLE_DTYPE)
    for k, n in enumerate(PARTICLE_DTYPE.names[:12]):
        recs[n] = f[:, k]
    recs["random_number_seed"] = q[:, 0]
    recs["identifier"] = q[:, 1]
    for k, n in enumerate(PARTICLE_DTYPE.names[14:]):
        recs[n] = i[:, k]
    return recs


def sort_records(recs: np.ndarray) -> np.ndarray:
    return recs[np.lexsort((recs["random_number_seed"], recs["identifier"]))]


def sha(arr: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()


def projection_weights(cells: int, groups: int) -> np.ndarray:
    return np.random.default_rng(20240601).uniform(0.5, 1.5, size=(4, cells * groups))


def ensure_harness(target: str = "ref") -> None:
    res = subprocess.run(["make", "-C", str(ROOT / "oracle"), target, f"REF_SRC={REF_SRC}", "-j8"],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise SystemExit(f"reference build failed:\n{res.stderr[-4000:]}")


def run_deck(deck: Path, workdir: Path, harness: Path = HARNESS) -> dict:
    dump = workdir / (deck.stem + ".dump")
    env = dict(os.environ, QS_DUMP=str(dump), QS_DUMP_TABLES="1", QS_DUMP_PARTICLES="1", OMP_NUM_THREADS="8")
    res = subprocess.run([str(harness), "-i", str(deck)], env=env, capture_output=True, text=True)
    if res.returncode != 0:
        raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
    return read_dump(dump)


STOCK_CYCLES = {"config2": 3, "config4": 3}   # the benchmark decks: their first three cycles
LARGE_FLUX = 1_000_000          # above this many (cell, group) entries, no per-cell sums either


def make(deck: Path, workdir: Path) -> None:
    if deck.stem in STOCK_CYCLES:
        import re
        text = deck.read_text()
        deck = workdir / deck.name
        deck.write_text(re.sub(r"nSteps: \d+", f"nSteps: {STOCK_CYCLES[deck.stem]}", text))
    d = run_deck(deck, workdir)
    cycles = sum(1 for k in d if k.startswith("balance_c"))
    G = len(d["energies"]) - 1
    C = len(d["cell_volume"])
    out = {"balance": np.stack([d[f"balance_c{c}"] for c in range(cycles)])}
    flux = np.stack([d[f"flux_c{c}"] for c in range(cycles)])
    if C * G <= FULL_FLUX_LIMIT:
        out["flux"] = flux.reshape(cycles, C, G)
    if C * G <= LARGE_FLUX:
        out["flux_cell"] = flux.reshape(cycles, C, G).sum(axis=2)
    out["flux_group"] = flux.reshape(cycles, C, G).sum(axis=1)
    out["flux_proj"] = flux @ projection_weights(C, G).T
    out["flux_total"] = flux.sum(axis=1)
    init_sha, census_sha, init_n, census_n = [], [], [], []
    for c in range(cycles):
        ini = sort_records(particles(d, f"init_c{c}"))
        cen = sort_records(particles(d, f"census_c{c}"))
        init_sha.append(sha(ini))
        census_sha.append(sha(cen))
        init_n.append(len(ini))
        census_n.append(len(cen))
        if c == 0:
            out["init_head"] = ini[:32]
            out["census_head"] = cen[:32]
    out["init_sha"] = np.array(init_sha)
    out["census_sha"] = np.array(census_sha)
    out["init_n"] = np.array(init_n, dtype=np.int64)
    out["census_n"] = np.array(census_n, dtype=np.int64)
    out["table_names"] = np.array(TABLES)
    out["table_sha"] = np.array([sha(d[t]) for t in TABLES])
    out["mat_names"] = np.array(bytes(d["mat_names"].astype(np.uint8)).decode().split("\n")[:-1])
    for k in ("rng_seeds", "rng_samples", "rng_states", "rng_spawned", "rng_parent_after", "track_seconds"):
        out[k] = d[k]
    np.savez_compressed(HERE / (deck.stem + ".npz"), **out)
    print(f"{deck.name}: cycles={cycles} cells={C} groups={G} segments={int(out['balance'][:, 12].sum())}")


HARNESS_PM = ROOT / "oracle" / "_ref" / "qs_ref_harness_pm"
PM_DECKS = ["t_homog", "t_escape", "t_scatter_octant", "t_fission", "t_nonflat", "config1", "config2"]
PM_FULL_FLUX_LIMIT = 20000    # above this, the whole flux of the first cycle only


PM_CYCLES = {"config2": 2}   # the benchmark deck: its first two cycles


def make_pm(deck: Path, workdir: Path) -> None:
    dump = workdir / (deck.stem + ".pm.dump")
    if deck.stem in PM_CYCLES:
        text = deck.read_text()
        import re
        deck = workdir / deck.name
        deck.write_text(re.sub(r"nSteps: \d+", f"nSteps: {PM_CYCLES[deck.stem]}", text))
    env = dict(os.environ, QS_DUMP=str(dump), QS_DUMP_PARTICLES="1", QS_DUMP_TABLES="1", QS_PORTABLE_MATH="1",
               OMP_NUM_THREADS="8")
    res = subprocess.run([str(HARNESS_PM), "-i", str(deck)], env=env, capture_output=True, text=True)
    if res.returncode != 0:
        raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
    d = read_dump(dump)
    cycles = sum(1 for k in d if k.startswith("balance_c"))
    G = len(d["energies"]) - 1
    C = len(d["cell_volume"])
    flux = np.stack([d[f"flux_c{c}"] for c in range(cycles)])
    out = {"balance": np.stack([d[f"balance_c{c}"] for c in range(cycles)])}
    if C * G <= PM_FULL_FLUX_LIMIT:
        out["flux"] = flux.reshape(cycles, C, G)
    elif C * G <= 16 * PM_FULL_FLUX_LIMIT:
        out["flux"] = flux[:1].reshape(1, C, G)
    out["flux_cell"] = flux.reshape(cycles, C, G).sum(axis=2)
    out["flux_group"] = flux.reshape(cycles, C, G).sum(axis=1)
    out["flux_total"] = flux.sum(axis=1)
    out["init_sha"] = np.array([sha(sort_records(particles(d, f"init_c{c}"))) for c in range(cycles)])
    out["census_sha"] = np.array([sha(sort_records(particles(d, f"census_c{c}"))) for c in range(cycles)])
    out["census_n"] = np.array([len(particles(d, f"census_c{c}")) for c in range(cycles)], dtype=np.int64)
    np.savez_compressed(HERE / f"pm_{deck.stem}.npz", **out)
    print(f"pm_{deck.name}: cycles={cycles} segments={int(out['balance'][:, 12].sum())}")


def make_exp(deck: Path, workdir: Path) -> None:
    d = run_deck(deck, workdir, HARNESS_EXP)
    cycles = sum(1 for k in d if k.startswith("balance_c"))
    G = len(d["energies"]) - 1
    C = len(d["cell_volume"])
    flux = np.stack([d[f"flux_c{c}"] for c in range(cycles)]).reshape(cycles, C, G)
    out = {"balance": np.stack([d[f"balance_c{c}"] for c in range(cycles)]),
           "flux_cell": flux.sum(axis=2), "flux_total": flux.sum(axis=(1, 2)),
           "cell_tally": np.stack([d[f"cell_tally_c{c}"] for c in range(cycles)])}
    cens = [sort_records(particles(d, f"census_c{c}")) for c in range(cycles)]
    out["census_sha"] = np.array([sha(c) for c in cens])
    out["census_n"] = np.array([len(c) for c in cens], dtype=np.int64)
    np.savez_compressed(HERE / ("exp_" + deck.stem + ".npz"), **out)
    print(f"exp_{deck.name}: cycles={cycles} cells={C} segments={int(out['balance'][:, 12].sum())} "
          f"cell tally total {out['cell_tally'].sum():.6e}")


# command lines whose echo pins the flags' meaning and precedence (Parameters.cc:80-95, 230-255)
ECHO_COMMAND_LINES = {
    "cli_default": ["-n", "100", "-N", "1", "-x", "2", "-y", "2", "-z", "2", "-X", "2", "-Y", "2", "-Z", "2",
                    "-l", "-B", "2", "-C", "3"],
    "cli_deck_and_flags": ["-i", "quicksilver_gb300/decks/t_homog.inp", "-n", "123", "-g", "50", "-D", "2e-08",
                           "-e", "spec", "-S", "xs", "-s", "17"],
}


def make_echo(names: list[str], workdir: Path) -> None:
    out = {}
    for name, args in ECHO_COMMAND_LINES.items():
        echo = workdir / f"{name}.echo"
        env = dict(os.environ, QS_ECHO=str(echo), QS_ECHO_ONLY="1")
        res = subprocess.run([str(HARNESS)] + args, env=env, cwd=ROOT, capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"reference run failed on {args}:\n{res.stderr[-4000:]}")
        out[name] = np.array(echo.read_text())
        out[name + "_args"] = np.array(args)
    for name in names:
        deck = (DECKS / f"{name}.inp").relative_to(ROOT)   # the echo records the path it was given
        echo = workdir / f"{name}.echo"
        env = dict(os.environ, QS_ECHO=str(echo), QS_ECHO_ONLY="1")
        res = subprocess.run([str(HARNESS), "-i", str(deck)], env=env, cwd=ROOT, capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
        out[name] = np.array(echo.read_text())
    np.savez_compressed(HERE / "deck_echo.npz", **out)
    print(f"deck_echo.npz: {len(out)} decks")


def make_xsec(names: list[str], workdir: Path) -> None:
    out = {}
    for name in names:
        deck = DECKS / f"{name}.inp"
        env = dict(os.environ, QS_INIT_ONLY="1")
        res = subprocess.run([str(HARNESS), "-i", str(deck), "-S", "xsout"], env=env, cwd=workdir,
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
        out[name] = np.array((workdir / "xsout.dat").read_text())
    np.savez_compressed(HERE / "xsec_out.npz", **out)
    print(f"xsec_out.npz: {len(out)} decks")


def make_spectrum(names: list[str], workdir: Path) -> None:
    out = {}
    for name in names:
        deck = DECKS / f"{name}.inp"
        env = dict(os.environ, QS_PRINT_SPECTRUM="1", OMP_NUM_THREADS="8")
        res = subprocess.run([str(HARNESS), "-i", str(deck), "-e", "spec"], env=env, cwd=workdir,
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
        out[name] = np.array((workdir / "spec.dat").read_text())
    np.savez_compressed(HERE / "spectrum_out.npz", **out)
    print(f"spectrum_out.npz: {len(out)} decks")


CORAL_RUNS = {"t_coral1": None, "t_homog": 1, "t_fission": 2}   # deck -> coralBenchmark set here (None: the deck's)


def make_coral(workdir: Path) -> None:
    out = {}
    for name, level in CORAL_RUNS.items():
        text = (DECKS / f"{name}.inp").read_text()
        if level is not None:
            text = text.replace("Simulation:\n", f"Simulation:\n   coralBenchmark: {level}\n", 1)
        deck = workdir / f"{name}.inp"
        deck.write_text(text)
        env = dict(os.environ, QS_CORAL="1", OMP_NUM_THREADS="8")
        res = subprocess.run([str(HARNESS), "-i", str(deck)], env=env, cwd=workdir, capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
        k = res.stdout.index("\nTesting Ratios")
        out[name] = np.array(res.stdout[k:])
    np.savez_compressed(HERE / "coral_out.npz", **out)
    print(f"coral_out.npz: {len(out)} runs")


def make_summary(names: list[str], workdir: Path) -> None:
    out = {}
    for name in names:
        deck = DECKS / f"{name}.inp"
        env = dict(os.environ, OMP_NUM_THREADS="8")
        res = subprocess.run([str(HARNESS), "-i", str(deck)], env=env, cwd=workdir, capture_output=True, text=True)
        if res.returncode != 0:
            raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
        lines = res.stdout.splitlines()
        k = next(i for i, l in enumerate(lines) if l.startswith("cycle "))
        out[name] = np.array("\n".join(l for l in lines[k:] if l.startswith("cycle ") or l[:8].strip().isdigit()))
    np.savez_compressed(HERE / "summary_out.npz", **out)
    print(f"summary_out.npz: {len(out)} decks")


def make_timers(workdir: Path) -> None:
    deck = DECKS / "t_homog.inp"
    env = dict(os.environ, QS_TIMERS="1", OMP_NUM_THREADS="8")
    res = subprocess.run([str(HARNESS), "-i", str(deck), "-c", "1"], env=env, cwd=workdir, capture_output=True,
                         text=True)
    if res.returncode != 0:
        raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
    k = res.stdout.index("cycle ")
    np.savez_compressed(HERE / "timers_out.npz", t_homog=np.array(res.stdout[k:]))
    print("timers_out.npz: t_homog")


def make_transcript(workdir: Path) -> None:
    deck = DECKS / "t_coral1.inp"
    env = dict(os.environ, QS_TIMERS="1", QS_CORAL="1", QS_PRINT_SPECTRUM="1", OMP_NUM_THREADS="8")
    res = subprocess.run([str(HARNESS), "-i", str(deck), "-e", "spectrum"], env=env, cwd=workdir,
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise SystemExit(f"reference run failed on {deck}:\n{res.stderr[-4000:]}")
    k = res.stdout.index("Building partition 0")
    helped = subprocess.run([str(HARNESS), "-h"], cwd=workdir, capture_output=True, text=True)
    if helped.returncode != 2 or not helped.stdout.startswith("\n  Arguments are: "):
        raise SystemExit(f"unexpected -h behaviour: rc={helped.returncode}")
    np.savez_compressed(HERE / "transcript_out.npz", stdout=np.array(res.stdout[k:]),
                        spectrum=np.array((workdir / "spectrum.dat").read_text()), help=np.array(helped.stdout))
    print("transcript_out.npz: t_coral1")


def make_config5(workdir: Path) -> None:
    """config5's first replica (make_decks.config5, 3e6 particles -- the smallest
    count at which every cell sources -- and 2 cycles), the benchmark's slab
    geometry, as ``config5_r0.npz``."""
    sys.path.insert(0, str(ROOT))
    from quicksilver_gb300.decks.make_decks import config5
    import re
    text = re.sub(r"nSteps: \d+", "nSteps: 2", config5(n_particles=3_000_000)[0])
    deck = workdir / "config5_r0.inp"
    deck.write_text(text)
    make(deck, workdir)


CONFIG3_PROBLEMS = [4, 6, 15, 26, 33]   # one per mesh edge 48 / 32 / 24 / 8 / 16, 1-3 materials


def make_config3(workdir: Path) -> None:
    """A few problems of the config3 ensemble (make_decks.config3), one per mesh
    edge, two cycles each with the reference's own seeding, as
    ``config3_pNN.npz``."""
    sys.path.insert(0, str(ROOT))
    from quicksilver_gb300.decks.make_decks import config3
    import re
    decks = config3()
    for p in CONFIG3_PROBLEMS:
        deck = workdir / f"config3_p{p:02d}.inp"
        deck.write_text(re.sub(r"nSteps: \d+", "nSteps: 2", decks[p]))
        make(deck, workdir)


def main(argv: list[str]) -> None:
    import tempfile
    if "--config3" in argv:
        ensure_harness("ref")
        with tempfile.TemporaryDirectory() as tmp:
            make_config3(Path(tmp))
        return
    if "--config5" in argv:
        ensure_harness("ref")
        with tempfile.TemporaryDirectory() as tmp:
            make_config5(Path(tmp))
        return
    if "--transcript" in argv:
        ensure_harness("ref")
        with tempfile.TemporaryDirectory() as tmp:
            make_transcript(Path(tmp))
        return
    if "--timers" in argv:
        ensure_harness("ref")
        with tempfile.TemporaryDirectory() as tmp:
            make_timers(Path(tmp))
        return
    if "--summary" in argv:
        ensure_harness("ref")
        names = [a for a in argv if a != "--summary"] or ["t_homog", "t_fission", "config1"]
        with tempfile.TemporaryDirectory() as tmp:
            make_summary(names, Path(tmp))
        return
    if "--coral" in argv:
        ensure_harness("ref")
        with tempfile.TemporaryDirectory() as tmp:
            make_coral(Path(tmp))
        return
    if "--spectrum" in argv:
        ensure_harness("ref")
        names = [a for a in argv if a != "--spectrum"] or ["t_homog", "t_fission", "t_nonflat"]
        with tempfile.TemporaryDirectory() as tmp:
            make_spectrum(names, Path(tmp))
        return
    if "--xsec" in argv:
        ensure_harness("ref")
        names = [a for a in argv if a != "--xsec"] or ["t_homog", "t_nonflat", "t_fission", "config2", "config4"]
        with tempfile.TemporaryDirectory() as tmp:
            make_xsec(names, Path(tmp))
        return
    if "--echo" in argv:
        ensure_harness("ref")
        names = [a for a in argv if a != "--echo"] or sorted(p.stem for p in DECKS.glob("*.inp"))
        with tempfile.TemporaryDirectory() as tmp:
            make_echo(names, Path(tmp))
        return
    if "--portable-math" in argv:
        ensure_harness("ref_pm")
        names = [a for a in argv if a != "--portable-math"] or PM_DECKS
        import tempfile
        with tempfile.TemporaryDirectory() as td:
            for n in names:
                make_pm(DECKS / f"{n}.inp", Path(td))
        return
    exp = "--exponential-tally" in argv
    argv = [a for a in argv if a != "--exponential-tally"]
    ensure_harness("ref_exp" if exp else "ref")
    if exp:
        names = argv or ["t_homog", "t_fission"]
    else:
        names = argv or sorted(p.stem for p in DECKS.glob("*.inp") if p.stem.startswith("t_") or p.stem == "config1")
    with tempfile.TemporaryDirectory() as tmp:
        for name in names:
            (make_exp if exp else make)(DECKS / f"{name}.inp", Path(tmp))


if __name__ == "__main__":
    main(sys.argv[1:])
