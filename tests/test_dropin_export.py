"""The drop-in adapter a maintainer adds to the reference
(oracle/dropin_adapter.hh), compiled
with the unmodified reference's sources:

* the table export after initMC, linked against libqsg.so
  (oracle/dropin_harness.cc): for every bundled deck it passes
  qsg_problem_check (the reference's mesh self-test included), and every
  table it hands the library is, bit for bit, the table this library's own
  deck reader builds (node numbering aside: the reference shares nodes
  between cells, so cell corners are compared as coordinates) -- so what the
  GPU tests prove for deck-built problems holds for a problem exported from
  the reference's own MonteCarlo object;
* the reference's own main loop with the adapter in place
  (oracle/dropin_cycle.cc), the library's calls answered on the CPU by a
  stand-in built on the oracle (oracle/qsg_cpu_standin.c; the GPU tests
  show the library's tracking is the oracle's): its whole printout --
  per-cycle counters and flux totals, timer tables, figure of merit, CORAL2
  checks -- and spectrum file are the unmodified reference's; with the
  reference built with -DEXPONENTIAL_TALLY, that build's counters and cell
  tally; a four-domain MonteCarlo is refused with a message;
* the cycle adapter's vault and tally halves around the reference's own
  first cycleInit: the particles it gathers from the processing vaults are
  the oracle's, bit for bit; scattering them into the processed vaults and
  gathering them back is exact, no vault above its size; the counters and
  flux it hands over are what the reference's Tallies then hold.

Runs where the reference's sources and the harness built from them are
present, and skips elsewhere."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import DECKS
from quicksilver_gb300 import Deck

ROOT = Path(__file__).resolve().parent.parent
HARNESS = ROOT / "oracle" / "_ref" / "qs_dropin_harness"
CYCLE = ROOT / "oracle" / "_ref" / "qs_dropin_cycle"
CYCLE_EXP = ROOT / "oracle" / "_ref_exp" / "qs_dropin_cycle"
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import read_dump   # noqa: E402

pytestmark = pytest.mark.skipif(not HARNESS.exists(), reason="the reference's sources or the drop-in harness are absent")

NAMES = sorted(p.stem for p in DECKS.glob("*.inp") if p.stem != "config2")   # config2: 64k cells, slow initMC


@pytest.mark.parametrize("name", NAMES)
def test_export_equals_deck_reader(name, tmp_path):
    dump = tmp_path / "export.bin"
    res = subprocess.run([str(HARNESS), "-i", str(DECKS / f"{name}.inp")], env=dict(os.environ, QS_DUMP=str(dump)),
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    got = read_dump(dump)
    hp = Deck.from_file(DECKS / f"{name}.inp").build()
    for key, arr in got.items():
        if key in ("nodes", "cell_points"):
            continue
        want = np.array([hp.view.time_step]) if key == "time_step" else hp.array(key)
        assert arr.dtype.itemsize == want.dtype.itemsize and arr.shape == want.shape, key
        np.testing.assert_array_equal(arr.view(f"u{arr.dtype.itemsize}"), want.view(f"u{want.dtype.itemsize}"),
                                      err_msg=key)
    corners = got["nodes"].reshape(-1, 3)[got["cell_points"].reshape(-1, 14)]
    ours = hp.array("nodes").reshape(-1, 3)[hp.array("cell_points").reshape(-1, 14)]
    np.testing.assert_array_equal(corners.view(np.uint64), ours.view(np.uint64))


@pytest.mark.parametrize("name", ["t_homog", "t_fission", "t_nonflat", "config1"])
def test_cycle_adapter_vaults_and_tallies(name, tmp_path):
    from helpers import load_problem, oracle_run, sort_particles
    dump = tmp_path / "vaults.bin"
    res = subprocess.run([str(HARNESS), "-i", str(DECKS / f"{name}.inp")],
                         env=dict(os.environ, QS_DUMP=str(dump), QS_VAULTS="1"), capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout[-1000:] + res.stderr[-2000:]
    got = read_dump(dump)
    _, sim, hp = load_problem(f"{name}.inp")
    run = oracle_run(hp, sim)
    run.cycle_init()
    want = run.processing()
    assert len(got["p_x"]) == len(want) > int(got["vault_size"][0])   # several vaults filled
    rec = np.zeros(len(want), want.dtype)
    for field in want.dtype.names:
        rec[field] = got["p_" + field]
    a, b = sort_particles(rec), sort_particles(want)
    for field in want.dtype.names:
        size = a[field].dtype.itemsize
        np.testing.assert_array_equal(a[field].view(f"u{size}"), b[field].view(f"u{size}"), err_msg=field)


GOLDEN = ROOT / "tests" / "golden"


@pytest.mark.skipif(not CYCLE.exists(), reason="the adapter's main-loop harness is absent")
def test_reference_main_loop_through_adapter(tmp_path):
    gold = np.load(GOLDEN / "transcript_out.npz")
    res = subprocess.run([str(CYCLE), "-i", str(DECKS / "t_coral1.inp"), "-e", "spectrum"], cwd=tmp_path,
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    got = res.stdout[res.stdout.index("Building partition 0"):].split("\n")
    want = str(gold["stdout"]).split("\n")
    assert len(got) == len(want)
    timers = False
    for g, w in zip(got, want):
        gf, wf = g.split(), w.split()
        assert gf[:1] == wf[:1] and len(g) == len(w), (g, w)
        if g.startswith("Timer"):
            timers = True
        elif g.startswith("Figure Of Merit"):
            timers = False
        elif not timers and g[:8].strip().isdigit():
            assert gf[:14] == wf[:14], (g, w)           # counters and scalar-flux total
        elif timers and gf and gf[0] in ("main", "cycleInit", "cycleTracking", "cycleFinalize"):
            assert gf[1] == wf[1], (g, w)                # call counts
        elif not timers and not g.startswith(("cycle ", "Figure Of Merit")):
            assert g == w                                # CORAL2 check text
    assert (tmp_path / "spectrum.dat").read_text() == str(gold["spectrum"])


@pytest.mark.skipif(not CYCLE.exists(), reason="the adapter's main-loop harness is absent")
@pytest.mark.parametrize("name", ["t_homog", "t_fission", "config1"])
def test_reference_summary_through_adapter(name, tmp_path):
    want = str(np.load(GOLDEN / "summary_out.npz")[name]).split("\n")
    res = subprocess.run([str(CYCLE), "-i", str(DECKS / f"{name}.inp")], cwd=tmp_path, capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = res.stdout.split("\n")
    k = next(i for i, line in enumerate(lines) if line.startswith("cycle "))
    got = [line for line in lines[k:] if line.startswith("cycle ") or line[:8].strip().isdigit()]
    assert got[0] == want[0] and len(got) == len(want)
    for g, w in zip(got[1:], want[1:]):
        assert g.split()[:14] == w.split()[:14], (g, w)


@pytest.mark.skipif(not CYCLE.exists(), reason="the adapter's main-loop harness is absent")
def test_adapter_refuses_more_than_one_domain(tmp_path):
    """The reference's one-rank default (xDom = yDom = zDom = 0) builds four
    domains; the adapter hands the library one and says so instead."""
    text = (DECKS / "t_homog.inp").read_text()
    for key in ("xDom", "yDom", "zDom"):
        text = text.replace(f"   {key}: 1\n", f"   {key}: 0\n")
    deck = tmp_path / "four_domains.inp"
    deck.write_text(text)
    res = subprocess.run([str(CYCLE), "-i", str(deck)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert res.returncode == 2 and "qsgAttach: 4 domains" in res.stdout


@pytest.mark.skipif(not CYCLE_EXP.exists(), reason="the adapter's main-loop harness for -DEXPONENTIAL_TALLY is absent")
@pytest.mark.parametrize("name", ["t_homog", "t_fission"])
def test_exponential_tally_build_through_adapter(name, tmp_path):
    """The reference built with -DEXPONENTIAL_TALLY, the adapter switching the
    library's exponential tally on: every cycle's counters are that build's
    (tests/golden/exp_<deck>.npz, from the unmodified reference built with the
    define) and the cell tally handed to its Tallies sums to that build's
    within 1e-12."""
    from quicksilver_gb300 import _native as N
    gold = np.load(GOLDEN / f"exp_{name}.npz")
    res = subprocess.run([str(CYCLE_EXP), "-i", str(DECKS / f"{name}.inp")], cwd=tmp_path, capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = res.stdout.split("\n")
    totals = [float(line.split()[1]) for line in lines if line.startswith("cell_tally_total ")]
    k = next(i for i, line in enumerate(lines) if line.startswith("cycle "))
    rows = [line.split() for line in lines[k + 1:] if line[:8].strip().isdigit()]
    cols = ["start", "source", "rr", "split", "absorb", "scatter", "fission", "produce", "collision", "escape",
            "census", "num_segments"]
    assert len(rows) == len(totals) == len(gold["balance"])
    for c, row in enumerate(rows):
        for j, col in enumerate(cols):
            assert int(row[1 + j]) == int(gold["balance"][c][N.BAL[col]]), (c, col)
        want = gold["cell_tally"][c].sum()
        assert abs(totals[c] - want) <= 1e-12 * want, c
