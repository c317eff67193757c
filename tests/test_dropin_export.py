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
  tally; and with the reference's one-rank default of four domains
  (xDom = yDom = zDom = 0), whose domains the adapter joins into one mesh,
  the unmodified four-domain reference's counters and flux totals;
* the cycle adapter's vault and tally halves around the reference's own
  first cycleInit: the particles it gathers from the processing vaults are
  the oracle's, bit for bit; scattering them into the processed vaults and
  gathering them back is exact, no vault above its size; the counters and
  flux it hands over are what the reference's Tallies then hold -- on one
  domain and on four;
* the export of a four-domain MonteCarlo, cells put in the reference's
  global cell-id order, is this library's single-domain mesh table for
  table (adjacency through the same permutation).

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


def _four_domain_deck(name, tmp_path):
    """The deck with the reference's one-rank default decomposition
    (xDom = yDom = zDom = 0: four domains, initMC.cc:255-270)."""
    text = (DECKS / f"{name}.inp").read_text()
    for key in ("xDom", "yDom", "zDom"):
        assert f"   {key}: 1\n" in text
        text = text.replace(f"   {key}: 1\n", f"   {key}: 0\n")
    path = tmp_path / f"{name}_4dom.inp"
    path.write_text(text)
    return path


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


REF = ROOT / "oracle" / "_ref" / "qs_ref_harness"


def _summary_rows(stdout):
    lines = stdout.split("\n")
    k = next(i for i, line in enumerate(lines) if line.startswith("cycle "))
    return [line.split()[:14] for line in lines[k + 1:] if line[:8].strip().isdigit()]


@pytest.mark.skipif(not (CYCLE.exists() and REF.exists()), reason="the adapter's main-loop harness is absent")
@pytest.mark.parametrize("name", ["t_homog", "t_fission", "t_nonflat", "t_escape"])
def test_four_domains_through_adapter(name, tmp_path):
    """The reference's one-rank default builds four domains; the adapter joins
    them into one mesh for the library and hands census particles and flux
    back per domain.  Every cycle's counters and scalar-flux total printed by
    the reference's main loop through the adapter are those printed by the
    unmodified reference on the same four domains."""
    deck = _four_domain_deck(name, tmp_path)
    env = dict(os.environ, OMP_NUM_THREADS="4")
    ref = subprocess.run([str(REF), "-i", str(deck)], cwd=tmp_path, capture_output=True, text=True, env=env,
                         timeout=600)
    got = subprocess.run([str(CYCLE), "-i", str(deck)], cwd=tmp_path, capture_output=True, text=True, env=env,
                         timeout=600)
    assert ref.returncode == 0 and got.returncode == 0, got.stdout[-2000:] + got.stderr[-2000:]
    assert got.stdout.count("Building partition") == 4
    want_rows, got_rows = _summary_rows(ref.stdout), _summary_rows(got.stdout)
    assert len(got_rows) == len(want_rows) > 1 and int(want_rows[0][12]) > 0
    for g, w in zip(got_rows, want_rows):
        assert g == w, (g, w)


def _by_cell_id(dump, hp):
    """Position in the deck reader's mesh of every exported cell."""
    ids = hp.array("cell_id")
    order = np.argsort(ids)
    pos = order[np.searchsorted(ids, dump["cell_id"], sorter=order)]
    assert (ids[pos] == dump["cell_id"]).all() and len(np.unique(pos)) == len(pos) == hp.num_cells
    return pos


@pytest.mark.parametrize("name", ["t_homog", "t_nonflat", "t_escape", "t_scatter_octant"])
def test_four_domain_export_is_one_mesh(name, tmp_path):
    dump = tmp_path / "export.bin"
    res = subprocess.run([str(HARNESS), "-i", str(_four_domain_deck(name, tmp_path))],
                         env=dict(os.environ, QS_DUMP=str(dump)), capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert "export accepted (4 domains" in res.stdout
    got = read_dump(dump)
    hp = Deck.from_file(DECKS / f"{name}.inp").build()
    pos = _by_cell_id(got, hp)
    C = hp.num_cells
    per_cell = {"facet_planes": 96, "facet_event": 24, "facet_adjacent_facet": 24, "cell_material": 1,
                "cell_number_density": 1, "cell_volume": 1}
    for key, width in per_cell.items():
        want = hp.array(key).reshape(C, width)[pos]
        arr = got[key].reshape(C, width)
        np.testing.assert_array_equal(arr.view(f"u{arr.dtype.itemsize}"), want.view(f"u{want.dtype.itemsize}"),
                                      err_msg=key)
    adj = got["facet_adjacent_cell"].reshape(C, 24)
    np.testing.assert_array_equal(pos[adj], hp.array("facet_adjacent_cell").reshape(C, 24)[pos])
    corners = got["nodes"].reshape(-1, 3)[got["cell_points"].reshape(-1, 14)]
    ours = hp.array("nodes").reshape(-1, 3)[hp.array("cell_points").reshape(-1, 14)][pos]
    np.testing.assert_array_equal(corners.view(np.uint64), ours.view(np.uint64))


@pytest.mark.parametrize("name", ["t_homog", "t_fission"])
def test_four_domain_vaults_and_tallies(name, tmp_path):
    """Gathered from four domains, the first cycle's particles are the
    oracle's (single domain) bit for bit once their joined-mesh cell is put
    back to the deck reader's numbering (the domain field names the
    reference's domain, so it is not compared); the round trip and the tally
    hand-over checks of the harness pass."""
    from helpers import load_problem, oracle_run, sort_particles
    dump = tmp_path / "vaults.bin"
    res = subprocess.run([str(HARNESS), "-i", str(_four_domain_deck(name, tmp_path))],
                         env=dict(os.environ, QS_DUMP=str(dump), QS_VAULTS="1"), capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout[-1000:] + res.stderr[-2000:]
    got = read_dump(dump)
    _, sim, hp = load_problem(f"{name}.inp")
    pos = _by_cell_id(got, hp)
    run = oracle_run(hp, sim)
    run.cycle_init()
    want = run.processing()
    rec = np.zeros(len(want), want.dtype)
    for field in want.dtype.names:
        rec[field] = got["p_" + field]
    rec["cell"] = pos[rec["cell"]]
    rec["domain"] = want["domain"][0]
    assert len(rec) == len(want)
    a, b = sort_particles(rec), sort_particles(want)
    for field in want.dtype.names:
        size = a[field].dtype.itemsize
        np.testing.assert_array_equal(a[field].view(f"u{size}"), b[field].view(f"u{size}"), err_msg=field)


@pytest.mark.skipif(not CYCLE_EXP.exists(), reason="the adapter's main-loop harness for -DEXPONENTIAL_TALLY is absent")
@pytest.mark.parametrize("domains", [1, 4])
@pytest.mark.parametrize("name", ["t_homog", "t_fission"])
def test_exponential_tally_build_through_adapter(name, domains, tmp_path):
    """The reference built with -DEXPONENTIAL_TALLY, the adapter switching the
    library's exponential tally on: every cycle's counters are that build's
    (tests/golden/exp_<deck>.npz, from the unmodified reference built with the
    define) and the cell tally handed to its Tallies sums to that build's
    within 1e-12 -- on one domain, and on the four-domain default, where the
    adapter hands each domain its cells' share."""
    from quicksilver_gb300 import _native as N
    gold = np.load(GOLDEN / f"exp_{name}.npz")
    deck = DECKS / f"{name}.inp" if domains == 1 else _four_domain_deck(name, tmp_path)
    res = subprocess.run([str(CYCLE_EXP), "-i", str(deck)], cwd=tmp_path, capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.count("Building partition") == domains
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
