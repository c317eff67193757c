"""Every example deck the reference ships reads through this library's deck
reader as the reference reads it: our start-up echo (qsg_deck_write) equals,
text for text, the echo the unmodified reference prints for the same file
(the harness built from its sources, QS_ECHO), and each deck builds a
problem that passes qsg_create's checks, the reference's mesh self-test
included.  Runs where the reference's sources and the harness built from
them are present (they are test infrastructure; nothing of the decks is
kept in this repository), and skips elsewhere."""
import ctypes
import os
import subprocess
from pathlib import Path

import pytest

from quicksilver_gb300 import Deck
from quicksilver_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent
import __graft_entry__ as _entry   # noqa: E402  (its REF_SRC names the reference's sources)

EXAMPLES = _entry.REF_SRC.parent / "Examples"
HARNESS = ROOT / "oracle" / "_ref" / "qs_ref_harness"
DECKS = sorted(EXAMPLES.rglob("*.inp")) if EXAMPLES.exists() else []

pytestmark = pytest.mark.skipif(not DECKS or not HARNESS.exists(),
                                reason="the reference's sources or the harness built from them are absent")


def _reference_echo(deck: Path, tmp_path: Path) -> str:
    out = tmp_path / "echo.txt"
    env = dict(os.environ, QS_ECHO=str(out), QS_ECHO_ONLY="1")
    res = subprocess.run([str(HARNESS), "-i", str(deck)], env=env, capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr[-2000:]
    return out.read_text()


@pytest.mark.parametrize("deck", DECKS, ids=[str(d.relative_to(EXAMPLES)) for d in DECKS])
def test_reference_example_deck_reads_the_same(deck, tmp_path):
    ours = Deck.from_file(deck)
    assert ours.text() == _reference_echo(deck, tmp_path)


@pytest.mark.parametrize("deck", [d for d in DECKS if "4096" not in d.name and "_36" not in d.name],
                         ids=lambda d: d.name)
def test_reference_example_deck_builds_a_valid_problem(deck):
    hp = Deck.from_file(deck, {"nx": 4, "ny": 4, "nz": 4}).build()   # mesh kept small; the tables' kind is the deck's
    assert N.lib().qsg_problem_check(ctypes.byref(hp.view)) == N.QSG_OK, N.last_error()


def _scaled_copy(deck: Path, tmp_path: Path, **keys) -> Path:
    """The deck with some Simulation keys set (the deck's own keys win over
    command-line flags in the reference, so the text itself is edited)."""
    lines = deck.read_text().splitlines()
    out, block, done = [], None, set()
    for line in lines:
        stripped = line.strip()
        if line and not line[0].isspace():
            if block == "Simulation":
                out.extend(f"   {k}: {v}" for k, v in keys.items() if k not in done)
                done.update(keys)
            block = stripped.rstrip(":")
            out.append(line)
            continue
        key = stripped.split(":", 1)[0].strip()
        if block == "Simulation" and key in keys:
            out.append(f"   {key}: {keys[key]}")
            done.add(key)
        else:
            out.append(line)
    if block == "Simulation":
        out.extend(f"   {k}: {v}" for k, v in keys.items() if k not in done)
    path = tmp_path / deck.name
    path.write_text("\n".join(out) + "\n")
    return path


@pytest.mark.parametrize("deck", DECKS, ids=[str(d.relative_to(EXAMPLES)) for d in DECKS])
def test_oracle_counters_match_reference_on_its_example_decks(deck, tmp_path):
    """The C oracle against the unmodified reference on its own example decks,
    scaled to 3000 particles, 2 cycles and a 6^3 mesh: all 13 counters bit for
    bit every cycle.  A deck's own xDom = yDom = zDom = 0 (the reference's four
    random domains on one rank) is kept; an explicit decomposition, which the
    reference runs only with one MPI rank per domain, becomes one domain."""
    import numpy as np
    import sys
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from make_golden import read_dump
    from helpers import oracle_run

    keys = dict(nParticles=3000, nSteps=2, nx=6, ny=6, nz=6)
    doms = [int(Deck.from_file(deck)._echo_values("Simulation", k)[0]) for k in ("xDom", "yDom", "zDom")]
    if any(doms):
        keys.update(xDom=1, yDom=1, zDom=1)
    if deck.stem == "NonFlatXC":
        # supercritical (fission ratio 1 against absorption 6e-3, nuBar 2.4): within a
        # time step of 1e-8 s the fission chains grow without bound; 1e-10 s keeps them short
        keys["dt"] = 1e-10
    small = _scaled_copy(deck, tmp_path, **keys)
    dump = tmp_path / "ref.dump"
    env = dict(os.environ, QS_DUMP=str(dump), OMP_NUM_THREADS="4")
    res = subprocess.run([str(HARNESS), "-i", str(small)], env=env, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.count("Building partition") == (1 if any(doms) else 4)
    ref = read_dump(dump)
    d = Deck.from_file(small)
    sim, hp = d.simulation, d.build()
    run = oracle_run(hp, sim)
    for c in range(sim.n_steps):
        run.cycle_init()
        run.cycle_tracking(4)
        bal = run.balance()
        bal[4] = len(run.processed())
        np.testing.assert_array_equal(bal, ref[f"balance_c{c}"], err_msg=f"cycle {c}")
        run.cycle_finalize()
