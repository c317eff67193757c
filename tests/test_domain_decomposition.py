"""The reference's default decomposition on one rank -- xDom = yDom = zDom
= 0 gives four domains with randomly placed centres (initMC.cc:255-270),
particles crossing between them through its in-process buffers -- tracks
the same histories as this library's single domain: for each deck, a copy
with the three keys set to 0 run by the unmodified reference (the harness
built from its sources) against the oracle on the same deck, counters bit
for bit on every cycle and scalar flux per (global cell id, group) within
1e-12.  (Explicit xDom * yDom * zDom > 1 on one rank is rejected by the
reference itself, initMC.cc:272.)  Runs where the harness is present."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import DECKS, oracle_run
from quicksilver_gb300 import Deck

ROOT = Path(__file__).resolve().parent.parent
HARNESS = ROOT / "oracle" / "_ref" / "qs_ref_harness"
sys.path.insert(0, str(ROOT / "tests" / "golden"))
from make_golden import read_dump   # noqa: E402

pytestmark = pytest.mark.skipif(not HARNESS.exists(), reason="the harness built from the reference's sources is absent")


@pytest.mark.parametrize("name", ["t_homog", "t_fission", "t_nonflat", "t_coral1", "t_escape"])
def test_four_random_domains_track_as_one(name, tmp_path):
    text = (DECKS / f"{name}.inp").read_text()
    for key in ("xDom", "yDom", "zDom"):
        assert f"   {key}: 1\n" in text
        text = text.replace(f"   {key}: 1\n", f"   {key}: 0\n")
    deck_path = tmp_path / f"{name}_4dom.inp"
    deck_path.write_text(text)
    dump = tmp_path / "dump.bin"
    res = subprocess.run([str(HARNESS), "-i", str(deck_path)], cwd=tmp_path, capture_output=True, text=True,
                         env=dict(os.environ, QS_DUMP=str(dump), OMP_NUM_THREADS="8"), timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.count("Building partition") == 4
    ref = read_dump(dump)
    deck = Deck.from_file(deck_path)
    sim, hp = deck.simulation, deck.build()
    run = oracle_run(hp, sim)
    for c in range(sim.n_steps):
        run.cycle_init()
        run.cycle_tracking(8)
        flux = run.flux()
        want_flux = ref[f"flux_c{c}"].reshape(flux.shape)
        run.cycle_finalize()
        np.testing.assert_array_equal(run.last_balance(), ref[f"balance_c{c}"], err_msg=f"cycle {c}")
        scale = np.abs(want_flux).max()
        assert np.abs(flux - want_flux).max() <= 1e-12 * scale, f"cycle {c}"
