"""Batched tracking: independent decks in one handle (qsg_batch_create), whole
cycles enqueued without host synchronisation and replayed from CUDA graphs.

Every problem of the batch must reproduce, cycle by cycle, the 13 balance
counters the unmodified reference produced for that deck alone (golden
fixtures) bit for bit, and its flux total within 1e-12; graph replay must
equal direct enqueueing; kernel-shape tunings must not change any result.
"""
import numpy as np
import pytest

from helpers import DECKS, load_problem
from quicksilver_gb300 import Deck
from quicksilver_gb300.monte_carlo import BatchMonteCarlo, MonteCarlo

pytestmark = pytest.mark.gpu

GOLDEN = DECKS.parent.parent / "tests" / "golden"
# decks sharing eMin, eMax, nGroups and dt (a batch's one energy grid / time step)
BATCH = ["t_homog", "t_escape", "t_nocoll", "t_scatter_octant", "t_default"]
CYCLES = 2


def golden(name):
    return np.load(GOLDEN / f"{name}.npz")


def check_against_golden(hist):
    for p, name in enumerate(BATCH):
        g = golden(name)
        for c in range(CYCLES):
            np.testing.assert_array_equal(hist.balance[c, p], g["balance"][c], err_msg=f"{name} cycle {c}")
            assert abs(hist.flux_total[c, p] - g["flux_total"][c]) <= 1e-12 * abs(g["flux_total"][c]), name


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_each_problem_alone(gpu, use_graph):
    decks = [Deck.from_file(DECKS / f"{n}.inp") for n in BATCH]
    bmc = BatchMonteCarlo(decks, max_passes=64)
    hist = bmc.run(CYCLES, use_graph=use_graph)
    check_against_golden(hist)
    bmc.close()


@pytest.mark.parametrize("block,batch,chunk,replicas,step,refill",
                         [(256, 8, 4, 2, 24, 8), (128, 24, 1, 1, 1, 64), (128, 1, 16, 3, 32, 1)])
def test_tunings_do_not_change_results(gpu, block, batch, chunk, replicas, step, refill):
    decks = [Deck.from_file(DECKS / f"{n}.inp") for n in BATCH]
    bmc = BatchMonteCarlo(decks, max_passes=64, flux_replicas=replicas)
    bmc.tune(block, batch, chunk, pool_collision_step=step, pool_refill=refill)
    check_against_golden(bmc.run(CYCLES, use_graph=True))
    bmc.close()


def test_single_problem_graph_cycles_config1(gpu):
    deck, sim, hp = load_problem("config1.inp")
    mc = MonteCarlo(deck, problem=hp, max_passes=16)
    mc.run_cycles(sim.n_steps, use_graph=True)
    hist = mc.history()
    g = golden("config1")
    np.testing.assert_array_equal(hist.balance, g["balance"])
    np.testing.assert_allclose(hist.flux_total, g["flux_total"], rtol=1e-12)
    assert mc.device_status() == 0
    mc.close()


def test_sync_and_graph_cycles_interleave(gpu):
    """Graph replays and host-driven cycles can follow one another."""
    deck, sim, hp = load_problem("t_homog.inp")
    mc = MonteCarlo(deck, problem=hp, max_passes=16)
    mc.cycle_init()
    mc.cycle_tracking()
    mc.cycle_finalize()
    mc.run_cycles(2, use_graph=True)
    hist = mc.history()
    np.testing.assert_array_equal(hist.balance, golden("t_homog")["balance"][:3])
    mc.close()


def test_autotuner_returns_a_candidate(gpu, tmp_path):
    from quicksilver_gb300.autotune import autotune
    texts = [(DECKS / f"{n}.inp").read_text() for n in BATCH]
    space = {"block_size": (128, 256), "pool_collision_step": (32,), "pool_refill": (8, 16), "flux_replicas": (1,)}
    best = autotune(texts, scale=1.0, cycles=1, warmup=1, cache_path=tmp_path / "t.json", space=space)
    assert best["block_size"] in (128, 256) and best["segments_per_s"] > 0 and len(best["trials"]) == 4
    again = autotune(texts, cache_path=tmp_path / "t.json", space=space)   # cached
    assert again["segments_per_s"] == best["segments_per_s"]
