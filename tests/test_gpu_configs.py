"""GPU parity on the benchmark workloads themselves, through the C ABI, against
the C oracle (whose own pinning to the unmodified reference is
tests/test_oracle_golden.py).

* config2 (the 40^3-cell three-shell deck every bench.py number is quoted
  on): three whole cycles on the device (qsg_cycle_init / qsg_track_cycle /
  qsg_cycle_finalize) beside the oracle's cycleInit / cycleTracking /
  cycleFinalize, and against the unmodified reference's own counters for
  those cycles (tests/golden/config2.npz). Each cycle: all 13 balance
  counters bit for bit; scalar
  flux per group and in total within 1e-12 relative; census particles
  matched one to one by identifier and seed (integer fields exactly,
  floating fields to 1e-7 relative). Per cell the flux is held to 1e-8
  relative and per (cell, group) to 1e-7 relative (the census floats' bound)
  plus a floor of 1e-12 x the mean entry, for this reason: the default build
  takes log / sin / cos from the CUDA math library, which rounds a few
  arguments per thousand differently in the last bit from the host libm the
  oracle (and the reference) use. A last-bit difference in a particle's
  position can decide whether the facet search finds no facet and moves the
  particle toward the cell centre by 5e-11 of its distance from it
  (MCT.cc:505-531, 656-666, the reference's own retry), and particles that
  stream through many cells without colliding (the highest group) take that
  retry on one side only -- their later positions then differ by ~1e-10 cm,
  the flux entries they feed by up to ~1e-8 relative by the third cycle
  (census particles carry the offsets into the next cycle), while every
  event stays the same. With the portable elementary functions on both sides
  (libqsg_pm.so, tests/test_gpu_portable_math.py) config2 agrees bit for
  bit: every census particle, and every flux entry within 1e-12 with no
  floor.
* config2 over all 20 cycles of the deck (whole device cycles, the
  reference's run length): all 13 counters bit for bit and the scalar-flux
  total within 1e-12 every cycle.
* config4 (the differentiated workload: 3 materials, escape boundaries, 12
  scale parameters) at 1e5 particles x 3 cycles with sensitivities on:
  counters bit for bit every cycle, forward per-cell flux within 1e-12,
  dflux / dleak within 1e-10 per entry (sums of terms of both signs); and at
  its full size, 1e6 particles x 20 cycles: counters bit for bit every
  cycle, per-cell forward flux within 1e-8, dflux / dleak within 1e-8 per
  entry (the bounds config5 needs for the same reason), flux and leakage
  totals within 1e-10.
* config3 (the uneven ensemble): its first 16 problems at full size in one
  batch, whole cycles replayed from CUDA graphs, per-problem seed offsets;
  each problem against its own oracle run with the same offset: 13 counters
  bit for bit and the flux total within 1e-12, every cycle.
* five config3 problems (one per mesh edge) and config5's first replica
  deck at 3e6 particles, two cycles each with the reference's own seeding:
  their 13 counters equal the unmodified reference's
  (tests/golden/config3_pNN.npz, config5_r0.npz).
* config5 (the large batched + differentiated run) at 0.3 of its particles
  (3e6 per replica, the smallest count at which every cell sources) x 2
  cycles: 8 replicas with distinct seed offsets and 20 parameters tied across
  them in one graph-replayed batch; four replicas against the oracle:
  counters bit for bit, flux totals within 1e-12, per-cell forward flux
  within 1e-8 (config2's per-cell bound), dflux and dleak within 1e-8 per
  entry (sums of terms of both signs), all moved by the retry of the facet
  search as config2's flux is; leakage within 1e-10 (one accumulator per
  replica summed in a different order).

* At full size, where the oracle would take minutes to hours, through the
  counters' identities, which the unmodified reference satisfies on every
  golden deck and cycle: start + source + split - rr + produce = absorb +
  escape + census + fission, collision = scatter + absorb + fission, end =
  census, and each cycle starts with the previous cycle's census.  config3's
  whole ensemble (64 problems, 10 cycles) in one graph-replayed batch, also
  bit for bit against the problems run one by one; config5 at its full 8 x
  1e7 particles x 20 cycles with its 20 tied sensitivities, where besides the
  sensitivity run's per-cell flux, summed over cells, equals the sum of the
  cycles' flux totals within 1e-12 (two tallies of one quantity).

Reference behaviour reproduced: CycleTracking.cc:33-120, Tallies.cc:25-98,
main.cc:96-324, MC_SourceNow.cc:28-164, PopulationControl.cc:20-171.
"""
import numpy as np
import pytest

from helpers import DECKS, assert_flux_close, balance_identities, load_problem, oracle_run, sort_particles
from quicksilver_gb300 import Deck
from quicksilver_gb300.monte_carlo import BatchMonteCarlo, MonteCarlo, seed_offset
from quicksilver_gb300.sensitivity import band_params, tie_across_problems

pytestmark = pytest.mark.gpu

FP_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "kinetic_energy", "weight", "time_to_census", "age",
             "num_mean_free_paths", "num_segments"]
INT_FIELDS = ["random_number_seed", "identifier", "last_event", "num_collisions", "breed", "species",
              "domain", "cell"]
TRACK_SLOTS = [0, 1, 2, 3, 5, 6, 7, 12]   # absorb census escape collision fission produce scatter num_segments


def _census_match(got, want):
    assert len(got) == len(want)
    g, w = sort_particles(got), sort_particles(want)
    for f in INT_FIELDS:
        np.testing.assert_array_equal(g[f], w[f], err_msg=f)
    for f in FP_FIELDS:
        np.testing.assert_allclose(g[f], w[f], rtol=1e-7, atol=1e-12, err_msg=f)


def _flux_match(flux, want):
    # the bounds of the module docstring (the default build's elementary functions)
    assert_flux_close(flux, want, rel=1e-7, scale_floor=1e-12)         # per (cell, group)
    assert_flux_close(flux.sum(axis=1), want.sum(axis=1), rel=1e-8)      # per cell
    assert_flux_close(flux.sum(axis=0), want.sum(axis=0), rel=1e-12)     # per group
    assert abs(flux.sum() - want.sum()) <= 1e-12 * abs(want.sum())


def _tuples(params):
    return [(p.material, p.reaction, p.group_lo, p.group_hi, p.theta) for p in params]


def test_config2_device_cycles_match_oracle(gpu):
    deck, sim, hp = load_problem("config2.inp")
    run = oracle_run(hp, sim)
    mc = MonteCarlo(deck, problem=hp)
    try:
        for c in range(3):
            run.cycle_init()
            mc.cycle_init()
            assert mc.tracker.sizes()[0] == len(run.processing()), f"cycle {c}: processing count"
            mc.cycle_tracking()
            bal, flux = mc.tracker.tallies()
            census = mc.tracker.census()
            run.cycle_tracking(0)
            want_bal = run.balance()
            np.testing.assert_array_equal(bal[TRACK_SLOTS], want_bal[TRACK_SLOTS], err_msg=f"cycle {c}")
            _flux_match(flux, run.flux())
            _census_match(census, run.processed())
            mc.cycle_finalize()
            run.cycle_finalize()
            np.testing.assert_array_equal(mc.history(c, 1).balance[0], run.last_balance(), err_msg=f"cycle {c}")
            assert int(run.last_balance()[12]) > 10_000_000   # the full workload, not a trivial cycle
        assert mc.device_status() == 0
        # and the unmodified reference's own counters for these cycles
        gold = np.load(DECKS.parent.parent / "tests" / "golden" / "config2.npz")["balance"]
        np.testing.assert_array_equal(mc.history(0, 3).balance, gold)
    finally:
        mc.close()


def test_config2_all_cycles_match_oracle(gpu):
    deck, sim, hp = load_problem("config2.inp")
    assert sim.n_steps == 20
    mc = MonteCarlo(deck, problem=hp)
    try:
        hist = mc.run()
    finally:
        mc.close()
    run = oracle_run(hp, sim)
    for c in range(sim.n_steps):
        run.cycle_init()
        run.cycle_tracking(0)
        want_total = run.flux().sum()
        run.cycle_finalize()
        np.testing.assert_array_equal(hist.balance[c], run.last_balance(), err_msg=f"cycle {c}")
        assert abs(hist.flux_total[c] - want_total) <= 1e-12 * abs(want_total), f"cycle {c}"
    run.close()
    assert int(hist.balance[:, 12].sum()) > 200_000_000   # the deck's whole run


def test_config4_full_size_sensitivities_match_oracle(gpu):
    deck, sim, hp = load_problem("config4.inp")
    assert sim.n_particles == 1_000_000 and sim.n_steps == 20
    params = band_params(hp.array("energies"), hp.num_materials)
    run = oracle_run(hp, sim)
    run.enable_sensitivity(_tuples(params))
    mc = MonteCarlo(deck, problem=hp)
    try:
        mc.tracker.enable_sensitivity(params)
        hist = mc.run()
        got = mc.tracker.read_sensitivity()
    finally:
        mc.close()
    for c in range(sim.n_steps):
        run.cycle_init()
        run.cycle_tracking(0)
        run.cycle_finalize()
        np.testing.assert_array_equal(hist.balance[c], run.last_balance(), err_msg=f"cycle {c}")
    gold = np.load(DECKS.parent.parent / "tests" / "golden" / "config4.npz")["balance"]
    np.testing.assert_array_equal(hist.balance[:len(gold)], gold)   # the unmodified reference's own counters
    fc, df, leak, dl = run.read_sensitivity()
    run.close()
    assert_flux_close(got["flux_cell"], fc, rel=1e-8)
    assert abs(got["flux_cell"].sum() - fc.sum()) <= 1e-10 * fc.sum()
    for k in range(df.shape[1]):
        assert_flux_close(got["dflux"][:, k], df[:, k], rel=1e-8, scale_floor=1e-12)
    np.testing.assert_allclose(got["leak"][0], leak, rtol=1e-10, atol=0)
    np.testing.assert_allclose(got["dleak"][0], dl, rtol=1e-8, atol=1e-12 * abs(leak))


def test_config4_sensitivity_cycles_match_oracle(gpu):
    deck, sim, hp = load_problem("config4.inp", {"nParticles": 100000, "nSteps": 3})
    params = band_params(hp.array("energies"), hp.num_materials)
    assert len(params) == 12
    run = oracle_run(hp, sim)
    run.enable_sensitivity(_tuples(params))
    mc = MonteCarlo(deck, problem=hp)
    try:
        mc.tracker.enable_sensitivity(params)
        for c in range(3):
            run.cycle_init()
            mc.cycle_init()
            mc.cycle_tracking()
            mc.cycle_finalize()
            run.cycle_tracking(0)
            run.cycle_finalize()
            np.testing.assert_array_equal(mc.history(c, 1).balance[0], run.last_balance(), err_msg=f"cycle {c}")
        got = mc.tracker.read_sensitivity()
        assert mc.device_status() == 0
    finally:
        mc.close()
    fc, df, leak, dl = run.read_sensitivity()
    assert leak > 0 and np.abs(df).sum() > 0
    assert_flux_close(got["flux_cell"], fc, rel=1e-12, scale_floor=1e-12)
    for k in range(df.shape[1]):
        assert_flux_close(got["dflux"][:, k], df[:, k], rel=1e-10, scale_floor=1e-12)
    np.testing.assert_allclose(got["leak"][0], leak, rtol=1e-12, atol=0)
    np.testing.assert_allclose(got["dleak"][0], dl, rtol=1e-10, atol=1e-12 * abs(leak))


def test_config3_subset_batch_matches_oracle(gpu):
    from quicksilver_gb300.decks.make_decks import config3
    cycles = 3
    decks = [Deck.from_string(t, {"nSteps": cycles}) for t in config3()[:16]]
    problems = [d.build() for d in decks]
    offs = [seed_offset(d.simulation.seed) for d in decks]
    bmc = BatchMonteCarlo(decks, problems=problems, seed_offsets=offs, max_passes=8)
    try:
        hist = bmc.run(cycles, use_graph=True)
        assert bmc.device_status() == 0
    finally:
        bmc.close()
    busy = 0
    for p, (d, hp, off) in enumerate(zip(decks, problems, offs)):
        run = oracle_run(hp, d.simulation)
        run.set_seed_offset(off)
        for c in range(cycles):
            run.cycle_init()
            run.cycle_tracking(0)
            want_total = run.flux().sum()
            run.cycle_finalize()
            np.testing.assert_array_equal(hist.balance[c, p], run.last_balance(), err_msg=f"problem {p} cycle {c}")
            assert abs(hist.flux_total[c, p] - want_total) <= 1e-12 * abs(want_total), f"problem {p} cycle {c}"
        busy += int(run.last_balance()[12] > 0)
        run.close()
    # the subset holds empty problems (fewer particles than the source's
    # per-cell floor needs) and busy ones; both kinds must match
    assert 4 <= busy < 16


def test_config3_problems_match_reference_counters(gpu):
    """Five problems of the config3 ensemble (one per mesh edge), two whole
    device cycles each with the reference's own seeding: all 13 counters
    equal the unmodified reference's (tests/golden/config3_pNN.npz)."""
    import re
    from quicksilver_gb300.decks.make_decks import config3
    texts = config3()
    for p in (4, 6, 15, 26, 33):
        deck = Deck.from_string(re.sub(r"nSteps: \d+", "nSteps: 2", texts[p]))
        gold = np.load(DECKS.parent.parent / "tests" / "golden" / f"config3_p{p:02d}.npz")["balance"]
        mc = MonteCarlo(deck)
        try:
            hist = mc.run(2)
        finally:
            mc.close()
        np.testing.assert_array_equal(hist.balance, gold, err_msg=f"problem {p}")


def test_config5_replica_matches_reference_counters(gpu):
    """config5's first replica deck (its slab geometry) at 3e6 particles, two
    whole device cycles with the reference's own seeding: all 13 counters of
    both cycles equal the unmodified reference's (tests/golden/config5_r0.npz)."""
    import re
    from quicksilver_gb300.decks.make_decks import config5
    deck = Deck.from_string(re.sub(r"nSteps: \d+", "nSteps: 2", config5(n_particles=3_000_000)[0]))
    gold = np.load(DECKS.parent.parent / "tests" / "golden" / "config5_r0.npz")["balance"]
    mc = MonteCarlo(deck)
    try:
        hist = mc.run(2)
    finally:
        mc.close()
    np.testing.assert_array_equal(hist.balance, gold)
    assert int(gold[:, 12].sum()) > 30_000_000


def test_config5_scaled_batch_with_sensitivities_matches_oracle(gpu):
    from quicksilver_gb300.decks.make_decks import config5
    cycles = 2
    n_part = 3_000_000
    decks = [Deck.from_string(t, {"nSteps": cycles}) for t in config5(n_particles=n_part)]
    problems = [d.build() for d in decks]
    offs = [seed_offset(d.simulation.seed) for d in decks]
    base = band_params(problems[0].array("energies"), problems[0].num_materials)
    assert len(base) == 20
    cap = int(1.3 * (n_part + n_part // 10)) + 1024
    bmc = BatchMonteCarlo(decks, problems=problems, seed_offsets=offs, store_capacity=cap, max_passes=2)
    try:
        bmc.tracker.enable_sensitivity(tie_across_problems(base, bmc.tracker.material_offsets()))
        hist = bmc.run(cycles, use_graph=True)
        sens = bmc.tracker.read_sensitivity()
        coff = bmc.tracker.cell_offsets
        assert bmc.device_status() == 0
    finally:
        bmc.close()
    assert len({int(hist.balance[0, p, 12]) for p in range(len(decks))}) == len(decks)   # distinct replicas
    for p in (0, 2, 5, 7):
        hp = problems[p]
        run = oracle_run(hp, decks[p].simulation)
        run.set_seed_offset(offs[p])
        run.enable_sensitivity(_tuples(base))
        for c in range(cycles):
            run.cycle_init()
            run.cycle_tracking(0)
            want_total = run.flux().sum()
            run.cycle_finalize()
            np.testing.assert_array_equal(hist.balance[c, p], run.last_balance(), err_msg=f"replica {p} cycle {c}")
            assert abs(hist.flux_total[c, p] - want_total) <= 1e-12 * abs(want_total)
        fc, df, leak, dl = run.read_sensitivity()
        run.close()
        rows = slice(int(coff[p]), int(coff[p + 1]))
        assert leak > 0
        assert_flux_close(sens["flux_cell"][rows], fc, rel=1e-8)
        assert abs(sens["flux_cell"][rows].sum() - fc.sum()) <= 1e-12 * fc.sum()
        for k in range(df.shape[1]):
            assert_flux_close(sens["dflux"][rows, k], df[:, k], rel=1e-8, scale_floor=1e-12)
        # one accumulator per replica, ~1e6 escaping weights added in a
        # different order: summation alone reaches ~1e-11 relative here
        np.testing.assert_allclose(sens["leak"][p], leak, rtol=1e-10, atol=0)
        np.testing.assert_allclose(sens["dleak"][p], dl, rtol=1e-8, atol=1e-12 * abs(leak))


def test_config3_full_ensemble_batch(gpu):
    from quicksilver_gb300.decks.make_decks import config3
    decks = [Deck.from_string(t) for t in config3()]
    assert len(decks) == 64
    problems = [d.build() for d in decks]
    offs = [seed_offset(d.simulation.seed) for d in decks]
    cycles = decks[0].simulation.n_steps
    bmc = BatchMonteCarlo(decks, problems=problems, seed_offsets=offs)
    try:
        hist = bmc.run(cycles, use_graph=True)
        assert bmc.device_status() == 0
    finally:
        bmc.close()
    busy = 0
    for p, (d, hp, off) in enumerate(zip(decks, problems, offs)):
        balance_identities(hist.balance[:, p], f"problem {p}")
        mc = MonteCarlo(d, problem=hp, seed_offset=off)
        try:
            one = mc.run(cycles)
        finally:
            mc.close()
        np.testing.assert_array_equal(hist.balance[:, p], one.balance, err_msg=f"problem {p}")
        busy += int(one.balance[:, 12].sum() > 0)
    assert busy >= 32


def test_config5_full_size_batch_with_sensitivities(gpu):
    from quicksilver_gb300.decks.make_decks import config5
    decks = [Deck.from_string(t) for t in config5()]
    assert len(decks) == 8 and decks[0].simulation.n_particles == 10_000_000
    problems = [d.build() for d in decks]
    offs = [seed_offset(d.simulation.seed) for d in decks]
    cycles = decks[0].simulation.n_steps
    n_part = decks[0].simulation.n_particles
    cap = int(1.3 * (n_part + n_part // 10)) + 1024
    base = band_params(problems[0].array("energies"), problems[0].num_materials)
    bmc = BatchMonteCarlo(decks, problems=problems, seed_offsets=offs, store_capacity=cap, max_passes=2)
    try:
        bmc.tracker.enable_sensitivity(tie_across_problems(base, bmc.tracker.material_offsets()))
        hist = bmc.run(cycles, use_graph=True)
        sens = bmc.tracker.read_sensitivity()
        coff = bmc.tracker.cell_offsets
        assert bmc.device_status() == 0
    finally:
        bmc.close()
    assert int(hist.balance[:, :, 12].sum()) > 5_000_000_000
    for p in range(len(decks)):
        balance_identities(hist.balance[:, p], f"replica {p}")
        cells = sens["flux_cell"][int(coff[p]):int(coff[p + 1])].sum()
        total = hist.flux_total[:, p].sum()
        assert total > 0 and abs(cells - total) <= 1e-12 * total, p
        assert sens["leak"][p] > 0 and np.abs(sens["dleak"][p]).sum() > 0
