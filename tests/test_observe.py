"""Observability outputs on the CPU: the CORAL2 checks (CoralBenchmark.cc)
on balances with known verdicts, on the oracle's run of a CORAL-style deck,
and the energy-spectrum file format (EnergySpectrum.cc:38-59)."""
import numpy as np

from helpers import OracleMonteCarlo, load_problem
from quicksilver_gb300 import _native as N
from quicksilver_gb300.observe import (balance_event_test, balance_ratio_test, coral_benchmark_correctness,
                                       cumulative_balance, fluence_test, missing_particle_test,
                                       write_energy_spectrum)


def _bal(**kw):
    b = {name: 0 for name in N.BALANCE_FIELDS}
    b.update(kw)
    return b


def test_balance_ratio_verdicts():
    ok, _, rel = balance_ratio_test(_bal(absorb=4000, fission=5000, scatter=100000), 1)
    assert ok and max(rel.values()) < 1e-12
    ok, msg, _ = balance_ratio_test(_bal(absorb=4100, fission=5000, scatter=100000), 1)   # 2.5% off
    assert not ok and msg.startswith("FAIL::")
    ok, _, _ = balance_ratio_test(_bal(absorb=9400, fission=7500, scatter=83000), 2)
    assert ok
    ok, _, _ = balance_ratio_test(_bal(absorb=9400 * 1.011, fission=7500, scatter=83000), 2)   # within 1.1%
    assert ok


def test_event_and_missing_particle_verdicts():
    assert balance_event_test(_bal(num_segments=2050, census=50, collision=1000))[0]
    assert not balance_event_test(_bal(num_segments=2100, census=50, collision=1000))[0]
    b = _bal(start=10, source=5, produce=7, split=3, absorb=6, census=9, escape=2, rr=4, fission=4)
    assert missing_particle_test(b)[0]
    b["escape"] += 1
    assert not missing_particle_test(b)[0]


def test_fluence_verdicts():
    assert fluence_test(np.full(27, 3.0))[0]
    f = np.full(27, 3.0)
    f[5] = 3.3   # ~9.5% from the mean
    ok, msg, diff = fluence_test(f)
    assert not ok and 9.0 < diff < 10.0 and "Max Percent Diff" in msg


def oracle_observe(name, cycles=None):
    """The oracle's run with the reference's observers restated
    (helpers.OracleMonteCarlo): cumulative counters per cycle, fluence per
    cell, census energy spectrum, group edges."""
    deck, sim, _ = load_problem(name)
    mc = OracleMonteCarlo(deck)
    mc.observe(fluence=True, spectrum=True)
    n = sim.n_steps if cycles is None else cycles
    for _ in range(n):
        mc.cycle_init()
        mc.cycle_tracking()
        mc.cycle_finalize()
    return mc.history(0, n).balance, mc.fluence(), mc.energy_spectrum()[0], mc.problem.array("energies")


def test_coral_checks_on_oracle_run(tmp_path):
    hist, fluence, spectrum, en = oracle_observe("t_coral1.inp")
    cum = cumulative_balance(hist)
    res = coral_benchmark_correctness(cum, fluence, 1, out=None)
    assert res["balance_ratio"] and res["balance_event"] and res["missing_particle"]
    assert spectrum.sum() == sum(int(h[N.BAL["census"]]) for h in hist)
    path = write_energy_spectrum(str(tmp_path / "spec"), en, spectrum)
    lines = open(path).read().splitlines()
    assert len(lines) == len(en)
    i, e, c = lines[3].split("\t")
    assert int(i) == 3 and float(e) == float(f"{en[3]:g}") and int(c) == int(spectrum[3])
