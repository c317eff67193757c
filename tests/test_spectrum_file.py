"""The census energy spectrum file (observe.write_energy_spectrum) against
the file the unmodified reference prints for the same decks
(EnergySpectrum::PrintSpectrum, EnergySpectrum.cc:38-59;
tests/golden/spectrum_out.npz, make_golden.py --spectrum): the oracle's
census particles (bitwise the reference's) binned by energy group after
every cycle, as UpdateSpectrum does (EnergySpectrum.cc:12-36), and written
with our writer must give the reference's text.  The GPU's own histogram is
checked against the oracle in tests/test_gpu_observe.py."""
import numpy as np
import pytest

from helpers import DECKS, load_problem, oracle_run
from quicksilver_gb300.observe import write_energy_spectrum

SPEC = np.load(DECKS.parent.parent / "tests" / "golden" / "spectrum_out.npz")


def energy_groups(energies: np.ndarray, e: np.ndarray) -> np.ndarray:
    """NuclearData::getEnergyGroup (NuclearData.cc:207-228) for an array."""
    n = len(energies)
    g = np.searchsorted(energies, e, side="right") - 1
    return np.where(e <= energies[0], 0, np.where(e > energies[-1], n - 1, g))


@pytest.mark.parametrize("name", sorted(SPEC.keys()))
def test_spectrum_file_matches_reference(name, tmp_path):
    _, sim, hp = load_problem(f"{name}.inp")
    run = oracle_run(hp, sim)
    energies = hp.array("energies")
    counts = np.zeros(len(energies), dtype=np.int64)
    for _ in range(sim.n_steps):
        run.cycle_init()
        run.cycle_tracking(4)
        counts += np.bincount(energy_groups(energies, run.processed()["kinetic_energy"]), minlength=len(energies))
        run.cycle_finalize()
    path = write_energy_spectrum(str(tmp_path / "spec"), energies, counts)
    assert open(path).read() == str(SPEC[name])
