"""Input decks and host-built problem tables.

Mirrors the reference's set-up layer: ``Deck`` is Quicksilver's ``Parameters``
(Parameters.hh:169-175, read by getParameters, Parameters.cc:80-95) and
``HostProblem`` holds what ``initMC`` builds (NuclearData, MaterialDatabase,
one MC_Domain; initMC.cc:53-320).  Both are native C++ in libqsg.so; this
module only owns their handles.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _native as N


class Deck:
    """A parsed Quicksilver input deck (same blocks, keys and defaults)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle

    @classmethod
    def from_file(cls, path: str | Path, overrides: dict | None = None) -> "Deck":
        h = C.c_void_p()
        N.check(N.lib().qsg_deck_parse_file(str(path).encode(), C.byref(h)))
        deck = cls(h)
        for k, v in (overrides or {}).items():
            deck.set(k, v)
        return deck

    @classmethod
    def from_string(cls, text: str, overrides: dict | None = None) -> "Deck":
        h = C.c_void_p()
        N.check(N.lib().qsg_deck_parse_string(text.encode(), C.byref(h)))
        deck = cls(h)
        for k, v in (overrides or {}).items():
            deck.set(k, v)
        return deck

    def set(self, key: str, value) -> None:
        """Override a Simulation key, like the reference's command-line flags."""
        N.check(N.lib().qsg_deck_set(self._h, key.encode(), str(value).encode()))

    @property
    def simulation(self) -> N.QsgSimulation:
        s = N.QsgSimulation()
        N.check(N.lib().qsg_deck_simulation(self._h, C.byref(s)))
        return s

    @property
    def energy_spectrum(self) -> str:
        """The Simulation block's energySpectrum file stem ("" when absent)."""
        buf = C.create_string_buffer(4096)
        N.check(N.lib().qsg_deck_energy_spectrum(self._h, buf, len(buf)))
        return buf.value.decode()

    def text(self) -> str:
        """The deck as the reference echoes it at start-up (printParameters,
        Parameters.cc:97-215), defaults filled in."""
        need = C.c_size_t(0)
        N.lib().qsg_deck_write(self._h, None, 0, C.byref(need))
        buf = C.create_string_buffer(need.value)
        N.check(N.lib().qsg_deck_write(self._h, buf, len(buf), C.byref(need)))
        return buf.value.decode()

    def _echo_values(self, block: str, key: str) -> list:
        out, cur = [], None
        for line in self.text().splitlines():
            if line and not line.startswith(" "):
                cur = line.rstrip(":")
            elif cur == block and line.strip().startswith(key + ":"):
                out.append(line.split(":", 1)[1].strip())
        return out

    @property
    def material_names(self) -> list:
        """The materials in name order -- the order of the built problem's materials."""
        return self._echo_values("Material", "name")

    @property
    def cross_sections_out(self) -> str:
        """The Simulation block's crossSectionsOut file stem ("" when absent)."""
        vals = self._echo_values("Simulation", "crossSectionsOut")
        return vals[0] if vals else ""

    def build(self) -> "HostProblem":
        h = C.c_void_p()
        N.check(N.lib().qsg_deck_build(self._h, C.byref(h)))
        return HostProblem(h)

    def close(self):
        if self._h:
            N.lib().qsg_deck_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HostProblem:
    """Host-side problem tables (one domain covering the whole grid)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self.view = N.QsgProblem()
        N.check(N.lib().qsg_host_problem_view(self._h, C.byref(self.view)))

    @property
    def ptr(self):
        """Address of the QsgProblem view (valid while this object lives)."""
        return C.addressof(self.view)

    @property
    def num_cells(self) -> int:
        return self.view.num_cells

    @property
    def num_groups(self) -> int:
        return self.view.num_groups

    @property
    def num_materials(self) -> int:
        return self.view.num_materials

    def source_rates(self) -> np.ndarray:
        out = np.zeros(self.num_materials, dtype=np.float64)
        N.check(N.lib().qsg_host_problem_source_rates(self._h, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                      self.num_materials))
        return out

    def scale_xs(self, material: int, reaction_type: int, g_lo: int, g_hi: int, factor: float) -> None:
        N.check(N.lib().qsg_host_problem_scale_xs(self._h, material, reaction_type, g_lo, g_hi, factor))
        N.check(N.lib().qsg_host_problem_view(self._h, C.byref(self.view)))

    def array(self, name: str) -> np.ndarray:
        """Copy of one table of the QsgProblem view."""
        v = self.view
        C_, G = v.num_cells, v.num_groups
        niso, nmat = v.num_isotopes, v.num_materials
        nreact = int(np.ctypeslib.as_array(v.isotope_reaction_offset, (niso + 1,))[-1])
        niso_entries = int(np.ctypeslib.as_array(v.material_isotope_offset, (nmat + 1,))[-1])
        sizes = {
            "energies": G + 1, "isotope_reaction_offset": niso + 1, "reaction_type": nreact,
            "reaction_nubar": nreact, "reaction_xs": nreact * G, "material_isotope_offset": nmat + 1,
            "material_isotope_gid": niso_entries, "material_atom_fraction": niso_entries,
            "material_mass": nmat, "nodes": v.num_nodes * 3, "cell_points": C_ * 14,
            "facet_local_points": 72, "facet_planes": C_ * 96, "facet_event": C_ * 24,
            "facet_adjacent_cell": C_ * 24, "facet_adjacent_facet": C_ * 24, "cell_material": C_,
            "cell_number_density": C_, "cell_volume": C_, "cell_id": C_,
        }
        return np.ctypeslib.as_array(getattr(v, name), (sizes[name],)).copy()

    def close(self):
        if self._h:
            N.lib().qsg_host_problem_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
