"""Problem tables built by libqsg's deck reader are bitwise equal to the
tables the reference's initMC builds from the same deck."""
import hashlib

import numpy as np
import pytest

from helpers import DECKS, load_problem

GOLDEN = DECKS.parent.parent / "tests" / "golden"
NAMES = sorted(p.stem for p in GOLDEN.glob("*.npz") if (DECKS / f"{p.stem}.inp").exists())   # per-deck fixtures


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def product_tables(hp):
    nodes = hp.array("nodes").reshape(-1, 3)
    pts = hp.array("cell_points").reshape(-1, 14)
    local = hp.array("facet_local_points").reshape(24, 3)
    cell_nodes = nodes[pts]                              # [C,14,3]
    facet_coords = cell_nodes[:, local, :]               # [C,24,3,3]
    return {
        "energies": hp.array("energies"),
        "iso_react_off": hp.array("isotope_reaction_offset"),
        "reaction_type": hp.array("reaction_type"),
        "reaction_nubar": hp.array("reaction_nubar"),
        "reaction_xs": hp.array("reaction_xs"),
        "mat_iso_off": hp.array("material_isotope_offset"),
        "mat_iso_gid": hp.array("material_isotope_gid"),
        "mat_iso_af": hp.array("material_atom_fraction"),
        "mat_mass": hp.array("material_mass"),
        "cell_volume": hp.array("cell_volume"),
        "cell_density": hp.array("cell_number_density"),
        "cell_material": hp.array("cell_material"),
        "cell_nodes": np.ascontiguousarray(cell_nodes.reshape(-1)),
        "cell_planes": hp.array("facet_planes"),
        "facet_point_coords": np.ascontiguousarray(facet_coords.reshape(-1)),
        "facet_event": hp.array("facet_event"),
        "facet_adj_facet": hp.array("facet_adjacent_facet"),
        "facet_adj_gid": hp.array("facet_adjacent_cell").astype(np.uint64),
        "time_step": np.array([hp.view.time_step]),
    }


@pytest.mark.parametrize("name", NAMES)
def test_tables_bitwise_equal(name):
    gold = np.load(GOLDEN / f"{name}.npz")
    _, _, hp = load_problem(f"{name}.inp")
    tabs = product_tables(hp)
    for tname, want in zip(gold["table_names"], gold["table_sha"]):
        assert _sha(tabs[str(tname)]) == want, f"{name}: table {tname} differs from the reference"
    # cell ids: gid << 32 (MC_Domain.cc:390), cell index == gid for one domain
    ids = hp.array("cell_id")
    np.testing.assert_array_equal(ids >> 32, np.arange(hp.num_cells, dtype=np.uint64))
