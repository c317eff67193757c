// Union of independent problems (host side of batched tracking).
#pragma once

#include <cstdint>
#include <vector>

#include "qsg.h"

namespace qsg {

struct UnionProblem {
    int32_t num_groups = 0;
    double time_step = 0.0;
    std::vector<double> energies, reaction_nubar, reaction_xs, material_atom_fraction, material_mass, nodes,
        facet_planes, cell_number_density, cell_volume;
    std::vector<int32_t> isotope_reaction_offset, reaction_type, material_isotope_offset, material_isotope_gid,
        cell_points, facet_local, facet_event, facet_adjacent_cell, facet_adjacent_facet, cell_material, cell_problem,
        problem_cell_offset, problem_material_offset;
    std::vector<uint64_t> cell_id;
    QsgProblem view{};
};

// Concatenate `n` problems; throws std::runtime_error when they cannot share
// one set of tables (different energy grid, time step or facet convention).
void build_union(const QsgProblem* problems, int n, UnionProblem& u);

}  // namespace qsg
