// Union of independent single-domain problems for batched tracking.
//
// Each problem keeps its own materials, isotopes, cells and nodes; indices are
// shifted into one set of tables and no facet of one problem is adjacent to a
// cell of another, so tracking the union is tracking every problem on its own.
// The problems must share the energy-group edges (the group search is over one
// table) and the time step.  Cell ids (MC_Cell_State::_id, the source seeds)
// stay problem-local, exactly as each problem alone would have them.
#include "batch.h"

#include <cstring>
#include <stdexcept>
#include <string>

namespace qsg {

namespace {
template <typename T>
void append(std::vector<T>& dst, const T* src, size_t n)
{
    if (n) dst.insert(dst.end(), src, src + n);
}
}  // namespace

void build_union(const QsgProblem* problems, int n, UnionProblem& u)
{
    if (n < 1) throw std::runtime_error("batch: need at least one problem");
    const QsgProblem& p0 = problems[0];
    const int G = p0.num_groups;
    u.num_groups = G;
    u.energies.assign(p0.energies, p0.energies + G + 1);
    u.time_step = p0.time_step;
    u.facet_local.assign(p0.facet_local_points, p0.facet_local_points + 72);
    u.isotope_reaction_offset.assign(1, 0);
    u.material_isotope_offset.assign(1, 0);
    u.problem_cell_offset.assign(1, 0);
    u.problem_material_offset.assign(1, 0);
    for (int k = 0; k < n; k++) {
        const QsgProblem& p = problems[k];
        if (p.num_groups != G || memcmp(p.energies, p0.energies, sizeof(double) * (G + 1)) != 0)
            throw std::runtime_error("batch: problem " + std::to_string(k) + " has a different energy grid");
        if (p.time_step != p0.time_step)
            throw std::runtime_error("batch: problem " + std::to_string(k) + " has a different time step");
        if (memcmp(p.facet_local_points, p0.facet_local_points, sizeof(int32_t) * 72) != 0)
            throw std::runtime_error("batch: problem " + std::to_string(k) + " uses another facet convention");
        if (!p.cell_volume || !p.cell_id)
            throw std::runtime_error("batch: problem " + std::to_string(k) + " lacks cell_volume / cell_id");
        const int32_t iso0 = (int32_t)u.isotope_reaction_offset.size() - 1;
        const int32_t r0 = u.isotope_reaction_offset.back();
        const int32_t mat0 = (int32_t)u.material_mass.size();
        const int32_t cell0 = (int32_t)u.cell_material.size();
        const int32_t node0 = (int32_t)(u.nodes.size() / 3);
        for (int i = 0; i < p.num_isotopes; i++)
            u.isotope_reaction_offset.push_back(r0 + p.isotope_reaction_offset[i + 1]);
        const int32_t R = p.isotope_reaction_offset[p.num_isotopes];
        append(u.reaction_type, p.reaction_type, R);
        append(u.reaction_nubar, p.reaction_nubar, R);
        append(u.reaction_xs, p.reaction_xs, (size_t)R * G);
        const int32_t e0 = u.material_isotope_offset.back();
        for (int m = 0; m < p.num_materials; m++) u.material_isotope_offset.push_back(e0 + p.material_isotope_offset[m + 1]);
        const int32_t E = p.material_isotope_offset[p.num_materials];
        for (int e = 0; e < E; e++) u.material_isotope_gid.push_back(iso0 + p.material_isotope_gid[e]);
        append(u.material_atom_fraction, p.material_atom_fraction, E);
        append(u.material_mass, p.material_mass, p.num_materials);
        append(u.nodes, p.nodes, (size_t)p.num_nodes * 3);
        const int64_t C = p.num_cells;
        for (int64_t i = 0; i < C * 14; i++) u.cell_points.push_back(node0 + p.cell_points[i]);
        append(u.facet_planes, p.facet_planes, (size_t)C * 96);
        append(u.facet_event, p.facet_event, (size_t)C * 24);
        for (int64_t i = 0; i < C * 24; i++) u.facet_adjacent_cell.push_back(cell0 + p.facet_adjacent_cell[i]);
        append(u.facet_adjacent_facet, p.facet_adjacent_facet, (size_t)C * 24);
        for (int64_t c = 0; c < C; c++) u.cell_material.push_back(mat0 + p.cell_material[c]);
        append(u.cell_number_density, p.cell_number_density, C);
        append(u.cell_volume, p.cell_volume, C);
        append(u.cell_id, p.cell_id, C);
        u.cell_problem.insert(u.cell_problem.end(), C, k);
        u.problem_cell_offset.push_back(cell0 + (int32_t)C);
        u.problem_material_offset.push_back(mat0 + p.num_materials);
        if (u.cell_material.size() > (size_t)INT32_MAX / 24) throw std::runtime_error("batch: too many cells");
    }
    QsgProblem& v = u.view;
    memset(&v, 0, sizeof(v));
    v.num_groups = G;
    v.energies = u.energies.data();
    v.num_isotopes = (int32_t)u.isotope_reaction_offset.size() - 1;
    v.isotope_reaction_offset = u.isotope_reaction_offset.data();
    v.reaction_type = u.reaction_type.data();
    v.reaction_nubar = u.reaction_nubar.data();
    v.reaction_xs = u.reaction_xs.data();
    v.num_materials = (int32_t)u.material_mass.size();
    v.material_isotope_offset = u.material_isotope_offset.data();
    v.material_isotope_gid = u.material_isotope_gid.data();
    v.material_atom_fraction = u.material_atom_fraction.data();
    v.material_mass = u.material_mass.data();
    v.num_cells = (int32_t)u.cell_material.size();
    v.num_nodes = (int32_t)(u.nodes.size() / 3);
    v.nodes = u.nodes.data();
    v.cell_points = u.cell_points.data();
    v.facet_local_points = u.facet_local.data();
    v.facet_planes = u.facet_planes.data();
    v.facet_event = u.facet_event.data();
    v.facet_adjacent_cell = u.facet_adjacent_cell.data();
    v.facet_adjacent_facet = u.facet_adjacent_facet.data();
    v.cell_material = u.cell_material.data();
    v.cell_number_density = u.cell_number_density.data();
    v.cell_volume = u.cell_volume.data();
    v.cell_id = u.cell_id.data();
    v.time_step = u.time_step;
}

}  // namespace qsg
