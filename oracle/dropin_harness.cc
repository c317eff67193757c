// Test-infrastructure check of the drop-in adapter a Quicksilver maintainer
// adds to the reference (the table export after initMC that hands the
// library its QsgProblem).  Compiled with the UNMODIFIED reference's own
// sources and linked against libqsg.so by oracle/Makefile (`make dropin`),
// never part of the product.  It
//
//   * builds the reference's MonteCarlo object for a deck (getParameters +
//     initMC, Parameters.cc:80-95, initMC.cc:53-74);
//   * runs qsgExport below -- the adapter, the same code the integration
//     guide shows -- over it;
//   * validates the export with qsg_problem_check (no GPU needed);
//   * writes every exported array, named after its QsgProblem field, to the
//     file QS_DUMP names (records as oracle/ref_harness.cc writes them), so
//     the tests can compare it with the library's own deck reader.
//
// Exit status: 0 when qsg_problem_check accepts the export, else 2 (the
// library's message on stderr).

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "MonteCarlo.hh"
#include "Parameters.hh"
#include "initMC.hh"
#include "NuclearData.hh"
#include "MaterialDatabase.hh"
#include "MC_Domain.hh"
#include "MC_Time_Info.hh"
#include "utilsMpi.hh"

#include "qsg.h"

extern MonteCarlo* mcco;

// ---- the adapter ----------------------------------------------------------

// Host copies of one domain's tables in the library's layout; `problem`
// points into them, so it stays valid while the QsgExport lives.
struct QsgExport {
    std::vector<int32_t> iso_off{0}, rtype, mat_off{0}, mat_gid, pts, local, ev, adj_cell, adj_facet, mat;
    std::vector<double> nubar, xs, af, mass, planes, density, volume, nodes;
    std::vector<uint64_t> ids;
    QsgProblem problem{};
};

// one domain (xDom = yDom = zDom = 1): MonteCarlo -> QsgProblem
void qsgExport(MonteCarlo* mc, QsgExport& e)
{
    NuclearData& nd = *mc->_nuclearData;
    MaterialDatabase& mdb = *mc->_materialDatabase;
    MC_Domain& dom = mc->domain[0];
    const int G = nd._numEnergyGroups, C = dom.cell_state.size();
    e.pts.resize(C * 14); e.local.resize(72); e.ev.resize(C * 24); e.adj_cell.resize(C * 24);
    e.adj_facet.resize(C * 24); e.mat.resize(C); e.planes.resize(C * 96); e.density.resize(C);
    e.volume.resize(C); e.ids.resize(C);
    for (int i = 0; i < nd._isotopes.size(); ++i) {
        qs_vector<NuclearDataReaction>& rs = nd._isotopes[i]._species[0]._reactions;
        for (int r = 0; r < rs.size(); ++r) {
            e.rtype.push_back(rs[r]._reactionType);   // Scatter 1, Absorption 2, Fission 3 = QSG_REACT_*
            e.nubar.push_back(rs[r]._nuBar);
            for (int g = 0; g < G; ++g) e.xs.push_back(rs[r]._crossSection[g]);
        }
        e.iso_off.push_back(e.rtype.size());
    }
    for (int m = 0; m < mdb._mat.size(); ++m) {
        for (int i = 0; i < mdb._mat[m]._iso.size(); ++i) {
            e.mat_gid.push_back(mdb._mat[m]._iso[i]._gid);
            e.af.push_back(mdb._mat[m]._iso[i]._atomFraction);
        }
        e.mat_off.push_back(e.mat_gid.size());
        e.mass.push_back(mdb._mat[m]._mass);
    }
    for (int v = 0; v < dom.mesh._node.size(); ++v) {
        e.nodes.push_back(dom.mesh._node[v].x);
        e.nodes.push_back(dom.mesh._node[v].y);
        e.nodes.push_back(dom.mesh._node[v].z);
    }
    for (int c = 0; c < C; ++c) {
        MC_Facet_Adjacency_Cell& cc = dom.mesh._cellConnectivity[c];
        for (int p = 0; p < 14; ++p) e.pts[c * 14 + p] = cc._point[p];
        for (int f = 0; f < 24; ++f) {
            MC_General_Plane& pl = dom.mesh._cellGeometry[c]._facet[f];
            double* o = &e.planes[(c * 24 + f) * 4];
            o[0] = pl.A; o[1] = pl.B; o[2] = pl.C; o[3] = pl.D;
            e.ev[c * 24 + f] = cc._facet[f].subfacet.event;   // same numbering as QSG_ADJ_*
            e.adj_cell[c * 24 + f] = cc._facet[f].subfacet.adjacent.cell;
            e.adj_facet[c * 24 + f] = cc._facet[f].subfacet.adjacent.facet;
            if (c == 0)   // facet corners as indices into the cell's 14 points
                for (int k = 0; k < 3; ++k)
                    e.local[f * 3 + k] = std::find(cc._point, cc._point + 14, cc._facet[f].point[k]) - cc._point;
        }
        e.mat[c] = dom.cell_state[c]._material;
        e.density[c] = dom.cell_state[c]._cellNumberDensity;
        e.volume[c] = dom.cell_state[c]._volume;
        e.ids[c] = dom.cell_state[c]._id;
    }
    QsgProblem& p = e.problem;
    p.num_groups = G;                   p.energies = &nd._energies[0];
    p.num_isotopes = nd._isotopes.size();
    p.isotope_reaction_offset = e.iso_off.data(); p.reaction_type = e.rtype.data();
    p.reaction_nubar = e.nubar.data();  p.reaction_xs = e.xs.data();
    p.num_materials = mdb._mat.size();
    p.material_isotope_offset = e.mat_off.data(); p.material_isotope_gid = e.mat_gid.data();
    p.material_atom_fraction = e.af.data();       p.material_mass = e.mass.data();
    p.num_cells = C;                    p.num_nodes = e.nodes.size() / 3;  p.nodes = e.nodes.data();
    p.cell_points = e.pts.data();       p.facet_local_points = e.local.data();
    p.facet_planes = e.planes.data();   p.facet_event = e.ev.data();
    p.facet_adjacent_cell = e.adj_cell.data(); p.facet_adjacent_facet = e.adj_facet.data();
    p.cell_material = e.mat.data();     p.cell_number_density = e.density.data();
    p.cell_volume = e.volume.data();    p.cell_id = e.ids.data();
    p.time_step = mc->time_info->time_step;
}

// ---- the check ------------------------------------------------------------

namespace {

FILE* g_out = nullptr;

// Record: u32 name length, name bytes, u8 dtype ('d' f64, 'q' u64, 'i' i32),
// u64 element count, raw little-endian elements.
void put(const char* name, char dtype, const void* data, uint64_t count)
{
    if (!g_out) return;
    const uint32_t nlen = (uint32_t)strlen(name);
    fwrite(&nlen, 4, 1, g_out);
    fwrite(name, 1, nlen, g_out);
    fwrite(&dtype, 1, 1, g_out);
    fwrite(&count, 8, 1, g_out);
    if (count) fwrite(data, dtype == 'i' ? 4 : 8, count, g_out);
}

}  // namespace

int main(int argc, char** argv)
{
    mpiInit(&argc, &argv);
    Parameters params = getParameters(argc, argv);
    mcco = initMC(params);
    if (mcco->domain.size() != 1) {
        fprintf(stderr, "dropin_harness: %d domains; the export covers one\n", (int)mcco->domain.size());
        return 2;
    }
    QsgExport e;
    qsgExport(mcco, e);
    const QsgProblem& p = e.problem;
    const int rc = qsg_problem_check(&p);
    if (rc != QSG_OK) {
        char msg[1024];
        qsg_last_error(msg, sizeof msg);
        fprintf(stderr, "dropin_harness: qsg_problem_check %d: %s\n", rc, msg);
        return 2;
    }
    const char* path = getenv("QS_DUMP");
    if (path && path[0]) {
        g_out = fopen(path, "wb");
        if (!g_out) { fprintf(stderr, "cannot open %s\n", path); return 1; }
        const uint64_t G = p.num_groups, C = p.num_cells;
        put("energies", 'd', p.energies, G + 1);
        put("isotope_reaction_offset", 'i', p.isotope_reaction_offset, e.iso_off.size());
        put("reaction_type", 'i', p.reaction_type, e.rtype.size());
        put("reaction_nubar", 'd', p.reaction_nubar, e.nubar.size());
        put("reaction_xs", 'd', p.reaction_xs, e.xs.size());
        put("material_isotope_offset", 'i', p.material_isotope_offset, e.mat_off.size());
        put("material_isotope_gid", 'i', p.material_isotope_gid, e.mat_gid.size());
        put("material_atom_fraction", 'd', p.material_atom_fraction, e.af.size());
        put("material_mass", 'd', p.material_mass, e.mass.size());
        put("nodes", 'd', p.nodes, e.nodes.size());
        put("cell_points", 'i', p.cell_points, C * 14);
        put("facet_local_points", 'i', p.facet_local_points, 72);
        put("facet_planes", 'd', p.facet_planes, C * 96);
        put("facet_event", 'i', p.facet_event, C * 24);
        put("facet_adjacent_cell", 'i', p.facet_adjacent_cell, C * 24);
        put("facet_adjacent_facet", 'i', p.facet_adjacent_facet, C * 24);
        put("cell_material", 'i', p.cell_material, C);
        put("cell_number_density", 'd', p.cell_number_density, C);
        put("cell_volume", 'd', p.cell_volume, C);
        put("cell_id", 'q', p.cell_id, C);
        put("time_step", 'd', &p.time_step, 1);
        fclose(g_out);
    }
    printf("dropin_harness: export accepted (%d cells, %d groups, %d isotopes, %d materials)\n",
           p.num_cells, p.num_groups, p.num_isotopes, p.num_materials);
    return 0;
}
