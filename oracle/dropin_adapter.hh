// The reference-side adapter that hands Quicksilver's tracking to libqsg
// (test infrastructure: the same code the integration guide shows, compiled
// here against the UNMODIFIED reference's headers).  Included by exactly one
// translation unit per binary: oracle/dropin_harness.cc (linked against
// libqsg.so) and oracle/dropin_cycle.cc (linked against the CPU stand-in
// oracle/qsg_cpu_standin.c).
//
//   qsgExport / qsgAttach   after initMC (initMC.cc:53-74): the tables
//   qsgCycleTracking        in place of cycleTracking (main.cc:138-307)

#ifndef QSG_DROPIN_ADAPTER_HH
#define QSG_DROPIN_ADAPTER_HH

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "MonteCarlo.hh"
#include "Parameters.hh"
#include "NuclearData.hh"
#include "MaterialDatabase.hh"
#include "MC_Domain.hh"
#include "MC_Time_Info.hh"
#include "MC_Base_Particle.hh"
#include "ParticleVault.hh"
#include "ParticleVaultContainer.hh"
#include "Tallies.hh"
#include "MC_Fast_Timer.hh"
#include <omp.h>

#include "qsg.h"

extern MonteCarlo* mcco;   // main.cc:36; the reference's timer macros name it

// Host copies of the rank's tables in the library's layout; `problem`
// points into them, so it stays valid while the QsgExport lives.  The rank's
// domains are laid end to end as one mesh: domain d's cell c is cell
// cell_offset[d] + c, its node v node node_offset[d] + v.
struct QsgExport {
    std::vector<int32_t> iso_off{0}, rtype, mat_off{0}, mat_gid, pts, local, ev, adj_cell, adj_facet, mat;
    std::vector<double> nubar, xs, af, mass, planes, density, volume, nodes;
    std::vector<uint64_t> ids;
    std::vector<int32_t> cell_offset{0}, cell_domain;   // [domains + 1], [cells]
    QsgProblem problem{};
};

// MonteCarlo -> QsgProblem.  On one rank every neighbouring domain is on the
// processor (MC_Domain.cc:262-268: Transit_On_Processor, the adjacent
// location given as domain index and local cell), and a boundary facet names
// its own cell, so every facet's neighbour is cell_offset[adjacent.domain] +
// adjacent.cell; histories on the joined mesh are the reference's on its
// domains (crossing between them only relabels the particle's domain).
void qsgExport(MonteCarlo* mc, QsgExport& e)
{
    NuclearData& nd = *mc->_nuclearData;
    MaterialDatabase& mdb = *mc->_materialDatabase;
    const int D = mc->domain.size();
    for (int d = 0; d < D; ++d) e.cell_offset.push_back(e.cell_offset.back() + (int)mc->domain[d].cell_state.size());
    const int G = nd._numEnergyGroups, C = e.cell_offset[D];
    e.pts.resize(C * 14); e.local.resize(72); e.ev.resize(C * 24); e.adj_cell.resize(C * 24);
    e.adj_facet.resize(C * 24); e.mat.resize(C); e.planes.resize(C * 96); e.density.resize(C);
    e.volume.resize(C); e.ids.resize(C); e.cell_domain.resize(C);
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
    for (int d = 0; d < D; ++d) {
        MC_Domain& dom = mc->domain[d];
        const int node0 = e.nodes.size() / 3;
        for (int v = 0; v < dom.mesh._node.size(); ++v) {
            e.nodes.push_back(dom.mesh._node[v].x);
            e.nodes.push_back(dom.mesh._node[v].y);
            e.nodes.push_back(dom.mesh._node[v].z);
        }
        for (int lc = 0; lc < (int)dom.cell_state.size(); ++lc) {
            const int c = e.cell_offset[d] + lc;
            MC_Facet_Adjacency_Cell& cc = dom.mesh._cellConnectivity[lc];
            for (int p = 0; p < 14; ++p) e.pts[c * 14 + p] = node0 + cc._point[p];
            for (int f = 0; f < 24; ++f) {
                MC_General_Plane& pl = dom.mesh._cellGeometry[lc]._facet[f];
                double* o = &e.planes[(c * 24 + f) * 4];
                o[0] = pl.A; o[1] = pl.B; o[2] = pl.C; o[3] = pl.D;
                const Subfacet_Adjacency& sf = cc._facet[f].subfacet;
                e.ev[c * 24 + f] = sf.event;   // same numbering as QSG_ADJ_*
                e.adj_cell[c * 24 + f] = e.cell_offset[sf.adjacent.domain] + sf.adjacent.cell;
                e.adj_facet[c * 24 + f] = sf.adjacent.facet;
                if (c == 0)   // facet corners as indices into the cell's 14 points
                    for (int k = 0; k < 3; ++k)
                        e.local[f * 3 + k] = std::find(cc._point, cc._point + 14, cc._facet[f].point[k]) - cc._point;
            }
            e.mat[c] = dom.cell_state[lc]._material;
            e.density[c] = dom.cell_state[lc]._cellNumberDensity;
            e.volume[c] = dom.cell_state[lc]._volume;
            e.ids[c] = dom.cell_state[lc]._id;
            e.cell_domain[c] = d;
        }
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

static QsgHandle* g_qsg = nullptr;
static QsgExport g_export;   // qsg_create copies the tables; the cycle code below reads the counts

void qsgAttach(MonteCarlo* mc)
{
    qsgExport(mc, g_export);
    QsgOptions o{};
    o.flux_replicas = mc->_params.simulationParams.fluxTallyReplications;
    if (qsg_create(&g_export.problem, &o, &g_qsg) != QSG_OK) {
        char e[512]; qsg_last_error(e, sizeof e); printf("%s\n", e);
    }
#ifdef EXPONENTIAL_TALLY   // the reference built with it: the library draws and tallies the same (CycleTracking.cc:48-50)
    if (g_qsg && qsg_set_exponential_tally(g_qsg, 1) != QSG_OK) {
        char e[512]; qsg_last_error(e, sizeof e); printf("%s\n", e);
        qsg_destroy(g_qsg);
        g_qsg = nullptr;
    }
#endif
}

// MC_Base_Particle records (MC_Base_Particle.hh:75-92) as host columns, and
// the QsgParticleSoA view of them.
struct QsgColumns {
    std::vector<double> d[12];
    std::vector<uint64_t> q[2];
    std::vector<int32_t> i[6];
    QsgParticleSoA soa{};
    void resize(size_t n)
    {
        for (auto& v : d) v.resize(n);
        for (auto& v : q) v.resize(n);
        for (auto& v : i) v.resize(n);
        soa = QsgParticleSoA{d[0].data(), d[1].data(), d[2].data(), d[3].data(), d[4].data(), d[5].data(),
                             d[6].data(), d[7].data(), d[8].data(), d[9].data(), d[10].data(), d[11].data(),
                             q[0].data(), q[1].data(), i[0].data(), i[1].data(), i[2].data(), i[3].data(),
                             i[4].data(), i[5].data()};
    }
};

// every particle of a list of vaults -> columns, in vault order
size_t qsgGather(ParticleVaultContainer& pvc, bool processed, QsgColumns& cols)
{
    const uint64_t nv = processed ? pvc.processedSize() : pvc.processingSize();
    cols.resize(processed ? pvc.sizeProcessed() : pvc.sizeProcessing());
    size_t k = 0;
    for (uint64_t v = 0; v < nv; ++v) {
        ParticleVault& vault = *(processed ? pvc.getTaskProcessedVault(v) : pvc.getTaskProcessingVault(v));
        for (size_t j = 0; j < vault.size(); ++j, ++k) {
            const MC_Base_Particle& b = vault[j];
            const double dd[12] = {b.coordinate.x, b.coordinate.y, b.coordinate.z, b.velocity.x, b.velocity.y,
                                   b.velocity.z, b.kinetic_energy, b.weight, b.time_to_census, b.age,
                                   b.num_mean_free_paths, b.num_segments};
            const int32_t ii[6] = {b.last_event, b.num_collisions, b.breed, b.species, b.domain,
                                   g_export.cell_offset[b.domain] + b.cell};   // the joined mesh's cell
            for (int f = 0; f < 12; ++f) cols.d[f][k] = dd[f];
            for (int f = 0; f < 6; ++f) cols.i[f][k] = ii[f];
            cols.q[0][k] = b.random_number_seed;
            cols.q[1][k] = b.identifier;
        }
    }
    return k;
}

// n census particles -> the processed vaults, each filled to the vault size
// (getFirstEmptyProcessedVault, ParticleVaultContainer.cc:111-128)
void qsgScatterCensus(const QsgColumns& cols, size_t n, ParticleVaultContainer& pvc)
{
    size_t k = 0;
    while (k < n) {
        ParticleVault& vault = *pvc.getTaskProcessedVault(pvc.getFirstEmptyProcessedVault());
        for (; k < n && vault.size() < pvc.getVaultSize(); ++k) {
            MC_Base_Particle b;
            b.coordinate = MC_Vector(cols.d[0][k], cols.d[1][k], cols.d[2][k]);
            b.velocity = MC_Vector(cols.d[3][k], cols.d[4][k], cols.d[5][k]);
            b.kinetic_energy = cols.d[6][k];        b.weight = cols.d[7][k];
            b.time_to_census = cols.d[8][k];        b.age = cols.d[9][k];
            b.num_mean_free_paths = cols.d[10][k];  b.num_segments = cols.d[11][k];
            b.random_number_seed = cols.q[0][k];    b.identifier = cols.q[1][k];
            b.last_event = (MC_Tally_Event::Enum)cols.i[0][k];
            b.num_collisions = cols.i[1][k];  b.breed = cols.i[2][k];   b.species = cols.i[3][k];
            // the joined mesh's cell -> its domain and the cell within it (the
            // domain a Transit_On_Processor crossing sets, MC_Facet_Crossing_Event.cc:29-34)
            b.domain = g_export.cell_domain[cols.i[5][k]];
            b.cell = cols.i[5][k] - g_export.cell_offset[b.domain];
            vault.pushBaseParticle(b);
        }
    }
}

// one cycle's counters (QSG_BAL_* order) and flux [cell][group] -> the
// first balance and flux replicas, which the reference sums over replicas
// at cycle finalize (Tallies.cc:16-23, 146-171)
void qsgAddTallies(MonteCarlo* mc, const uint64_t* bal, const double* flux)
{
    Balance& b = mc->_tallies->_balanceTask[0];
    b._absorb += bal[QSG_BAL_ABSORB];       b._census += bal[QSG_BAL_CENSUS];
    b._escape += bal[QSG_BAL_ESCAPE];       b._collision += bal[QSG_BAL_COLLISION];
    b._fission += bal[QSG_BAL_FISSION];     b._produce += bal[QSG_BAL_PRODUCE];
    b._scatter += bal[QSG_BAL_SCATTER];     b._numSegments += bal[QSG_BAL_NUM_SEGMENTS];
    const int G = g_export.problem.num_groups;
    for (int d = 0; d + 1 < (int)g_export.cell_offset.size(); ++d) {
        ScalarFluxTask& t = mc->_tallies->_scalarFluxDomain[d]._task[0];
        for (int c = g_export.cell_offset[d]; c < g_export.cell_offset[d + 1]; ++c)
            for (int g = 0; g < G; ++g) t._cell[c - g_export.cell_offset[d]]._group[g] += flux[(size_t)c * G + g];
    }
}

#ifdef EXPONENTIAL_TALLY
// the cycle's exponential cell tally [cell] -> the first cell-tally replica
// (Tallies.hh:126-165), which cycleFinalize resets (Tallies.cc:91)
void qsgAddCellTally(MonteCarlo* mc, const double* cell_tally)
{
    for (int d = 0; d + 1 < (int)g_export.cell_offset.size(); ++d) {
        CellTallyTask& t = mc->_tallies->_cellTallyDomain[d]._task[0];
        for (int c = g_export.cell_offset[d]; c < g_export.cell_offset[d + 1]; ++c)
            t._cell[c - g_export.cell_offset[d]] += cell_tally[c];
    }
}
#endif

// replaces cycleTracking (main.cc:138-307): the processing vaults tracked in
// one call, fission products included; census particles land in the
// processed vaults and the cycle's tallies in the reference's Tallies
void qsgCycleTracking(MonteCarlo* mc)
{
    MC_FASTTIMER_START(MC_Fast_Timer::cycleTracking);   // the figure of merit's denominator
    static QsgColumns in, census;
    ParticleVaultContainer& pvc = *mc->_particleVaultContainer;
    const size_t n = qsgGather(pvc, false, in);
    uint64_t n_processing = 0, n_census = 0, bal[QSG_BAL_COUNT];
    std::vector<double> flux((size_t)g_export.problem.num_cells * g_export.problem.num_groups);
    MC_FASTTIMER_START(MC_Fast_Timer::cycleTracking_Kernel);
    int rc = qsg_set_particles(g_qsg, &in.soa, n);
    if (rc == QSG_OK) rc = qsg_track_cycle_sync(g_qsg);
    if (rc == QSG_OK) rc = qsg_sizes(g_qsg, &n_processing, &n_census);
    if (rc == QSG_OK) { census.resize(n_census); rc = qsg_get_census(g_qsg, &census.soa, n_census, &n_census); }
    if (rc == QSG_OK) rc = qsg_read_tallies(g_qsg, bal, flux.data());
#ifdef EXPONENTIAL_TALLY
    std::vector<double> cell_tally(g_export.problem.num_cells);
    if (rc == QSG_OK) rc = qsg_read_cell_tally(g_qsg, cell_tally.data());
#endif
    if (rc == QSG_OK) rc = qsg_reset_tallies(g_qsg);
    MC_FASTTIMER_STOP(MC_Fast_Timer::cycleTracking_Kernel);
    if (rc != QSG_OK) { char e[512]; qsg_last_error(e, sizeof e); printf("%s\n", e); }
    for (uint64_t v = 0; v < pvc.processingSize(); ++v) pvc.getTaskProcessingVault(v)->clear();
    if (rc == QSG_OK) {
        qsgScatterCensus(census, n_census, pvc);
        qsgAddTallies(mc, bal, flux.data());
#ifdef EXPONENTIAL_TALLY
        qsgAddCellTally(mc, cell_tally.data());
#endif
    }
    MC_FASTTIMER_STOP(MC_Fast_Timer::cycleTracking);
}

#endif
