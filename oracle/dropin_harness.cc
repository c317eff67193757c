// Test-infrastructure check of the drop-in adapter a Quicksilver maintainer
// adds to the reference (the table export after initMC that hands the
// library its QsgProblem).  Compiled with the UNMODIFIED reference's own
// sources and linked against libqsg.so by oracle/Makefile (`make dropin`),
// never part of the product.  It
//
//   * builds the reference's MonteCarlo object for a deck (getParameters +
//     initMC, Parameters.cc:80-95, initMC.cc:53-74);
//   * runs qsgExport (oracle/dropin_adapter.hh -- the adapter, the same
//     code the integration guide shows) over it;
//   * validates the export with qsg_problem_check (no GPU needed);
//   * writes every exported array, named after its QsgProblem field, to the
//     file QS_DUMP names (records as oracle/ref_harness.cc writes them), so
//     the tests can compare it with the library's own deck reader;
//   * with QS_VAULTS=1, checks the vault and tally halves of the cycle
//     adapter (qsgGather / qsgScatterCensus / qsgAddTallies) around the
//     reference's own first cycleInit, and dumps the gathered processing
//     particles (p_<field>) and the vault size.
//
// The library calls that need a GPU (qsgAttach, qsgCycleTracking) are
// compiled and linked here but not run.  Exit status: 0 when everything
// passes, 2 when qsg_problem_check rejects the export (the library's message
// on stderr), 3 when a vault or tally check fails.

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "initMC.hh"
#include "utilsMpi.hh"
#include "dropin_adapter.hh"

void cycleInit(bool loadBalance);

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

// The vault and tally halves of qsgCycleTracking on the CPU (the tracking
// call between them needs a GPU): after the reference's own cycleInit, the
// processing vaults gathered into columns, scattered into the processed
// vaults and gathered back must be the same records, no vault above the
// vault size; and counters / flux added through qsgAddTallies must be what
// the reference's Tallies then hold.  Returns the number of failures.
int check_vaults_and_tallies(MonteCarlo* mc, const Parameters& params)
{
    int bad = 0;
    cycleInit(bool(params.simulationParams.loadBalance));
    ParticleVaultContainer& pvc = *mc->_particleVaultContainer;
    QsgColumns in, back;
    const size_t n = qsgGather(pvc, false, in);
    if (n == 0 || pvc.sizeProcessed() != 0) { fprintf(stderr, "unexpected vault sizes\n"); return 1; }
    qsgScatterCensus(in, n, pvc);
    for (uint64_t v = 0; v < pvc.processedSize(); ++v)
        if (pvc.getTaskProcessedVault(v)->size() > pvc.getVaultSize()) { fprintf(stderr, "vault %d over size\n", (int)v); ++bad; }
    if (qsgGather(pvc, true, back) != n) { fprintf(stderr, "census count differs\n"); return bad + 1; }
    for (int f = 0; f < 12; ++f) bad += memcmp(in.d[f].data(), back.d[f].data(), n * 8) != 0;
    for (int f = 0; f < 2; ++f) bad += memcmp(in.q[f].data(), back.q[f].data(), n * 8) != 0;
    for (int f = 0; f < 6; ++f) bad += memcmp(in.i[f].data(), back.i[f].data(), n * 4) != 0;
    if (bad) fprintf(stderr, "vault round trip differs\n");
    put("vault_size", 'q', std::vector<uint64_t>{pvc.getVaultSize()}.data(), 1);
    const char* dnames[12] = {"x", "y", "z", "vx", "vy", "vz", "kinetic_energy", "weight", "time_to_census", "age",
                              "num_mean_free_paths", "num_segments"};
    const char* inames[6] = {"last_event", "num_collisions", "breed", "species", "domain", "cell"};
    for (int f = 0; f < 12; ++f) put((std::string("p_") + dnames[f]).c_str(), 'd', in.d[f].data(), n);
    put("p_random_number_seed", 'q', in.q[0].data(), n);
    put("p_identifier", 'q', in.q[1].data(), n);
    for (int f = 0; f < 6; ++f) put((std::string("p_") + inames[f]).c_str(), 'i', in.i[f].data(), n);

    const int C = g_export.problem.num_cells, G = g_export.problem.num_groups;
    Balance before = mc->_tallies->_balanceTask[0];
    uint64_t bal[QSG_BAL_COUNT];
    for (int k = 0; k < QSG_BAL_COUNT; ++k) bal[k] = 1000 + 17 * k;
    std::vector<double> flux((size_t)C * G);
    double want = mc->_tallies->ScalarFluxSum(mc);
    for (size_t k = 0; k < flux.size(); ++k) { flux[k] = (double)(k % 13); want += flux[k]; }
    qsgAddTallies(mc, bal, flux.data());
    const Balance& b = mc->_tallies->_balanceTask[0];
    const uint64_t got[8] = {b._absorb - before._absorb, b._census - before._census, b._escape - before._escape,
                             b._collision - before._collision, b._fission - before._fission,
                             b._produce - before._produce, b._scatter - before._scatter,
                             b._numSegments - before._numSegments};
    const int slot[8] = {QSG_BAL_ABSORB, QSG_BAL_CENSUS, QSG_BAL_ESCAPE, QSG_BAL_COLLISION, QSG_BAL_FISSION,
                         QSG_BAL_PRODUCE, QSG_BAL_SCATTER, QSG_BAL_NUM_SEGMENTS};
    for (int k = 0; k < 8; ++k)
        if (got[k] != bal[slot[k]]) { fprintf(stderr, "counter slot %d differs\n", slot[k]); ++bad; }
    if (b._start != before._start || b._source != before._source || b._rr != before._rr ||
        b._split != before._split || b._end != before._end) { fprintf(stderr, "population counters touched\n"); ++bad; }
    if (mc->_tallies->ScalarFluxSum(mc) != want) { fprintf(stderr, "flux sum differs\n"); ++bad; }
    return bad;
}

int main(int argc, char** argv)
{
    mpiInit(&argc, &argv);
    Parameters params = getParameters(argc, argv);
    mcco = initMC(params);
    qsgExport(mcco, g_export);   // the rank's domains joined into one mesh
    const QsgProblem& p = g_export.problem;
    const QsgExport& e = g_export;
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
    }
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
    printf("dropin_harness: export accepted (%d domains, %d cells, %d groups, %d isotopes, %d materials)\n",
           (int)mcco->domain.size(), p.num_cells, p.num_groups, p.num_isotopes, p.num_materials);
    int bad = 0;
    if (getenv("QS_VAULTS")) {
        bad = check_vaults_and_tallies(mcco, params);
        printf("dropin_harness: vault round trip and tally hand-over %s\n", bad ? "FAILED" : "ok");
    }
    if (g_out) fclose(g_out);
    return bad ? 3 : 0;
}
