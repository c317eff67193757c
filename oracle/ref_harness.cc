// Test-infrastructure harness around the UNMODIFIED Quicksilver reference.
//
// This file is compiled together with the reference's own sources (see
// oracle/Makefile; the reference's main.cc is built with -Dmain=qs_ref_main so
// that its cycleInit / cycleTracking / cycleFinalize, main.cc:96-324, can be
// driven from here).  It is never linked into the product library.  It exists
// to produce golden vectors from the reference itself:
//
//   * per cycle, the 13 balance counters (Tallies.cc:400-414 order) and the
//     scalar flux per (global cell id, group), read after cycleTracking and
//     before cycleFinalize zeroes them (Tallies.cc:446-467);
//   * the problem tables built by initMC (NuclearData, MaterialDatabase,
//     MC_Domain planes / nodes / adjacency / volumes / ids) indexed by global
//     cell id, so the product's deck-to-table builder can be compared bitwise;
//   * optionally the particles of the processing vaults after cycleInit and
//     the census (processed) particles after cycleTracking;
//   * known-answer vectors of rngSample and rngSpawn_Random_Number_Seed
//     (MC_RNG_State.hh:22-33, MC_RNG_State.cc:106-113);
//   * the cycleTracking wall time (the reference's FOM denominator,
//     MC_Fast_Timer.cc:97-104).
//
// Environment knobs (argv is passed through untouched to getParameters):
//   QS_DUMP=<file>        write the binary dump there (format: see write_arr)
//   QS_DUMP_TABLES=1      include problem tables
//   QS_DUMP_PARTICLES=1   include initial and census particle records
//   QS_ECHO=<file>        write the reference's start-up deck echo there
//                         (QS_ECHO_ONLY=1: then stop)
//   QS_PRINT_SPECTRUM=1   print the energy spectrum file after the last cycle
//   QS_CORAL=1            run coralBenchmarkCorrectness after the last cycle
//   QS_TIMERS=1           print the reference's timer reports to stdout: the
//                         last-cycle table after every cycle (when the deck or
//                         -c sets cycleTimers 1) and the cumulative table
//   QS_INIT_ONLY=1        stop after initMC (which writes the crossSectionsOut
//                         file when the deck or -S names one)
//   Built with -DEXPONENTIAL_TALLY (make -C oracle ref_exp) it also writes,
//   per cycle, the reference's exponential cell tally.
//
//   QS_PORTABLE_MATH=1    (harness built by `make -C oracle ref_pm` only)
//                         from the first cycle on, the reference's log / sin
//                         / cos / sincos calls go to the portable functions
//                         of quicksilver_gb300/csrc/portable_math.h through
//                         the linker's --wrap (oracle/pm_wrap.c); initMC's
//                         table construction keeps the host libm
//   QS_THETA=<file>       cross-section scale factors applied after initMC;
//                         lines "material reactionType gLo gHi factor" with
//                         reactionType 1=scatter 2=absorption 3=fission and
//                         groups [gLo, gHi)

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <fstream>
#include <sstream>

#include "MonteCarlo.hh"
#include "Parameters.hh"
#include "initMC.hh"
#include "Tallies.hh"
#include "NuclearData.hh"
#include "MaterialDatabase.hh"
#include "ParticleVaultContainer.hh"
#include "ParticleVault.hh"
#include "MC_Base_Particle.hh"
#include "MC_RNG_State.hh"
#include "MC_Time_Info.hh"
#include "utilsMpi.hh"
#include "CoralBenchmark.hh"
#include "MC_Fast_Timer.hh"
#include "MC_Processor_Info.hh"
#include "utilsMpi.hh"
#include <omp.h>

extern MonteCarlo* mcco;
// defined only by oracle/pm_wrap.c (the ref_pm build)
extern "C" __attribute__((weak)) int qs_portable_math_on;
void cycleInit(bool loadBalance);
void cycleTracking(MonteCarlo* monteCarlo);
void cycleFinalize();

namespace {

FILE* g_dump = nullptr;

// Record: u32 name length, name bytes, u8 dtype ('d' f64, 'q' u64, 'i' i32),
// u64 element count, raw little-endian elements.
void write_arr(const std::string& name, char dtype, const void* data, uint64_t count)
{
   if (!g_dump) return;
   uint32_t nlen = (uint32_t)name.size();
   fwrite(&nlen, 4, 1, g_dump);
   fwrite(name.data(), 1, nlen, g_dump);
   fwrite(&dtype, 1, 1, g_dump);
   fwrite(&count, 8, 1, g_dump);
   size_t esz = (dtype == 'i') ? 4 : 8;
   if (count) fwrite(data, esz, count, g_dump);
}

void write_d(const std::string& n, const std::vector<double>& v) { write_arr(n, 'd', v.data(), v.size()); }
void write_q(const std::string& n, const std::vector<uint64_t>& v) { write_arr(n, 'q', v.data(), v.size()); }
void write_i(const std::string& n, const std::vector<int32_t>& v) { write_arr(n, 'i', v.data(), v.size()); }

bool env_on(const char* k)
{
   const char* v = getenv(k);
   return v && v[0] && v[0] != '0';
}

int64_t total_cells(const Parameters& p)
{
   return (int64_t)p.simulationParams.nx * p.simulationParams.ny * p.simulationParams.nz;
}

void apply_theta(const char* path)
{
   std::ifstream in(path);
   std::string line;
   MaterialDatabase* mdb = mcco->_materialDatabase;
   NuclearData* nd = mcco->_nuclearData;
   while (std::getline(in, line))
   {
      if (line.empty() || line[0] == '#') continue;
      std::istringstream ss(line);
      std::string mat; int rtype, glo, ghi; double factor;
      if (!(ss >> mat >> rtype >> glo >> ghi >> factor)) continue;
      for (int m = 0; m < mdb->_mat.size(); ++m)
      {
         if (mdb->_mat[m]._name != mat) continue;
         for (int i = 0; i < mdb->_mat[m]._iso.size(); ++i)
         {
            int gid = mdb->_mat[m]._iso[i]._gid;
            qs_vector<NuclearDataReaction>& rs = nd->_isotopes[gid]._species[0]._reactions;
            for (int r = 0; r < rs.size(); ++r)
            {
               if ((int)rs[r]._reactionType != rtype) continue;
               for (int g = glo; g < ghi && g < rs[r]._crossSection.size(); ++g)
                  rs[r]._crossSection[g] *= factor;
            }
         }
      }
   }
}

void dump_tables(const Parameters& params)
{
   NuclearData* nd = mcco->_nuclearData;
   MaterialDatabase* mdb = mcco->_materialDatabase;
   const int G = nd->_numEnergyGroups;

   std::vector<double> energies(nd->_energies.size());
   for (int i = 0; i < nd->_energies.size(); ++i) energies[i] = nd->_energies[i];
   write_d("energies", energies);

   std::vector<int32_t> iso_react_off(1, 0), rtype;
   std::vector<double> nubar, xs;
   for (int iso = 0; iso < nd->_isotopes.size(); ++iso)
   {
      qs_vector<NuclearDataReaction>& rs = nd->_isotopes[iso]._species[0]._reactions;
      for (int r = 0; r < rs.size(); ++r)
      {
         rtype.push_back((int32_t)rs[r]._reactionType);
         nubar.push_back(rs[r]._nuBar);
         for (int g = 0; g < G; ++g) xs.push_back(rs[r]._crossSection[g]);
      }
      iso_react_off.push_back((int32_t)rtype.size());
   }
   write_i("iso_react_off", iso_react_off);
   write_i("reaction_type", rtype);
   write_d("reaction_nubar", nubar);
   write_d("reaction_xs", xs);

   std::vector<int32_t> mat_iso_off(1, 0), mat_iso_gid;
   std::vector<double> mat_iso_af, mat_mass;
   std::string names;
   for (int m = 0; m < mdb->_mat.size(); ++m)
   {
      for (int i = 0; i < mdb->_mat[m]._iso.size(); ++i)
      {
         mat_iso_gid.push_back(mdb->_mat[m]._iso[i]._gid);
         mat_iso_af.push_back(mdb->_mat[m]._iso[i]._atomFraction);
      }
      mat_iso_off.push_back((int32_t)mat_iso_gid.size());
      mat_mass.push_back(mdb->_mat[m]._mass);
      names += mdb->_mat[m]._name + "\n";
   }
   write_i("mat_iso_off", mat_iso_off);
   write_i("mat_iso_gid", mat_iso_gid);
   write_d("mat_iso_af", mat_iso_af);
   write_d("mat_mass", mat_mass);
   std::vector<int32_t> name_bytes(names.begin(), names.end());
   write_i("mat_names", name_bytes);

   const int64_t NC = total_cells(params);
   std::vector<double> volume(NC, 0.0), density(NC, 0.0), planes(NC * 96, 0.0), nodes(NC * 42, 0.0),
      fpts(NC * 24 * 9, 0.0);
   std::vector<int32_t> material(NC, -1), event(NC * 24, -1), adj_facet(NC * 24, -1), owner_domain(NC, -1);
   std::vector<uint64_t> adj_gid(NC * 24, 0);
   for (int d = 0; d < mcco->domain.size(); ++d)
   {
      MC_Domain& dom = mcco->domain[d];
      for (int c = 0; c < dom.cell_state.size(); ++c)
      {
         int64_t gid = (int64_t)(dom.cell_state[c]._id >> 32);
         volume[gid] = dom.cell_state[c]._volume;
         density[gid] = dom.cell_state[c]._cellNumberDensity;
         material[gid] = dom.cell_state[c]._material;
         owner_domain[gid] = d;
         for (int p = 0; p < 14; ++p)
         {
            const MC_Vector& v = dom.mesh._node[dom.mesh._cellConnectivity[c]._point[p]];
            nodes[gid * 42 + p * 3 + 0] = v.x;
            nodes[gid * 42 + p * 3 + 1] = v.y;
            nodes[gid * 42 + p * 3 + 2] = v.z;
         }
         for (int f = 0; f < 24; ++f)
         {
            const MC_General_Plane& pl = dom.mesh._cellGeometry[c]._facet[f];
            planes[gid * 96 + f * 4 + 0] = pl.A;
            planes[gid * 96 + f * 4 + 1] = pl.B;
            planes[gid * 96 + f * 4 + 2] = pl.C;
            planes[gid * 96 + f * 4 + 3] = pl.D;
            const MC_Facet_Adjacency& fa = dom.mesh._cellConnectivity[c]._facet[f];
            for (int k = 0; k < 3; ++k)
            {
               const MC_Vector& v = dom.mesh._node[fa.point[k]];
               fpts[(gid * 24 + f) * 9 + k * 3 + 0] = v.x;
               fpts[(gid * 24 + f) * 9 + k * 3 + 1] = v.y;
               fpts[(gid * 24 + f) * 9 + k * 3 + 2] = v.z;
            }
            event[gid * 24 + f] = (int32_t)fa.subfacet.event;
            adj_facet[gid * 24 + f] = fa.subfacet.adjacent.facet;
            const MC_Domain& adom = mcco->domain[fa.subfacet.adjacent.domain];
            adj_gid[gid * 24 + f] = adom.cell_state[fa.subfacet.adjacent.cell]._id >> 32;
         }
      }
   }
   write_d("cell_volume", volume);
   write_d("cell_density", density);
   write_i("cell_material", material);
   write_i("cell_domain", owner_domain);
   write_d("cell_nodes", nodes);
   write_d("cell_planes", planes);
   write_d("facet_point_coords", fpts);
   write_i("facet_event", event);
   write_i("facet_adj_facet", adj_facet);
   write_q("facet_adj_gid", adj_gid);
   std::vector<double> misc = {mcco->time_info->time_step};
   write_d("time_step", misc);
}

void dump_particles(const std::string& name, bool processing)
{
   ParticleVaultContainer& pvc = *mcco->_particleVaultContainer;
   std::vector<double> d;
   std::vector<uint64_t> q;
   std::vector<int32_t> i;
   uint64_t nv = processing ? pvc.processingSize() : pvc.processedSize();
   for (uint64_t v = 0; v < nv; ++v)
   {
      ParticleVault* vault = processing ? pvc.getTaskProcessingVault(v) : pvc.getTaskProcessedVault(v);
      for (size_t k = 0; k < vault->size(); ++k)
      {
         const MC_Base_Particle& p = (*vault)[k];
         const double dd[12] = {p.coordinate.x, p.coordinate.y, p.coordinate.z,
                                p.velocity.x, p.velocity.y, p.velocity.z,
                                p.kinetic_energy, p.weight, p.time_to_census, p.age,
                                p.num_mean_free_paths, p.num_segments};
         d.insert(d.end(), dd, dd + 12);
         q.push_back(p.random_number_seed);
         q.push_back(p.identifier);
         const int32_t ii[6] = {(int32_t)p.last_event, p.num_collisions, p.breed, p.species, p.domain,
                                (int32_t)(mcco->domain[p.domain].cell_state[p.cell]._id >> 32)};
         i.insert(i.end(), ii, ii + 6);
      }
   }
   write_d(name + "_f64", d);
   write_q(name + "_u64", q);
   write_i(name + "_i32", i);
}

void dump_rng_kat()
{
   std::vector<uint64_t> seeds = {0ULL, 1ULL, 1029384756ULL, 0x0123456789abcdefULL, 0xffffffffffffffffULL,
                                  (uint64_t)7 << 32, ((uint64_t)999 << 32) + 17, 0x8000000000000000ULL};
   std::vector<double> samples;
   std::vector<uint64_t> states, spawned, parent_after;
   for (uint64_t s0 : seeds)
   {
      uint64_t s = s0;
      for (int k = 0; k < 8; ++k)
      {
         samples.push_back(rngSample(&s));
         states.push_back(s);
      }
      uint64_t p = s0;
      spawned.push_back(rngSpawn_Random_Number_Seed(&p));
      parent_after.push_back(p);
   }
   write_q("rng_seeds", seeds);
   write_d("rng_samples", samples);
   write_q("rng_states", states);
   write_q("rng_spawned", spawned);
   write_q("rng_parent_after", parent_after);
}

} // namespace

int main(int argc, char** argv)
{
   mpiInit(&argc, &argv);
   Parameters params = getParameters(argc, argv);
   if (const char* echo = getenv("QS_ECHO"))
   {
      // the reference's start-up echo of the deck (printParameters, Parameters.cc:97-215)
      std::ofstream f(echo);
      printParameters(params, f);
      if (getenv("QS_ECHO_ONLY")) return 0;
   }
   mcco = initMC(params);
   if (getenv("QS_INIT_ONLY")) return 0;   // e.g. for initMC's crossSectionsOut file only
   if (getenv("QS_PORTABLE_MATH")) {
      if (!&qs_portable_math_on) { fprintf(stderr, "QS_PORTABLE_MATH: this harness was not built with pm_wrap.c\n"); return 2; }
      qs_portable_math_on = 1;
   }

   const char* theta = getenv("QS_THETA");
   if (theta && theta[0]) apply_theta(theta);

   const char* dump_path = getenv("QS_DUMP");
   if (dump_path && dump_path[0])
   {
      g_dump = fopen(dump_path, "wb");
      if (!g_dump) { fprintf(stderr, "cannot open %s\n", dump_path); return 1; }
   }
   const bool want_tables = env_on("QS_DUMP_TABLES");
   const bool want_particles = env_on("QS_DUMP_PARTICLES");
   if (want_tables) dump_tables(params);
   dump_rng_kat();

   // the reference's timer reports as main.cc prints them: main timed from
   // here (main.cc:51), Last_Cycle_Report after every cycle (main.cc:61-65,
   // prints only when cycleTimers is 1), Cumulative_Report at the end
   // (main.cc:87-91)
   const bool want_timers = env_on("QS_TIMERS");
   if (want_timers) MC_FASTTIMER_START(MC_Fast_Timer::main);

   const int G = mcco->_nuclearData->_numEnergyGroups;
   const int64_t NC = total_cells(params);
   const int nSteps = params.simulationParams.nSteps;
   std::vector<double> track_seconds;
   uint64_t total_segments = 0;
   for (int cyc = 0; cyc < nSteps; ++cyc)
   {
      cycleInit(bool(params.simulationParams.loadBalance));
      if (want_particles) dump_particles("init_c" + std::to_string(cyc), true);

      auto t0 = std::chrono::steady_clock::now();
      cycleTracking(mcco);
      auto t1 = std::chrono::steady_clock::now();
      track_seconds.push_back(std::chrono::duration<double>(t1 - t0).count());

      Tallies* t = mcco->_tallies;
      std::vector<uint64_t> bal(13, 0);
      for (int r = 0; r < t->GetNumBalanceReplications(); ++r)
      {
         Balance& b = t->_balanceTask[r];
         const uint64_t vals[13] = {b._absorb, b._census, b._escape, b._collision, b._end, b._fission,
                                    b._produce, b._scatter, b._start, b._source, b._rr, b._split,
                                    b._numSegments};
         for (int k = 0; k < 13; ++k) bal[k] += vals[k];
      }
      bal[4] = mcco->_particleVaultContainer->sizeProcessed();  // _end, set by cycleFinalize (main.cc:314)
      write_q("balance_c" + std::to_string(cyc), bal);
      total_segments += bal[12];

      std::vector<double> flux(NC * G, 0.0);
      for (int d = 0; d < mcco->domain.size(); ++d)
      {
         MC_Domain& dom = mcco->domain[d];
         for (int r = 0; r < t->GetNumFluxReplications(); ++r)
         {
            ScalarFluxTask& task = t->_scalarFluxDomain[d]._task[r];
            for (int c = 0; c < dom.cell_state.size(); ++c)
            {
               int64_t gid = (int64_t)(dom.cell_state[c]._id >> 32);
               for (int g = 0; g < G; ++g) flux[gid * G + g] += task._cell[c]._group[g];
            }
         }
      }
      write_d("flux_c" + std::to_string(cyc), flux);
#ifdef EXPONENTIAL_TALLY
      // the exponential cell tally (CycleTracking.cc:48-50), summed over its
      // replications, before cycleFinalize resets it (Tallies.cc:91)
      std::vector<double> cell_tally(NC, 0.0);
      for (int d = 0; d < mcco->domain.size(); ++d)
      {
         MC_Domain& dom = mcco->domain[d];
         for (int r = 0; r < t->GetNumCellTallyReplications(); ++r)
         {
            CellTallyTask& task = t->_cellTallyDomain[d]._task[r];
            for (int c = 0; c < dom.cell_state.size(); ++c)
               cell_tally[(int64_t)(dom.cell_state[c]._id >> 32)] += task._cell[c];
         }
      }
      write_d("cell_tally_c" + std::to_string(cyc), cell_tally);
#endif
      if (want_particles) dump_particles("census_c" + std::to_string(cyc), false);

      cycleFinalize();
      if (want_timers)
         mcco->fast_timer->Last_Cycle_Report(params.simulationParams.cycleTimers, mcco->processor_info->rank,
                                             mcco->processor_info->num_processors,
                                             mcco->processor_info->comm_mc_world);
   }
   if (want_timers)
   {
      MC_FASTTIMER_STOP(MC_Fast_Timer::main);
      mcco->fast_timer->Cumulative_Report(mcco->processor_info->rank, mcco->processor_info->num_processors,
                                          mcco->processor_info->comm_mc_world,
                                          mcco->_tallies->_balanceCumulative._numSegments);
   }
   write_d("track_seconds", track_seconds);
   // the census energy spectrum file (EnergySpectrum.cc:38-59), which the
   // reference's gameOver prints when energySpectrum (-e) is set
   if (getenv("QS_PRINT_SPECTRUM")) mcco->_tallies->_spectrum.PrintSpectrum(mcco);
   // the CORAL2 correctness checks main.cc runs after the cycles (to stdout)
   if (getenv("QS_CORAL")) coralBenchmarkCorrectness(mcco, params);
   double tsum = 0;
   for (double s : track_seconds) tsum += s;
   fprintf(stderr, "qs_ref_harness: segments=%llu tracking_s=%.6f FOM=%.6e seg/s\n",
           (unsigned long long)total_segments, tsum, tsum > 0 ? total_segments / tsum : 0.0);
   if (g_dump) fclose(g_dump);
   return 0;
}
