/*
 * qs_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of Quicksilver's cycle (source, population control,
 * roulette, and the cycle-tracking hot path) used as the checker for the
 * CUDA library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  It is pinned against the reference itself:
 * tests/golden/ holds vectors produced by the unmodified reference
 * (oracle/ref_harness.cc, built by `make -C oracle ref`), and the tests check
 * this oracle reproduces them (balance counters bit for bit, flux and census
 * particle states to the last bit on the same host).
 */
#ifndef QS_ORACLE_H
#define QS_ORACLE_H

#include <stdint.h>
#include "qsg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Same fields and order as MC_Base_Particle (MC_Base_Particle.hh:75-92):
 * 12 doubles, 2 uint64, 6 int32 = 136 bytes. */
typedef struct OracleParticle {
    double x, y, z, vx, vy, vz;
    double kinetic_energy, weight, time_to_census, age, num_mean_free_paths, num_segments;
    uint64_t random_number_seed, identifier;
    int32_t last_event, num_collisions, breed, species, domain, cell;
} OracleParticle;

typedef struct OracleRun OracleRun;

/* Keeps pointers into `problem` and `source_rate` (the caller keeps them alive). */
OracleRun* oracle_create(const QsgProblem* problem, const double* source_rate,
                         uint64_t n_particles, double e_min, double e_max,
                         double low_weight_cutoff, int load_balance);
void oracle_destroy(OracleRun* run);
/* An offset added to every source seed (MC_SourceNow.cc:90-97 adds the cell's
 * _id to its source tally; this adds `offset` on top), giving an independent
 * replica of the same problem as the library's per-problem seed offsets do.
 * 0, the default, is the reference's seeding.  Call before the first cycle. */
void oracle_set_seed_offset(OracleRun* run, uint64_t offset);
/* Process-wide: 1 = the tracking path's log / sin / cos are the portable
 * functions of quicksilver_gb300/csrc/portable_math.h (as in the GPU
 * library's portable-math build and the reference built with `make -C oracle
 * ref_pm`); 0 (default) = the host libm's, as the reference uses them. */
void oracle_use_portable_math(int on);
/* log, sin and cos of x[0..n) by the portable functions. */
void oracle_pm_eval(const double* x, uint64_t n, double* lg, double* sn, double* cs);

/* cycleInit (main.cc:96-121): swap census into processing, MC_SourceNow,
 * PopulationControl, RouletteLowWeightParticles. */
int oracle_cycle_init(OracleRun* run);
/* cycleTracking (main.cc:138-307) with `nthreads` OpenMP threads (0 = all). */
int oracle_cycle_tracking(OracleRun* run, int nthreads);
/* cycleFinalize (main.cc:310-324): records _end, keeps the finished cycle's
 * counters for oracle_last_balance, resets counters and flux. */
int oracle_cycle_finalize(OracleRun* run);

uint64_t oracle_num_processing(const OracleRun* run);
uint64_t oracle_num_processed(const OracleRun* run);
const OracleParticle* oracle_processing(const OracleRun* run);
const OracleParticle* oracle_processed(const OracleRun* run);
int oracle_set_processing(OracleRun* run, const OracleParticle* p, uint64_t n);
/* Current counters (13, QSG_BAL_* order) and flux [num_cells*G]. */
void oracle_balance(const OracleRun* run, uint64_t* out13);
const double* oracle_flux(const OracleRun* run);
/* Counters of the cycle most recently finalised. */
void oracle_last_balance(const OracleRun* run, uint64_t* out13);
/* Warnings the reference would print and continue from (qs_assert). */
uint64_t oracle_warning_count(const OracleRun* run);

/* Sensitivity (differential-operator) scores, restating what the CUDA
 * library's sensitivity tallies compute (qsg_enable_sensitivity in qsg.h; the
 * reference has no such capability).  Parameter k scales the cross sections
 * of reaction type reaction[k] of every isotope of material[k] in groups
 * [group_lo[k], group_hi[k]).  Outputs are accumulated: flux_cell [C],
 * dflux [C*K], leak [1], dleak [K]. */
typedef struct OracleSens {
    int32_t K;
    int32_t material[QSG_MAX_PARAMS], reaction[QSG_MAX_PARAMS];
    int32_t group_lo[QSG_MAX_PARAMS], group_hi[QSG_MAX_PARAMS];
    double theta[QSG_MAX_PARAMS];
    double* flux_cell;
    double* dflux;
    double* leak;
    double* dleak;
} OracleSens;

/* Switch a run's sensitivity tallies on (before its first cycle); the run
 * copies the parameters and owns the output arrays. */
int oracle_enable_sensitivity(OracleRun* run, const OracleSens* spec);
/* Accumulated flux_cell [C], dflux [C*K], leak [1], dleak [K] (any may be NULL). */
int oracle_read_sensitivity(const OracleRun* run, double* flux_cell, double* dflux, double* leak, double* dleak);
/* Scores [n*K] of the processing / processed particles (row per particle). */
const double* oracle_processing_scores(const OracleRun* run);
const double* oracle_processed_scores(const OracleRun* run);

/* One-shot tracking with sensitivity scores: in_scores [n*K] (NULL: zero),
 * census_scores [cap*K] (may be NULL); tallies accumulate into sens's outputs. */
int oracle_track_sens(const QsgProblem* problem, OracleSens* sens, const OracleParticle* in, const double* in_scores,
                      uint64_t n, OracleParticle* census_out, double* census_scores, uint64_t cap, uint64_t* n_census,
                      uint64_t* balance13, double* flux, int nthreads);

/* One-shot tracking of a particle set (no cycle init): census particles go to
 * census_out (capacity cap), counters and flux accumulate into the outputs
 * (flux must hold num_cells*G doubles, zeroed by the caller). */
int oracle_track(const QsgProblem* problem, const OracleParticle* in, uint64_t n,
                 OracleParticle* census_out, uint64_t cap, uint64_t* n_census,
                 uint64_t* balance13, double* flux, int nthreads);

/* The reference built with -DEXPONENTIAL_TALLY (CycleTracking.cc:48-50):
 * before every segment a random number r is drawn from the particle's stream
 * and exp(r) added to the particle's cell in a per-cell tally
 * (Tallies.hh:357-360), which cycleFinalize resets (Tallies.cc:91).
 * oracle_enable_exponential_tally switches a run to that build's behaviour;
 * oracle_read_cell_tally copies the current tally ([num_cells]).
 * oracle_track_cell_tally is oracle_track with it (cell_tally NULL: off;
 * otherwise num_cells doubles, added to). */
int oracle_enable_exponential_tally(OracleRun* run);
int oracle_read_cell_tally(const OracleRun* run, double* out);
int oracle_track_cell_tally(const QsgProblem* problem, const OracleParticle* in, uint64_t n,
                            OracleParticle* census_out, uint64_t cap, uint64_t* n_census,
                            uint64_t* balance13, double* flux, double* cell_tally, int nthreads);

/* FP64 operations and elementary-function calls of the tracking path since
 * the last reset (out2[0], out2[1]), counted as the reference writes them
 * (qs_oracle.c states the rules): the algorithm's FP64 work per segment. */
void oracle_flop_counts(uint64_t* out2);
void oracle_reset_flop_counts(void);

/* MC_RNG_State restated (MC_RNG_State.hh:22-33, MC_RNG_State.cc:29-113). */
double oracle_rng_sample(uint64_t* seed);
uint64_t oracle_rng_spawn(uint64_t* parent_seed);

#ifdef __cplusplus
}
#endif

#endif
