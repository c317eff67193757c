/*
 * qsg.h -- C ABI of the GB300 cycle-tracking library (libqsg.so).
 *
 * The library replaces the per-vault tracking launch inside Quicksilver's
 * cycleTracking() (main.cc:155-236): CycleTrackingKernel / CycleTrackingGuts
 * (main.cc:126-134, CycleTracking.cc:14-120) and everything they call
 * (MC_Segment_Outcome.cc, MCT.cc, CollisionEvent.cc, NuclearData.cc,
 * MacroscopicCrossSection.cc, MC_Facet_Crossing_Event.cc, Tallies.hh:350-354,
 * ParticleVault.hh:86-93, ParticleVaultContainer.cc:340-400).
 *
 * Conventions
 *   - Every entry point returns int: 0 (QSG_OK) or a QSG_ERR_* code.  The text
 *     of the last error on the calling thread is available from
 *     qsg_last_error().  Nothing throws or aborts across the ABI.  (The
 *     reference's qs_assert only prints and carries on, qs_assert.hh:9-26; this
 *     library reports the same conditions as error codes instead.)
 *   - Plain pointers and sizes only.  Host arrays passed in are read during
 *     the call and may be freed afterwards.
 *   - One thread at a time per handle; handles are independent.
 *   - Calls that take a cudaStream_t-compatible `stream` (passed as void*) are
 *     asynchronous on that stream; everything else is synchronous.
 */
#ifndef QSG_H
#define QSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QSG_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
    QSG_OK = 0,
    QSG_ERR_INVALID = 1,      /* bad argument or malformed problem / deck     */
    QSG_ERR_CUDA = 2,         /* a CUDA runtime call failed                   */
    QSG_ERR_CAPACITY = 3,     /* a particle store is too small                */
    QSG_ERR_DEVICE = 4,       /* the kernel raised its device error flag      */
    QSG_ERR_UNSUPPORTED = 5,  /* feature outside the single-domain hot path   */
    QSG_ERR_IO = 6,           /* file could not be read                       */
    QSG_ERR_NO_DEVICE = 7     /* no CUDA device visible                       */
};

/* Device error flag bits reported by qsg_device_status (QSG_ERR_DEVICE). */
enum {
    QSG_DEV_SEGMENT_LIMIT = 1u << 0,    /* a history exceeded max_segments    */
    QSG_DEV_TRACKING_LIMIT = 1u << 1,   /* 10000 facet retries (MCT.cc:518)   */
    QSG_DEV_NO_REACTION = 1u << 2,      /* reaction sampling found none       */
    QSG_DEV_OFF_PROCESSOR = 1u << 3,    /* Transit_Off_Processor facet hit    */
    QSG_DEV_STORE_OVERFLOW = 1u << 4,   /* census / extra store overflow      */
    QSG_DEV_BAD_FACET = 1u << 5,        /* no facet bounds the particle       */
    QSG_DEV_NEGATIVE_DISTANCE = 1u << 6,/* MC_Segment_Outcome.cc:265-276      */
    QSG_DEV_PASS_LIMIT = 1u << 7,       /* fission products left after max_passes */
    QSG_DEV_SCREEN_MISS = 1u << 8       /* verification build only: the FP32 facet
                                           screen skipped a facet FP64 accepts, or an
                                           integer-pipe conversion or corrected-
                                           reciprocal quotient differed from the
                                           FP64 operation it replaces */
};

/* ---- enums shared with the reference ------------------------------------ */
/* MC_Tally_Event::Enum, Tallies.hh:22-34 (persisted in the particle record). */
enum {
    QSG_EVENT_COLLISION = 0,
    QSG_EVENT_FACET_TRANSIT_EXIT = 1,
    QSG_EVENT_CENSUS = 2,
    QSG_EVENT_FACET_TRACKING_ERROR = 3,
    QSG_EVENT_FACET_ESCAPE = 4,
    QSG_EVENT_FACET_REFLECTION = 5,
    QSG_EVENT_FACET_COMMUNICATION = 6
};
/* MC_Subfacet_Adjacency_Event::Enum, MC_Facet_Adjacency.hh:11-20. */
enum {
    QSG_ADJ_UNDEFINED = 0,
    QSG_ADJ_BOUNDARY_ESCAPE = 1,
    QSG_ADJ_BOUNDARY_REFLECTION = 2,
    QSG_ADJ_TRANSIT_ON_PROCESSOR = 3,
    QSG_ADJ_TRANSIT_OFF_PROCESSOR = 4
};
/* NuclearDataReaction::Enum, NuclearData.hh:33-40. */
enum { QSG_REACT_UNDEFINED = 0, QSG_REACT_SCATTER = 1, QSG_REACT_ABSORPTION = 2, QSG_REACT_FISSION = 3 };

/* Balance counter slots, in the order Tallies::CycleFinalize packs them for
 * its allreduce (Tallies.cc:400-414). */
enum {
    QSG_BAL_ABSORB = 0, QSG_BAL_CENSUS, QSG_BAL_ESCAPE, QSG_BAL_COLLISION, QSG_BAL_END,
    QSG_BAL_FISSION, QSG_BAL_PRODUCE, QSG_BAL_SCATTER, QSG_BAL_START, QSG_BAL_SOURCE,
    QSG_BAL_RR, QSG_BAL_SPLIT, QSG_BAL_NUM_SEGMENTS, QSG_BAL_COUNT
};

/* ---- problem description ------------------------------------------------ */
/*
 * Read-only tables of one spatial domain, as built by initMC
 * (initMC.cc:130-320).  The caller fills it from its own MonteCarlo object
 * (NuclearData, MaterialDatabase, MC_Domain) or from qsg_deck_build().
 * Cell-local node numbering: facet f of cell c uses the nodes
 * cell_points[c*14 + facet_local_points[f*3 + k]] for k = 0,1,2 -- this is how
 * MC_Domain.cc:41-46,292-303 builds facets; facet_local_points is shared by
 * all cells and validated against facet_points when both are given.
 */
typedef struct QsgProblem {
    int32_t num_groups;                 /* G                                  */
    const double* energies;             /* [G+1] group edges (NuclearData.cc:105-119) */

    int32_t num_isotopes;
    const int32_t* isotope_reaction_offset; /* [num_isotopes+1]               */
    const int32_t* reaction_type;       /* [R] QSG_REACT_*                    */
    const double* reaction_nubar;       /* [R]                                */
    const double* reaction_xs;          /* [R*G] microscopic cross sections   */

    int32_t num_materials;
    const int32_t* material_isotope_offset; /* [num_materials+1]              */
    const int32_t* material_isotope_gid;    /* isotope index per entry        */
    const double* material_atom_fraction;   /* per entry                      */
    const double* material_mass;           /* [num_materials]                */

    int32_t num_cells;
    int32_t num_nodes;
    const double* nodes;                /* [num_nodes*3]                      */
    const int32_t* cell_points;         /* [num_cells*14] node indices        */
    const int32_t* facet_local_points;  /* [24*3] indices into a cell's 14 points */
    const double* facet_planes;         /* [num_cells*24*4] A,B,C,D           */
    const int32_t* facet_event;         /* [num_cells*24] QSG_ADJ_*           */
    const int32_t* facet_adjacent_cell; /* [num_cells*24]                     */
    const int32_t* facet_adjacent_facet;/* [num_cells*24]                     */
    const int32_t* cell_material;       /* [num_cells]                        */
    const double* cell_number_density;  /* [num_cells]                        */
    const double* cell_volume;          /* [num_cells]                        */
    const uint64_t* cell_id;            /* [num_cells] MC_Cell_State::_id     */

    double time_step;                   /* MC_Time_Info::time_step            */
} QsgProblem;

/* Structure-of-arrays view of MC_Base_Particle (MC_Base_Particle.hh:75-92).
 * `cell` is the domain-local cell index. */
typedef struct QsgParticleSoA {
    double *x, *y, *z;
    double *vx, *vy, *vz;
    double *kinetic_energy, *weight, *time_to_census, *age, *num_mean_free_paths, *num_segments;
    uint64_t *random_number_seed, *identifier;
    int32_t *last_event, *num_collisions, *breed, *species, *domain, *cell;
} QsgParticleSoA;

/* Tuning and sizing knobs; zero-initialise and set what you need. */
typedef struct QsgOptions {
    int32_t device;              /* CUDA ordinal (default 0)                   */
    int32_t block_size;          /* threads per block for tracking (0 = auto)  */
    int32_t flux_replicas;       /* privatised flux copies (0 = 1)             */
    int32_t balance_replicas;    /* privatised counter copies (0 = 1)          */
    uint64_t particle_capacity;  /* per store (0 = grow on demand)             */
    uint64_t max_segments;       /* per history per launch guard (0 = 2^40)    */
    int32_t max_passes;          /* fission passes per asynchronous cycle (0 = 8) */
    int32_t collision_batch;     /* one-history-per-lane kernel: parked collisions per
                                    warp collision step (0 = 16); the default pool
                                    kernel's thresholds are qsg_set_pool_tuning's */
} QsgOptions;

typedef struct QsgHandle QsgHandle;

/* ---- library ------------------------------------------------------------ */
int qsg_abi_version(void);
/* Copies the last error text of the calling thread (always NUL-terminated). */
int qsg_last_error(char* buf, size_t len);
/* Number of visible CUDA devices (0 when none; never fails on a CPU host). */
int qsg_device_count(int* count);
/* The checks qsg_create makes on a problem before it touches a device (host
 * only): tables present, indices in range, the 24-facet hex-cell convention
 * (MC_Domain.cc:41-46), nuclear data, and the reference's mesh self-test
 * consistencyCheck (initMC.cc:202-234): every facet's neighbour across leads
 * back to it.  QSG_OK, or the first problem found (QSG_ERR_INVALID /
 * QSG_ERR_UNSUPPORTED with a message). */
int qsg_problem_check(const QsgProblem* problem);

/* ---- tracking handle ----------------------------------------------------- */
/* Copies every table into device memory owned by the handle
 * (replaces the UVM placement of initMC.cc:56-62,132-146). */
int qsg_create(const QsgProblem* problem, const QsgOptions* options, QsgHandle** out);
int qsg_destroy(QsgHandle* h);

/* Start a cycle from n host particles (H2D copy): they replace the processing
 * store and the processed (census) store is emptied.  Replaces handing the
 * processing ParticleVaults to CycleTrackingKernel. */
int qsg_set_particles(QsgHandle* h, const QsgParticleSoA* host, uint64_t n);
/* Start a cycle from the census of the previous one without leaving the
 * device: the processed store becomes the processing store
 * (swapProcessingProcessedVaults, ParticleVaultContainer.cc:278-311). */
int qsg_begin_cycle_from_census(QsgHandle* h, uint64_t* n);
/* Number of particles in the processing / processed (census) stores. */
int qsg_sizes(QsgHandle* h, uint64_t* processing, uint64_t* processed);
/* Copy up to `cap` census particles to host arrays (D2H); *n_out = count.
 * Replaces reading the processed ParticleVaults after the launch. */
int qsg_get_census(QsgHandle* h, QsgParticleSoA* host, uint64_t cap, uint64_t* n_out);

/* Track every particle of the processing store to census, escape, absorption
 * or fission; fission products (ParticleVaultContainer::addExtraParticle) are
 * tracked in follow-up passes inside the same call, as cycleTracking's
 * while(!done) loop does (main.cc:155-299).  Census particles are appended to
 * the processed store.  Work is enqueued on `stream` (a cudaStream_t or NULL);
 * the call waits on that stream once per pass to read the remaining count and
 * grow the stores, so it returns when the last pass has been enqueued. */
int qsg_track_cycle(QsgHandle* h, void* stream);
/* Like qsg_track_cycle, but synchronous and reporting the device error flag
 * as QSG_ERR_DEVICE. */
int qsg_track_cycle_sync(QsgHandle* h);
/* Exactly QsgOptions::max_passes passes with no host synchronisation (CUDA
 * graph capturable); the stores must already be large enough
 * (qsg_configure_cycle sizes them).  Fission products still left afterwards
 * raise QSG_DEV_PASS_LIMIT, overflow raises QSG_DEV_STORE_OVERFLOW. */
int qsg_track_cycle_async(QsgHandle* h, void* stream);

/* Balance counters summed over replicas (13 x u64, QSG_BAL_* order) and the
 * scalar flux [num_cells*G] summed over replicas (Tallies.cc:16-23,75-96). */
int qsg_read_tallies(QsgHandle* h, uint64_t* balance, double* flux);
/* Zero counters, flux and, when on, the exponential cell tally
 * (Tallies::CycleFinalize reset, Tallies.cc:63-96). */
int qsg_reset_tallies(QsgHandle* h);
/* Device error flag bits (QSG_DEV_*) raised since the last reset, and clear. */
int qsg_device_status(QsgHandle* h, uint32_t* flags, int clear);

/* ---- whole cycle on the device ------------------------------------------ */
/* Constants of the cycle set-up (SimulationParameters / MaterialParameters,
 * Parameters.hh:45-167). */
typedef struct QsgCycleConfig {
    const double* source_rate;   /* [num_materials] MaterialParameters::sourceRate     */
    uint64_t n_particles;        /* population target, SimulationParameters::nParticles */
    double e_min, e_max;         /* source energy range (MeV)                           */
    double low_weight_cutoff;    /* SimulationParameters::lowWeightCutoff               */
    int32_t load_balance;        /* SimulationParameters::loadBalance                   */
    int32_t reserved;
    uint64_t store_capacity;     /* particles per store (0 = 4 x (n_particles + source)) */
} QsgCycleConfig;
/* Precompute the source (MC_SourceNow.cc:35-64: particle weight and per-cell
 * counts are constant over the run) and size the particle stores.  Needs the
 * problem's cell_volume and cell_id. */
int qsg_configure_cycle(QsgHandle* h, const QsgCycleConfig* config);
/* cycleInit (main.cc:96-121) on the device, asynchronous on `stream`: the
 * previous census becomes the processing store, then MC_SourceNow,
 * PopulationControl and RouletteLowWeightParticles. */
int qsg_cycle_init(QsgHandle* h, void* stream);
/* cycleFinalize (main.cc:310-324), asynchronous: the cycle's 13 counters
 * (END = census count) and scalar-flux total are appended to a device-resident
 * history, then counters, flux and (when on) the exponential cell tally are
 * zeroed (Tallies.cc:25-98). */
int qsg_cycle_finalize(QsgHandle* h, void* stream);
/* Copy history rows [first, first+n): balance [n*13] and flux totals [n]
 * (either may be NULL).  Synchronous. */
int qsg_cycle_history(QsgHandle* h, uint64_t first, uint64_t n, uint64_t* balance, double* flux_total);
/* Copy the processing store (e.g. after qsg_cycle_init) to host arrays. */
int qsg_get_processing(QsgHandle* h, QsgParticleSoA* host, uint64_t cap, uint64_t* n_out);

/* ---- observability: fluence and census energy spectrum ----------------- */
/* Tallies kept across cycles by qsg_cycle_finalize when switched on:
 *   QSG_OBSERVE_FLUENCE   per-cell fluence, the replica-summed scalar flux of
 *     every cycle added group by group to the cell's running total
 *     (Fluence::compute, Tallies.cc:92,100-118; the reference keeps it for the
 *     CORAL2 decks' FluenceTest, CoralBenchmark.cc:177-228);
 *   QSG_OBSERVE_SPECTRUM  per-problem histogram [G+1] of the energy groups of
 *     the particles left in the stores at the end of each cycle (the census;
 *     EnergySpectrum::UpdateSpectrum, EnergySpectrum.cc:12-36). */
enum { QSG_OBSERVE_FLUENCE = 1, QSG_OBSERVE_SPECTRUM = 2 };
/* Switch the tallies in `flags` on (others off); the ones switched on start
 * from zero. */
int qsg_set_observers(QsgHandle* h, int32_t flags);
/* fluence [num_cells], spectrum [problems][G+1] (either may be NULL). */
int qsg_read_observers(QsgHandle* h, double* fluence, uint64_t* spectrum);

/* ---- sensitivities (adjoint / differential-operator tallies) ------------- */
#define QSG_MAX_PARAMS 32
/* K scale parameters theta_k.  Entry e says that theta[param[e]] multiplies
 * the microscopic cross sections of every reaction of type reaction[e]
 * (QSG_REACT_*) of every isotope of material material[e] (the handle's
 * material index: for a batch, problem p's materials start at
 * qsg_material_offsets()[p]) in groups [group_lo[e], group_hi[e]).  One
 * parameter may have several entries (e.g. the same physical parameter in
 * every problem of a batch); entries must not overlap.  The tables given to
 * qsg_create must already be scaled by theta.
 *
 * Each history then carries a score vector S (d log-probability / d theta):
 * a flight of length l in a cell adds -l dSigma_t/dtheta; a collision adds
 * d log Sigma_r / dtheta of the selected reaction; fission products, census
 * and population-control copies inherit their parent's S.  Tallied:
 *   flux_cell[cell]  += l w,  dflux[cell][k] += l w (S_k + [flight ends in a collision] dSigma_t/dtheta_k / Sigma_t)
 *   leak[problem]    += w at escape,  dleak[problem][k] += w S_k at escape
 * (group-summed per-cell flux, leakage and their derivatives).  Forward
 * tracking is unchanged, bit for bit.  No counterpart in the reference, which
 * has no sensitivity tallies. */
typedef struct QsgSensitivity {
    int32_t num_params;          /* K (0 switches sensitivities off)          */
    const double* theta;         /* [K] value of each parameter (> 0)         */
    int32_t num_entries;
    const int32_t* param;        /* [num_entries] parameter index, 0..K-1     */
    const int32_t* material;     /* [num_entries]                             */
    const int32_t* reaction;     /* [num_entries] QSG_REACT_*                 */
    const int32_t* group_lo;     /* [num_entries]                             */
    const int32_t* group_hi;     /* [num_entries]                             */
} QsgSensitivity;
/* num_params == 0 switches the sensitivity tallies off.  Enabling (re)sizes
 * the particle stores to carry K scores per particle (particles already
 * stored keep their records and get zero scores) and zeroes the tallies. */
int qsg_enable_sensitivity(QsgHandle* h, const QsgSensitivity* s);
/* Group-summed track-length flux flux_cell [num_cells] (the forward value
 * whose derivatives dflux holds), dflux [num_cells][K], leak [problems],
 * dleak [problems][K] (any may be NULL), accumulated over every tracking call
 * since the last qsg_reset_sensitivity / qsg_enable_sensitivity (they are not
 * cleared by qsg_cycle_finalize).  qsg_track_particles_noalloc tallies no
 * sensitivities. */
int qsg_read_sensitivity(QsgHandle* h, double* flux_cell, double* dflux, double* leak, double* dleak);
int qsg_reset_sensitivity(QsgHandle* h);
/* [problems + 1] offsets of each problem's materials in the handle. */
int qsg_material_offsets(QsgHandle* h, int32_t* offsets);

/* ---- batches of independent problems ------------------------------------ */
/* One handle over n independent problems (each a single domain; they must
 * share the energy grid, the time step and the facet convention).  Every
 * kernel covers all of them at once; counters and flux stay per problem.
 * Tracking the batch gives each problem exactly what tracking it alone gives
 * (Quicksilver has no such mode: it runs one problem per process). */
int qsg_batch_create(const QsgProblem* problems, int32_t n_problems, const QsgOptions* options, QsgHandle** out);
/* Number of problems and, when cell_offsets is not NULL, the [n+1] offsets of
 * each problem's cells in the handle's flux array. */
int qsg_num_problems(QsgHandle* h, int32_t* n_problems, int32_t* cell_offsets);
/* Per-problem cycle constants (configs[n_problems]); seed_offsets (may be
 * NULL = all 0, the reference's seeding) is added to each problem's source
 * seeds so that problems with identical meshes get distinct streams.
 * qsg_cycle_history then returns [n][n_problems][13] counters and
 * [n][n_problems] flux totals. */
int qsg_configure_cycle_batch(QsgHandle* h, const QsgCycleConfig* configs, const uint64_t* seed_offsets);
/* n whole cycles (init, QsgOptions::max_passes tracking passes, finalize)
 * enqueued on `stream` without host synchronisation; with use_graph each
 * cycle is replayed from a CUDA graph captured on first use (one per role
 * permutation of the three particle stores). */
int qsg_run_cycles(QsgHandle* h, int32_t n_cycles, int32_t use_graph, void* stream);
/* Kernel-shape knobs picked by the autotuner: threads per block of the
 * tracking kernel (128 or 256) and, for the one-history-per-lane kernel,
 * collisions batched per warp step (1-32) and particles claimed per
 * work-queue atomic (1-1024); 0 keeps a value. */
int qsg_set_tuning(QsgHandle* h, int32_t block_size, int32_t collision_batch, int32_t queue_chunk);
/* Tracking kernel: 1 (default) = each warp keeps a pool of 64 particles in
 * shared memory and hands 32 of one kind (segment or collision) to its lanes
 * per step; 0 = one history per lane (collisions batched per warp).  Both
 * give the same results. */
int qsg_set_track_kernel(QsgHandle* h, int32_t kind);
/* Pool-kernel knobs: a collision step runs once this many pooled particles
 * wait at a collision (1-32, default 32; otherwise the larger kind runs), and
 * empty pool slots are refilled from the work queue once this many are empty
 * (1-64, default 16); 0 keeps a value. */
int qsg_set_pool_tuning(QsgHandle* h, int32_t collision_step, int32_t refill);

/* ---- tracking without allocation ---------------------------------------- */
/* No counterpart in the reference (Quicksilver allocates its vaults itself).
 * For callers that cannot let a library call cudaMalloc or cudaFree while
 * they run: a process that has given (nearly) all of the GPU's memory to a
 * pool allocator -- PyTorch's caching allocator, an application arena -- would
 * see such an allocation fail or escape the pool's accounting, and cudaFree
 * synchronises the whole device, stalling the caller's other streams.
 *
 * Tracks the n particles of `particles` (device arrays, read only) through
 * the handle's tables exactly as qsg_track_cycle_sync does, fission passes
 * included, with the tracking kernel qsg_set_track_kernel selects and
 * without sensitivity scores.  Census particles go to `census` (device
 * arrays with room for census_capacity particles; *n_census receives the
 * count); scalar flux is ADDED into `flux` (device, [num_cells * G], the
 * handle's cell numbering) and the balance counters into `balance` (device,
 * [problems * 13], QSG_BAL_* order), so zero them first for fresh tallies.
 * No output may share memory with `particles` or with another output
 * (QSG_ERR_INVALID).  The handle's own stores and tallies are left alone,
 * except the exponential cell tally: with qsg_set_exponential_tally on, the
 * per-segment draw happens here too and its tally adds to the handle's
 * (allocated when it was switched on).  n == 0 returns at once with
 * *n_census = 0.  The call returns when the work on `stream` (a cudaStream_t,
 * or NULL) has finished.
 *
 * Allocates nothing: the fission products handed from one pass to the next
 * live in a fixed array inside the library, two stores of
 * QSG_NOALLOC_MAX_PRODUCTS particles (QSG_NOALLOC_SCRATCH_BYTES in all), which
 * every GPU that loads libqsg.so holds until the process exits.  A pass that
 * makes more fission products than that, or a census beyond census_capacity,
 * ends the call with QSG_ERR_CAPACITY and a message naming the limit; the
 * outputs of that call are then incomplete.  The array's memory is reserved
 * by the CUDA driver when it loads this library's device code on a device
 * (with the default lazy loading: at the first use of the library's kernels
 * there, which qsg_create already makes), never by this call.  The first
 * call in each CUDA context looks up the array's device address
 * (cudaGetSymbolAddress) and later calls reuse it, so make that first call
 * before any stream capture begins -- also after a cudaDeviceReset, which
 * replaces the context and reloads the device code.  Every call on a device shares the
 * one array, and each call clears the parts that must start at zero: calls
 * whose work overlaps on the GPU (other threads, other streams) race on it and
 * must be serialised by the caller. */
#define QSG_NOALLOC_MAX_PRODUCTS 32768
#define QSG_NOALLOC_SCRATCH_BYTES 8913664u /* 256 + 2 x 4456704 */
int qsg_track_particles_noalloc(QsgHandle* h, const QsgParticleSoA* particles, uint64_t n,
                                QsgParticleSoA* census, uint64_t census_capacity, uint64_t* n_census,
                                double* flux, uint64_t* balance, void* stream);

/* No reference counterpart: a self-check of the library's replacements of
 * FP64 operations in the tracking loop, which keep its results bit-identical
 * while moving work off the FP64 pipe -- the double-to-float conversion of the
 * facet screen, the corrected-reciprocal quotient of the mean-free-path
 * update, the bit-pattern comparisons and the random-number sample's
 * integer-to-double conversion -- against the FP64 operations themselves on
 * `n` pseudo-random operands per kind (hard cases mixed in), drawn from
 * `seed`, on CUDA device `device`.  mismatches[0..3] receive the disagreements
 * of the conversion, the quotient, the comparisons and the sample (all zero
 * on a correct build). */
int qsg_check_arithmetic(int32_t device, uint64_t n, uint64_t seed, uint64_t* mismatches);

/* No reference counterpart: log, sin and cos of the n host values x by the
 * portable elementary functions (quicksilver_gb300/csrc/portable_math.h)
 * evaluated on CUDA device `device`, into host arrays.  Those functions use
 * only correctly rounded IEEE operations, so the results must equal a CPU's
 * bit for bit; the library built with them (build.py --portable-math,
 * libqsg_pm.so) then tracks the trajectories the reference tracks when it is
 * linked with the same functions. */
int qsg_portable_math_eval(int32_t device, const double* x, uint64_t n, double* lg, double* sn, double* cs);

/* No reference counterpart: the FP64 issue rate of CUDA device `device`, in
 * FP64 warp instructions per second, measured with independent multiply-add
 * chains at 16 warps per SM (the best of two timed launches).  It is the roof
 * of the tracking loop, whose binding resource is FP64 warp instructions: on
 * this architecture their cost does not depend on how many lanes are active. */
int qsg_measure_fp64_rate(int32_t device, double* warp_instructions_per_second);

/* The reference's -DEXPONENTIAL_TALLY build (CycleTracking.cc:48-50) as a
 * run-time switch: before every segment one random number r is drawn from the
 * particle's stream and exp(r) added to its cell in a per-cell tally
 * (Tallies.hh:357-360, TallyCellValue).  The extra draw moves every later
 * random number, so with it on every result is that build's, not the default
 * build's.  qsg_read_cell_tally copies the tally ([num_cells], this handle's
 * cell order) accumulated since qsg_reset_tallies or the last
 * qsg_cycle_finalize, both of which zero it as the reference's cycleFinalize
 * does (Tallies.cc:91); the reference keeps one copy per cTally replication
 * and sums them there, this library keeps the sum.  Off by default. */
int qsg_set_exponential_tally(QsgHandle* h, int32_t enabled);
int qsg_read_cell_tally(QsgHandle* h, double* cell_tally);

/* Tracks particles that live in the caller's page-locked host arrays
 * (cudaHostAlloc / cudaHostRegister; device arrays work too) without staging
 * copies: the tracking launch reads each particle from `particles` (n of them)
 * and appends each census particle to `census` (room for census_capacity;
 * *n_census receives the count) over the host link while it tracks, so the
 * transfers overlap the tracking.  The replacement, for a host whose vaults
 * live in host memory, of qsg_set_particles + qsg_track_cycle + qsg_get_census
 * (the processing-vault hand-off and census collection around
 * CycleTrackingKernel, main.cc:166-197), with the same results.  Fission
 * products between passes stay in the handle's device stores, whose contents
 * afterwards are unspecified; tallies accumulate in the handle
 * (qsg_read_tallies).  Pageable arrays are rejected (QSG_ERR_INVALID), as is a
 * handle with sensitivities on (QSG_ERR_UNSUPPORTED: scores do not travel
 * through host arrays).  More census particles than census_capacity: the
 * arrays hold the first census_capacity, the call returns QSG_ERR_CAPACITY
 * with the full count in *n_census.  The census arrays must not overlap the
 * particle arrays (particles are still being read while census particles are
 * appended); the particle arrays are only read, so a call can be repeated.
 * Returns when the work on `stream` has finished. */
int qsg_track_host(QsgHandle* h, const QsgParticleSoA* particles, uint64_t n, QsgParticleSoA* census,
                   uint64_t census_capacity, uint64_t* n_census, void* stream);

/* Device pointers of the stores, for zero-copy callers (e.g. torch). */
int qsg_processing_view(QsgHandle* h, QsgParticleSoA* device_view, uint64_t* n);
int qsg_processed_view(QsgHandle* h, QsgParticleSoA* device_view, uint64_t* n);

/* ---- input deck (host only; no CUDA calls) ------------------------------- */
/* Parser for Quicksilver's input-deck format (Parameters.cc:280-493,
 * parseUtils.cc:17-87): blocks Simulation / Geometry / Material /
 * CrossSection with `key: value` lines; unknown keys are ignored;
 * supplyDefaults (Parameters.cc:350-379) applies when no Geometry is given. */
typedef struct QsgDeck QsgDeck;
int qsg_deck_parse_file(const char* path, QsgDeck** out);
int qsg_deck_parse_string(const char* text, QsgDeck** out);
/* Command-line style override of a Simulation key (Parameters.cc:230-255). */
int qsg_deck_set(QsgDeck* deck, const char* key, const char* value);
int qsg_deck_free(QsgDeck* deck);
/* Simulation block values as a flat struct. */
typedef struct QsgSimulation {
    double dt, lx, ly, lz, e_min, e_max, low_weight_cutoff;
    uint64_t n_particles, batch_size, n_batches;
    int32_t n_steps, nx, ny, nz, seed, x_dom, y_dom, z_dom, n_groups;
    int32_t load_balance, balance_replications, flux_replications, cell_replications, coral_benchmark;
    int32_t boundary_condition; /* 0 reflect, 1 escape, 2 octant */
} QsgSimulation;
int qsg_deck_simulation(const QsgDeck* deck, QsgSimulation* out);
/* The Simulation block's energySpectrum value (output file stem, "" when
 * absent; EnergySpectrum.cc:38-59 appends ".dat"). */
int qsg_deck_energy_spectrum(const QsgDeck* deck, char* buf, size_t len);
/* printParameters (Parameters.cc:97-215): the deck as the reference echoes it
 * at start-up (Simulation, Geometry, Material and CrossSection blocks, with
 * every default filled in, text for text).  It reads back as the same deck,
 * except that, as in the reference, a sphere's radius is not printed and
 * inputFile comes from the command line.  *needed receives the size with the
 * terminating NUL; a NULL or short buffer gives QSG_ERR_CAPACITY. */
int qsg_deck_write(const QsgDeck* deck, char* buf, size_t len, size_t* needed);

/* Host-built problem tables (initNuclearData / initMesh restated,
 * initMC.cc:130-320, NuclearData.cc:12-187, MC_Domain.cc:77-394,
 * GlobalFccGrid.cc:17-131) for a single domain covering the whole grid. */
typedef struct QsgHostProblem QsgHostProblem;
int qsg_deck_build(const QsgDeck* deck, QsgHostProblem** out);
int qsg_host_problem_view(const QsgHostProblem* hp, QsgProblem* view);
/* Per-material source rate (MaterialParameters::sourceRate), indexed like
 * QsgProblem materials. */
int qsg_host_problem_source_rates(const QsgHostProblem* hp, double* rates, int32_t n);
/* Scale reaction cross sections: for every isotope of `material`, every
 * reaction of `reaction_type` and groups [g_lo, g_hi): xs *= factor. */
int qsg_host_problem_scale_xs(QsgHostProblem* hp, int32_t material, int32_t reaction_type,
                              int32_t g_lo, int32_t g_hi, double factor);
int qsg_host_problem_free(QsgHostProblem* hp);

#ifdef __cplusplus
}
#endif

#endif /* QSG_H */
