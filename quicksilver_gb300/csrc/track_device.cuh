// Device-side history tracking for one spatial domain.
//
// Every routine reproduces the reference's floating-point expression order
// (the library is compiled with --fmad=false, so each * and + rounds on its
// own exactly as the reference's CPU build does).  Comments name the
// reference lines each step follows.
#pragma once

#include <cooperative_groups.h>

#include <cstdint>

#include "portable_math.h"
#include "qsg.h"

// The tracking path's elementary functions: the CUDA math library's, or with
// -DQSG_PORTABLE_MATH (build.py --portable-math, libqsg_pm.so) the portable
// ones of portable_math.h, which the oracle and the reference can use too.
#ifdef QSG_PORTABLE_MATH
#define QSG_LOG(x) qsg_log(x)
#define QSG_SINCOS(x, s, c) qsg_sincos((x), (s), (c))
#define QSG_SIN(x) qsg_sin(x)
#define QSG_COS(x) qsg_cos(x)
#else
#define QSG_LOG(x) log(x)
#define QSG_SINCOS(x, s, c) sincos((x), (s), (c))
#define QSG_SIN(x) sin(x)
#define QSG_COS(x) cos(x)
#endif

namespace qsg {

// PhysicalConstants.hh:9-16
constexpr double kNeutronRestMassEnergy = 9.395656981095e+2;
constexpr double kPi = 3.1415926535897932;
constexpr double kSpeedOfLight = 2.99792458e+10;
constexpr double kTinyDouble = 1.0e-13;
constexpr double kSmallDouble = 1.0e-10;
constexpr double kHugeDouble = 1.0e+75;

constexpr int kFacets = 24;
// Tracking-kernel shape (tuned on GB300; QSG_* macros override for sweeps)
#ifndef QSG_MIN_BLOCKS
#define QSG_MIN_BLOCKS 3
#endif
#ifndef QSG_COLLISION_BATCH
#define QSG_COLLISION_BATCH 16
#endif
constexpr int kTrackBlock = 128;                       // threads per block
constexpr int kTrackMinBlocks = QSG_MIN_BLOCKS;        // resident blocks per SM the registers must allow
constexpr int kCollisionBatch = QSG_COLLISION_BATCH;   // parked collisions that trigger a warp's collision step
constexpr int kCellPoints = 14;

// Corners of the 24 triangular facets as indices into a cell's 14 points:
// the mesh convention of the reference (MC_Domain.cc:41-46), which fixes facet
// numbering and therefore tie-breaks.  qsg_create checks the problem's table
// against it.
static __constant__ int8_t kFacetLocal[kFacets][3] = {
    {1, 3, 8}, {3, 7, 8}, {7, 5, 8}, {5, 1, 8},  {0, 4, 9},  {4, 6, 9},  {6, 2, 9},  {2, 0, 9},
    {3, 2, 10}, {2, 6, 10}, {6, 7, 10}, {7, 3, 10}, {0, 1, 11}, {1, 5, 11}, {5, 4, 11}, {4, 0, 11},
    {4, 5, 12}, {5, 7, 12}, {7, 6, 12}, {6, 4, 12}, {0, 2, 13}, {2, 3, 13}, {3, 1, 13}, {1, 0, 13}};
static const int8_t kFacetLocalHost[kFacets][3] = {
    {1, 3, 8}, {3, 7, 8}, {7, 5, 8}, {5, 1, 8},  {0, 4, 9},  {4, 6, 9},  {6, 2, 9},  {2, 0, 9},
    {3, 2, 10}, {2, 6, 10}, {6, 7, 10}, {7, 3, 10}, {0, 1, 11}, {1, 5, 11}, {5, 4, 11}, {4, 0, 11},
    {4, 5, 12}, {5, 7, 12}, {7, 6, 12}, {6, 4, 12}, {0, 2, 13}, {2, 3, 13}, {3, 1, 13}, {1, 0, 13}};

// Structure-of-arrays particle store in device memory (136 B per particle,
// the MC_Base_Particle fields).  `count` lives in device memory so kernels
// can append with atomics.
struct DevStore {
    double *x, *y, *z, *vx, *vy, *vz;
    double *kinetic_energy, *weight, *time_to_census, *age, *num_mean_free_paths, *num_segments;
    uint64_t *seed, *identifier;
    int32_t *last_event, *num_collisions, *breed, *species, *domain, *cell;
    double* score;          // [score_fields][capacity] sensitivity scores (null: none)
    int32_t score_fields;
    unsigned long long* count;
    uint64_t capacity;
};

// Sensitivity tables and tallies (qsg_enable_sensitivity).
struct DevSens {
    int32_t K;                 // parameters (0: sensitivities off)
    const int16_t* param_of;   // [classes][G][3] parameter of (class, group, reaction type - 1), or -1
    const double* dsig;        // [classes][G][3] dSigma_t/dtheta contributed by that reaction type
    const double* inv_theta;   // [K] d log Sigma_r / dtheta for a reaction the parameter scales
    double* flux_cell;         // [C] group-summed track-length flux (the differentiated forward tally)
    double* dflux;             // [C][K]
    double* leak;              // [problems]
    double* dleak;             // [problems][K]
};

// Read-only problem tables in device memory.
struct DevTables {
    int32_t num_groups;            // G
    int32_t num_cells;
    int32_t max_reactions;         // K: reactions per cross-section class row
    const double* energies;        // [G+1]
    const double* sigma_total;     // [classes][G]  weightedMacroscopicCrossSection values
    const double* mfp_table;       // [classes][G]  1/Sigma_t, or _hugeDouble when Sigma_t = 0 (MC_Segment_Outcome.cc:129-131)
    const double* inv_mfp_table;   // [classes][G]  RN(1 / mfp_table), for div_rn
    // energy-group hint for log-spaced grids: group ~ (ln E - ln E_0) * scale
    // (scale = 0: no hint); the exact search below confirms it
    float group_hint_ln0, group_hint_scale;
    const double* macro_xs;        // [classes][G][K] macroscopicCrossSection per (iso, reaction)
    const int32_t* class_num_reactions;  // [classes]
    const int32_t* class_material;       // [classes]
    const int8_t* class_reaction_type;   // [classes][K]
    const double* class_reaction_nubar;  // [classes][K]
    const double* material_inv_mass;     // [materials] 1.0 / MaterialDatabase mass
    const int32_t* cell_class;     // [C]
    const double* cell_nodes;      // [C][14][3]
    const double* cell_center;     // [C][3] MCT_Cell_Position_3D_G
    const double* planes;          // [C][24][4]
    const int32_t* adj_cell;       // [C][24]
    const uint8_t* adj_facet_event;// [C][24] facet | (event << 5)
    double time_step;
    // FP32 pre-filter of the facet search, in cell-local coordinates
    // (origin at cell_center): each hex face's plane (A, B, C, D + A cx + B cy
    // + C cz) rounded to float, with per-cell bounds on how far the face's
    // four facets' FP64 planes differ from it, node coordinates minus the
    // centre rounded to float, and the projection the FP64 inside test uses
    // for each facet (u | v << 2, or 0xff when no normal component exceeds
    // 0.5 in magnitude).
    const float4* face32;          // [C][6]
    const float2* face_slack;      // [C] (normal, offset)
    const float* node32;           // [C][14][3]
    const uint8_t* proj;           // [C][24]
    double abs_slack;              // bound on FP64 rounding of global-coordinate quantities
};

struct DevTally {
    double* flux;                  // [replicas][C][G]
    unsigned long long* balance;   // [replicas][problems][QSG_BAL_COUNT]
    unsigned int* error_flags;
    const int32_t* cell_problem;   // [C] problem of each cell (null: one problem)
    int32_t num_problems;
    int32_t flux_replicas;
    int32_t balance_replicas;
    int32_t collision_batch;       // parked collisions that trigger a warp's collision step
    int32_t queue_chunk;           // consecutive particles a lane claims per work-queue atomic
    int32_t pool_collision_step;   // pool kernel: parked collisions that make a collision step (1-32)
    int32_t pool_refill;           // pool kernel: empty slots that trigger a refill from the queue (1-64)
    uint64_t max_segments;
    double* cell_tally;            // [C] exponential cell tally (the reference's EXPONENTIAL_TALLY build); null: off
};

// Problems whose counters a tracking block accumulates in shared memory
// before one global flush; larger batches add to global memory directly.
constexpr int kSmemProblems = 256;

__device__ __forceinline__ void raise_flag(const DevTally& tally, unsigned int bit)
{
    atomicOr(tally.error_flags, bit);
}

// Reserve one slot of `s` for each calling lane with one atomic per warp.
__device__ __forceinline__ uint64_t append_slot(const DevStore& s)
{
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(s.count, (unsigned long long)g.size());
    base = g.shfl(base, 0);
    return base + g.thread_rank();
}

// IEEE 754 comparisons of doubles evaluated on their bit patterns, for
// operands that are never NaN.  They answer as the FP64 comparisons do (-0.0
// equals +0.0) but run on the integer pipe: the tracking loop keeps the FP64
// pipe busy, where a comparison costs as much as a multiply.
__device__ __forceinline__ long long f64_bits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool f64_gt0(double x) { return f64_bits(x) > 0; }    // x > 0.0
__device__ __forceinline__ bool f64_lt0(double x)                                // x < 0.0
{
    return (unsigned long long)f64_bits(x) > 0x8000000000000000ull;
}
__device__ __forceinline__ bool f64_eq0(double x) { return ((unsigned long long)f64_bits(x) << 1) == 0; }
// x == c for a nonzero c
__device__ __forceinline__ bool f64_eq(double x, double c) { return f64_bits(x) == f64_bits(c); }
// a key whose signed order is the IEEE order (-0.0 and +0.0 share key 0)
__device__ __forceinline__ long long f64_key(double x)
{
    const long long b = f64_bits(x);
    return b >= 0 ? b : (long long)(0x8000000000000000ull - (unsigned long long)b);
}
__device__ __forceinline__ bool f64_lt(double a, double b) { return f64_key(a) < f64_key(b); }
__device__ __forceinline__ bool f64_le(double a, double b) { return f64_key(a) <= f64_key(b); }

// double -> float rounded to nearest even on the integer pipe: the 29
// dropped mantissa bits are rounded into the kept ones by one 64-bit add
// (a carry may step the exponent, as rounding does), then the exponent is
// rebiased from 1023 to 127 and the fields shifted into place.  The same
// value as (float)x for every x whose rounded magnitude is at least 2^-126
// and below 2^128; smaller magnitudes give a zero of x's sign (an error
// below 2^-126).
__device__ __forceinline__ float f64_to_f32_rn(double x)
{
    unsigned long long b = (unsigned long long)f64_bits(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    b += 0x0fffffffull + ((b >> 29) & 1ull);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned f = __funnelshift_l(lo, hi - 0x38000000u, 3);
    return __uint_as_float(((hi & 0x7fffffffu) < 0x38100000u) ? sign : (f | sign));
}

// a / b correctly rounded (round to nearest), given y = RN(1 / b): Markstein's
// correction (P. Markstein, IBM J. Res. Dev. 34(1), 1990; Muller et al.,
// Handbook of Floating-Point Arithmetic, the theorem on division with a
// correctly rounded reciprocal).  q0 = RN(a y) is within 1.5 ulp of a/b; one
// correction makes q1 faithful; for a faithful q1 and a reciprocal with
// relative error below 2^-53, RN(q1 + (a - b q1) y) equals RN(a / b).  Three
// FP64 multiply-adds and one multiply instead of a division, for normal
// operands whose residuals do not underflow (a = 0 gives +0 as a / b does).
__device__ __forceinline__ double div_rn(double a, double b, double y)
{
    const double q0 = a * y;
    const double q1 = fma(fma(-q0, b, a), y, q0);
    return fma(fma(-q1, b, a), y, q1);
}

// 2^-64 * (double)x with the conversion rounded to nearest even, assembled on
// the integer pipe: the leading bit is found, the 64 - 53 = 11 low bits are
// rounded into the kept ones (a carry steps the exponent, as rounding does),
// and the 2^-64 scale goes into the exponent (exact: no result is subnormal).
__device__ __forceinline__ double u64_scaled_2m64(uint64_t x)
{
    if (x == 0) return 0.0;
    const int lz = __clzll((long long)x);
    const uint64_t m = x << lz;   // leading 1 at bit 63
    const uint64_t round_up = (m >> 10) & 1ull & ((uint64_t)((m & 0x3ffull) != 0) | (m >> 11));
    const uint64_t r = (m >> 11) + round_up;   // 2^52 <= r <= 2^53
    return __longlong_as_double((long long)(((uint64_t)(1022 - lz) << 52) + r - (1ull << 52)));
}

// MC_RNG_State.hh:22-33.  The reference's 5.4210108624275222e-20 is 2^-64
// exactly, so the sample is u64_scaled_2m64 of the new seed (same bits).
static_assert(5.4210108624275222e-20 == 0x1p-64, "the sample scale is 2^-64");
__device__ __forceinline__ double rng_sample(uint64_t& seed)
{
    seed = 2862933555777941757ULL * seed + 3037000493ULL;
    return u64_scaled_2m64(seed);
}

// Numerical Recipes psdes (2 rounds) as MC_RNG_State.cc:29-52, used by
// rngSpawn_Random_Number_Seed (MC_RNG_State.cc:106-113).
__device__ __forceinline__ uint64_t rng_spawn(uint64_t& parent)
{
    const uint32_t c1[2] = {0xbaa96887u, 0x1e17d32cu};
    const uint32_t c2[2] = {0x4b0f3b58u, 0xe874f0c3u};
    uint32_t lword = (uint32_t)(parent >> 32);
    uint32_t irword = (uint32_t)(parent & 0xffffffffu);
#pragma unroll
    for (int i = 0; i < 2; i++) {
        uint32_t iswap = irword;
        uint32_t ia = iswap ^ c1[i];
        uint32_t lo = ia & 0xffffu;
        uint32_t hi = ia >> 16;
        uint32_t ib = lo * lo + ~(hi * hi);
        ia = (ib >> 16) | ((ib & 0xffffu) << 16);
        irword = lword ^ ((ia ^ c2[i]) + lo * hi);
        lword = iswap;
    }
    uint64_t spawned = ((uint64_t)lword << 32) | (uint64_t)irword;
    rng_sample(parent);
    return spawned;
}

// NuclearData::getEnergyGroup, NuclearData.cc:207-228
__device__ __forceinline__ int energy_group(const DevTables& t, double e)
{
    const int n = t.num_groups + 1;
    const double* en = t.energies;
    if (e <= __ldg(en)) return 0;
    if (e > __ldg(en + n - 1)) return n - 1;
    // The binary search below returns the largest k <= n-2 with en[k] <= e.
    // On a log-spaced grid a float estimate lands within a group of it; two
    // exact comparisons on each side confirm it, else the search runs.
    if (t.group_hint_scale > 0.0f) {
        int g = (int)((__logf(f64_to_f32_rn(e)) - t.group_hint_ln0) * t.group_hint_scale);
        g = max(0, min(g, n - 2));
        if (__ldg(en + g) <= e) {
            if (g + 1 > n - 2 || e < __ldg(en + g + 1)) return g;
            if (g + 2 > n - 2 || e < __ldg(en + g + 2)) return g + 1;
        } else {
            if (g >= 1 && __ldg(en + g - 1) <= e) return g - 1;
            if (g >= 2 && __ldg(en + g - 2) <= e) return g - 2;
        }
    }
    int high = n - 1, low = 0;
    while (high != low + 1) {
        int mid = (high + low) / 2;
        if (e < __ldg(en + mid)) high = mid;
        else low = mid;
    }
    return low;
}

struct Particle {
    double x, y, z, vx, vy, vz;
    double alpha, beta, gamma;
    double kinetic_energy, weight, time_to_census, age;
    double num_mean_free_paths, num_segments, inv_mfp, mean_free_path;
    uint64_t seed, identifier;
    int32_t last_event, num_collisions, breed, species, domain, cell, facet, group;
    // caches of values the reference recomputes every segment from unchanged
    // inputs (same bits): |velocity| until the velocity changes, and
    // 1/Sigma_t for the (cross-section class, group) key it was computed for;
    // inv_mfp = RN(1 / mean_free_path) for the mean-free-path update
    double speed;                  // < 0: stale
    int32_t xs_key;                // -1: stale
    double seg_len;                // length of the last segment (MC_Particle::segment_path_length)
    // a collision waiting for its warp's batched trajectory update: scatter's
    // outgoing energy and direction cosine, or the fission reaction's nuBar
    double pend_e, pend_a;
};

__device__ __forceinline__ void load_particle(const DevTables& t, const DevStore& s, uint64_t i, Particle& p)
{
    p.x = s.x[i]; p.y = s.y[i]; p.z = s.z[i];
    p.vx = s.vx[i]; p.vy = s.vy[i]; p.vz = s.vz[i];
    p.kinetic_energy = s.kinetic_energy[i];
    p.weight = s.weight[i];
    p.time_to_census = s.time_to_census[i];
    p.age = s.age[i];
    p.num_mean_free_paths = s.num_mean_free_paths[i];
    p.num_segments = s.num_segments[i];
    p.seed = s.seed[i];
    p.identifier = s.identifier[i];
    p.last_event = s.last_event[i];
    p.num_collisions = s.num_collisions[i];
    p.breed = s.breed[i];
    p.species = s.species[i];
    p.domain = s.domain[i];
    p.cell = s.cell[i];
    p.facet = 0;
    p.inv_mfp = 0.0;
    p.mean_free_path = 0.0;
    p.xs_key = -1;
    // direction from velocity (MC_Base_Particle.hh:317-325)
    // MC_Vector::Length(), the same value MC_Segment_Outcome computes next
    double speed = sqrt(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
    p.speed = speed;
    double factor = 1.0 / speed;
    p.alpha = factor * p.vx;
    p.beta = factor * p.vy;
    p.gamma = factor * p.vz;
    // MC_Load_Particle.cc:18-26
    if (p.time_to_census <= 0.0) p.time_to_census += t.time_step;
    if (p.age < 0.0) p.age = 0.0;
    p.group = energy_group(t, p.kinetic_energy);
}

// A history's sensitivity scores live in shared memory, S[k * stride] for
// parameter k (stride = threads per block), so that the parameter picked by a
// collision can index them without spilling a register array.
__device__ __forceinline__ void load_scores(const DevStore& s, uint64_t i, double* S, int stride, int K)
{
    for (int k = 0; k < K; k++) S[k * stride] = (k < s.score_fields) ? s.score[(uint64_t)k * s.capacity + i] : 0.0;
}

__device__ __forceinline__ void store_scores(const DevStore& s, uint64_t i, const double* S, int stride, int K)
{
    for (int k = 0; k < K && k < s.score_fields; k++) s.score[(uint64_t)k * s.capacity + i] = S[k * stride];
}

__device__ __forceinline__ void store_particle(const DevStore& s, uint64_t i, const Particle& p)
{
    s.x[i] = p.x; s.y[i] = p.y; s.z[i] = p.z;
    s.vx[i] = p.vx; s.vy[i] = p.vy; s.vz[i] = p.vz;
    s.kinetic_energy[i] = p.kinetic_energy;
    s.weight[i] = p.weight;
    s.time_to_census[i] = p.time_to_census;
    s.age[i] = p.age;
    s.num_mean_free_paths[i] = p.num_mean_free_paths;
    s.num_segments[i] = p.num_segments;
    s.seed[i] = p.seed;
    s.identifier[i] = p.identifier;
    s.last_event[i] = p.last_event;
    s.num_collisions[i] = p.num_collisions;
    s.breed[i] = p.breed;
    s.species[i] = p.species;
    s.domain[i] = p.domain;
    s.cell[i] = p.cell;
}

}  // namespace qsg
