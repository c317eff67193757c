/*
 * qs_oracle.c -- TEST INFRASTRUCTURE ONLY (see qs_oracle.h).
 *
 * A plain-C restatement of Quicksilver's per-cycle algorithm on one spatial
 * domain.  Every routine names the reference lines it follows.  Floating
 * point expressions keep the reference's operation order; the file is built
 * with -ffp-contract=off so no fused multiply-add changes a rounding.
 * libm's log/sin/cos/sqrt are used exactly where the reference uses them
 * (log/sin/cos: or the portable functions, oracle_use_portable_math).
 */
#include "../quicksilver_gb300/csrc/portable_math.h"
#include "qs_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Elementary functions of the tracking path: the host libm's (the
 * reference's), or, after oracle_use_portable_math(1), the portable
 * functions that the GPU library's portable-math build and the reference
 * built by `make -C oracle ref_pm` also use. */
static int g_portable_math = 0;

void oracle_use_portable_math(int on) { g_portable_math = on != 0; }

static inline double ora_log(double x) { return g_portable_math ? qsg_log(x) : log(x); }

/* FP64 work of the tracking path, counted as the reference writes it: every
 * +, -, *, / and sqrt of a double is one operation (a multiplication by -1.0
 * included, comparisons and conversions not), log / sin / cos / exp calls
 * are counted apart.  The macroscopic total cross section, which the
 * reference caches per (cell, group) for the cycle, is not counted per
 * segment.  Per thread while tracking, summed into the totals after each
 * pass (oracle_flop_counts). */
#ifdef _OPENMP
static __thread uint64_t t_flops, t_elem;
#else
static uint64_t t_flops, t_elem;
#endif
static uint64_t g_flops, g_elem;
#define FL(n) (t_flops += (uint64_t)(n))
#define EL(n) (t_elem += (uint64_t)(n))

void oracle_flop_counts(uint64_t* out2)
{
    out2[0] = g_flops;
    out2[1] = g_elem;
}

void oracle_reset_flop_counts(void) { g_flops = g_elem = 0; }

static inline void ora_sincos(double x, double* s, double* c)
{
    if (g_portable_math) {
        qsg_sincos(x, s, c);
    } else {
        *s = sin(x);
        *c = cos(x);
    }
}

void oracle_pm_eval(const double* x, uint64_t n, double* lg, double* sn, double* cs)
{
    for (uint64_t i = 0; i < n; i++) {
        lg[i] = qsg_log(x[i]);
        qsg_sincos(x[i], &sn[i], &cs[i]);
    }
}

/* PhysicalConstants.hh:9-16 */
#define QS_NEUTRON_REST_MASS_ENERGY 9.395656981095e+2
#define QS_PI 3.1415926535897932
#define QS_SPEED_OF_LIGHT 2.99792458e+10
#define QS_TINY_DOUBLE 1.0e-13
#define QS_SMALL_DOUBLE 1.0e-10
#define QS_HUGE_DOUBLE 1.0e+75

/* ------------------------------------------------------------------------ */
/* RNG: MC_RNG_State.hh:22-33 (64-bit LCG) and MC_RNG_State.cc:29-113
 * (Numerical Recipes psdes hash, 2 rounds, used to spawn child seeds). */
double oracle_rng_sample(uint64_t* seed)
{
    *seed = 2862933555777941757ULL * (*seed) + 3037000493ULL;
    return 5.4210108624275222e-20 * (double)(*seed);
}

static void psdes_hash(uint32_t* lword, uint32_t* irword)
{
    static const uint32_t c1[4] = {0xbaa96887u, 0x1e17d32cu, 0x03bcdc3cu, 0x0f33d1b2u};
    static const uint32_t c2[4] = {0x4b0f3b58u, 0xe874f0c3u, 0x6955c5a6u, 0x55a7ca46u};
    for (int i = 0; i < 2; i++) {
        uint32_t iswap = *irword;
        uint32_t ia = iswap ^ c1[i];
        uint32_t itmpl = ia & 0xffffu;
        uint32_t itmph = ia >> 16;
        uint32_t ib = itmpl * itmpl + ~(itmph * itmph);
        ia = (ib >> 16) | ((ib & 0xffffu) << 16);
        *irword = *lword ^ ((ia ^ c2[i]) + itmpl * itmph);
        *lword = iswap;
    }
}

uint64_t oracle_rng_spawn(uint64_t* parent_seed)
{
    uint32_t front = (uint32_t)(*parent_seed >> 32);
    uint32_t back = (uint32_t)(*parent_seed & 0xffffffffu);
    psdes_hash(&front, &back);
    uint64_t spawned = ((uint64_t)front << 32) | (uint64_t)back;
    oracle_rng_sample(parent_seed);
    return spawned;
}

/* ------------------------------------------------------------------------ */
/* Working particle: MC_Particle (MC_Particle.hh:18-88). */
typedef struct WorkParticle {
    double x, y, z, vx, vy, vz;
    double alpha, beta, gamma;
    double kinetic_energy, weight, time_to_census, total_xs, age;
    double num_mean_free_paths, mean_free_path, segment_path_length, num_segments;
    uint64_t seed, identifier;
    int32_t last_event, num_collisions, species, breed, group, domain, cell, facet;
    double S[QSG_MAX_PARAMS];   /* sensitivity scores (when enabled) */
} WorkParticle;

typedef struct Counters {
    uint64_t v[QSG_BAL_COUNT];
} Counters;

typedef struct Store {
    OracleParticle* p;
    uint64_t n, cap;
    double* sc;              /* [cap*K] sensitivity scores, row per particle (K > 0) */
    int K;
} Store;

typedef struct TrackCtx {
    const QsgProblem* pb;
    double* flux;            /* [C*G] */
    Counters* bal;
    Store* census;
    Store* extra;
    uint64_t* warnings;
    int overflow;
    OracleSens* sens;        /* NULL: no sensitivity scores */
    double* cell_tally;      /* [C] exponential cell tally (the reference's EXPONENTIAL_TALLY build); NULL: off */
} TrackCtx;

static void atomic_inc(uint64_t* a, uint64_t v)
{
#pragma omp atomic
    *a += v;
}

static void atomic_add_d(double* a, double v)
{
#pragma omp atomic
    *a += v;
}

static int store_reserve(Store* s, uint64_t want)
{
    if (want <= s->cap) return 0;
    uint64_t nc = s->cap ? s->cap : 1024;
    while (nc < want) nc *= 2;
    OracleParticle* np = (OracleParticle*)realloc(s->p, nc * sizeof(OracleParticle));
    if (!np) return -1;
    s->p = np;
    if (s->K > 0) {
        double* ns = (double*)realloc(s->sc, nc * (size_t)s->K * sizeof(double));
        if (!ns) return -1;
        s->sc = ns;
    }
    s->cap = nc;
    return 0;
}

/* Scores of slot i of s: copied from sc (NULL: zeros). */
static void store_set_scores(Store* s, uint64_t i, const double* sc)
{
    if (s->K <= 0) return;
    if (sc) memcpy(s->sc + i * (size_t)s->K, sc, (size_t)s->K * sizeof(double));
    else memset(s->sc + i * (size_t)s->K, 0, (size_t)s->K * sizeof(double));
}

/* Append from inside a parallel region: capacity is reserved beforehand by
 * the caller; an overflow is reported, never written. */
static void store_push_atomic(TrackCtx* ctx, Store* s, const OracleParticle* p, const double* sc)
{
    uint64_t idx;
#pragma omp atomic capture
    idx = s->n++;
    if (idx < s->cap) {
        s->p[idx] = *p;
        store_set_scores(s, idx, sc);
    } else {
#pragma omp atomic write
        ctx->overflow = 1;
    }
}

/* MC_Base_Particle(const MC_Particle&), MC_Base_Particle.hh:197-215. */
static void to_base(const WorkParticle* w, OracleParticle* b)
{
    b->x = w->x; b->y = w->y; b->z = w->z;
    b->vx = w->vx; b->vy = w->vy; b->vz = w->vz;
    b->kinetic_energy = w->kinetic_energy; b->weight = w->weight;
    b->time_to_census = w->time_to_census; b->age = w->age;
    b->num_mean_free_paths = w->num_mean_free_paths; b->num_segments = w->num_segments;
    b->random_number_seed = w->seed; b->identifier = w->identifier;
    b->last_event = w->last_event; b->num_collisions = w->num_collisions; b->breed = w->breed;
    b->species = w->species; b->domain = w->domain; b->cell = w->cell;
}

/* NuclearData::getEnergyGroup, NuclearData.cc:207-228. */
static int energy_group(const QsgProblem* pb, double e)
{
    int n = pb->num_groups + 1;
    const double* en = pb->energies;
    if (e <= en[0]) return 0;
    if (e > en[n - 1]) return n - 1;
    int high = n - 1, low = 0;
    while (high != low + 1) {
        int mid = (high + low) / 2;
        if (e < en[mid]) high = mid;
        else low = mid;
    }
    return low;
}

/* MC_Particle(const MC_Base_Particle&) (MC_Base_Particle.hh:286-331) plus
 * MC_Load_Particle (MC_Load_Particle.cc:11-29). */
static void load_particle(const QsgProblem* pb, const OracleParticle* b, WorkParticle* w, uint64_t* warnings)
{
    memset(w, 0, sizeof(*w));
    w->x = b->x; w->y = b->y; w->z = b->z;
    w->vx = b->vx; w->vy = b->vy; w->vz = b->vz;
    w->kinetic_energy = b->kinetic_energy; w->weight = b->weight;
    w->time_to_census = b->time_to_census; w->age = b->age;
    w->num_mean_free_paths = b->num_mean_free_paths; w->num_segments = b->num_segments;
    w->seed = b->random_number_seed; w->identifier = b->identifier;
    w->last_event = b->last_event; w->num_collisions = b->num_collisions;
    w->species = b->species; w->breed = b->breed; w->domain = b->domain; w->cell = b->cell;
    double speed = sqrt(b->vx * b->vx + b->vy * b->vy + b->vz * b->vz);
    FL(6);
    if (speed > 0) {
        double factor = 1.0 / speed;
        w->alpha = factor * b->vx;
        w->beta = factor * b->vy;
        w->gamma = factor * b->vz;
        FL(4);
    } else {
        atomic_inc(warnings, 1);
    }
    if (w->time_to_census <= 0.0) { w->time_to_census += pb->time_step; FL(1); }
    if (w->age < 0.0) w->age = 0.0;
    w->group = energy_group(pb, w->kinetic_energy);
}

/* macroscopicCrossSection (MacroscopicCrossSection.cc:14-48) with
 * reactionIndex = -1 summed over isotopes as weightedMacroscopicCrossSection
 * does (MacroscopicCrossSection.cc:58-81) and NuclearData::
 * getTotalCrossSection (NuclearData.cc:232-244).  The reference caches the
 * result per (cell, group) for the cycle; the cached value is this same sum. */
static double total_macro_xs(const QsgProblem* pb, int cell, int group)
{
    int mat = pb->cell_material[cell];
    double nd = pb->cell_number_density[cell];
    double sum = 0.0;
    for (int k = pb->material_isotope_offset[mat]; k < pb->material_isotope_offset[mat + 1]; k++) {
        double af = pb->material_atom_fraction[k];
        double micro;
        if (af == 0.0 || nd == 0.0) {
            sum += 1e-20;
            continue;
        }
        int iso = pb->material_isotope_gid[k];
        micro = 0.0;
        for (int r = pb->isotope_reaction_offset[iso]; r < pb->isotope_reaction_offset[iso + 1]; r++)
            micro += pb->reaction_xs[(int64_t)r * pb->num_groups + group];
        sum += af * nd * micro;
    }
    return sum;
}

/* MCT_Cell_Position_3D_G, MCT.cc:231-253. */
static void cell_position(const QsgProblem* pb, int cell, double* cx, double* cy, double* cz)
{
    double x = 0, y = 0, z = 0;
    for (int p = 0; p < 14; p++) {
        const double* nd = pb->nodes + 3 * (int64_t)pb->cell_points[(int64_t)cell * 14 + p];
        x += nd[0]; y += nd[1]; z += nd[2];
    }
    double one_over = 1.0 / ((double)14);
    *cx = x * one_over; *cy = y * one_over; *cz = z * one_over;
}

static const double* facet_point(const QsgProblem* pb, int cell, int facet, int k)
{
    int local = pb->facet_local_points[facet * 3 + k];
    return pb->nodes + 3 * (int64_t)pb->cell_points[(int64_t)cell * 14 + local];
}

/* MCT_Nearest_Facet_3D_G_Distance_To_Segment, MCT.cc:280-395. */
static double distance_to_segment(double plane_tolerance, double dot, double A, double B, double C, double D,
                                  const double* p0, const double* p1, const double* p2,
                                  double x, double y, double z, double alpha, double beta, double gamma)
{
    const double bb_tol = 1e-9;
    double numerator = -1.0 * (A * x + B * y + C * z + D);
    FL(7);
    if (numerator < 0.0) {
        FL(1);
        if (numerator * numerator > plane_tolerance) return QS_HUGE_DOUBLE;
    }
    double distance = numerator / dot;
    double ip[3];
    ip[0] = x + distance * alpha;
    ip[1] = y + distance * beta;
    ip[2] = z + distance * gamma;
    FL(7);

#define BELOW(ax) FL(1); if (p0[ax] > ip[ax] + bb_tol && p1[ax] > ip[ax] + bb_tol && p2[ax] > ip[ax] + bb_tol) return QS_HUGE_DOUBLE;
#define ABOVE(ax) FL(1); if (p0[ax] < ip[ax] - bb_tol && p1[ax] < ip[ax] - bb_tol && p2[ax] < ip[ax] - bb_tol) return QS_HUGE_DOUBLE;
#define XCROSS(ax, ay, bx, by, cx, cy) ((bx - ax) * (cy - ay) - (by - ay) * (cx - ax))
    double cross0 = 0, cross1 = 0, cross2 = 0;
    int u, v;
    if (C < -0.5 || C > 0.5) {
        BELOW(0) ABOVE(0) BELOW(1) ABOVE(1)
        u = 0; v = 1;
    } else if (B < -0.5 || B > 0.5) {
        BELOW(0) ABOVE(0) BELOW(2) ABOVE(2)
        u = 2; v = 0;
    } else if (A < -0.5 || A > 0.5) {
        BELOW(2) ABOVE(2) BELOW(1) ABOVE(1)
        u = 1; v = 2;
    } else {
        u = -1; v = -1;
    }
    if (u >= 0) {
        cross1 = XCROSS(p0[u], p0[v], p1[u], p1[v], ip[u], ip[v]);
        cross2 = XCROSS(p1[u], p1[v], p2[u], p2[v], ip[u], ip[v]);
        cross0 = XCROSS(p2[u], p2[v], p0[u], p0[v], ip[u], ip[v]);
        FL(21);
    }
#undef BELOW
#undef ABOVE
#undef XCROSS
    double s = cross0 + cross1 + cross2;
    double cross_tol = 1e-9 * (s < 0 ? -s : s);
    FL(3);
    if ((cross0 > -cross_tol && cross1 > -cross_tol && cross2 > -cross_tol) ||
        (cross0 < cross_tol && cross1 < cross_tol && cross2 < cross_tol))
        return distance;
    return QS_HUGE_DOUBLE;
}

/* MCT_Nearest_Facet (MCT.cc:86-137) -> MCT_Nearest_Facet_3D_G
 * (MCT.cc:549-621) -> MCT_Nearest_Facet_Find_Nearest (MCT.cc:436-536).
 * The particle coordinate is moved in place on a retry (MCT.cc:510,656-666). */
static double nearest_facet(const QsgProblem* pb, WorkParticle* w, int* facet_out, uint64_t* warnings)
{
    const int cell = w->cell;
    const double* planes = pb->facet_planes + (int64_t)cell * 96;
    int iteration = 0;
    double move_factor = 0.5 * QS_SMALL_DOUBLE;
    double dist[24];
    for (;;) {
        double plane_tolerance = 1e-16 * (w->x * w->x + w->y * w->y + w->z * w->z);
        FL(6);
        for (int f = 0; f < 24; f++) {
            dist[f] = QS_HUGE_DOUBLE;
            const double* pl = planes + 4 * f;
            double dot = pl[0] * w->alpha + pl[1] * w->beta + pl[2] * w->gamma;
            FL(5);
            if (dot <= 0.0) continue;
            dist[f] = distance_to_segment(plane_tolerance, dot, pl[0], pl[1], pl[2], pl[3],
                                          facet_point(pb, cell, f, 0), facet_point(pb, cell, f, 1),
                                          facet_point(pb, cell, f, 2), w->x, w->y, w->z,
                                          w->alpha, w->beta, w->gamma);
        }
        /* Find_Nearest, MCT.cc:436-479 (ties on `<=` go to the later facet). */
        double best = 1e80;
        int best_f = 0;
        double neg = -QS_HUGE_DOUBLE;
        int neg_f = 0;
        for (int f = 0; f < 24; f++) {
            if (dist[f] > 0.0) {
                if (dist[f] <= best) { best = dist[f]; best_f = f; }
            } else if (dist[f] > neg) {
                neg = dist[f]; neg_f = f;
            }
        }
        if (best == QS_HUGE_DOUBLE && neg != -QS_HUGE_DOUBLE) { best = neg; best_f = neg_f; }

        /* Retry logic, MCT.cc:497-535. */
        int retry = 0;
        if ((best == QS_HUGE_DOUBLE && move_factor > 0) || (w->num_segments > 10000000 && best <= 0.0)) {
            double cx, cy, cz;
            cell_position(pb, cell, &cx, &cy, &cz);
            w->x += move_factor * (cx - w->x);
            w->y += move_factor * (cy - w->y);
            w->z += move_factor * (cz - w->z);
            iteration++;
            move_factor *= 2.0;
            FL(42 + 4 + 9 + 1);   /* the centre (MCT.cc:231-253), the move, the factor */
            if (move_factor > 1.0e-2) move_factor = 1.0e-2;
            if (iteration == 10000) { atomic_inc(warnings, 1); retry = 0; }
            else retry = 1;
        }
        if (!retry) {
            /* MCT.cc:114-130 */
            if (best < 0) best = 0;
            if (best >= QS_HUGE_DOUBLE) atomic_inc(warnings, 1);
            *facet_out = best_f;
            return best;
        }
    }
}

enum { OUT_COLLISION = 0, OUT_FACET = 1, OUT_CENSUS = 2 };

/* MC_Segment_Outcome, MC_Segment_Outcome.cc:30-226. */
static int segment_outcome(TrackCtx* ctx, WorkParticle* w)
{
    const QsgProblem* pb = ctx->pb;
    double distance[3];
    double speed = sqrt(w->vx * w->vx + w->vy * w->vy + w->vz * w->vz);
    FL(6);
    int force_collision = 0;
    if (w->num_mean_free_paths < 0.0) {
        force_collision = 1;
        if (w->num_mean_free_paths > -900.0) atomic_inc(ctx->warnings, 1);
        w->num_mean_free_paths = QS_SMALL_DOUBLE;
    }
    double sigma = total_macro_xs(pb, w->cell, w->group);
    w->total_xs = sigma;
    if (sigma == 0.0) w->mean_free_path = QS_HUGE_DOUBLE;
    else { w->mean_free_path = 1.0 / sigma; FL(1); }
    if (w->num_mean_free_paths == 0.0) {
        double r = oracle_rng_sample(&w->seed);
        w->num_mean_free_paths = -1.0 * ora_log(r);
        FL(2); EL(1);
    }
    if (force_collision) distance[OUT_COLLISION] = QS_SMALL_DOUBLE;
    else { distance[OUT_COLLISION] = w->num_mean_free_paths * w->mean_free_path; FL(1); }
    distance[OUT_CENSUS] = speed * w->time_to_census;
    FL(1);

    int facet = 0;
    distance[OUT_FACET] = nearest_facet(pb, w, &facet, ctx->warnings);

    if (w->last_event == QSG_EVENT_FACET_TRACKING_ERROR) return OUT_FACET;

    if (force_collision) {
        distance[OUT_FACET] = QS_HUGE_DOUBLE;
        distance[OUT_CENSUS] = QS_HUGE_DOUBLE;
        distance[OUT_COLLISION] = QS_TINY_DOUBLE;
    }
    /* MC_Find_Min, MC_Segment_Outcome.cc:232-248 */
    int outcome = 0;
    double mn = distance[0];
    for (int k = 1; k < 3; k++)
        if (distance[k] < mn) { mn = distance[k]; outcome = k; }
    if (distance[outcome] < 0) atomic_inc(ctx->warnings, 1);
    w->segment_path_length = distance[outcome];
    w->num_mean_free_paths -= w->segment_path_length / w->mean_free_path;
    FL(2);
    static const int to_event[3] = {QSG_EVENT_COLLISION, QSG_EVENT_FACET_TRANSIT_EXIT, QSG_EVENT_CENSUS};
    w->last_event = to_event[outcome];
    if (outcome == OUT_COLLISION) w->num_mean_free_paths = 0.0;
    else if (outcome == OUT_FACET) w->facet = facet;
    else w->time_to_census = (w->time_to_census < 0.0) ? w->time_to_census : 0.0;
    if (force_collision) w->num_mean_free_paths = 0.0;
    if (w->segment_path_length == 0.0) return outcome;

    /* MC_Particle::Move_Particle, MC_Particle.hh:139-146 */
    w->x += (w->alpha * w->segment_path_length);
    w->y += (w->beta * w->segment_path_length);
    w->z += (w->gamma * w->segment_path_length);
    double seg_time = (w->segment_path_length / speed);
    w->time_to_census -= seg_time;
    w->age += seg_time;
    if (w->time_to_census < 0.0) w->time_to_census = 0.0;
    FL(6 + 3 + 2);   /* the move (MC_Particle.hh:139-146), the time, the flux tally */
    /* Tallies::TallyScalarFlux, Tallies.hh:350-354 */
    atomic_add_d(&ctx->flux[(int64_t)w->cell * pb->num_groups + w->group], w->segment_path_length * w->weight);
    return outcome;
}

/* ------------------------------------------------------------------------ */
/* Sensitivity scores (no counterpart in the reference; what the CUDA
 * library's qsg_enable_sensitivity tallies).  Parameter of (material,
 * reaction type, group), or -1. */
static int sens_param(const OracleSens* se, int mat, int type, int group)
{
    for (int k = 0; k < se->K; k++)
        if (se->material[k] == mat && se->reaction[k] == type && group >= se->group_lo[k] && group < se->group_hi[k])
            return k;
    return -1;
}

/* dSigma_t/dtheta_k contributed by reaction type `type` in this cell and
 * group: the macroscopic cross sections af * nd * xs of that type summed in
 * isotope / reaction order (MacroscopicCrossSection.cc:14-48), over theta_k. */
static double sens_dsig(const QsgProblem* pb, const OracleSens* se, int k, int cell, int group, int type)
{
    const int G = pb->num_groups;
    int mat = pb->cell_material[cell];
    double nd = pb->cell_number_density[cell];
    double sum = 0.0;
    for (int j = pb->material_isotope_offset[mat]; j < pb->material_isotope_offset[mat + 1]; j++) {
        int iso = pb->material_isotope_gid[j];
        double af = pb->material_atom_fraction[j];
        for (int r = pb->isotope_reaction_offset[iso]; r < pb->isotope_reaction_offset[iso + 1]; r++)
            if (pb->reaction_type[r] == type) sum += af * nd * pb->reaction_xs[(int64_t)r * G + group];
    }
    return sum / se->theta[k];
}

/* One flight of length l through cell / group: scores gain -l dSigma_t/dtheta;
 * the flight's track-length flux l w is tallied with its full score
 * l w (S_k + [collision] dSigma_t/dtheta_k / Sigma_t). */
static void sens_segment(TrackCtx* ctx, WorkParticle* w, int collided)
{
    OracleSens* se = ctx->sens;
    const QsgProblem* pb = ctx->pb;
    const double l = w->segment_path_length;
    if (l == 0.0) return;
    int mat = pb->cell_material[w->cell];
    int pk[3];
    double pd[3];
    for (int j = 0; j < 3; j++) {
        pk[j] = sens_param(se, mat, j + 1, w->group);
        pd[j] = pk[j] >= 0 ? sens_dsig(pb, se, pk[j], w->cell, w->group, j + 1) : 0.0;
        if (pk[j] >= 0) w->S[pk[j]] -= l * pd[j];
    }
    const double lw = l * w->weight;
    atomic_add_d(&se->flux_cell[w->cell], lw);
    for (int k = 0; k < se->K; k++) {
        double v = w->S[k];
        if (collided)
            for (int j = 0; j < 3; j++)
                if (pk[j] == k) v += pd[j] * w->mean_free_path;
        if (v != 0.0) atomic_add_d(&se->dflux[(int64_t)w->cell * se->K + k], lw * v);
    }
}

/* DirectionCosine::Rotate3DVector, DirectionCosine.hh:122-147. */
static void rotate3d(WorkParticle* w, double sin_Theta, double cos_Theta, double sin_Phi, double cos_Phi)
{
    double cos_theta = w->gamma;
    double sin_theta = sqrt((1.0 - (cos_theta * cos_theta)));
    double cos_phi, sin_phi;
    FL(3 + 22);
    if (sin_theta < 1e-6) {
        cos_phi = 1.0;
        sin_phi = 0.0;
    } else {
        cos_phi = w->alpha / sin_theta;
        sin_phi = w->beta / sin_theta;
        FL(2);
    }
    double a = cos_theta * cos_phi * (sin_Theta * cos_Phi) - sin_phi * (sin_Theta * sin_Phi) + sin_theta * cos_phi * cos_Theta;
    double b = cos_theta * sin_phi * (sin_Theta * cos_Phi) + cos_phi * (sin_Theta * sin_Phi) + sin_theta * sin_phi * cos_Theta;
    double g = -sin_theta * (sin_Theta * cos_Phi) + cos_theta * cos_Theta;
    w->alpha = a; w->beta = b; w->gamma = g;
}

/* updateTrajectory, CollisionEvent.cc:24-46. */
static void update_trajectory(double energy, double angle, WorkParticle* w)
{
    w->kinetic_energy = energy;
    double cosTheta = angle;
    double r = oracle_rng_sample(&w->seed);
    double phi = 2 * 3.14159265 * r;
    double sinPhi, cosPhi;
    ora_sincos(phi, &sinPhi, &cosPhi);
    double sinTheta = sqrt((1.0 - (cosTheta * cosTheta)));
    FL(2 + 3 + 8 + 3 + 2); EL(3);   /* sample, phi, sin theta, speed, velocity, the log's sample and sign */
    rotate3d(w, sinTheta, cosTheta, sinPhi, cosPhi);
    const double m = QS_NEUTRON_REST_MASS_ENERGY;
    double speed = (QS_SPEED_OF_LIGHT * sqrt((1.0 - ((m * m) / ((energy + m) * (energy + m))))));
    w->vx = speed * w->alpha;
    w->vy = speed * w->beta;
    w->vz = speed * w->gamma;
    r = oracle_rng_sample(&w->seed);
    w->num_mean_free_paths = -1.0 * ora_log(r);
}

/* CollisionEvent, CollisionEvent.cc:48-148 (with NuclearDataReaction::
 * sampleCollision, NuclearData.cc:52-88).  Returns 1 to continue tracking. */
static int collision_event(TrackCtx* ctx, WorkParticle* w)
{
    const QsgProblem* pb = ctx->pb;
    const int G = pb->num_groups;
    int mat = pb->cell_material[w->cell];
    double nd = pb->cell_number_density[w->cell];
    double r = oracle_rng_sample(&w->seed);
    double current = w->total_xs * r;
    FL(2);
    int sel_iso = -1, sel_r = -1;
    int k0 = pb->material_isotope_offset[mat], k1 = pb->material_isotope_offset[mat + 1];
    for (int k = k0; k < k1 && current >= 0; k++) {
        int iso = pb->material_isotope_gid[k];
        double af = pb->material_atom_fraction[k];
        int r0 = pb->isotope_reaction_offset[iso], r1 = pb->isotope_reaction_offset[iso + 1];
        for (int rr = r0; rr < r1; rr++) {
            double macro;
            if (af == 0.0 || nd == 0.0) macro = 1e-20;
            else { macro = af * nd * pb->reaction_xs[(int64_t)rr * G + w->group]; FL(2); }
            current -= macro;
            FL(1);
            if (current < 0) { sel_iso = iso; sel_r = rr; break; }
        }
    }
    if (sel_iso < 0) {
        /* qs_assert(selectedIso != -1) prints and continues with an invalid
         * index (CollisionEvent.cc:84); take the material's last reaction. */
        atomic_inc(ctx->warnings, 1);
        int iso = pb->material_isotope_gid[k1 - 1];
        sel_iso = iso;
        sel_r = pb->isotope_reaction_offset[iso + 1] - 1;
    }
    double energy_out[4] = {0}, angle_out[4] = {0};
    int n_out = 0;
    double mass = pb->material_mass[mat];
    int type = pb->reaction_type[sel_r];
    if (ctx->sens) {
        /* d log Sigma_r / dtheta of the selected reaction, in the incoming group */
        int k = sens_param(ctx->sens, mat, type, w->group);
        if (k >= 0) w->S[k] += 1.0 / ctx->sens->theta[k];
    }
    switch (type) {
    case QSG_REACT_SCATTER: {
        n_out = 1;
        double rn = oracle_rng_sample(&w->seed);
        energy_out[0] = w->kinetic_energy * (1.0 - (rn * (1.0 / mass)));
        rn = oracle_rng_sample(&w->seed) * 2.0 - 1.0;
        angle_out[0] = rn;
        FL(1 + 4 + 1 + 2);
        break;
    }
    case QSG_REACT_ABSORPTION:
        break;
    case QSG_REACT_FISSION: {
        int num = (int)(pb->reaction_nubar[sel_r] + oracle_rng_sample(&w->seed));
        FL(2);
        if (num > 4) { atomic_inc(ctx->warnings, 1); num = 4; }
        n_out = num;
        for (int o = 0; o < num; o++) {
            double rn = oracle_rng_sample(&w->seed) / 2.0 + 0.5;
            energy_out[o] = (20 * rn * rn);
            rn = oracle_rng_sample(&w->seed) * 2.0 - 1.0;
            angle_out[o] = rn;
            FL(3 + 2 + 3);
        }
        break;
    }
    default:
        atomic_inc(ctx->warnings, 1);
        break;
    }
    atomic_inc(&ctx->bal->v[QSG_BAL_COLLISION], 1);
    if (type == QSG_REACT_SCATTER) atomic_inc(&ctx->bal->v[QSG_BAL_SCATTER], 1);
    else if (type == QSG_REACT_ABSORPTION) atomic_inc(&ctx->bal->v[QSG_BAL_ABSORB], 1);
    else if (type == QSG_REACT_FISSION) {
        atomic_inc(&ctx->bal->v[QSG_BAL_FISSION], 1);
        atomic_inc(&ctx->bal->v[QSG_BAL_PRODUCE], (uint64_t)n_out);
    }
    if (n_out == 0) return 0;
    for (int s = 1; s < n_out; s++) {
        WorkParticle sec = *w;
        sec.seed = oracle_rng_spawn(&w->seed);
        sec.identifier = sec.seed;
        update_trajectory(energy_out[s], angle_out[s], &sec);
        OracleParticle b;
        to_base(&sec, &b);
        store_push_atomic(ctx, ctx->extra, &b, sec.S);
    }
    update_trajectory(energy_out[0], angle_out[0], w);
    if (n_out > 1) {
        OracleParticle b;
        to_base(w, &b);
        store_push_atomic(ctx, ctx->extra, &b, w->S);
    }
    w->group = energy_group(pb, w->kinetic_energy);
    return n_out == 1;
}

/* MCT_Reflect_Particle, MCT.cc:400-430. */
static void reflect_particle(const QsgProblem* pb, WorkParticle* w)
{
    const double* pl = pb->facet_planes + (int64_t)w->cell * 96 + 4 * w->facet;
    double nx = pl[0], ny = pl[1], nz = pl[2];
    double dot = 2.0 * (w->alpha * nx + w->beta * ny + w->gamma * nz);
    if (dot > 0) {
        w->alpha -= dot * nx;
        w->beta -= dot * ny;
        w->gamma -= dot * nz;
        FL(6);
    }
    double speed = sqrt(w->vx * w->vx + w->vy * w->vy + w->vz * w->vz);
    FL(6 + 6 + 3);
    w->vx = speed * w->alpha;
    w->vy = speed * w->beta;
    w->vz = speed * w->gamma;
}

/* CycleTrackingGuts + CycleTrackingFunction, CycleTracking.cc:14-120. */
static void track_one(TrackCtx* ctx, const OracleParticle* in, const double* in_scores)
{
    const QsgProblem* pb = ctx->pb;
    WorkParticle w;
    load_particle(pb, in, &w, ctx->warnings);
    if (ctx->sens && in_scores) memcpy(w.S, in_scores, (size_t)ctx->sens->K * sizeof(double));
    int keep;
    do {
        if (ctx->sens) w.segment_path_length = 0.0;   /* a segment that returns early moves nothing */
        /* EXPONENTIAL_TALLY build of the reference (CycleTracking.cc:48-50,
         * Tallies.hh:357-360): one random number per segment, its exp tallied
         * in the particle's cell, before the segment outcome */
        if (ctx->cell_tally) {
            atomic_add_d(&ctx->cell_tally[w.cell], exp(oracle_rng_sample(&w.seed)));
            FL(2); EL(1);
        }
        int outcome = segment_outcome(ctx, &w);
        if (ctx->sens) sens_segment(ctx, &w, outcome == OUT_COLLISION);
        atomic_inc(&ctx->bal->v[QSG_BAL_NUM_SEGMENTS], 1);
        w.num_segments += 1.;
        switch (outcome) {
        case OUT_COLLISION:
            keep = collision_event(ctx, &w);
            break;
        case OUT_FACET: {
            /* MC_Facet_Crossing_Event, MC_Facet_Crossing_Event.cc:23-70 */
            int64_t fi = (int64_t)w.cell * 24 + w.facet;
            int ev = pb->facet_event[fi];
            if (ev == QSG_ADJ_TRANSIT_ON_PROCESSOR) {
                int nc = pb->facet_adjacent_cell[fi];
                int nf = pb->facet_adjacent_facet[fi];
                w.cell = nc;
                w.facet = nf;
                w.last_event = QSG_EVENT_FACET_TRANSIT_EXIT;
                keep = 1;
            } else if (ev == QSG_ADJ_BOUNDARY_ESCAPE) {
                atomic_inc(&ctx->bal->v[QSG_BAL_ESCAPE], 1);
                if (ctx->sens) {
                    OracleSens* se = ctx->sens;
                    atomic_add_d(&se->leak[0], w.weight);
                    for (int k = 0; k < se->K; k++)
                        if (w.S[k] != 0.0) atomic_add_d(&se->dleak[k], w.weight * w.S[k]);
                }
                w.last_event = QSG_EVENT_FACET_ESCAPE;
                w.species = -1;
                keep = 0;
            } else if (ev == QSG_ADJ_BOUNDARY_REFLECTION) {
                w.last_event = QSG_EVENT_FACET_REFLECTION;
                reflect_particle(pb, &w);
                keep = 1;
            } else {
                /* Off-processor transit needs a second domain; the
                 * single-domain path counts it as a warning and drops it. */
                atomic_inc(ctx->warnings, 1);
                w.last_event = (ev == QSG_ADJ_TRANSIT_OFF_PROCESSOR) ? QSG_EVENT_FACET_COMMUNICATION : w.last_event;
                keep = 0;
            }
            break;
        }
        default: { /* census: ParticleVault::pushParticle, ParticleVault.hh:86-93 */
            OracleParticle b;
            to_base(&w, &b);
            store_push_atomic(ctx, ctx->census, &b, w.S);
            atomic_inc(&ctx->bal->v[QSG_BAL_CENSUS], 1);
            keep = 0;
            break;
        }
        }
    } while (keep);
}

static void set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    else omp_set_num_threads(omp_get_num_procs());
#else
    (void)nthreads;
#endif
}

/* The while(!done) loop of cycleTracking (main.cc:155-299) on one domain:
 * track the processing list; fission products collected in the extra store
 * (ParticleVaultContainer::addExtraParticle, :340-349) become the next
 * processing list (cleanExtraVaults, :357-400) until none are left. */
static int track_all(const QsgProblem* pb, Store* processing, Store* census, Counters* bal, double* flux,
                     uint64_t* warnings, int nthreads, OracleSens* sens, double* cell_tally)
{
    Store extra = {0, 0, 0, NULL, processing->K};
    set_threads(nthreads);
    int status = 0;
    while (processing->n > 0) {
        uint64_t n = processing->n;
        /* worst case: every particle censuses; every fission makes <= 4 */
        if (store_reserve(census, census->n + n) || store_reserve(&extra, 4 * n)) { status = -1; break; }
        extra.n = 0;
        TrackCtx ctx = {pb, flux, bal, census, &extra, warnings, 0, sens, cell_tally};
        const OracleParticle* src = processing->p;
        const double* src_sc = processing->K > 0 ? processing->sc : NULL;
        const int K = processing->K;
#pragma omp parallel
        {
            t_flops = t_elem = 0;
#pragma omp for schedule(dynamic, 64)
            for (int64_t i = 0; i < (int64_t)n; i++)
                track_one(&ctx, &src[i], src_sc ? src_sc + i * (size_t)K : NULL);
#pragma omp atomic
            g_flops += t_flops;
#pragma omp atomic
            g_elem += t_elem;
        }
        if (ctx.overflow) { status = -2; break; }
        /* swap: extras become the processing list */
        Store tmp = *processing;
        *processing = extra;
        extra = tmp;
        extra.n = 0;
    }
    free(extra.p);
    free(extra.sc);
    processing->n = 0;
    return status;
}

/* ------------------------------------------------------------------------ */
struct OracleRun {
    const QsgProblem* pb;
    const double* source_rate;
    uint64_t n_particles;
    double e_min, e_max, low_weight_cutoff;
    int load_balance;
    Store processing, processed;
    Counters bal, last;
    double* flux;
    uint64_t* source_tally;     /* MC_Cell_State::_sourceTally, persists across cycles */
    double source_particle_weight;
    uint64_t warnings;
    OracleSens sens;            /* sens.K == 0: off */
    int has_sens;
    double* cell_tally;         /* [C] exponential cell tally, NULL: off */
    uint64_t seed_offset;       /* added to every source seed (0: the reference's seeding) */
};

OracleRun* oracle_create(const QsgProblem* pb, const double* source_rate, uint64_t n_particles,
                         double e_min, double e_max, double low_weight_cutoff, int load_balance)
{
    OracleRun* r = (OracleRun*)calloc(1, sizeof(OracleRun));
    if (!r) return NULL;
    r->pb = pb;
    r->source_rate = source_rate;
    r->n_particles = n_particles;
    r->e_min = e_min;
    r->e_max = e_max;
    r->low_weight_cutoff = low_weight_cutoff;
    r->load_balance = load_balance;
    r->flux = (double*)calloc((size_t)pb->num_cells * pb->num_groups, sizeof(double));
    r->source_tally = (uint64_t*)calloc((size_t)pb->num_cells, sizeof(uint64_t));
    if (!r->flux || !r->source_tally) { oracle_destroy(r); return NULL; }
    return r;
}

void oracle_set_seed_offset(OracleRun* r, uint64_t offset) { r->seed_offset = offset; }

void oracle_destroy(OracleRun* r)
{
    if (!r) return;
    free(r->processing.p);
    free(r->processed.p);
    free(r->processing.sc);
    free(r->processed.sc);
    if (r->has_sens) {
        free(r->sens.flux_cell);
        free(r->sens.dflux);
        free(r->sens.leak);
        free(r->sens.dleak);
    }
    free(r->flux);
    free(r->source_tally);
    free(r->cell_tally);
    free(r);
}

/* Append p with scores sc (NULL: zeros). */
static int store_push(Store* s, const OracleParticle* p, const double* sc)
{
    if (store_reserve(s, s->n + 1)) return -1;
    store_set_scores(s, s->n, sc);
    s->p[s->n++] = *p;
    return 0;
}

/* Erase particle i by moving the last particle into its slot
 * (ParticleVault::eraseSwapParticle, ParticleVault.hh:199-207). */
static void store_erase_swap(Store* s, uint64_t i)
{
    s->p[i] = s->p[s->n - 1];
    if (s->K > 0) store_set_scores(s, i, s->sc + (s->n - 1) * (size_t)s->K);
    s->n--;
}

/* MCT_Cell_Volume_3D_G_vector_tetDet, MCT.cc:633-648. */
static double tet_det(const double* v0_, const double* v1_, const double* v2_, const double* v3)
{
    double v0x = v0_[0], v0y = v0_[1], v0z = v0_[2];
    double v1x = v1_[0], v1y = v1_[1], v1z = v1_[2];
    double v2x = v2_[0], v2y = v2_[1], v2z = v2_[2];
    v0x -= v3[0]; v0y -= v3[1]; v0z -= v3[2];
    v1x -= v3[0]; v1y -= v3[1]; v1z -= v3[2];
    v2x -= v3[0]; v2y -= v3[1]; v2z -= v3[2];
    return v0z * (v1x * v2y - v1y * v2x) + v0y * (v1z * v2x - v1x * v2z) + v0x * (v1y * v2z - v1z * v2y);
}

/* MCT_Generate_Coordinate_3D_G, MCT.cc:143-226. */
static void generate_coordinate(const QsgProblem* pb, uint64_t* seed, int cell, double* out, uint64_t* warnings)
{
    double center[3];
    cell_position(pb, cell, &center[0], &center[1], &center[2]);
    double r = oracle_rng_sample(seed);
    double which_volume = r * 6.0 * pb->cell_volume[cell];
    double current = 0.0;
    int facet = -1;
    const double *p0 = NULL, *p1 = NULL, *p2 = NULL;
    while (current < which_volume) {
        facet++;
        if (facet == 24) break;
        p0 = facet_point(pb, cell, facet, 0);
        p1 = facet_point(pb, cell, facet, 1);
        p2 = facet_point(pb, cell, facet, 2);
        current += tet_det(p0, p1, p2, center);
    }
    double r1 = oracle_rng_sample(seed);
    double r2 = oracle_rng_sample(seed);
    double r3 = oracle_rng_sample(seed);
    if (r1 + r2 > 1.0) { r1 = 1.0 - r1; r2 = 1.0 - r2; }
    if (r2 + r3 > 1.0) {
        double tmp = r3;
        r3 = 1.0 - r1 - r2;
        r2 = 1.0 - tmp;
    } else if (r1 + r2 + r3 > 1.0) {
        double tmp = r3;
        r3 = r1 + r2 + r3 - 1.0;
        r1 = 1.0 - r2 - tmp;
    }
    double r4 = 1.0 - r1 - r2 - r3;
    if (!p0) { atomic_inc(warnings, 1); out[0] = out[1] = out[2] = 0; return; }
    for (int a = 0; a < 3; a++) out[a] = (r4 * center[a] + r1 * p0[a] + r2 * p1[a] + r3 * p2[a]);
}

/* MC_SourceNow, MC_SourceNow.cc:28-164 (one domain, cells in index order). */
static int source_now(OracleRun* run)
{
    const QsgProblem* pb = run->pb;
    const double dt = pb->time_step;
    double total_weight = 0;
    for (int c = 0; c < pb->num_cells; c++)
        total_weight += pb->cell_volume[c] * run->source_rate[pb->cell_material[c]] * dt;
    double source_fraction = 0.1;
    double spw = total_weight / (source_fraction * run->n_particles);
    run->source_particle_weight = spw;
    for (int c = 0; c < pb->num_cells; c++) {
        double cell_weight = pb->cell_volume[c] * run->source_rate[pb->cell_material[c]] * dt;
        double cell_num_float = cell_weight / spw;
        int n = (int)cell_num_float;
        for (int k = 0; k < n; k++) {
            uint64_t seed0 = run->source_tally[c]++;
            seed0 += pb->cell_id[c];
            seed0 += run->seed_offset;
            WorkParticle w;
            memset(&w, 0, sizeof(w));
            w.seed = oracle_rng_spawn(&seed0);
            w.identifier = seed0;
            double coord[3];
            generate_coordinate(pb, &w.seed, c, coord, &run->warnings);
            w.x = coord[0]; w.y = coord[1]; w.z = coord[2];
            /* DirectionCosine::Sample_Isotropic, DirectionCosine.cc:5-12 */
            w.gamma = 1.0 - 2.0 * oracle_rng_sample(&w.seed);
            double sine_gamma = sqrt((1.0 - (w.gamma * w.gamma)));
            double phi = QS_PI * (2.0 * oracle_rng_sample(&w.seed) - 1.0);
            double sin_phi, cos_phi;
            ora_sincos(phi, &sin_phi, &cos_phi);
            w.alpha = sine_gamma * cos_phi;
            w.beta = sine_gamma * sin_phi;
            w.kinetic_energy = (run->e_max - run->e_min) * oracle_rng_sample(&w.seed) + run->e_min;
            /* Get_Speed_From_Energy, MC_SourceNow.cc:169-177 */
            const double m = QS_NEUTRON_REST_MASS_ENERGY;
            double E = w.kinetic_energy;
            double speed = QS_SPEED_OF_LIGHT * sqrt(E * (E + 2.0 * (m)) / ((E + m) * (E + m)));
            w.vx = speed * w.alpha;
            w.vy = speed * w.beta;
            w.vz = speed * w.gamma;
            w.domain = 0;
            w.cell = c;
            w.weight = spw;
            double rn = oracle_rng_sample(&w.seed);
            w.num_mean_free_paths = -1.0 * ora_log(rn);
            rn = oracle_rng_sample(&w.seed);
            w.time_to_census = dt * rn;
            w.last_event = QSG_EVENT_CENSUS; /* MC_Particle default */
            w.species = 0;
            OracleParticle b;
            to_base(&w, &b);
            if (store_push(&run->processing, &b, NULL)) return -1;
            run->bal.v[QSG_BAL_SOURCE]++;
        }
    }
    return 0;
}

/* PopulationControl + PopulationControlGuts, PopulationControl.cc:20-122.
 * The processing vaults are one flat list here; particles are visited from
 * the back and each draws from its own stream, so the surviving set does not
 * depend on how the reference splits the list into vaults. */
static int population_control(OracleRun* run)
{
    uint64_t target = run->n_particles;
    uint64_t local = run->processing.n;
    double factor;
    if (run->load_balance) {
        target = (uint64_t)ceil((double)target / (double)1);
        int current = (int)local;
        factor = (current != 0) ? (double)target / (double)current : 1.0;
    } else {
        factor = (double)target / (double)local;
    }
    if (factor != 1.0) {
        for (int64_t i = (int64_t)local - 1; i >= 0; i--) {
            OracleParticle* p = &run->processing.p[i];
            double r = oracle_rng_sample(&p->random_number_seed);
            if (factor < 1) {
                if (r > factor) {
                    store_erase_swap(&run->processing, (uint64_t)i);
                    run->bal.v[QSG_BAL_RR]++;
                } else {
                    p->weight /= factor;
                }
            } else if (factor > 1) {
                int split = (int)floor(factor);
                if (r > (factor - split)) split--;
                p->weight /= factor;
                OracleParticle sp = *p;
                double parent_sc[QSG_MAX_PARAMS];   /* split copies inherit the scores */
                if (run->processing.K > 0)
                    memcpy(parent_sc, run->processing.sc + (size_t)i * run->processing.K,
                           (size_t)run->processing.K * sizeof(double));
                for (int k = 0; k < split; k++) {
                    run->bal.v[QSG_BAL_SPLIT]++;
                    sp.random_number_seed = oracle_rng_spawn(&run->processing.p[i].random_number_seed);
                    sp.identifier = sp.random_number_seed;
                    if (store_push(&run->processing, &sp, run->processing.K > 0 ? parent_sc : NULL)) return -1;
                }
            }
        }
    }
    return 0;
}

/* RouletteLowWeightParticles, PopulationControl.cc:127-171. */
static void roulette_low_weight(OracleRun* run)
{
    const double cutoff = run->low_weight_cutoff;
    if (!(cutoff > 0.0)) return;
    const double weight_cutoff = cutoff * run->source_particle_weight;
    for (int64_t i = (int64_t)run->processing.n - 1; i >= 0; i--) {
        OracleParticle* p = &run->processing.p[i];
        if (p->weight <= weight_cutoff) {
            double r = oracle_rng_sample(&p->random_number_seed);
            if (r <= cutoff) {
                p->weight /= cutoff;
            } else {
                store_erase_swap(&run->processing, (uint64_t)i);
                run->bal.v[QSG_BAL_RR]++;
            }
        }
    }
}

int oracle_cycle_init(OracleRun* run)
{
    /* swapProcessingProcessedVaults (ParticleVaultContainer.cc:278-311) */
    Store tmp = run->processing;
    run->processing = run->processed;
    run->processed = tmp;
    run->processed.n = 0;
    run->bal.v[QSG_BAL_START] = run->processing.n;
    if (source_now(run)) return -1;
    if (population_control(run)) return -1;
    roulette_low_weight(run);
    return 0;
}

int oracle_cycle_tracking(OracleRun* run, int nthreads)
{
    return track_all(run->pb, &run->processing, &run->processed, &run->bal, run->flux, &run->warnings, nthreads,
                     run->has_sens ? &run->sens : NULL, run->cell_tally);
}

int oracle_cycle_finalize(OracleRun* run)
{
    run->bal.v[QSG_BAL_END] = run->processed.n;
    run->last = run->bal;
    memset(&run->bal, 0, sizeof(run->bal));
    run->bal.v[QSG_BAL_START] = run->last.v[QSG_BAL_END];
    memset(run->flux, 0, sizeof(double) * (size_t)run->pb->num_cells * run->pb->num_groups);
    /* the reference resets its cell tally every cycle (Tallies.cc:91) */
    if (run->cell_tally) memset(run->cell_tally, 0, sizeof(double) * (size_t)run->pb->num_cells);
    return 0;
}

int oracle_enable_exponential_tally(OracleRun* r)
{
    if (!r->cell_tally) r->cell_tally = (double*)calloc((size_t)r->pb->num_cells, sizeof(double));
    return r->cell_tally ? 0 : -1;
}

int oracle_read_cell_tally(const OracleRun* r, double* out)
{
    if (!r->cell_tally) return -1;
    memcpy(out, r->cell_tally, sizeof(double) * (size_t)r->pb->num_cells);
    return 0;
}

uint64_t oracle_num_processing(const OracleRun* r) { return r->processing.n; }
uint64_t oracle_num_processed(const OracleRun* r) { return r->processed.n; }
const OracleParticle* oracle_processing(const OracleRun* r) { return r->processing.p; }
const OracleParticle* oracle_processed(const OracleRun* r) { return r->processed.p; }
uint64_t oracle_warning_count(const OracleRun* r) { return r->warnings; }

int oracle_set_processing(OracleRun* r, const OracleParticle* p, uint64_t n)
{
    if (store_reserve(&r->processing, n)) return -1;
    memcpy(r->processing.p, p, n * sizeof(OracleParticle));
    for (uint64_t i = 0; i < n; i++) store_set_scores(&r->processing, i, NULL);
    r->processing.n = n;
    return 0;
}

int oracle_enable_sensitivity(OracleRun* r, const OracleSens* spec)
{
    if (!spec || spec->K < 1 || spec->K > QSG_MAX_PARAMS || r->has_sens) return -1;
    if (r->processing.n || r->processed.n) return -1;   /* before the first cycle */
    r->sens = *spec;
    const size_t C = (size_t)r->pb->num_cells, K = (size_t)spec->K;
    r->sens.flux_cell = (double*)calloc(C, sizeof(double));
    r->sens.dflux = (double*)calloc(C * K, sizeof(double));
    r->sens.leak = (double*)calloc(1, sizeof(double));
    r->sens.dleak = (double*)calloc(K, sizeof(double));
    if (!r->sens.flux_cell || !r->sens.dflux || !r->sens.leak || !r->sens.dleak) return -1;
    r->has_sens = 1;
    free(r->processing.p);
    free(r->processed.p);
    memset(&r->processing, 0, sizeof(Store));
    memset(&r->processed, 0, sizeof(Store));
    r->processing.K = r->processed.K = spec->K;
    return 0;
}

int oracle_read_sensitivity(const OracleRun* r, double* flux_cell, double* dflux, double* leak, double* dleak)
{
    if (!r->has_sens) return -1;
    const size_t C = (size_t)r->pb->num_cells, K = (size_t)r->sens.K;
    if (flux_cell) memcpy(flux_cell, r->sens.flux_cell, C * sizeof(double));
    if (dflux) memcpy(dflux, r->sens.dflux, C * K * sizeof(double));
    if (leak) memcpy(leak, r->sens.leak, sizeof(double));
    if (dleak) memcpy(dleak, r->sens.dleak, K * sizeof(double));
    return 0;
}

const double* oracle_processing_scores(const OracleRun* r) { return r->processing.sc; }
const double* oracle_processed_scores(const OracleRun* r) { return r->processed.sc; }

void oracle_balance(const OracleRun* r, uint64_t* out) { memcpy(out, r->bal.v, sizeof(r->bal.v)); }
void oracle_last_balance(const OracleRun* r, uint64_t* out) { memcpy(out, r->last.v, sizeof(r->last.v)); }
const double* oracle_flux(const OracleRun* r) { return r->flux; }

int oracle_track(const QsgProblem* pb, const OracleParticle* in, uint64_t n, OracleParticle* census_out,
                 uint64_t cap, uint64_t* n_census, uint64_t* balance13, double* flux, int nthreads)
{
    return oracle_track_cell_tally(pb, in, n, census_out, cap, n_census, balance13, flux, NULL, nthreads);
}

int oracle_track_cell_tally(const QsgProblem* pb, const OracleParticle* in, uint64_t n, OracleParticle* census_out,
                            uint64_t cap, uint64_t* n_census, uint64_t* balance13, double* flux, double* cell_tally,
                            int nthreads)
{
    Store processing = {0, 0, 0, NULL, 0}, census = {0, 0, 0, NULL, 0};
    if (store_reserve(&processing, n ? n : 1)) return -1;
    memcpy(processing.p, in, n * sizeof(OracleParticle));
    processing.n = n;
    Counters bal;
    memset(&bal, 0, sizeof(bal));
    uint64_t warnings = 0;
    int st = track_all(pb, &processing, &census, &bal, flux, &warnings, nthreads, NULL, cell_tally);
    for (int k = 0; k < QSG_BAL_COUNT; k++) balance13[k] += bal.v[k];
    uint64_t ncopy = census.n < cap ? census.n : cap;
    if (census_out && ncopy) memcpy(census_out, census.p, ncopy * sizeof(OracleParticle));
    *n_census = census.n;
    free(processing.p);
    free(census.p);
    if (st) return st;
    return census.n > cap ? -3 : 0;
}

int oracle_track_sens(const QsgProblem* pb, OracleSens* sens, const OracleParticle* in, const double* in_scores,
                      uint64_t n, OracleParticle* census_out, double* census_scores, uint64_t cap, uint64_t* n_census,
                      uint64_t* balance13, double* flux, int nthreads)
{
    if (!sens || sens->K < 1 || sens->K > QSG_MAX_PARAMS) return -1;
    const int K = sens->K;
    Store processing = {0, 0, 0, NULL, K}, census = {0, 0, 0, NULL, K};
    if (store_reserve(&processing, n ? n : 1)) return -1;
    memcpy(processing.p, in, n * sizeof(OracleParticle));
    for (uint64_t i = 0; i < n; i++) store_set_scores(&processing, i, in_scores ? in_scores + i * (size_t)K : NULL);
    processing.n = n;
    Counters bal;
    memset(&bal, 0, sizeof(bal));
    uint64_t warnings = 0;
    int st = track_all(pb, &processing, &census, &bal, flux, &warnings, nthreads, sens, NULL);
    for (int k = 0; k < QSG_BAL_COUNT; k++) balance13[k] += bal.v[k];
    uint64_t ncopy = census.n < cap ? census.n : cap;
    if (census_out && ncopy) memcpy(census_out, census.p, ncopy * sizeof(OracleParticle));
    if (census_scores && ncopy) memcpy(census_scores, census.sc, ncopy * (size_t)K * sizeof(double));
    *n_census = census.n;
    free(processing.p);
    free(processing.sc);
    free(census.p);
    free(census.sc);
    if (st) return st;
    return census.n > cap ? -3 : 0;
}
