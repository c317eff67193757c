// Device-side cycle set-up and finalisation, so that a whole cycle runs on the
// GPU without host round trips and can be captured in a CUDA graph:
//
//   qsg_cycle_init      cycleInit (main.cc:96-121): the previous census becomes
//                       the processing store (swapProcessingProcessedVaults,
//                       ParticleVaultContainer.cc:278-311), MC_SourceNow
//                       (MC_SourceNow.cc:28-164), PopulationControl
//                       (PopulationControl.cc:20-122) and
//                       RouletteLowWeightParticles (PopulationControl.cc:127-171)
//   qsg_cycle_finalize  cycleFinalize (main.cc:310-324) with the replica sum and
//                       reset of Tallies::CycleFinalize (Tallies.cc:25-98); each
//                       problem's 13 counters and scalar-flux total
//                       (Tallies::ScalarFluxSum, Tallies.cc:146-171) go to a
//                       device-resident history.
//   qsg_run_cycles      init + tracking passes + finalize for n cycles, each
//                       cycle replayed from a captured CUDA graph.
//
// Everything here is per problem, so one handle can hold a batch of
// independent problems (qsg_batch_create); a single problem is a batch of one.
// What is constant over the run is computed once on the host at
// qsg_configure_cycle_batch: a problem's source particle weight and per-cell
// source counts depend only on its cell volumes, source rates, dt and
// nParticles.  Each source particle, split and roulette decision draws only
// from its own random stream, so the set of particles a cycle produces does
// not depend on the order the device produces them in.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "handle.cuh"
#include "qsg.h"
#include "status.h"
#include "track_device.cuh"

namespace qsg {
namespace {

constexpr int kInitBlock = 256;
constexpr int kFluxPartials = 256;   // blocks per problem for the flux total (fixed shape: reproducible)

struct CycleArgs {
    CycleScalars* sc;
    unsigned long long* balance;       // [replicas][P][13]
    unsigned int* flags;
    const int32_t* cell_problem;       // null: one problem
    int32_t num_problems;
    // per problem
    const double* weight;              // source particle weight
    const double* e_min;
    const double* e_max;
    const double* low_cut;             // lowWeightCutoff
    const uint64_t* target;            // nParticles
    const uint64_t* n_source;
    const uint64_t* seed_offset;
    const int32_t* load_balance;
    unsigned long long* carry;         // census count carried into the cycle
    double* factor;                    // population-control factor of the running cycle
};

__device__ __forceinline__ int problem_of(const CycleArgs& a, int cell)
{
    return a.cell_problem ? __ldg(a.cell_problem + cell) : 0;
}

// Census -> processing bookkeeping; START / SOURCE counters and the
// population-control factor of every problem (PopulationControl.cc:24-58).
__global__ void cycle_begin_kernel(CycleArgs a, unsigned long long* processing_count,
                                   unsigned long long* processed_count, unsigned long long n_source_total)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long start = *processing_count;
        a.sc->start = start;
        a.sc->source_round = a.sc->source_calls;
        a.sc->source_calls += 1;
        *processing_count = start + n_source_total;
        *processed_count = 0;
    }
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.num_problems; p += gridDim.x * blockDim.x) {
        const unsigned long long start = a.carry[p];
        unsigned long long* bal = a.balance + (int64_t)p * QSG_BAL_COUNT;
        bal[QSG_BAL_START] = start;                 // main.cc:110 sets _start after the swap
        bal[QSG_BAL_SOURCE] += a.n_source[p];
        const unsigned long long current = start + a.n_source[p];
        double f;
        if (a.load_balance[p]) {
            const double target = ceil((double)a.target[p] / (double)1);
            const int cur = (int)current;
            f = (cur != 0) ? target / (double)cur : 1.0;
        } else {
            f = (double)a.target[p] / (double)current;
        }
        a.factor[p] = f;
    }
}

struct SourceArgs {
    DevTables t;
    DevStore out;
    CycleArgs c;
    const int32_t* src_cell;
    const uint64_t* src_cell_offset;
    const int32_t* src_cell_count;
    const uint64_t* cell_id;
    const double* cell_volume;
    uint64_t n_source;
};

// MCT_Cell_Volume_3D_G_vector_tetDet, MCT.cc:633-648: 6x the signed tet volume.
__device__ __forceinline__ double tet_det(const double* a, const double* b, const double* c, const double* d)
{
    double v0x = a[0] - d[0], v0y = a[1] - d[1], v0z = a[2] - d[2];
    double v1x = b[0] - d[0], v1y = b[1] - d[1], v1z = b[2] - d[2];
    double v2x = c[0] - d[0], v2y = c[1] - d[1], v2z = c[2] - d[2];
    return v0z * (v1x * v2y - v1y * v2x) + v0y * (v1z * v2x - v1x * v2z) + v0x * (v1y * v2z - v1z * v2y);
}

// One source particle per thread: MC_SourceNow's inner loop body
// (MC_SourceNow.cc:90-131) with MCT_Generate_Coordinate_3D_G (MCT.cc:143-226)
// and DirectionCosine::Sample_Isotropic (DirectionCosine.cc:5-12).
__global__ void __launch_bounds__(kInitBlock) source_kernel(SourceArgs a)
{
    const uint64_t t = (uint64_t)blockIdx.x * kInitBlock + threadIdx.x;
    if (t >= a.n_source) return;
    const DevTables& tb = a.t;
    const int cell = a.src_cell[t];
    const int prob = problem_of(a.c, cell);
    const uint64_t k = t - a.src_cell_offset[cell];
    // the cell's source tally counts every particle it ever sourced
    // (MC_SourceNow.cc:90-93); the offset is 0 unless a batch asks otherwise
    uint64_t seed0 = a.c.sc->source_round * (uint64_t)a.src_cell_count[cell] + k;
    seed0 += a.cell_id[cell] + a.c.seed_offset[prob];
    Particle p;
    p.seed = rng_spawn(seed0);
    p.identifier = seed0;
    // position: pick a tet by volume, then a uniform point inside it
    const double* center = tb.cell_center + 3 * (int64_t)cell;
    const double* nodes = tb.cell_nodes + (int64_t)cell * (kCellPoints * 3);
    double c[3] = {center[0], center[1], center[2]};
    double which_volume = rng_sample(p.seed) * 6.0 * a.cell_volume[cell];
    double current = 0.0;
    int facet = -1;
    const double *p0 = nullptr, *p1 = nullptr, *p2 = nullptr;
    while (current < which_volume) {
        facet++;
        if (facet == kFacets) break;
        p0 = nodes + 3 * kFacetLocal[facet][0];
        p1 = nodes + 3 * kFacetLocal[facet][1];
        p2 = nodes + 3 * kFacetLocal[facet][2];
        current += tet_det(p0, p1, p2, c);
    }
    double r1 = rng_sample(p.seed);
    double r2 = rng_sample(p.seed);
    double r3 = rng_sample(p.seed);
    if (r1 + r2 > 1.0) {
        r1 = 1.0 - r1;
        r2 = 1.0 - r2;
    }
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
    if (p0) {
        p.x = (r4 * c[0] + r1 * p0[0] + r2 * p1[0] + r3 * p2[0]);
        p.y = (r4 * c[1] + r1 * p0[1] + r2 * p1[1] + r3 * p2[1]);
        p.z = (r4 * c[2] + r1 * p0[2] + r2 * p1[2] + r3 * p2[2]);
    } else {
        p.x = p.y = p.z = 0.0;
    }
    // isotropic direction
    p.gamma = 1.0 - 2.0 * rng_sample(p.seed);
    double sine_gamma = sqrt((1.0 - (p.gamma * p.gamma)));
    double phi = kPi * (2.0 * rng_sample(p.seed) - 1.0);
    p.alpha = sine_gamma * QSG_COS(phi);
    p.beta = sine_gamma * QSG_SIN(phi);
    // energy uniform in [eMin, eMax]; Get_Speed_From_Energy (MC_SourceNow.cc:169-177)
    p.kinetic_energy = (a.c.e_max[prob] - a.c.e_min[prob]) * rng_sample(p.seed) + a.c.e_min[prob];
    const double m = kNeutronRestMassEnergy;
    const double E = p.kinetic_energy;
    double speed = kSpeedOfLight * sqrt(E * (E + 2.0 * (m)) / ((E + m) * (E + m)));
    p.vx = speed * p.alpha;
    p.vy = speed * p.beta;
    p.vz = speed * p.gamma;
    p.domain = 0;
    p.cell = cell;
    p.weight = a.c.weight[prob];
    p.num_mean_free_paths = -1.0 * QSG_LOG(rng_sample(p.seed));
    p.time_to_census = tb.time_step * rng_sample(p.seed);
    p.age = 0.0;
    p.num_segments = 0.0;
    p.last_event = QSG_EVENT_CENSUS;   // MC_Particle default
    p.num_collisions = 0;
    p.breed = 0;
    p.species = 0;
    const uint64_t slot = a.c.sc->start + t;
    if (slot < a.out.capacity) {
        store_particle(a.out, slot, p);
        // a source particle starts with zero sensitivity scores
        for (int k = 0; k < a.out.score_fields; k++) a.out.score[(uint64_t)k * a.out.capacity + slot] = 0.0;
    } else {
        atomicOr(a.c.flags, QSG_DEV_STORE_OVERFLOW);
    }
}

__device__ __forceinline__ void load_record(const DevStore& s, uint64_t i, Particle& p)
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
}

// RouletteLowWeightParticles' per-particle body (PopulationControl.cc:153-167);
// returns whether the particle survives.
__device__ __forceinline__ bool roulette(double low_cut, double weight_cutoff, Particle& p, uint32_t& rr)
{
    if (!(low_cut > 0.0)) return true;
    if (p.weight <= weight_cutoff) {
        double r = rng_sample(p.seed);
        if (r <= low_cut) {
            p.weight /= low_cut;
        } else {
            rr++;
            return false;
        }
    }
    return true;
}

// Append p to `out`; its sensitivity scores (if the stores carry them) are
// those of particle i of `in`, the particle it was copied or split from.
__device__ __forceinline__ void emit(const DevStore& out, unsigned int* flags, const Particle& p, const DevStore& in,
                                     uint64_t i)
{
    uint64_t slot = append_slot(out);
    if (slot < out.capacity) {
        store_particle(out, slot, p);
        for (int k = 0; k < out.score_fields; k++)
            out.score[(uint64_t)k * out.capacity + slot] =
                k < in.score_fields ? in.score[(uint64_t)k * in.capacity + i] : 0.0;
    } else {
        atomicOr(flags, QSG_DEV_STORE_OVERFLOW);
    }
}

// PopulationControlGuts (PopulationControl.cc:71-122) followed by the low-weight
// roulette, fused: every particle of `in` is visited once; survivors and split
// copies are appended to `out`.  RR / SPLIT counts per problem gather in shared
// memory (when the batch fits) before one global add per block.
__global__ void __launch_bounds__(kInitBlock) population_kernel(CycleArgs a, DevStore in, DevStore out)
{
    extern __shared__ unsigned long long s_rr[];   // [P][2] when P <= kSmemProblems
    const bool use_smem = a.num_problems <= kSmemProblems;
    if (use_smem)
        for (int k = threadIdx.x; k < 2 * a.num_problems; k += kInitBlock) s_rr[k] = 0;
    __syncthreads();
    // a store that overflowed holds `capacity` particles (the writers raised
    // QSG_DEV_STORE_OVERFLOW)
    const uint64_t n = min((uint64_t)*in.count, in.capacity);
    for (uint64_t i = (uint64_t)blockIdx.x * kInitBlock + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kInitBlock) {
        Particle p;
        load_record(in, i, p);
        const int prob = problem_of(a, p.cell);
        const double factor = a.factor[prob];
        const double low_cut = a.low_cut[prob];
        const double weight_cutoff = low_cut * a.weight[prob];   // PopulationControl.cc:142-143
        uint32_t rr = 0, split_count = 0;
        bool survive = true;
        if (factor != 1.0) {
            double r = rng_sample(p.seed);
            if (factor < 1) {
                if (r > factor) {
                    survive = false;
                    rr++;
                } else {
                    p.weight /= factor;
                }
            } else if (factor > 1) {
                int split = (int)floor(factor);
                if (r > (factor - split)) split--;
                p.weight /= factor;
                Particle child = p;
                for (int k = 0; k < split; k++) {
                    split_count++;
                    child.seed = rng_spawn(p.seed);
                    child.identifier = child.seed;
                    Particle c2 = child;
                    if (roulette(low_cut, weight_cutoff, c2, rr)) emit(out, a.flags, c2, in, i);
                }
            }
        }
        if (survive && roulette(low_cut, weight_cutoff, p, rr)) emit(out, a.flags, p, in, i);
        if (rr | split_count) {
            if (use_smem) {
                if (rr) atomicAdd(&s_rr[2 * prob], (unsigned long long)rr);
                if (split_count) atomicAdd(&s_rr[2 * prob + 1], (unsigned long long)split_count);
            } else {
                if (rr) atomicAdd(a.balance + (int64_t)prob * QSG_BAL_COUNT + QSG_BAL_RR, (unsigned long long)rr);
                if (split_count)
                    atomicAdd(a.balance + (int64_t)prob * QSG_BAL_COUNT + QSG_BAL_SPLIT,
                              (unsigned long long)split_count);
            }
        }
    }
    if (use_smem) {
        __syncthreads();
        for (int k = threadIdx.x; k < 2 * a.num_problems; k += kInitBlock) {
            const unsigned long long v = s_rr[k];
            if (v) atomicAdd(a.balance + (int64_t)(k / 2) * QSG_BAL_COUNT + ((k & 1) ? QSG_BAL_SPLIT : QSG_BAL_RR), v);
        }
    }
}

// Fixed-shape partial sums of each problem's flux range (all replicas):
// block (b, p) sums chunk b of problem p.
__global__ void __launch_bounds__(256) flux_partial_kernel(const double* flux, const int32_t* cell_offset,
                                                           int groups, int replicas, int64_t replica_stride,
                                                           double* partial)
{
    __shared__ double s[256];
    const int prob = blockIdx.y;
    const uint64_t lo_all = (uint64_t)cell_offset[prob] * groups, hi_all = (uint64_t)cell_offset[prob + 1] * groups;
    const uint64_t n = hi_all - lo_all;
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t lo = lo_all + (uint64_t)blockIdx.x * chunk;
    const uint64_t hi = min(lo + chunk, hi_all);
    double acc = 0.0;
    for (int r = 0; r < replicas; r++)
        for (uint64_t i = lo + threadIdx.x; i < hi; i += 256) acc += flux[r * replica_stride + i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[(int64_t)prob * gridDim.x + blockIdx.x] = s[0];
}

// Fluence::compute (Tallies.cc:100-118) after the replica sum of
// Tallies.cc:84-89: each cell's scalar flux summed over replicas in replica
// order, then added group by group, in group order, to the cell's fluence.
__global__ void fluence_kernel(const double* flux, int64_t cells, int groups, int replicas, int64_t replica_stride,
                               double* fluence)
{
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x) {
        const double* row = flux + c * groups;
        double f = fluence[c];
        for (int g = 0; g < groups; g++) {
            double v = row[g];
            for (int r = 1; r < replicas; r++) v += row[r * replica_stride + g];
            f += v;
        }
        fluence[c] = f;
    }
}

// EnergySpectrum::UpdateSpectrum (EnergySpectrum.cc:12-36): the energy group
// (NuclearData::getEnergyGroup, as MC_Load_Particle computes it) of every
// particle of a store, counted per problem into [problems][G+1].
__global__ void spectrum_kernel(DevTables t, DevStore s, const int32_t* cell_problem, unsigned long long* spectrum)
{
    const uint64_t n = min((uint64_t)*s.count, s.capacity);
    const int width = t.num_groups + 1;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const int g = energy_group(t, s.kinetic_energy[i]);
        const int prob = cell_problem ? cell_problem[s.cell[i]] : 0;
        atomicAdd(spectrum + (int64_t)prob * width + g, 1ull);
    }
}

// Block p records problem p's cycle: counters summed over replicas, END = its
// census count (main.cc:314), the flux total; carries the census count into
// the next cycle and clears the counters.
__global__ void cycle_finalize_kernel(CycleArgs a, int replicas, const double* partial, int n_partial,
                                      CycleRecord* history)
{
    const int prob = blockIdx.x;
    CycleRecord* rec = history + a.sc->cycle * (uint64_t)a.num_problems + prob;
    if (threadIdx.x < QSG_BAL_COUNT) {
        unsigned long long s = 0;
        for (int r = 0; r < replicas; r++)
            s += a.balance[((int64_t)r * a.num_problems + prob) * QSG_BAL_COUNT + threadIdx.x];
        rec->balance[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        rec->balance[QSG_BAL_END] = rec->balance[QSG_BAL_CENSUS];
        a.carry[prob] = rec->balance[QSG_BAL_CENSUS];
        double total = 0.0;
        for (int k = 0; k < n_partial; k++) total += partial[(int64_t)prob * n_partial + k];
        rec->flux_total = total;
    }
    for (int k = threadIdx.x; k < replicas * QSG_BAL_COUNT; k += blockDim.x)
        a.balance[((int64_t)(k / QSG_BAL_COUNT) * a.num_problems + prob) * QSG_BAL_COUNT + k % QSG_BAL_COUNT] = 0;
}

__global__ void cycle_advance_kernel(CycleScalars* sc) { sc->cycle += 1; }

CycleArgs cycle_args(QsgHandle* h)
{
    CycleArgs a;
    a.sc = h->scalars.ptr;
    a.balance = h->balance.ptr;
    a.flags = h->flags.ptr;
    a.cell_problem = h->num_problems > 1 ? h->cell_problem.ptr : nullptr;
    a.num_problems = h->num_problems;
    a.weight = h->prob_weight.ptr;
    a.e_min = h->prob_emin.ptr;
    a.e_max = h->prob_emax.ptr;
    a.low_cut = h->prob_lowcut.ptr;
    a.target = h->prob_target.ptr;
    a.n_source = h->prob_nsource.ptr;
    a.seed_offset = h->prob_seed_offset.ptr;
    a.load_balance = h->prob_load_balance.ptr;
    a.carry = h->prob_carry.ptr;
    a.factor = h->prob_factor.ptr;
    return a;
}

// Host-side preparation that may allocate (and therefore synchronise); never
// called while a stream is being captured.
int cycle_prepare(QsgHandle* h)
{
    int st;
    const uint64_t need = h->known_census + h->n_source;
    if ((st = h->processed.reserve(need)) || (st = h->extra.reserve(std::max<uint64_t>(need, 2 * h->n_target))))
        return st;
    if (h->cycles_finalized >= h->history_capacity) {
        DevBuf<CycleRecord> bigger;
        const uint64_t cap = 2 * h->history_capacity;
        if ((st = bigger.alloc(cap * h->num_problems))) return st;
        QSG_CUDA(cudaDeviceSynchronize());
        QSG_CUDA(cudaMemcpy(bigger.ptr, h->history.ptr, h->history_capacity * h->num_problems * sizeof(CycleRecord),
                            cudaMemcpyDeviceToDevice));
        h->history.free();
        h->history = bigger;
        bigger.ptr = nullptr;
        h->history_capacity = cap;
    }
    return QSG_OK;
}

int cycle_init_enqueue(QsgHandle* h, cudaStream_t s)
{
    std::swap(h->processing, h->processed);
    CycleArgs ca = cycle_args(h);
    cycle_begin_kernel<<<1, 256, 0, s>>>(ca, h->processing.count, h->processed.count,
                                         (unsigned long long)h->n_source);
    QSG_CUDA(cudaGetLastError());
    if (h->n_source) {
        SourceArgs a;
        a.t = h->tables;
        a.out = h->processing.view;
        a.c = ca;
        a.src_cell = h->src_cell.ptr;
        a.src_cell_offset = h->src_cell_offset.ptr;
        a.src_cell_count = h->src_cell_count.ptr;
        a.cell_id = h->cell_id.ptr;
        a.cell_volume = h->cell_volume.ptr;
        a.n_source = h->n_source;
        unsigned blocks = (unsigned)((h->n_source + kInitBlock - 1) / kInitBlock);
        source_kernel<<<blocks, kInitBlock, 0, s>>>(a);
        QSG_CUDA(cudaGetLastError());
    }
    QSG_CUDA(cudaMemsetAsync(h->extra.count, 0, sizeof(unsigned long long), s));
    const size_t smem = h->num_problems <= kSmemProblems ? 2 * h->num_problems * sizeof(unsigned long long) : 0;
    population_kernel<<<h->num_sms * 8, kInitBlock, smem, s>>>(ca, h->processing.view, h->extra.view);
    QSG_CUDA(cudaGetLastError());
    std::swap(h->processing, h->extra);
    h->processing_on_device = true;
    return QSG_OK;
}

int cycle_finalize_enqueue(QsgHandle* h, cudaStream_t s)
{
    CycleArgs ca = cycle_args(h);
    const int64_t stride = (int64_t)h->num_cells * h->num_groups;
    if (h->observe_flags & QSG_OBSERVE_FLUENCE) {
        fluence_kernel<<<h->num_sms * 4, 128, 0, s>>>(h->flux.ptr, h->num_cells, h->num_groups, h->flux_replicas,
                                                      stride, h->fluence.ptr);
        QSG_CUDA(cudaGetLastError());
    }
    if (h->observe_flags & QSG_OBSERVE_SPECTRUM) {
        const int32_t* cp = h->num_problems > 1 ? h->cell_problem.ptr : nullptr;
        spectrum_kernel<<<h->num_sms * 4, 256, 0, s>>>(h->tables, h->processed.view, cp, h->spectrum.ptr);
        spectrum_kernel<<<h->num_sms, 256, 0, s>>>(h->tables, h->processing.view, cp, h->spectrum.ptr);
        QSG_CUDA(cudaGetLastError());
    }
    flux_partial_kernel<<<dim3(kFluxPartials, h->num_problems), 256, 0, s>>>(
        h->flux.ptr, h->prob_cell_offset.ptr, h->num_groups, h->flux_replicas, stride, h->flux_partial.ptr);
    QSG_CUDA(cudaGetLastError());
    cycle_finalize_kernel<<<h->num_problems, 64, 0, s>>>(ca, h->balance_replicas, h->flux_partial.ptr, kFluxPartials,
                                                         h->history.ptr);
    QSG_CUDA(cudaGetLastError());
    cycle_advance_kernel<<<1, 1, 0, s>>>(h->scalars.ptr);
    QSG_CUDA(cudaGetLastError());
    QSG_CUDA(cudaMemsetAsync(h->flux.ptr, 0, (size_t)h->flux_replicas * stride * sizeof(double), s));
    // the reference's cycleFinalize resets its cell tally too (Tallies.cc:91)
    if (h->exp_tally) QSG_CUDA(cudaMemsetAsync(h->cell_tally.ptr, 0, h->cell_tally.n * sizeof(double), s));
    h->cycles_finalized++;
    return QSG_OK;
}

}  // namespace
}  // namespace qsg

using namespace qsg;

extern "C" int qsg_set_observers(QsgHandle* h, int32_t flags)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_set_observers: null handle");
    if (flags & ~(QSG_OBSERVE_FLUENCE | QSG_OBSERVE_SPECTRUM))
        return fail(QSG_ERR_INVALID, "qsg_set_observers: unknown flag bits 0x%x", (unsigned)flags);
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    if (flags & QSG_OBSERVE_FLUENCE) {
        if ((st = h->fluence.alloc((size_t)h->num_cells))) return st;
        QSG_CUDA(cudaMemset(h->fluence.ptr, 0, h->fluence.n * sizeof(double)));
    }
    if (flags & QSG_OBSERVE_SPECTRUM) {
        if ((st = h->spectrum.alloc((size_t)h->num_problems * (h->num_groups + 1)))) return st;
        QSG_CUDA(cudaMemset(h->spectrum.ptr, 0, h->spectrum.n * sizeof(unsigned long long)));
    }
    h->observe_flags = flags;
    h->clear_graphs();   // captured cycles carry the old finalize sequence
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_read_observers(QsgHandle* h, double* fluence, uint64_t* spectrum)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_read_observers: null handle");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    if (fluence) {
        if (!(h->observe_flags & QSG_OBSERVE_FLUENCE)) return fail(QSG_ERR_INVALID, "qsg_read_observers: fluence is off");
        QSG_CUDA(cudaMemcpy(fluence, h->fluence.ptr, h->fluence.n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (spectrum) {
        if (!(h->observe_flags & QSG_OBSERVE_SPECTRUM)) return fail(QSG_ERR_INVALID, "qsg_read_observers: spectrum is off");
        QSG_CUDA(cudaMemcpy(spectrum, h->spectrum.ptr, h->spectrum.n * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    }
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_configure_cycle_batch(QsgHandle* h, const QsgCycleConfig* cfgs, const uint64_t* seed_offsets)
{
    QSG_API_BEGIN
    if (!h || !cfgs) return fail(QSG_ERR_INVALID, "qsg_configure_cycle: null argument");
    const int P = h->num_problems;
    if ((int64_t)h->h_cell_volume.size() != h->num_cells || (int64_t)h->h_cell_id.size() != h->num_cells)
        return fail(QSG_ERR_INVALID, "qsg_configure_cycle: the problem given to qsg_create had no cell_volume / cell_id");
    for (int p = 0; p < P; p++) {
        if (!cfgs[p].source_rate) return fail(QSG_ERR_INVALID, "qsg_configure_cycle: problem %d has no source rates", p);
        if (cfgs[p].n_particles == 0)
            return fail(QSG_ERR_INVALID, "qsg_configure_cycle: problem %d needs n_particles > 0", p);
    }
    int st = set_device(h);
    if (st) return st;
    const int64_t C = h->num_cells;
    const double dt = h->tables.time_step;
    std::vector<double> weight(P), emin(P), emax(P), lowcut(P);
    std::vector<uint64_t> target(P), nsrc(P), seedoff(P);
    std::vector<int32_t> lb(P), count(C), cell_off(P + 1);
    std::vector<uint64_t> offset(C);
    uint64_t n_source = 0;
    for (int p = 0; p < P; p++) {
        const QsgCycleConfig& cf = cfgs[p];
        const int32_t c0 = h->h_problem_cell_offset[p], c1 = h->h_problem_cell_offset[p + 1];
        const int32_t m0 = h->h_problem_material_offset[p];
        cell_off[p] = c0;
        // MC_SourceNow.cc:35-64: total source weight in cell order, particle weight
        double total_weight = 0;
        for (int64_t c = c0; c < c1; c++)
            total_weight += h->h_cell_volume[c] * cf.source_rate[h->h_cell_material[c] - m0] * dt;
        double source_fraction = 0.1;
        double spw = total_weight / (source_fraction * cf.n_particles);
        uint64_t ns = 0;
        for (int64_t c = c0; c < c1; c++) {
            double cell_weight = h->h_cell_volume[c] * cf.source_rate[h->h_cell_material[c] - m0] * dt;
            double cell_num_float = cell_weight / spw;
            int n = (int)cell_num_float;
            if (n < 0) n = 0;
            count[c] = n;
            offset[c] = n_source;
            n_source += (uint64_t)n;
            ns += (uint64_t)n;
        }
        weight[p] = spw;
        emin[p] = cf.e_min;
        emax[p] = cf.e_max;
        lowcut[p] = cf.low_weight_cutoff;
        target[p] = cf.n_particles;
        nsrc[p] = ns;
        seedoff[p] = seed_offsets ? seed_offsets[p] : 0;
        lb[p] = cf.load_balance;
    }
    cell_off[P] = (int32_t)C;
    std::vector<int32_t> src_cell(n_source);
    for (int64_t c = 0; c < C; c++)
        for (int32_t k = 0; k < count[c]; k++) src_cell[offset[c] + k] = (int32_t)c;
    std::vector<double> vol(h->h_cell_volume.begin(), h->h_cell_volume.end());
    std::vector<uint64_t> ids(h->h_cell_id.begin(), h->h_cell_id.end());
    std::vector<unsigned long long> carry(P, 0);
    std::vector<double> factor(P, 1.0);
    if ((st = h->src_cell.upload(src_cell)) || (st = h->src_cell_count.upload(count)) ||
        (st = h->src_cell_offset.upload(offset)) || (st = h->cell_volume.upload(vol)) ||
        (st = h->cell_id.upload(ids)) || (st = h->prob_weight.upload(weight)) || (st = h->prob_emin.upload(emin)) ||
        (st = h->prob_emax.upload(emax)) || (st = h->prob_lowcut.upload(lowcut)) ||
        (st = h->prob_target.upload(target)) || (st = h->prob_nsource.upload(nsrc)) ||
        (st = h->prob_seed_offset.upload(seedoff)) || (st = h->prob_load_balance.upload(lb)) ||
        (st = h->prob_carry.upload(carry)) || (st = h->prob_factor.upload(factor)) ||
        (st = h->prob_cell_offset.upload(cell_off)))
        return st;
    uint64_t n_target = 0, cap = 0;
    for (int p = 0; p < P; p++) {
        n_target += target[p];
        cap += cfgs[p].store_capacity ? cfgs[p].store_capacity : 4 * (target[p] + nsrc[p]);
    }
    h->n_target = n_target;
    h->source_particle_weight = weight[0];
    h->n_source = n_source;
    if ((st = h->processing.reserve(cap)) || (st = h->processed.reserve(cap)) || (st = h->extra.reserve(cap)))
        return st;
    if ((st = h->flux_partial.alloc((size_t)kFluxPartials * P))) return st;
    if (!h->history.ptr) {
        if ((st = h->history.alloc(1024 * (size_t)P))) return st;
        h->history_capacity = 1024;
    }
    h->cycle_configured = true;
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_configure_cycle(QsgHandle* h, const QsgCycleConfig* cfg)
{
    if (h && h->num_problems != 1)
        return fail(QSG_ERR_INVALID, "qsg_configure_cycle: a batch needs qsg_configure_cycle_batch");
    return qsg_configure_cycle_batch(h, cfg, nullptr);
}

extern "C" int qsg_cycle_init(QsgHandle* h, void* stream)
{
    QSG_API_BEGIN
    QSG_RANGE("cycleInit");
    if (!h) return fail(QSG_ERR_INVALID, "qsg_cycle_init: null handle");
    if (!h->cycle_configured) return fail(QSG_ERR_INVALID, "qsg_cycle_init: call qsg_configure_cycle first");
    int st = set_device(h);
    if (st) return st;
    if ((st = cycle_prepare(h))) return st;
    return cycle_init_enqueue(h, static_cast<cudaStream_t>(stream));
    QSG_API_END
}

extern "C" int qsg_cycle_finalize(QsgHandle* h, void* stream)
{
    QSG_API_BEGIN
    QSG_RANGE("cycleFinalize");
    if (!h) return fail(QSG_ERR_INVALID, "qsg_cycle_finalize: null handle");
    if (!h->cycle_configured) return fail(QSG_ERR_INVALID, "qsg_cycle_finalize: call qsg_configure_cycle first");
    int st = set_device(h);
    if (st) return st;
    if ((st = cycle_prepare(h))) return st;
    return cycle_finalize_enqueue(h, static_cast<cudaStream_t>(stream));
    QSG_API_END
}

// Key of the role -> store permutation (the stores swap roles during a cycle;
// a graph captured for one permutation only fits cycles that start from it).
static bool same_roles(const QsgHandle* h, const QsgHandle::GraphEntry& g)
{
    return g.proc == h->processing.base && g.done == h->processed.base && g.extra == h->extra.base &&
           g.generation == h->store_generation;
}

extern "C" int qsg_run_cycles(QsgHandle* h, int32_t n_cycles, int32_t use_graph, void* stream)
{
    QSG_API_BEGIN
    QSG_RANGE("qsg_run_cycles");
    if (!h || n_cycles < 0) return fail(QSG_ERR_INVALID, "qsg_run_cycles: bad argument");
    if (!h->cycle_configured) return fail(QSG_ERR_INVALID, "qsg_run_cycles: call qsg_configure_cycle first");
    int st = set_device(h);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int c = 0; c < n_cycles; c++) {
        // allocation-free from here on unless a store or the history must grow;
        // a reallocated store invalidates every captured graph
        const uint64_t gen_before = h->processing.generation + h->processed.generation + h->extra.generation;
        if ((st = cycle_prepare(h))) return st;
        const uint64_t gen_after = h->processing.generation + h->processed.generation + h->extra.generation;
        if (gen_after != gen_before) {
            h->store_generation++;
            h->clear_graphs();
        }
        if (!use_graph) {
            if ((st = cycle_init_enqueue(h, s)) || (st = track_passes_async(h, s)) ||
                (st = cycle_finalize_enqueue(h, s)))
                return st;
            continue;
        }
        // the history may be reallocated: graphs captured with the old buffer are stale
        if (h->history.ptr != h->graph_history) {
            h->clear_graphs();
            h->graph_history = h->history.ptr;
        }
        QsgHandle::GraphEntry* entry = nullptr;
        for (auto& g : h->graphs)
            if (same_roles(h, g)) entry = &g;
        if (!entry) {
            QsgHandle::GraphEntry g;
            g.proc = h->processing.base;
            g.done = h->processed.base;
            g.extra = h->extra.base;
            g.generation = h->store_generation;
            if (!h->capture_stream) QSG_CUDA(cudaStreamCreateWithFlags(&h->capture_stream, cudaStreamNonBlocking));
            // capture one cycle (it swaps the host-side roles as it goes; restore
            // them afterwards so the graph is launched from the same roles)
            Store sp = h->processing, sd = h->processed, se = h->extra;
            const uint64_t fin = h->cycles_finalized;
            QSG_CUDA(cudaStreamBeginCapture(h->capture_stream, cudaStreamCaptureModeThreadLocal));
            int cst = cycle_init_enqueue(h, h->capture_stream);
            if (!cst) cst = track_passes_async(h, h->capture_stream);
            if (!cst) cst = cycle_finalize_enqueue(h, h->capture_stream);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(h->capture_stream, &graph);
            g.after_proc = h->processing;
            g.after_done = h->processed;
            g.after_extra = h->extra;
            h->processing = sp;
            h->processed = sd;
            h->extra = se;
            h->cycles_finalized = fin;
            if (cst) {
                if (graph) cudaGraphDestroy(graph);
                return cst;
            }
            if (e != cudaSuccess) return fail(QSG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&g.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return fail(QSG_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
            h->graphs.push_back(g);
            entry = &h->graphs.back();
        }
        QSG_CUDA(cudaGraphLaunch(entry->exec, s));
        h->processing = entry->after_proc;
        h->processed = entry->after_done;
        h->extra = entry->after_extra;
        h->cycles_finalized++;
        h->processing_on_device = true;
    }
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_cycle_history(QsgHandle* h, uint64_t first, uint64_t n, uint64_t* balance, double* flux_total)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_cycle_history: null handle");
    if (first + n > h->cycles_finalized)
        return fail(QSG_ERR_INVALID, "qsg_cycle_history: only %llu cycles finalised",
                    (unsigned long long)h->cycles_finalized);
    int st = set_device(h);
    if (st) return st;
    if (n == 0) return QSG_OK;
    const int P = h->num_problems;
    std::vector<CycleRecord> rec(n * P);
    QSG_CUDA(cudaDeviceSynchronize());
    QSG_CUDA(cudaMemcpy(rec.data(), h->history.ptr + first * P, n * P * sizeof(CycleRecord), cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < n * P; i++) {
        if (balance)
            for (int k = 0; k < QSG_BAL_COUNT; k++) balance[i * QSG_BAL_COUNT + k] = rec[i].balance[k];
        if (flux_total) flux_total[i] = rec[i].flux_total;
    }
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_get_processing(QsgHandle* h, QsgParticleSoA* host, uint64_t cap, uint64_t* n_out)
{
    QSG_API_BEGIN
    if (!h || !n_out) return fail(QSG_ERR_INVALID, "qsg_get_processing: null argument");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    unsigned long long c = 0;
    QSG_CUDA(cudaMemcpy(&c, h->processing.count, sizeof(c), cudaMemcpyDeviceToHost));
    *n_out = c;
    if (c > cap) return fail(QSG_ERR_CAPACITY, "qsg_get_processing: %llu particles, capacity %llu", c,
                             (unsigned long long)cap);
    if (c > h->processing.capacity)
        return fail(QSG_ERR_DEVICE, "qsg_get_processing: store overflowed (%llu > %llu)", c,
                    (unsigned long long)h->processing.capacity);
    return copy_store_to_host(h->processing.view, host, c);
    QSG_API_END
}
