// Device-side cycle set-up and finalisation, so that a whole cycle runs on the
// GPU without host round trips (and can be captured in a CUDA graph):
//
//   qsg_cycle_init      cycleInit (main.cc:96-121): the previous census becomes
//                       the processing store (swapProcessingProcessedVaults,
//                       ParticleVaultContainer.cc:278-311), MC_SourceNow
//                       (MC_SourceNow.cc:28-164), PopulationControl
//                       (PopulationControl.cc:20-122) and
//                       RouletteLowWeightParticles (PopulationControl.cc:127-171)
//   qsg_cycle_finalize  cycleFinalize (main.cc:310-324) with the replica sum and
//                       reset of Tallies::CycleFinalize (Tallies.cc:25-98); the
//                       cycle's 13 counters and scalar-flux total
//                       (Tallies::ScalarFluxSum, Tallies.cc:146-171) go to a
//                       device-resident history.
//
// Everything that is constant over the run is computed once on the host at
// qsg_configure_cycle: the source particle weight and the per-cell source
// counts depend only on cell volumes, source rates, dt and nParticles.
// Each source particle, split and roulette decision draws only from its own
// random stream, so the set of particles a cycle produces does not depend on
// the order the device produces them in.
#include <cuda_runtime.h>

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
constexpr int kFluxPartials = 1024;   // fixed shape, so the flux total is reproducible

// Census -> processing bookkeeping, START / SOURCE counters.
__global__ void cycle_begin_kernel(CycleScalars* sc, unsigned long long* processing_count,
                                   unsigned long long* processed_count, unsigned long long* balance,
                                   unsigned long long n_source)
{
    const unsigned long long start = *processing_count;
    sc->start = start;
    sc->source_round = sc->source_calls;
    sc->source_calls += 1;
    balance[QSG_BAL_START] = start;            // main.cc:110 sets _start after the swap
    balance[QSG_BAL_SOURCE] += n_source;
    *processing_count = start + n_source;
    *processed_count = 0;
}

struct SourceArgs {
    DevTables t;
    DevStore out;
    const CycleScalars* sc;
    const int32_t* src_cell;
    const uint64_t* src_cell_offset;
    const int32_t* src_cell_count;
    const uint64_t* cell_id;
    const double* cell_volume;
    unsigned int* flags;
    uint64_t n_source;
    double e_min, e_max, weight;
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
    const uint64_t k = t - a.src_cell_offset[cell];
    // the cell's source tally counts every particle it ever sourced
    uint64_t seed0 = a.sc->source_round * (uint64_t)a.src_cell_count[cell] + k;
    seed0 += a.cell_id[cell];
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
    p.alpha = sine_gamma * cos(phi);
    p.beta = sine_gamma * sin(phi);
    // energy uniform in [eMin, eMax]; Get_Speed_From_Energy (MC_SourceNow.cc:169-177)
    p.kinetic_energy = (a.e_max - a.e_min) * rng_sample(p.seed) + a.e_min;
    const double m = kNeutronRestMassEnergy;
    const double E = p.kinetic_energy;
    double speed = kSpeedOfLight * sqrt(E * (E + 2.0 * (m)) / ((E + m) * (E + m)));
    p.vx = speed * p.alpha;
    p.vy = speed * p.beta;
    p.vz = speed * p.gamma;
    p.domain = 0;
    p.cell = cell;
    p.weight = a.weight;
    p.num_mean_free_paths = -1.0 * log(rng_sample(p.seed));
    p.time_to_census = tb.time_step * rng_sample(p.seed);
    p.age = 0.0;
    p.num_segments = 0.0;
    p.last_event = QSG_EVENT_CENSUS;   // MC_Particle default
    p.num_collisions = 0;
    p.breed = 0;
    p.species = 0;
    const uint64_t slot = a.sc->start + t;
    if (slot < a.out.capacity) store_particle(a.out, slot, p);
    else atomicOr(a.flags, QSG_DEV_STORE_OVERFLOW);
}

struct PopArgs {
    DevStore in, out;
    unsigned long long* balance;
    unsigned int* flags;
    uint64_t n_target;
    double weight_cutoff;       // lowWeightCutoff * source particle weight
    double low_weight_cutoff;
    int32_t load_balance;
};

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
__device__ __forceinline__ bool roulette(const PopArgs& a, Particle& p, uint32_t& rr)
{
    if (!(a.low_weight_cutoff > 0.0)) return true;
    if (p.weight <= a.weight_cutoff) {
        double r = rng_sample(p.seed);
        if (r <= a.low_weight_cutoff) {
            p.weight /= a.low_weight_cutoff;
        } else {
            rr++;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void emit(const PopArgs& a, const Particle& p)
{
    uint64_t slot = append_slot(a.out);
    if (slot < a.out.capacity) store_particle(a.out, slot, p);
    else atomicOr(a.flags, QSG_DEV_STORE_OVERFLOW);
}

// PopulationControlGuts (PopulationControl.cc:71-122) followed by the low-weight
// roulette, fused: every particle of `in` is visited once; survivors and split
// copies are appended to `out`.
__global__ void __launch_bounds__(kInitBlock) population_kernel(PopArgs a)
{
    __shared__ unsigned long long red[2];
    if (threadIdx.x < 2) red[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t n = *a.in.count;
    double factor;
    if (a.load_balance) {
        int current = (int)n;
        factor = (current != 0) ? (double)a.n_target / (double)current : 1.0;
    } else {
        factor = (double)a.n_target / (double)n;
    }
    uint32_t rr = 0, split_count = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * kInitBlock + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kInitBlock) {
        Particle p;
        load_record(a.in, i, p);
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
                    if (roulette(a, c2, rr)) emit(a, c2);
                }
            }
        }
        if (survive && roulette(a, p, rr)) emit(a, p);
    }
    if (rr) atomicAdd(&red[0], (unsigned long long)rr);
    if (split_count) atomicAdd(&red[1], (unsigned long long)split_count);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (red[0]) atomicAdd(a.balance + QSG_BAL_RR, red[0]);
        if (red[1]) atomicAdd(a.balance + QSG_BAL_SPLIT, red[1]);
    }
}

// Fixed-shape partial sums of the flux array (all replicas).
__global__ void __launch_bounds__(256) flux_partial_kernel(const double* flux, uint64_t n, double* partial)
{
    __shared__ double s[256];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t lo = (uint64_t)blockIdx.x * chunk;
    const uint64_t hi = lo + chunk < n ? lo + chunk : n;
    double acc = 0.0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += 256) acc += flux[i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// Record the cycle: counters summed over replicas, END = census count, the
// flux total; then clear the counters (flux is cleared by a memset after).
__global__ void cycle_finalize_kernel(CycleScalars* sc, unsigned long long* balance, int replicas,
                                      const unsigned long long* processed_count, const double* partial,
                                      int n_partial, CycleRecord* history)
{
    CycleRecord* rec = history + sc->cycle;
    if (threadIdx.x < QSG_BAL_COUNT) {
        unsigned long long s = 0;
        for (int r = 0; r < replicas; r++) s += balance[r * QSG_BAL_COUNT + threadIdx.x];
        if (threadIdx.x == QSG_BAL_END) s = *processed_count;   // main.cc:314
        rec->balance[threadIdx.x] = s;
    }
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int k = 0; k < n_partial; k++) total += partial[k];
        rec->flux_total = total;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < replicas * QSG_BAL_COUNT; k += blockDim.x) balance[k] = 0;
    __syncthreads();
    if (threadIdx.x == 0) sc->cycle += 1;
}

}  // namespace
}  // namespace qsg

using namespace qsg;

extern "C" int qsg_configure_cycle(QsgHandle* h, const QsgCycleConfig* cfg)
{
    QSG_API_BEGIN
    if (!h || !cfg || !cfg->source_rate) return fail(QSG_ERR_INVALID, "qsg_configure_cycle: null argument");
    if ((int64_t)h->h_cell_volume.size() != h->num_cells || (int64_t)h->h_cell_id.size() != h->num_cells)
        return fail(QSG_ERR_INVALID, "qsg_configure_cycle: the problem given to qsg_create had no cell_volume / cell_id");
    if (cfg->n_particles == 0) return fail(QSG_ERR_INVALID, "qsg_configure_cycle: n_particles must be positive");
    int st = set_device(h);
    if (st) return st;
    const int64_t C = h->num_cells;
    const double dt = h->tables.time_step;
    // MC_SourceNow.cc:35-64: total source weight in cell order, particle weight
    double total_weight = 0;
    for (int64_t c = 0; c < C; c++) total_weight += h->h_cell_volume[c] * cfg->source_rate[h->h_cell_material[c]] * dt;
    double source_fraction = 0.1;
    double spw = total_weight / (source_fraction * cfg->n_particles);
    std::vector<int32_t> count(C);
    std::vector<uint64_t> offset(C);
    uint64_t n_source = 0;
    for (int64_t c = 0; c < C; c++) {
        double cell_weight = h->h_cell_volume[c] * cfg->source_rate[h->h_cell_material[c]] * dt;
        double cell_num_float = cell_weight / spw;
        int n = (int)cell_num_float;
        if (n < 0) n = 0;
        count[c] = n;
        offset[c] = n_source;
        n_source += (uint64_t)n;
    }
    std::vector<int32_t> src_cell(n_source);
    for (int64_t c = 0; c < C; c++)
        for (int32_t k = 0; k < count[c]; k++) src_cell[offset[c] + k] = (int32_t)c;
    std::vector<double> vol(h->h_cell_volume.begin(), h->h_cell_volume.end());
    std::vector<uint64_t> ids(h->h_cell_id.begin(), h->h_cell_id.end());
    if ((st = h->src_cell.upload(src_cell)) || (st = h->src_cell_count.upload(count)) ||
        (st = h->src_cell_offset.upload(offset)) || (st = h->cell_volume.upload(vol)) || (st = h->cell_id.upload(ids)))
        return st;
    h->n_target = cfg->n_particles;
    h->e_min = cfg->e_min;
    h->e_max = cfg->e_max;
    h->low_weight_cutoff = cfg->low_weight_cutoff;
    h->load_balance = cfg->load_balance;
    h->source_particle_weight = spw;
    h->n_source = n_source;
    uint64_t cap = cfg->store_capacity ? cfg->store_capacity : 4 * (cfg->n_particles + n_source);
    if ((st = h->processing.reserve(cap)) || (st = h->processed.reserve(cap)) || (st = h->extra.reserve(cap)))
        return st;
    if ((st = h->flux_partial.alloc(kFluxPartials))) return st;
    if (!h->history.ptr) {
        if ((st = h->history.alloc(1024))) return st;
        h->history_capacity = 1024;
    }
    h->cycle_configured = true;
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_cycle_init(QsgHandle* h, void* stream)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_cycle_init: null handle");
    if (!h->cycle_configured) return fail(QSG_ERR_INVALID, "qsg_cycle_init: call qsg_configure_cycle first");
    int st = set_device(h);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // room for the census carried in plus this cycle's source, and for the
    // population-controlled output (growing a store synchronises once)
    const uint64_t need = h->known_census + h->n_source;
    if ((st = h->processed.reserve(need)) ||
        (st = h->extra.reserve(std::max<uint64_t>(need, 2 * h->n_target))))
        return st;
    std::swap(h->processing, h->processed);
    cycle_begin_kernel<<<1, 1, 0, s>>>(h->scalars.ptr, h->processing.count, h->processed.count, h->balance.ptr,
                                       (unsigned long long)h->n_source);
    QSG_CUDA(cudaGetLastError());
    if (h->n_source) {
        SourceArgs a;
        a.t = h->tables;
        a.out = h->processing.view;
        a.sc = h->scalars.ptr;
        a.src_cell = h->src_cell.ptr;
        a.src_cell_offset = h->src_cell_offset.ptr;
        a.src_cell_count = h->src_cell_count.ptr;
        a.cell_id = h->cell_id.ptr;
        a.cell_volume = h->cell_volume.ptr;
        a.n_source = h->n_source;
        a.flags = h->flags.ptr;
        a.e_min = h->e_min;
        a.e_max = h->e_max;
        a.weight = h->source_particle_weight;
        unsigned blocks = (unsigned)((h->n_source + kInitBlock - 1) / kInitBlock);
        source_kernel<<<blocks, kInitBlock, 0, s>>>(a);
        QSG_CUDA(cudaGetLastError());
    }
    QSG_CUDA(cudaMemsetAsync(h->extra.count, 0, sizeof(unsigned long long), s));
    PopArgs pa;
    pa.in = h->processing.view;
    pa.out = h->extra.view;
    pa.balance = h->balance.ptr;
    pa.flags = h->flags.ptr;
    pa.n_target = h->n_target;
    pa.low_weight_cutoff = h->low_weight_cutoff;
    pa.weight_cutoff = h->low_weight_cutoff * h->source_particle_weight;
    pa.load_balance = h->load_balance;
    population_kernel<<<h->num_sms * 8, kInitBlock, 0, s>>>(pa);
    QSG_CUDA(cudaGetLastError());
    std::swap(h->processing, h->extra);
    h->processing_on_device = true;
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_cycle_finalize(QsgHandle* h, void* stream)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_cycle_finalize: null handle");
    if (!h->cycle_configured) return fail(QSG_ERR_INVALID, "qsg_cycle_finalize: call qsg_configure_cycle first");
    int st = set_device(h);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (h->cycles_finalized >= h->history_capacity) {
        // grow the history (synchronous; happens once per 1024 cycles)
        DevBuf<CycleRecord> bigger;
        if ((st = bigger.alloc(2 * h->history_capacity))) return st;
        QSG_CUDA(cudaStreamSynchronize(s));
        QSG_CUDA(cudaMemcpy(bigger.ptr, h->history.ptr, h->history_capacity * sizeof(CycleRecord),
                            cudaMemcpyDeviceToDevice));
        h->history.free();
        h->history = bigger;
        bigger.ptr = nullptr;
        h->history_capacity *= 2;
    }
    const uint64_t nflux = (uint64_t)h->flux_replicas * h->num_cells * h->num_groups;
    flux_partial_kernel<<<kFluxPartials, 256, 0, s>>>(h->flux.ptr, nflux, h->flux_partial.ptr);
    QSG_CUDA(cudaGetLastError());
    cycle_finalize_kernel<<<1, 64, 0, s>>>(h->scalars.ptr, h->balance.ptr, h->balance_replicas, h->processed.count,
                                           h->flux_partial.ptr, kFluxPartials, h->history.ptr);
    QSG_CUDA(cudaGetLastError());
    QSG_CUDA(cudaMemsetAsync(h->flux.ptr, 0, nflux * sizeof(double), s));
    h->cycles_finalized++;
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
    std::vector<CycleRecord> rec(n);
    QSG_CUDA(cudaDeviceSynchronize());
    QSG_CUDA(cudaMemcpy(rec.data(), h->history.ptr + first, n * sizeof(CycleRecord), cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < n; i++) {
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
