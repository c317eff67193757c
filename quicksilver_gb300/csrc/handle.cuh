// Device-memory containers and the QsgHandle layout shared by the CUDA
// translation units of libqsg.so (tracking and cycle set-up).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "qsg.h"
#include "status.h"
#include "track_device.cuh"

// NVTX ranges around the phases, named as the reference's -DUSE_NVTX build
// names them (NVTX_Range.hh; main.cc:175), for profilers that filter or
// group by range.  Off unless built with -DQSG_NVTX
// (python -m quicksilver_gb300.build --nvtx): then QSG_RANGE opens a range
// that closes at the end of the enclosing scope.
#ifdef QSG_NVTX
#include <nvtx3/nvToolsExt.h>
struct QsgNvtxRange {
    explicit QsgNvtxRange(const char* name) { nvtxRangePushA(name); }
    ~QsgNvtxRange() { nvtxRangePop(); }
    QsgNvtxRange(const QsgNvtxRange&) = delete;
    QsgNvtxRange& operator=(const QsgNvtxRange&) = delete;
};
#define QSG_RANGE(name) QsgNvtxRange qsg_nvtx_range_(name)
#else
#define QSG_RANGE(name) ((void)0)
#endif

namespace qsg {

#define QSG_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t err__ = (call);                                                         \
        if (err__ != cudaSuccess)                                                           \
            return ::qsg::fail(QSG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(err__)); \
    } while (0)

template <typename T>
struct DevBuf {
    T* ptr = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        free();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&ptr, count * sizeof(T));
        if (e != cudaSuccess) {
            ptr = nullptr;
            return fail(QSG_ERR_CUDA, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
        }
        n = count;
        return QSG_OK;
    }
    int upload(const std::vector<T>& v)
    {
        int st = alloc(v.size());
        if (st) return st;
        if (!v.empty()) QSG_CUDA(cudaMemcpy(ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return QSG_OK;
    }
    void free()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        n = 0;
    }
};

// One particle store: 20 field arrays carved out of one allocation.
struct Store {
    void* base = nullptr;
    unsigned long long* count = nullptr;  // device counter
    uint64_t capacity = 0;
    uint64_t generation = 0;              // bumped on every reallocation
    int score_fields = 0;                 // sensitivity score arrays carried per particle
    DevStore view{};

    // Grow to at least `cap` particles (keeping the contents); `force`
    // reallocates even when large enough (after score_fields changed).
    int reserve(uint64_t cap, bool force = false)
    {
        if (cap <= capacity && base && !force) return QSG_OK;
        uint64_t nc = capacity ? capacity : 1024;
        while (nc < cap) nc *= 2;
        size_t bytes = nc * 136 + 256 * 21 + (size_t)score_fields * (nc * 8 + 256);
        void* nb = nullptr;
        cudaError_t e = cudaMalloc(&nb, bytes);
        if (e != cudaSuccess) return fail(QSG_ERR_CUDA, "cudaMalloc store (%zu bytes): %s", bytes, cudaGetErrorString(e));
        if (score_fields) {
            e = cudaMemset(nb, 0, bytes);
            if (e != cudaSuccess) {
                cudaFree(nb);
                return fail(QSG_ERR_CUDA, "store init: %s", cudaGetErrorString(e));
            }
        }
        DevStore nv = carve(nb, nc, score_fields);
        if (base) {
            unsigned long long n_old = 0;
            e = cudaMemcpy(&n_old, count, sizeof(n_old), cudaMemcpyDeviceToHost);
            if (e == cudaSuccess && n_old) e = copy_fields(nv, view, 0, 0, std::min<uint64_t>(n_old, capacity));
            if (e == cudaSuccess) e = cudaMemcpy(nv.count, &n_old, sizeof(n_old), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                cudaFree(nb);
                return fail(QSG_ERR_CUDA, "store grow: %s", cudaGetErrorString(e));
            }
            cudaFree(base);
        } else {
            e = cudaMemset(nv.count, 0, sizeof(unsigned long long));
            if (e != cudaSuccess) {
                cudaFree(nb);
                return fail(QSG_ERR_CUDA, "store init: %s", cudaGetErrorString(e));
            }
        }
        base = nb;
        view = nv;
        count = nv.count;
        capacity = nc;
        generation++;
        return QSG_OK;
    }

    static DevStore carve(void* b, uint64_t cap, int score_fields)
    {
        DevStore v{};
        char* p = static_cast<char*>(b);
        auto take = [&](size_t esz) {
            char* r = p;
            p += (cap * esz + 255) & ~size_t(255);
            return r;
        };
        v.count = reinterpret_cast<unsigned long long*>(p);
        p += 256;
        double** dfields[12] = {&v.x, &v.y, &v.z, &v.vx, &v.vy, &v.vz, &v.kinetic_energy, &v.weight,
                                &v.time_to_census, &v.age, &v.num_mean_free_paths, &v.num_segments};
        for (double** f : dfields) *f = reinterpret_cast<double*>(take(8));
        v.seed = reinterpret_cast<uint64_t*>(take(8));
        v.identifier = reinterpret_cast<uint64_t*>(take(8));
        int32_t** ifields[6] = {&v.last_event, &v.num_collisions, &v.breed, &v.species, &v.domain, &v.cell};
        for (int32_t** f : ifields) *f = reinterpret_cast<int32_t*>(take(4));
        v.score = score_fields ? reinterpret_cast<double*>(take(8 * (size_t)score_fields)) : nullptr;
        v.score_fields = score_fields;
        v.capacity = cap;
        return v;
    }

    static cudaError_t copy_fields(const DevStore& dst, const DevStore& src, uint64_t dst_off, uint64_t src_off,
                                   uint64_t n, cudaStream_t s = 0)
    {
        if (n == 0) return cudaSuccess;
        double* dd[12] = {dst.x, dst.y, dst.z, dst.vx, dst.vy, dst.vz, dst.kinetic_energy, dst.weight,
                          dst.time_to_census, dst.age, dst.num_mean_free_paths, dst.num_segments};
        double* sd[12] = {src.x, src.y, src.z, src.vx, src.vy, src.vz, src.kinetic_energy, src.weight,
                          src.time_to_census, src.age, src.num_mean_free_paths, src.num_segments};
        for (int k = 0; k < 12; k++) {
            cudaError_t e = cudaMemcpyAsync(dd[k] + dst_off, sd[k] + src_off, n * 8, cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return e;
        }
        uint64_t* du[2] = {dst.seed, dst.identifier};
        uint64_t* su[2] = {src.seed, src.identifier};
        for (int k = 0; k < 2; k++) {
            cudaError_t e = cudaMemcpyAsync(du[k] + dst_off, su[k] + src_off, n * 8, cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return e;
        }
        int32_t* di[6] = {dst.last_event, dst.num_collisions, dst.breed, dst.species, dst.domain, dst.cell};
        int32_t* si[6] = {src.last_event, src.num_collisions, src.breed, src.species, src.domain, src.cell};
        for (int k = 0; k < 6; k++) {
            cudaError_t e = cudaMemcpyAsync(di[k] + dst_off, si[k] + src_off, n * 4, cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return e;
        }
        for (int k = 0; k < dst.score_fields && k < src.score_fields; k++) {
            cudaError_t e = cudaMemcpyAsync(dst.score + (size_t)k * dst.capacity + dst_off,
                                            src.score + (size_t)k * src.capacity + src_off, n * 8,
                                            cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    void release()
    {
        if (base) cudaFree(base);
        base = nullptr;
        count = nullptr;
        capacity = 0;
        view = DevStore{};
    }
};

// Device scalars used by the cycle kernels (one allocation).
struct CycleScalars {
    unsigned long long cursor;        // work-queue cursor of the running tracking pass
    unsigned long long start;         // particles at cycle start (census of the previous cycle)
    unsigned long long cycle;         // cycles finalised so far (history row)
    unsigned long long source_calls;  // cycle inits so far
    unsigned long long source_round;  // index of the running cycle init (source seeds)
    unsigned long long host_in_count;      // qsg_track_host: particles in the caller's input arrays
    unsigned long long host_census_count;  // qsg_track_host: census particles appended to the caller's arrays
    unsigned long long pad;
};

// Per-cycle record written by the finalize kernel (device-resident history).
struct CycleRecord {
    unsigned long long balance[QSG_BAL_COUNT];
    double flux_total;
    double pad[2];
};

}  // namespace qsg

struct QsgHandle {
    int device = 0;
    int block_size = qsg::kTrackBlock;
    int num_sms = 0;
    int track_blocks = 0;            // persistent grid of the tracking kernel
    int kernel_kind = 1;             // 0: one history per lane; 1: warp particle pool (qsg_set_track_kernel)
    int pool_blocks = 0, pool_sens_blocks = 0;   // persistent grids of the pool kernel
    int pool_sens = 64;                           // pool size of the sensitivity instantiation
    int pool_collision_step = 32;                 // qsg_set_pool_tuning
    int pool_refill = 16;
    int max_passes = 8;              // fission passes per asynchronous cycle
    int collision_batch = qsg::kCollisionBatch;
    int queue_chunk = 1;
    int32_t num_problems = 1;        // > 1: a batch built by qsg_batch_create
    std::vector<int32_t> h_problem_cell_offset;   // [problems + 1]
    qsg::DevBuf<int32_t> cell_problem;            // [C] (batches only)
    int32_t flux_replicas = 1, balance_replicas = 1;
    uint64_t max_segments = (uint64_t)1 << 40;
    int32_t num_cells = 0, num_groups = 0, num_materials = 0;
    // tables
    bool exp_tally = false;          // the reference's EXPONENTIAL_TALLY build (qsg_set_exponential_tally)
    qsg::DevBuf<double> cell_tally;  // [num_cells]
    qsg::DevBuf<double> energies, sigma_total, mfp_table, inv_mfp_table, macro_xs, class_nubar, material_mass, cell_nodes, cell_center, planes;
    qsg::DevBuf<int32_t> class_num_reactions, class_material, cell_class, adj_cell;
    qsg::DevBuf<int8_t> class_type;
    qsg::DevBuf<uint8_t> adj_facet_event, proj;
    qsg::DevBuf<float4> face32;
    qsg::DevBuf<float2> face_slack;
    qsg::DevBuf<float> node32;
    qsg::DevTables tables{};
    // host copies needed by the cycle set-up
    std::vector<double> h_cell_volume;
    std::vector<int32_t> h_cell_material;
    std::vector<uint64_t> h_cell_id;
    // tallies
    qsg::DevBuf<double> flux;
    qsg::DevBuf<unsigned long long> balance;
    qsg::DevBuf<unsigned int> flags;
    qsg::DevBuf<double> flux_partial;             // fixed-shape partial sums for the flux total
    // particle stores: processing, processed (census), extra (fission products)
    qsg::Store processing, processed, extra;
    uint64_t n_processing = 0;   // host mirror of processing count (valid after qsg_set_particles)
    uint64_t known_census = 0;   // census count read back by the last complete tracking call
    bool processing_on_device = false;  // count known only on the device (cycle kernels)
    // cycle set-up (qsg_configure_cycle)
    bool cycle_configured = false;
    uint64_t n_target = 0;
    double e_min = 0, e_max = 0, low_weight_cutoff = 0, source_particle_weight = 0;
    int32_t load_balance = 0;
    uint64_t n_source = 0;
    qsg::DevBuf<double> cell_volume;
    qsg::DevBuf<uint64_t> cell_id;
    qsg::DevBuf<int32_t> src_cell, src_cell_count;   // [n_source] cell of each source particle, [C] per-cell count
    qsg::DevBuf<uint64_t> src_cell_offset;            // [C] first source slot of each cell
    qsg::DevBuf<qsg::CycleScalars> scalars;
    qsg::DevBuf<qsg::CycleRecord> history;        // [cycles][problems]
    uint64_t history_capacity = 0;                // in cycles
    uint64_t cycles_finalized = 0;
    // per problem (index p of a batch; one entry for a single problem)
    std::vector<int32_t> h_problem_material_offset;   // [problems + 1]
    qsg::DevBuf<double> prob_weight, prob_emin, prob_emax, prob_lowcut, prob_factor;
    qsg::DevBuf<uint64_t> prob_target, prob_nsource, prob_seed_offset;
    qsg::DevBuf<int32_t> prob_load_balance, prob_cell_offset;
    qsg::DevBuf<unsigned long long> prob_carry;
    // host copies of the cross-section classes (sensitivity tables are built from them)
    std::vector<int32_t> h_class_material;        // [classes]
    std::vector<int8_t> h_class_type;             // [classes][max_reactions]
    std::vector<uint8_t> h_class_const;           // [classes][max_reactions] 1: the 1e-20 placeholder entry
    std::vector<double> h_class_macro;            // [classes][G][max_reactions]
    int32_t num_classes = 0, max_reactions = 0;
    // observability tallies (qsg_set_observers)
    int observe_flags = 0;
    qsg::DevBuf<double> fluence;                  // [C]
    qsg::DevBuf<unsigned long long> spectrum;     // [problems][G+1]
    // sensitivities (qsg_enable_sensitivity); sens.K == 0: off
    qsg::DevSens sens{};
    int sens_track_blocks = 0;
    qsg::DevBuf<int16_t> sens_param;              // [classes][G][3]
    qsg::DevBuf<double> sens_dsig, sens_inv_theta, sens_flux_cell, sens_dflux, sens_leak, sens_dleak;
    // CUDA graphs of whole cycles, one per role permutation of the stores
    struct GraphEntry {
        void *proc = nullptr, *done = nullptr, *extra = nullptr;
        uint64_t generation = 0;
        cudaGraphExec_t exec = nullptr;
        qsg::Store after_proc, after_done, after_extra;
    };
    std::vector<GraphEntry> graphs;
    uint64_t store_generation = 0;
    const qsg::CycleRecord* graph_history = nullptr;
    cudaStream_t capture_stream = nullptr;
    void clear_graphs()
    {
        for (auto& g : graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }
};

namespace qsg {
int set_device(const QsgHandle* h);
DevTally tally_view(QsgHandle* h);
int check_soa(const QsgParticleSoA* s);
int copy_soa(const DevStore& d, const QsgParticleSoA* h, uint64_t n, bool to_device);
inline int copy_store_to_host(const DevStore& d, const QsgParticleSoA* h, uint64_t n)
{
    if (n == 0) return QSG_OK;
    int st = check_soa(h);
    return st ? st : copy_soa(d, h, n, false);
}
// Persistent grids of the tracking kernels for the handle's block size (track.cu).
int configure_track_grid(QsgHandle* h);
// Tracking passes of one cycle (track.cu).
int track_passes_async(QsgHandle* h, cudaStream_t s);
int track_passes_sync(QsgHandle* h, cudaStream_t s);
}  // namespace qsg
