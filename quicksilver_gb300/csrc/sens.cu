// Sensitivity (differential-operator) tallies: parameter tables and the C ABI
// that switches them on, reads and clears them.  The kernel side is the SENS
// instantiation of the tracking kernel (track.cu).  The reference has no
// sensitivity capability; the forward quantities being differentiated are its
// scalar flux (Tallies.hh:350-354) and its escape events
// (MC_Facet_Crossing_Event.cc:23-70, counted in Tallies::_balanceTask._escape).

#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "handle.cuh"

using namespace qsg;

namespace {

int zero_sensitivity(QsgHandle* h)
{
    if (h->sens.K == 0) return QSG_OK;
    QSG_CUDA(cudaMemset(h->sens_flux_cell.ptr, 0, h->sens_flux_cell.n * sizeof(double)));
    QSG_CUDA(cudaMemset(h->sens_dflux.ptr, 0, h->sens_dflux.n * sizeof(double)));
    QSG_CUDA(cudaMemset(h->sens_leak.ptr, 0, h->sens_leak.n * sizeof(double)));
    QSG_CUDA(cudaMemset(h->sens_dleak.ptr, 0, h->sens_dleak.n * sizeof(double)));
    return QSG_OK;
}

}  // namespace

extern "C" int qsg_enable_sensitivity(QsgHandle* h, const QsgSensitivity* s)
{
    QSG_API_BEGIN
    if (!h || !s) return fail(QSG_ERR_INVALID, "qsg_enable_sensitivity: null argument");
    const int K = s->num_params;
    if (K < 0 || K > QSG_MAX_PARAMS)
        return fail(QSG_ERR_INVALID, "qsg_enable_sensitivity: num_params %d outside 0..%d", K, QSG_MAX_PARAMS);
    const int E = s->num_entries;
    if (K > 0 && (!s->theta || E < 1 || !s->param || !s->material || !s->reaction || !s->group_lo || !s->group_hi))
        return fail(QSG_ERR_INVALID, "qsg_enable_sensitivity: missing theta or entries");
    int st = set_device(h);
    if (st) return st;
    h->clear_graphs();   // captured cycles carry the old kernel arguments
    if (K == 0) {
        h->sens = DevSens{};
        return QSG_OK;
    }
    const int G = h->num_groups, M = h->num_materials, NCL = h->num_classes, R = h->max_reactions;
    for (int k = 0; k < K; k++)
        if (!(s->theta[k] > 0.0) || !std::isfinite(s->theta[k]))
            return fail(QSG_ERR_INVALID, "sensitivity parameter %d: theta %.17g must be positive and finite", k,
                        s->theta[k]);
    // owner of each (material, reaction type, group)
    std::vector<int16_t> owner((size_t)M * 3 * G, -1);
    for (int e = 0; e < E; e++) {
        const int k = s->param[e], m = s->material[e], r = s->reaction[e], lo = s->group_lo[e], hi = s->group_hi[e];
        if (k < 0 || k >= K) return fail(QSG_ERR_INVALID, "sensitivity entry %d: parameter %d outside 0..%d", e, k, K - 1);
        if (m < 0 || m >= M) return fail(QSG_ERR_INVALID, "sensitivity entry %d: material %d outside 0..%d", e, m, M - 1);
        if (r < QSG_REACT_SCATTER || r > QSG_REACT_FISSION)
            return fail(QSG_ERR_INVALID, "sensitivity entry %d: reaction type %d is not scatter/absorption/fission", e, r);
        if (lo < 0 || hi > G || lo >= hi)
            return fail(QSG_ERR_INVALID, "sensitivity entry %d: group range [%d, %d) outside [0, %d)", e, lo, hi, G);
        for (int g = lo; g < hi; g++) {
            int16_t& o = owner[((size_t)m * 3 + (r - 1)) * G + g];
            if (o >= 0)
                return fail(QSG_ERR_INVALID, "sensitivity entries overlap at material %d, reaction %d, group %d "
                            "(parameters %d and %d)", m, r, g, (int)o, k);
            o = (int16_t)k;
        }
    }
    // per (class, group, reaction type): its parameter and dSigma_t/dtheta
    std::vector<int16_t> param((size_t)NCL * G * 3, -1);
    std::vector<double> dsig((size_t)NCL * G * 3, 0.0);
    for (int c = 0; c < NCL; c++) {
        const int m = h->h_class_material[c];
        for (int t = 0; t < 3; t++)
            for (int g = 0; g < G; g++) {
                const int k = owner[((size_t)m * 3 + t) * G + g];
                if (k < 0) continue;
                double sum = 0.0;
                for (int kk = 0; kk < R; kk++) {
                    if (h->h_class_type[(size_t)c * R + kk] != t + 1) continue;
                    if (h->h_class_const[(size_t)c * R + kk])
                        return fail(QSG_ERR_UNSUPPORTED, "sensitivity parameter %d: material %d has a zero atom fraction "
                                    "or number density, whose cross sections do not scale", k, m);
                    sum += h->h_class_macro[((size_t)c * G + g) * R + kk];
                }
                param[((size_t)c * G + g) * 3 + t] = (int16_t)k;
                dsig[((size_t)c * G + g) * 3 + t] = sum / s->theta[k];
            }
    }
    std::vector<double> inv_theta(K);
    for (int k = 0; k < K; k++) inv_theta[k] = 1.0 / s->theta[k];
    const size_t C = (size_t)h->num_cells, P = (size_t)h->num_problems;
    if ((st = h->sens_param.upload(param)) || (st = h->sens_dsig.upload(dsig)) ||
        (st = h->sens_inv_theta.upload(inv_theta)) || (st = h->sens_flux_cell.alloc(C)) ||
        (st = h->sens_dflux.alloc(C * K)) || (st = h->sens_leak.alloc(P)) || (st = h->sens_dleak.alloc(P * K)))
        return st;
    // every store carries K score columns from now on
    for (Store* store : {&h->processing, &h->processed, &h->extra}) {
        if (store->score_fields == K) continue;
        store->score_fields = K;
        if (store->base && (st = store->reserve(store->capacity, true))) return st;
    }
    DevSens& d = h->sens;
    d.K = K;
    d.param_of = h->sens_param.ptr;
    d.dsig = h->sens_dsig.ptr;
    d.inv_theta = h->sens_inv_theta.ptr;
    d.flux_cell = h->sens_flux_cell.ptr;
    d.dflux = h->sens_dflux.ptr;
    d.leak = h->sens_leak.ptr;
    d.dleak = h->sens_dleak.ptr;
    if ((st = zero_sensitivity(h))) return st;
    return configure_track_grid(h);
    QSG_API_END
}

extern "C" int qsg_read_sensitivity(QsgHandle* h, double* flux_cell, double* dflux, double* leak, double* dleak)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_read_sensitivity: null handle");
    if (h->sens.K == 0) return fail(QSG_ERR_INVALID, "qsg_read_sensitivity: sensitivities are not enabled");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    if (flux_cell)
        QSG_CUDA(cudaMemcpy(flux_cell, h->sens_flux_cell.ptr, h->sens_flux_cell.n * sizeof(double), cudaMemcpyDeviceToHost));
    if (dflux) QSG_CUDA(cudaMemcpy(dflux, h->sens_dflux.ptr, h->sens_dflux.n * sizeof(double), cudaMemcpyDeviceToHost));
    if (leak) QSG_CUDA(cudaMemcpy(leak, h->sens_leak.ptr, h->sens_leak.n * sizeof(double), cudaMemcpyDeviceToHost));
    if (dleak) QSG_CUDA(cudaMemcpy(dleak, h->sens_dleak.ptr, h->sens_dleak.n * sizeof(double), cudaMemcpyDeviceToHost));
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_reset_sensitivity(QsgHandle* h)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_reset_sensitivity: null handle");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    return zero_sensitivity(h);
    QSG_API_END
}

extern "C" int qsg_material_offsets(QsgHandle* h, int32_t* offsets)
{
    if (!h || !offsets) return fail(QSG_ERR_INVALID, "qsg_material_offsets: null argument");
    for (size_t i = 0; i < h->h_problem_material_offset.size(); i++) offsets[i] = h->h_problem_material_offset[i];
    return QSG_OK;
}
