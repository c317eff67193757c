// Cycle-tracking kernel (one thread per history) and the C-ABI handle.
//
// Replaces CycleTrackingKernel / CycleTrackingGuts (main.cc:126-134,
// CycleTracking.cc:14-120) for one spatial domain.  Design:
//   * particles live in HBM as structure-of-arrays (coalesced 8-byte loads
//     and stores per field), read once at history start, written once at
//     census / fission;
//   * cross sections are pre-reduced per (cross-section class, group): the
//     reference's per-cell cached total (MacroscopicCrossSection.cc:58-81) is
//     identical for every cell of one (material, number density) class, so one
//     table row serves all of them with the same bits;
//   * mesh tables per cell: 24 planes, the 14 nodes, adjacency packed to
//     5 bytes per facet -- L2-resident for the benchmark meshes;
//   * balance counters are accumulated per thread, reduced per block and
//     added with one 64-bit atomic per counter per block; scalar flux uses
//     FP64 atomics into `flux_replicas` privatised copies;
//   * census and fission products are appended with warp-aggregated atomics.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "qsg.h"
#include "status.h"
#include "track_device.cuh"
#include "batch.h"

namespace cg = cooperative_groups;

namespace qsg {

enum LocalCounter { LC_SEG = 0, LC_COLL, LC_SCAT, LC_ABS, LC_FIS, LC_PROD, LC_ESC, LC_CEN, LC_N };

// MCT_Nearest_Facet_3D_G_Distance_To_Segment, MCT.cc:280-395.
__device__ __forceinline__ double distance_to_segment(double plane_tolerance, double dot, double A, double B, double C,
                                                      double D, const double* p0, const double* p1,
                                                      const double* p2, const Particle& p)
{
    const double bb_tol = 1e-9;
    double numerator = -1.0 * (A * p.x + B * p.y + C * p.z + D);
    if (numerator < 0.0 && numerator * numerator > plane_tolerance) return kHugeDouble;
    double distance = numerator / dot;
    double ip[3];
    ip[0] = p.x + distance * p.alpha;
    ip[1] = p.y + distance * p.beta;
    ip[2] = p.z + distance * p.gamma;
    int u, v;
    if (C < -0.5 || C > 0.5) { u = 0; v = 1; }
    else if (B < -0.5 || B > 0.5) { u = 2; v = 0; }
    else if (A < -0.5 || A > 0.5) { u = 1; v = 2; }
    else return kHugeDouble;  // no dominant normal component: crosses stay 0 and the test fails
    // bounding-box rejects on the two projected axes (first axis u, then v)
    {
        double hi = ip[u] + bb_tol, lo = ip[u] - bb_tol;
        if (p0[u] > hi && p1[u] > hi && p2[u] > hi) return kHugeDouble;
        if (p0[u] < lo && p1[u] < lo && p2[u] < lo) return kHugeDouble;
    }
    {
        double hi = ip[v] + bb_tol, lo = ip[v] - bb_tol;
        if (p0[v] > hi && p1[v] > hi && p2[v] > hi) return kHugeDouble;
        if (p0[v] < lo && p1[v] < lo && p2[v] < lo) return kHugeDouble;
    }
    double cross1 = (p1[u] - p0[u]) * (ip[v] - p0[v]) - (p1[v] - p0[v]) * (ip[u] - p0[u]);
    double cross2 = (p2[u] - p1[u]) * (ip[v] - p1[v]) - (p2[v] - p1[v]) * (ip[u] - p1[u]);
    double cross0 = (p0[u] - p2[u]) * (ip[v] - p2[v]) - (p0[v] - p2[v]) * (ip[u] - p2[u]);
    double s = cross0 + cross1 + cross2;
    double cross_tol = 1e-9 * (s < 0 ? -s : s);
    if ((cross0 > -cross_tol && cross1 > -cross_tol && cross2 > -cross_tol) ||
        (cross0 < cross_tol && cross1 < cross_tol && cross2 < cross_tol))
        return distance;
    return kHugeDouble;
}

// FP32 screen of one facet.  Returns true when the reference's FP64
// computation for this facet (MCT.cc:580-606 and :280-395) is *proven* to end
// in _hugeDouble, so the facet can be skipped: either its outward normal does
// not face the direction (dot <= 0), or the FP64 inside test must see crosses
// of clearly mixed sign.  Every quantity is computed in float in cell-local
// coordinates with an explicit bound on its distance from the FP64 value the
// reference computes (u = 2^-24 is the float unit roundoff; the factors are
// several times the rounding-error counts); any doubt -- a tiny dot, NaN, a
// bound that does not separate -- answers false and the facet is evaluated
// exactly in FP64.
enum ScreenResult { SCREEN_EXACT = 0, SCREEN_HUGE = 1, SCREEN_ACCEPT = 2 };

// The four facets of one hex face (facets 4k..4k+3 share the face-centre node
// 8+k) lie in one plane up to FP64 rounding, so the screen takes the normal
// and offset of the face once: `pl` is the face's plane in float (cell-local
// offset), and sn / sd bound how far any of its facets' FP64 planes differ
// from the one rounded (|dA|+|dB|+|dC| and |d offset|).  The quantities the
// four facets share -- direction dot, numerator, distance along the ray --
// are computed here with their error bounds.
struct FaceScreen {
    int state;   // SCREEN_HUGE or SCREEN_EXACT for all four facets, or -1: screen each facet
    float n, e_n, d, e_d, tt, att, e_t;
};

__device__ __forceinline__ FaceScreen face_screen(const float4 pl, float x, float y, float z, float a, float b,
                                                  float g, float pos_max, float slack, float sn, float sd)
{
    constexpr float u = 5.9604645e-8f;
    FaceScreen fs;
    fs.state = -1;
    const float s_dot = fabsf(pl.x * a) + fabsf(pl.y * b) + fabsf(pl.z * g);
    const float d = pl.x * a + pl.y * b + pl.z * g;
    const float e_d = 16.0f * u * s_dot + 1e-12f + sn;
    fs.d = d;
    fs.e_d = e_d;
    if (d < -e_d) {                  // every facet's FP64 dot <= 0: not a candidate
        fs.state = SCREEN_HUGE;
        return fs;
    }
    if (!(d > 2.0f * e_d)) {         // sign uncertain (or NaN): evaluate exactly
        fs.state = SCREEN_EXACT;
        return fs;
    }
    const float t_n = fabsf(pl.x * x) + fabsf(pl.y * y) + fabsf(pl.z * z) + fabsf(pl.w);
    const float n = -(pl.x * x + pl.y * y + pl.z * z + pl.w);
    const float e_n = 16.0f * u * t_n + slack + sn * pos_max + sd;
    const float tt = n * __frcp_rn(d);
    const float att = fabsf(tt);
    fs.n = n;
    fs.e_n = e_n;
    fs.tt = tt;
    fs.att = att;
    fs.e_t = (e_n + att * e_d * 1.01f) / (d - e_d) + 4.0f * u * att;
    return fs;
}

// The rest of the screen for one facet of a face that passed face_screen:
// returns SCREEN_HUGE when the reference's FP64 inside test (MCT.cc:331-393)
// must fail, SCREEN_ACCEPT when it must pass (then the FP64 distance is just
// numerator / dot), SCREEN_EXACT when the bounds do not decide.
__device__ __forceinline__ int facet_screen(const FaceScreen& fs, uint8_t proj, const float* n32, const int8_t* loc,
                                            float x, float y, float z, float a, float b, float g,
                                            float pos_max, float slack)
{
    constexpr float u = 5.9604645e-8f;
    if (proj == 0xff) return SCREEN_HUGE;   // no dominant normal component: the FP64 test always fails
    const float n = fs.n, e_n = fs.e_n, tt = fs.tt, att = fs.att, e_t = fs.e_t;
    const int iu = proj & 3, iv = proj >> 2;
    const float pu = (iu == 0) ? x : ((iu == 1) ? y : z);
    const float pv = (iv == 0) ? x : ((iv == 1) ? y : z);
    const float du = (iu == 0) ? a : ((iu == 1) ? b : g);
    const float dv = (iv == 0) ? a : ((iv == 1) ? b : g);
    const float ipu = pu + tt * du;
    const float ipv = pv + tt * dv;
    const float ip_max = fmaxf(fabsf(ipu), fabsf(ipv));
    const float e_ip = e_t + 3.0f * u * (pos_max + att + ip_max) + slack;
    float cmin = 3.4e38f, cmax = -3.4e38f, csum = 0.0f, ecmax = 0.0f, amax = 0.0f;
    float vu[3], vv[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        vu[k] = __ldg(n32 + 3 * loc[k] + iu);
        vv[k] = __ldg(n32 + 3 * loc[k] + iv);
        amax = fmaxf(amax, fmaxf(fabsf(vu[k]), fabsf(vv[k])));
    }
    const float e_v = 3.0f * u * amax + slack;   // vertex: float rounding of (node - centre)
#pragma unroll
    for (int k = 0; k < 3; k++) {
        // the reference's crosses are cross1 (0->1), cross2 (1->2), cross0 (2->0)
        const int k1 = (k + 1) % 3;
        const float eu = vu[k1] - vu[k], ev = vv[k1] - vv[k];
        const float ru = ipu - vu[k], rv = ipv - vv[k];
        const float c = eu * rv - ev * ru;
        // edge error (two vertices) times the lever arm, lever-arm error
        // (intersection point and vertex) times the edge, and float rounding
        const float ec = (fabsf(ru) + fabsf(rv)) * (2.0f * e_v) + (fabsf(eu) + fabsf(ev)) * (e_ip + e_v) +
                         8.0f * u * (fabsf(eu * rv) + fabsf(ev * ru));
        cmin = fminf(cmin, c);
        cmax = fmaxf(cmax, c);
        csum += c;
        ecmax = fmaxf(ecmax, ec);
    }
    const float cabs = fmaxf(fabsf(cmin), fabsf(cmax));
    const float tol = 1.01e-9f * (fabsf(csum) + 3.0f * ecmax + 12.0f * u * cabs) + 1e-30f;
    const float thr = tol + ecmax;
    if ((cmin <= -thr) && (cmax >= thr)) return SCREEN_HUGE;
    // Proven acceptance: FP64 numerator > 0 (so the plane test of MCT.cc:303
    // passes), the intersection lies inside the vertex range on both projected
    // axes by more than the error bounds (bounding-box tests of MCT.cc:333-374
    // pass), and all crosses share one sign by more than their bounds (the
    // inside test of MCT.cc:389-393 passes).  Then the FP64 result is exactly
    // numerator / dot.
    const float m = e_ip + e_v + slack;
    const float umin = fminf(vu[0], fminf(vu[1], vu[2])), umax = fmaxf(vu[0], fmaxf(vu[1], vu[2]));
    const float vmin = fminf(vv[0], fminf(vv[1], vv[2])), vmax = fmaxf(vv[0], fmaxf(vv[1], vv[2]));
    const bool bbox_in = (umin <= ipu - m) && (umax >= ipu + m) && (vmin <= ipv - m) && (vmax >= ipv + m);
    const bool same_sign = (cmin > ecmax) || (cmax < -ecmax);
    if (n > e_n && bbox_in && same_sign) return SCREEN_ACCEPT;
    return SCREEN_EXACT;
}

// The four facets of face fc together, when they share one projection (the
// usual case: one normal): facet k of the face is the triangle (corner k,
// corner k+1, centre) of the face's corner cycle (kFacetLocal[4fc+k] =
// {corner k, corner k+1, centre}), so its three crosses are the rim cross
// corner k -> corner k+1, the spoke cross corner k+1 -> centre, and the
// reverse of the spoke cross corner k -> centre (in exact arithmetic
// (c - m) x (ip - m) = -(m - c) x (ip - c)).  Eight crosses instead of twelve
// and five vertex loads instead of twelve; each estimate keeps the error bound
// of the cross it was computed as.  Bits 0-3 of the result: facets to
// evaluate exactly; bits 4-7: proven accepted.
__device__ __forceinline__ uint32_t face_facets_screen(const FaceScreen& fs, uint8_t proj, const float* n32, int fc,
                                                       float x, float y, float z, float a, float b, float g,
                                                       float pos_max, float slack)
{
    constexpr float u = 5.9604645e-8f;
    const float n = fs.n, e_n = fs.e_n, tt = fs.tt, att = fs.att, e_t = fs.e_t;
    const int iu = proj & 3, iv = proj >> 2;
    const float pu = (iu == 0) ? x : ((iu == 1) ? y : z);
    const float pv = (iv == 0) ? x : ((iv == 1) ? y : z);
    const float du = (iu == 0) ? a : ((iu == 1) ? b : g);
    const float dv = (iv == 0) ? a : ((iv == 1) ? b : g);
    const float ipu = pu + tt * du;
    const float ipv = pv + tt * dv;
    const float ip_max = fmaxf(fabsf(ipu), fabsf(ipv));
    const float e_ip = e_t + 3.0f * u * (pos_max + att + ip_max) + slack;
    float cu[4], cv[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int node = kFacetLocal[4 * fc + k][0];
        cu[k] = __ldg(n32 + 3 * node + iu);
        cv[k] = __ldg(n32 + 3 * node + iv);
    }
    const int centre = kFacetLocal[4 * fc][2];
    const float mu = __ldg(n32 + 3 * centre + iu), mv = __ldg(n32 + 3 * centre + iv);
    float amax = fmaxf(fabsf(mu), fabsf(mv));
#pragma unroll
    for (int k = 0; k < 4; k++) amax = fmaxf(amax, fmaxf(fabsf(cu[k]), fabsf(cv[k])));
    const float e_v = 3.0f * u * amax + slack;   // vertex: float rounding of (node - centre)
    // rim[k]: corner k -> corner k+1; spoke[k]: corner k -> face centre
    float rim[4], erim[4], spoke[4], espoke[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int k1 = (k + 1) & 3;
        const float ru = ipu - cu[k], rv = ipv - cv[k];
        {
            const float eu = cu[k1] - cu[k], ev = cv[k1] - cv[k];
            rim[k] = eu * rv - ev * ru;
            erim[k] = (fabsf(ru) + fabsf(rv)) * (2.0f * e_v) + (fabsf(eu) + fabsf(ev)) * (e_ip + e_v) +
                      8.0f * u * (fabsf(eu * rv) + fabsf(ev * ru));
        }
        {
            const float eu = mu - cu[k], ev = mv - cv[k];
            spoke[k] = eu * rv - ev * ru;
            espoke[k] = (fabsf(ru) + fabsf(rv)) * (2.0f * e_v) + (fabsf(eu) + fabsf(ev)) * (e_ip + e_v) +
                        8.0f * u * (fabsf(eu * rv) + fabsf(ev * ru));
        }
    }
    uint32_t res = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int k1 = (k + 1) & 3;
        // the reference's cross1 (0->1), cross2 (1->2), cross0 (2->0)
        const float c1 = rim[k], c2 = spoke[k1], c0 = -spoke[k];
        const float cmin = fminf(c0, fminf(c1, c2)), cmax = fmaxf(c0, fmaxf(c1, c2));
        const float csum = c0 + c1 + c2;
        const float ecmax = fmaxf(erim[k], fmaxf(espoke[k1], espoke[k]));
        const float cabs = fmaxf(fabsf(cmin), fabsf(cmax));
        const float tol = 1.01e-9f * (fabsf(csum) + 3.0f * ecmax + 12.0f * u * cabs) + 1e-30f;
        const float thr = tol + ecmax;
        if ((cmin <= -thr) && (cmax >= thr)) continue;   // proven outside: _hugeDouble
        // proven acceptance, as in facet_screen
        const float m = e_ip + e_v + slack;
        const float umin = fminf(cu[k], fminf(cu[k1], mu)), umax = fmaxf(cu[k], fmaxf(cu[k1], mu));
        const float vmin = fminf(cv[k], fminf(cv[k1], mv)), vmax = fmaxf(cv[k], fmaxf(cv[k1], mv));
        const bool bbox_in = (umin <= ipu - m) && (umax >= ipu + m) && (vmin <= ipv - m) && (vmax >= ipv + m);
        const bool same_sign = (cmin > ecmax) || (cmax < -ecmax);
        res |= (n > e_n && bbox_in && same_sign) ? (16u << k) : (1u << k);
    }
    return res;
}

// Find_Nearest's rules (MCT.cc:436-479) for one facet's value, stated so that
// the facets may be visited in any order: the smallest positive distance, a
// later facet winning a tie (the reference's `<=` in ascending order); else the
// largest non-positive one, an earlier facet winning a tie (its strict `>`);
// _hugeDouble is kept apart as the highest facet holding it.  Ties compare
// IEEE order keys, as the reference's comparisons do (-0.0 equals +0.0).
__device__ __forceinline__ void nearest_visit(double d, int f, double& best, int& best_f, double& neg, int& neg_f,
                                              int& huge_f)
{
    if (f64_eq(d, kHugeDouble)) {
        if (f > huge_f) huge_f = f;
    } else if (f64_gt0(d)) {
        const long long kd = f64_key(d), kb = f64_key(best);
        if (kd < kb || (kd == kb && f > best_f)) { best = d; best_f = f; }
    } else {
        const long long kd = f64_key(d), kn = f64_key(neg);
        if (kn < kd || (kn == kd && f < neg_f)) { neg = d; neg_f = f; }
    }
}

// MCT_Nearest_Facet (MCT.cc:86-137) with MCT_Nearest_Facet_3D_G
// (MCT.cc:549-621) and both Find_Nearest overloads (MCT.cc:436-536).
// Facets the FP32 screen proves to be _hugeDouble are not evaluated; the rest
// go through the reference's FP64 computation.  Find_Nearest is then applied
// to the 24 values: the smallest positive distance with `<=` (a later facet
// wins a tie); if none, the largest non-positive one; _hugeDouble entries
// count as positive, so when no finite positive distance exists the result is
// _hugeDouble at the highest-numbered facet holding it.  The proven-accepted
// facets (numerator / dot) and the facets that need the full test are visited
// in two loops, so a warp whose lanes hold some of each runs each body once per
// facet of the lane with most of that kind, not both bodies per facet.
// Moves the particle toward the cell centre on a retry, as the reference
// does through its coordinate reference (MCT.cc:510, 656-666).
__device__ double nearest_facet(const DevTables& t, const DevTally& tally, Particle& p, int& facet_out)
{
    const int cell = p.cell;
    const double* planes = t.planes + (int64_t)cell * (kFacets * 4);
    const double* nodes = t.cell_nodes + (int64_t)cell * (kCellPoints * 3);
    const float4* pf32 = t.face32 + (int64_t)cell * 6;
    const float2 fsl = __ldg(t.face_slack + cell);
    const float* n32 = t.node32 + (int64_t)cell * (kCellPoints * 3);
    const uint8_t* proj = t.proj + (int64_t)cell * kFacets;
    const double* ctr = t.cell_center + 3 * (int64_t)cell;
    const double cx = __ldg(ctr + 0), cy = __ldg(ctr + 1), cz = __ldg(ctr + 2);
    // float copies for the screen, converted on the integer pipe (bounds as for (float))
    const float a32 = f64_to_f32_rn(p.alpha), b32 = f64_to_f32_rn(p.beta), g32 = f64_to_f32_rn(p.gamma);
    const float slack = (float)t.abs_slack;
    int iteration = 0;
    double move_factor = 0.5 * kSmallDouble;
    for (;;) {
        const float x32 = f64_to_f32_rn(p.x - cx), y32 = f64_to_f32_rn(p.y - cy), z32 = f64_to_f32_rn(p.z - cz);
#ifdef QSG_VERIFY_SCREEN
        {
            // verification build: the integer-pipe conversions equal (float) in float's normal range
            const double src[6] = {p.alpha, p.beta, p.gamma, p.x - cx, p.y - cy, p.z - cz};
            const float got[6] = {a32, b32, g32, x32, y32, z32};
            for (int k = 0; k < 6; k++) {
                const float want = (float)src[k];
                if (fabsf(want) >= 1.17549435e-38f && __float_as_uint(want) != __float_as_uint(got[k]))
                    raise_flag(tally, QSG_DEV_SCREEN_MISS);
            }
        }
#endif
        const float pos_max = fmaxf(fabsf(x32), fmaxf(fabsf(y32), fabsf(z32)));
        uint32_t exact = 0, accept = 0;
#pragma unroll 1
        for (int fc = 0; fc < 6; fc++) {
            const FaceScreen fs = face_screen(__ldg(pf32 + fc), x32, y32, z32, a32, b32, g32, pos_max, slack, fsl.x,
                                              fsl.y);
            if (fs.state == SCREEN_HUGE) continue;
            if (fs.state == SCREEN_EXACT) {
                exact |= 0xfu << (4 * fc);
                continue;
            }
            const uchar4 pr4 = __ldg(reinterpret_cast<const uchar4*>(proj) + fc);
            if (pr4.x == pr4.y && pr4.x == pr4.z && pr4.x == pr4.w && pr4.x != 0xff) {
                const uint32_t r = face_facets_screen(fs, pr4.x, n32, fc, x32, y32, z32, a32, b32, g32, pos_max, slack);
                exact |= (r & 0xfu) << (4 * fc);
                accept |= ((r >> 4) & 0xfu) << (4 * fc);
                continue;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int f = 4 * fc + k;
                const int s = facet_screen(fs, __ldg(proj + f), n32, kFacetLocal[f], x32, y32, z32, a32, b32, g32,
                                           pos_max, slack);
                if (s == SCREEN_EXACT) exact |= 1u << f;
                else if (s == SCREEN_ACCEPT) accept |= 1u << f;
            }
        }
        // proven-accepted facets need only the reference's numerator / dot
        // (MCT.cc:291-307, 582-585); everything else screened is _hugeDouble
        exact |= accept;
        double best = 1e80;
        int best_f = 0;
        double neg = -kHugeDouble;
        int neg_f = 0;
        int huge_f = -1;   // highest facet whose value is _hugeDouble
        const uint32_t screened = ~exact & 0xffffffu;
        if (screened) huge_f = 31 - __clz(screened);
#ifdef QSG_VERIFY_SCREEN
        {
            // verification build: every screened facet must be _hugeDouble in FP64
            const double plane_tolerance = 1e-16 * (p.x * p.x + p.y * p.y + p.z * p.z);
            for (int f = 0; f < kFacets; f++) {
                if (!((screened >> f) & 1u)) continue;
                const double* pl = planes + 4 * f;
                const double dot = pl[0] * p.alpha + pl[1] * p.beta + pl[2] * p.gamma;
                if (!(dot > 0.0)) continue;
                double q0[3], q1[3], q2[3];
                for (int k = 0; k < 3; k++) {
                    q0[k] = nodes[3 * kFacetLocal[f][0] + k];
                    q1[k] = nodes[3 * kFacetLocal[f][1] + k];
                    q2[k] = nodes[3 * kFacetLocal[f][2] + k];
                }
                if (distance_to_segment(plane_tolerance, dot, pl[0], pl[1], pl[2], pl[3], q0, q1, q2, p) != kHugeDouble)
                    raise_flag(tally, QSG_DEV_SCREEN_MISS);
            }
        }
#endif
        for (uint32_t m = accept; m != 0; m &= m - 1) {
            const int f = __ffs(m) - 1;
            const double2 ab = __ldg(reinterpret_cast<const double2*>(planes + 4 * f));
            const double2 cd = __ldg(reinterpret_cast<const double2*>(planes + 4 * f + 2));
            const double dot = ab.x * p.alpha + ab.y * p.beta + cd.x * p.gamma;
            const double numerator = -1.0 * (ab.x * p.x + ab.y * p.y + cd.x * p.z + cd.y);
            const double d = numerator / dot;
#ifdef QSG_VERIFY_SCREEN
            double q0[3], q1[3], q2[3];
            for (int k = 0; k < 3; k++) {
                q0[k] = nodes[3 * kFacetLocal[f][0] + k];
                q1[k] = nodes[3 * kFacetLocal[f][1] + k];
                q2[k] = nodes[3 * kFacetLocal[f][2] + k];
            }
            const double plane_tolerance = 1e-16 * (p.x * p.x + p.y * p.y + p.z * p.z);
            const double full = (dot > 0.0) ? distance_to_segment(plane_tolerance, dot, ab.x, ab.y, cd.x, cd.y,
                                                                  q0, q1, q2, p)
                                            : kHugeDouble;
            if (full != d) raise_flag(tally, QSG_DEV_SCREEN_MISS);
#endif
            nearest_visit(d, f, best, best_f, neg, neg_f, huge_f);
        }
        for (uint32_t m = exact & ~accept; m != 0; m &= m - 1) {
            const int f = __ffs(m) - 1;
            const double2 ab = __ldg(reinterpret_cast<const double2*>(planes + 4 * f));
            const double2 cd = __ldg(reinterpret_cast<const double2*>(planes + 4 * f + 2));
            double d = kHugeDouble;
            const double dot = ab.x * p.alpha + ab.y * p.beta + cd.x * p.gamma;
            if (dot > 0.0) {
                double q0[3], q1[3], q2[3];
                const double* n0 = nodes + 3 * kFacetLocal[f][0];
                const double* n1 = nodes + 3 * kFacetLocal[f][1];
                const double* n2 = nodes + 3 * kFacetLocal[f][2];
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    q0[k] = __ldg(n0 + k);
                    q1[k] = __ldg(n1 + k);
                    q2[k] = __ldg(n2 + k);
                }
                // (1e-8 * |r|)^2 of MCT.cc:569-571, which only the full test uses
                const double plane_tolerance = 1e-16 * (p.x * p.x + p.y * p.y + p.z * p.z);
                d = distance_to_segment(plane_tolerance, dot, ab.x, ab.y, cd.x, cd.y, q0, q1, q2, p);
            }
            nearest_visit(d, f, best, best_f, neg, neg_f, huge_f);
        }
        // _hugeDouble is positive and larger than any finite distance, so it
        // only wins when no finite positive distance exists
        if (f64_eq(best, 1e80) && huge_f >= 0) {
            best = kHugeDouble;
            best_f = huge_f;
        }
        if (f64_eq(best, kHugeDouble) && !f64_eq(neg, -kHugeDouble)) { best = neg; best_f = neg_f; }
        bool retry = false;
        if ((f64_eq(best, kHugeDouble) && move_factor > 0) ||
            (f64_lt(10000000.0, p.num_segments) && !f64_gt0(best))) {
            const double* c = t.cell_center + 3 * (int64_t)cell;
            p.x += move_factor * (__ldg(c + 0) - p.x);
            p.y += move_factor * (__ldg(c + 1) - p.y);
            p.z += move_factor * (__ldg(c + 2) - p.z);
            iteration++;
            move_factor *= 2.0;
            if (move_factor > 1.0e-2) move_factor = 1.0e-2;
            if (iteration == 10000) raise_flag(tally, QSG_DEV_TRACKING_LIMIT);
            else retry = true;
        }
        if (!retry) {
            if (f64_lt0(best)) best = 0;
            if (!f64_lt(best, kHugeDouble)) raise_flag(tally, QSG_DEV_BAD_FACET);
            facet_out = best_f;
            return best;
        }
    }
}

enum { OUT_COLLISION = 0, OUT_FACET = 1, OUT_CENSUS = 2 };

// MC_Segment_Outcome, MC_Segment_Outcome.cc:30-226.
__device__ __forceinline__ int segment_outcome(const DevTables& t, const DevTally& tally, Particle& p,
                                               int cls, double* flux_row)
{
    // The reference's EXPONENTIAL_TALLY build (CycleTracking.cc:48-50,
    // Tallies.hh:357-360): one random number per segment, its exp added to
    // the particle's cell, before the segment outcome
    if (tally.cell_tally) atomicAdd(tally.cell_tally + p.cell, exp(rng_sample(p.seed)));
    double d_coll, d_facet, d_census;
    p.seg_len = 0.0;
    if (f64_lt0(p.speed)) p.speed = sqrt(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
    const double speed = p.speed;
    bool force_collision = false;
    if (f64_lt0(p.num_mean_free_paths)) {
        force_collision = true;
        p.num_mean_free_paths = kSmallDouble;
    }
    const int key = cls * t.num_groups + p.group;
    if (key != p.xs_key) {
        p.mean_free_path = __ldg(t.mfp_table + key);   // same bits as the reference's 1.0 / sigma
        p.inv_mfp = __ldg(t.inv_mfp_table + key);
        p.xs_key = key;
    }
    if (f64_eq0(p.num_mean_free_paths)) {
        double r = rng_sample(p.seed);
        p.num_mean_free_paths = -1.0 * QSG_LOG(r);
    }
    d_coll = force_collision ? kSmallDouble : p.num_mean_free_paths * p.mean_free_path;
    d_census = speed * p.time_to_census;
    int facet = 0;
    d_facet = nearest_facet(t, tally, p, facet);
    if (p.last_event == QSG_EVENT_FACET_TRACKING_ERROR) return OUT_FACET;
    if (force_collision) {
        d_facet = kHugeDouble;
        d_census = kHugeDouble;
        d_coll = kTinyDouble;
    }
    // MC_Find_Min (MC_Segment_Outcome.cc:232-248): strict <, ties keep the lower index
    int outcome = OUT_COLLISION;
    double seg = d_coll;
    if (f64_lt(d_facet, seg)) { seg = d_facet; outcome = OUT_FACET; }
    if (f64_lt(d_census, seg)) { seg = d_census; outcome = OUT_CENSUS; }
    if (f64_lt0(seg)) raise_flag(tally, QSG_DEV_NEGATIVE_DISTANCE);
    p.seg_len = seg;
    // a collision resets the mean free paths to 0 below: the reference's
    // subtraction there is dead, so it is skipped (same bits); the division
    // is div_rn's correctly rounded quotient (same bits)
    if (outcome != OUT_COLLISION) {
        const double q = div_rn(seg, p.mean_free_path, p.inv_mfp);
#ifdef QSG_VERIFY_SCREEN
        if (f64_bits(q) != f64_bits(seg / p.mean_free_path)) raise_flag(tally, QSG_DEV_SCREEN_MISS);
#endif
        p.num_mean_free_paths -= q;
    }
    if (outcome == OUT_COLLISION) {
        p.last_event = QSG_EVENT_COLLISION;
        p.num_mean_free_paths = 0.0;
    } else if (outcome == OUT_FACET) {
        p.last_event = QSG_EVENT_FACET_TRANSIT_EXIT;
        p.facet = facet;
    } else {
        p.last_event = QSG_EVENT_CENSUS;
        p.time_to_census = f64_lt0(p.time_to_census) ? p.time_to_census : 0.0;
    }
    if (force_collision) p.num_mean_free_paths = 0.0;
    if (f64_eq0(seg)) return outcome;
    p.x += (p.alpha * seg);
    p.y += (p.beta * seg);
    p.z += (p.gamma * seg);
    double seg_time = (seg / speed);
    p.time_to_census -= seg_time;
    p.age += seg_time;
    if (f64_lt0(p.time_to_census)) p.time_to_census = 0.0;
    atomicAdd(flux_row + (int64_t)p.cell * t.num_groups + p.group, seg * p.weight);
    return outcome;
}

// updateTrajectory (CollisionEvent.cc:24-46) with DirectionCosine::
// Rotate3DVector (DirectionCosine.hh:122-147).
__device__ __forceinline__ void update_trajectory(double energy, double angle, Particle& p)
{
    p.kinetic_energy = energy;
    double cosTheta = angle;
    double r = rng_sample(p.seed);
    double phi = 2 * 3.14159265 * r;
    double sinPhi, cosPhi;
    QSG_SINCOS(phi, &sinPhi, &cosPhi);
    double sinTheta = sqrt((1.0 - (cosTheta * cosTheta)));
    double cos_theta = p.gamma;
    double sin_theta = sqrt((1.0 - (cos_theta * cos_theta)));
    double cos_phi, sin_phi;
    if (sin_theta < 1e-6) {
        cos_phi = 1.0;
        sin_phi = 0.0;
    } else {
        cos_phi = p.alpha / sin_theta;
        sin_phi = p.beta / sin_theta;
    }
    double a = cos_theta * cos_phi * (sinTheta * cosPhi) - sin_phi * (sinTheta * sinPhi) + sin_theta * cos_phi * cosTheta;
    double b = cos_theta * sin_phi * (sinTheta * cosPhi) + cos_phi * (sinTheta * sinPhi) + sin_theta * sin_phi * cosTheta;
    double g = -sin_theta * (sinTheta * cosPhi) + cos_theta * cosTheta;
    p.alpha = a;
    p.beta = b;
    p.gamma = g;
    const double m = kNeutronRestMassEnergy;
    double speed = (kSpeedOfLight * sqrt((1.0 - ((m * m) / ((energy + m) * (energy + m))))));
    p.vx = speed * p.alpha;
    p.vy = speed * p.beta;
    p.vz = speed * p.gamma;
    p.speed = -1.0;   // |velocity| of the new velocity is recomputed when next needed
    r = rng_sample(p.seed);
    p.num_mean_free_paths = -1.0 * QSG_LOG(r);
}

// CollisionEvent (CollisionEvent.cc:48-148) with NuclearDataReaction::
// sampleCollision (NuclearData.cc:52-88), split in two so that a warp runs the
// expensive part (trajectory update: log, sincos, square roots, rotation) for
// many lanes at once.  A particle's own random stream is consumed in the
// reference's order either way, so the results are unchanged.
enum CollisionKind { COLL_ENDS = 0, COLL_SCATTER = 1, COLL_FISSION = 2 };

// First part, right after the segment: reaction selection, the scatter's
// outgoing energy and direction cosine, the counters.  Returns COLL_ENDS when
// the history ends here (absorption), otherwise the kind of the pending
// second part.  SENS: the selected reaction adds d log Sigma_r / dtheta to the
// history's scores S (stride `ss`).
template <bool SENS>
__device__ __forceinline__ int collision_select(const DevTables& t, const DevTally& tally, Particle& p, int cls,
                                                uint32_t* cnt, const DevSens& sens, double* S, int ss)
{
    const int G = t.num_groups;
    const int K = t.max_reactions;
    const int nk = __ldg(t.class_num_reactions + cls);
    const double* row = t.macro_xs + ((int64_t)cls * G + p.group) * K;
    double current = __ldg(t.sigma_total + cls * G + p.group) * rng_sample(p.seed);
    int sel = -1;
    for (int k = 0; k < nk; k++) {
        current -= __ldg(row + k);
        if (f64_lt0(current)) { sel = k; break; }
    }
    if (sel < 0) {
        // the reference asserts and carries on with an invalid index
        // (CollisionEvent.cc:84); flag it and take the class's last reaction
        raise_flag(tally, QSG_DEV_NO_REACTION);
        sel = nk - 1;
    }
    const int type = t.class_reaction_type[cls * K + sel];
    if (SENS) {
        // group of the incoming particle: the reaction was sampled in it
        const int k = __ldg(sens.param_of + ((int64_t)cls * G + p.group) * 3 + (type - 1));
        if (k >= 0) S[k * ss] += __ldg(sens.inv_theta + k);
    }
    cnt[LC_COLL]++;
    if (type == QSG_REACT_SCATTER) {
        cnt[LC_SCAT]++;
        // 1.0 / mass of NuclearData.cc:64, divided once on the host (same bits)
        const double inv_mass = __ldg(t.material_inv_mass + __ldg(t.class_material + cls));
        double rn = rng_sample(p.seed);
        p.pend_e = p.kinetic_energy * (1.0 - (rn * inv_mass));
        rn = rng_sample(p.seed) * 2.0 - 1.0;
        p.pend_a = rn;
        return COLL_SCATTER;
    }
    if (type == QSG_REACT_FISSION) {
        cnt[LC_FIS]++;
        p.pend_e = __ldg(t.class_reaction_nubar + cls * K + sel);
        return COLL_FISSION;
    }
    if (type == QSG_REACT_ABSORPTION) cnt[LC_ABS]++;
    return COLL_ENDS;
}

// Second part, run by the warp for its parked lanes together: fission
// products (CollisionEvent.cc:125-142; products 1.. to the extra store, and
// the particle itself too when there is more than one), the trajectory update
// and the new energy group.  Returns true to keep tracking.  SENS: fission
// products carry the scores along.
template <bool SENS>
__device__ __forceinline__ bool collision_finish(const DevTables& t, const DevTally& tally, Particle& p, int kind,
                                                 const DevStore& extra, uint32_t* cnt, const DevSens& sens,
                                                 double* S, int ss)
{
    if (kind == COLL_SCATTER) {
        update_trajectory(p.pend_e, p.pend_a, p);
        p.group = energy_group(t, p.kinetic_energy);
        // |velocity| of the new velocity, which the next segment needs
        // (MC_Segment_Outcome.cc recomputes it there; same expression, same
        // bits), computed here while the warp's lanes run together
        p.speed = sqrt(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
        return true;
    }
    double e_out[4], a_out[4];
    int num = (int)(p.pend_e + rng_sample(p.seed));
    if (num > 4) num = 4;  // nuBar < 4 is checked at qsg_create
    for (int o = 0; o < num; o++) {
        double rn = rng_sample(p.seed) / 2.0 + 0.5;
        e_out[o] = (20 * rn * rn);
        rn = rng_sample(p.seed) * 2.0 - 1.0;
        a_out[o] = rn;
    }
    cnt[LC_PROD] += (uint32_t)num;
    if (num == 0) return false;
    for (int s = 1; s < num; s++) {
        Particle sec = p;
        sec.seed = rng_spawn(p.seed);
        sec.identifier = sec.seed;
        update_trajectory(e_out[s], a_out[s], sec);
        uint64_t slot = append_slot(extra);
        if (slot < extra.capacity) {
            store_particle(extra, slot, sec);
            if (SENS) store_scores(extra, slot, S, ss, sens.K);
        } else {
            raise_flag(tally, QSG_DEV_STORE_OVERFLOW);
        }
    }
    update_trajectory(e_out[0], a_out[0], p);
    if (num > 1) {
        uint64_t slot = append_slot(extra);
        if (slot < extra.capacity) {
            store_particle(extra, slot, p);
            if (SENS) store_scores(extra, slot, S, ss, sens.K);
        } else {
            raise_flag(tally, QSG_DEV_STORE_OVERFLOW);
        }
    }
    p.group = energy_group(t, p.kinetic_energy);
    if (num == 1) p.speed = sqrt(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
    return num == 1;
}

// MCT_Reflect_Particle, MCT.cc:400-430.
__device__ __forceinline__ void reflect_particle(const DevTables& t, Particle& p)
{
    const double* pl = t.planes + ((int64_t)p.cell * kFacets + p.facet) * 4;
    double nx = __ldg(pl + 0), ny = __ldg(pl + 1), nz = __ldg(pl + 2);
    double dot = 2.0 * (p.alpha * nx + p.beta * ny + p.gamma * nz);
    if (dot > 0) {
        p.alpha -= dot * nx;
        p.beta -= dot * ny;
        p.gamma -= dot * nz;
    }
    // |velocity| of the unchanged velocity: the cached value has the same bits
    const double speed = (p.speed < 0.0) ? sqrt(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz) : p.speed;
    p.vx = speed * p.alpha;
    p.vy = speed * p.beta;
    p.vz = speed * p.gamma;
    p.speed = -1.0;   // the next segment recomputes |velocity| of the new velocity
}

__device__ __forceinline__ int balance_slot(int local)
{
    switch (local) {
    case LC_SEG: return QSG_BAL_NUM_SEGMENTS;
    case LC_COLL: return QSG_BAL_COLLISION;
    case LC_SCAT: return QSG_BAL_SCATTER;
    case LC_ABS: return QSG_BAL_ABSORB;
    case LC_FIS: return QSG_BAL_FISSION;
    case LC_PROD: return QSG_BAL_PRODUCE;
    case LC_ESC: return QSG_BAL_ESCAPE;
    default: return QSG_BAL_CENSUS;
    }
}

// Per-problem balance counters of a tracking block: a lane keeps the counts of
// the problem it is tracking in registers and adds them here when it moves to
// a particle of another problem or finishes; the block adds the table to
// global memory once at the end.
struct BlockCounters {
    unsigned long long* smem;   // [problems][LC_N], or null when the batch is too large
    const DevTally* tally;
    int replica;

    __device__ __forceinline__ void add(int prob, uint32_t* cnt) const
    {
#pragma unroll
        for (int k = 0; k < LC_N; k++) {
            if (cnt[k]) {
                if (smem) atomicAdd(smem + prob * LC_N + k, (unsigned long long)cnt[k]);
                else
                    atomicAdd(tally->balance + ((int64_t)replica * tally->num_problems + prob) * QSG_BAL_COUNT +
                                  balance_slot(k),
                              (unsigned long long)cnt[k]);
                cnt[k] = 0;
            }
        }
    }

    // Final add of every lane's counts: when the whole warp holds the same
    // problem, the counts are summed with shuffles first.
    __device__ __forceinline__ void add_final(int prob, uint32_t* cnt) const
    {
        const int p0 = __shfl_sync(0xffffffffu, prob, 0);
        if (__all_sync(0xffffffffu, prob == p0)) {
            if (p0 < 0) return;
#pragma unroll
            for (int k = 0; k < LC_N; k++) {
                uint32_t v = cnt[k];
                for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
                cnt[k] = ((threadIdx.x & 31) == 0) ? v : 0;
            }
            if ((threadIdx.x & 31) == 0) add(p0, cnt);
        } else if (prob >= 0) {
            add(prob, cnt);
        }
    }

    template <int BLOCK>
    __device__ __forceinline__ void flush_block() const
    {
        if (!smem) return;
        __syncthreads();
        const int n = tally->num_problems * LC_N;
        for (int k = threadIdx.x; k < n; k += BLOCK) {
            const unsigned long long v = smem[k];
            if (v)
                atomicAdd(tally->balance + ((int64_t)replica * tally->num_problems + k / LC_N) * QSG_BAL_COUNT +
                              balance_slot(k % LC_N),
                          v);
        }
    }
};

// Differential-operator (likelihood-ratio) scores of one flight of length
// l = p.seg_len through cell p.cell in group p.group: the flight's probability
// exp(-Sigma_t l) (times Sigma_t when it ends in a collision) gives
// d log / dtheta_k = -l dSigma_t/dtheta_k (+ dSigma_t/dtheta_k / Sigma_t).  The
// scores S then carry -l dSigma_t/dtheta_k; the collision's own factor is
// folded with reaction selection into d log Sigma_r / dtheta_k in
// collision_event.  The flight's track-length flux l w is tallied with the
// flight's full score, l w (S_k + [collision] dSigma_t/dtheta_k / Sigma_t).
// No counterpart in the reference, which has no sensitivity tallies; the flux
// estimator is Tallies::TallyScalarFlux (Tallies.hh:350-354) summed over groups.
__device__ __forceinline__ void sens_segment(const DevTables& t, const DevSens& sens, const Particle& p, int cls,
                                             bool collided, double* S, int ss)
{
    const double l = p.seg_len;
    if (f64_eq0(l)) return;   // nothing moved: no flight score and no flux tally
    const int64_t base = ((int64_t)cls * t.num_groups + p.group) * 3;
    int pk[3];
    double pd[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        pk[j] = __ldg(sens.param_of + base + j);
        pd[j] = pk[j] >= 0 ? __ldg(sens.dsig + base + j) : 0.0;
        if (pk[j] >= 0) S[pk[j] * ss] -= l * pd[j];
    }
    const double lw = l * p.weight;
    atomicAdd(sens.flux_cell + p.cell, lw);
    double* row = sens.dflux + (int64_t)p.cell * sens.K;
    // parameters without a collision term in this flight
    for (int k = 0; k < sens.K; k++) {
        if (collided && (k == pk[0] || k == pk[1] || k == pk[2])) continue;
        const double v = S[k * ss];
        if (!f64_eq0(v)) atomicAdd(row + k, lw * v);
    }
    if (!collided) return;
    // the (at most three) parameters the collision's cross sections depend
    // on: S_k plus dSigma_t/dtheta_k / Sigma_t of each reaction type that
    // parameter scales, added in reaction order -- the same sum as adding
    // them inside the loop above, which a warp would run for every (k, j)
    // some lane matches
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const int k = pk[j];
        if (k < 0 || (j >= 1 && pk[0] == k) || (j == 2 && pk[1] == k)) continue;   // first occurrence only
        double v = S[k * ss];
#pragma unroll
        for (int j2 = j; j2 < 3; j2++)
            if (pk[j2] == k) v += pd[j2] * p.mean_free_path;
        if (!f64_eq0(v)) atomicAdd(row + k, lw * v);
    }
}

// Persistent tracking pass over the store `in` (its count is read on the
// device): CycleTrackingGuts + CycleTrackingFunction (CycleTracking.cc:14-120)
// one segment per loop trip.  A lane whose history ends pulls the next
// particle index from the work cursor at once (warp-aggregated atomic), so
// long histories do not hold idle lanes; the warp leaves when every lane has
// finished and the queue is empty.
//
// SENS: every history also carries sensitivity scores (shared memory, one
// column per thread after the counters), tallied by sens_segment, at escape
// (leakage and its derivatives) and stored with census / fission particles.
template <int BLOCK, bool SENS>
__global__ void __launch_bounds__(BLOCK, (kTrackMinBlocks * 128 + BLOCK - 1) / BLOCK)
    track_kernel(DevTables t, DevTally tally, DevStore in, DevStore census, DevStore extra,
                 unsigned long long* cursor, DevSens sens)
{
    extern __shared__ unsigned long long s_counts[];
    BlockCounters bc;
    const bool counts_in_smem = tally.num_problems <= kSmemProblems;
    bc.smem = counts_in_smem ? s_counts : nullptr;
    double* S = nullptr;
    if (SENS) S = reinterpret_cast<double*>(s_counts + (counts_in_smem ? tally.num_problems * LC_N : 0)) + threadIdx.x;
    bc.tally = &tally;
    bc.replica = (int)(blockIdx.x % (unsigned)tally.balance_replicas);
    if (bc.smem)
        for (int k = threadIdx.x; k < tally.num_problems * LC_N; k += BLOCK) s_counts[k] = 0;
    __syncthreads();
    uint32_t cnt[LC_N];
#pragma unroll
    for (int k = 0; k < LC_N; k++) cnt[k] = 0;
    int cur_prob = -1;
    // a store that overflowed holds `capacity` particles (its writers raised
    // QSG_DEV_STORE_OVERFLOW)
    const uint64_t n = min((uint64_t)*in.count, in.capacity);
    Particle p;
    bool active = false, exhausted = false;
    int stage = 0;   // 1: parked at a collision
    double* flux_row = tally.flux;
    uint64_t segs_this_history = 0;
    uint64_t next = 0, end = 0;   // this lane's claimed run of queue positions
    const uint64_t chunk = (uint64_t)tally.queue_chunk;
    for (;;) {
        if (!active && !exhausted) {
            if (next >= end) {
                cg::coalesced_group g = cg::coalesced_threads();
                unsigned long long base = 0;
                if (g.thread_rank() == 0) base = atomicAdd(cursor, (unsigned long long)g.size() * chunk);
                base = g.shfl(base, 0);
                next = base + g.thread_rank() * chunk;
                end = next + chunk;
            }
            const uint64_t i = next++;
            if (i < n) {
                load_particle(t, in, i, p);
                if (SENS) load_scores(in, i, S, BLOCK, sens.K);
                if (!(p.speed > 0.0)) raise_flag(tally, QSG_DEV_BAD_FACET);
                const int prob = tally.cell_problem ? __ldg(tally.cell_problem + p.cell) : 0;
                if (prob != cur_prob) {
                    if (cur_prob >= 0) bc.add(cur_prob, cnt);
                    cur_prob = prob;
                }
                // CycleTracking.cc:37-39 replica selection by particle index
                flux_row = tally.flux + (int64_t)(i % (uint64_t)tally.flux_replicas) * t.num_cells * t.num_groups;
                segs_this_history = 0;
                active = true;
            } else {
                exhausted = true;
            }
        }
        if (__all_sync(0xffffffffu, !active)) break;
        // Deferred collisions: a lane whose segment ends in a collision parks
        // its particle; the warp runs the collision work for its parked lanes
        // together once enough of them wait, or when nothing else can run.  A
        // particle's own state and random stream are untouched while it waits,
        // so the results are unchanged.
        const unsigned pend_mask = __ballot_sync(0xffffffffu, active && stage != 0);
        const unsigned run_mask = __ballot_sync(0xffffffffu, active && stage == 0);
        if (pend_mask != 0u && (__popc(pend_mask) >= tally.collision_batch || run_mask == 0u)) {
            if (stage != 0) {
                const int kind =
                    collision_select<SENS>(t, tally, p, __ldg(t.cell_class + p.cell), cnt, sens, S, BLOCK);
                stage = 0;
                active = (kind != COLL_ENDS) && collision_finish<SENS>(t, tally, p, kind, extra, cnt, sens, S, BLOCK);
            }
            continue;
        }
        if (active && stage == 0) {
            bool keep;
            const int cls = __ldg(t.cell_class + p.cell);
            int outcome = segment_outcome(t, tally, p, cls, flux_row);
            if (SENS) sens_segment(t, sens, p, cls, outcome == OUT_COLLISION, S, BLOCK);
            cnt[LC_SEG]++;
            p.num_segments += 1.;
            if (outcome == OUT_COLLISION) {
                stage = 1;
                keep = true;
            } else if (outcome == OUT_FACET) {
                // MC_Facet_Crossing_Event, MC_Facet_Crossing_Event.cc:23-70
                const int64_t fi = (int64_t)p.cell * kFacets + p.facet;
                const uint8_t fe = __ldg(t.adj_facet_event + fi);
                const int ev = fe >> 5;
                if (ev == QSG_ADJ_TRANSIT_ON_PROCESSOR) {
                    p.cell = __ldg(t.adj_cell + fi);
                    p.facet = fe & 31;
                    p.last_event = QSG_EVENT_FACET_TRANSIT_EXIT;
                    keep = true;
                } else if (ev == QSG_ADJ_BOUNDARY_ESCAPE) {
                    cnt[LC_ESC]++;
                    if (SENS) {
                        // leakage (escaping weight) and d leakage / dtheta
                        atomicAdd(sens.leak + cur_prob, p.weight);
                        for (int k = 0; k < sens.K; k++) {
                            const double v = S[k * BLOCK];
                            if (v != 0.0) atomicAdd(sens.dleak + (int64_t)cur_prob * sens.K + k, p.weight * v);
                        }
                    }
                    p.last_event = QSG_EVENT_FACET_ESCAPE;
                    p.species = -1;
                    keep = false;
                } else if (ev == QSG_ADJ_BOUNDARY_REFLECTION) {
                    p.last_event = QSG_EVENT_FACET_REFLECTION;
                    reflect_particle(t, p);
                    keep = true;
                } else {
                    raise_flag(tally, QSG_DEV_OFF_PROCESSOR);
                    keep = false;
                }
            } else {
                // census: ParticleVault::pushParticle (ParticleVault.hh:86-93)
                uint64_t slot = append_slot(census);
                if (slot < census.capacity) {
                    store_particle(census, slot, p);
                    if (SENS) store_scores(census, slot, S, BLOCK, sens.K);
                } else {
                    raise_flag(tally, QSG_DEV_STORE_OVERFLOW);
                }
                cnt[LC_CEN]++;
                keep = false;
            }
            if (keep && ++segs_this_history >= tally.max_segments) {
                raise_flag(tally, QSG_DEV_SEGMENT_LIMIT);
                keep = false;
                stage = 0;
            }
            active = keep;
        }
    }
    bc.add_final(cur_prob, cnt);
    bc.flush_block<BLOCK>();
}

// ------------------------------------------------------------------------
// Particle-pool variant of the tracking pass.
//
// The lane-resident kernel above keeps one history per lane, so a warp's steps
// run with the lanes whose particle happens to need that step (on config2
// about 21 of 32 lanes in segment steps and 18 in collision steps), and an
// FP64 warp instruction costs the FP64 pipe the same whatever its active
// lanes.  Here each warp owns a pool of POOL particles in shared memory;
// every step picks one kind of work -- a segment for particles ready to move,
// or the collision (reaction selection + trajectory update) for particles
// parked at a collision -- and hands up to 32 such particles to the lanes, so
// steps run full while the pool holds enough of one kind.  Every particle
// still follows its own history with its own random stream, in the
// reference's order, so the results are those of the lane-resident kernel.
//
// Pool sizes: 64 particles per warp for the plain kernel; with K sensitivity
// scores per particle, 64, 48 or 32, the largest that still leaves room for
// three 4-warp blocks per SM (pool_for_scores).
#ifndef QSG_POOL
#define QSG_POOL 64
#endif
#ifndef QSG_POOL_SENS_MAX
#define QSG_POOL_SENS_MAX 64
#endif
constexpr int kPoolPlain = QSG_POOL;
constexpr int kPoolD = 18, kPoolU = 2, kPoolI = 9;
constexpr int kSlotBytes = kPoolD * 8 + kPoolU * 8 + kPoolI * 4;   // 196
__host__ __device__ constexpr size_t pool_bytes_per_warp(int pool) { return (size_t)kSlotBytes * pool; }
enum { PD_X, PD_Y, PD_Z, PD_VX, PD_VY, PD_VZ, PD_A, PD_B, PD_G, PD_E, PD_W, PD_TTC, PD_AGE, PD_NMFP, PD_NSEG,
       PD_SPEED, PD_IMFP, PD_MFP };
// PI_PACK = facet | flux replica << 8 | group << 16
enum { PI_LAST, PI_NCOLL, PI_BREED, PI_SPECIES, PI_DOMAIN, PI_CELL, PI_PACK, PI_KEY, PI_SEGS };

// Shared memory a block of the pool kernel needs (counters, pools, scores).
size_t track_pool_smem_bytes(int block, int num_problems, int K, int pool)
{
    const size_t counts = num_problems <= kSmemProblems ? (size_t)num_problems * LC_N * 8 : 0;
    const int warps = block / 32;
    return counts + (size_t)warps * pool_bytes_per_warp(pool) + (size_t)warps * K * pool * sizeof(double);
}

// Pool size of the sensitivity kernel for K scores: the largest of 64, 48, 32
// whose 4-warp block fits three times into an SM's 228 KB of shared memory.
int pool_for_scores(int K, int num_problems)
{
    for (int pool : {64, 48, 32})
        if (pool <= QSG_POOL_SENS_MAX && 3 * (track_pool_smem_bytes(128, num_problems, K, pool) + 1024) <= 228 * 1024)
            return pool;
    return 32;
}

struct PoolView {
    double* d;      // [kPoolD][POOL]
    uint64_t* u;    // [2][POOL]: seed, identifier
    int32_t* i;     // [kPoolI][POOL]
};

// Extra per-slot state the pool keeps beside the particle record.
struct SlotState {
    int prob, rep;
    uint32_t segs;
};

template <int POOL>
__device__ __forceinline__ void pool_get(const PoolView& v, int s, const DevTally& tally, Particle& p, SlotState& st)
{
    const double* d = v.d + s;
    p.x = d[PD_X * POOL]; p.y = d[PD_Y * POOL]; p.z = d[PD_Z * POOL];
    p.vx = d[PD_VX * POOL]; p.vy = d[PD_VY * POOL]; p.vz = d[PD_VZ * POOL];
    p.alpha = d[PD_A * POOL]; p.beta = d[PD_B * POOL]; p.gamma = d[PD_G * POOL];
    p.kinetic_energy = d[PD_E * POOL]; p.weight = d[PD_W * POOL];
    p.time_to_census = d[PD_TTC * POOL]; p.age = d[PD_AGE * POOL];
    p.num_mean_free_paths = d[PD_NMFP * POOL]; p.num_segments = d[PD_NSEG * POOL];
    p.speed = d[PD_SPEED * POOL]; p.inv_mfp = d[PD_IMFP * POOL]; p.mean_free_path = d[PD_MFP * POOL];
    p.seed = v.u[s]; p.identifier = v.u[POOL + s];
    const int32_t* i = v.i + s;
    p.last_event = i[PI_LAST * POOL]; p.num_collisions = i[PI_NCOLL * POOL]; p.breed = i[PI_BREED * POOL];
    p.species = i[PI_SPECIES * POOL]; p.domain = i[PI_DOMAIN * POOL]; p.cell = i[PI_CELL * POOL];
    const uint32_t pack = (uint32_t)i[PI_PACK * POOL];
    p.facet = (int)(pack & 0xffu);
    st.rep = (int)((pack >> 8) & 0xffu);
    p.group = (int)(pack >> 16);
    p.xs_key = i[PI_KEY * POOL];
    st.segs = (uint32_t)i[PI_SEGS * POOL];
    st.prob = tally.cell_problem ? __ldg(tally.cell_problem + p.cell) : 0;
}

template <int POOL>
__device__ __forceinline__ void pool_put(const PoolView& v, int s, const Particle& p, const SlotState& st)
{
    double* d = v.d + s;
    d[PD_X * POOL] = p.x; d[PD_Y * POOL] = p.y; d[PD_Z * POOL] = p.z;
    d[PD_VX * POOL] = p.vx; d[PD_VY * POOL] = p.vy; d[PD_VZ * POOL] = p.vz;
    d[PD_A * POOL] = p.alpha; d[PD_B * POOL] = p.beta; d[PD_G * POOL] = p.gamma;
    d[PD_E * POOL] = p.kinetic_energy; d[PD_W * POOL] = p.weight;
    d[PD_TTC * POOL] = p.time_to_census; d[PD_AGE * POOL] = p.age;
    d[PD_NMFP * POOL] = p.num_mean_free_paths; d[PD_NSEG * POOL] = p.num_segments;
    d[PD_SPEED * POOL] = p.speed; d[PD_IMFP * POOL] = p.inv_mfp; d[PD_MFP * POOL] = p.mean_free_path;
    v.u[s] = p.seed; v.u[POOL + s] = p.identifier;
    int32_t* i = v.i + s;
    i[PI_LAST * POOL] = p.last_event; i[PI_NCOLL * POOL] = p.num_collisions; i[PI_BREED * POOL] = p.breed;
    i[PI_SPECIES * POOL] = p.species; i[PI_DOMAIN * POOL] = p.domain; i[PI_CELL * POOL] = p.cell;
    i[PI_PACK * POOL] = (int32_t)((uint32_t)p.facet | ((uint32_t)st.rep << 8) | ((uint32_t)p.group << 16));
    i[PI_KEY * POOL] = p.xs_key;
    i[PI_SEGS * POOL] = (int32_t)st.segs;
}

// Position of the n-th (0-based) set bit of m; n < popcount(m).
__device__ __forceinline__ int nth_set_bit(uint64_t m, int n)
{
    const uint32_t lo = (uint32_t)m;
    const int c = __popc(lo);
    uint32_t w32 = lo;
    int base = 0;
    if (n >= c) {
        n -= c;
        w32 = (uint32_t)(m >> 32);
        base = 32;
    }
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) {
        const uint32_t low = w32 & ((1u << w) - 1u);
        const int cl = __popc(low);
        if (n >= cl) {
            n -= cl;
            w32 >>= w;
            base += w;
        } else {
            w32 = low;
        }
    }
    return base;
}

// Warp-uniform set of pool slots (up to 128): bits 0..63 in lo, 64..127 in hi.
struct SlotMask {
    uint64_t lo, hi;
    __device__ __forceinline__ int count() const { return __popcll(lo) + __popcll(hi); }
    __device__ __forceinline__ int nth(int n) const
    {
        const int c = __popcll(lo);
        return n < c ? nth_set_bit(lo, n) : 64 + nth_set_bit(hi, n - c);
    }
    __device__ __forceinline__ SlotMask operator|(const SlotMask& o) const { return {lo | o.lo, hi | o.hi}; }
    __device__ __forceinline__ SlotMask operator&(const SlotMask& o) const { return {lo & o.lo, hi & o.hi}; }
    __device__ __forceinline__ SlotMask operator~() const { return {~lo, ~hi}; }
};

template <int POOL>
__device__ __forceinline__ SlotMask all_slots()
{
    return {POOL >= 64 ? ~0ull : ((1ull << POOL) - 1ull), POOL <= 64 ? 0ull : (POOL >= 128 ? ~0ull : ((1ull << (POOL - 64)) - 1ull))};
}

// OR over the warp of one slot bit per lane (slot < 0: none).
template <int POOL>
__device__ __forceinline__ SlotMask warp_slots(int slot)
{
    SlotMask m;
    const uint32_t b0 = __reduce_or_sync(0xffffffffu, (slot >= 0 && slot < 32) ? (1u << slot) : 0u);
    const uint32_t b1 = __reduce_or_sync(0xffffffffu, (slot >= 32 && slot < 64) ? (1u << (slot - 32)) : 0u);
    m.lo = ((uint64_t)b1 << 32) | b0;
    m.hi = 0;
    if (POOL > 64) {
        const uint32_t b2 = __reduce_or_sync(0xffffffffu, (slot >= 64 && slot < 96) ? (1u << (slot - 64)) : 0u);
        uint32_t b3 = 0;
        if (POOL > 96) b3 = __reduce_or_sync(0xffffffffu, (slot >= 96) ? (1u << (slot - 96)) : 0u);
        m.hi = ((uint64_t)b3 << 32) | b2;
    }
    return m;
}

template <int BLOCK, bool SENS, int POOL>
__global__ void __launch_bounds__(BLOCK, (kTrackMinBlocks * 128 + BLOCK - 1) / BLOCK)
    track_pool_kernel(DevTables t, DevTally tally, DevStore in, DevStore census, DevStore extra,
                      unsigned long long* cursor, DevSens sens)
{
    static_assert(POOL >= 32 && POOL <= 128, "pool size");
    constexpr size_t kPoolBytesPerWarp = pool_bytes_per_warp(POOL);
    extern __shared__ unsigned long long s_counts[];
    BlockCounters bc;
    const bool counts_in_smem = tally.num_problems <= kSmemProblems;
    bc.smem = counts_in_smem ? s_counts : nullptr;
    bc.tally = &tally;
    bc.replica = (int)(blockIdx.x % (unsigned)tally.balance_replicas);
    if (bc.smem)
        for (int k = threadIdx.x; k < tally.num_problems * LC_N; k += BLOCK) s_counts[k] = 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    char* pool_base = reinterpret_cast<char*>(s_counts + (counts_in_smem ? tally.num_problems * LC_N : 0));
    char* mine = pool_base + (size_t)warp * kPoolBytesPerWarp;
    PoolView v;
    v.d = reinterpret_cast<double*>(mine);
    v.u = reinterpret_cast<uint64_t*>(mine + (size_t)kPoolD * 8 * POOL);
    v.i = reinterpret_cast<int32_t*>(mine + (size_t)(kPoolD + kPoolU) * 8 * POOL);
    double* s_scores = nullptr;   // [K][POOL] of this warp
    if (SENS)
        s_scores = reinterpret_cast<double*>(pool_base + (size_t)(BLOCK / 32) * kPoolBytesPerWarp) +
                   (size_t)warp * sens.K * POOL;
    __syncthreads();
    uint32_t cnt[LC_N];
#pragma unroll
    for (int k = 0; k < LC_N; k++) cnt[k] = 0;
    int cur_prob = -1;
    // a store that overflowed holds `capacity` particles (its writers raised
    // QSG_DEV_STORE_OVERFLOW)
    const uint64_t n = min((uint64_t)*in.count, in.capacity);
    SlotMask ready = {0, 0}, coll = {0, 0};   // warp-uniform
    bool exhausted = false;
    for (;;) {
        // refill empty slots from the work queue (warp-aggregated claim)
        const SlotMask empty = ~(ready | coll) & all_slots<POOL>();
        const int n_empty = empty.count();
        const int nr0 = ready.count(), nc0 = coll.count();
        if (!exhausted && n_empty > 0 && (n_empty >= tally.pool_refill || (nr0 < 32 && nc0 < 32))) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(cursor, (unsigned long long)n_empty);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + (unsigned long long)n_empty >= n) exhausted = true;
            int filled[(POOL + 31) / 32];
#pragma unroll
            for (int r = 0; r < (POOL + 31) / 32; r++) {
                filled[r] = -1;
                const int k = lane + 32 * r;
                const uint64_t i = base + (uint64_t)k;
                if (k < n_empty && i < n) {
                    const int slot = empty.nth(k);
                    Particle p;
                    load_particle(t, in, i, p);
                    if (!(p.speed > 0.0)) raise_flag(tally, QSG_DEV_BAD_FACET);
                    SlotState st;
                    // CycleTracking.cc:37-39 replica selection by particle index
                    st.rep = (int)(i % (uint64_t)tally.flux_replicas);
                    st.segs = 0;
                    st.prob = 0;
                    pool_put<POOL>(v, slot, p, st);
                    if (SENS) load_scores(in, i, s_scores + slot, POOL, sens.K);
                    filled[r] = slot;
                }
            }
#pragma unroll
            for (int r = 0; r < (POOL + 31) / 32; r++) ready = ready | warp_slots<POOL>(filled[r]);
        }
        const int nr = ready.count(), nc = coll.count();
        if (nr == 0 && nc == 0) {
            if (exhausted) break;
            continue;
        }
        const bool do_coll = (nc >= tally.pool_collision_step) || (nc > nr);
        const SlotMask sel = do_coll ? coll : ready;
        const int nsel = do_coll ? nc : nr;
        int slot = -1, next_state = 0;   // 0 empty, 1 ready, 2 collision pending
        if (lane < nsel) {
            slot = sel.nth(lane);
            Particle p;
            SlotState st;
            pool_get<POOL>(v, slot, tally, p, st);
            if (st.prob != cur_prob) {
                if (cur_prob >= 0) bc.add(cur_prob, cnt);
                cur_prob = st.prob;
            }
            double* S = SENS ? s_scores + slot : nullptr;
            const int cls = __ldg(t.cell_class + p.cell);
            if (do_coll) {
                // CollisionEvent, both parts (see collision_select / collision_finish)
                const int kind = collision_select<SENS>(t, tally, p, cls, cnt, sens, S, POOL);
                const bool alive = (kind != COLL_ENDS) &&
                                   collision_finish<SENS>(t, tally, p, kind, extra, cnt, sens, S, POOL);
                next_state = alive ? 1 : 0;
            } else {
                double* flux_row = tally.flux + (int64_t)st.rep * t.num_cells * t.num_groups;
                const int outcome = segment_outcome(t, tally, p, cls, flux_row);
                if (SENS) sens_segment(t, sens, p, cls, outcome == OUT_COLLISION, S, POOL);
                cnt[LC_SEG]++;
                p.num_segments += 1.;
                if (outcome == OUT_COLLISION) {
                    next_state = 2;
                } else if (outcome == OUT_FACET) {
                    // MC_Facet_Crossing_Event, MC_Facet_Crossing_Event.cc:23-70
                    const int64_t fi = (int64_t)p.cell * kFacets + p.facet;
                    const uint8_t fe = __ldg(t.adj_facet_event + fi);
                    const int ev = fe >> 5;
                    if (ev == QSG_ADJ_TRANSIT_ON_PROCESSOR) {
                        p.cell = __ldg(t.adj_cell + fi);
                        p.facet = fe & 31;
                        p.last_event = QSG_EVENT_FACET_TRANSIT_EXIT;
                        next_state = 1;
                    } else if (ev == QSG_ADJ_BOUNDARY_ESCAPE) {
                        cnt[LC_ESC]++;
                        if (SENS) {
                            atomicAdd(sens.leak + st.prob, p.weight);
                            for (int k = 0; k < sens.K; k++) {
                                const double sv = S[k * POOL];
                                if (!f64_eq0(sv)) atomicAdd(sens.dleak + (int64_t)st.prob * sens.K + k, p.weight * sv);
                            }
                        }
                        p.last_event = QSG_EVENT_FACET_ESCAPE;
                        p.species = -1;
                        next_state = 0;
                    } else if (ev == QSG_ADJ_BOUNDARY_REFLECTION) {
                        p.last_event = QSG_EVENT_FACET_REFLECTION;
                        reflect_particle(t, p);
                        next_state = 1;
                    } else {
                        raise_flag(tally, QSG_DEV_OFF_PROCESSOR);
                        next_state = 0;
                    }
                } else {
                    // census: ParticleVault::pushParticle (ParticleVault.hh:86-93)
                    uint64_t cs = append_slot(census);
                    if (cs < census.capacity) {
                        store_particle(census, cs, p);
                        if (SENS) store_scores(census, cs, S, POOL, sens.K);
                    } else {
                        raise_flag(tally, QSG_DEV_STORE_OVERFLOW);
                    }
                    cnt[LC_CEN]++;
                    next_state = 0;
                }
                if (next_state != 0 && (uint64_t)(++st.segs) >= tally.max_segments) {
                    raise_flag(tally, QSG_DEV_SEGMENT_LIMIT);
                    next_state = 0;
                }
            }
            if (next_state != 0) pool_put<POOL>(v, slot, p, st);
        }
        const SlotMask taken = warp_slots<POOL>(slot);
        const SlotMask now_ready = warp_slots<POOL>(next_state == 1 ? slot : -1);
        const SlotMask now_coll = warp_slots<POOL>(next_state == 2 ? slot : -1);
        if (do_coll) coll = coll & ~taken;
        else ready = ready & ~taken;
        ready = ready | now_ready;
        coll = coll | now_coll;
    }
    bc.add_final(cur_prob, cnt);
    bc.flush_block<BLOCK>();
}

// ------------------------------------------------------------------------
// Host side.

}  // namespace qsg

#include "handle.cuh"

namespace qsg {

int set_device(const QsgHandle* h) {
    QSG_CUDA(cudaSetDevice(h->device));
    return QSG_OK;
}

DevTally tally_view(QsgHandle* h)
{
    DevTally t{};
    t.flux = h->flux.ptr;
    t.balance = h->balance.ptr;
    t.error_flags = h->flags.ptr;
    t.flux_replicas = h->flux_replicas;
    t.balance_replicas = h->balance_replicas;
    t.max_segments = h->max_segments;
    t.cell_problem = h->num_problems > 1 ? h->cell_problem.ptr : nullptr;
    t.num_problems = h->num_problems;
    t.collision_batch = h->collision_batch;
    t.queue_chunk = h->queue_chunk;
    t.pool_collision_step = h->pool_collision_step;
    t.pool_refill = h->pool_refill;
    t.cell_tally = h->exp_tally ? h->cell_tally.ptr : nullptr;
    return t;
}

size_t track_smem_bytes(const QsgHandle* h)
{
    return h->num_problems <= kSmemProblems ? (size_t)h->num_problems * LC_N * sizeof(unsigned long long) : 0;
}

size_t track_smem_bytes_sens(const QsgHandle* h)
{
    return track_smem_bytes(h) + (size_t)h->sens.K * h->block_size * sizeof(double);
}

size_t track_pool_smem_bytes(int block, int num_problems, int K, int pool);
int pool_for_scores(int K, int num_problems);

// The pool packs facet, flux replica and group into one word.
bool pool_kernel_usable(const QsgHandle* h) { return h->num_groups <= 65535 && h->flux_replicas <= 255; }

template <int B>
const void* pool_kernel_fn(bool sens, int pool)
{
    if (!sens) return (const void*)track_pool_kernel<B, false, kPoolPlain>;
    if (pool == 64) return (const void*)track_pool_kernel<B, true, 64>;
    if (pool == 48) return (const void*)track_pool_kernel<B, true, 48>;
    return (const void*)track_pool_kernel<B, true, 32>;
}

// The stores of one tracking pass: input, census, fission products.
struct PassStores {
    DevStore in, census, extra;
};

template <int B, bool SENS, int POOL>
void launch_pool_t(QsgHandle* h, int grid, size_t smem, cudaStream_t s, const DevTally& tv,
                   unsigned long long* cursor, const PassStores& ps)
{
    track_pool_kernel<B, SENS, POOL><<<grid, B, smem, s>>>(h->tables, tv, ps.in, ps.census, ps.extra, cursor,
                                                           SENS ? h->sens : DevSens{});
}

template <int B>
void launch_pool(QsgHandle* h, cudaStream_t s, const DevTally& tv, unsigned long long* cursor, const PassStores& ps,
                 bool sens)
{
    if (!sens || h->sens.K == 0) {
        launch_pool_t<B, false, kPoolPlain>(h, h->pool_blocks,
                                            track_pool_smem_bytes(B, h->num_problems, 0, kPoolPlain), s, tv, cursor,
                                            ps);
        return;
    }
    const size_t smem = track_pool_smem_bytes(B, h->num_problems, h->sens.K, h->pool_sens);
    if (h->pool_sens == 64) launch_pool_t<B, true, 64>(h, h->pool_sens_blocks, smem, s, tv, cursor, ps);
    else if (h->pool_sens == 48) launch_pool_t<B, true, 48>(h, h->pool_sens_blocks, smem, s, tv, cursor, ps);
    else launch_pool_t<B, true, 32>(h, h->pool_sens_blocks, smem, s, tv, cursor, ps);
}

// Persistent grid for the current block size: SMs x resident blocks.
int configure_track_grid(QsgHandle* h)
{
    int per_sm = 0;
    const size_t smem = track_smem_bytes(h);
    if (h->block_size == 256)
        QSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel<256, false>, 256, smem));
    else
        QSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel<128, false>, 128, smem));
    h->track_blocks = h->num_sms * (per_sm > 0 ? per_sm : 1);
    if (h->sens.K > 0) {
        // the sensitivity kernel adds one column of K scores per thread
        const size_t ss = track_smem_bytes_sens(h);
        per_sm = 0;
        if (h->block_size == 256) {
            QSG_CUDA(cudaFuncSetAttribute(track_kernel<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ss));
            QSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel<256, true>, 256, ss));
        } else {
            QSG_CUDA(cudaFuncSetAttribute(track_kernel<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ss));
            QSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel<128, true>, 128, ss));
        }
        h->sens_track_blocks = h->num_sms * (per_sm > 0 ? per_sm : 1);
    }
    // particle-pool kernels (their pools live in dynamic shared memory)
    h->pool_sens = pool_for_scores(h->sens.K, h->num_problems);
    for (int sens = 0; sens < 2; sens++) {
        if (sens && h->sens.K == 0) continue;
        const int pool = sens ? h->pool_sens : kPoolPlain;
        const size_t ps = track_pool_smem_bytes(h->block_size, h->num_problems, sens ? h->sens.K : 0, pool);
        const void* fn = h->block_size == 256 ? pool_kernel_fn<256>(sens, pool) : pool_kernel_fn<128>(sens, pool);
        QSG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ps));
        per_sm = 0;
        QSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, h->block_size, ps));
        (sens ? h->pool_sens_blocks : h->pool_blocks) = h->num_sms * (per_sm > 0 ? per_sm : 1);
    }
    return QSG_OK;
}

namespace {

int validate_problem(const QsgProblem* p)
{
    if (p->num_groups < 1 || !p->energies) return fail(QSG_ERR_INVALID, "problem: num_groups/energies missing");
    if (p->num_isotopes < 1 || !p->isotope_reaction_offset || !p->reaction_type || !p->reaction_nubar ||
        !p->reaction_xs)
        return fail(QSG_ERR_INVALID, "problem: nuclear data missing");
    if (p->num_materials < 1 || !p->material_isotope_offset || !p->material_isotope_gid ||
        !p->material_atom_fraction || !p->material_mass)
        return fail(QSG_ERR_INVALID, "problem: materials missing");
    if (p->num_cells < 1 || !p->nodes || !p->cell_points || !p->facet_local_points || !p->facet_planes ||
        !p->facet_event || !p->facet_adjacent_cell || !p->facet_adjacent_facet || !p->cell_material ||
        !p->cell_number_density)
        return fail(QSG_ERR_INVALID, "problem: mesh tables missing");
    for (int k = 0; k < 72; k++)
        if (p->facet_local_points[k] != kFacetLocalHost[k / 3][k % 3])
            return fail(QSG_ERR_UNSUPPORTED, "problem: facet_local_points differ from Quicksilver's 24-facet "
                        "hex-cell convention (MC_Domain.cc:41-46)");
    for (int i = 0; i < p->num_isotopes; i++)
        if (p->isotope_reaction_offset[i + 1] < p->isotope_reaction_offset[i])
            return fail(QSG_ERR_INVALID, "problem: isotope_reaction_offset not monotone");
    const int R = p->isotope_reaction_offset[p->num_isotopes];
    for (int r = 0; r < R; r++) {
        if (p->reaction_type[r] < QSG_REACT_SCATTER || p->reaction_type[r] > QSG_REACT_FISSION)
            return fail(QSG_ERR_INVALID, "problem: reaction %d has undefined type", r);
        if (p->reaction_type[r] == QSG_REACT_FISSION && !(p->reaction_nubar[r] < 4.0))
            return fail(QSG_ERR_INVALID, "problem: fission nuBar %.17g can exceed the 4 products per collision "
                        "(CollisionEvent.cc:15)", p->reaction_nubar[r]);
    }
    for (int m = 0; m < p->num_materials; m++) {
        int k0 = p->material_isotope_offset[m], k1 = p->material_isotope_offset[m + 1];
        if (k1 <= k0) return fail(QSG_ERR_INVALID, "problem: material %d has no isotopes", m);
        for (int k = k0; k < k1; k++)
            if (p->material_isotope_gid[k] < 0 || p->material_isotope_gid[k] >= p->num_isotopes)
                return fail(QSG_ERR_INVALID, "problem: material %d names isotope out of range", m);
    }
    const int64_t C = p->num_cells;
    for (int64_t c = 0; c < C; c++) {
        if (p->cell_material[c] < 0 || p->cell_material[c] >= p->num_materials)
            return fail(QSG_ERR_INVALID, "problem: cell %lld material out of range", (long long)c);
        for (int k = 0; k < kCellPoints; k++)
            if (p->cell_points[c * kCellPoints + k] < 0 || p->cell_points[c * kCellPoints + k] >= p->num_nodes)
                return fail(QSG_ERR_INVALID, "problem: cell %lld point out of range", (long long)c);
        for (int f = 0; f < kFacets; f++) {
            int ev = p->facet_event[c * kFacets + f];
            int ac = p->facet_adjacent_cell[c * kFacets + f];
            int af = p->facet_adjacent_facet[c * kFacets + f];
            if (ev < QSG_ADJ_UNDEFINED || ev > QSG_ADJ_TRANSIT_OFF_PROCESSOR)
                return fail(QSG_ERR_INVALID, "problem: facet event out of range");
            if (ev == QSG_ADJ_TRANSIT_OFF_PROCESSOR)
                return fail(QSG_ERR_UNSUPPORTED, "problem: off-processor facets need the multi-domain exchange, "
                            "which this single-domain library does not implement");
            if (ac < 0 || ac >= C || af < 0 || af >= kFacets)
                return fail(QSG_ERR_INVALID, "problem: facet adjacency out of range");
        }
    }
    // consistencyCheck (initMC.cc:202-234): the facet across from a facet
    // leads back to it (a boundary facet is its own neighbour)
    for (int64_t c = 0; c < C; c++)
        for (int f = 0; f < kFacets; f++) {
            const int64_t ac = p->facet_adjacent_cell[c * kFacets + f];
            const int af = p->facet_adjacent_facet[c * kFacets + f];
            if (p->facet_adjacent_cell[ac * kFacets + af] != c || p->facet_adjacent_facet[ac * kFacets + af] != f)
                return fail(QSG_ERR_INVALID, "problem: facet adjacency not symmetric: cell %lld facet %d -> cell %lld "
                            "facet %d, which leads to cell %d facet %d", (long long)c, f, (long long)ac, af,
                            p->facet_adjacent_cell[ac * kFacets + af], p->facet_adjacent_facet[ac * kFacets + af]);
        }
    return QSG_OK;
}

// Fold the per-cell tables into cross-section classes and upload.
int upload_tables(QsgHandle* h, const QsgProblem* p)
{
    const int G = p->num_groups;
    const int64_t C = p->num_cells;
    // class = (material, number density) pair
    std::map<std::pair<int, uint64_t>, int> class_of;
    std::vector<int32_t> cell_class(C);
    std::vector<std::pair<int, double>> classes;
    for (int64_t c = 0; c < C; c++) {
        double nd = p->cell_number_density[c];
        uint64_t bits;
        memcpy(&bits, &nd, 8);
        auto key = std::make_pair((int)p->cell_material[c], bits);
        auto it = class_of.find(key);
        if (it == class_of.end()) {
            int id = (int)classes.size();
            class_of.emplace(key, id);
            classes.emplace_back(p->cell_material[c], nd);
            cell_class[c] = id;
        } else {
            cell_class[c] = it->second;
        }
    }
    int K = 1;
    for (auto& cl : classes) {
        int m = cl.first, nk = 0;
        for (int k = p->material_isotope_offset[m]; k < p->material_isotope_offset[m + 1]; k++) {
            int iso = p->material_isotope_gid[k];
            nk += p->isotope_reaction_offset[iso + 1] - p->isotope_reaction_offset[iso];
        }
        K = std::max(K, nk);
    }
    const int NCL = (int)classes.size();
    std::vector<double> sigma_total((size_t)NCL * G), macro((size_t)NCL * G * K, 0.0), nubar((size_t)NCL * K, 0.0);
    std::vector<int32_t> nreact(NCL), cmat(NCL);
    std::vector<int8_t> ctype((size_t)NCL * K, 0);
    std::vector<uint8_t> cconst((size_t)NCL * K, 0);
    for (int ci = 0; ci < NCL; ci++) {
        int m = classes[ci].first;
        double nd = classes[ci].second;
        cmat[ci] = m;
        int kk = 0;
        for (int k = p->material_isotope_offset[m]; k < p->material_isotope_offset[m + 1]; k++) {
            int iso = p->material_isotope_gid[k];
            for (int r = p->isotope_reaction_offset[iso]; r < p->isotope_reaction_offset[iso + 1]; r++) {
                ctype[(size_t)ci * K + kk] = (int8_t)p->reaction_type[r];
                nubar[(size_t)ci * K + kk] = p->reaction_nubar[r];
                kk++;
            }
        }
        nreact[ci] = kk;
        for (int g = 0; g < G; g++) {
            // weightedMacroscopicCrossSection (MacroscopicCrossSection.cc:58-81)
            double sum = 0.0;
            kk = 0;
            for (int k = p->material_isotope_offset[m]; k < p->material_isotope_offset[m + 1]; k++) {
                int iso = p->material_isotope_gid[k];
                double af = p->material_atom_fraction[k];
                double micro_total = 0.0;
                for (int r = p->isotope_reaction_offset[iso]; r < p->isotope_reaction_offset[iso + 1]; r++)
                    micro_total += p->reaction_xs[(int64_t)r * G + g];
                bool zero = (af == 0.0 || nd == 0.0);
                sum += zero ? 1e-20 : af * nd * micro_total;
                for (int r = p->isotope_reaction_offset[iso]; r < p->isotope_reaction_offset[iso + 1]; r++) {
                    macro[((size_t)ci * G + g) * K + kk] = zero ? 1e-20 : af * nd * p->reaction_xs[(int64_t)r * G + g];
                    cconst[(size_t)ci * K + kk] = zero ? 1 : 0;
                    kk++;
                }
            }
            sigma_total[(size_t)ci * G + g] = sum;
        }
    }
    // mesh
    std::vector<double> nodes((size_t)C * kCellPoints * 3), center((size_t)C * 3), planes((size_t)C * kFacets * 4);
    std::vector<int32_t> adj_cell((size_t)C * kFacets);
    std::vector<uint8_t> adj_fe((size_t)C * kFacets);
    for (int64_t c = 0; c < C; c++) {
        double sx = 0, sy = 0, sz = 0;
        for (int k = 0; k < kCellPoints; k++) {
            const double* nd = p->nodes + 3 * (int64_t)p->cell_points[c * kCellPoints + k];
            nodes[(c * kCellPoints + k) * 3 + 0] = nd[0];
            nodes[(c * kCellPoints + k) * 3 + 1] = nd[1];
            nodes[(c * kCellPoints + k) * 3 + 2] = nd[2];
            sx += nd[0];
            sy += nd[1];
            sz += nd[2];
        }
        // MCT_Cell_Position_3D_G (MCT.cc:231-253)
        double one_over = 1.0 / ((double)kCellPoints);
        center[c * 3 + 0] = sx * one_over;
        center[c * 3 + 1] = sy * one_over;
        center[c * 3 + 2] = sz * one_over;
        for (int f = 0; f < kFacets; f++) {
            for (int a = 0; a < 4; a++) planes[(c * kFacets + f) * 4 + a] = p->facet_planes[(c * kFacets + f) * 4 + a];
            adj_cell[c * kFacets + f] = p->facet_adjacent_cell[c * kFacets + f];
            adj_fe[c * kFacets + f] =
                (uint8_t)(p->facet_adjacent_facet[c * kFacets + f] | (p->facet_event[c * kFacets + f] << 5));
        }
    }
    std::vector<double> energies(p->energies, p->energies + G + 1);
    std::vector<double> mass(p->num_materials);
    for (int m = 0; m < p->num_materials; m++) mass[m] = 1.0 / p->material_mass[m];
    int st;
    // mean free path per (class, group): the reference's 1.0 / sigma, an IEEE
    // division whose bits the host reproduces
    std::vector<double> mfp(sigma_total.size());
    for (size_t k = 0; k < mfp.size(); k++) mfp[k] = (sigma_total[k] == 0.0) ? kHugeDouble : 1.0 / sigma_total[k];
    std::vector<double> inv_mfp(mfp.size());
    for (size_t k = 0; k < mfp.size(); k++) inv_mfp[k] = 1.0 / mfp[k];   // IEEE division: RN(1 / mfp)
    if ((st = h->mfp_table.upload(mfp)) || (st = h->inv_mfp_table.upload(inv_mfp))) return st;
    if ((st = h->energies.upload(energies)) || (st = h->sigma_total.upload(sigma_total)) ||
        (st = h->macro_xs.upload(macro)) || (st = h->class_nubar.upload(nubar)) ||
        (st = h->material_mass.upload(mass)) || (st = h->cell_nodes.upload(nodes)) ||
        (st = h->cell_center.upload(center)) || (st = h->planes.upload(planes)) ||
        (st = h->class_num_reactions.upload(nreact)) || (st = h->class_material.upload(cmat)) ||
        (st = h->cell_class.upload(cell_class)) || (st = h->adj_cell.upload(adj_cell)) ||
        (st = h->class_type.upload(ctype)) || (st = h->adj_facet_event.upload(adj_fe)))
        return st;
    h->h_class_material = cmat;
    h->h_class_type = ctype;
    h->h_class_const = cconst;
    h->h_class_macro = macro;
    h->num_classes = NCL;
    h->max_reactions = K;
    DevTables& t = h->tables;
    t.num_groups = G;
    t.num_cells = (int32_t)C;
    t.max_reactions = K;
    t.energies = h->energies.ptr;
    t.sigma_total = h->sigma_total.ptr;
    t.mfp_table = h->mfp_table.ptr;
    t.inv_mfp_table = h->inv_mfp_table.ptr;
    // group hint: accepted when every edge but the last lies within a quarter
    // group of the log-linear fit through the first two
    t.group_hint_ln0 = 0.0f;
    t.group_hint_scale = 0.0f;
    if (G >= 2 && energies[0] > 0.0 && energies[1] > energies[0]) {
        const double ln0 = std::log(energies[0]), delta = std::log(energies[1]) - ln0;
        bool ok = delta > 0.0;
        for (int k = 0; ok && k <= G - 1; k++)
            ok = energies[k] > 0.0 && std::fabs(std::log(energies[k]) - (ln0 + k * delta)) < 0.25 * delta;
        if (ok) {
            t.group_hint_ln0 = (float)ln0;
            t.group_hint_scale = (float)(1.0 / delta);
        }
    }
    t.macro_xs = h->macro_xs.ptr;
    t.class_num_reactions = h->class_num_reactions.ptr;
    t.class_material = h->class_material.ptr;
    t.class_reaction_type = h->class_type.ptr;
    t.class_reaction_nubar = h->class_nubar.ptr;
    t.material_inv_mass = h->material_mass.ptr;
    t.cell_class = h->cell_class.ptr;
    t.cell_nodes = h->cell_nodes.ptr;
    t.cell_center = h->cell_center.ptr;
    t.planes = h->planes.ptr;
    t.adj_cell = h->adj_cell.ptr;
    t.adj_facet_event = h->adj_facet_event.ptr;
    t.time_step = p->time_step;

    // FP32 screening tables in cell-local coordinates (origin: the cell's
    // MCT_Cell_Position_3D_G centre), and the projection of each facet's FP64
    // inside test (MCT.cc:331-385: C, then B, then A dominant).
    std::vector<float4> face32((size_t)C * 6);
    std::vector<float2> face_slack((size_t)C);
    std::vector<float> node32((size_t)C * kCellPoints * 3);
    std::vector<uint8_t> proj((size_t)C * kFacets);
    double lmax = 0.0, dmax = 0.0;
    for (int64_t c = 0; c < C; c++) {
        const double cx = center[c * 3 + 0], cy = center[c * 3 + 1], cz = center[c * 3 + 2];
        for (int k = 0; k < kCellPoints; k++) {
            const double* nd = &nodes[(c * kCellPoints + k) * 3];
            node32[(c * kCellPoints + k) * 3 + 0] = (float)(nd[0] - cx);
            node32[(c * kCellPoints + k) * 3 + 1] = (float)(nd[1] - cy);
            node32[(c * kCellPoints + k) * 3 + 2] = (float)(nd[2] - cz);
            lmax = std::max(lmax, fabs(nd[0]) + fabs(nd[1]) + fabs(nd[2]));
        }
        double sn = 0.0, sd = 0.0;
        for (int f = 0; f < kFacets; f++) {
            const double* pl = &planes[(c * kFacets + f) * 4];
            const double A = pl[0], B = pl[1], Cc = pl[2], D = pl[3];
            const double dl = D + A * cx + B * cy + Cc * cz;
            // the face's plane is its first facet's; the others' differences
            // from it go into the face slack
            const double* rep = &planes[(c * kFacets + (f & ~3)) * 4];
            const double dlr = rep[3] + rep[0] * cx + rep[1] * cy + rep[2] * cz;
            if ((f & 3) == 0) face32[c * 6 + f / 4] = make_float4((float)A, (float)B, (float)Cc, (float)dl);
            sn = std::max(sn, fabs(A - rep[0]) + fabs(B - rep[1]) + fabs(Cc - rep[2]));
            sd = std::max(sd, fabs(dl - dlr));
            dmax = std::max(dmax, fabs(D));
            uint8_t pr;
            if (Cc < -0.5 || Cc > 0.5) pr = 0 | (1 << 2);
            else if (B < -0.5 || B > 0.5) pr = 2 | (0 << 2);
            else if (A < -0.5 || A > 0.5) pr = 1 | (2 << 2);
            else pr = 0xff;
            proj[c * kFacets + f] = pr;
        }
        // twice the largest difference, rounded up to float (and above the
        // FP64 rounding of the differences themselves)
        face_slack[c] = make_float2((float)(2.0 * sn * (1.0 + 1e-6)) + 1e-30f, (float)(2.0 * sd * (1.0 + 1e-6)) + 1e-30f);
    }
    if ((st = h->face32.upload(face32)) || (st = h->face_slack.upload(face_slack)) || (st = h->node32.upload(node32)) ||
        (st = h->proj.upload(proj)))
        return st;
    t.face32 = h->face32.ptr;
    t.face_slack = h->face_slack.ptr;
    t.node32 = h->node32.ptr;
    t.proj = h->proj.ptr;
    // FP64 rounding of quantities formed from global coordinates (numerator,
    // intersection point, the shifted plane offset) stays below a few units of
    // 2^-53 times these magnitudes; 16x that is the screen's absolute slack
    t.abs_slack = 16.0 * 1.1102230246251565e-16 * (4.0 * lmax + 2.0 * dmax) + 1e-30;
    return QSG_OK;
}

}  // namespace

int check_soa(const QsgParticleSoA* s)
{
    if (!s || !s->x || !s->y || !s->z || !s->vx || !s->vy || !s->vz || !s->kinetic_energy || !s->weight ||
        !s->time_to_census || !s->age || !s->num_mean_free_paths || !s->num_segments || !s->random_number_seed ||
        !s->identifier || !s->last_event || !s->num_collisions || !s->breed || !s->species || !s->domain || !s->cell)
        return fail(QSG_ERR_INVALID, "particle SoA has a null field");
    return QSG_OK;
}

int copy_soa(const DevStore& d, const QsgParticleSoA* h, uint64_t n, bool to_device)
{
    if (n == 0) return QSG_OK;
    // the 20 field copies are issued back to back on the legacy stream and
    // waited for once (they overlap when the host arrays are pinned)
    cudaMemcpyKind kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    void* dev[20] = {d.x, d.y, d.z, d.vx, d.vy, d.vz, d.kinetic_energy, d.weight, d.time_to_census, d.age,
                     d.num_mean_free_paths, d.num_segments, d.seed, d.identifier, d.last_event, d.num_collisions,
                     d.breed, d.species, d.domain, d.cell};
    void* host[20] = {h->x, h->y, h->z, h->vx, h->vy, h->vz, h->kinetic_energy, h->weight, h->time_to_census,
                      h->age, h->num_mean_free_paths, h->num_segments, h->random_number_seed, h->identifier,
                      h->last_event, h->num_collisions, h->breed, h->species, h->domain, h->cell};
    for (int k = 0; k < 20; k++) {
        const size_t bytes = n * (k < 14 ? 8 : 4);
        QSG_CUDA(to_device ? cudaMemcpyAsync(dev[k], host[k], bytes, kind, 0)
                           : cudaMemcpyAsync(host[k], dev[k], bytes, kind, 0));
    }
    QSG_CUDA(cudaStreamSynchronize(0));
    return QSG_OK;
}

namespace {

// The tracking kernel the handle selects (qsg_set_track_kernel, block size,
// sensitivities when `sens` and enabled) over explicit stores, tallies and
// work cursor.
int launch_track_kernel(QsgHandle* h, cudaStream_t s, const DevTally& tv, unsigned long long* cursor,
                        const PassStores& ps, bool sens)
{
    if (h->kernel_kind == 1 && pool_kernel_usable(h)) {
        if (h->block_size == 256) launch_pool<256>(h, s, tv, cursor, ps, sens);
        else launch_pool<128>(h, s, tv, cursor, ps, sens);
    } else if (sens && h->sens.K > 0) {
        const size_t smem = track_smem_bytes_sens(h);
        if (h->block_size == 256)
            track_kernel<256, true><<<h->sens_track_blocks, 256, smem, s>>>(h->tables, tv, ps.in, ps.census,
                                                                            ps.extra, cursor, h->sens);
        else
            track_kernel<128, true><<<h->sens_track_blocks, 128, smem, s>>>(h->tables, tv, ps.in, ps.census,
                                                                            ps.extra, cursor, h->sens);
    } else {
        const size_t smem = track_smem_bytes(h);
        if (h->block_size == 256)
            track_kernel<256, false><<<h->track_blocks, 256, smem, s>>>(h->tables, tv, ps.in, ps.census, ps.extra,
                                                                        cursor, DevSens{});
        else
            track_kernel<128, false><<<h->track_blocks, 128, smem, s>>>(h->tables, tv, ps.in, ps.census, ps.extra,
                                                                        cursor, DevSens{});
    }
    QSG_CUDA(cudaGetLastError());
    return QSG_OK;
}

// One tracking pass over explicit stores: input -> census + fission
// products.  The pass's particle count is read by the kernel from the input's
// device counter, so nothing here waits for the device.
int launch_pass_stores(QsgHandle* h, cudaStream_t s, const PassStores& ps)
{
    unsigned long long* cursor = &h->scalars.ptr->cursor;
    QSG_CUDA(cudaMemsetAsync(ps.extra.count, 0, sizeof(unsigned long long), s));
    QSG_CUDA(cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), s));
    return launch_track_kernel(h, s, tally_view(h), cursor, ps, true);
}

// One tracking pass over the handle's stores: processing -> processed +
// extra; the extra store then becomes the next pass's input.
int launch_pass(QsgHandle* h, cudaStream_t s)
{
    const int st = launch_pass_stores(h, s, PassStores{h->processing.view, h->processed.view, h->extra.view});
    if (st) return st;
    std::swap(h->processing, h->extra);
    return QSG_OK;
}

__global__ void leftover_check_kernel(const unsigned long long* count, unsigned int* flags)
{
    if (*count != 0) atomicOr(flags, QSG_DEV_PASS_LIMIT);
}

}  // namespace

// Asynchronous cycle: a fixed number of passes, no host synchronisation.
// Stores must already hold enough capacity (qsg_configure_cycle sizes them);
// overflow and leftover fission products raise device flags.
int track_passes_async(QsgHandle* h, cudaStream_t s)
{
    int st;
    for (int pass = 0; pass < h->max_passes; pass++)
        if ((st = launch_pass(h, s))) return st;
    leftover_check_kernel<<<1, 1, 0, s>>>(h->processing.count, h->flags.ptr);
    QSG_CUDA(cudaGetLastError());
    h->n_processing = 0;
    return QSG_OK;
}

// Synchronous cycle: passes until no fission products are left, growing the
// stores between passes from the counts read back after each pass.
int track_passes_sync(QsgHandle* h, cudaStream_t s)
{
    int st;
    unsigned long long counts[2];
    for (;;) {
        QSG_CUDA(cudaMemcpyAsync(&counts[0], h->processing.count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        QSG_CUDA(cudaMemcpyAsync(&counts[1], h->processed.count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        QSG_CUDA(cudaStreamSynchronize(s));
        const uint64_t n = counts[0];
        if (n == 0) break;
        if ((st = h->processed.reserve(counts[1] + n))) return st;
        if ((st = h->extra.reserve(4 * n))) return st;
        if ((st = launch_pass(h, s))) return st;
    }
    h->n_processing = 0;
    h->known_census = counts[1];
    return QSG_OK;
}

}  // namespace qsg

using namespace qsg;

extern "C" int qsg_problem_check(const QsgProblem* problem)
{
    QSG_API_BEGIN
    if (!problem) return fail(QSG_ERR_INVALID, "qsg_problem_check: null problem");
    return validate_problem(problem);
    QSG_API_END
}

extern "C" int qsg_device_count(int* count)
{
    if (!count) return fail(QSG_ERR_INVALID, "qsg_device_count: null argument");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return QSG_OK;
}

namespace {

// Shared by qsg_create (one problem) and qsg_batch_create (the union of
// several; `uni` holds the per-problem cell ranges).
int create_impl(const QsgProblem* problem, const QsgOptions* options, const UnionProblem* uni, int n_problems,
                QsgHandle** out)
{
    *out = nullptr;
    int st = validate_problem(problem);
    if (st) return st;
    int ndev = 0;
    qsg_device_count(&ndev);
    if (ndev == 0) return fail(QSG_ERR_NO_DEVICE, "qsg_create: no CUDA device visible");
    QsgHandle* h = new QsgHandle();
    if (options) {
        h->device = options->device;
        if (options->flux_replicas > 0) h->flux_replicas = options->flux_replicas;
        if (options->balance_replicas > 0) h->balance_replicas = options->balance_replicas;
        if (options->max_segments > 0) h->max_segments = options->max_segments;
        if (options->max_passes > 0) h->max_passes = options->max_passes;
        if (options->block_size == 128 || options->block_size == 256) h->block_size = options->block_size;
        if (options->collision_batch > 0) h->collision_batch = std::min<int>(options->collision_batch, 32);
    }
    h->num_cells = problem->num_cells;
    h->num_groups = problem->num_groups;
    h->num_problems = n_problems;
    if (uni) {
        h->h_problem_cell_offset = uni->problem_cell_offset;
        h->h_problem_material_offset = uni->problem_material_offset;
    } else {
        h->h_problem_cell_offset = {0, problem->num_cells};
        h->h_problem_material_offset = {0, problem->num_materials};
    }
    auto cleanup = [&](int code) {
        qsg_destroy(h);
        return code;
    };
    if ((st = set_device(h))) return cleanup(st);
    if ((st = upload_tables(h, problem))) return cleanup(st);
    if (uni && (st = h->cell_problem.upload(uni->cell_problem))) return cleanup(st);
    {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess)
            return cleanup(fail(QSG_ERR_CUDA, "cudaGetDeviceProperties failed"));
        h->num_sms = prop.multiProcessorCount;
        if ((st = configure_track_grid(h))) return cleanup(st);
    }
    h->num_materials = problem->num_materials;
    if (problem->cell_volume) h->h_cell_volume.assign(problem->cell_volume, problem->cell_volume + problem->num_cells);
    if (problem->cell_id) h->h_cell_id.assign(problem->cell_id, problem->cell_id + problem->num_cells);
    h->h_cell_material.assign(problem->cell_material, problem->cell_material + problem->num_cells);
    if ((st = h->scalars.alloc(1))) return cleanup(st);
    if (cudaMemset(h->scalars.ptr, 0, sizeof(CycleScalars)) != cudaSuccess)
        return cleanup(fail(QSG_ERR_CUDA, "qsg_create: memset failed"));
    if ((st = h->flux.alloc((size_t)h->flux_replicas * h->num_cells * h->num_groups))) return cleanup(st);
    if ((st = h->balance.alloc((size_t)h->balance_replicas * h->num_problems * QSG_BAL_COUNT))) return cleanup(st);
    if ((st = h->flags.alloc(1))) return cleanup(st);
    if (cudaMemset(h->flux.ptr, 0, h->flux.n * sizeof(double)) != cudaSuccess ||
        cudaMemset(h->balance.ptr, 0, h->balance.n * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(h->flags.ptr, 0, sizeof(unsigned int)) != cudaSuccess)
        return cleanup(fail(QSG_ERR_CUDA, "qsg_create: memset failed"));
    uint64_t cap = options && options->particle_capacity ? options->particle_capacity : 1024;
    if ((st = h->processing.reserve(cap)) || (st = h->processed.reserve(cap)) || (st = h->extra.reserve(cap)))
        return cleanup(st);
    *out = h;
    return QSG_OK;
}

}  // namespace

extern "C" int qsg_create(const QsgProblem* problem, const QsgOptions* options, QsgHandle** out)
{
    QSG_API_BEGIN
    if (!problem || !out) return fail(QSG_ERR_INVALID, "qsg_create: null argument");
    return create_impl(problem, options, nullptr, 1, out);
    QSG_API_END
}

extern "C" int qsg_batch_create(const QsgProblem* problems, int32_t n_problems, const QsgOptions* options,
                                QsgHandle** out)
{
    QSG_API_BEGIN
    if (!problems || !out || n_problems < 1) return fail(QSG_ERR_INVALID, "qsg_batch_create: bad argument");
    *out = nullptr;
    UnionProblem u;
    build_union(problems, n_problems, u);
    return create_impl(&u.view, options, &u, n_problems, out);
    QSG_API_END
}

extern "C" int qsg_num_problems(QsgHandle* h, int32_t* n, int32_t* cell_offsets)
{
    if (!h || !n) return fail(QSG_ERR_INVALID, "qsg_num_problems: null argument");
    *n = h->num_problems;
    if (cell_offsets)
        for (int k = 0; k <= h->num_problems; k++) cell_offsets[k] = h->h_problem_cell_offset[k];
    return QSG_OK;
}

extern "C" int qsg_set_pool_tuning(QsgHandle* h, int32_t collision_step, int32_t refill)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_set_pool_tuning: null handle");
    if (collision_step < 0 || collision_step > 32 || refill < 0 || refill > 64)
        return fail(QSG_ERR_INVALID, "qsg_set_pool_tuning: collision step 1-32 and refill 1-64 (0 keeps a value)");
    if (collision_step) h->pool_collision_step = collision_step;
    if (refill) h->pool_refill = refill;
    h->clear_graphs();   // captured launches carry the old values
    return QSG_OK;
}

extern "C" int qsg_set_tuning(QsgHandle* h, int32_t block_size, int32_t collision_batch, int32_t queue_chunk)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_set_tuning: null handle");
    if (block_size != 0 && block_size != 128 && block_size != 256)
        return fail(QSG_ERR_INVALID, "qsg_set_tuning: block size must be 128 or 256");
    int st = set_device(h);
    if (st) return st;
    if (block_size) h->block_size = block_size;
    if (collision_batch > 0) h->collision_batch = std::min<int>(collision_batch, 32);
    if (queue_chunk > 0) h->queue_chunk = std::min<int>(queue_chunk, 1024);
    h->clear_graphs();   // captured launches carry the old shape
    return configure_track_grid(h);
}

extern "C" int qsg_set_track_kernel(QsgHandle* h, int32_t kind)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_set_track_kernel: null handle");
    if (kind != 0 && kind != 1) return fail(QSG_ERR_INVALID, "qsg_set_track_kernel: kind must be 0 or 1");
    h->kernel_kind = kind;
    h->clear_graphs();   // captured launches carry the old kernel
    return QSG_OK;
}

extern "C" int qsg_destroy(QsgHandle* h)
{
    if (!h) return QSG_OK;
    cudaSetDevice(h->device);
    h->energies.free(); h->sigma_total.free(); h->mfp_table.free(); h->inv_mfp_table.free(); h->cell_tally.free(); h->macro_xs.free(); h->class_nubar.free();
    h->material_mass.free(); h->cell_nodes.free(); h->cell_center.free(); h->planes.free();
    h->class_num_reactions.free(); h->class_material.free(); h->cell_class.free(); h->adj_cell.free();
    h->class_type.free(); h->adj_facet_event.free();
    h->face32.free(); h->face_slack.free(); h->node32.free(); h->proj.free();
    h->flux.free(); h->balance.free(); h->flags.free(); h->flux_partial.free();
    h->cell_volume.free(); h->cell_id.free(); h->src_cell.free(); h->src_cell_count.free();
    h->src_cell_offset.free(); h->scalars.free(); h->history.free();
    h->cell_problem.free(); h->prob_weight.free(); h->prob_emin.free(); h->prob_emax.free(); h->prob_lowcut.free();
    h->prob_factor.free(); h->prob_target.free(); h->prob_nsource.free(); h->prob_seed_offset.free();
    h->prob_load_balance.free(); h->prob_cell_offset.free(); h->prob_carry.free();
    h->sens_param.free(); h->sens_dsig.free(); h->sens_inv_theta.free(); h->sens_flux_cell.free();
    h->sens_dflux.free(); h->sens_leak.free(); h->sens_dleak.free();
    h->fluence.free(); h->spectrum.free();
    h->clear_graphs();
    if (h->capture_stream) cudaStreamDestroy(h->capture_stream);
    h->processing.release(); h->processed.release(); h->extra.release();
    delete h;
    return QSG_OK;
}

extern "C" int qsg_set_particles(QsgHandle* h, const QsgParticleSoA* host, uint64_t n)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_set_particles: null handle");
    int st = check_soa(host);
    if (st && n) return st;
    if ((st = set_device(h))) return st;
    if ((st = h->processing.reserve(n))) return st;
    if ((st = copy_soa(h->processing.view, host, n, true))) return st;
    if (h->processing.view.score)   // particles from the host start with zero sensitivity scores
        QSG_CUDA(cudaMemset(h->processing.view.score, 0,
                            (size_t)h->processing.view.score_fields * h->processing.capacity * sizeof(double)));
    unsigned long long nn = n;
    QSG_CUDA(cudaMemcpy(h->processing.count, &nn, sizeof(nn), cudaMemcpyHostToDevice));
    QSG_CUDA(cudaMemset(h->processed.count, 0, sizeof(unsigned long long)));
    h->n_processing = n;
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_begin_cycle_from_census(QsgHandle* h, uint64_t* n)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_begin_cycle_from_census: null handle");
    int st = set_device(h);
    if (st) return st;
    unsigned long long c = 0;
    QSG_CUDA(cudaMemcpy(&c, h->processed.count, sizeof(c), cudaMemcpyDeviceToHost));
    std::swap(h->processing, h->processed);
    QSG_CUDA(cudaMemset(h->processed.count, 0, sizeof(unsigned long long)));
    h->n_processing = c;
    if (n) *n = c;
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_sizes(QsgHandle* h, uint64_t* processing, uint64_t* processed)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_sizes: null handle");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    unsigned long long c = 0, p = 0;
    QSG_CUDA(cudaMemcpy(&c, h->processed.count, sizeof(c), cudaMemcpyDeviceToHost));
    QSG_CUDA(cudaMemcpy(&p, h->processing.count, sizeof(p), cudaMemcpyDeviceToHost));
    if (processing) *processing = p;
    if (processed) *processed = c;
    return QSG_OK;
}

extern "C" int qsg_get_census(QsgHandle* h, QsgParticleSoA* host, uint64_t cap, uint64_t* n_out)
{
    QSG_API_BEGIN
    if (!h || !n_out) return fail(QSG_ERR_INVALID, "qsg_get_census: null argument");
    int st = set_device(h);
    if (st) return st;
    unsigned long long c = 0;
    QSG_CUDA(cudaMemcpy(&c, h->processed.count, sizeof(c), cudaMemcpyDeviceToHost));
    *n_out = c;
    if (c > cap) return fail(QSG_ERR_CAPACITY, "qsg_get_census: %llu particles, capacity %llu", c,
                             (unsigned long long)cap);
    if (c > h->processed.capacity)
        return fail(QSG_ERR_DEVICE, "qsg_get_census: store overflowed (%llu > %llu)", c,
                    (unsigned long long)h->processed.capacity);
    if (c == 0) return QSG_OK;
    if ((st = check_soa(host))) return st;
    return copy_soa(h->processed.view, host, c, false);
    QSG_API_END
}

namespace {

// Whether any field array of `a` (n particles) overlaps any of `b` (m particles).
bool soa_ranges_overlap(const QsgParticleSoA* a, uint64_t n, const QsgParticleSoA* b, uint64_t m)
{
    const void* fa[20] = {a->x, a->y, a->z, a->vx, a->vy, a->vz, a->kinetic_energy, a->weight, a->time_to_census,
                          a->age, a->num_mean_free_paths, a->num_segments, a->random_number_seed, a->identifier,
                          a->last_event, a->num_collisions, a->breed, a->species, a->domain, a->cell};
    const void* fb[20] = {b->x, b->y, b->z, b->vx, b->vy, b->vz, b->kinetic_energy, b->weight, b->time_to_census,
                          b->age, b->num_mean_free_paths, b->num_segments, b->random_number_seed, b->identifier,
                          b->last_event, b->num_collisions, b->breed, b->species, b->domain, b->cell};
    for (int i = 0; i < 20; i++) {
        const uintptr_t a0 = (uintptr_t)fa[i], a1 = a0 + n * (i < 14 ? 8 : 4);
        for (int j = 0; j < 20; j++) {
            const uintptr_t b0 = (uintptr_t)fb[j], b1 = b0 + m * (j < 14 ? 8 : 4);
            if (a0 < b1 && b0 < a1) return true;
        }
    }
    return false;
}

bool ranges_overlap(const void* a, uint64_t a_bytes, const void* b, uint64_t b_bytes)
{
    const uintptr_t a0 = (uintptr_t)a, b0 = (uintptr_t)b;
    return a0 < b0 + b_bytes && b0 < a0 + a_bytes;
}

// Whether any field array of `a` (n particles) overlaps [p, p + bytes).
bool soa_overlaps_range(const QsgParticleSoA* a, uint64_t n, const void* p, uint64_t bytes)
{
    const void* fa[20] = {a->x, a->y, a->z, a->vx, a->vy, a->vz, a->kinetic_energy, a->weight, a->time_to_census,
                          a->age, a->num_mean_free_paths, a->num_segments, a->random_number_seed, a->identifier,
                          a->last_event, a->num_collisions, a->breed, a->species, a->domain, a->cell};
    for (int i = 0; i < 20; i++)
        if (ranges_overlap(fa[i], n * (i < 14 ? 8 : 4), p, bytes)) return true;
    return false;
}

// Device view of a caller's particle arrays for qsg_track_host: each field
// must be page-locked host memory (cudaHostAlloc / cudaHostRegister, which the
// GPU reads and writes over the host link) or device memory.
int device_soa_view(const QsgParticleSoA* soa, const char* what, DevStore& v)
{
    void* fields[20] = {soa->x, soa->y, soa->z, soa->vx, soa->vy, soa->vz, soa->kinetic_energy, soa->weight,
                        soa->time_to_census, soa->age, soa->num_mean_free_paths, soa->num_segments,
                        soa->random_number_seed, soa->identifier, soa->last_event, soa->num_collisions, soa->breed,
                        soa->species, soa->domain, soa->cell};
    void* dev[20];
    for (int k = 0; k < 20; k++) {
        cudaPointerAttributes a{};
        QSG_CUDA(cudaPointerGetAttributes(&a, fields[k]));
        if (a.type == cudaMemoryTypeHost && a.devicePointer) dev[k] = a.devicePointer;
        else if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) dev[k] = fields[k];
        else
            return fail(QSG_ERR_INVALID, "qsg_track_host: %s field %d is pageable host memory; page-lock it "
                        "(cudaHostAlloc / cudaHostRegister) or use qsg_set_particles", what, k);
    }
    v = DevStore{};
    v.x = (double*)dev[0]; v.y = (double*)dev[1]; v.z = (double*)dev[2];
    v.vx = (double*)dev[3]; v.vy = (double*)dev[4]; v.vz = (double*)dev[5];
    v.kinetic_energy = (double*)dev[6]; v.weight = (double*)dev[7]; v.time_to_census = (double*)dev[8];
    v.age = (double*)dev[9]; v.num_mean_free_paths = (double*)dev[10]; v.num_segments = (double*)dev[11];
    v.seed = (uint64_t*)dev[12]; v.identifier = (uint64_t*)dev[13];
    v.last_event = (int32_t*)dev[14]; v.num_collisions = (int32_t*)dev[15]; v.breed = (int32_t*)dev[16];
    v.species = (int32_t*)dev[17]; v.domain = (int32_t*)dev[18]; v.cell = (int32_t*)dev[19];
    return QSG_OK;
}

}  // namespace

extern "C" int qsg_track_host(QsgHandle* h, const QsgParticleSoA* particles, uint64_t n, QsgParticleSoA* census,
                              uint64_t census_capacity, uint64_t* n_census, void* stream)
{
    QSG_API_BEGIN
    QSG_RANGE("cycleTracking_TrackingKernel");
    if (!h || !n_census) return fail(QSG_ERR_INVALID, "qsg_track_host: null argument");
    *n_census = 0;
    if (h->sens.K > 0)
        return fail(QSG_ERR_UNSUPPORTED, "qsg_track_host: sensitivity scores do not travel through host arrays; "
                    "use qsg_set_particles / qsg_track_cycle");
    if (n == 0) return QSG_OK;
    int st;
    if ((st = check_soa(particles)) || (st = check_soa(census))) return st;
    if (soa_ranges_overlap(particles, n, census, census_capacity))
        return fail(QSG_ERR_INVALID, "qsg_track_host: the census arrays overlap the particle arrays");
    if ((st = set_device(h))) return st;
    PassStores ps;
    if ((st = device_soa_view(particles, "particles", ps.in)) || (st = device_soa_view(census, "census", ps.census)))
        return st;
    ps.in.count = &h->scalars.ptr->host_in_count;
    ps.in.capacity = n;
    ps.census.count = &h->scalars.ptr->host_census_count;
    ps.census.capacity = census_capacity;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned long long nn = n;
    QSG_CUDA(cudaMemcpyAsync(ps.in.count, &nn, sizeof(nn), cudaMemcpyHostToDevice, s));
    QSG_CUDA(cudaMemsetAsync(ps.census.count, 0, sizeof(unsigned long long), s));
    // pass 0 reads the caller's arrays; fission products go to the handle's
    // stores, which later passes read; every pass appends census particles
    // to the caller's arrays
    if ((st = h->extra.reserve(4 * n))) return st;
    ps.extra = h->extra.view;
    if ((st = launch_pass_stores(h, s, ps))) return st;
    unsigned long long counts[2] = {0, 0};
    for (int pass = 1;; pass++) {
        QSG_CUDA(cudaMemcpyAsync(&counts[0], h->extra.count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        QSG_CUDA(cudaMemcpyAsync(&counts[1], ps.census.count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        QSG_CUDA(cudaStreamSynchronize(s));
        if (counts[0] == 0) break;
        if (counts[0] > h->extra.capacity)
            return fail(QSG_ERR_CAPACITY, "qsg_track_host: pass %d made %llu fission products, more than the "
                        "%llu the product store holds", pass - 1, counts[0], (unsigned long long)h->extra.capacity);
        std::swap(h->processing, h->extra);   // this pass's input: the products
        if ((st = h->extra.reserve(4 * counts[0]))) return st;
        ps.in = h->processing.view;
        ps.extra = h->extra.view;
        if ((st = launch_pass_stores(h, s, ps))) return st;
    }
    QSG_CUDA(cudaMemsetAsync(h->processing.count, 0, sizeof(unsigned long long), s));
    QSG_CUDA(cudaStreamSynchronize(s));
    h->n_processing = 0;
    *n_census = counts[1];
    if (counts[1] > census_capacity)
        return fail(QSG_ERR_CAPACITY, "qsg_track_host: %llu census particles exceed census_capacity %llu -- the "
                    "census arrays hold the first %llu", counts[1], (unsigned long long)census_capacity,
                    (unsigned long long)census_capacity);
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_track_cycle(QsgHandle* h, void* stream)
{
    QSG_API_BEGIN
    QSG_RANGE("cycleTracking_TrackingKernel");
    if (!h) return fail(QSG_ERR_INVALID, "qsg_track_cycle: null handle");
    int st = set_device(h);
    if (st) return st;
    return track_passes_sync(h, static_cast<cudaStream_t>(stream));
    QSG_API_END
}

extern "C" int qsg_track_cycle_async(QsgHandle* h, void* stream)
{
    QSG_API_BEGIN
    QSG_RANGE("cycleTracking_TrackingKernel");
    if (!h) return fail(QSG_ERR_INVALID, "qsg_track_cycle_async: null handle");
    int st = set_device(h);
    if (st) return st;
    return track_passes_async(h, static_cast<cudaStream_t>(stream));
    QSG_API_END
}

extern "C" int qsg_track_cycle_sync(QsgHandle* h)
{
    QSG_API_BEGIN
    QSG_RANGE("cycleTracking_TrackingKernel");
    if (!h) return fail(QSG_ERR_INVALID, "qsg_track_cycle_sync: null handle");
    int st = set_device(h);
    if (st) return st;
    if ((st = track_passes_sync(h, nullptr))) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    unsigned int flags = 0;
    QSG_CUDA(cudaMemcpy(&flags, h->flags.ptr, sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags) return fail(QSG_ERR_DEVICE, "tracking kernel raised device flags 0x%x", flags);
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_read_tallies(QsgHandle* h, uint64_t* balance, double* flux)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_read_tallies: null handle");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    if (balance) {
        std::vector<unsigned long long> b(h->balance.n);
        QSG_CUDA(cudaMemcpy(b.data(), h->balance.ptr, b.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        for (int k = 0; k < QSG_BAL_COUNT; k++) {
            uint64_t s = 0;
            for (int r = 0; r < h->balance_replicas * h->num_problems; r++) s += b[(size_t)r * QSG_BAL_COUNT + k];
            balance[k] = s;
        }
    }
    if (flux) {
        const size_t cg_n = (size_t)h->num_cells * h->num_groups;
        QSG_CUDA(cudaMemcpy(flux, h->flux.ptr, cg_n * sizeof(double), cudaMemcpyDeviceToHost));
        if (h->flux_replicas > 1) {
            std::vector<double> tmp(cg_n);
            for (int r = 1; r < h->flux_replicas; r++) {
                QSG_CUDA(cudaMemcpy(tmp.data(), h->flux.ptr + r * cg_n, cg_n * sizeof(double), cudaMemcpyDeviceToHost));
                for (size_t i = 0; i < cg_n; i++) flux[i] += tmp[i];
            }
        }
    }
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_reset_tallies(QsgHandle* h)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_reset_tallies: null handle");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaMemset(h->flux.ptr, 0, h->flux.n * sizeof(double)));
    QSG_CUDA(cudaMemset(h->balance.ptr, 0, h->balance.n * sizeof(unsigned long long)));
    if (h->cell_tally.ptr) QSG_CUDA(cudaMemset(h->cell_tally.ptr, 0, h->cell_tally.n * sizeof(double)));
    return QSG_OK;
}

extern "C" int qsg_set_exponential_tally(QsgHandle* h, int32_t enabled)
{
    QSG_API_BEGIN
    if (!h) return fail(QSG_ERR_INVALID, "qsg_set_exponential_tally: null handle");
    if (enabled != 0 && enabled != 1) return fail(QSG_ERR_INVALID, "qsg_set_exponential_tally: enabled must be 0 or 1");
    int st = set_device(h);
    if (st) return st;
    if (enabled && !h->cell_tally.ptr) {
        if ((st = h->cell_tally.alloc((size_t)h->num_cells))) return st;
        QSG_CUDA(cudaMemset(h->cell_tally.ptr, 0, h->cell_tally.n * sizeof(double)));
    }
    h->exp_tally = enabled != 0;
    h->clear_graphs();   // captured launches carry the old tally view
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_read_cell_tally(QsgHandle* h, double* cell_tally)
{
    QSG_API_BEGIN
    if (!h || !cell_tally) return fail(QSG_ERR_INVALID, "qsg_read_cell_tally: null argument");
    if (!h->exp_tally) return fail(QSG_ERR_INVALID, "qsg_read_cell_tally: the exponential tally is off");
    int st = set_device(h);
    if (st) return st;
    QSG_CUDA(cudaDeviceSynchronize());
    QSG_CUDA(cudaMemcpy(cell_tally, h->cell_tally.ptr, h->cell_tally.n * sizeof(double), cudaMemcpyDeviceToHost));
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_device_status(QsgHandle* h, uint32_t* flags, int clear)
{
    if (!h || !flags) return fail(QSG_ERR_INVALID, "qsg_device_status: null argument");
    int st = set_device(h);
    if (st) return st;
    unsigned int f = 0;
    QSG_CUDA(cudaMemcpy(&f, h->flags.ptr, sizeof(f), cudaMemcpyDeviceToHost));
    *flags = f;
    if (clear) QSG_CUDA(cudaMemset(h->flags.ptr, 0, sizeof(unsigned int)));
    return QSG_OK;
}

static void fill_view(const DevStore& d, QsgParticleSoA* v)
{
    v->x = d.x; v->y = d.y; v->z = d.z; v->vx = d.vx; v->vy = d.vy; v->vz = d.vz;
    v->kinetic_energy = d.kinetic_energy; v->weight = d.weight; v->time_to_census = d.time_to_census;
    v->age = d.age; v->num_mean_free_paths = d.num_mean_free_paths; v->num_segments = d.num_segments;
    v->random_number_seed = d.seed; v->identifier = d.identifier; v->last_event = d.last_event;
    v->num_collisions = d.num_collisions; v->breed = d.breed; v->species = d.species; v->domain = d.domain;
    v->cell = d.cell;
}

extern "C" int qsg_processing_view(QsgHandle* h, QsgParticleSoA* v, uint64_t* n)
{
    if (!h || !v || !n) return fail(QSG_ERR_INVALID, "qsg_processing_view: null argument");
    fill_view(h->processing.view, v);
    *n = h->n_processing;
    return QSG_OK;
}

extern "C" int qsg_processed_view(QsgHandle* h, QsgParticleSoA* v, uint64_t* n)
{
    if (!h || !v || !n) return fail(QSG_ERR_INVALID, "qsg_processed_view: null argument");
    int st = set_device(h);
    if (st) return st;
    unsigned long long c = 0;
    QSG_CUDA(cudaMemcpy(&c, h->processed.count, sizeof(c), cudaMemcpyDeviceToHost));
    fill_view(h->processed.view, v);
    *n = c;
    return QSG_OK;
}

// ------------------------------------------------------------------------
// Tracking without allocation (qsg_track_particles_noalloc).
//
// Callers whose device memory all belongs to a pool allocator (PyTorch's
// caching allocator, an application arena) cannot have this library call
// cudaMalloc or cudaFree while they run: the allocation may fail or escape the
// pool's accounting, and cudaFree synchronises the whole device.  For them
// the fission products that one tracking pass hands to the next live in the
// fixed array below instead of the handle's growable stores.  Layout: a
// 256-byte header of 64-bit words (0: work cursor, 1: input count, 2: census
// count, 3: device error flags) and two particle stores of
// QSG_NOALLOC_MAX_PRODUCTS particles each, carved like the handle's stores.
// The array is shared by every call on a device and keeps what the last call
// left in it; each call clears the header and the store counts first.

namespace qsg {
namespace {

constexpr size_t noalloc_field_bytes(size_t esz)
{
    return ((size_t)QSG_NOALLOC_MAX_PRODUCTS * esz + 255) & ~size_t(255);
}
constexpr size_t kNoallocHeaderBytes = 256;
// per store: its count word (256 bytes), 14 eight-byte and 6 four-byte fields
constexpr size_t kNoallocStoreBytes = 256 + 14 * noalloc_field_bytes(8) + 6 * noalloc_field_bytes(4);
static_assert(kNoallocHeaderBytes + 2 * kNoallocStoreBytes == QSG_NOALLOC_SCRATCH_BYTES,
              "QSG_NOALLOC_SCRATCH_BYTES does not match the scratch layout");

}  // namespace

}  // namespace qsg

// The scratch itself.  In host code this name only stands in for the symbol;
// its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char qsg_noalloc_scratch[QSG_NOALLOC_SCRATCH_BYTES];

namespace qsg {
namespace {

// Device address of the scratch in the current context (device `device`
// current).  The lookup (cudaGetSymbolAddress) runs once per CUDA context and
// is cached under the context's unique id, so a context that replaces one
// destroyed by cudaDeviceReset -- which reloads this library's device code at
// a new address -- gets a fresh lookup.  Where the driver cannot name the
// context, every call looks the address up (no allocation either way once the
// device code is loaded).
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);

std::mutex g_noalloc_mutex;
std::map<unsigned long long, unsigned char*> g_noalloc_address;   // context id -> address

bool current_context_id(unsigned long long* id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        looked_up = true;
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1{}, q2{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        cudaGetLastError();
    }
    void* ctx = nullptr;
    return get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, id) == 0;
}

int noalloc_scratch_address(int device, unsigned char** out)
{
    unsigned long long ctx_id = 0;
    const bool named = current_context_id(&ctx_id);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (named) {
        auto it = g_noalloc_address.find(ctx_id);
        if (it != g_noalloc_address.end()) {
            *out = it->second;
            return QSG_OK;
        }
    }
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, qsg_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
        return fail(QSG_ERR_CUDA, "qsg_track_particles_noalloc: cudaGetSymbolAddress of the scratch array on "
                    "device %d failed: %s", device, cudaGetErrorString(e));
    if (named) g_noalloc_address[ctx_id] = static_cast<unsigned char*>(ptr);
    *out = static_cast<unsigned char*>(ptr);
    return QSG_OK;
}

// Zero the header and both store counts, then set the input count.
__global__ void noalloc_begin_kernel(unsigned long long* header, unsigned long long* count0,
                                     unsigned long long* count1, unsigned long long n)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int k = 0; k < (int)(kNoallocHeaderBytes / 8); k++) header[k] = 0;
        header[1] = n;
        *count0 = 0;
        *count1 = 0;
    }
}

DevStore noalloc_caller_store(const QsgParticleSoA* s, uint64_t capacity, unsigned long long* count)
{
    DevStore v{};
    v.x = s->x; v.y = s->y; v.z = s->z; v.vx = s->vx; v.vy = s->vy; v.vz = s->vz;
    v.kinetic_energy = s->kinetic_energy; v.weight = s->weight; v.time_to_census = s->time_to_census;
    v.age = s->age; v.num_mean_free_paths = s->num_mean_free_paths; v.num_segments = s->num_segments;
    v.seed = s->random_number_seed; v.identifier = s->identifier;
    v.last_event = s->last_event; v.num_collisions = s->num_collisions; v.breed = s->breed;
    v.species = s->species; v.domain = s->domain; v.cell = s->cell;
    v.count = count;
    v.capacity = capacity;
    return v;
}

// The caller's arrays must be device memory of the handle's device (or
// managed), aligned for their element type.
int noalloc_check_pointer(const void* p, size_t align, int device, const char* what)
{
    if (!p) return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: %s is null", what);
    if (reinterpret_cast<uintptr_t>(p) % align)
        return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: %s is not %zu-byte aligned", what, align);
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: %s is not a CUDA pointer (%s)", what,
                    cudaGetErrorString(e));
    }
    if (a.type == cudaMemoryTypeManaged) return QSG_OK;
    if (a.type != cudaMemoryTypeDevice || a.device != device)
        return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: %s must be device memory on device %d", what,
                    device);
    return QSG_OK;
}

int noalloc_check_soa(const QsgParticleSoA* s, int device, const char* which)
{
    if (!s) return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: %s is null", which);
    const void* p8[14] = {s->x, s->y, s->z, s->vx, s->vy, s->vz, s->kinetic_energy, s->weight,
                          s->time_to_census, s->age, s->num_mean_free_paths, s->num_segments,
                          s->random_number_seed, s->identifier};
    const void* p4[6] = {s->last_event, s->num_collisions, s->breed, s->species, s->domain, s->cell};
    int st;
    for (const void* p : p8)
        if ((st = noalloc_check_pointer(p, 8, device, which))) return st;
    for (const void* p : p4)
        if ((st = noalloc_check_pointer(p, 4, device, which))) return st;
    return QSG_OK;
}

}  // namespace
}  // namespace qsg

extern "C" int qsg_track_particles_noalloc(QsgHandle* h, const QsgParticleSoA* particles, uint64_t n,
                                           QsgParticleSoA* census, uint64_t census_capacity, uint64_t* n_census,
                                           double* flux, uint64_t* balance, void* stream)
{
    QSG_API_BEGIN
    QSG_RANGE("cycleTracking_TrackingKernel");
    if (!h || !n_census) return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: null handle or n_census");
    *n_census = 0;
    if (n == 0) return QSG_OK;
    int st = set_device(h);
    if (st) return st;
    if ((st = noalloc_check_soa(particles, h->device, "particles")) ||
        (st = noalloc_check_soa(census, h->device, "census")) ||
        (st = noalloc_check_pointer(flux, 8, h->device, "flux")) ||
        (st = noalloc_check_pointer(balance, 8, h->device, "balance")))
        return st;
    // the kernels read the particles while other threads append census
    // records and add tallies: no output may share memory with the input or
    // with another output
    const uint64_t flux_n = (uint64_t)h->num_cells * h->num_groups;
    const uint64_t bal_n = (uint64_t)h->num_problems * QSG_BAL_COUNT;
    if (soa_ranges_overlap(particles, n, census, census_capacity))
        return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: the census arrays overlap the particle arrays");
    if (ranges_overlap(flux, flux_n * 8, balance, bal_n * 8) || soa_overlaps_range(particles, n, flux, flux_n * 8) ||
        soa_overlaps_range(particles, n, balance, bal_n * 8) ||
        soa_overlaps_range(census, census_capacity, flux, flux_n * 8) ||
        soa_overlaps_range(census, census_capacity, balance, bal_n * 8))
        return fail(QSG_ERR_INVALID, "qsg_track_particles_noalloc: flux or balance overlaps another argument");
    unsigned char* scratch = nullptr;
    if ((st = noalloc_scratch_address(h->device, &scratch))) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    unsigned long long* header = reinterpret_cast<unsigned long long*>(scratch);
    unsigned long long* cursor = header + 0;
    DevStore prod[2] = {Store::carve(scratch + kNoallocHeaderBytes, QSG_NOALLOC_MAX_PRODUCTS, 0),
                        Store::carve(scratch + kNoallocHeaderBytes + kNoallocStoreBytes, QSG_NOALLOC_MAX_PRODUCTS,
                                     0)};
    const DevStore in0 = noalloc_caller_store(particles, n, header + 1);
    const DevStore out = noalloc_caller_store(census, census_capacity, header + 2);
    DevTally tally = tally_view(h);
    tally.flux = flux;
    tally.balance = reinterpret_cast<unsigned long long*>(balance);
    tally.error_flags = reinterpret_cast<unsigned int*>(header + 3);
    tally.flux_replicas = 1;
    tally.balance_replicas = 1;

    noalloc_begin_kernel<<<1, 1, 0, s>>>(header, prod[0].count, prod[1].count, (unsigned long long)n);
    QSG_CUDA(cudaGetLastError());
    unsigned long long remaining = n, counts[3] = {0, 0, 0};
    for (int pass = 0; remaining != 0; pass++) {
        const DevStore in = pass == 0 ? in0 : prod[(pass + 1) & 1];
        const DevStore extra = prod[pass & 1];
        QSG_CUDA(cudaMemsetAsync(extra.count, 0, sizeof(unsigned long long), s));
        QSG_CUDA(cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), s));
        // the kernel qsg_set_track_kernel selects, without sensitivity scores
        if ((st = launch_track_kernel(h, s, tally, cursor, PassStores{in, out, extra}, false))) return st;
        // products of this pass, census so far, device flags
        QSG_CUDA(cudaMemcpyAsync(&counts[0], extra.count, 8, cudaMemcpyDeviceToHost, s));
        QSG_CUDA(cudaMemcpyAsync(&counts[1], header + 2, 8, cudaMemcpyDeviceToHost, s));
        QSG_CUDA(cudaMemcpyAsync(&counts[2], header + 3, 8, cudaMemcpyDeviceToHost, s));
        QSG_CUDA(cudaStreamSynchronize(s));
        const unsigned int flags = (unsigned int)counts[2];
        if (counts[0] > (unsigned long long)QSG_NOALLOC_MAX_PRODUCTS)
            return fail(QSG_ERR_CAPACITY, "qsg_track_particles_noalloc: tracking pass %d made %llu fission products; "
                        "the no-allocation scratch holds at most %d per pass (QSG_NOALLOC_MAX_PRODUCTS) -- "
                        "outputs are incomplete", pass, counts[0], QSG_NOALLOC_MAX_PRODUCTS);
        if (counts[1] > census_capacity)
            return fail(QSG_ERR_CAPACITY, "qsg_track_particles_noalloc: %llu census particles exceed "
                        "census_capacity %llu -- outputs are incomplete", counts[1],
                        (unsigned long long)census_capacity);
        if (flags) return fail(QSG_ERR_DEVICE, "tracking kernel raised device flags 0x%x", flags);
        remaining = counts[0];
    }
    QSG_CUDA(cudaStreamSynchronize(s));
    *n_census = counts[1];
    return QSG_OK;
    QSG_API_END
}

// ------------------------------------------------------------------------
// Self-check of the tracking loop's replacements of FP64 operations
// (f64_to_f32_rn, div_rn, the bit-pattern comparisons, u64_scaled_2m64)
// against the FP64 operations themselves, on pseudo-random operands with hard
// cases mixed in.

namespace qsg {
namespace {

// splitmix64's output function (Steele, Lea and Flood, OOPSLA 2014)
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double f64_make(uint64_t sign, int biased_exp, uint64_t mantissa)
{
    return __longlong_as_double((long long)((sign << 63) | ((uint64_t)biased_exp << 52) |
                                            (mantissa & 0xfffffffffffffull)));
}

// one operand of the comparison check: zeros of both signs, tiny, ordinary
// and huge magnitudes of both signs, or the other operand itself
__device__ __forceinline__ double cmp_operand(uint64_t r, double other)
{
    const uint64_t s = r & 1;
    switch ((r >> 1) & 7) {
    case 0: return 0.0;
    case 1: return -0.0;
    case 2: return f64_make(s, 1 + (int)((r >> 8) % 40u), r >> 12);          // near the smallest normals
    case 3: return s ? -kHugeDouble : kHugeDouble;
    case 4: return other;
    case 5: return f64_make(s, 1 + (int)((r >> 8) % 2046u), r >> 12);        // any normal magnitude
    default: return f64_make(s, 1013 + (int)((r >> 8) % 20u), r >> 12);     // near 1
    }
}

__global__ void check_arith_kernel(uint64_t n, uint64_t seed, unsigned long long* bad)
{
    unsigned long long nbad[4] = {0, 0, 0, 0};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t r[8];
#pragma unroll
        for (int k = 0; k < 8; k++) r[k] = mix64(seed ^ mix64(8 * i + k));
        {
            // double -> float: |x| from 2^-140 to 2^100, with round-half,
            // just-below/above-half and carry-into-the-exponent mantissas
            uint64_t mant = r[0];
            switch ((r[1] >> 60) & 7) {
            case 0: mant = (mant & ~0x1fffffffull) | 0x10000000ull; break;
            case 1: mant = (mant & ~0x1fffffffull) | 0x0fffffffull; break;
            case 2: mant = (mant & ~0x1fffffffull) | 0x10000001ull; break;
            case 3: mant = (mant & ~0x1fffffffull) | 0x30000000ull; break;
            case 4: mant = ~0ull; break;
            default: break;
            }
            const double x = f64_make(r[1] & 1, 1023 - 140 + (int)((r[1] >> 8) % 240u), mant);
            const float want = (float)x, got = f64_to_f32_rn(x);
            const bool ok = (fabsf(want) >= 1.17549435e-38f)
                                ? __float_as_uint(got) == __float_as_uint(want)
                                : __float_as_uint(got) == (__float_as_uint(want) & 0x80000000u);
            nbad[0] += ok ? 0 : 1;
        }
        {
            // a / b with y = RN(1 / b): a from 2^-60 to 2^40 (or 0), b from
            // 2^-40 to 2^260, powers of two and all-ones mantissas included
            uint64_t mb = r[3];
            if (((r[2] >> 56) & 7) == 0) mb = 0;
            if (((r[2] >> 56) & 7) == 1) mb = ~0ull;
            const double b = f64_make(0, 1023 - 40 + (int)((r[2] >> 8) % 301u), mb);
            double a = f64_make(0, 1023 - 60 + (int)((r[2] >> 24) % 101u), r[4]);
            if (((r[2] >> 59) & 7) == 0) a = 0.0;
            if (((r[2] >> 59) & 7) == 1) a = b * (double)(1 + (r[4] & 1023));
            const double y = 1.0 / b;
            const double got = div_rn(a, b, y), want = a / b;
            nbad[1] += (f64_bits(got) == f64_bits(want)) ? 0 : 1;
        }
        {
            const double a = cmp_operand(r[5], 1.0);
            const double b = cmp_operand(r[5] >> 32, a);
            bool ok = (f64_lt(a, b) == (a < b)) && (f64_le(a, b) == (a <= b)) && (f64_gt0(a) == (a > 0.0)) &&
                      (f64_lt0(a) == (a < 0.0)) && (f64_eq0(a) == (a == 0.0));
            if (!(b == 0.0)) ok = ok && (f64_eq(a, b) == (a == b));
            nbad[2] += ok ? 0 : 1;
        }
        {
            // the random-number sample 2^-64 (double)x: any x, small x, powers
            // of two, round-half patterns of the 11 dropped bits, all ones, 0
            uint64_t x = r[6];
            switch ((r[7] >> 60) & 7) {
            case 0: x >>= (r[7] & 63); break;
            case 1: x = 1ull << (r[7] & 63); break;
            case 2: x = (x & ~0x7ffull) | 0x400ull; break;
            case 3: x = (x & ~0xfffull) | 0xc00ull; break;
            case 4: x = ~0ull; break;
            case 5: x = (x & ~0x7ffull) | 0x3ffull; break;
            case 6: x = 0; break;
            default: break;
            }
            const double want = 5.4210108624275222e-20 * __ull2double_rn(x);
            nbad[3] += (f64_bits(u64_scaled_2m64(x)) == f64_bits(want)) ? 0 : 1;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (nbad[k]) atomicAdd(bad + k, nbad[k]);
}

}  // namespace
}  // namespace qsg

extern "C" int qsg_check_arithmetic(int32_t device, uint64_t n, uint64_t seed, uint64_t* mismatches)
{
    QSG_API_BEGIN
    if (!mismatches) return fail(QSG_ERR_INVALID, "qsg_check_arithmetic: null argument");
    int ndev = 0;
    qsg_device_count(&ndev);
    if (ndev == 0) return fail(QSG_ERR_NO_DEVICE, "qsg_check_arithmetic: no CUDA device visible");
    if (device < 0 || device >= ndev)
        return fail(QSG_ERR_INVALID, "qsg_check_arithmetic: device %d of %d", (int)device, ndev);
    QSG_CUDA(cudaSetDevice(device));
    qsg::DevBuf<unsigned long long> bad;
    int st = bad.alloc(4);
    if (st) return st;
    unsigned long long host[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemset(bad.ptr, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess && n > 0) {
        qsg::check_arith_kernel<<<4 * 152, 256>>>(n, seed, bad.ptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(host, bad.ptr, sizeof(host), cudaMemcpyDeviceToHost);
    bad.free();
    if (e != cudaSuccess) return fail(QSG_ERR_CUDA, "qsg_check_arithmetic: %s", cudaGetErrorString(e));
    for (int k = 0; k < 4; k++) mismatches[k] = host[k];
    return QSG_OK;
    QSG_API_END
}

// ------------------------------------------------------------------------
// The portable elementary functions evaluated on the device, for the check
// that the GPU gives the host's bits (portable_math.h).

namespace qsg {
namespace {

__global__ void portable_math_kernel(const double* x, uint64_t n, double* lg, double* sn, double* cs)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        lg[i] = qsg_log(x[i]);
        qsg_sincos(x[i], sn + i, cs + i);
    }
}

}  // namespace
}  // namespace qsg

extern "C" int qsg_portable_math_eval(int32_t device, const double* x, uint64_t n, double* lg, double* sn,
                                      double* cs)
{
    QSG_API_BEGIN
    if (n > 0 && (!x || !lg || !sn || !cs)) return fail(QSG_ERR_INVALID, "qsg_portable_math_eval: null argument");
    int ndev = 0;
    qsg_device_count(&ndev);
    if (ndev == 0) return fail(QSG_ERR_NO_DEVICE, "qsg_portable_math_eval: no CUDA device visible");
    if (device < 0 || device >= ndev)
        return fail(QSG_ERR_INVALID, "qsg_portable_math_eval: device %d of %d", (int)device, ndev);
    if (n == 0) return QSG_OK;
    QSG_CUDA(cudaSetDevice(device));
    qsg::DevBuf<double> buf;
    int st = buf.alloc(4 * n);
    if (st) return st;
    cudaError_t e = cudaMemcpy(buf.ptr, x, n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        qsg::portable_math_kernel<<<4 * 152, 256>>>(buf.ptr, n, buf.ptr + n, buf.ptr + 2 * n, buf.ptr + 3 * n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(lg, buf.ptr + n, n * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(sn, buf.ptr + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(cs, buf.ptr + 3 * n, n * sizeof(double), cudaMemcpyDeviceToHost);
    buf.free();
    if (e != cudaSuccess) return fail(QSG_ERR_CUDA, "qsg_portable_math_eval: %s", cudaGetErrorString(e));
    return QSG_OK;
    QSG_API_END
}

// ------------------------------------------------------------------------
// FP64 issue rate of the device: the roof of the tracking loop, whose
// binding resource is FP64 warp instructions (their cost does not depend on
// how many lanes are active).

namespace qsg {
namespace {

constexpr int kFp64ProbeBlock = 256;     // 8 warps; two blocks per SM keep the pipe saturated
constexpr int kFp64ProbeChains = 4;      // independent multiply-add chains per thread

__global__ void fp64_rate_kernel(int iters, double* out)
{
    double v[kFp64ProbeChains];
#pragma unroll
    for (int k = 0; k < kFp64ProbeChains; k++) v[k] = 1.0 + 1e-9 * (threadIdx.x + 1024 * k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < kFp64ProbeChains; k++) v[k] = fma(v[k], 0.999999999, 1e-12);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kFp64ProbeChains; k++) s += v[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace qsg

extern "C" int qsg_measure_fp64_rate(int32_t device, double* warp_instructions_per_second)
{
    QSG_API_BEGIN
    if (!warp_instructions_per_second) return fail(QSG_ERR_INVALID, "qsg_measure_fp64_rate: null argument");
    int ndev = 0;
    qsg_device_count(&ndev);
    if (ndev == 0) return fail(QSG_ERR_NO_DEVICE, "qsg_measure_fp64_rate: no CUDA device visible");
    if (device < 0 || device >= ndev)
        return fail(QSG_ERR_INVALID, "qsg_measure_fp64_rate: device %d of %d", (int)device, ndev);
    QSG_CUDA(cudaSetDevice(device));
    int sms = 0;
    QSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int blocks = 2 * sms, iters = 20000;
    qsg::DevBuf<double> out;
    int st = out.alloc((size_t)blocks * qsg::kFp64ProbeBlock);
    if (st) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best_ms = 0.0f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; rep++) {   // the first launch warms up
        e = cudaEventRecord(e0, 0);
        if (e == cudaSuccess) {
            qsg::fp64_rate_kernel<<<blocks, qsg::kFp64ProbeBlock>>>(iters, out.ptr);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best_ms == 0.0f || ms < best_ms)) best_ms = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    out.free();
    if (e != cudaSuccess) return fail(QSG_ERR_CUDA, "qsg_measure_fp64_rate: %s", cudaGetErrorString(e));
    const double warp_instr = (double)blocks * (qsg::kFp64ProbeBlock / 32) * qsg::kFp64ProbeChains * iters;
    *warp_instructions_per_second = warp_instr / (1e-3 * best_ms);
    return QSG_OK;
    QSG_API_END
}
