// vpf_common.cuh -- shared device code of the GB300 VPF / VSWRM kernels.
//
// Pixel decisions follow vf_supcalc.projection_field (vf_supcalc.py:20-138):
//   bearing ca = calculate_closed_angle(v1, v2)          (vf_supcalc.py:142-158)
//   t  = argmin_k |linspace(-pi, pi, Rv)[k] - ca|        (supcalc.find_nearest, supcalc.py:8-11)
//   h  = floor(proj_size / 2), proj_size = 2 atan(R/d) / (2 pi) * Rv   (vf_supcalc.py:96-117)
//   pixels [t-h, t+h) with the reference's wrap rules    (vf_supcalc.py:119-129)
// Both discrete decisions are first taken in FP32.  When the FP32 value lies inside a guard
// band around a decision boundary (width derived from the FP32 error bound), the decision is
// taken again exactly in double-float ("df", a pair of floats, ~2^-44 relative) from the
// exact coordinate differences: the bearing side of a pixel midpoint is the sign of a 2-D
// cross product with the midpoint's direction, and the width side of floor(.) is a
// comparison of d^2 with R^2 cot^2(2 pi k / Rv).  No FP64 arithmetic is used per pair.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define ABM_FULL_MASK 0xffffffffu

namespace abm {

constexpr float kPiF = 3.14159265358979f;
constexpr float kHalfPiF = 1.57079632679490f;
constexpr double kPi = 3.141592653589793;
constexpr double kFix = 1099511627776.0;          // 2^40: fixed-point scale of the tables
constexpr double kInvFix = 1.0 / 1099511627776.0;

// ------------------------------------------------------------------ double-float arithmetic
struct dfl {
    float hi, lo;
};

__device__ __forceinline__ dfl two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {  // |a| >= |b|
    float s = a + b;
    float e = b - (s - a);
    return {s, e};
}
__device__ __forceinline__ dfl two_prod(float a, float b) {
    float p = a * b;
    float e = fmaf(a, b, -p);
    return {p, e};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    dfl s = two_sum(a.hi, b.hi);
    dfl t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    dfl p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, p.lo);
    p.lo = fmaf(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ int df_sign(dfl a) {
    if (a.hi > 0.f) return 1;
    if (a.hi < 0.f) return -1;
    return (a.lo > 0.f) - (a.lo < 0.f);
}
__device__ __forceinline__ bool df_gt(dfl a, float b) {  // a > b
    return a.hi > b || (a.hi == b && a.lo > 0.f);
}
__device__ __forceinline__ dfl df_split(double v) {
    float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}

// ------------------------------------------------------------------ FP32 arctangent
// atan(r) = r * P(r^2) on [0, 1]; P fitted by abm_gb300/csrc/fit_atan.py (Lawson near-minimax
// of the absolute error), max error 2.0e-8 with these float32 coefficients.
__device__ __forceinline__ float atan_poly(float s) {
    float p = 2.456724644e-03f;
    p = fmaf(p, s, -1.440135855e-02f);
    p = fmaf(p, s, 3.978122398e-02f);
    p = fmaf(p, s, -7.234857231e-02f);
    p = fmaf(p, s, 1.049894616e-01f);
    p = fmaf(p, s, -1.416122913e-01f);
    p = fmaf(p, s, 1.998590678e-01f);
    p = fmaf(p, s, -3.333259821e-01f);
    p = fmaf(p, s, 9.999998808e-01f);
    return p;
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Closed angle of vf_supcalc.calculate_closed_angle in FP32: ca = -angle_between(v1, v2)
// = atan2(-P, Q) with P = cross(v1, v2), Q = dot(v1, v2) (v1 the heading), and the
// reference's convention that P == 0 counts as non-negative (target exactly behind -> -pi).
__device__ __forceinline__ float closed_angle_f32(float P, float Q) {
    float ay = fabsf(P), ax = fabsf(Q);
    float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    float r = mn * rcp_approx(mx);
    float a = r * atan_poly(r * r);
    a = (ay > ax) ? kHalfPiF - a : a;
    a = (Q < 0.f) ? kPiF - a : a;
    return (P >= 0.f) ? -a : a;
}

// Half visual angle alpha = atan(R / d) from d^2 and rsqrt(d^2).
__device__ __forceinline__ float half_angle_f32(float R, float invR, float d2, float rsq) {
    float xr = R * rsq;
    bool big = xr > 1.f;
    float r = big ? (d2 * rsq) * invR : xr;
    float a = r * atan_poly(r * r);
    return big ? kHalfPiF - a : a;
}

// ------------------------------------------------------------------ grid tables
// One set per (Rv, field of view): built on the host in FP64 (abm_vpf_tables.cu), read-only.
struct GridDev {
    int rv, words, f0, f1;     // f0/f1: find_nearest(phis, fov0 / fov1)
    int kmax;                  // cot2 valid for 1 <= k < kmax (2 pi k / Rv < pi / 2)
    int phi_ok;                // len(np.arange(-pi, pi, 2pi/Rv)) == Rv
    float inv_delta;           // (Rv - 1) / (2 pi): linspace pixels per radian
    float half_rm1;            // (Rv - 1) / 2 (exact)
    float rvm1;                // Rv - 1
    float ps2_scale;           // Rv / (2 pi): proj_size / 2 per radian of half angle
    float band_t;              // guard band of the bearing decision, in pixels
    float band_h;              // guard band of floor(proj_size/2), relative
    float cull;                // d^2 > R^2 * cull  =>  proj_size/2 < 1 certainly (h = 0)
    const float4 *mid;         // [Rv-1]: df cos, df sin of the midpoint of linspace px k, k+1
    const float2 *cot2;        // [kmax]: df cot^2(2 pi k / Rv)
    const longlong2 *q;        // [Rv+1]: trapezoid prefix sums (cos, sin) * 2^40
    const longlong2 *cpt;      // [Rv]:   cos, sin of PHI_k * 2^40
    long long qc_total, qs_total;
};

// Inclusive-exclusive pixel run [a, b), 0 <= a < b <= Rv, OR-ed into a shared bitmask.
__device__ __forceinline__ void raster_run(uint32_t *vb, int a, int b) {
    int wa = a >> 5, wb = (b - 1) >> 5;
    uint32_t ma = ABM_FULL_MASK << (a & 31);
    uint32_t mb = ABM_FULL_MASK >> (31 - ((b - 1) & 31));
    if (wa == wb) {
        atomicOr(&vb[wa], ma & mb);
        return;
    }
    atomicOr(&vb[wa], ma);
    for (int w = wa + 1; w < wb; ++w) vb[w] = ABM_FULL_MASK;  // idempotent with racing ORs
    atomicOr(&vb[wb], mb);
}

// The reference's fill of one visible projection (vf_supcalc.py:119-129) given s = t - h,
// e = t + h; only called for visible projections, for which Rv + s > 0.
__device__ __forceinline__ void raster_projection(uint32_t *vb, int rv, int s, int e) {
    if (s < 0) {
        raster_run(vb, rv + s, rv);
        s = 0;
    }
    if (e >= rv) {
        int b = e - (rv - 1);
        raster_run(vb, 0, b < rv ? b : rv);
        e = rv;
    }
    if (s < e) raster_run(vb, s, e);
}

// ------------------------------------------------------------------ pair decisions
struct FocalDev {
    float x, y, r, invr;   // top-left position and radius (float32 state)
    float c, s;            // cos/sin(theta) rounded to float
    dfl cd, sd;            // cos/sin(theta) in double-float
};

// Exact centre offset (object centre - focal centre) as double-float, with the torus minimal
// image of vf_supcalc.py:70-83 decided on the exact value.  W/H as double-float.
template <bool TORUS, bool HETERO>
__device__ __forceinline__ void exact_offset(const FocalDev &f, float xj, float yj, float rj,
                                             dfl W, dfl H, dfl &ex, dfl &ey) {
    ex = two_sum(xj, -f.x);
    ey = two_sum(yj, -f.y);
    if (HETERO) {
        dfl dr = two_sum(rj, -f.r);
        ex = df_add(ex, dr);
        ey = df_add(ey, dr);
    }
    if (TORUS) {
        dfl hw = {W.hi * 0.5f, W.lo * 0.5f}, hh = {H.hi * 0.5f, H.lo * 0.5f};
        if (df_sign(df_sub(ex, hw)) > 0) ex = df_sub(ex, W);
        else if (df_sign(df_add(ex, hw)) < 0) ex = df_add(ex, W);
        if (df_sign(df_sub(ey, hh)) > 0) ey = df_sub(ey, H);
        else if (df_sign(df_add(ey, hh)) < 0) ey = df_add(ey, H);
    }
}

// Double-float re-decision of the pixel index t and/or the half width h of one pair.
// u: FP32 pixel coordinate of the bearing; ps2: FP32 proj_size/2.  Counts the pair in
// diag[0], and in diag[1] when a decision lies within 1e-9 rad of its boundary.
struct ResolveGrid {  // the parts of GridDev the double-float re-decision needs
    const float4 *mid;
    const float2 *cot2;
    int rv, kmax;
    float band_t, rvm1;
};

__device__ __forceinline__ ResolveGrid resolve_grid(const GridDev &g) {
    return {g.mid, g.cot2, g.rv, g.kmax, g.band_t, g.rvm1};
}

// Returns the re-decided (t, h).
static __device__ __noinline__ int2 resolve_pair(dfl cd, dfl sd, dfl ex, dfl ey, float rj,
                                          ResolveGrid g, bool unc_t, bool unc_h, float u,
                                          float ps2, int t, int h,
                                          unsigned long long *diag) {
    dfl P = df_add(df_mul(cd, ey), df_mul(sd, ex));  // cross(v1, v2) / R
    dfl Q = df_sub(df_mul(cd, ex), df_mul(sd, ey));  // dot(v1, v2) / R
    dfl d2 = df_add(df_mul(ex, ex), df_mul(ey, ey));
    float d = sqrtf(d2.hi);
    bool near = false;
    if (unc_t) {
        if (u < g.band_t || u > g.rvm1 - g.band_t) {
            // seam at +-pi: P >= 0 -> ca just above -pi (pixel 0), P < 0 -> just below pi
            t = (df_sign(P) >= 0) ? 0 : g.rv - 1;
            near |= fabsf(P.hi) < 1e-9f * d;
        } else {
            int k = (int)floorf(u);
            k = k < 0 ? 0 : (k > g.rv - 2 ? g.rv - 2 : k);
            float4 m = g.mid[k];
            dfl S = df_add(df_mul(dfl{m.x, m.y}, P), df_mul(dfl{m.z, m.w}, Q));
            // ca > midpoint  <=>  cos(m) P + sin(m) Q < 0; ties go to the lower pixel
            t = (df_sign(S) < 0) ? k + 1 : k;
            near |= fabsf(S.hi) < 1e-9f * d;
        }
    }
    if (unc_h) {
        int k = (int)rintf(ps2);
        if (k <= 0) {
            h = 0;
        } else if (k >= g.kmax) {
            h = k - 1;                      // 2 pi k / Rv >= pi/2 > atan(R/d) for d > 0
        } else {
            float2 c2 = g.cot2[k];
            dfl thr = df_mul(two_prod(rj, rj), dfl{c2.x, c2.y});
            dfl diff = df_sub(thr, d2);     // >= 0  <=>  atan(R/d) >= 2 pi k / Rv
            h = (df_sign(diff) >= 0) ? k : k - 1;
            // |d alpha| ~ R |d^2 - thr| / (2 d (d^2 + R^2))
            float da = rj * fabsf(diff.hi) / (2.f * d * (d2.hi + rj * rj));
            near |= da < 1e-9f;
        }
    }
    if (diag) {
        atomicAdd(&diag[0], 1ull);
        if (near) atomicAdd(&diag[1], 1ull);
    }
    return make_int2(t, h);
}

// Full decision for one ordered pair (all 32 lanes call it; `live` masks the lane's pair).
// Returns the visible projection's (s, e) or vis = false.
template <bool TORUS, bool HETERO>
__device__ __forceinline__ void pair_projection(const FocalDev &f, float xj, float yj, float rj,
                                                float invrj, bool valid, const GridDev &g,
                                                dfl W, dfl H, int &s_out, int &e_out,
                                                bool &vis, unsigned long long *diag) {
    float dx, dy;
    if (!TORUS && !HETERO) {
        dx = xj - f.x;
        dy = yj - f.y;
    } else {
        dfl ex, ey;
        exact_offset<TORUS, HETERO>(f, xj, yj, rj, W, H, ex, ey);
        dx = ex.hi + ex.lo;
        dy = ey.hi + ey.lo;
    }
    bool same = (xj == f.x) && (yj == f.y);   // vf_supcalc.py:57-58 (covers j == i)
    float d2 = fmaf(dx, dx, dy * dy);
    bool live = valid && !same && (d2 <= rj * rj * g.cull);
    float rsq = rsqrtf(d2);
    float P = fmaf(f.c, dy, f.s * dx);
    float Q = fmaf(f.c, dx, -(f.s * dy));
    float ca = closed_angle_f32(P, Q);
    float u = fmaf(ca, g.inv_delta, g.half_rm1);
    float kf = floorf(u);
    float fr = u - kf;
    int t = (int)kf + (fr > 0.5f ? 1 : 0);
    t = t < 0 ? 0 : (t > g.rv - 1 ? g.rv - 1 : t);
    bool unc_t = fabsf(fr - 0.5f) < g.band_t || u < g.band_t || u > g.rvm1 - g.band_t;
    float al = half_angle_f32(rj, invrj, d2, rsq);
    float ps2 = al * g.ps2_scale;
    float hf = floorf(ps2);
    int h = (int)hf;
    float frh = ps2 - hf;
    float bh = g.band_h * fmaxf(ps2, 1.f);
    bool unc_h = frh < bh || frh > 1.f - bh;
    if (d2 == 0.f) {  // coincident centres, different top-left: atan(R/0) = pi/2, NaN bearing -> 0
        t = 0;
        h = g.rv >> 2;
        unc_t = unc_h = false;
    }
    bool unc = live && (unc_t || unc_h);
    if (__any_sync(ABM_FULL_MASK, unc)) {
        if (unc) {
            dfl ex, ey;
            exact_offset<TORUS, HETERO>(f, xj, yj, rj, W, H, ex, ey);
            int2 th = resolve_pair(f.cd, f.sd, ex, ey, rj, resolve_grid(g), unc_t, unc_h, u,
                                   ps2, t, h, diag);
            t = th.x;
            h = th.y;
        }
    }
    int s = t - h, e = t + h;
    vis = live && ((g.f0 < s && s < g.f1) || (g.f0 < e && e < g.f1));
    s_out = s;
    e_out = e;
}

// ------------------------------------------------------------------ VSWRM integrals
// For a warp's bitmask vb (raw pixel order), the four fixed-point sums
//   blob_c = sum_k w_k cos(PHI_k) V_k, blob_s likewise, edge_c = sum_k cos(PHI_k) E_k, edge_s
// where w_k are the trapezoid weights of scipy's trapz over PHI and E = dPhi_V_of(V)^2
// (vf_supcalc.py:257-277: forward circular difference, backward when V[0]=1, V[Rv-1]=0).
// Uses sum_k w_k f_k V_k = Q[Rv] V[Rv-1] + sum_{j=1..Rv-1} Q[j] (V[j-1] - V[j]) with Q the
// prefix sums, so only the transitions of V are visited.  Result valid in lane 0.
__device__ __forceinline__ void warp_integrals(const uint32_t *vb, const GridDev &g,
                                               long long &bc, long long &bs, long long &ec,
                                               long long &es) {
    const int lane = threadIdx.x & 31;
    const int rv = g.rv;
    const uint32_t v0 = vb[0] & 1u;
    const uint32_t vl = (vb[(rv - 1) >> 5] >> ((rv - 1) & 31)) & 1u;
    const int bwd = (v0 == 1u && vl == 0u) ? 1 : 0;
    bc = bs = ec = es = 0;
    for (int w = lane; w < g.words; w += 32) {
        uint32_t cur = vb[w];
        uint32_t prev = (w > 0) ? (vb[w - 1] >> 31) : (cur & 1u);
        uint32_t D = cur ^ ((cur << 1) | prev);
        if (w == g.words - 1 && (rv & 31)) D &= (1u << (rv & 31)) - 1u;
        while (D) {
            int b = __ffs(D) - 1;
            D &= D - 1u;
            int j = (w << 5) + b;
            longlong2 qv = g.q[j];
            if ((cur >> b) & 1u) {   // run starts at j
                bc -= qv.x;
                bs -= qv.y;
            } else {                  // run ends at j
                bc += qv.x;
                bs += qv.y;
            }
            longlong2 cv = g.cpt[j - 1 + bwd];
            ec += cv.x;
            es += cv.y;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bc += __shfl_xor_sync(ABM_FULL_MASK, bc, o);
        bs += __shfl_xor_sync(ABM_FULL_MASK, bs, o);
        ec += __shfl_xor_sync(ABM_FULL_MASK, ec, o);
        es += __shfl_xor_sync(ABM_FULL_MASK, es, o);
    }
    if (vl) {
        bc += g.qc_total;
        bs += g.qs_total;
    }
    if (v0 != vl) {  // the circular edge between pixels Rv-1 and 0
        longlong2 cv = g.cpt[bwd ? 0 : rv - 1];
        ec += cv.x;
        es += cv.y;
    }
}

// ------------------------------------------------------------------ agent update (FP64)
struct UpdateParams {
    double gam, v0, alp0, alp1, bet0, bet1;
    double max_vel, max_th, dt;
    double bx0, bx1, by0, by1;
    int limit, torus;
};

__device__ __forceinline__ double prove_orientation(double th) {  // agent.py:605-610
    if (th < 0) th = 2 * kPi + th;
    if (th > kPi * 2) th = th - 2 * kPi;
    return th;
}

// VFAgent.update_agent_position (vf_agent.py:289-309), prove_turning/prove_velocity
// (:311-327), then Agent.reflect_from_walls (agent.py:347-394) or
// VFAgent.teleport_infinite_arena (vf_agent.py:188-204).
__device__ __forceinline__ void update_agent(const UpdateParams &p, double R, double dpsi,
                                             double dv, double &x, double &y, double &th,
                                             double &v) {
    double theta = dpsi * p.dt;
    if (p.limit && fabs(theta) > p.max_th) theta = p.max_th * (theta < 0 ? -1.0 : 1.0);
    th = prove_orientation(th + theta);
    v += dv * p.dt;
    if (p.limit && fabs(v) > p.max_vel) v = p.max_vel * (v < 0 ? -1.0 : 1.0);
    double sn, cs;
    sincos(th, &sn, &cs);
    x = x + (v * p.dt) * cs;
    y = y - (v * p.dt) * sn;
    const double cx = x + R, cy = y + R;
    if (!p.torus) {
        if (cx < p.bx0) {
            x = p.bx0 - R;
            if (kPi / 2 <= th && th < kPi) th -= kPi / 2;
            else if (kPi <= th && th <= 3 * kPi / 2) th += kPi / 2;
            th = prove_orientation(th);
        }
        if (cx > p.bx1) {
            x = p.bx1 - R - 1;
            if (3 * kPi / 2 <= th && th < 2 * kPi) th -= kPi / 2;
            else if (0 <= th && th <= kPi / 2) th += kPi / 2;
            th = prove_orientation(th);
        }
        if (cy < p.by0) {
            y = p.by0 - R;
            if (kPi / 2 <= th && th <= kPi) th += kPi / 2;
            else if (0 <= th && th < kPi / 2) th -= kPi / 2;
            th = prove_orientation(th);
        }
        if (cy > p.by1) {
            y = p.by1 - R - 1;
            if (3 * kPi / 2 <= th && th <= 2 * kPi) th += kPi / 2;
            else if (kPi <= th && th < 3 * kPi / 2) th -= kPi / 2;
            th = prove_orientation(th);
        }
    } else {
        if (cx < p.bx0) x = p.bx1 - R;
        else if (cx > p.bx1) x = p.bx0 + R;
        if (cy < p.by0) y = p.by1 - R;
        else if (cy > p.by1) y = p.by0 + R;
    }
}

// ------------------------------------------------------------------ TMA bulk staging
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// 1-D bulk copy global -> shared (TMA engine), completion signalled on `bar`.  dst, src and
// bytes must be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// Bounded wait on an mbarrier phase; false when the limit was reached.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    for (int it = 0; it < (1 << 20); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

}  // namespace abm
