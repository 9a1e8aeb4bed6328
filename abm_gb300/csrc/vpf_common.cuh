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

// Programmatic dependent launch: a kernel launched with programmatic stream serialisation may
// be scheduled while the previous kernel on the stream drains (once every block of that kernel
// has called allow_dependent_launch or exited); wait_primary_grid returns once the previous
// kernel has completed and its memory is visible, so a dependent kernel touches nothing that
// earlier work writes or reads before it.  Without such a launch both return at once.
__device__ __forceinline__ void allow_dependent_launch() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void wait_primary_grid() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// The calling grid's share of the 128-byte lines of a read-only table, prefetched into L2
// (each thread of the grid takes lines tid, tid + grid threads, ...; only lines inside
// [base, base + bytes) are touched).
__device__ __forceinline__ void prefetch_table_l2(const void *base, size_t bytes) {
    const size_t lines = (bytes + 127) / 128;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t l = (size_t)blockIdx.x * blockDim.x + threadIdx.x; l < lines; l += stride)
        asm volatile("prefetch.global.L2 [%0];" ::"l"((const char *)base + l * 128));
}

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
// a + b for a float b: df_add(a, {b, 0}) without the operations on the zero low part (the same
// value; only the sign of a zero low part can differ)
__device__ __forceinline__ dfl df_add_f(dfl a, float b) {
    dfl s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}
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

__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
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
    int full_fov;              // f0 == 0 and f1 == Rv - 1: every projection with h >= 1 is
                               // visible (vf_supcalc.py:119 can only fail when 2h >= Rv - 1,
                               // and h < Rv / 4 since atan(R/d) < pi/2)
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

struct ResolveGrid {  // the parts of GridDev the double-float re-decision needs
    const float4 *mid;
    const float2 *cot2;
    int rv, kmax;
    float band_t, rvm1;
};

__device__ __forceinline__ ResolveGrid resolve_grid(const GridDev &g) {
    return {g.mid, g.cot2, g.rv, g.kmax, g.band_t, g.rvm1};
}

// Double-float re-decision of the pixel index t and/or the half width h of one pair.
// u: FP32 pixel coordinate of the bearing; ps2: FP32 proj_size/2.  Returns (t, h) in x, y and
// in z whether a re-decided boundary lies within 1e-9 rad of the pair's edge angle.
static __device__ __noinline__ int3 resolve_pair(dfl cd, dfl sd, dfl ex, dfl ey, float rj,
                                                 ResolveGrid g, bool unc_t, bool unc_h, float u,
                                                 float ps2, int t, int h) {
    // the table entries first (predicated loads of clamped indices), so that their latency
    // overlaps the double-float products below
    const int kt = min(max((int)floorf(u), 0), max(g.rv - 2, 0));
    const int kh = (int)rintf(ps2);
    const int khc = min(max(kh, 0), max(g.kmax - 1, 0));
    const float4 m = unc_t ? __ldg(g.mid + kt) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 c2 = unc_h ? __ldg(g.cot2 + khc) : make_float2(0.f, 0.f);
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
            dfl S = df_add(df_mul(dfl{m.x, m.y}, P), df_mul(dfl{m.z, m.w}, Q));
            // ca > midpoint  <=>  cos(m) P + sin(m) Q < 0; ties go to the lower pixel
            t = (df_sign(S) < 0) ? kt + 1 : kt;
            near |= fabsf(S.hi) < 1e-9f * d;
        }
    }
    if (unc_h) {
        const int k = kh;
        if (k <= 0) {
            h = 0;
        } else if (k >= g.kmax) {
            h = k - 1;                      // 2 pi k / Rv >= pi/2 > atan(R/d) for d > 0
        } else {
            dfl thr = df_mul(two_prod(rj, rj), dfl{c2.x, c2.y});
            dfl diff = df_sub(thr, d2);     // >= 0  <=>  atan(R/d) >= 2 pi k / Rv
            h = (df_sign(diff) >= 0) ? k : k - 1;
            // |d alpha| ~ R |d^2 - thr| / (2 d (d^2 + R^2))
            float da = rj * fabsf(diff.hi) / (2.f * d * (d2.hi + rj * rj));
            near |= da < 1e-9f;
        }
    }
    return make_int3(t, h, near ? 1 : 0);
}

// FP32 centre offset of one ordered pair (exact differences rounded once; the torus image
// and unequal radii go through the exact double-float offset).
template <bool TORUS, bool HETERO>
__device__ __forceinline__ void pair_offset(const FocalDev &f, float xj, float yj, float rj,
                                            dfl W, dfl H, float &dx, float &dy) {
    if (!TORUS && !HETERO) {
        const float2 d = __fadd2_rn(make_float2(xj, yj), make_float2(-f.x, -f.y));
        dx = d.x;
        dy = d.y;
    } else {
        dfl ex, ey;
        exact_offset<TORUS, HETERO>(f, xj, yj, rj, W, H, ex, ey);
        dx = ex.hi + ex.lo;
        dy = ey.hi + ey.lo;
    }
}

// FP32 estimate of the pixel index t and half width h of one live pair, with the flags of
// decisions that fall inside the guard bands.
struct PairEst {
    int t, h;
    float u, ps2, ca;
    bool unc_t, unc_h;
};

// Both arctangents of a pair share one packed (FP32x2) Horner chain: lane .x is the bearing
// ratio, lane .y the half-angle ratio.
__device__ __forceinline__ float2 atan_poly2(float2 s) {
    float2 p = make_float2(2.456724644e-03f, 2.456724644e-03f);
    p = __ffma2_rn(p, s, make_float2(-1.440135855e-02f, -1.440135855e-02f));
    p = __ffma2_rn(p, s, make_float2(3.978122398e-02f, 3.978122398e-02f));
    p = __ffma2_rn(p, s, make_float2(-7.234857231e-02f, -7.234857231e-02f));
    p = __ffma2_rn(p, s, make_float2(1.049894616e-01f, 1.049894616e-01f));
    p = __ffma2_rn(p, s, make_float2(-1.416122913e-01f, -1.416122913e-01f));
    p = __ffma2_rn(p, s, make_float2(1.998590678e-01f, 1.998590678e-01f));
    p = __ffma2_rn(p, s, make_float2(-3.333259821e-01f, -3.333259821e-01f));
    p = __ffma2_rn(p, s, make_float2(9.999998808e-01f, 9.999998808e-01f));
    return p;
}

template <bool HETERO>
__device__ __forceinline__ PairEst estimate_pair(const FocalDev &f, float dx, float dy, float rj,
                                                 float invrj, const GridDev &g) {
    PairEst r;
    // d^2 >= 1e-30 keeps rsqrt finite for offsets below 1e-15 px (flush-to-zero range)
    const float d2raw = fmaf(dx, dx, dy * dy);
    const float d2 = fmaxf(d2raw, 1e-30f);
    const float rsq = rsqrt_approx(d2);
    // (P, Q) = (c dy + s dx, c dx - s dy): cross and dot of the heading with the offset
    const float2 PQ = __ffma2_rn(make_float2(f.c, f.c), make_float2(dy, dx),
                                 __fmul2_rn(make_float2(f.s, -f.s), make_float2(dx, dy)));
    const float P = PQ.x, Q = PQ.y;
    const float ay = fabsf(P), ax = fabsf(Q);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    const float rb = mn * rcp_approx(mx);                  // bearing ratio in [0, 1]
    const float xr = rj * rsq;                             // R / d
    const bool big = xr > 1.f;
    const float rh = big ? (d2 * rsq) * invrj : xr;        // half-angle ratio in [0, 1]
    const float2 rr = make_float2(rb, rh);
    const float2 at = __fmul2_rn(rr, atan_poly2(__fmul2_rn(rr, rr)));
    float a = at.x;
    a = (ay > ax) ? kHalfPiF - a : a;
    a = (Q < 0.f) ? kPiF - a : a;
    const float ca = (P >= 0.f) ? -a : a;
    const float al = big ? kHalfPiF - at.y : at.y;
    // (u, ps2): pixel coordinate of the bearing and proj_size / 2
    const float2 up = __ffma2_rn(make_float2(ca, al), make_float2(g.inv_delta, g.ps2_scale),
                                 make_float2(g.half_rm1, 0.f));
    const float u = up.x, ps2 = up.y;
    const float kf = floorf(u), hf = floorf(ps2);
    const float2 fr = __fadd2_rn(up, make_float2(-kf - 0.5f, -hf - 0.5f));  // frac - 1/2
    int t = (int)kf + (fr.x > 0.f ? 1 : 0);
    r.t = min(max(t, 0), g.rv - 1);
    r.h = (int)hf;
    r.unc_t = fabsf(fr.x) < g.band_t || fabsf(u - g.half_rm1) > g.half_rm1 - g.band_t;
    r.unc_h = fabsf(fr.y) > 0.5f - g.band_h * fmaxf(ps2, 1.f);
    if (HETERO && d2raw == 0.f) {  // coincident centres: atan(R/0) = pi/2, NaN bearing -> px 0
        r.t = 0;
        r.h = g.rv >> 2;
        r.unc_t = r.unc_h = false;
    }
    r.u = u;
    r.ps2 = ps2;
    r.ca = ca;
    return r;
}

// FP32 decisions of one live pair of equal radii from its queued offset (dx, dy) and d^2:
// t (nearest linspace pixel of the bearing, round to nearest) and h = floor(proj_size / 2).
// unc: a decision lies inside its guard band (the double-float re-decision takes it), the
// bearing lies near the +-pi seam, or the discs overlap (R / d > 1, where the arctangent
// argument leaves [0, 1]); t and h are meaningful only when unc is false, and then
// 0 <= t < Rv.
struct FastEst {
    int t, h;
    bool unc;
};

__device__ __forceinline__ FastEst estimate_fast(const FocalDev &f, float dx, float dy, float d2,
                                                 float R, float R2, const GridDev &g) {
    FastEst r;
    const float rsq = rsqrt_approx(d2);
    // (P, Q) = (c dy + s dx, c dx - s dy): cross and dot of the heading with the offset
    const float2 PQ = __ffma2_rn(make_float2(f.c, f.c), make_float2(dy, dx),
                                 __fmul2_rn(make_float2(f.s, -f.s), make_float2(dx, dy)));
    const float P = PQ.x, Q = PQ.y;
    const float ay = fabsf(P), ax = fabsf(Q);
    const float2 rr = make_float2(fminf(ax, ay) * rcp_approx(fmaxf(ax, ay)), R * rsq);
    const float2 at = __fmul2_rn(rr, atan_poly2(__fmul2_rn(rr, rr)));
    float a = at.x;
    a = (ay > ax) ? kHalfPiF - a : a;
    a = (Q < 0.f) ? kPiF - a : a;
    const float ca = (P >= 0.f) ? -a : a;
    // (u, ps2): pixel coordinate of the bearing and proj_size / 2
    const float2 up = __ffma2_rn(make_float2(ca, at.y), make_float2(g.inv_delta, g.ps2_scale),
                                 make_float2(g.half_rm1, 0.f));
    const float ut = rintf(up.x), hf = floorf(up.y);
    const float2 fr = __fadd2_rn(up, make_float2(-ut, -hf - 0.5f));   // |fr.x|, |fr.y| <= 1/2
    r.t = (int)ut;
    r.h = (int)hf;
    r.unc = fabsf(fr.x) > 0.5f - g.band_t || fabsf(up.x - g.half_rm1) > g.half_rm1 - g.band_t ||
            fabsf(fr.y) > __fmaf_rn(-g.band_h, fmaxf(up.y, 1.f), 0.5f) || d2 < R2;
    return r;
}

// Visibility test of vf_supcalc.py:119 (strict, on the pixel indices).
__device__ __forceinline__ bool projection_visible(const GridDev &g, int s, int e) {
    // f0 < k < f1  <=>  (unsigned)(k - f0 - 1) < (unsigned)(f1 - f0 - 1)
    const unsigned span = (unsigned)(g.f1 - g.f0 - 1);
    return (unsigned)(s - g.f0 - 1) < span || (unsigned)(e - g.f0 - 1) < span;
}

// OR a run [s, s + len) of at most 32 pixels (0 <= s, s + len <= Rv) into the bitmask: at most
// two words.  The first word's OR is unconditional (an OR of zero for len = 0 changes nothing;
// measured 2-3 % faster steps than testing the mask first), the second is predicated.
__device__ __forceinline__ void raster_short(uint32_t *vb, int s, unsigned len) {
    // len ones (0xffffffff >> (32 - len), none for len = 0) shifted to bit s & 31
    const uint32_t m = __funnelshift_rc(ABM_FULL_MASK, 0u, 32u - len);
    const int w0 = s >> 5, sh = s & 31;
    const uint32_t hi = __funnelshift_l(m, 0u, sh);
    atomicOr(&vb[w0], m << sh);
    if (hi) atomicOr(&vb[w0 + 1], hi);
}

// OR a visible projection [s, e) into the bitmask; the common case (no wrap, at most 32
// pixels) is two predicated shared atomics, the rest goes through raster_projection.
__device__ __forceinline__ void raster_fast(uint32_t *vb, int rv, int s, int e) {
    const unsigned len = (unsigned)(e - s);
    if (s >= 0 && e < rv && len <= 32u) {
        // run mask of `len` ones (0xffffffff >> (32 - len), none for len = 0) shifted to bit
        // s & 31, split over words w0, w0 + 1
        const uint32_t m = __funnelshift_rc(ABM_FULL_MASK, 0u, 32u - len);
        const int w0 = s >> 5, sh = s & 31;
        const uint32_t hi = __funnelshift_l(m, 0u, sh);
        atomicOr(&vb[w0], m << sh);
        if (hi) atomicOr(&vb[w0 + 1], hi);
    } else {
        raster_projection(vb, rv, s, e);
    }
}

// ------------------------------------------------------------------ VSWRM integrals
// For a warp's bitmask vb (raw pixel order), the four fixed-point sums
//   blob_c = sum_k w_k cos(PHI_k) V_k, blob_s likewise, edge_c = sum_k cos(PHI_k) E_k, edge_s
// where w_k are the trapezoid weights of scipy's trapz over PHI and E = dPhi_V_of(V)^2
// (vf_supcalc.py:257-277: forward circular difference, backward when V[0]=1, V[Rv-1]=0).
// Uses sum_k w_k f_k V_k = Q[Rv] V[Rv-1] + sum_{j=1..Rv-1} Q[j] (V[j-1] - V[j]) with Q the
// prefix sums, so only the transitions of V are visited.  The warp lists the transitions in
// `list` (per-warp shared scratch of `cap` >= 32 entries: pixel index | run-start bit 31):
// per group of 32 WPL words each lane takes words g0 + lane + 32u (u < WPL), and one warp
// prefix sum of the lanes' transition counts places every lane's transitions in the list.  The list
// is then split evenly over the lanes, CW entries a lane per round with the table loads issued
// first: about ceil(transitions / (32 CW)) memory latencies per agent.  Result valid in every
// lane.
template <int CW>
struct IntegralAcc {
    long long bc = 0, bs = 0, ec = 0, es = 0;

    __device__ __forceinline__ void consume(const uint32_t *list, int count, const GridDev &g,
                                            int bwd) {
        const int lane = threadIdx.x & 31;
        __syncwarp();
        for (int k0 = 0; k0 < count; k0 += 32 * CW) {
            uint32_t e[CW];
            longlong2 qv[CW], cv[CW];
#pragma unroll
            for (int u = 0; u < CW; ++u) {
                const int k = k0 + 32 * u + lane;
                e[u] = k < count ? list[k] : 0u;
            }
#pragma unroll
            for (int u = 0; u < CW; ++u) {
                // every listed pixel index is >= 1 (pixel 0 is never a transition)
                const int j = (int)(e[u] & 0x7fffffffu);
                qv[u] = j ? __ldg(g.q + j) : make_longlong2(0, 0);
                cv[u] = j ? __ldg(g.cpt + j - 1 + bwd) : make_longlong2(0, 0);
            }
#pragma unroll
            for (int u = 0; u < CW; ++u) {
                if (e[u] >> 31) {   // run starts at j
                    bc -= qv[u].x;
                    bs -= qv[u].y;
                } else {            // run ends at j (or an empty slot: zero)
                    bc += qv[u].x;
                    bs += qv[u].y;
                }
                ec += cv[u].x;
                es += cv[u].y;
            }
        }
        __syncwarp();
    }
};

template <int CW = 4, int WPL = 1>
__device__ __forceinline__ void warp_integrals(const uint32_t *vb, const GridDev &g,
                                               uint32_t *list, int cap, long long &bc,
                                               long long &bs, long long &ec, long long &es) {
    const int lane = threadIdx.x & 31;
    const int rv = g.rv, words = g.words;
    const uint32_t v0 = vb[0] & 1u;
    const uint32_t vl = (vb[(rv - 1) >> 5] >> ((rv - 1) & 31)) & 1u;
    const int bwd = (v0 == 1u && vl == 0u) ? 1 : 0;
    IntegralAcc<CW> acc;
    int fill = 0;   // entries in the list (warp-uniform)
    for (int g0 = 0; g0 < words; g0 += 32 * WPL) {
        uint32_t cur[WPL], D[WPL];
        int c = 0;
#pragma unroll
        for (int u = 0; u < WPL; ++u) {
            const int w = g0 + 32 * u + lane;
            cur[u] = 0u;
            D[u] = 0u;
            if (w < words) {
                cur[u] = vb[w];
                const uint32_t prev = w > 0 ? (vb[w - 1] >> 31) : (cur[u] & 1u);
                D[u] = cur[u] ^ ((cur[u] << 1) | prev);
                if (w == words - 1 && (rv & 31)) D[u] &= (1u << (rv & 31)) - 1u;
            }
            c += __popc(D[u]);
        }
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(ABM_FULL_MASK, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(ABM_FULL_MASK, incl, 31);
        const int first = incl - c;   // this lane's first rank within the group
        for (int done = 0; done < total;) {   // warp-uniform; one pass unless the list fills
            if (fill == cap) {
                acc.consume(list, fill, g, bwd);
                fill = 0;
            }
            const int take = min(total - done, cap - fill);
            if (take == total) {   // the whole group fits: no rank test
                int pos = fill + first;
#pragma unroll
                for (int u = 0; u < WPL; ++u) {
                    const uint32_t base = (uint32_t)(g0 + 32 * u + lane) << 5;
                    for (uint32_t d = D[u]; d; d &= d - 1u) {
                        const int b = __ffs(d) - 1;
                        list[pos++] = (base + b) | (((cur[u] >> b) & 1u) << 31);
                    }
                }
            } else {
                int r = first;
#pragma unroll
                for (int u = 0; u < WPL; ++u) {
                    const uint32_t base = (uint32_t)(g0 + 32 * u + lane) << 5;
                    for (uint32_t d = D[u]; d; d &= d - 1u, ++r) {
                        const int b = __ffs(d) - 1;
                        if (r >= done && r < done + take)
                            list[fill + r - done] = (base + b) | (((cur[u] >> b) & 1u) << 31);
                    }
                }
            }
            fill += take;
            done += take;
        }
    }
    acc.consume(list, fill, g, bwd);
    bc = acc.bc;
    bs = acc.bs;
    ec = acc.ec;
    es = acc.es;
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

// The same sums with each lane walking the transitions of its own words one by one (one table
// latency per transition of the busiest lane).  Fewer instructions than warp_integrals when
// the bitmask has few transitions per word, as in the small swarms of a batched sweep.
__device__ __forceinline__ void warp_integrals_loop(const uint32_t *vb, const GridDev &g,
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

// ------------------------------------------------------------------ double-float sincos
// cos/sin of a float32 angle to ~1e-14 using FP32 arithmetic only (GB300's FP64 pipe is
// ~1/64 of its FP32 rate, and a lane-masked FP64 instruction costs a full warp's time):
// theta = k h + r with h = 2 pi / 1024 (Cody-Waite in double-float), a table of cos/sin(k h)
// (kSinCosTab entries of df pairs, built on the host in FP64), and Taylor series of cos/sin(r)
// for |r| <= pi / 1024 (truncation errors r^7/5040 and r^6/720 below 2e-18).
constexpr int kSinCosTab = 1024;

__device__ __forceinline__ void df_sincos(float theta, const float4 *tab, dfl &c, dfl &s) {
    const float inv_h = 1.629746552e+02f;             // 1024 / (2 pi)
    const dfl H = {6.135923322e-03f, -1.707476105e-10f};      // 2 pi / 1024 in double-float
    const float kf = rintf(theta * inv_h);
    int k = (int)kf;
    dfl r = df_add_f(df_neg(df_add(two_prod(kf, H.hi), two_prod(kf, H.lo))), theta);
    k &= (kSinCosTab - 1);
    const dfl r2 = df_mul(r, r);
    // sin r = r (1 - r2 (1/6 - r2/120)),  cos r = 1 - r2 (1/2 - r2/24)
    const dfl sixth = {1.666666716e-01f, -4.967053879e-09f};
    const dfl s_in = df_sub(sixth, df_mul(r2, dfl{8.333333768e-03f, -4.346172033e-10f}));
    const dfl sr = df_mul(r, df_add_f(df_neg(df_mul(r2, s_in)), 1.f));
    const dfl c_in =
        df_add_f(df_neg(df_mul(r2, dfl{4.166666791e-02f, -1.241763470e-09f})), 0.5f);
    const dfl cr = df_add_f(df_neg(df_mul(r2, c_in)), 1.f);
    const float4 t = tab[k];
    const dfl ck = {t.x, t.y}, sk = {t.z, t.w};
    c = df_sub(df_mul(ck, cr), df_mul(sk, sr));
    s = df_add(df_mul(sk, cr), df_mul(ck, sr));
}

// cos/sin of a double-float angle (same method; the low part joins the reduced argument).
__device__ __forceinline__ void df_sincos_df(dfl theta, const float4 *tab, dfl &c, dfl &s) {
    const float inv_h = 1.629746552e+02f;
    const dfl H = {6.135923322e-03f, -1.707476105e-10f};
    const float kf = rintf(theta.hi * inv_h);
    int k = (int)kf;
    dfl r = df_sub(theta, df_add(two_prod(kf, H.hi), two_prod(kf, H.lo)));
    k &= (kSinCosTab - 1);
    const dfl r2 = df_mul(r, r);
    const dfl sixth = {1.666666716e-01f, -4.967053879e-09f};
    const dfl s_in = df_sub(sixth, df_mul(r2, dfl{8.333333768e-03f, -4.346172033e-10f}));
    const dfl sr = df_mul(r, df_add_f(df_neg(df_mul(r2, s_in)), 1.f));
    const dfl c_in =
        df_add_f(df_neg(df_mul(r2, dfl{4.166666791e-02f, -1.241763470e-09f})), 0.5f);
    const dfl cr = df_add_f(df_neg(df_mul(r2, c_in)), 1.f);
    const float4 t = tab[k];
    const dfl ck = {t.x, t.y}, sk = {t.z, t.w};
    c = df_sub(df_mul(ck, cr), df_mul(sk, sr));
    s = df_add(df_mul(sk, cr), df_mul(ck, sr));
}

// ------------------------------------------------------------------ agent update (double-float)
// The reference's update (vf_agent.py:289-327, agent.py:347-394 / vf_agent.py:188-204) in
// double-float arithmetic on the FP32 pipe, so it can run in the pair kernel's epilogue (one
// lane per agent) without FP64 instructions.  Results are rounded to float32 once at the end.
struct UpdateDf {
    dfl gam, v0, alp0, alp1, bet0, bet1;   // parameters (per-agent overrides replace alp0...)
    dfl max_vel, max_th, dt;
    dfl bx0, bx1, by0, by1;
    int limit, torus, phi_ok;
};

__device__ __forceinline__ dfl df_from_fix(long long v) {   // v * 2^-40 in double-float
    const float hi = (float)v;
    const float lo = (float)(v - (long long)hi);
    return fast_two_sum(hi * 9.094947017729282e-13f, lo * 9.094947017729282e-13f);
}

// Comparisons of normalised double-floats (hi = RN(hi + lo) with ties to even, as every
// double-float here is: the results of fast_two_sum, float values with lo = 0 and the split
// constants).  A value then has one representation, so ordering (hi, lo) lexicographically
// is the sign of the exact difference (the same decision as df_sign(df_sub(a, b)) in three
// instructions instead of ~23).
__device__ __forceinline__ bool df_lt(dfl a, dfl b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool df_le(dfl a, dfl b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}

__device__ __forceinline__ dfl df_prove_orientation(dfl t) {   // agent.py:605-610
    const dfl two_pi = {6.283185482e+00f, -1.748455531e-07f};
    if (df_sign(t) < 0) t = df_add(two_pi, t);
    if (df_lt(two_pi, t)) t = df_sub(t, two_pi);
    return t;
}

struct UpdateOut {
    float x, y, th, v;
    dfl terms[6];   // dvel, dpsi, alpha_blob, alpha_edge, beta_blob, beta_edge
};

__device__ __forceinline__ UpdateOut update_agent_df(const UpdateDf &p, const float4 *sctab,
                                                  float xf, float yf, float thf, float vf,
                                                  float Rf, long long bc, long long bs,
                                                  long long ec, long long es, dfl alp0,
                                                  dfl bet0, dfl v0) {
    const dfl half_pi = {1.570796371e+00f, -4.371138829e-08f};
    const dfl pi = {3.141592741e+00f, -8.742277657e-08f};
    const dfl three_half_pi = {4.712388992e+00f, -1.192488064e-08f};
    const dfl two_pi = {6.283185482e+00f, -1.748455531e-07f};
    const dfl zero = {0.f, 0.f};
    UpdateOut o;
    dfl ab = zero, ae = zero, bb = zero, be = zero, dv = zero, dpsi = zero;
    if (p.phi_ok) {
        ab = df_mul(alp0, df_neg(df_from_fix(bc)));
        ae = df_mul(df_mul(alp0, p.alp1), df_from_fix(ec));
        bb = df_mul(bet0, df_neg(df_from_fix(bs)));
        be = df_mul(df_mul(bet0, p.bet1), df_from_fix(es));
        dv = df_add(df_add(df_mul(p.gam, df_add_f(v0, -vf)), ab), ae);
        dpsi = df_add(bb, be);
    }
    o.terms[0] = dv;
    o.terms[1] = dpsi;
    o.terms[2] = ab;
    o.terms[3] = ae;
    o.terms[4] = bb;
    o.terms[5] = be;
    dfl theta = df_mul(dpsi, p.dt);
    if (p.limit && df_lt(p.max_th, dfl{fabsf(theta.hi), theta.hi < 0 ? -theta.lo : theta.lo}))
        theta = (df_sign(theta) < 0) ? df_neg(p.max_th) : p.max_th;
    dfl th = df_prove_orientation(df_add_f(theta, thf));
    dfl v = df_add_f(df_mul(dv, p.dt), vf);
    if (p.limit && df_lt(p.max_vel, dfl{fabsf(v.hi), v.hi < 0 ? -v.lo : v.lo}))
        v = (df_sign(v) < 0) ? df_neg(p.max_vel) : p.max_vel;
    dfl cs, sn;
    df_sincos_df(th, sctab, cs, sn);
    const dfl vdt = df_mul(v, p.dt);
    dfl x = df_add_f(df_mul(vdt, cs), xf);
    dfl y = df_add_f(df_neg(df_mul(vdt, sn)), yf);
    const dfl cx = df_add_f(x, Rf), cy = df_add_f(y, Rf);
    if (!p.torus) {
        if (df_lt(cx, p.bx0)) {
            x = df_add_f(p.bx0, -Rf);
            if (df_le(half_pi, th) && df_lt(th, pi)) th = df_sub(th, half_pi);
            else if (df_le(pi, th) && df_le(th, three_half_pi)) th = df_add(th, half_pi);
            th = df_prove_orientation(th);
        }
        if (df_lt(p.bx1, cx)) {
            x = df_add_f(df_add_f(p.bx1, -Rf), -1.f);
            if (df_le(three_half_pi, th) && df_lt(th, two_pi)) th = df_sub(th, half_pi);
            else if (df_le(zero, th) && df_le(th, half_pi)) th = df_add(th, half_pi);
            th = df_prove_orientation(th);
        }
        if (df_lt(cy, p.by0)) {
            y = df_add_f(p.by0, -Rf);
            if (df_le(half_pi, th) && df_le(th, pi)) th = df_add(th, half_pi);
            else if (df_le(zero, th) && df_lt(th, half_pi)) th = df_sub(th, half_pi);
            th = df_prove_orientation(th);
        }
        if (df_lt(p.by1, cy)) {
            y = df_add_f(df_add_f(p.by1, -Rf), -1.f);
            if (df_le(three_half_pi, th) && df_le(th, two_pi)) th = df_add(th, half_pi);
            else if (df_le(pi, th) && df_lt(th, three_half_pi)) th = df_sub(th, half_pi);
            th = df_prove_orientation(th);
        }
    } else {
        if (df_lt(cx, p.bx0)) x = df_add_f(p.bx1, -Rf);
        else if (df_lt(p.bx1, cx)) x = df_add_f(p.bx0, Rf);
        if (df_lt(cy, p.by0)) y = df_add_f(p.by1, -Rf);
        else if (df_lt(p.by1, cy)) y = df_add_f(p.by0, Rf);
    }
    o.x = x.hi + x.lo;
    o.y = y.hi + y.lo;
    o.th = th.hi + th.lo;
    o.v = v.hi + v.lo;
    return o;
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
// Bounded wait on an mbarrier phase: at most `polls` try_wait rounds; false when the limit was
// reached (the phase has not completed).
constexpr int kMbarPolls = 1 << 20;

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int polls = kMbarPolls) {
    const uint32_t addr = smem_u32(bar);
    for (int it = 0; it < polls; ++it) {
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

// Bit of the step kernels' status word (vpf_step.cu) set by a block whose bounded wait gave up.
constexpr unsigned kStatusWaitTimeout = 1u;

}  // namespace abm
