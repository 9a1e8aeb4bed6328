/*
 * vpf_oracle.c -- FP64 CPU restatement of the scioip34/ABM visual-flocking hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the smoke check and
 * the CPU-baseline leg of bench.py load it to check (and time) the CUDA library.  Nothing in
 * the product path links it or falls back to it.
 *
 * Every function restates one reference function step by step in IEEE double precision, in
 * the same operation order numpy uses, so that the oracle reproduces the reference's discrete
 * decisions (pixel indices, projection widths, wrap rules) and its floating-point results to
 * within a few ulps.  The pinning evidence is tests/golden/: fixtures produced by running the
 * reference itself, plus the reference's own known-answer test vectors.
 *
 * Compile with -ffp-contract=off (no FMA contraction) so results are the same on x86-64 and
 * aarch64 hosts.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793

/* ---------------------------------------------------------------- numpy helpers */

/* np.linspace(start, stop, n): y = arange(n) * step; y += start; y[-1] = stop. */
void orc_linspace(double start, double stop, int n, double *out)
{
    if (n <= 0) return;
    if (n == 1) { out[0] = start; return; }
    double delta = stop - start;
    double step = delta / (double)(n - 1);
    for (int k = 0; k < n; ++k) {
        double y = (double)k * step;
        out[k] = y + start;
    }
    out[n - 1] = stop;
}

/* np.arange(start, stop, step) for doubles: length ceil((stop-start)/step); a[0] = start,
 * a[1] = start + step, a[i] = start + i * (a[1] - a[0]) (numpy's DOUBLE_fill). Returns the
 * length; writes at most cap values. */
int orc_arange(double start, double stop, double step, double *out, int cap)
{
    double len_d = ceil((stop - start) / step);
    int len = len_d > 0 ? (int)len_d : 0;
    if (len <= 0) return 0;
    double a0 = start, a1 = start + step;
    double delta = a1 - a0;
    for (int i = 0; i < len && i < cap; ++i) {
        if (i == 0) out[i] = a0;
        else if (i == 1) out[i] = a1;
        else out[i] = a0 + (double)i * delta;
    }
    return len;
}

/* supcalc.find_nearest (abm/agent/supcalc.py:8-11): argmin |array - value|, first index on
 * ties; a NaN value makes every difference NaN and numpy's argmin returns index 0. */
int orc_find_nearest(const double *arr, int n, double value)
{
    if (isnan(value)) return 0;
    /* two passes (minimum, then its first index) so the O(n) scan vectorises */
    double bv = fabs(arr[0] - value);
    for (int k = 1; k < n; ++k) {
        double d = fabs(arr[k] - value);
        bv = d < bv ? d : bv;
    }
    for (int k = 0; k < n; ++k)
        if (fabs(arr[k] - value) == bv) return k;
    return 0;
}

/* numpy float remainder (npy_divmod): fmod, then shift into the divisor's sign. */
static double np_remainder(double a, double b)
{
    double mod = fmod(a, b);
    if (mod != 0.0) {
        if ((b < 0) != (mod < 0)) mod += b;
    } else {
        mod = copysign(0.0, b);
    }
    return mod;
}

/* Fill out[a:b] = value with numpy slice semantics (negative indices count from the end,
 * then clamp to [0, n]). */
static void np_fill(double *row, int n, long long a, long long b, double value)
{
    if (a < 0) { a += n; if (a < 0) a = 0; }
    if (b < 0) { b += n; if (b < 0) b = 0; }
    if (a > n) a = n;
    if (b > n) b = n;
    for (long long k = a; k < b; ++k) row[k] = value;
}

/* ---------------------------------------------------------------- geometry */

/* supcalc.angle_between (abm/agent/supcalc.py:14-34). */
double orc_angle_between(double v1x, double v1y, double v2x, double v2y)
{
    double n1 = sqrt(v1x * v1x + v1y * v1y);
    double u1x = v1x / n1, u1y = v1y / n1;
    double n2 = sqrt(v2x * v2x + v2y * v2y);
    double u2x = v2x / n2, u2y = v2y / n2;
    double dot = u1x * u2x + u1y * u2y;
    if (dot < -1.0) dot = -1.0;          /* np.clip keeps NaN */
    if (dot > 1.0) dot = 1.0;
    double angle = acos(dot);
    if (u1x * u2y - u1y * u2x < 0) angle = -angle;
    return angle;
}

/* vf_supcalc.calculate_closed_angle (vf_supcalc.py:142-158): 0 <= c <= pi is inclusive. */
double orc_closed_angle_vf(double v1x, double v1y, double v2x, double v2y)
{
    double c = np_remainder(orc_angle_between(v1x, v1y, v2x, v2y), 2 * ORC_PI);
    if (0 <= c && c <= ORC_PI) return -c;
    return 2 * ORC_PI - c;
}

/* Agent.projection_field's inline closed angle (agent.py:515-523): 0 < c < pi is strict. */
double orc_closed_angle_agent(double v1x, double v1y, double v2x, double v2y)
{
    double c = np_remainder(orc_angle_between(v1x, v1y, v2x, v2y), 2 * ORC_PI);
    if (0 < c && c < ORC_PI) return -c;
    return 2 * ORC_PI - c;
}

/* Decision margin (radians) of a bearing `ca` and half visual angle `half` on a linspace grid
 * of Rv pixels: distance of `ca` to the nearest argmin switch (midpoints between grid
 * points, and the +-pi seam) and of `half` to the nearest floor(proj_size/2) switch
 * (half = 2*pi*k/Rv).  The tests excuse pixels of pairs whose margin is below 1e-9 rad. */
static double decision_margin(const double *phis, int Rv, int t, double ca, double half)
{
    double m = INFINITY;
    if (t + 1 < Rv) m = fmin(m, fabs(ca - 0.5 * (phis[t] + phis[t + 1])));
    if (t >= 1) m = fmin(m, fabs(ca - 0.5 * (phis[t - 1] + phis[t])));
    m = fmin(m, ORC_PI - fabs(ca));
    double unit = 2 * ORC_PI / Rv;
    double k = floor(half / unit);
    m = fmin(m, fabs(half - k * unit));
    m = fmin(m, fabs((k + 1) * unit - half));
    return m;
}

/* The pixel decisions of one object (vf_supcalc.py:55-117): the bearing `ca`, the half visual
 * angle `half` = vis / 2, the nearest linspace pixel t and h = floor(proj_size / 2).  Returns 0
 * when the object is skipped (same top-left position, :57-58, or beyond vision_range). */
typedef struct {
    double ca, half;
    long long t, h;
} PairDecision;

static int pair_decision(const double *phis, int Rv, double acx, double acy, double v1x,
                         double v1y, double px, double py, double ox, double oy, double size,
                         int infinite, double W, double H, double vision_range, PairDecision *d)
{
    if (ox == px && oy == py) return 0;
    double ocx = ox + size, ocy = oy + size;
    double v2x = ocx - acx, v2y = ocy - acy;
    if (infinite) {
        if (fabs(v2x) > W / 2) {
            if (acx < ocx) ocx -= W;
            else if (acx > ocx) ocx += W;
        }
        if (fabs(v2y) > H / 2) {
            if (acy < ocy) ocy -= H;
            else if (acy > ocy) ocy += H;
        }
        v2x = ocx - acx;
        v2y = ocy - acy;
    }
    double ca = orc_closed_angle_vf(v1x, v1y, v2x, v2y);
    double dx = ocx - acx, dy = ocy - acy;
    double dist = sqrt(dx * dx + dy * dy);
    if (!isnan(vision_range) && dist > vision_range) return 0;
    double vis = 2 * atan(size / (1 * dist));
    int t = orc_find_nearest(phis, Rv, ca);
    double ps = (vis / (2 * ORC_PI)) * Rv;
    d->ca = ca;
    d->half = vis / 2;
    d->t = t;
    d->h = (long long)floor(ps / 2);
    return 1;
}

/* The runs a decision (t, h) contributes to the raw (unflipped) row (vf_supcalc.py:114-129):
 * up to three [a, b) slices in numpy slice semantics; returns the number written (0 when the
 * projection is not visible). */
static int runs_of(int Rv, int f0, int f1, long long t, long long h, long long runs[6])
{
    long long s = t - h, e = t + h;
    int nr = 0;
    if ((f0 < s && s < f1) || (f0 < e && e < f1)) {
        if (s < 0) { runs[2 * nr] = Rv + s; runs[2 * nr + 1] = Rv; ++nr; s = 0; }
        if (e >= Rv) { runs[2 * nr] = 0; runs[2 * nr + 1] = e - (Rv - 1); ++nr; e = Rv; }
        runs[2 * nr] = s; runs[2 * nr + 1] = e; ++nr;
    }
    return nr;
}

/* The runs one object contributes to the raw (unflipped) row and its decision margin (both
 * used by the dense-row and the union forms below). */
static int projection_runs(const double *phis, int Rv, int f0, int f1, double acx, double acy,
                           double v1x, double v1y, double px, double py, double ox, double oy,
                           double size, int infinite, double W, double H, double vision_range,
                           long long runs[6], double *margin)
{
    if (margin) *margin = INFINITY;
    PairDecision d;
    if (!pair_decision(phis, Rv, acx, acy, v1x, v1y, px, py, ox, oy, size, infinite, W, H,
                       vision_range, &d))
        return 0;
    if (margin) *margin = decision_margin(phis, Rv, (int)d.t, d.ca, d.half);
    return runs_of(Rv, f0, f1, d.t, d.h, runs);
}

static void fill_runs_u8(uint8_t *row, int Rv, const long long runs[6], int nr)
{
    for (int r = 0; r < nr; ++r) {
        long long a = runs[2 * r], b = runs[2 * r + 1];
        if (a < 0) { a += Rv; if (a < 0) a = 0; }      /* numpy slice semantics */
        if (b < 0) { b += Rv; if (b < 0) b = 0; }
        if (a > Rv) a = Rv;
        if (b > Rv) b = Rv;
        for (long long k = a; k < b; ++k) row[k] = 1;
    }
}

/* Pixels (raw order) that a pair within `band` rad of a decision boundary can flip: the
 * symmetric differences between the row of the decision taken and the rows of its
 * alternatives -- t moved across a midpoint (or across the +-pi seam, pixel 0 <-> Rv-1) that
 * the bearing lies within `band` of, h moved across a floor(proj_size/2) switch that the half
 * angle lies within `band` of, and both.  OR-ed into `excuse` (Rv bytes); `work` holds 2 Rv
 * bytes of scratch.  Returns 1 when the pair is near a boundary. */
static int pair_alternatives(const double *phis, int Rv, int f0, int f1, const PairDecision *d,
                             double band, uint8_t *excuse, uint8_t *work)
{
    long long ts[3] = {d->t, -1, -1}, hs[3] = {d->h, -1, -1};
    int nt = 1, nh = 1;
    const long long t = d->t;
    if (t + 1 < Rv && fabs(d->ca - 0.5 * (phis[t] + phis[t + 1])) < band) ts[nt++] = t + 1;
    if (t >= 1 && fabs(d->ca - 0.5 * (phis[t - 1] + phis[t])) < band) ts[nt++] = t - 1;
    if (ORC_PI - fabs(d->ca) < band && (t == 0 || t == Rv - 1) && nt < 3)
        ts[nt++] = Rv - 1 - t;
    const double unit = 2 * ORC_PI / Rv;
    if (d->h >= 1 && fabs(d->half - (double)d->h * unit) < band) hs[nh++] = d->h - 1;
    if (fabs((double)(d->h + 1) * unit - d->half) < band) hs[nh++] = d->h + 1;
    if (nt == 1 && nh == 1) return 0;
    uint8_t *a = work, *b = work + Rv;
    long long runs[6];
    memset(a, 0, (size_t)Rv);
    fill_runs_u8(a, Rv, runs, runs_of(Rv, f0, f1, d->t, d->h, runs));
    for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nh; ++j) {
            if (i == 0 && j == 0) continue;
            memset(b, 0, (size_t)Rv);
            fill_runs_u8(b, Rv, runs, runs_of(Rv, f0, f1, ts[i], hs[j], runs));
            for (int k = 0; k < Rv; ++k) excuse[k] |= (uint8_t)(a[k] ^ b[k]);
        }
    return 1;
}

/* OR of all objects' rows in raw pixel order (calc_soc_v_proj's sum + binarise,
 * vf_agent.py:233-236, without materialising the n x Rv rows).  excuse (nullable, Rv bytes):
 * the pixels that objects within `band` rad of a decision boundary can flip
 * (pair_alternatives), their count in *near. */
void orc_projection_union_ex(double fov0, double fov1, int Rv, double px, double py,
                             double radius, double orientation, int n, const double *obj_xy,
                             const double *obj_sizes, int infinite, double W, double H, double *V,
                             double *margins, double band, uint8_t *excuse, int *near)
{
    double *phis = (double *)malloc(sizeof(double) * (size_t)Rv);
    uint8_t *work = excuse ? (uint8_t *)malloc(2 * (size_t)Rv) : NULL;
    orc_linspace(-ORC_PI, ORC_PI, Rv, phis);
    int f0 = orc_find_nearest(phis, Rv, fov0), f1 = orc_find_nearest(phis, Rv, fov1);
    double acx = px + radius, acy = py + radius;
    double aex = px + (1 + cos(orientation)) * radius;
    double aey = py + (1 - sin(orientation)) * radius;
    double v1x = aex - acx, v1y = aey - acy;
    for (int k = 0; k < Rv; ++k) V[k] = 0.0;
    if (excuse) memset(excuse, 0, (size_t)Rv);
    int cnt = 0;
    for (int i = 0; i < n; ++i) {
        long long runs[6];
        PairDecision d;
        if (margins) margins[i] = INFINITY;
        if (!pair_decision(phis, Rv, acx, acy, v1x, v1y, px, py, obj_xy[2 * i],
                           obj_xy[2 * i + 1], obj_sizes ? obj_sizes[i] : radius, infinite, W, H,
                           NAN, &d))
            continue;
        if (margins) margins[i] = decision_margin(phis, Rv, (int)d.t, d.ca, d.half);
        int nr = runs_of(Rv, f0, f1, d.t, d.h, runs);
        for (int r = 0; r < nr; ++r) np_fill(V, Rv, runs[2 * r], runs[2 * r + 1], 1.0);
        if (excuse) cnt += pair_alternatives(phis, Rv, f0, f1, &d, band, excuse, work);
    }
    if (near) *near = cnt;
    free(work);
    free(phis);
}

void orc_projection_union(double fov0, double fov1, int Rv, double px, double py, double radius,
                          double orientation, int n, const double *obj_xy,
                          const double *obj_sizes, int infinite, double W, double H,
                          double *V, double *margins)
{
    orc_projection_union_ex(fov0, fov1, Rv, px, py, radius, orientation, n, obj_xy, obj_sizes,
                            infinite, W, H, V, margins, 0.0, NULL, NULL);
}

/*
 * vf_supcalc.projection_field (vf_supcalc.py:20-138).
 * obj_xy: n objects as (x, y) top-left positions; obj_sizes may be NULL (use `radius`).
 * infinite != 0 selects the torus minimal image (boundary_cond == "infinite").
 * vision_range: NaN means None.
 * out: n x Rv rows, flipped along the pixel axis like the reference's return value.
 * margins (nullable): per object, the decision margin in radians (INFINITY when skipped).
 */
void orc_projection_field(double fov0, double fov1, int Rv, double px, double py, double radius,
                          double orientation, int n, const double *obj_xy, const double *obj_sizes,
                          int infinite, double W, double H, double vision_range, double *out,
                          double *margins)
{
    double *phis = (double *)malloc(sizeof(double) * (size_t)Rv);
    double *raw = (double *)malloc(sizeof(double) * (size_t)Rv);
    orc_linspace(-ORC_PI, ORC_PI, Rv, phis);
    /* fov_px (vf_supcalc.py:105) */
    int f0 = orc_find_nearest(phis, Rv, fov0), f1 = orc_find_nearest(phis, Rv, fov1);
    double acx = px + radius, acy = py + radius;
    double aex = px + (1 + cos(orientation)) * radius;
    double aey = py + (1 - sin(orientation)) * radius;
    double v1x = aex - acx, v1y = aey - acy;
    for (int i = 0; i < n; ++i) {
        long long runs[6];
        for (int k = 0; k < Rv; ++k) raw[k] = 0.0;
        int nr = projection_runs(phis, Rv, f0, f1, acx, acy, v1x, v1y, px, py, obj_xy[2 * i],
                                 obj_xy[2 * i + 1], obj_sizes ? obj_sizes[i] : radius, infinite,
                                 W, H, vision_range, runs, margins ? &margins[i] : NULL);
        for (int r = 0; r < nr; ++r) np_fill(raw, Rv, runs[2 * r], runs[2 * r + 1], 1.0);
        /* np.flip(v_field, axis=1) (vf_supcalc.py:134) */
        for (int k = 0; k < Rv; ++k) out[(size_t)i * Rv + k] = raw[Rv - 1 - k];
    }
    free(raw);
    free(phis);
}

/*
 * Excuse rows of projection_field's objects: for every object whose pixel decisions lie
 * within `band` rad of a boundary, the pixels its alternative decisions would flip
 * (pair_alternatives).  per_object != 0: one row per object, flipped like projection_field's
 * rows (n x Rv bytes); otherwise the OR over all objects in raw pixel order (Rv bytes), the
 * mask that applies to calc_soc_v_proj's union.  near: per object, 1 when near a boundary
 * (nullable).  Same arguments as orc_projection_field otherwise.
 */
void orc_projection_excuse(double fov0, double fov1, int Rv, double px, double py, double radius,
                           double orientation, int n, const double *obj_xy,
                           const double *obj_sizes, int infinite, double W, double H,
                           double vision_range, double band, int per_object, uint8_t *excuse,
                           int *near)
{
    double *phis = (double *)malloc(sizeof(double) * (size_t)Rv);
    uint8_t *work = (uint8_t *)malloc(3 * (size_t)Rv);
    uint8_t *row = work + 2 * (size_t)Rv;
    orc_linspace(-ORC_PI, ORC_PI, Rv, phis);
    int f0 = orc_find_nearest(phis, Rv, fov0), f1 = orc_find_nearest(phis, Rv, fov1);
    double acx = px + radius, acy = py + radius;
    double aex = px + (1 + cos(orientation)) * radius;
    double aey = py + (1 - sin(orientation)) * radius;
    double v1x = aex - acx, v1y = aey - acy;
    if (!per_object) memset(excuse, 0, (size_t)Rv);
    for (int i = 0; i < n; ++i) {
        PairDecision d;
        int nb = 0;
        if (per_object) memset(row, 0, (size_t)Rv);
        if (pair_decision(phis, Rv, acx, acy, v1x, v1y, px, py, obj_xy[2 * i],
                          obj_xy[2 * i + 1], obj_sizes ? obj_sizes[i] : radius, infinite, W, H,
                          vision_range, &d))
            nb = pair_alternatives(phis, Rv, f0, f1, &d, band, per_object ? row : excuse, work);
        if (near) near[i] = nb;
        if (per_object)
            for (int k = 0; k < Rv; ++k) excuse[(size_t)i * Rv + k] = row[Rv - 1 - k];
    }
    free(work);
    free(phis);
}

/* ---------------------------------------------------------------- VSWRM */

/* vf_supcalc.dPhi_V_of (vf_supcalc.py:257-277). */
void orc_dphi_v(const double *V, int n, double *out)
{
    /* raw = diff(wrap-pad(V, 1)): raw[0] = V[0]-V[n-1]; raw[k] = V[k]-V[k-1]; raw[n] = raw[0] */
    double r0 = V[0] - V[n - 1];
    int backward = (r0 > 0) && (r0 > 0);
    for (int k = 0; k < n; ++k) {
        if (backward) out[k] = (k == 0) ? r0 : V[k] - V[k - 1];
        else out[k] = (k == n - 1) ? r0 : V[k + 1] - V[k];
    }
}

static double trapz(const double *y, const double *x, int n)
{
    double s = 0.0;
    for (int k = 0; k + 1 < n; ++k) s += ((x[k + 1] - x[k]) * (y[k + 1] + y[k])) / 2.0;
    return s;
}

/*
 * vf_supcalc.VSWRM_flocking_state_variables (vf_supcalc.py:161-254), verbose form.
 * prm = {GAM, V0, ALP0, ALP1, ALP2, BET0, BET1, BET2}; alp0/bet0/v0 override when not NaN
 * (the per-agent ALP0/BET0/V0 arguments).  out = {dvel, dpsi, alpha_blob, alpha_edge,
 * beta_blob, beta_edge}.
 */
void orc_vswrm(double vel, const double *Phi, const double *V, int n, const double *prm,
               double alp0, double bet0, double v0, double *out)
{
    double GAM = prm[0], ALP1 = prm[3], ALP2 = prm[4], BET1 = prm[6], BET2 = prm[7];
    double ALP0 = isnan(alp0) ? prm[2] : alp0;
    double BET0 = isnan(bet0) ? prm[5] : bet0;
    double V0 = isnan(v0) ? prm[1] : v0;
    double *dphi = (double *)malloc(sizeof(double) * (size_t)n);
    double *yc = (double *)malloc(sizeof(double) * (size_t)n);
    double *ys = (double *)malloc(sizeof(double) * (size_t)n);
    orc_dphi_v(V, n, dphi);
    double ecos = 0.0, esin = 0.0;
    for (int k = 0; k < n; ++k) {
        double gv = -V[k] + ALP2 * 0.0;
        double gp = -V[k] + BET2 * 0.0;
        double sp = dphi[k] * dphi[k];
        yc[k] = cos(Phi[k]) * gv;
        ys[k] = sin(Phi[k]) * gp;
        ecos += cos(Phi[k]) * sp;
        esin += sin(Phi[k]) * sp;
    }
    double alpha_blob = ALP0 * trapz(yc, Phi, n);
    double alpha_edge = ALP0 * ALP1 * ecos;
    double beta_blob = BET0 * trapz(ys, Phi, n);
    double beta_edge = BET0 * BET1 * esin;
    out[0] = GAM * (V0 - vel) + alpha_blob + alpha_edge;
    out[1] = beta_blob + beta_edge;
    out[2] = alpha_blob;
    out[3] = alpha_edge;
    out[4] = beta_blob;
    out[5] = beta_edge;
    free(dphi);
    free(yc);
    free(ys);
}

/* ---------------------------------------------------------------- agent update */

/* Agent.prove_orientation (agent.py:605-610). */
static double prove_orientation(double th)
{
    if (th < 0) th = 2 * ORC_PI + th;
    if (th > ORC_PI * 2) th = th - 2 * ORC_PI;
    return th;
}

static double np_sign_nonzero(double a) { return a > 0 ? 1.0 : (a < 0 ? -1.0 : 1.0); }

/*
 * Simulation parameters, one double array (mirrors abm_vf_params of include/abm_vpf.h):
 *  [0] GAM [1] V0 [2] ALP0 [3] ALP1 [4] ALP2 [5] BET0 [6] BET1 [7] BET2
 *  [8] boundary (0 walls, 1 infinite) [9] limit_movement [10] max_vel [11] max_th
 *  [12] width [13] height [14] window_pad [15] fov0 [16] fov1 [17] Rv [18] radius [19] dt
 */
enum { P_GAM, P_V0, P_ALP0, P_ALP1, P_ALP2, P_BET0, P_BET1, P_BET2, P_BOUNDARY, P_LIMIT,
       P_MAXVEL, P_MAXTH, P_W, P_H, P_PAD, P_FOV0, P_FOV1, P_RV, P_RADIUS, P_DT, P_COUNT };

/* VFAgent.update_agent_position (vf_agent.py:289-309) with prove_turning/prove_velocity
 * (:311-327), then reflect_from_walls (agent.py:347-394) or teleport_infinite_arena
 * (vf_agent.py:188-204).  dt scales the increments (dt = 1 is the reference). */
static void update_agent(const double *P, double R, double dpsi, double dv, double *x, double *y,
                         double *th, double *v)
{
    double dt = P[P_DT];
    double theta = dpsi * dt;
    if (P[P_LIMIT] != 0) {
        if (fabs(theta) > P[P_MAXTH]) theta = P[P_MAXTH] * np_sign_nonzero(theta);
    }
    *th += theta;
    *th = prove_orientation(*th);
    *v += dv * dt;
    if (P[P_LIMIT] != 0) {
        if (fabs(*v) > P[P_MAXVEL]) *v = P[P_MAXVEL] * np_sign_nonzero(*v);
    }
    double nx = *x + (*v * dt) * cos(*th);
    double ny = *y - (*v * dt) * sin(*th);
    *x = nx;
    *y = ny;

    double pad = P[P_PAD];
    double bx0 = pad, bx1 = pad + P[P_W], by0 = pad, by1 = pad + P[P_H];
    double cx = *x + R, cy = *y + R;
    if (P[P_BOUNDARY] == 0) {
        if (cx < bx0) {
            *x = bx0 - R;
            if (ORC_PI / 2 <= *th && *th < ORC_PI) *th -= ORC_PI / 2;
            else if (ORC_PI <= *th && *th <= 3 * ORC_PI / 2) *th += ORC_PI / 2;
            *th = prove_orientation(*th);
        }
        if (cx > bx1) {
            *x = bx1 - R - 1;
            if (3 * ORC_PI / 2 <= *th && *th < 2 * ORC_PI) *th -= ORC_PI / 2;
            else if (0 <= *th && *th <= ORC_PI / 2) *th += ORC_PI / 2;
            *th = prove_orientation(*th);
        }
        if (cy < by0) {
            *y = by0 - R;
            if (ORC_PI / 2 <= *th && *th <= ORC_PI) *th += ORC_PI / 2;
            else if (0 <= *th && *th < ORC_PI / 2) *th -= ORC_PI / 2;
            *th = prove_orientation(*th);
        }
        if (cy > by1) {
            *y = by1 - R - 1;
            if (3 * ORC_PI / 2 <= *th && *th <= 2 * ORC_PI) *th += ORC_PI / 2;
            else if (ORC_PI <= *th && *th < 3 * ORC_PI / 2) *th -= ORC_PI / 2;
            *th = prove_orientation(*th);
        }
    } else {
        if (cx < bx0) *x = bx1 - R;
        else if (cx > bx1) *x = bx0 + R;
        if (cy < by0) *y = by1 - R;
        else if (cy > by1) *y = by0 + R;
    }
}

/* One agent's perception + VSWRM + update from the positions in (x, y). Writes the raw
 * (unflipped) OR-ed VPF into vraw (Rv bytes) when given, the six VSWRM terms, and the new
 * state into the *_new outputs. */
static void agent_step(int i, int n, const double *x, const double *y, const double *th,
                       const double *v, const double *radii, const double *P,
                       const double *alp0_i, const double *bet0_i, const double *v0_i,
                       double *xn, double *yn, double *thn, double *vn, uint8_t *vraw,
                       double *terms, double *margins_row, int *phi_mismatch, double band,
                       uint8_t *excuse, int *near)
{
    int Rv = (int)P[P_RV];
    double R = radii ? radii[i] : P[P_RADIUS];
    double *objs = (double *)malloc(sizeof(double) * 2 * (size_t)(n > 1 ? n - 1 : 1));
    double *sizes = (double *)malloc(sizeof(double) * (size_t)(n > 1 ? n - 1 : 1));
    double *marg = (double *)malloc(sizeof(double) * (size_t)(n > 1 ? n - 1 : 1));
    double *V = (double *)calloc((size_t)Rv, sizeof(double));
    int m = 0;
    for (int j = 0; j < n; ++j) {
        if (j == i) continue;               /* agents_of_interest excludes self by id */
        objs[2 * m] = x[j];
        objs[2 * m + 1] = y[j];
        sizes[m] = radii ? radii[j] : P[P_RADIUS];
        ++m;
    }
    /* calc_soc_v_proj (vf_agent.py:216-237): sum of the flipped rows, binarised; VSWRM gets
     * np.flip of that field, i.e. the OR of the rows in raw pixel order. */
    orc_projection_union_ex(P[P_FOV0], P[P_FOV1], Rv, x[i], y[i], R, th[i], m, objs, sizes,
                            P[P_BOUNDARY] != 0, P[P_W], P[P_H], V, marg, band, excuse, near);
    if (vraw)
        for (int k = 0; k < Rv; ++k) vraw[k] = V[k] > 0;
    if (margins_row) {
        int r = 0;
        for (int j = 0; j < n; ++j) {
            if (j == i) { margins_row[j] = INFINITY; continue; }
            margins_row[j] = marg[r++];
        }
    }

    double PHI[8192 + 8];
    int nphi = orc_arange(-ORC_PI, ORC_PI, (2 * ORC_PI) / Rv, PHI, 8192 + 8);
    double out[6] = {0, 0, 0, 0, 0, 0};
    double dv = 0, dpsi = 0;
    if (nphi == Rv) {
        orc_vswrm(v[i], PHI, V, Rv, P, alp0_i ? alp0_i[i] : NAN, bet0_i ? bet0_i[i] : NAN,
                  v0_i ? v0_i[i] : NAN, out);
        dv = out[0];
        dpsi = out[1];
    } else if (phi_mismatch) {
        *phi_mismatch = 1;   /* vf_agent.py:283-284: dv = dphi = 0 with a printed warning */
    }
    if (terms) memcpy(terms, out, sizeof(out));
    double nx = x[i], ny = y[i], nth = th[i], nv = v[i];
    update_agent(P, R, dpsi, dv, &nx, &ny, &nth, &nv);
    *xn = nx;
    *yn = ny;
    *thn = nth;
    *vn = nv;
    free(objs);
    free(sizes);
    free(marg);
    free(V);
}

/*
 * One simulation step of all n agents (VFSimulation.step_sim, vf_sims.py:291-340, with
 * agents.update at :302).  sequential = 1 reproduces pygame's Group.update order (agent i
 * sees the already-moved positions of agents < i); sequential = 0 is the snapshot (Jacobi)
 * form that the GPU kernels implement.  vraw: n x Rv bytes (nullable); terms: n x 6
 * (nullable); margins: n x n decision margins (nullable); excuse: n x Rv bytes (nullable),
 * per agent the pixels (raw order) that its pairs within `band` rad of a pixel / width
 * decision boundary can flip, with the number of such pairs in near[i].  Returns 1 when
 * len(PHI) != Rv.
 */
int orc_vf_step_ex(int n, const double *x, const double *y, const double *th, const double *v,
                   const double *radii, const double *P, const double *alp0_i,
                   const double *bet0_i, const double *v0_i, int sequential, double *x_out,
                   double *y_out, double *th_out, double *v_out, uint8_t *vraw, double *terms,
                   double *margins, double band, uint8_t *excuse, int *near)
{
    int Rv = (int)P[P_RV];
    int mismatch = 0;
    if (sequential) {
        double *cx = (double *)malloc(sizeof(double) * (size_t)n);
        double *cy = (double *)malloc(sizeof(double) * (size_t)n);
        double *ct = (double *)malloc(sizeof(double) * (size_t)n);
        double *cv = (double *)malloc(sizeof(double) * (size_t)n);
        memcpy(cx, x, sizeof(double) * (size_t)n);
        memcpy(cy, y, sizeof(double) * (size_t)n);
        memcpy(ct, th, sizeof(double) * (size_t)n);
        memcpy(cv, v, sizeof(double) * (size_t)n);
        for (int i = 0; i < n; ++i) {
            double a, b, c, d;
            agent_step(i, n, cx, cy, ct, cv, radii, P, alp0_i, bet0_i, v0_i, &a, &b, &c, &d,
                       vraw ? vraw + (size_t)i * Rv : NULL, terms ? terms + 6 * (size_t)i : NULL,
                       margins ? margins + (size_t)i * n : NULL, &mismatch, band,
                       excuse ? excuse + (size_t)i * Rv : NULL, near ? near + i : NULL);
            cx[i] = a; cy[i] = b; ct[i] = c; cv[i] = d;
        }
        memcpy(x_out, cx, sizeof(double) * (size_t)n);
        memcpy(y_out, cy, sizeof(double) * (size_t)n);
        memcpy(th_out, ct, sizeof(double) * (size_t)n);
        memcpy(v_out, cv, sizeof(double) * (size_t)n);
        free(cx); free(cy); free(ct); free(cv);
    } else {
#pragma omp parallel for schedule(dynamic, 1) reduction(| : mismatch)
        for (int i = 0; i < n; ++i) {
            int mm = 0;
            agent_step(i, n, x, y, th, v, radii, P, alp0_i, bet0_i, v0_i, &x_out[i], &y_out[i],
                       &th_out[i], &v_out[i], vraw ? vraw + (size_t)i * Rv : NULL,
                       terms ? terms + 6 * (size_t)i : NULL,
                       margins ? margins + (size_t)i * n : NULL, &mm, band,
                       excuse ? excuse + (size_t)i * Rv : NULL, near ? near + i : NULL);
            mismatch |= mm;
        }
    }
    return mismatch;
}

int orc_vf_step(int n, const double *x, const double *y, const double *th, const double *v,
                const double *radii, const double *P, const double *alp0_i,
                const double *bet0_i, const double *v0_i, int sequential, double *x_out,
                double *y_out, double *th_out, double *v_out, uint8_t *vraw, double *terms,
                double *margins)
{
    return orc_vf_step_ex(n, x, y, th, v, radii, P, alp0_i, bet0_i, v0_i, sequential, x_out,
                          y_out, th_out, v_out, vraw, terms, margins, 0.0, NULL, NULL);
}

/* Snapshot step restricted to focal agents [i0, i1) (the bounded CPU-baseline sample). */
int orc_vf_step_range(int n, int i0, int i1, const double *x, const double *y, const double *th,
                      const double *v, const double *radii, const double *P, double *x_out,
                      double *y_out, double *th_out, double *v_out)
{
    int mismatch = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : mismatch)
    for (int i = i0; i < i1; ++i) {
        int mm = 0;
        agent_step(i, n, x, y, th, v, radii, P, NULL, NULL, NULL, &x_out[i], &y_out[i],
                   &th_out[i], &v_out[i], NULL, NULL, NULL, &mm, 0.0, NULL, NULL);
        mismatch |= mm;
    }
    return mismatch;
}

/* numpy's pairwise summation of float64 (the add reduction's inner loop, numpy
 * _core/src/umath/loops_utils.h.src: pairwise_sum): below 8 elements a plain loop, up to 128
 * eight interleaved accumulators combined as ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)) followed
 * by the remainder, above that the two halves split at a multiple of 8.  a[k * stride]. */
static double np_pairwise_sum(const double *a, long long n, long long stride)
{
    if (n < 8) {
        double res = 0.0;
        for (long long k = 0; k < n; ++k) res += a[k * stride];
        return res;
    }
    if (n <= 128) {
        double r[8];
        for (int j = 0; j < 8; ++j) r[j] = a[j * stride];
        long long k;
        for (k = 8; k < n - (n % 8); k += 8)
            for (int j = 0; j < 8; ++j) r[j] += a[(k + j) * stride];
        double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; k < n; ++k) res += a[k * stride];
        return res;
    }
    long long n2 = n / 2;
    n2 -= n2 % 8;
    return np_pairwise_sum(a, n2, stride) + np_pairwise_sum(a + n2 * stride, n - n2, stride);
}

/* np.mean of a float64 view: (0 + pairwise sum) / n; NaN for an empty view. */
static double np_mean(const double *a, long long n, long long stride)
{
    if (n <= 0) return NAN;
    return (0.0 + np_pairwise_sum(a, n, stride)) / (double)n;
}

double orc_np_mean(const double *a, long long n, long long stride) { return np_mean(a, n, stride); }

int orc_num_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Threads of the OpenMP loops from now on (for timing on one core). */
void orc_set_threads(int n)
{
#ifdef _OPENMP
    extern void omp_set_num_threads(int);
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

/* ---------------------------------------------------------------- foraging social channel */

/*
 * Agent.projection_field (agent.py:457-597).
 * obs_xy: n_obs obstacle top-left positions, the first n_social of them social cues and the
 * rest (present only when has_non_social) non-social occluders.  Every obstacle centre uses
 * the focal radius R (agent.py:504-505).  visual_exclusion applies the distance-ordered
 * interval trimming of exlude_V_source_data (agent.py:421-445).  The surviving social
 * intervals are filled in the order of rank_V_source_data("vis_angle") (agent.py:599-603: a
 * stable sort by visual angle, descending); with keep_distance_info the main run of each
 * interval is set to 1 - distance / vision_range, where `distance` is the loop variable of
 * the obstacle loop, i.e. the distance of the LAST non-coincident obstacle (agent.py:526,
 * :584-586), while the wrapped parts are set to 1 (agent.py:576-582).  out: Rv values, flipped
 * and FOV-masked like the reference's return value.
 */
static void agent_projection_core(int Rv, double fov0, double fov1, double px, double py,
                                  double R, double orientation, int visual_exclusion, int n_obs,
                                  const double *obs_xy, int n_social, int has_non_social,
                                  int keep_distance_info, double vision_range, double *out)
{
    double *phis = (double *)malloc(sizeof(double) * (size_t)Rv);
    double *raw = (double *)calloc((size_t)Rv, sizeof(double));
    orc_linspace(-ORC_PI, ORC_PI, Rv, phis);
    int cap = n_obs > 0 ? n_obs : 1;
    double *dist = (double *)malloc(sizeof(double) * (size_t)cap);
    double *vis = (double *)malloc(sizeof(double) * (size_t)cap);
    long long *ps0 = (long long *)malloc(sizeof(long long) * (size_t)cap);
    long long *pe0 = (long long *)malloc(sizeof(long long) * (size_t)cap);
    long long *sx = (long long *)malloc(sizeof(long long) * (size_t)cap);
    long long *ex = (long long *)malloc(sizeof(long long) * (size_t)cap);
    int *social = (int *)malloc(sizeof(int) * (size_t)cap);
    int *order = (int *)malloc(sizeof(int) * (size_t)cap);
    int m = 0;
    double last_d = 0.0;

    double v1sx = px + R, v1sy = py + R;
    double v1ex = px + (1 + cos(orientation)) * R;
    double v1ey = py + (1 - sin(orientation)) * R;
    double v1x = v1ex - v1sx, v1y = v1ey - v1sy;
    for (int i = 0; i < n_obs; ++i) {
        double ox = obs_xy[2 * i], oy = obs_xy[2 * i + 1];
        if (ox == px && oy == py) continue;
        double v2ex = ox + R, v2ey = oy + R;
        double v2x = v2ex - v1sx, v2y = v2ey - v1sy;
        double ca = orc_closed_angle_agent(v1x, v1y, v2x, v2y);
        double ddx = v2ex - v1sx, ddy = v2ey - v1sy;
        double d = sqrt(ddx * ddx + ddy * ddy);
        double va = 2 * atan(R / (1 * d));
        int t = orc_find_nearest(phis, Rv, ca);
        last_d = d;
        if (fov0 < ca && ca < fov1) {
            double ps = (va / (2 * ORC_PI)) * Rv;
            dist[m] = d;
            vis[m] = va;
            ps0[m] = (long long)((double)t - ps / 2);
            pe0[m] = (long long)((double)t + ps / 2);
            sx[m] = ps0[m];
            ex[m] = pe0[m];
            social[m] = has_non_social ? (i < n_social) : 1;
            ++m;
        }
    }
    if (visual_exclusion) {
        /* rank_V_source_data("distance"): stable ascending sort (insertion order = index) */
        for (int a = 0; a < m; ++a) order[a] = a;
        for (int a = 1; a < m; ++a) {
            int key = order[a], b = a - 1;
            while (b >= 0 && dist[order[b]] > dist[key]) { order[b + 1] = order[b]; --b; }
            order[b + 1] = key;
        }
        for (int r = 0; r < m; ++r) {
            int f = order[r];
            if (r > 0) {
                for (int q = 0; q < m; ++q) {
                    int i = order[q];
                    if (dist[i] < dist[f]) {
                        if (sx[f] <= ps0[i] && ps0[i] <= ex[f]) ex[f] = ps0[i];
                        if (sx[f] <= pe0[i] && pe0[i] <= ex[f]) sx[f] = pe0[i];
                        if (ps0[i] <= sx[f] && pe0[i] >= ex[f]) { sx[f] = 0; ex[f] = 0; }
                    }
                }
            } else {
                sx[f] = ps0[f];
                ex[f] = pe0[f];
            }
        }
    }
    /* fill order: the distance order of the exclusion step (or list order without it), then
     * a stable descending sort by visual angle */
    if (!visual_exclusion)
        for (int a = 0; a < m; ++a) order[a] = a;
    for (int a = 1; a < m; ++a) {
        int key = order[a], b = a - 1;
        while (b >= 0 && vis[order[b]] < vis[key]) { order[b + 1] = order[b]; --b; }
        order[b + 1] = key;
    }
    const double value = keep_distance_info ? 1 - last_d / vision_range : 1.0;
    for (int q = 0; q < m; ++q) {
        int a = order[q];
        if (!social[a]) continue;          /* remove_nonsocial_V_source_data */
        long long s = sx[a], e = ex[a];
        if (s < 0) { np_fill(raw, Rv, Rv + s, Rv, 1.0); s = 0; }
        if (e >= Rv) { np_fill(raw, Rv, 0, e - Rv, 1.0); e = Rv - 1; }
        np_fill(raw, Rv, s, e, value);
    }
    for (int k = 0; k < Rv; ++k) {
        double val = raw[Rv - 1 - k];
        if (phis[k] < fov0) val = 0;
        if (phis[k] > fov1) val = 0;
        out[k] = val;
    }
    free(phis); free(raw); free(dist); free(vis); free(ps0); free(pe0); free(sx); free(ex);
    free(social); free(order);
}

/* Agent.projection_field with keep_distance_info = False (the social channel). */
void orc_agent_projection_field(int Rv, double fov0, double fov1, double px, double py, double R,
                                double orientation, int visual_exclusion, int n_obs,
                                const double *obs_xy, int n_social, int has_non_social,
                                double *out)
{
    agent_projection_core(Rv, fov0, fov1, px, py, R, orientation, visual_exclusion, n_obs,
                          obs_xy, n_social, has_non_social, 0, 1.0, out);
}

/*
 * Agent.calc_social_V_proj (agent.py:396-419) for focal agent i: candidates within
 * vision_range (centre distance with each agent's own radius, supcalc.py:73-78), social =
 * exploiting agents other than i whose patch differs from i's (when patchwise) and is not -1;
 * every other candidate only occludes.  exploit[j] != 0 means mode "exploit".
 * out: Rv values (flipped, FOV-masked) = the agent's soc_v_field.
 */
void orc_social_vpf(int i, int n, const double *x, const double *y, const double *radii,
                    const double *th, const int *exploit, const int *patch, double vision_range,
                    int visual_exclusion, int patchwise, int Rv, double fov0, double fov1,
                    double *out)
{
    int *inr = (int *)malloc(sizeof(int) * (size_t)n);
    int *expl = (int *)malloc(sizeof(int) * (size_t)n);
    int *nonx = (int *)malloc(sizeof(int) * (size_t)n * 2);
    double *xy = (double *)malloc(sizeof(double) * 2 * (size_t)n * 2);
    int n_in = 0, n_ex = 0, n_nx = 0;
    double c1x = x[i] + radii[i], c1y = y[i] + radii[i];
    for (int j = 0; j < n; ++j) {
        double c2x = x[j] + radii[j], c2y = y[j] + radii[j];
        double ddx = c2x - c1x, ddy = c2y - c1y;
        if (sqrt(ddx * ddx + ddy * ddy) <= vision_range) inr[n_in++] = j;
    }
    for (int a = 0; a < n_in; ++a) {
        int j = inr[a];
        if (j != i && exploit[j]) expl[n_ex++] = j;
    }
    for (int a = 0; a < n_in; ++a) {
        int j = inr[a], is_ex = 0;
        for (int b = 0; b < n_ex; ++b) if (expl[b] == j) is_ex = 1;
        if (!is_ex) nonx[n_nx++] = j;
    }
    if (patchwise) {
        int keep = 0;
        for (int b = 0; b < n_ex; ++b) {
            if (patch[expl[b]] == patch[i]) nonx[n_nx++] = expl[b];
        }
        for (int b = 0; b < n_ex; ++b)
            if (patch[expl[b]] != patch[i]) expl[keep++] = expl[b];
        n_ex = keep;
    }
    {
        int keep = 0;
        for (int b = 0; b < n_ex; ++b) if (patch[expl[b]] != -1) expl[keep++] = expl[b];
        n_ex = keep;
    }
    int n_obs = 0;
    for (int b = 0; b < n_ex; ++b) { xy[2 * n_obs] = x[expl[b]]; xy[2 * n_obs + 1] = y[expl[b]]; ++n_obs; }
    if (visual_exclusion) {
        for (int b = 0; b < n_nx; ++b) { xy[2 * n_obs] = x[nonx[b]]; xy[2 * n_obs + 1] = y[nonx[b]]; ++n_obs; }
    }
    orc_agent_projection_field(Rv, fov0, fov1, x[i], y[i], radii[i], th[i], visual_exclusion,
                               n_obs, xy, n_ex, visual_exclusion, out);
    free(inr); free(expl); free(nonx); free(xy);
}

/* ---------------------------------------------------------------- foraging step
 *
 * One step of the foraging simulation (abm/simulation/sims.py:734-858, the agent-agent
 * collisions when collide_agents is set; Agent.update, abm/agent/agent.py:213-283), agents
 * updated from one snapshot.
 * Positions, orientation and speed are stored as float32 where the GPU step stores them, so
 * the two can be compared exactly; decision variables, collected units and patches are FP64.
 * Random draws: Philox-4x32-10 (Salmon et al., SC 2011) with the GPU step's counters, or the
 * injected uniforms of the random walk.
 *
 * FP[30]: T_w Eps_w g_w B_w w_max T_u Eps_u g_u B_u u_max S_wu S_uw F_N F_R exp_vel_max
 *         exp_theta_min exp_theta_max reloc_theta_max exp_stop_ratio width height window_pad
 *         agent_radius consumption min_resc_quality max_resc_quality patch_radius fov0 fov1
 *         vision_range
 * IP[12]: Tau pooling_time teleport_exploit regenerate_patches allow_border_patch_overlap
 *         min_resc_units max_resc_units rv visual_exclusion patchwise_exclusion
 *         collide_agents ghost_mode
 */
enum { M_EXPLORE = 0, M_RELOCATE = 1, M_EXPLOIT = 2, M_POOL = 3, M_COLLIDE = 4, M_NONE = -1 };

void orc_philox4x32(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t out[4])
{
    uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
    uint32_t k0 = k_in[0], k1 = k_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double orc_u01(uint32_t a, uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

static void orc_draw(uint64_t seed, uint32_t who, uint64_t count, uint32_t tag, uint32_t out[4])
{
    uint32_t c[4] = {who, (uint32_t)count, (uint32_t)(count >> 32), tag};
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    orc_philox4x32(c, k, out);
}

typedef struct {
    float *x, *y, *th, *v;
    double *w, *u, *col, *colb;
    int *mode, *ovr, *env, *envb, *pool, *patch;
    uint32_t *nov;
    uint64_t *draws;
} ForagerArrays;

static int f_get_mode(const ForagerArrays *a, const double *FP, int i)
{
    if (a->ovr[i] != M_NONE) return a->ovr[i];
    return a->w[i] > FP[0] ? M_RELOCATE : M_EXPLORE;
}

/* notify_agent (sims.py:29-42) */
static void f_notify(ForagerArrays *a, int Tau, int i, int status, int res_id)
{
    int before = a->env[i];
    a->envb[i] = before;
    a->env[i] = status;
    uint32_t mask = Tau >= 32 ? 0xFFFFFFFFu : ((1u << Tau) - 1u);
    a->nov[i] = ((a->nov[i] << 1) & mask) | ((status - before) > 0 ? 1u : 0u);
    a->pool[i] = 1;
    a->patch[i] = res_id;
}

static int f_pooling_done(const ForagerArrays *a, const int *IP, int i, int m)
{
    return ((m == M_POOL || m == M_RELOCATE) && a->pool[i]) || IP[1] == 0;
}

static double f_prove_orientation(double t)
{
    if (t < 0) t = 2 * ORC_PI + t;
    if (t > ORC_PI * 2) t = t - 2 * ORC_PI;
    return t;
}

/* add_new_resource_patch (sims.py:332-374) for slot k; returns 0 when no place was found */
static int f_regenerate(int k, int np, double *px, double *py, double *pr, double *pu,
                        double *pl, double *pq, const int *pid, uint64_t *pdraws,
                        const double *FP, const int *IP, uint64_t seed)
{
    double r = FP[26], pad = FP[21], lox, hix, loy, hiy;
    if (IP[4]) { lox = pad - r; hix = FP[19] + pad - r; loy = pad - r; hiy = FP[20] + pad - r; }
    else { lox = pad; hix = FP[19] + pad - 2 * r; loy = pad; hiy = FP[20] + pad - 2 * r; }
    uint64_t cnt = pdraws[k];
    for (int tries = 0; tries <= 10000; ++tries) {
        uint32_t w[4];
        orc_draw(seed, (uint32_t)k, cnt++, 0x50415443u, w);
        double x = lox + floor(orc_u01(w[0], w[1]) * (hix - lox));
        double y = loy + floor(orc_u01(w[2], w[3]) * (hiy - loy));
        int clear = 1;
        for (int q = 0; q < np && clear; ++q) {
            if (q == k || pid[q] < 0) continue;
            double dx = (x + r) - (px[q] + pr[q]), dy = (y + r) - (py[q] + pr[q]);
            double rr = r + pr[q];
            clear = dx * dx + dy * dy >= rr * rr;
        }
        if (!clear) continue;
        orc_draw(seed, (uint32_t)k, cnt++, 0x50415443u, w);
        int span = IP[6] - IP[5];
        double units = span > 0 ? (double)(IP[5] + (int)floor(orc_u01(w[0], w[1]) * span))
                                : (double)IP[5];
        px[k] = x; py[k] = y; pr[k] = r; pu[k] = units; pl[k] = units;
        pq[k] = FP[24] + orc_u01(w[2], w[3]) * (FP[25] - FP[24]);
        pdraws[k] = cnt;
        return 1;
    }
    pdraws[k] = cnt;
    return 0;
}

/* pygame.sprite.collide_circle (pygame's sprite module) on the agents' rects while their
 * radius is raised by the proximity distance 2 (sims.py:737-751): rect = int(position)
 * (pygame stores integer rect coordinates; a float assignment truncates), width int(2R), so
 * the centre is int(position) + int(2R) / 2; collision when the squared centre distance is at
 * most ((R + 2) + (R + 2))^2. */
static int f_rects_collide(const float *x, const float *y, double R, int a, int b)
{
    long long half = (long long)(2 * R) / 2;
    long long dx = ((long long)x[a] + half) - ((long long)x[b] + half);
    long long dy = ((long long)y[a] + half) - ((long long)y[b] + half);
    double rr = (R + 2) + (R + 2);
    return (double)(dx * dx + dy * dy) <= rr * rr;
}

/* Simulation.agent_agent_collision_proximity (sims.py:421-474) for one collided agent b: the
 * LIDAR-like proximity field of the agents within 2R + 20 of it (Agent.projection_field with
 * keep_distance_info, full circle), the turn away from the fuller half and the stop when the
 * 200 pixels ahead are occupied.  th: the FP64 orientations of this phase. */
static void f_collide_process(ForagerArrays *A, const double *FP, const int *IP, int n, int b,
                              const int *expl, double *th, double *obs, double *pf)
{
    const double R = FP[22];
    const int Rv = IP[7];
    if (!expl[b]) { A->ovr[b] = M_COLLIDE; A->mode[b] = M_COLLIDE; }
    int n_obs = 0;
    double c1x = (double)A->x[b] + R, c1y = (double)A->y[b] + R;
    for (int j = 0; j < n; ++j) {
        if (j == b) continue;
        double ddx = ((double)A->x[j] + R) - c1x, ddy = ((double)A->y[j] + R) - c1y;
        if (sqrt(ddx * ddx + ddy * ddy) < 2 * R + 20) {
            obs[2 * n_obs] = A->x[j];
            obs[2 * n_obs + 1] = A->y[j];
            ++n_obs;
        }
    }
    agent_projection_core(Rv, -ORC_PI, ORC_PI, A->x[b], A->y[b], R, th[b], IP[8], n_obs, obs,
                          n_obs, 0, 1, FP[29], pf);
    const long long h = Rv / 2;
    double le = np_mean(pf, h, 1), re = np_mean(pf + h, Rv - h, 1);
    double D = (le - re > 0) ? 1.0 : (le - re < 0) ? -1.0 : 0.0;   /* np.sign */
    if (D == 0) D = -1;
    if (!expl[b]) th[b] -= D * 0.2;
    long long lo = h - 100, hi = h + 100;                            /* Python slice rules */
    if (lo < 0) { lo += Rv; if (lo < 0) lo = 0; }
    if (hi > Rv) hi = Rv;
    double front = np_mean(pf + lo, hi - lo, 1);
    if (front > 0) A->v[b] = 0.0f;
    else if (!expl[b]) A->v[b] = (float)FP[14];
}

/* The agent-agent interaction block of Simulation.start (sims.py:735-784): pygame's
 * groupcollide of the agents with themselves (agent order, each agent's list in agent order),
 * the proximity manoeuvre for every listed agent (skipped in ghost mode when either agent
 * exploits), then the collided agents' bookkeeping: an agent left in collide mode returns to
 * explore, a collided one in collide mode is notified with -1. */
static void f_collide_phase(ForagerArrays *A, const double *FP, const int *IP, int n)
{
    const int ghost = IP[11], tele = IP[2];
    const double R = FP[22];
    int *expl = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *coll = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
    double *th = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double *obs = (double *)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    double *pf = (double *)malloc(sizeof(double) * (size_t)IP[7]);
    for (int i = 0; i < n; ++i) { expl[i] = A->ovr[i] == M_EXPLOIT; th[i] = A->th[i]; }
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            if (b == a || !f_rects_collide(A->x, A->y, R, a, b)) continue;
            if (ghost && (expl[b] || expl[a])) continue;
            f_collide_process(A, FP, IP, n, b, expl, th, obs, pf);
        }
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            if (b == a || !f_rects_collide(A->x, A->y, R, a, b)) continue;
            if (tele) {
                if (!expl[a]) coll[a] = 1;
                if (!expl[b]) coll[b] = 1;
            } else if (!ghost || (!expl[a] && !expl[b])) {
                coll[a] = coll[b] = 1;
            }
        }
    for (int i = 0; i < n; ++i) {
        A->th[i] = (float)th[i];
        int cur = f_get_mode(A, FP, i);
        if (!coll[i] && cur == M_COLLIDE) { A->ovr[i] = M_NONE; A->mode[i] = M_EXPLORE; }
        if (coll[i] && cur == M_COLLIDE) f_notify(A, IP[0], i, -1, -1);
    }
    free(expl); free(coll); free(th); free(obs); free(pf);
}

int orc_forage_step(int n, float *x, float *y, float *th, float *v, double *w, double *u,
                    double *col, double *colb, int *mode, int *ovr, int *env, int *envb,
                    int *pool, int *patch, uint32_t *nov, uint64_t *draws, int np, double *px,
                    double *py, double *pr, double *pu, double *pl, double *pq, int *pid,
                    uint64_t *pdraws, const double *FP, const int *IP, uint64_t seed,
                    const double *uniforms, double *soc_out)
{
    ForagerArrays A = {x, y, th, v, w, u, col, colb, mode, ovr, env, envb, pool, patch, nov, draws};
    const int Tau = IP[0], Rv = IP[7];
    const double R = FP[22];
    int failed = 0;
    int *patch_of = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *destroyed = (int *)calloc((size_t)(np > 0 ? np : 1), sizeof(int));
    /* 0. agent-agent collisions (sims.py:735-784), when enabled */
    if (IP[10]) f_collide_phase(&A, FP, IP, n);
    /* 1. agent-resource interaction (sims.py:789-846) */
    for (int i = 0; i < n; ++i) {
        double cx = (double)x[i] + R, cy = (double)y[i] + R;
        patch_of[i] = -1;
        for (int k = 0; k < np && patch_of[i] < 0; ++k) {
            if (pid[k] < 0) continue;
            double dx = (px[k] + pr[k]) - cx, dy = (py[k] + pr[k]) - cy;
            if (sqrt(dx * dx + dy * dy) < pr[k]) patch_of[i] = k;
        }
    }
    for (int k = 0; k < np; ++k) {
        if (pid[k] < 0) continue;
        double pcx = px[k] + pr[k], pcy = py[k] + pr[k];
        int destroy = 0;
        for (int i = 0; i < n; ++i) {
            if (patch_of[i] != k) continue;
            double dx = pcx - ((double)x[i] + R), dy = pcy - ((double)y[i] + R);
            double cl = fmod(atan2(dy, dx) + (double)th[i], 2.0 * ORC_PI);
            if (cl < 0) cl += 2.0 * ORC_PI;
            th[i] = (float)((double)th[i] + (cl - ORC_PI) * 0.02);
            if (destroy) { f_notify(&A, Tau, i, -1, -1); continue; }
            if (f_pooling_done(&A, IP, i, f_get_mode(&A, FP, i))) {
                f_notify(&A, Tau, i, 1, pid[k]);
                if (IP[2]) {
                    x[i] = (float)(px[k] + pr[k] - R);
                    y[i] = (float)(py[k] + pr[k] - R);
                }
            }
            if (f_get_mode(&A, FP, i) == M_EXPLOIT) {
                double want = FP[23], got;
                if (want > pq[k]) want = pq[k];
                if (pl[k] >= want) { pl[k] -= want; got = want; }
                else { got = pl[k]; pl[k] = 0.0; }
                colb[i] = col[i];
                col[i] += got;
                if (!(pl[k] > 0.0)) {
                    destroy = 1;
                    for (int j = 0; j < n; ++j) if (patch_of[j] == k) f_notify(&A, Tau, j, -1, -1);
                }
            }
        }
        destroyed[k] = destroy;
    }
    for (int k = 0; k < np; ++k) {
        if (!destroyed[k]) continue;
        if (!IP[3] || !f_regenerate(k, np, px, py, pr, pu, pl, pq, pid, pdraws, FP, IP, seed)) {
            if (IP[3]) failed++;
            pid[k] = -1;
        }
    }
    int *exploit = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) {
        if (patch_of[i] < 0) {
            int m = f_get_mode(&A, FP, i);
            if (f_pooling_done(&A, IP, i, m) || m == M_EXPLOIT) f_notify(&A, Tau, i, -1, -1);
        }
        exploit[i] = ovr[i] == M_EXPLOIT;
    }
    /* 2. social fields from the post-interaction snapshot (Agent.calc_social_V_proj) */
    double *xd = (double *)malloc(sizeof(double) * 4 * (size_t)(n > 0 ? n : 1));
    double *yd = xd + n, *rd = xd + 2 * (size_t)n, *td = xd + 3 * (size_t)n;
    for (int i = 0; i < n; ++i) { xd[i] = x[i]; yd[i] = y[i]; rd[i] = R; td[i] = th[i]; }
    for (int i = 0; i < n; ++i)
        orc_social_vpf(i, n, xd, yd, rd, td, exploit, patch, FP[29], IP[8], IP[9], Rv, FP[27],
                       FP[28], soc_out + (size_t)i * Rv);
    /* 3. agent update (agent.py:213-283) */
    for (int i = 0; i < n; ++i) {
        const double *V = soc_out + (size_t)i * Rv;
        int half = Rv / 2;
        double total = 0, left = 0;
        for (int k = 0; k < Rv; ++k) { total += V[k]; if (k < half) left += V[k]; }
        double I_priv = FP[12] * (nov[i] ? 1.0 : 0.0) + FP[13] * (col[i] - colb[i]);
        double wv = w[i], uv = u[i];
        double w_p = wv > FP[0] ? wv : 0.0, u_p = uv > FP[5] ? uv : 0.0;
        double dw = FP[1] * (total / Rv) - FP[2] * (wv - FP[3]) - u_p * FP[11];
        double du = FP[6] * I_priv - FP[7] * (uv - FP[8]) - w_p * FP[10];
        wv += dw; uv += du;
        if (wv > FP[4]) wv = FP[4];
        if (wv < -FP[4]) wv = -FP[4];
        if (uv > FP[9]) uv = FP[9];
        if (uv < -FP[9]) uv = -FP[9];
        w[i] = wv; u[i] = uv;
        int o = ovr[i], md = mode[i];
        double vel0 = (double)v[i], vel = 0.0, theta = 0.0;
        int cur = o != M_NONE ? o : (wv > FP[0] ? M_RELOCATE : M_EXPLORE);
        if (cur != M_COLLIDE) {
            int tw = wv > FP[0], tu = uv > FP[0], on = env[i] == 1, act;
            if (!tw && !tu) act = 0;
            else if (tw && tu) act = on ? 2 : 1;
            else if (tw) act = 1;
            else act = on ? 2 : 0;
            if (act == 0) {
                double r01;
                if (uniforms) r01 = uniforms[i];
                else {
                    uint32_t wd[4];
                    orc_draw(seed, (uint32_t)i, draws[i], 0x57414C4Bu, wd);
                    r01 = orc_u01(wd[0], wd[1]);
                    draws[i] += 1;
                }
                vel = FP[14];
                theta = FP[15] + (FP[16] - FP[15]) * r01;
                md = M_EXPLORE; o = M_NONE;
            } else if (act == 1) {
                double le = left / half, re = (total - left) / (Rv - half);
                vel = FP[14] - vel0;
                theta = (le - re) * FP[17];
                md = M_RELOCATE; o = M_NONE;
            } else {
                vel = -vel0 * FP[18];
                theta = 0.0;
                md = M_EXPLOIT; o = M_EXPLOIT;
            }
        }
        mode[i] = md; ovr[i] = o;
        double t = f_prove_orientation((double)th[i] + theta);
        double vv = vel0 + vel;
        int after = o != M_NONE ? o : (wv > FP[0] ? M_RELOCATE : M_EXPLORE);
        if (after == M_EXPLORE && fabs(vv) > 1.0) vv = FP[14];
        double xx = (double)x[i] + vv * cos(t), yy = (double)y[i] - vv * sin(t);
        double bx0 = FP[21], bx1 = FP[21] + FP[19], by0 = FP[21], by1 = FP[21] + FP[20];
        double cx = xx + R, cy = yy + R;
        if (cx < bx0) {
            xx = bx0 - R;
            if (ORC_PI / 2 <= t && t < ORC_PI) t -= ORC_PI / 2;
            else if (ORC_PI <= t && t <= 3 * ORC_PI / 2) t += ORC_PI / 2;
            t = f_prove_orientation(t);
        }
        if (cx > bx1) {
            xx = bx1 - R - 1;
            if (3 * ORC_PI / 2 <= t && t < 2 * ORC_PI) t -= ORC_PI / 2;
            else if (0 <= t && t <= ORC_PI / 2) t += ORC_PI / 2;
            t = f_prove_orientation(t);
        }
        if (cy < by0) {
            yy = by0 - R;
            if (ORC_PI / 2 <= t && t <= ORC_PI) t += ORC_PI / 2;
            else if (0 <= t && t < ORC_PI / 2) t -= ORC_PI / 2;
            t = f_prove_orientation(t);
        }
        if (cy > by1) {
            yy = by1 - R - 1;
            if (3 * ORC_PI / 2 <= t && t <= 2 * ORC_PI) t += ORC_PI / 2;
            else if (ORC_PI <= t && t < 3 * ORC_PI / 2) t -= ORC_PI / 2;
            t = f_prove_orientation(t);
        }
        x[i] = (float)xx; y[i] = (float)yy; th[i] = (float)t; v[i] = (float)vv;
        colb[i] = col[i];
    }
    free(patch_of); free(destroyed); free(exploit); free(xd);
    return failed;
}
