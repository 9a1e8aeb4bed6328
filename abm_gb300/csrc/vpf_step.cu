// vpf_step.cu -- the fused per-timestep kernel (VPF rasterisation + VSWRM + update) and the
// drop-in twins of projection_field / VSWRM_flocking_state_variables.
//
// Work decomposition: one warp per focal agent.  A block of `warps` focal agents streams the
// neighbour positions through shared memory in tiles (n-body style), staged by the TMA bulk
// engine (cp.async.bulk + mbarrier, double-buffered) when the state arrays are 16-byte
// aligned.  Each lane evaluates one neighbour per iteration, and OR-s the visible pixel run
// into the warp's VPF bitmask (ceil(Rv/32) words in shared memory).  The warp then walks the
// bitmask's transitions to form the VSWRM integrals against fixed-point tables and lane 0
// applies the FP64 state update.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

struct StepArgs {
    const float *x, *y, *th, *v;
    float *xo, *yo, *tho, *vo;
    const float *radius, *alp0, *bet0, *v0;
    int n, tile;
    float radius0;
    uint32_t *bits;
    double *terms;
    unsigned long long *diag;
    dfl W, H;
    UpdateParams up;
    GridDev g;
};

static int g_warps = 8;
static int g_tile = 2048;
static std::mutex g_cfg_mu;

static size_t step_smem_bytes(int warps, int tile, int words, bool hetero) {
    const int nf = hetero ? 3 : 2;
    return 16 + 2 * (size_t)nf * tile * sizeof(float) + (size_t)warps * words * sizeof(uint32_t);
}

template <bool TORUS, bool HETERO, bool TMA>
__global__ void __launch_bounds__(1024) vpf_flock_step_kernel(const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const int tile = a.tile, n = a.n;
    constexpr int NF = HETERO ? 3 : 2;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    float *buf0 = reinterpret_cast<float *>(smem + 16);
    uint32_t *vb = reinterpret_cast<uint32_t *>(buf0 + 2 * NF * tile) + warp * a.g.words;
    const int i = blockIdx.x * nw + warp;
    const bool active = i < n;

    FocalDev f;
    double thd = 0.0;
    if (active) {
        f.x = a.x[i];
        f.y = a.y[i];
        f.r = HETERO ? a.radius[i] : a.radius0;
        thd = (double)a.th[i];
    } else {
        f.x = f.y = 0.f;
        f.r = a.radius0;
    }
    f.invr = 1.f / f.r;
    double sn, cs;
    sincos(thd, &sn, &cs);
    f.c = (float)cs;
    f.s = (float)sn;
    f.cd = df_split(cs);
    f.sd = df_split(sn);
    for (int w = lane; w < a.g.words; w += 32) vb[w] = 0u;

    if (TMA && tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    __syncthreads();

    const int ntiles = (n + tile - 1) / tile;
    auto issue = [&](int k) {
        const int base = k * tile;
        const int tn = min(tile, n - base);
        const int tn4 = tn & ~3;
        if (tn4 > 0) {
            float *dst = buf0 + (k & 1) * NF * tile;
            const uint32_t bytes = (uint32_t)tn4 * 4u;
            fence_proxy_async();
            mbar_expect_tx(&bars[k & 1], bytes * NF);
            bulk_g2s(dst, a.x + base, bytes, &bars[k & 1]);
            bulk_g2s(dst + tile, a.y + base, bytes, &bars[k & 1]);
            if (HETERO) bulk_g2s(dst + 2 * tile, a.radius + base, bytes, &bars[k & 1]);
        }
    };
    if (TMA && tid == 0) issue(0);

    for (int k = 0; k < ntiles; ++k) {
        const int base = k * tile;
        const int tn = min(tile, n - base);
        int tn_s;   // neighbours of this tile that are in shared memory
        float *cur = buf0 + (k & 1) * NF * tile;
        if (TMA) {
            if (tid == 0 && k + 1 < ntiles) issue(k + 1);
            tn_s = tn & ~3;
            if (tn_s > 0 && !mbar_wait(&bars[k & 1], (uint32_t)((k >> 1) & 1))) {
                if (a.diag && lane == 0) atomicAdd(&a.diag[ABM_DIAG_TIMEOUTS], 1ull);
            }
        } else {
            for (int q = tid; q < tn; q += blockDim.x) {
                cur[q] = a.x[base + q];
                cur[tile + q] = a.y[base + q];
                if (HETERO) cur[2 * tile + q] = a.radius[base + q];
            }
            tn_s = tn;
            __syncthreads();
        }
        if (active) {
            for (int jb = 0; jb < tn; jb += 32) {
                const int jj = jb + lane;
                const bool valid = jj < tn;
                float xj = f.x, yj = f.y, rj = f.r;
                if (jj < tn_s) {
                    xj = cur[jj];
                    yj = cur[tile + jj];
                    if (HETERO) rj = cur[2 * tile + jj];
                } else if (valid) {
                    xj = a.x[base + jj];
                    yj = a.y[base + jj];
                    if (HETERO) rj = a.radius[base + jj];
                }
                int s, e;
                bool vis;
                pair_projection<TORUS, HETERO>(f, xj, yj, rj, HETERO ? rcp_approx(rj) : f.invr,
                                               valid, a.g, a.W, a.H, s, e, vis, a.diag);
                if (vis) raster_projection(vb, a.g.rv, s, e);
            }
        }
        __syncthreads();
    }
    if (!active) return;

    long long bc, bs, ec, es;
    warp_integrals(vb, a.g, bc, bs, ec, es);
    if (a.bits) {
        uint32_t *dst = a.bits + (size_t)i * a.g.words;
        for (int w = lane; w < a.g.words; w += 32) dst[w] = vb[w];
    }
    if (lane == 0) {
        const UpdateParams &p = a.up;
        const double alp0 = a.alp0 ? (double)a.alp0[i] : p.alp0;
        const double bet0 = a.bet0 ? (double)a.bet0[i] : p.bet0;
        const double v0 = a.v0 ? (double)a.v0[i] : p.v0;
        double vel = (double)a.v[i];
        double ab = 0, ae = 0, bb = 0, be = 0, dv = 0, dpsi = 0;
        if (a.g.phi_ok) {
            ab = alp0 * (-(double)bc * kInvFix);
            ae = alp0 * p.alp1 * ((double)ec * kInvFix);
            bb = bet0 * (-(double)bs * kInvFix);
            be = bet0 * p.bet1 * ((double)es * kInvFix);
            dv = p.gam * (v0 - vel) + ab + ae;
            dpsi = bb + be;
        }
        if (a.terms) {
            double *t = a.terms + 6 * (size_t)i;
            t[0] = dv;
            t[1] = dpsi;
            t[2] = ab;
            t[3] = ae;
            t[4] = bb;
            t[5] = be;
        }
        double x = (double)f.x, y = (double)f.y, th = thd;
        update_agent(p, (double)f.r, dpsi, dv, x, y, th, vel);
        a.xo[i] = (float)x;
        a.yo[i] = (float)y;
        a.tho[i] = (float)th;
        a.vo[i] = (float)vel;
        if (a.diag && !(isfinite(x) && isfinite(y) && isfinite(th) && isfinite(vel)))
            atomicAdd(&a.diag[ABM_DIAG_NONFINITE], 1ull);
    }
}

template <bool TORUS, bool HETERO, bool TMA>
static int launch_step(const StepArgs &a, int warps, cudaStream_t stream) {
    auto kern = vpf_flock_step_kernel<TORUS, HETERO, TMA>;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    const size_t smem = step_smem_bytes(warps, a.tile, a.g.words, HETERO);
    const int blocks = (a.n + warps - 1) / warps;
    kern<<<blocks, warps * 32, smem, stream>>>(a);
    return check_cuda(cudaGetLastError(), "vpf_flock_step_kernel launch");
}

static bool aligned16(const void *p) { return p == nullptr || ((uintptr_t)p & 15u) == 0; }

UpdateParams make_update(const abm_vf_params *p) {
    UpdateParams u;
    u.gam = p->gam;
    u.v0 = p->v0;
    u.alp0 = p->alp0;
    u.alp1 = p->alp1;
    u.bet0 = p->bet0;
    u.bet1 = p->bet1;
    u.max_vel = p->max_vel;
    u.max_th = p->max_th;
    u.dt = p->dt;
    u.bx0 = p->window_pad;
    u.bx1 = p->window_pad + p->width;
    u.by0 = p->window_pad;
    u.by1 = p->window_pad + p->height;
    u.limit = p->limit_movement != 0;
    u.torus = p->boundary == ABM_BOUNDARY_INFINITE;
    return u;
}

int validate_params(const abm_vf_params *p, const char *fn) {
    if (!p) return set_error(ABM_ERR_INVALID_ARG, "%s: params is NULL", fn);
    if (p->rv < 2 || p->rv > ABM_MAX_RV)
        return set_error(ABM_ERR_RV, "%s: rv=%d outside [2, %d]", fn, p->rv, ABM_MAX_RV);
    if (p->boundary != ABM_BOUNDARY_WALLS && p->boundary != ABM_BOUNDARY_INFINITE)
        return set_error(ABM_ERR_INVALID_ARG, "%s: boundary=%d", fn, p->boundary);
    if (!(p->radius > 0) || !std::isfinite(p->radius))
        return set_error(ABM_ERR_INVALID_ARG, "%s: radius=%g", fn, p->radius);
    if (p->boundary == ABM_BOUNDARY_INFINITE && !(p->width > 0 && p->height > 0))
        return set_error(ABM_ERR_INVALID_ARG, "%s: torus needs width, height > 0", fn);
    return ABM_OK;
}

// ------------------------------------------------------------------ projection_field twin
struct ProjArgs {
    dfl px, py;            // focal top-left, double-float
    float R;               // focal radius
    FocalDev f;
    const double *obj, *sizes;
    int n, torus, has_vr;
    dfl W, H, vr2;
    int *runs;             // n * 6 ints: three [a, b) runs in raw pixel order (empty: a >= b)
    unsigned long long *diag;
    GridDev g;
};

__global__ void project_pairs_kernel(const ProjArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    int *run = a.runs + 6 * (size_t)j;
    for (int q = 0; q < 6; ++q) run[q] = 0;
    const double ox = a.obj[2 * j], oy = a.obj[2 * j + 1];
    const dfl ox2 = df_split(ox), oy2 = df_split(oy);
    if (ox2.hi == a.px.hi && ox2.lo == a.px.lo && oy2.hi == a.py.hi && oy2.lo == a.py.lo)
        return;  // vf_supcalc.py:57-58
    const float rj = a.sizes ? (float)a.sizes[j] : a.R;
    // centre offset: (o + size) - (p + R), exact in double-float for these magnitudes
    dfl ex = df_add(df_sub(ox2, a.px), two_sum(rj, -a.R));
    dfl ey = df_add(df_sub(oy2, a.py), two_sum(rj, -a.R));
    if (a.torus) {
        dfl hw = {a.W.hi * 0.5f, a.W.lo * 0.5f}, hh = {a.H.hi * 0.5f, a.H.lo * 0.5f};
        if (df_sign(df_sub(ex, hw)) > 0) ex = df_sub(ex, a.W);
        else if (df_sign(df_add(ex, hw)) < 0) ex = df_add(ex, a.W);
        if (df_sign(df_sub(ey, hh)) > 0) ey = df_sub(ey, a.H);
        else if (df_sign(df_add(ey, hh)) < 0) ey = df_add(ey, a.H);
    }
    if (a.has_vr) {  // vision_range cut (vf_supcalc.py:91-93): d > vision_range
        dfl d2 = df_add(df_mul(ex, ex), df_mul(ey, ey));
        if (df_sign(df_sub(d2, a.vr2)) > 0) return;
    }
    const float dx = ex.hi + ex.lo, dy = ey.hi + ey.lo;
    const FocalDev &f = a.f;
    const GridDev &g = a.g;
    const float d2 = fmaf(dx, dx, dy * dy);
    const float rsq = rsqrtf(d2);
    const float P = fmaf(f.c, dy, f.s * dx);
    const float Q = fmaf(f.c, dx, -(f.s * dy));
    const float ca = closed_angle_f32(P, Q);
    const float u = fmaf(ca, g.inv_delta, g.half_rm1);
    const float kf = floorf(u);
    const float fr = u - kf;
    int t = (int)kf + (fr > 0.5f ? 1 : 0);
    t = t < 0 ? 0 : (t > g.rv - 1 ? g.rv - 1 : t);
    bool unc_t = fabsf(fr - 0.5f) < g.band_t || u < g.band_t || u > g.rvm1 - g.band_t;
    const float ps2 = half_angle_f32(rj, 1.f / rj, d2, rsq) * g.ps2_scale;
    const float hf = floorf(ps2);
    int h = (int)hf;
    const float frh = ps2 - hf;
    const float bh = g.band_h * fmaxf(ps2, 1.f);
    bool unc_h = frh < bh || frh > 1.f - bh;
    if (df_sign(ex) == 0 && df_sign(ey) == 0) {
        t = 0;
        h = g.rv >> 2;
        unc_t = unc_h = false;
    }
    if (unc_t || unc_h) {
        int2 th = resolve_pair(f.cd, f.sd, ex, ey, rj, resolve_grid(g), unc_t, unc_h, u, ps2, t,
                               h, a.diag);
        t = th.x;
        h = th.y;
    }
    int s = t - h, e = t + h;
    const int rv = g.rv;
    if (!((g.f0 < s && s < g.f1) || (g.f0 < e && e < g.f1))) return;
    if (s < 0) {
        run[0] = rv + s;
        run[1] = rv;
        s = 0;
    }
    if (e >= rv) {
        run[2] = 0;
        run[3] = min(e - (rv - 1), rv);
        e = rv;
    }
    run[4] = s;
    run[5] = e;
}

__global__ void project_fill_kernel(const int *runs, int n, int rv, double *rows) {
    const int j = blockIdx.y;
    const int *r = runs + 6 * (size_t)j;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < rv; k += gridDim.x * blockDim.x) {
        const int raw = rv - 1 - k;  // np.flip(v_field, axis=1)
        bool on = (raw >= r[0] && raw < r[1]) || (raw >= r[2] && raw < r[3]) ||
                  (raw >= r[4] && raw < r[5]);
        rows[(size_t)j * rv + k] = on ? 1.0 : 0.0;
    }
}

// ------------------------------------------------------------------ VSWRM twin
struct VswrmArgs {
    const uint32_t *bits;
    const float *vel, *alp0, *bet0, *v0;
    double prm[8];
    int n;
    double *out;
    GridDev g;
};

__global__ void vswrm_kernel(const VswrmArgs a) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.n) return;
    const uint32_t *vb = a.bits + (size_t)warp * a.g.words;
    long long bc, bs, ec, es;
    warp_integrals(vb, a.g, bc, bs, ec, es);
    if (lane == 0) {
        const double GAM = a.prm[0], ALP1 = a.prm[3], BET1 = a.prm[6];
        const double ALP0 = a.alp0 ? (double)a.alp0[warp] : a.prm[2];
        const double BET0 = a.bet0 ? (double)a.bet0[warp] : a.prm[5];
        const double V0 = a.v0 ? (double)a.v0[warp] : a.prm[1];
        const double ab = ALP0 * (-(double)bc * kInvFix);
        const double ae = ALP0 * ALP1 * ((double)ec * kInvFix);
        const double bb = BET0 * (-(double)bs * kInvFix);
        const double be = BET0 * BET1 * ((double)es * kInvFix);
        double *o = a.out + 6 * (size_t)warp;
        o[0] = GAM * (V0 - (double)a.vel[warp]) + ab + ae;
        o[1] = bb + be;
        o[2] = ab;
        o[3] = ae;
        o[4] = bb;
        o[5] = be;
    }
}

}  // namespace abm

using namespace abm;

extern "C" {

int abm_vpf_set_step_config(int32_t warps_per_block, int32_t tile) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    if (warps_per_block) {
        if (warps_per_block < 1 || warps_per_block > 32 ||
            (warps_per_block & (warps_per_block - 1)))
            return set_error(ABM_ERR_INVALID_ARG, "warps_per_block=%d", warps_per_block);
        g_warps = warps_per_block;
    }
    if (tile) {
        if (tile < 32 || tile > 8192 || tile % 32)
            return set_error(ABM_ERR_INVALID_ARG, "tile=%d", tile);
        g_tile = tile;
    }
    return ABM_OK;
}

int abm_vpf_get_step_config(int32_t *warps_per_block, int32_t *tile) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    if (warps_per_block) *warps_per_block = g_warps;
    if (tile) *tile = g_tile;
    return ABM_OK;
}

int abm_vpf_flock_step(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                       const abm_vf_params *p, const abm_agent_overrides *ov,
                       uint32_t *vpf_bits_dev, double *terms_dev,
                       unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_flock_step";
    int st = validate_params(p, fn);
    if (st) return st;
    if (!in || !out) return set_error(ABM_ERR_INVALID_ARG, "%s: state is NULL", fn);
    if (n < 0) return set_error(ABM_ERR_INVALID_ARG, "%s: n=%d", fn, n);
    if (n == 0) return ABM_OK;
    if (!in->x || !in->y || !in->theta || !in->v || !out->x || !out->y || !out->theta ||
        !out->v)
        return set_error(ABM_ERR_INVALID_ARG, "%s: a state array is NULL", fn);
    if (in->x == out->x || in->y == out->y || in->theta == out->theta || in->v == out->v)
        return set_error(ABM_ERR_INVALID_ARG, "%s: out must not alias in", fn);
    const GridDev *g = grid_for(p->rv, p->fov0, p->fov1, &st);
    if (!g) return st;
    int warps, tile;
    abm_vpf_get_step_config(&warps, &tile);
    StepArgs a;
    memset(&a, 0, sizeof(a));
    a.x = in->x;
    a.y = in->y;
    a.th = in->theta;
    a.v = in->v;
    a.xo = out->x;
    a.yo = out->y;
    a.tho = out->theta;
    a.vo = out->v;
    a.radius = ov ? ov->radius : nullptr;
    a.alp0 = ov ? ov->alp0 : nullptr;
    a.bet0 = ov ? ov->bet0 : nullptr;
    a.v0 = ov ? ov->v0 : nullptr;
    a.n = n;
    a.tile = std::min(tile, ((n + 31) / 32) * 32);
    {   // keep the tiles + bitmasks within the 200 KiB of dynamic shared memory we opt into
        const size_t words_bytes = (size_t)warps * g->words * sizeof(uint32_t);
        const int nf = (ov && ov->radius) ? 3 : 2;
        const long fit = ((long)(200 * 1024) - 16 - (long)words_bytes) / (2L * nf * 4);
        if (fit < 32)
            return set_error(ABM_ERR_UNSUPPORTED, "%s: rv=%d too large for %d warps per block",
                             fn, p->rv, warps);
        a.tile = std::min<int>(a.tile, (int)(fit / 32) * 32);
    }
    a.radius0 = (float)p->radius;
    a.bits = vpf_bits_dev;
    a.terms = terms_dev;
    a.diag = diag_dev;
    a.W = {(float)p->width, (float)(p->width - (double)(float)p->width)};
    a.H = {(float)p->height, (float)(p->height - (double)(float)p->height)};
    a.up = make_update(p);
    a.g = *g;
    const bool torus = p->boundary == ABM_BOUNDARY_INFINITE;
    const bool hetero = a.radius != nullptr;
    const bool tma = aligned16(a.x) && aligned16(a.y) && aligned16(a.radius);
    cudaStream_t s = (cudaStream_t)stream;
    if (!torus && !hetero) st = tma ? launch_step<false, false, true>(a, warps, s)
                                     : launch_step<false, false, false>(a, warps, s);
    else if (!torus && hetero) st = tma ? launch_step<false, true, true>(a, warps, s)
                                         : launch_step<false, true, false>(a, warps, s);
    else if (torus && !hetero) st = tma ? launch_step<true, false, true>(a, warps, s)
                                         : launch_step<true, false, false>(a, warps, s);
    else st = tma ? launch_step<true, true, true>(a, warps, s)
                  : launch_step<true, true, false>(a, warps, s);
    if (st) return st;
    return g->phi_ok ? ABM_OK : ABM_WARN_PHI_MISMATCH;
}

int abm_vpf_project_rows(const double fov[2], int32_t rv, const double pos_host[2],
                         double radius, double orientation, int32_t n_obj,
                         const double *obj_xy_dev, const double *obj_sizes_dev,
                         int32_t boundary, double width, double height, double vision_range,
                         double *rows_dev, unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_project_rows";
    if (!fov || !pos_host) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    if (rv < 2 || rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "%s: rv=%d", fn, rv);
    if (n_obj < 0) return set_error(ABM_ERR_INVALID_ARG, "%s: n_obj=%d", fn, n_obj);
    if (n_obj == 0) return ABM_OK;
    if (!obj_xy_dev || !rows_dev) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL array", fn);
    if (!(radius > 0)) return set_error(ABM_ERR_INVALID_ARG, "%s: radius=%g", fn, radius);
    int st;
    const GridDev *g = grid_for(rv, fov[0], fov[1], &st);
    if (!g) return st;
    ProjArgs a;
    memset(&a, 0, sizeof(a));
    a.px = {(float)pos_host[0], (float)(pos_host[0] - (double)(float)pos_host[0])};
    a.py = {(float)pos_host[1], (float)(pos_host[1] - (double)(float)pos_host[1])};
    a.R = (float)radius;
    const double c = std::cos(orientation), s = std::sin(orientation);
    a.f.x = a.f.y = 0.f;
    a.f.r = (float)radius;
    a.f.invr = 1.f / a.f.r;
    a.f.c = (float)c;
    a.f.s = (float)s;
    a.f.cd = {(float)c, (float)(c - (double)(float)c)};
    a.f.sd = {(float)s, (float)(s - (double)(float)s)};
    a.obj = obj_xy_dev;
    a.sizes = obj_sizes_dev;
    a.n = n_obj;
    a.torus = boundary == ABM_BOUNDARY_INFINITE;
    a.W = {(float)width, (float)(width - (double)(float)width)};
    a.H = {(float)height, (float)(height - (double)(float)height)};
    a.has_vr = vision_range >= 0;
    const double vr2 = vision_range * vision_range;
    a.vr2 = {(float)vr2, (float)(vr2 - (double)(float)vr2)};
    a.diag = diag_dev;
    a.g = *g;
    int *runs = nullptr;
    cudaStream_t cs = (cudaStream_t)stream;
    st = check_cuda(cudaMallocAsync((void **)&runs, 6 * sizeof(int) * (size_t)n_obj, cs),
                    "cudaMallocAsync(runs)");
    if (st) return st;
    a.runs = runs;
    project_pairs_kernel<<<(n_obj + 127) / 128, 128, 0, cs>>>(a);
    dim3 grid((rv + 255) / 256, n_obj);
    project_fill_kernel<<<grid, 256, 0, cs>>>(runs, n_obj, rv, rows_dev);
    st = check_cuda(cudaGetLastError(), "project kernels launch");
    cudaFreeAsync(runs, cs);
    return st;
}

int abm_vswrm_integrals(int32_t n_fields, int32_t rv, const uint32_t *bits_dev,
                        const double *phi_host, const float *vel_dev, const double prm[8],
                        const float *alp0_dev, const float *bet0_dev, const float *v0_dev,
                        double *out_dev, void *stream) {
    const char *fn = "abm_vswrm_integrals";
    if (rv < 2 || rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "%s: rv=%d", fn, rv);
    if (n_fields < 0) return set_error(ABM_ERR_INVALID_ARG, "%s: n_fields=%d", fn, n_fields);
    if (n_fields == 0) return ABM_OK;
    if (!bits_dev || !phi_host || !vel_dev || !prm || !out_dev)
        return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    int st;
    const GridDev *g = grid_for_phi(rv, phi_host, &st);
    if (!g) return st;
    VswrmArgs a;
    memset(&a, 0, sizeof(a));
    a.bits = bits_dev;
    a.vel = vel_dev;
    a.alp0 = alp0_dev;
    a.bet0 = bet0_dev;
    a.v0 = v0_dev;
    for (int k = 0; k < 8; ++k) a.prm[k] = prm[k];
    a.n = n_fields;
    a.out = out_dev;
    a.g = *g;
    const int threads = 256;
    const int blocks = (n_fields * 32 + threads - 1) / threads;
    vswrm_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(a);
    return check_cuda(cudaGetLastError(), "vswrm_kernel launch");
}

}  // extern "C"
