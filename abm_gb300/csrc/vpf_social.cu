// vpf_social.cu -- the foraging variant's social VPF channel (Agent.calc_social_V_proj,
// abm/agent/agent.py:396-419, with Agent.projection_field :457-597 and the distance-ordered
// interval trimming exlude_V_source_data :421-445).
//
// One warp per focal agent (one block each).  Lanes classify the agents within vision range
// (exploiting agents of another patch are social cues, every other one only occludes), keep
// those inside the field of view with their untrimmed [start, end) pixel interval, rank them
// by distance (stable: ties keep the reference's list order), trim every interval against the
// strictly closer ones in ascending order, and OR the surviving social intervals into a
// bitmask that is finally flipped and FOV-masked like the reference's soc_v_field.  Pixel and
// width decisions use the same FP32 estimate + double-float re-decision as the flocking
// channel; the distance order is decided on exact double-float squared distances.
#include <cstring>

#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

struct SocialArgs {
    const float *x, *y, *th, *radius;
    const int *exploit, *patch;
    const float4 *sctab;     // df sincos table (global copy)
    float radius0;
    int n, visual_exclusion, patchwise, cap;
    dfl vr2;                 // vision_range^2
    int fov0_open, fov1_open;          // fov0 == -pi / fov1 == pi (no test needed)
    float fov0, fov1;                  // FP32 limits for the certain cases
    dfl f0c, f0s, f1c, f1s;            // cos/sin of the limits (double-float) near the limits
    int k_lo, k_hi;          // output pixels k with fov0 <= phis[k] <= fov1
    uint32_t *out;           // n x words, stored (flipped, FOV-masked) order
    unsigned long long *diag;
    GridDev g;
};

struct SocialEntry {
    float dkh, dkl;          // exact squared distance (double-float key)
    int ord;                 // position in the reference's obstacle list (group * n + index)
    int s0, e0;              // untrimmed int(t - ps/2), int(t + ps/2)
    int social;
};

// Sign of the angle from a direction (c, s) to the bearing atan2(-P, Q) (exact inputs;
// meaningful when the two are less than pi apart).
__device__ __forceinline__ int bearing_side(dfl P, dfl Q, dfl c, dfl s) {
    return -df_sign(df_add(df_mul(c, P), df_mul(s, Q)));
}

// Unsigned key ordered like the float (negative values below positive ones, -0 as +0, NaN
// above +inf).
__device__ __forceinline__ unsigned float_order_key(float v) {
    const unsigned b = __float_as_uint(v + 0.0f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// numpy slice a[lo:hi] = 1 on the raw bitmask (negative indices count from the end).
__device__ __forceinline__ void np_slice_fill(uint32_t *vb, int rv, int lo, int hi) {
    if (lo < 0) { lo += rv; if (lo < 0) lo = 0; }
    if (hi < 0) { hi += rv; if (hi < 0) hi = 0; }
    if (lo > rv) lo = rv;
    if (hi > rv) hi = rv;
    if (lo < hi) raster_run(vb, lo, hi);
}

static __host__ __device__ __forceinline__ size_t align16(size_t b) {
    return (b + 15) & ~size_t(15);
}

// Shared-memory carve-up of vpf_social_kernel: bitmask, entries, sorted index, trimmed
// intervals, the entries in rank order (distance keys and untrimmed interval, one 16-byte
// record each), each region starting on a 16-byte boundary.
struct SocialSmem {
    size_t ent, sidx, trim, srt, total;
};

static __host__ __device__ __forceinline__ SocialSmem social_smem(int words, int cap) {
    SocialSmem l;
    l.ent = align16((size_t)words * 4);
    l.sidx = align16(l.ent + (size_t)cap * sizeof(SocialEntry));
    l.trim = align16(l.sidx + (size_t)cap * sizeof(int));
    l.srt = align16(l.trim + (size_t)cap * sizeof(int2));
    l.total = align16(l.srt + (size_t)cap * sizeof(uint4));
    return l;
}

static size_t social_smem_bytes(int words, int cap) { return social_smem(words, cap).total; }

constexpr int kSocialWarps = 4;

__global__ void __launch_bounds__(32 * kSocialWarps) vpf_social_kernel(const SocialArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_count, s_over;
    __shared__ unsigned s_resolved, s_near;
    const int tid = threadIdx.x, lane = tid & 31, nthr = blockDim.x;
    const int i = blockIdx.x;
    const int words = a.g.words, rv = a.g.rv, cap = a.cap;
    wait_primary_grid();
    allow_dependent_launch();
    const SocialSmem L = social_smem(words, cap);
    uint32_t *vb = reinterpret_cast<uint32_t *>(smem);
    SocialEntry *ent = reinterpret_cast<SocialEntry *>(smem + L.ent);
    int *sidx = reinterpret_cast<int *>(smem + L.sidx);     // entries by ascending distance
    int2 *trim = reinterpret_cast<int2 *>(smem + L.trim);   // trimmed (start, end) per entry
    uint4 *srt = reinterpret_cast<uint4 *>(smem + L.srt);   // by rank: key hi, key lo, s0, e0
    // the first chunk of candidates is loaded now, overlapping the focal agent's set-up (the
    // loop below loads each next chunk while it classifies the current one)
    auto load_cand = [&](int j, float &xj, float &yj, float &rj, int &ej, int &pj) {
        if (j < a.n) {
            xj = a.x[j];
            yj = a.y[j];
            rj = a.radius ? a.radius[j] : a.radius0;
            ej = a.exploit[j];
            pj = a.patch[j];
        }
    };
    float cx_ = 0.f, cy_ = 0.f, cr_ = a.radius0;
    int ce_ = 0, cp_ = 0;
    load_cand(tid, cx_, cy_, cr_, ce_, cp_);
    for (int w = tid; w < words; w += nthr) vb[w] = 0u;
    if (tid == 0) {
        s_count = 0;
        s_over = 0;
        s_resolved = 0;
        s_near = 0;
    }

    const float xi = a.x[i], yi = a.y[i];
    const float ri = a.radius ? a.radius[i] : a.radius0;
    const int pi = a.patch[i];
    FocalDev f;
    f.x = xi;
    f.y = yi;
    f.r = ri;
    f.invr = 1.f / ri;
    df_sincos(a.th[i], a.sctab, f.cd, f.sd);
    f.c = f.cd.hi + f.cd.lo;
    f.s = f.sd.hi + f.sd.lo;
    const float band = 4e-6f;   // FP32 bearing error bound (1e-6 rad) with margin
    unsigned resolved = 0, nearc = 0;
    __syncthreads();

    // ---- obstacles: in vision range, classified, inside the FOV (one candidate per thread;
    // the entries' storage order is free: the rank below orders them)
    bool overflow = false;
    for (int jb = 0; jb < a.n; jb += nthr) {
        const int j = jb + tid;
        bool keep = false;
        SocialEntry e;
        const float xj = cx_, yj = cy_, rj = cr_;
        const int ej = ce_, pj = cp_;
        load_cand(j + nthr, cx_, cy_, cr_, ce_, cp_);
        if (j < a.n) {
            // supcalc.distance with each agent's own radius (agent.py:400)
            const dfl dr = two_sum(rj, -ri);
            const dfl ox = df_add(two_sum(xj, -xi), dr), oy = df_add(two_sum(yj, -yi), dr);
            const bool in_range =
                df_sign(df_sub(df_add(df_mul(ox, ox), df_mul(oy, oy)), a.vr2)) <= 0;
            // obstacle list groups (agent.py:402-413): 0 social, 1 non-exploiting in range
            // (incl. the focal agent), 2 exploiting on the focal agent's own patch; an
            // exploiter of patch -1 on another patch is dropped
            int group = -1;
            if (in_range) {
                const bool expl = (j != i) && ej;
                if (!expl) group = 1;
                else if (a.patchwise && pj == pi) group = 2;
                else if (pj != -1) group = 0;
            }
            if (group > 0 && !a.visual_exclusion) group = -1;  // occluders only with exclusion
            const bool same = (xj == xi) && (yj == yi);         // agent.py:500
            if (group >= 0 && !same) {
                // obstacle centre with the focal radius (agent.py:504-505): offset = positions
                const dfl px = two_sum(xj, -xi), py = two_sum(yj, -yi);
                const PairEst est = estimate_pair<false>(f, px.hi + px.lo, py.hi + py.lo, ri,
                                                         f.invr, a.g);
                int t = est.t, h = est.h;
                const float ca = est.ca;
                const bool near0 = !a.fov0_open && fabsf(ca - a.fov0) < band;
                const bool near1 = !a.fov1_open && fabsf(ca - a.fov1) < band;
                const bool near_axis = fabsf(ca) < band || fabsf(ca) > kPiF - band;
                bool in_fov;
                if (near0 || near1 || near_axis || est.unc_t || est.unc_h) {
                    ++resolved;
                    const dfl P = df_add(df_mul(f.cd, py), df_mul(f.sd, px));
                    const dfl Q = df_sub(df_mul(f.cd, px), df_mul(f.sd, py));
                    if (df_sign(P) == 0) {
                        // exactly ahead (ca = 2 pi) or behind (ca = pi): outside (-pi, pi)
                        in_fov = false;
                    } else {
                        const bool lo_ok = a.fov0_open ? true
                                           : (near0 ? bearing_side(P, Q, a.f0c, a.f0s) > 0
                                                    : ca > a.fov0);
                        const bool hi_ok = a.fov1_open ? true
                                           : (near1 ? bearing_side(P, Q, a.f1c, a.f1s) < 0
                                                    : ca < a.fov1);
                        in_fov = lo_ok && hi_ok;
                        if (in_fov && (est.unc_t || est.unc_h)) {
                            const int3 rs = resolve_pair(f.cd, f.sd, px, py, ri,
                                                         resolve_grid(a.g), est.unc_t,
                                                         est.unc_h, est.u, est.ps2, t, h);
                            t = rs.x;
                            h = rs.y;
                            nearc += rs.z;
                        }
                    }
                } else {
                    in_fov = (a.fov0_open || a.fov0 < ca) && (a.fov1_open || ca < a.fov1);
                }
                if (in_fov) {
                    // start = int(t - ps/2), end = int(t + ps/2): truncation toward zero with
                    // ps/2 = h + frac, frac in (0, 1)
                    e.s0 = (t - h >= 1) ? t - h - 1 : t - h;
                    e.e0 = t + h;
                    const dfl d2 = df_add(df_mul(px, px), df_mul(py, py));
                    e.dkh = d2.hi;
                    e.dkl = d2.lo;
                    e.ord = group * a.n + j;
                    e.social = group == 0;
                    keep = true;
                }
            }
        }
        const unsigned km = __ballot_sync(ABM_FULL_MASK, keep);
        int base = 0;
        if (lane == 0 && km) base = atomicAdd(&s_count, __popc(km));
        base = __shfl_sync(ABM_FULL_MASK, base, 0);
        const int pos = base + __popc(km & ((1u << lane) - 1u));
        if (keep) {
            if (pos < cap) ent[pos] = e;
            else overflow = true;
        }
    }
    if (__any_sync(ABM_FULL_MASK, overflow) && lane == 0) s_over = 1;
    __syncthreads();
    const bool over = s_over != 0;
    int m = over ? 0 : s_count;   // more obstacles than the capacity: reported, field empty

    // ---- stable ascending rank by exact squared distance (ties keep the list order): one
    // entry per thread, every other entry read at the same address by the whole block.  The
    // key compares as (hi, lo) bit patterns mapped to order-preserving unsigned integers, a
    // total order even for non-finite input, so the ranks are always a permutation.
    for (int e = tid; e < m; e += nthr) {
        const unsigned kh = float_order_key(ent[e].dkh), kl = float_order_key(ent[e].dkl);
        const int ko = ent[e].ord;
        int rank = 0;
#pragma unroll 4
        for (int q = 0; q < m; ++q) {
            const unsigned oh = float_order_key(ent[q].dkh), ol = float_order_key(ent[q].dkl);
            const int oo = ent[q].ord;
            rank += (oh < kh) || (oh == kh && ol < kl) || (oh == kh && ol == kl && oo < ko);
        }
        sidx[rank] = e;
        srt[rank] = make_uint4(kh, kl, (unsigned)ent[e].s0, (unsigned)ent[e].e0);
    }
    __syncthreads();
    // ---- trim each interval against the strictly closer ones, in ascending order (one
    // focal interval per thread; the closer ones read in rank order, one record each).  The
    // trimmed interval only shrinks inside the untrimmed one [s0, e0] or collapses to [0, 0],
    // which no later step changes, so a closer interval disjoint from [s0, e0] never acts:
    // only the intersecting ones enter the dependent chain of updates.
    for (int r = tid; r < m; r += nthr) {
        const int fe = sidx[r];
        const uint4 F = srt[r];
        const int s0 = (int)F.z, e0 = (int)F.w;
        int sx = s0, ex = e0;
        if (a.visual_exclusion) {
#pragma unroll 4
            for (int q = 0; q < r; ++q) {
                const uint4 I = srt[q];
                const int is0 = (int)I.z, ie0 = (int)I.w;
                const bool closer = (I.x < F.x) || (I.x == F.x && I.y < F.y);   // strictly
                if (!(closer && is0 <= e0 && ie0 >= s0)) continue;
                if (sx <= is0 && is0 <= ex) ex = is0;
                if (sx <= ie0 && ie0 <= ex) sx = ie0;
                if (is0 <= sx && ie0 >= ex) {
                    sx = 0;
                    ex = 0;
                }
            }
        }
        trim[fe] = make_int2(sx, ex);
    }
    __syncthreads();
    // ---- fill the surviving social intervals (agent.py:576-588)
    for (int e = tid; e < m; e += nthr) {
        if (!ent[e].social) continue;
        int s = trim[e].x, en = trim[e].y;
        if (s < 0) {
            np_slice_fill(vb, rv, rv + s, rv);
            s = 0;
        }
        if (en >= rv) {
            np_slice_fill(vb, rv, 0, en - rv);
            en = rv - 1;
        }
        np_slice_fill(vb, rv, s, en);
    }
    __syncthreads();
    // ---- flip and FOV mask (agent.py:591-595): out[k] = raw[rv - 1 - k], 0 outside the FOV
    const int shift = words * 32 - rv;
    uint32_t *dst = a.out + (size_t)i * words;
    for (int w = tid; w < words; w += nthr) {
        const uint32_t lo = __brev(vb[words - 1 - w]);
        const uint32_t hi = (w + 1 < words) ? __brev(vb[words - 2 - w]) : 0u;
        uint32_t word = shift ? __funnelshift_r(lo, hi, shift) : lo;
        const int k0 = w * 32;
        uint32_t keepm = ABM_FULL_MASK;
        if (k0 < a.k_lo) keepm &= (a.k_lo - k0 >= 32) ? 0u : (ABM_FULL_MASK << (a.k_lo - k0));
        const int top = min(a.k_hi, rv - 1) - k0;   // last kept bit of this word
        if (top < 31) keepm &= (top < 0) ? 0u : (ABM_FULL_MASK >> (31 - top));
        dst[w] = word & keepm;
    }
    const unsigned tr = __reduce_add_sync(ABM_FULL_MASK, resolved);
    const unsigned tn = __reduce_add_sync(ABM_FULL_MASK, nearc);
    if (lane == 0 && (tr || tn)) {
        atomicAdd(&s_resolved, tr);
        atomicAdd(&s_near, tn);
    }
    __syncthreads();
    if (a.diag && tid == 0) {
        if (s_resolved) atomicAdd(&a.diag[ABM_DIAG_PAIRS_RESOLVED], (unsigned long long)s_resolved);
        if (s_near) atomicAdd(&a.diag[ABM_DIAG_NEAR_BOUNDARY], (unsigned long long)s_near);
        if (over) atomicAdd(&a.diag[ABM_DIAG_CAPACITY], 1ull);
    }
}

}  // namespace abm

using namespace abm;

extern "C" int abm_vpf_social_fields(const float *x_dev, const float *y_dev,
                                     const float *theta_dev, const float *radius_dev,
                                     double radius, const int32_t *exploit_dev,
                                     const int32_t *patch_dev, int32_t n, double vision_range,
                                     int32_t visual_exclusion, int32_t patchwise, int32_t rv,
                                     double fov0, double fov1, uint32_t *out_bits_dev,
                                     unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_social_fields";
    if (n < 0) return set_error(ABM_ERR_INVALID_ARG, "%s: n=%d", fn, n);
    if (rv < 2 || rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "%s: rv=%d", fn, rv);
    if (n == 0) return ABM_OK;
    if (!x_dev || !y_dev || !theta_dev || !exploit_dev || !patch_dev || !out_bits_dev)
        return set_error(ABM_ERR_INVALID_ARG, "%s: NULL array", fn);
    if (!radius_dev && !(radius > 0))
        return set_error(ABM_ERR_INVALID_ARG, "%s: radius=%g", fn, radius);
    if (!(fov0 >= -kPi && fov1 <= kPi && fov0 < fov1))
        return set_error(ABM_ERR_INVALID_ARG, "%s: fov must satisfy -pi <= fov0 < fov1 <= pi",
                         fn);
    int st;
    const GridDev *g = grid_for(rv, fov0, fov1, &st);
    if (!g) return st;
    const float4 *tab = sincos_table_dev(&st);
    if (!tab) return st;
    SocialArgs a;
    memset(&a, 0, sizeof(a));
    a.x = x_dev;
    a.y = y_dev;
    a.th = theta_dev;
    a.radius = radius_dev;
    a.exploit = exploit_dev;
    a.patch = patch_dev;
    a.sctab = tab;
    a.radius0 = (float)radius;
    a.n = n;
    a.visual_exclusion = visual_exclusion != 0;
    a.patchwise = patchwise != 0;
    a.cap = std::min(n, 4096);
    const double vr2 = vision_range * vision_range;
    a.vr2 = {(float)vr2, (float)(vr2 - (double)(float)vr2)};
    a.fov0_open = fov0 <= -kPi;
    a.fov1_open = fov1 >= kPi;
    a.fov0 = (float)fov0;
    a.fov1 = (float)fov1;
    auto split = [](double v) { return dfl{(float)v, (float)(v - (double)(float)v)}; };
    a.f0c = split(std::cos(fov0));
    a.f0s = split(std::sin(fov0));
    a.f1c = split(std::cos(fov1));
    a.f1s = split(std::sin(fov1));
    {   // output pixels k with fov0 <= phis[k] <= fov1 (agent.py:594-595 zero the rest)
        std::vector<double> phis;
        np_linspace_pi(rv, phis);
        int lo = rv, hi = -1;
        for (int k = 0; k < rv; ++k) {
            if (!(phis[k] < fov0) && !(phis[k] > fov1)) {
                lo = std::min(lo, k);
                hi = std::max(hi, k);
            }
        }
        a.k_lo = lo;
        a.k_hi = hi;
    }
    a.out = out_bits_dev;
    a.diag = diag_dev;
    a.g = *g;
    const size_t smem = social_smem_bytes(g->words, a.cap);
    if ((st = allow_dynamic_smem((const void *)vpf_social_kernel, (int)smem,
                                 "vpf_social_kernel smem")))
        return st;
    return check_cuda(launch_pdl(vpf_social_kernel, (unsigned)n, 32 * kSocialWarps, smem,
                                 (cudaStream_t)stream, a),
                      "vpf_social_kernel launch");
}
