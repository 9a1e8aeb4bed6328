// vpf_edge.cu -- continuum edge form of the VSWRM integrals, forward step and hand-written
// adjoint (the differentiable form of the visual-flocking step).
//
// For focal agent i, neighbour j covers the arc [b_j - a_j, b_j + a_j] of the retina, with b_j
// the bearing (the reference's closed angle, vf_supcalc.py:142-158) and a_j the half visual
// angle atan(R/d_j) (the reference's pixel path, vf_supcalc.py:96-99) or asin(R/d_j).  The
// covered set U is the union of these arcs on the circle; with its merged arcs [l_m, u_m]
//   blob_c = -sum (sin u - sin l), blob_s = sum (cos u - cos l)    (trapz of -cos/sin(Phi) V)
//   edge_c =  sum (cos l + cos u), edge_s = sum (sin l + sin u)     (sum over dPhi_V^2 edges)
// which is the Rv -> infinity limit of the pixel form (vf_supcalc.py:233-238).  The update is
// the reference's (vf_agent.py:289-309, walls agent.py:347-394) with increments scaled by dt.
//
// One warp per focal agent: intervals are built in shared memory, bitonic-sorted by lower end,
// merged with a warp prefix-max scan that remembers which neighbour defines every arc end, and
// the seam is closed by folding the first arcs into the last one when it wraps past pi.  The
// adjoint kernel recomputes the same arcs from the step's input state (checkpoint-and-recompute)
// and propagates d loss / d(arc ends) to the bearings and half angles, hence to the focal
// heading and to both agents' positions (neighbour adjoints are scattered with atomics).
#include <cfloat>
#include <cstring>

#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

constexpr int kEdgeMaxN = 2048;      // agents per swarm in the edge form (intervals per warp)

// Scalar-type helpers: the edge form runs in float (FP32 pipe) or double (exact event order
// against an FP64 reference over long horizons; GB300's FP64 pipe is slow but N <= 2048).
__device__ __forceinline__ float m_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double m_atan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float m_atan(float x) { return atanf(x); }
__device__ __forceinline__ double m_atan(double x) { return atan(x); }
__device__ __forceinline__ float m_asin(float x) { return asinf(x); }
__device__ __forceinline__ double m_asin(double x) { return asin(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_rint(float x) { return rintf(x); }
__device__ __forceinline__ double m_rint(double x) { return rint(x); }
__device__ __forceinline__ void m_sincos(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ void m_sincos(double x, double *s, double *c) { sincos(x, s, c); }
template <typename T> struct Lim;
template <> struct Lim<float> { __device__ static constexpr float big() { return FLT_MAX; } };
template <> struct Lim<double> { __device__ static constexpr double big() { return DBL_MAX; } };

template <typename T>
struct EdgeArgs {
    const T *x, *y, *th, *v;                // state at t
    T *xo, *yo, *tho, *vo;                  // state at t + 1 (forward)
    const T *gx1, *gy1, *gth1, *gv1;        // adjoint of the state at t + 1 (backward)
    T *gx0, *gy0, *gth0, *gv0;              // adjoint of the state at t (accumulated)
    double *gparams;                        // d loss / d (alp0, alp1, bet0, bet1, v0)
    T *terms;                               // optional n x 4: blob_c, blob_s, edge_c, edge_s
    int n, use_asin, cap;
    T R, dt;
    T gam, v0, alp0, alp1, bet0, bet1;
    T bx0, bx1, by0, by1;
};

struct EdgeSmem {   // per-warp shared memory layout
    size_t key, up, id, pm, pmi, arc, total;
};

__host__ __device__ __forceinline__ size_t e_align(size_t b) { return (b + 15) & ~size_t(15); }

template <typename T>
struct EdgeArc {      // one merged arc: ends and the neighbours that define them
    T lo, hi;
    int lid, pos;     // pos: sorted position of the arc start, then the upper end's neighbour
};

template <typename T>
__host__ __device__ __forceinline__ EdgeSmem edge_smem(int cap) {
    EdgeSmem l;
    l.key = 0;
    l.up = e_align(l.key + (size_t)cap * sizeof(T));
    l.id = e_align(l.up + (size_t)cap * sizeof(T));
    l.pm = e_align(l.id + (size_t)cap * 4);
    l.pmi = e_align(l.pm + (size_t)cap * sizeof(T));
    l.arc = e_align(l.pmi + (size_t)cap * 4);
    l.total = e_align(l.arc + (size_t)cap * sizeof(EdgeArc<T>));
    return l;
}

template <typename T>
struct Arcs {
    T *lo, *hi;
    int *lid, *hid;   // neighbour index of the arc's lower / upper end
    int count;        // -1: the whole circle is covered
};

// Geometry of one pair: bearing b and half angle a of neighbour j seen from focal i.
template <typename T>
__device__ __forceinline__ void edge_geometry(T dx, T dy, T th, T R, int use_asin, T &b, T &a) {
    T bx = m_atan2(-dy, dx) - th;                    // math-frame bearing (y up), rel. heading
    bx = bx - T(6.283185307179586) * m_rint(bx * T(0.15915494309189535));   // to [-pi, pi]
    b = bx;
    const T d = m_sqrt(dx * dx + dy * dy);
    if (use_asin) a = (d > R) ? m_asin(R / d) : T(1.5707963267948966);
    else a = m_atan(R / d);
}

constexpr int kEdgeWarps = 4;   // warps per focal agent

template <typename T>
__device__ int edge_merge(unsigned char *smem, const EdgeSmem &L, int P, int lane, T kTwoPi,
                          const Arcs<T> &r);

// Builds the merged arcs of focal agent i in the block's shared memory: the intervals and
// their sort use every thread of the block, the scans over the sorted intervals warp 0.  The
// result is valid in every thread.
template <typename T>
__device__ Arcs<T> edge_arcs(const EdgeArgs<T> &p, int i, unsigned char *smem) {
    __shared__ int s_count;
    const int tid = threadIdx.x, lane = tid & 31, nthr = blockDim.x;
    const EdgeSmem L = edge_smem<T>(p.cap);
    T *key = reinterpret_cast<T *>(smem + L.key);
    T *up = reinterpret_cast<T *>(smem + L.up);
    int *id = reinterpret_cast<int *>(smem + L.id);
    const T xi = p.x[i], yi = p.y[i], th = p.th[i];
    const T kTwoPi = T(6.283185307179586), kPiT = T(3.141592653589793);
    // intervals (lower end in [-pi, pi), upper = lower + 2a), padded to a power of two
    const int P = p.cap;
    for (int j = tid; j < P; j += nthr) {
        T k = Lim<T>::big(), u = -Lim<T>::big();
        int jj = -1;
        if (j < p.n && j != i) {
            const T dx = p.x[j] - xi, dy = p.y[j] - yi;
            if (dx != T(0) || dy != T(0)) {   // vf_supcalc.py:57-58: same position is skipped
                T b, a;
                edge_geometry<T>(dx, dy, th, p.R, p.use_asin, b, a);
                T lo = b - a;
                if (lo < -kPiT) lo += kTwoPi;
                k = lo;
                u = lo + T(2) * a;
                jj = j;
            }
        }
        key[j] = k;
        up[j] = u;
        id[j] = jj;
    }
    __syncthreads();
    // bitonic sort by lower end
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = tid; t < P / 2; t += nthr) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const T kl = key[lo], kh = key[hi];
                if ((kl > kh) == asc) {
                    key[lo] = kh;
                    key[hi] = kl;
                    const T ul = up[lo];
                    up[lo] = up[hi];
                    up[hi] = ul;
                    const int il = id[lo];
                    id[lo] = id[hi];
                    id[hi] = il;
                }
            }
            __syncthreads();
        }
    }
    Arcs<T> r;
    r.lo = reinterpret_cast<T *>(smem + L.key);   // reuse key/up/id/pmi as arc arrays
    r.hi = reinterpret_cast<T *>(smem + L.up);
    r.lid = reinterpret_cast<int *>(smem + L.id);
    r.hid = reinterpret_cast<int *>(smem + L.pmi);
    if (tid < 32) s_count = edge_merge<T>(smem, L, P, lane, kTwoPi, r);
    __syncthreads();
    r.count = s_count;
    return r;
}

// Warp 0: merges the sorted intervals into arcs (prefix max of the upper ends, arc starts,
// closing ends, seam fold) and writes them to r; returns their count (-1: the whole circle).
template <typename T>
__device__ int edge_merge(unsigned char *smem, const EdgeSmem &L, int P, int lane, T kTwoPi,
                          const Arcs<T> &r) {
    T *key = reinterpret_cast<T *>(smem + L.key);
    T *up = reinterpret_cast<T *>(smem + L.up);
    int *id = reinterpret_cast<int *>(smem + L.id);
    T *pm = reinterpret_cast<T *>(smem + L.pm);
    int *pmi = reinterpret_cast<int *>(smem + L.pmi);
    EdgeArc<T> *arc = reinterpret_cast<EdgeArc<T> *>(smem + L.arc);
    // prefix max of the upper ends (with the index of the maximiser), chunk per lane
    const int C = P / 32;
    const int c0 = lane * C;
    T run = -Lim<T>::big();
    int runi = -1;
    for (int q = 0; q < C; ++q) {
        const T u = up[c0 + q];
        if (u > run) {
            run = u;
            runi = c0 + q;
        }
    }
    T carry = run;
    int carryi = runi;
    for (int o = 1; o < 32; o <<= 1) {   // inclusive scan of chunk maxima
        const T cv = __shfl_up_sync(ABM_FULL_MASK, carry, o);
        const int ci = __shfl_up_sync(ABM_FULL_MASK, carryi, o);
        if (lane >= o && cv > carry) {
            carry = cv;
            carryi = ci;
        }
    }
    T ex = __shfl_up_sync(ABM_FULL_MASK, carry, 1);   // exclusive
    int exi = __shfl_up_sync(ABM_FULL_MASK, carryi, 1);
    if (lane == 0) {
        ex = -Lim<T>::big();
        exi = -1;
    }
    run = ex;
    runi = exi;
    for (int q = 0; q < C; ++q) {
        const T u = up[c0 + q];
        if (u > run) {
            run = u;
            runi = c0 + q;
        }
        pm[c0 + q] = run;
        pmi[c0 + q] = runi;
    }
    __syncwarp();
    // arcs: an arc starts at sorted position k when key[k] > pm[k - 1]
    int K = 0;
    for (int kb = 0; kb < P; kb += 32) {
        const int k = kb + lane;
        const bool valid = id[k] >= 0;
        const bool start = valid && (k == 0 || key[k] > pm[k - 1]);
        const unsigned sm = __ballot_sync(ABM_FULL_MASK, start);
        if (start) {
            const int a = K + __popc(sm & ((1u << lane) - 1u));
            arc[a] = EdgeArc<T>{key[k], T(0), id[k], k};
        }
        K += __popc(sm);
    }
    __syncwarp();
    // close every arc at the position before the next start (valid entries sort first)
    int nvalid = 0;
    for (int kb = 0; kb < P; kb += 32) nvalid += __popc(__ballot_sync(ABM_FULL_MASK, id[kb + lane] >= 0));
    for (int ab = 0; ab < K; ab += 32) {   // read all next-start positions, then write
        const int a = ab + lane;
        int endpos = 0;
        if (a < K) endpos = (a + 1 < K) ? arc[a + 1].pos - 1 : nvalid - 1;
        __syncwarp();
        if (a < K) {
            EdgeArc<T> A = arc[a];
            A.hi = pm[endpos];
            A.pos = id[pmi[endpos]];
            arc[a] = A;
        }
        __syncwarp();
    }
    // seam: arcs whose lower end + 2 pi lies under the last arc's upper end fold into it
    if (K == 0) return 0;
    const EdgeArc<T> last = arc[K - 1];
    const T ulast = last.hi;
    int fold = 0;   // number of leading arcs folded into the last one
    for (int a = 0; a < K; ++a) {   // prefix: lower ends increase
        if (arc[a].lo + kTwoPi <= ulast) ++fold;
        else break;
    }
    if (fold >= K) return -1;   // the whole circle is covered: no edges, zero blob integrals
    T new_hi = ulast;
    int new_hid = last.pos;
    if (fold > 0) {
        const EdgeArc<T> pa = arc[fold - 1];
        if (pa.hi + kTwoPi > new_hi) {
            new_hi = pa.hi + kTwoPi;
            new_hid = pa.pos;
        }
    }
    __syncwarp();
    const int cnt = K - fold;
    for (int a = lane; a < cnt; a += 32) {
        const EdgeArc<T> A = arc[fold + a];
        r.lo[a] = A.lo;
        r.hi[a] = (fold + a == K - 1) ? new_hi : A.hi;
        r.lid[a] = A.lid;
        r.hid[a] = (fold + a == K - 1) ? new_hid : A.pos;
    }
    __syncwarp();
    return cnt;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(ABM_FULL_MASK, v, o);
    return v;
}

// Integrals of the covered set.
template <typename T>
__device__ __forceinline__ void edge_integrals(const Arcs<T> &A, T &bc, T &bs, T &ec, T &es) {
    const int lane = threadIdx.x & 31;
    bc = bs = ec = es = T(0);
    for (int a = lane; a < A.count; a += 32) {
        T sl, cl, su, cu;
        m_sincos(A.lo[a], &sl, &cl);
        m_sincos(A.hi[a], &su, &cu);
        bc -= su - sl;
        bs += cu - cl;
        ec += cl + cu;
        es += sl + su;
    }
    bc = warp_sum(bc);
    bs = warp_sum(bs);
    ec = warp_sum(ec);
    es = warp_sum(es);
}

template <typename T>
struct EdgeUpd {
    T th1, v1, x1, y1;          // new state
    T c1, s1;                   // cos/sin of the new heading
    int rx, ry;                 // wall hits that reset x / y
};

// Heading / speed / position update with dt and the wall rule (agent.py:347-394).
template <typename T>
__device__ __forceinline__ EdgeUpd<T> edge_update(const EdgeArgs<T> &p, T x, T y, T th, T v,
                                                  T dv, T dpsi) {
    const T kPI = T(3.141592653589793), k2PI = T(6.283185307179586);
    EdgeUpd<T> u;
    T t = th + dpsi * p.dt;
    if (t < T(0)) t += k2PI;
    if (t > k2PI) t -= k2PI;
    const T v1 = v + dv * p.dt;
    T s1, c1;
    m_sincos(t, &s1, &c1);
    T x1 = x + v1 * c1 * p.dt;
    T y1 = y - v1 * s1 * p.dt;
    u.rx = u.ry = 0;
    const T cx = x1 + p.R, cy = y1 + p.R;
    if (cx < p.bx0) {
        x1 = p.bx0 - p.R;
        u.rx = 1;
        if (kPI / 2 <= t && t < kPI) t -= kPI / 2;
        else if (kPI <= t && t <= T(3) * kPI / 2) t += kPI / 2;
        if (t < T(0)) t += k2PI;
        if (t > k2PI) t -= k2PI;
    }
    if (cx > p.bx1) {
        x1 = p.bx1 - p.R - T(1);
        u.rx = 1;
        if (T(3) * kPI / 2 <= t && t < k2PI) t -= kPI / 2;
        else if (T(0) <= t && t <= kPI / 2) t += kPI / 2;
        if (t < T(0)) t += k2PI;
        if (t > k2PI) t -= k2PI;
    }
    if (cy < p.by0) {
        y1 = p.by0 - p.R;
        u.ry = 1;
        if (kPI / 2 <= t && t <= kPI) t += kPI / 2;
        else if (T(0) <= t && t < kPI / 2) t -= kPI / 2;
        if (t < T(0)) t += k2PI;
        if (t > k2PI) t -= k2PI;
    }
    if (cy > p.by1) {
        y1 = p.by1 - p.R - T(1);
        u.ry = 1;
        if (T(3) * kPI / 2 <= t && t <= k2PI) t += kPI / 2;
        else if (kPI <= t && t < T(3) * kPI / 2) t -= kPI / 2;
        if (t < T(0)) t += k2PI;
        if (t > k2PI) t -= k2PI;
    }
    u.th1 = t;
    u.v1 = v1;
    u.x1 = x1;
    u.y1 = y1;
    u.c1 = c1;
    u.s1 = s1;
    return u;
}

template <typename T>
__global__ void __launch_bounds__(32 * kEdgeWarps) edge_fwd_kernel(const EdgeArgs<T> p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int i = blockIdx.x, lane = threadIdx.x;
    wait_primary_grid();   // programmatic launch: the previous step's state
    allow_dependent_launch();
    const Arcs<T> A = edge_arcs<T>(p, i, smem);
    if (threadIdx.x >= 32) return;   // integrals and update: warp 0
    T bc = 0, bs = 0, ec = 0, es = 0;
    if (A.count > 0) edge_integrals<T>(A, bc, bs, ec, es);
    if (lane == 0) {
        const T v = p.v[i];
        const T dv = p.gam * (p.v0 - v) + p.alp0 * bc + p.alp0 * p.alp1 * ec;
        const T dpsi = p.bet0 * bs + p.bet0 * p.bet1 * es;
        const EdgeUpd<T> u = edge_update<T>(p, p.x[i], p.y[i], p.th[i], v, dv, dpsi);
        p.xo[i] = u.x1;
        p.yo[i] = u.y1;
        p.tho[i] = u.th1;
        p.vo[i] = u.v1;
        if (p.terms) {
            T *t = p.terms + 4 * (size_t)i;
            t[0] = bc;
            t[1] = bs;
            t[2] = ec;
            t[3] = es;
        }
    }
}

// Adjoint of one step: given d loss / d state(t+1), accumulate d loss / d state(t) and the
// parameter gradients.  gx0.. must be zero before the launch (contributions are atomics).
template <typename T>
__global__ void __launch_bounds__(32 * kEdgeWarps) edge_bwd_kernel(const EdgeArgs<T> p) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ T s_terms[4], s_part[3][kEdgeWarps];
    const int i = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthr = blockDim.x;
    wait_primary_grid();   // programmatic launch: the previous step's adjoint
    allow_dependent_launch();
    const Arcs<T> A = edge_arcs<T>(p, i, smem);
    if (warp == 0) {   // integrals: warp 0, then shared with the block
        T tb = 0, tbs = 0, te = 0, tes = 0;
        if (A.count > 0) edge_integrals<T>(A, tb, tbs, te, tes);
        if (lane == 0) {
            s_terms[0] = tb;
            s_terms[1] = tbs;
            s_terms[2] = te;
            s_terms[3] = tes;
        }
    }
    __syncthreads();
    const T bc = s_terms[0], bs = s_terms[1], ec = s_terms[2], es = s_terms[3];
    const T x = p.x[i], y = p.y[i], th = p.th[i], v = p.v[i];
    const T dv = p.gam * (p.v0 - v) + p.alp0 * bc + p.alp0 * p.alp1 * ec;
    const T dpsi = p.bet0 * bs + p.bet0 * p.bet1 * es;
    const EdgeUpd<T> u = edge_update<T>(p, x, y, th, v, dv, dpsi);
    // ---- through the update (all lanes hold the same scalars)
    const T gx1 = p.gx1[i], gy1 = p.gy1[i], gth1 = p.gth1[i], gv1 = p.gv1[i];
    // x1 = x + v1 c1 dt (reset by a wall: constant), y1 = y - v1 s1 dt
    const T gxr = u.rx ? T(0) : gx1, gyr = u.ry ? T(0) : gy1;
    const T g_v1 = gv1 + gxr * u.c1 * p.dt - gyr * u.s1 * p.dt;
    const T g_t = gth1 + gxr * (-u.v1 * u.s1 * p.dt) + gyr * (-u.v1 * u.c1 * p.dt);
    const T g_x = gxr, g_y = gyr;
    // th1 = th + dpsi dt (+ constants), v1 = v + dv dt
    const T g_th = g_t;
    const T g_dpsi = g_t * p.dt;
    const T g_dv = g_v1 * p.dt;
    const T g_v = g_v1 - p.gam * g_dv;
    // dv = gam (v0 - v) + alp0 bc + alp0 alp1 ec ; dpsi = bet0 bs + bet0 bet1 es
    const T g_bc = g_dv * p.alp0, g_ec = g_dv * p.alp0 * p.alp1;
    const T g_bs = g_dpsi * p.bet0, g_es = g_dpsi * p.bet0 * p.bet1;
    // ---- through the arc ends to bearings / half angles, then to positions and heading
    T g_thf = 0, g_xf = 0, g_yf = 0;
    if (A.count > 0) {
        for (int a = tid; a < 2 * A.count; a += nthr) {
            const int arc = a >> 1;
            const bool upper = a & 1;
            const T e = upper ? A.hi[arc] : A.lo[arc];
            const int j = upper ? A.hid[arc] : A.lid[arc];
            T se, ce;
            m_sincos(e, &se, &ce);
            // d(bc, bs, ec, es)/d(end): upper: (-c, -s, -s, c); lower: (c, s, -s, c)
            const T ge = upper ? (g_bc * -ce + g_bs * -se + g_ec * -se + g_es * ce)
                               : (g_bc * ce + g_bs * se + g_ec * -se + g_es * ce);
            // end = b_j +/- a_j
            const T g_b = ge, g_a = upper ? ge : -ge;
            const T dx = p.x[j] - x, dy = p.y[j] - y;
            const T d2 = dx * dx + dy * dy, d = m_sqrt(d2);
            // b = atan2(-dy, dx) - th: db/ddx = dy/d2, db/ddy = -dx/d2, db/dth = -1
            T dadd;   // d a / d d
            if (p.use_asin) dadd = (d > p.R) ? -p.R / (d * m_sqrt(d2 - p.R * p.R)) : T(0);
            else dadd = -p.R / (d2 + p.R * p.R);
            const T gdx = g_b * (dy / d2) + g_a * dadd * (dx / d);
            const T gdy = g_b * (-dx / d2) + g_a * dadd * (dy / d);
            g_thf -= g_b;
            g_xf -= gdx;
            g_yf -= gdy;
            atomicAdd(&p.gx0[j], gdx);
            atomicAdd(&p.gy0[j], gdy);
        }
    }
    g_thf = warp_sum(g_thf);
    g_xf = warp_sum(g_xf);
    g_yf = warp_sum(g_yf);
    if (lane == 0) {
        s_part[0][warp] = g_thf;
        s_part[1][warp] = g_xf;
        s_part[2][warp] = g_yf;
    }
    __syncthreads();
    if (tid == 0) {
        g_thf = g_xf = g_yf = T(0);
        for (int w = 0; w < nthr / 32; ++w) {   // fixed order
            g_thf += s_part[0][w];
            g_xf += s_part[1][w];
            g_yf += s_part[2][w];
        }
        atomicAdd(&p.gx0[i], g_x + g_xf);
        atomicAdd(&p.gy0[i], g_y + g_yf);
        atomicAdd(&p.gth0[i], g_th + g_thf);
        atomicAdd(&p.gv0[i], g_v);
        // parameters: alp0, alp1, bet0, bet1, v0
        atomicAdd(&p.gparams[0], (double)(g_dv * (bc + p.alp1 * ec)));
        atomicAdd(&p.gparams[1], (double)(g_dv * p.alp0 * ec));
        atomicAdd(&p.gparams[2], (double)(g_dpsi * (bs + p.bet1 * es)));
        atomicAdd(&p.gparams[3], (double)(g_dpsi * p.bet0 * es));
        atomicAdd(&p.gparams[4], (double)(g_dv * p.gam));
    }
}

template <typename T, typename S>
static int edge_setup(const S *in, int32_t n, const abm_vf_params *p, int32_t use_asin,
                      EdgeArgs<T> &a, size_t &smem, const char *fn) {
    if (!p || !in) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    if (n < 0 || n > kEdgeMaxN)
        return set_error(ABM_ERR_INVALID_ARG, "%s: n=%d outside [0, %d]", fn, n, kEdgeMaxN);
    if (p->boundary != ABM_BOUNDARY_WALLS)
        return set_error(ABM_ERR_UNSUPPORTED, "%s: the edge form supports walls only", fn);
    if (!(p->radius > 0)) return set_error(ABM_ERR_INVALID_ARG, "%s: radius", fn);
    memset(&a, 0, sizeof(a));
    a.x = in->x;
    a.y = in->y;
    a.th = in->theta;
    a.v = in->v;
    a.n = n;
    a.use_asin = use_asin != 0;
    int P = 32;
    while (P < n) P <<= 1;
    a.cap = P;
    a.R = (T)p->radius;
    a.dt = (T)p->dt;
    a.gam = (T)p->gam;
    a.v0 = (T)p->v0;
    a.alp0 = (T)p->alp0;
    a.alp1 = (T)p->alp1;
    a.bet0 = (T)p->bet0;
    a.bet1 = (T)p->bet1;
    a.bx0 = (T)p->window_pad;
    a.bx1 = (T)(p->window_pad + p->width);
    a.by0 = (T)p->window_pad;
    a.by1 = (T)(p->window_pad + p->height);
    smem = edge_smem<T>(P).total;
    return ABM_OK;
}

template <typename T, typename S>
static int edge_fwd(const S *in, S *out, int32_t n, const abm_vf_params *p, int32_t use_asin,
                    T *terms_dev, void *stream, const char *fn) {
    EdgeArgs<T> a;
    size_t smem;
    int st = edge_setup<T, S>(in, n, p, use_asin, a, smem, fn);
    if (st || n == 0) return st;
    if (!out || !out->x || !out->y || !out->theta || !out->v)
        return set_error(ABM_ERR_INVALID_ARG, "%s: NULL output", fn);
    a.xo = out->x;
    a.yo = out->y;
    a.tho = out->theta;
    a.vo = out->v;
    a.terms = terms_dev;
    st = allow_dynamic_smem((const void *)edge_fwd_kernel<T>, 200 * 1024, "edge_fwd_kernel smem");
    if (st) return st;
    return check_cuda(launch_pdl(edge_fwd_kernel<T>, (unsigned)n, 32 * kEdgeWarps, smem,
                                 (cudaStream_t)stream, a),
                      "edge_fwd_kernel launch");
}

template <typename T, typename S>
static int edge_bwd(const S *in, const S *grad_out, S *grad_in, double *grad_params_dev,
                    int32_t n, const abm_vf_params *p, int32_t use_asin, void *stream,
                    const char *fn) {
    EdgeArgs<T> a;
    size_t smem;
    int st = edge_setup<T, S>(in, n, p, use_asin, a, smem, fn);
    if (st || n == 0) return st;
    if (!grad_out || !grad_in || !grad_params_dev)
        return set_error(ABM_ERR_INVALID_ARG, "%s: NULL gradient argument", fn);
    a.gx1 = grad_out->x;
    a.gy1 = grad_out->y;
    a.gth1 = grad_out->theta;
    a.gv1 = grad_out->v;
    a.gx0 = grad_in->x;
    a.gy0 = grad_in->y;
    a.gth0 = grad_in->theta;
    a.gv0 = grad_in->v;
    a.gparams = grad_params_dev;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t bytes = sizeof(T) * (size_t)n;
    T *const grads[4] = {a.gx0, a.gy0, a.gth0, a.gv0};
    if (a.gy0 == a.gx0 + n && a.gth0 == a.gy0 + n && a.gv0 == a.gth0 + n) {
        // one (4, n) array: one memset
        st = check_cuda(cudaMemsetAsync(a.gx0, 0, 4 * bytes, s), "cudaMemsetAsync(grad_in)");
        if (st) return st;
    } else {
        for (int k = 0; k < 4; ++k) {
            st = check_cuda(cudaMemsetAsync(grads[k], 0, bytes, s), "cudaMemsetAsync(grad_in)");
            if (st) return st;
        }
    }
    st = allow_dynamic_smem((const void *)edge_bwd_kernel<T>, 200 * 1024, "edge_bwd_kernel smem");
    if (st) return st;
    return check_cuda(launch_pdl(edge_bwd_kernel<T>, (unsigned)n, 32 * kEdgeWarps, smem, s, a),
                      "edge_bwd_kernel launch");
}

}  // namespace abm

using namespace abm;

extern "C" int abm_vpf_edge_fwd(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                                const abm_vf_params *p, int32_t use_asin, float *terms_dev,
                                void *stream) {
    return edge_fwd<float>(in, out, n, p, use_asin, terms_dev, stream, "abm_vpf_edge_fwd");
}

extern "C" int abm_vpf_edge_bwd(const abm_swarm_state *in, const abm_swarm_state *grad_out,
                                abm_swarm_state *grad_in, double *grad_params_dev, int32_t n,
                                const abm_vf_params *p, int32_t use_asin, void *stream) {
    return edge_bwd<float>(in, grad_out, grad_in, grad_params_dev, n, p, use_asin, stream,
                           "abm_vpf_edge_bwd");
}

extern "C" int abm_vpf_edge_fwd_f64(const abm_swarm_state_f64 *in, abm_swarm_state_f64 *out,
                                    int32_t n, const abm_vf_params *p, int32_t use_asin,
                                    double *terms_dev, void *stream) {
    return edge_fwd<double>(in, out, n, p, use_asin, terms_dev, stream, "abm_vpf_edge_fwd_f64");
}

extern "C" int abm_vpf_edge_bwd_f64(const abm_swarm_state_f64 *in,
                                    const abm_swarm_state_f64 *grad_out,
                                    abm_swarm_state_f64 *grad_in, double *grad_params_dev,
                                    int32_t n, const abm_vf_params *p, int32_t use_asin,
                                    void *stream) {
    return edge_bwd<double>(in, grad_out, grad_in, grad_params_dev, n, p, use_asin, stream,
                            "abm_vpf_edge_bwd_f64");
}
