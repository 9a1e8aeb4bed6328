// vpf_step.cu -- the per-timestep hot path (VPF rasterisation + VSWRM integrals + agent update)
// and the drop-in twins of projection_field / VSWRM_flocking_state_variables.
//
// One step is two launches.  The pair kernel evaluates every neighbour of its focal agents
// (FP32 with a guard band and a double-float re-decision inside it), OR-s the visible pixel runs
// into each agent's VPF bitmask in shared memory and reduces the bitmask's transitions to the
// four VSWRM sums (fixed point).  The second kernel (the update kernel, or the finish kernel
// after a pair kernel split into neighbour chunks, which also reduces the sums) applies the
// reference's heading / speed / position update and boundary rule in double-float arithmetic
// on the FP32 pipe (GB300's FP64 rate is a small fraction of its FP32 rate).  Forms of the
// pair kernel:
//  * `group`: one warp per group of 4 consecutive agents of one swarm (8 entries of a batched
//    sweep's schedule), each neighbour read once for the group (equal radii; walls, or a torus
//    whose width and height are floats);
//  * `l1`: single-warp blocks, one focal agent each, neighbours read through the read-only L1
//    path (per-agent radii, the other tori);
//  * `tiled`: several focal warps per block share neighbour tiles staged in shared memory by the
//    TMA bulk engine (double-buffered with mbarriers), for swarms whose positions exceed L1.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

constexpr int kMaxChunkRounds = 16;

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
    GridDev g;
    UpdateDf ud;           // the update's parameters in double-float
    const float4 *sctab;   // global copy of the double-float sincos table
    long long *sums;       // n x 4 workspace: bc, bs, ec, es of every agent
    // split l1 form: block b works on neighbour chunk (b & (2^chunk_shift - 1)) of agent
    // b >> chunk_shift (chunk_len neighbours, a multiple of 32) and ORs its partial bitmask
    // into vbits (n x words, zero between steps); NULL for the one-block-per-agent form
    uint32_t *vbits;
    int chunk_shift, chunk_len;
    // single-swarm group form, round-major chunk plan (chunk_rounds > 0): block b works on
    // neighbours [chunk_off[r], chunk_off[r + 1]) of group b - r * groups, r = b / groups
    int chunk_rounds, groups;
    int chunk_off[kMaxChunkRounds + 1];
    // x and y 8-byte aligned: the l1 form reads two adjacent neighbours per lane (walls, equal
    // radii)
    int pair_loads;
    // batched sweeps: agent i sees the agents [seg_begin[i], seg_end[i]) of its instance;
    // block b works on agent order[b] (largest instances first); all NULL for one swarm
    const int *seg_begin, *seg_end, *order;
};

static int g_warps = 8;    // tiled form: focal warps per block
static int g_tile = 8192;  // tiled form: neighbour tile length
static int g_mode = 0;     // 0 auto, 1 l1, 2 tiled, 3 group
static int g_wpa = 1;      // l1 form: warps per focal agent
static int g_split = 0;    // l1 form: neighbour chunks per agent (0 auto, else a power of two)
static std::mutex g_cfg_mu;

// cos/sin(k 2pi/1024) as double-float pairs, read with warp-uniform indices (constant cache).
__constant__ float4 c_sincos[kSinCosTab];

// Status word of the step kernels on this device (kStatusWaitTimeout: a block's bounded wait
// gave up); read and cleared by abm_vpf_status.  A module global: no allocation.
__device__ unsigned int g_kernel_status = 0u;

static int ensure_sincos_table() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && done[dev]) return ABM_OK;
    float4 tab[kSinCosTab];
    for (int k = 0; k < kSinCosTab; ++k) {
        const long double a = (long double)k * 2.0L * 3.14159265358979323846264338327950288L /
                              (long double)kSinCosTab;
        const long double c = cosl(a), sn = sinl(a);
        const float ch = (float)c, sh = (float)sn;
        tab[k] = make_float4(ch, (float)(c - (long double)ch), sh, (float)(sn - (long double)sh));
    }
    int st = check_cuda(cudaMemcpyToSymbol(c_sincos, tab, sizeof(tab)), "sincos table upload");
    if (!st && dev < 64) done[dev] = true;
    return st;
}

// Per-(device, stream) workspace: the split form's per-agent bitmasks (zero between steps: the
// finish kernel clears what the pair kernel set) at offset 0, then the per-agent sums handed
// to the update (32 B per agent).  Zeroed when allocated.  A workspace that grows is replaced
// but the old one stays allocated, since a CUDA graph captured from the stream may still use
// it.
struct Workspace {
    uint32_t *vbits = nullptr;
    long long *sums = nullptr;
};

static Workspace workspace(cudaStream_t stream, int n, int words, int *status) {
    struct Entry {
        unsigned char *p = nullptr;
        long agents = 0;
        size_t vbits_bytes = 0;
    };
    static std::mutex mu;
    static std::map<std::pair<int, void *>, Entry> ws;
    static std::vector<void *> retired;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    Entry &e = ws[{dev, (void *)stream}];
    const size_t vb_need = ((size_t)n * words * 4 + 255) & ~size_t(255);
    if (e.agents < n || e.vbits_bytes < vb_need) {
        Entry ne;
        ne.agents = std::max<long>({(long)n, e.agents, 1024L});
        ne.vbits_bytes = std::max(vb_need, e.vbits_bytes);
        const size_t bytes = ne.vbits_bytes + (size_t)ne.agents * 32;
        *status = check_cuda(cudaMalloc((void **)&ne.p, bytes), "cudaMalloc(step workspace)");
        if (*status) return Workspace();
        *status = check_cuda(cudaMemsetAsync(ne.p, 0, bytes, stream), "cudaMemsetAsync(workspace)");
        if (*status) {
            cudaFree(ne.p);
            return Workspace();
        }
        if (e.p) retired.push_back(e.p);
        e = ne;
    }
    *status = ABM_OK;
    Workspace w;
    w.vbits = (uint32_t *)e.p;
    w.sums = (long long *)(e.p + e.vbits_bytes);
    return w;
}

// Per-(device, stream) staging of abm_vpf_flock_step_host: the input state (4 n floats)
// followed by room for the output state (used when the caller's output is not addressable).
static float *host_staging(cudaStream_t stream, int n, int *status) {
    static std::mutex mu;
    static std::map<std::pair<int, void *>, std::pair<float *, long>> st;
    static std::vector<void *> retired;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto &e = st[{dev, (void *)stream}];
    if (e.second < n) {
        const long cap = std::max<long>(n, 1024);
        float *p = nullptr;
        *status = check_cuda(cudaMalloc((void **)&p, sizeof(float) * 8 * (size_t)cap),
                             "cudaMalloc(host staging)");
        if (*status) return nullptr;
        if (e.first) retired.push_back(e.first);
        e = {p, cap};
    }
    *status = ABM_OK;
    return e.first;
}

// Device-usable address of an array registered with CUDA (page-locked host memory, managed or
// device memory), else NULL: unregistered (pageable) memory is only ever copied by the driver.
static void *device_view(const void *host) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeManaged ||
        at.type == cudaMemoryTypeDevice)
        return at.devicePointer;
    return nullptr;
}

// Per-warp work queues of the step kernel: candidate neighbours that survived the cull (their
// positions, so the queue outlives the tile) and pairs whose FP32 decision needs the
// double-float re-decision.
constexpr int kQueue = 96;    // < 32 left + up to 64 appended per phase-A round
constexpr int kQueue2 = 64;
constexpr int kQueueW = 64;   // runs longer than 32 pixels or wrapping at the seam (s, e)

// A queued candidate.  Equal radii: the pair's FP32 centre offset, d^2 and the neighbour's
// index (so phase B starts from the offset, and the rare double-float re-decision reloads the
// neighbour's position); per-agent radii: the neighbour's position and radius.
template <bool HETERO>
struct QEntry;
template <>
struct QEntry<false> {
    float4 v;   // dx, dy, d^2, index (int bits)
    __device__ __forceinline__ int j() const { return __float_as_int(v.w); }
    __device__ __forceinline__ static QEntry make(float dx, float dy, float d2, int j) {
        return QEntry{make_float4(dx, dy, d2, __int_as_float(j))};
    }
};
template <>
struct QEntry<true> {
    float4 v;
    __device__ __forceinline__ float x() const { return v.x; }
    __device__ __forceinline__ float y() const { return v.y; }
    __device__ __forceinline__ float r(float) const { return v.z; }
    __device__ __forceinline__ static QEntry make(float x, float y, float r) {
        return QEntry{make_float4(x, y, r, 0.f)};
    }
};

// Transition-list capacity of a warp's drained queues (both queues, 4 B entries).
template <bool HETERO>
constexpr int kListCap = (kQueue + kQueue2) * (int)sizeof(QEntry<HETERO>) / 4;

// ---------------------------------------------------------------------------- no-alloc scratch
// Scratch of abm_vpf_flock_step_noalloc, for callers that cannot allocate device memory: the
// per-agent sums (up to kNoAllocMaxAgents agents), one grid's lookup tables (Rv up to
// kNoAllocMaxRv) and the double-float sincos table, carved out of one file-scope array that
// every GPU loading the library holds until the process exits (about 2.5 MiB).
constexpr int kNoAllocMaxAgents = 65536;
constexpr int kNoAllocMaxRv = 8192;
constexpr size_t kNaAlign = 256;
constexpr size_t na_round(size_t b) { return (b + kNaAlign - 1) & ~(kNaAlign - 1); }
constexpr size_t kNaSums = 0;
constexpr size_t kNaSin = kNaSums + na_round(32ull * kNoAllocMaxAgents);
constexpr size_t kNaMid = kNaSin + na_round(sizeof(float4) * kSinCosTab);
constexpr size_t kNaCot2 = kNaMid + na_round(sizeof(float4) * kNoAllocMaxRv);
constexpr size_t kNaQ = kNaCot2 + na_round(sizeof(float2) * (kNoAllocMaxRv / 4 + 2));
constexpr size_t kNaCpt = kNaQ + na_round(sizeof(longlong2) * (kNoAllocMaxRv + 1));
constexpr size_t kNaBytes = kNaCpt + na_round(sizeof(longlong2) * kNoAllocMaxRv);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct NoAllocDevice {
    std::mutex mu;                   // serialises the host-side state below and its uploads
    unsigned char *base = nullptr;   // device address of g_noalloc_scratch on this device
    bool sincos_loaded = false;
    bool grid_loaded = false;        // which grid's tables the array holds
    int rv = 0;
    double fov0 = 0, fov1 = 0;
    GridDev g;
};

// The current device's no-alloc record; set-up once per device (with that device current):
// the device address of the scratch array.  Call with the record's mutex held.
static NoAllocDevice *noalloc_device(int *status) {
    static NoAllocDevice devs[64];
    int dev = 0;
    *status = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (*status) return nullptr;
    if (dev < 0 || dev >= 64) {
        *status = set_error(ABM_ERR_UNSUPPORTED, "device %d beyond the no-alloc table", dev);
        return nullptr;
    }
    *status = ABM_OK;
    return &devs[dev];
}

// The rare paths of the per-agent forms (L1 and tiled), out of line so that the inlined copies
// of phase B stay small, as in the group forms.
//
// 32 queued long or wrapping runs of one agent's bitmask (one per lane) through the general
// fill.
static __device__ __noinline__ void drain_runs_one(const int2 *wq, uint32_t *vb, int rv) {
    const int lane = threadIdx.x & 31;
    const int2 r = wq[lane];
    raster_projection(vb, rv, r.x, r.y);
}

// Double-float re-decision and rasterisation of focal agent f's deferred pairs qe[0 .. cnt)
// (one per lane); returns the ballot of the pairs with a re-decided boundary within 1e-9 rad of
// their edge angle.
template <bool TORUS, bool HETERO>
static __device__ __noinline__ unsigned drain_deferred_one(const FocalDev f,
                                                           const QEntry<HETERO> *qe, int cnt,
                                                           uint32_t *vb, const float *x,
                                                           const float *y, float R0, dfl W,
                                                           dfl H, GridDev g) {
    const int lane = threadIdx.x & 31;
    bool near = false;
    if (lane < cnt) {
        float xj, yj, rj;
        if constexpr (HETERO) {
            xj = qe[lane].x();
            yj = qe[lane].y();
            rj = qe[lane].r(R0);
        } else {
            const int j = qe[lane].j();
            xj = __ldg(x + j);
            yj = __ldg(y + j);
            rj = R0;
        }
        float dx, dy;
        pair_offset<TORUS, HETERO>(f, xj, yj, rj, W, H, dx, dy);
        const PairEst de = estimate_pair<HETERO>(f, dx, dy, rj, HETERO ? rcp_approx(rj) : f.invr,
                                                 g);
        dfl ex, ey;
        exact_offset<TORUS, HETERO>(f, xj, yj, rj, W, H, ex, ey);
        const int3 th = resolve_pair(f.cd, f.sd, ex, ey, rj, resolve_grid(g), de.unc_t,
                                     de.unc_h, de.u, de.ps2, de.t, de.h);
        const int ds = th.x - th.y, dn = th.x + th.y;
        if (projection_visible(g, ds, dn)) raster_fast(vb, g.rv, ds, dn);
        near = th.z != 0;
    }
    return __ballot_sync(ABM_FULL_MASK, near);
}

// Heavy decision + rasterisation of up to 32 queued candidates (lane < cnt holds one).
template <bool TORUS, bool HETERO, bool FULL = false>
__device__ __forceinline__ void process_candidates(const FocalDev &f, const QEntry<HETERO> *q,
                                                   int cnt, QEntry<HETERO> *q2, int &q2n,
                                                   int2 *wq, int &wqn, uint32_t *vb,
                                                   const StepArgs &a, unsigned *cnt_resolved,
                                                   unsigned *cnt_near) {
    const int lane = threadIdx.x & 31;
    const bool have = FULL || lane < cnt;   // FULL: a batch of 32, every lane has a candidate
    bool unc;
    int s, en;
    QEntry<HETERO> e;
    if constexpr (!HETERO) {
        // from the queued offset; overlapping discs and guard-band decisions are deferred
        e = (FULL || have) ? q[lane] : QEntry<false>::make(1.f, 0.f, 1.f, 0);
        const FastEst est = estimate_fast(f, e.v.x, e.v.y, e.v.z, f.r, f.r * f.r, a.g);
        unc = have && est.unc;
        s = est.t - est.h;
        en = est.t + est.h;
        const bool vis = have && !est.unc && (a.g.full_fov || projection_visible(a.g, s, en));
        const unsigned len = (unsigned)(en - s);
        const bool short_run = s >= 0 && en < a.g.rv && len <= 32u;
        if (vis && short_run) raster_short(vb, s, len);
        // long and wrapping runs wait in the warp's run queue, drained 32 at a time, so that
        // the rare lane that needs the general fill does not hold up the other 31
        const unsigned wm = __ballot_sync(ABM_FULL_MASK, vis && !short_run);
        if (wm) {
            if (vis && !short_run) wq[wqn + __popc(wm & ((1u << lane) - 1u))] = make_int2(s, en);
            wqn += __popc(wm);
            __syncwarp();
            if (wqn >= 32) {
                wqn -= 32;
                drain_runs_one(wq + wqn, vb, a.g.rv);
                __syncwarp();
            }
        }
    } else {
        e = (FULL || have) ? q[lane] : QEntry<true>::make(f.x, f.y, f.r);
        const float xj = e.x(), yj = e.y(), rj = e.r(a.radius0);
        float dx, dy;
        pair_offset<TORUS, HETERO>(f, xj, yj, rj, a.W, a.H, dx, dy);
        const PairEst est = estimate_pair<HETERO>(f, dx, dy, rj, rcp_approx(rj), a.g);
        unc = have && (est.unc_t || est.unc_h);
        s = est.t - est.h;
        en = est.t + est.h;
        if (have && !unc && projection_visible(a.g, s, en)) raster_fast(vb, a.g.rv, s, en);
    }
    const unsigned um = __ballot_sync(ABM_FULL_MASK, unc);
    if (um) {  // defer the uncertain ones to the double-float queue
        if (unc) q2[q2n + __popc(um & ((1u << lane) - 1u))] = e;
        q2n += __popc(um);
    }
    __syncwarp();
    if (q2n >= 32) {   // drain 32 deferred pairs (warp-uniform)
        q2n -= 32;
        const unsigned nm = drain_deferred_one<TORUS, HETERO>(f, q2 + q2n, 32, vb, a.x, a.y,
                                                              a.radius0, a.W, a.H, a.g);
        if (lane == 0) {
            atomicAdd(cnt_resolved, 32u);
            if (nm) atomicAdd(cnt_near, (unsigned)__popc(nm));
        }
        __syncwarp();
    }
}

// The last (< 32) queued long or wrapping runs.
__device__ __forceinline__ void flush_runs(const int2 *wq, int wqn, uint32_t *vb, int rv) {
    const int lane = threadIdx.x & 31;
    if (wqn == 0) return;
    if (lane < wqn) {
        const int2 r = wq[lane];
        raster_projection(vb, rv, r.x, r.y);
    }
    __syncwarp();
}

// Double-float resolution of the last (< 32) deferred pairs.
template <bool TORUS, bool HETERO>
__device__ __forceinline__ void drain_deferred(const FocalDev &f, const QEntry<HETERO> *q2,
                                               int q2n, uint32_t *vb, const StepArgs &a,
                                               unsigned *cnt_resolved, unsigned *cnt_near) {
    const int lane = threadIdx.x & 31;
    if (q2n == 0) return;
    const unsigned nm = drain_deferred_one<TORUS, HETERO>(f, q2, q2n, vb, a.x, a.y, a.radius0,
                                                          a.W, a.H, a.g);
    if (lane == 0) {
        atomicAdd(cnt_resolved, (unsigned)q2n);
        if (nm) atomicAdd(cnt_near, (unsigned)__popc(nm));
    }
    __syncwarp();
}

// Focal agent of a warp: float32 state plus cos/sin(theta) in double-float (FP32 pipe only).
template <bool HETERO>
__device__ __forceinline__ FocalDev load_focal(const StepArgs &a, int i) {
    FocalDev f;
    f.x = a.x[i];
    f.y = a.y[i];
    f.r = HETERO ? a.radius[i] : a.radius0;
    f.invr = 1.f / f.r;
    df_sincos(a.th[i], c_sincos, f.cd, f.sd);
    f.c = f.cd.hi + f.cd.lo;
    f.s = f.sd.hi + f.sd.lo;
    return f;
}

// Phase A for one lane's neighbour j: the exact-zero / cull test of vf_supcalc.py:57-58 and
// h = 0 (projections narrower than 2 pixels never fill anything); the live candidate is
// appended to the warp queue, and phase B runs on every full batch of 32.
template <bool TORUS, bool HETERO>
__device__ __forceinline__ void phase_a(const FocalDev &f, float xj, float yj, float rj, int j,
                                        bool valid, float cull_r2, QEntry<HETERO> *q, int &qn,
                                        QEntry<HETERO> *q2, int &q2n, int2 *wq, int &wqn,
                                        uint32_t *vb, const StepArgs &a, unsigned *counters) {
    const int lane = threadIdx.x & 31;
    float dx, dy;
    pair_offset<TORUS, HETERO>(f, xj, yj, rj, a.W, a.H, dx, dy);
    const float d2 = fmaf(dx, dx, dy * dy);
    bool live;
    if constexpr (HETERO) {
        const bool same = (xj == f.x) && (yj == f.y);
        live = valid && !same && d2 <= rj * rj * a.g.cull;
    } else {
        live = valid && d2 > 0.f && d2 <= cull_r2;   // equal radii: same position <=> zero offset
    }
    const unsigned lm = __ballot_sync(ABM_FULL_MASK, live);
    if (live) {
        QEntry<HETERO> *slot = q + qn + __popc(lm & ((1u << lane) - 1u));
        if constexpr (HETERO) *slot = QEntry<true>::make(xj, yj, rj);
        else *slot = QEntry<false>::make(dx, dy, d2, j);
    }
    qn += __popc(lm);
    __syncwarp();
    if (qn >= 32) {   // warp-uniform
        qn -= 32;
        process_candidates<TORUS, HETERO, true>(f, q + qn, 32, q2, q2n, wq, wqn, vb, a,
                                                &counters[0], &counters[1]);
    }
}

// Warp epilogue of a focal agent: VSWRM integrals (listing the transitions in the warp's
// drained queue space), the optional bitmask output and (lane 0) the sums for the update.
__device__ __forceinline__ void finish_agent(const StepArgs &a, int i, const uint32_t *vb,
                                             uint32_t *list, int cap) {
    const int lane = threadIdx.x & 31;
    long long bc, bs, ec, es;
    if (a.seg_begin) warp_integrals_loop(vb, a.g, bc, bs, ec, es);   // small batched swarms
    else warp_integrals(vb, a.g, list, cap, bc, bs, ec, es);
    if (a.bits) {
        uint32_t *dst = a.bits + (size_t)i * a.g.words;
        for (int w = lane; w < a.g.words; w += 32) dst[w] = vb[w];
    }
    if (lane == 0) {
        longlong2 *sp = reinterpret_cast<longlong2 *>(a.sums) + 2 * (size_t)i;
        sp[0] = make_longlong2(bc, bs);
        sp[1] = make_longlong2(ec, es);
    }
}

__device__ __forceinline__ void flush_counters(const StepArgs &a, const unsigned *counters) {
    if (!a.diag) return;
    if (counters[0]) atomicAdd(&a.diag[ABM_DIAG_PAIRS_RESOLVED], (unsigned long long)counters[0]);
    if (counters[1]) atomicAdd(&a.diag[ABM_DIAG_NEAR_BOUNDARY], (unsigned long long)counters[1]);
    if (counters[2]) atomicAdd(&a.diag[ABM_DIAG_TIMEOUTS], (unsigned long long)counters[2]);
}

// ---------------------------------------------------------------------------- l1 form
// One block = one focal agent, WPA warps share its bitmask and split its neighbours.
static size_t l1_smem_bytes(int wpa, int words, bool hetero) {
    const size_t qe = sizeof(QEntry<false>);
    (void)hetero;
    size_t b = (size_t)words * sizeof(uint32_t);
    b = (b + 15) & ~size_t(15);
    b += (size_t)wpa * ((kQueue + kQueue2) * qe + kQueueW * sizeof(int2));
    return b + 16;
}

template <bool TORUS, bool HETERO, int WPA>
__global__ void __launch_bounds__(32 * WPA) vpf_pairs_l1_kernel(const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int words = a.g.words;
    const bool split = a.vbits != nullptr;
    wait_primary_grid();   // the previous step's state (programmatic launch)
    const int i = a.order ? a.order[blockIdx.x] : (blockIdx.x >> a.chunk_shift);
    int j0 = a.seg_begin ? a.seg_begin[i] : 0;
    int n = a.seg_end ? a.seg_end[i] : a.n;   // neighbours are [j0, n)
    if (split) {
        j0 = (blockIdx.x & ((1 << a.chunk_shift) - 1)) * a.chunk_len;
        n = min(n, j0 + a.chunk_len);
    }
    uint32_t *vb = reinterpret_cast<uint32_t *>(smem);
    size_t off = ((size_t)words * 4 + 15) & ~size_t(15);
    QEntry<HETERO> *q = reinterpret_cast<QEntry<HETERO> *>(smem + off) + warp * (kQueue + kQueue2);
    QEntry<HETERO> *q2 = q + kQueue;
    off += (size_t)WPA * (kQueue + kQueue2) * sizeof(QEntry<HETERO>);
    int2 *wq = reinterpret_cast<int2 *>(smem + off) + warp * kQueueW;
    off += (size_t)WPA * kQueueW * sizeof(int2);
    unsigned *counters = reinterpret_cast<unsigned *>(smem + off);

    for (int w = threadIdx.x; w < words; w += 32 * WPA) vb[w] = 0u;
    if (threadIdx.x < 4) counters[threadIdx.x] = 0u;
    allow_dependent_launch();
    const FocalDev f = load_focal<HETERO>(a, i);
    const float cull_r2 = f.r * f.r * a.g.cull;
    if (WPA > 1) __syncthreads(); else __syncwarp();

    int qn = 0, q2n = 0, wqn = 0;
    bool paired = false;
    if constexpr (!TORUS && !HETERO) {
      paired = a.pair_loads != 0;
      if (paired) {
        // two adjacent neighbours per lane, 64 per warp and round: one 8-byte load per
        // coordinate, packed FP32x2 offsets and distances (the same roundings as one by one)
        constexpr int kStep2 = 64 * WPA;
        const int jb0 = (j0 & ~1) + warp * 64;   // even, so the pairs are 8-byte aligned
        float2 xn2 = make_float2(f.x, f.x), yn2 = make_float2(f.y, f.y);
        auto load2 = [&](int jj, float2 &xv, float2 &yv) {
            if (jj + 1 < n) {
                xv = __ldg(reinterpret_cast<const float2 *>(a.x + jj));
                yv = __ldg(reinterpret_cast<const float2 *>(a.y + jj));
            } else if (jj < n) {
                xv = make_float2(__ldg(a.x + jj), f.x);
                yv = make_float2(__ldg(a.y + jj), f.y);
            }
        };
        load2(jb0 + 2 * lane, xn2, yn2);
        const unsigned lt = (1u << lane) - 1u;
        for (int jb = jb0; jb < n; jb += kStep2) {
            const float2 xv = xn2, yv = yn2;
            const int jj = jb + 2 * lane;
            load2(jb + kStep2 + 2 * lane, xn2, yn2);   // prefetch the next round through L1
            const float2 dx = __fadd2_rn(xv, make_float2(-f.x, -f.x));
            const float2 dy = __fadd2_rn(yv, make_float2(-f.y, -f.y));
            const float2 d2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
            const bool live0 = jj >= j0 && jj < n && d2.x > 0.f && d2.x <= cull_r2;
            const bool live1 = jj + 1 >= j0 && jj + 1 < n && d2.y > 0.f && d2.y <= cull_r2;
            const unsigned lm0 = __ballot_sync(ABM_FULL_MASK, live0);
            const unsigned lm1 = __ballot_sync(ABM_FULL_MASK, live1);
            const int c0 = __popc(lm0);
            if (live0) q[qn + __popc(lm0 & lt)] = QEntry<HETERO>::make(dx.x, dy.x, d2.x, jj);
            if (live1)
                q[qn + c0 + __popc(lm1 & lt)] = QEntry<HETERO>::make(dx.y, dy.y, d2.y, jj + 1);
            qn += c0 + __popc(lm1);
            __syncwarp();
            while (qn >= 32) {   // warp-uniform; at most two batches
                qn -= 32;
                process_candidates<TORUS, HETERO, true>(f, q + qn, 32, q2, q2n, wq, wqn, vb,
                                                        a, &counters[0], &counters[1]);
            }
        }
      }
    }
    constexpr int kStep = 32 * WPA;
    int j = j0 + warp * 32 + lane;
    float xn = f.x, yn = f.y, rn = f.r;
    if (!paired && j < n) {
        xn = __ldg(a.x + j);
        yn = __ldg(a.y + j);
        if (HETERO) rn = __ldg(a.radius + j);
    }
    for (int jb = j0 + warp * 32; !paired && jb < n; jb += kStep) {
        const float xj = xn, yj = yn, rj = rn;
        const bool valid = jb + lane < n;
        const int jn = jb + kStep + lane;   // prefetch the next chunk through L1
        if (jn < n) {
            xn = __ldg(a.x + jn);
            yn = __ldg(a.y + jn);
            if (HETERO) rn = __ldg(a.radius + jn);
        }
        phase_a<TORUS, HETERO>(f, xj, yj, rj, jb + lane, valid, cull_r2, q, qn, q2, q2n, wq,
                               wqn, vb, a, counters);
    }
    if (qn > 0) process_candidates<TORUS, HETERO>(f, q, qn, q2, q2n, wq, wqn, vb, a,
                                                  &counters[0], &counters[1]);
    flush_runs(wq, wqn, vb, a.g.rv);
    drain_deferred<TORUS, HETERO>(f, q2, q2n, vb, a, &counters[0], &counters[1]);
    if (WPA > 1) __syncthreads(); else __syncwarp();
    if (split) {   // partial bitmask into the agent's global one; integrals in the finish kernel
        uint32_t *gb = a.vbits + (size_t)i * words;
        for (int w = threadIdx.x; w < words; w += 32 * WPA) {
            const uint32_t v = vb[w];
            if (v) atomicOr(gb + w, v);
        }
        if (threadIdx.x == 0) flush_counters(a, counters);
    } else if (warp == 0) {
        finish_agent(a, i, vb, reinterpret_cast<uint32_t *>(q), kListCap<HETERO>);
        if (lane == 0) flush_counters(a, counters);
    }
}

// ---------------------------------------------------------------------------- group form
// One warp serves kGroup consecutive focal agents of a single swarm (equal radii; walls, or a
// torus whose width and height are floats):
// phase A reads each neighbour once for the whole group, and the candidate queue mixes the
// group's agents -- each entry carries the agent's slot in the group in the top byte of its
// neighbour index -- so the batches of phase B stay full, and the per-block costs (focal
// set-up, the last partial batch, the double-float drain, the long-run flush, the epilogue)
// are paid once per kGroup agents.  With a.vbits set the neighbours are split into chunks
// exactly as in the l1 form and the group's partial bitmasks are OR-ed into the workspace.
constexpr int kGroup = 4;
constexpr int kGroupTagShift = 24;   // neighbour indices below 2^24
// batched sweeps: groups of 8 schedule entries (512-instance sweep step 256.0 -> 239.6 us
// against groups of 4: the per-block costs are shared by twice the agents)
constexpr int kSegGroup = 8;

constexpr int kCounters = 4;   // a group block's counters, then 33 spare words (lane, lane + 1)

// Shared memory of a group block: the agents' bitmasks (the second OR of a short run may name
// the word after the last agent's bitmask: the padding or the focal records, which an OR of
// zero leaves unchanged), the focal records, the queues, the counters and the spare words.
static size_t group_smem_bytes(int words, int gs = kGroup) {
    size_t b = ((size_t)gs * words * sizeof(uint32_t) + 15) & ~size_t(15);
    b += ((size_t)gs * sizeof(FocalDev) + 15) & ~size_t(15);
    b += (size_t)(kQueue + kQueue2) * sizeof(QEntry<false>) + kQueueW * sizeof(int2);
    return b + (kCounters + 33) * sizeof(unsigned);
}

// The rare paths of the group kernels, out of line so that the inlined copies of phase B stay
// small (both drains inline: N=4096 step 66.5 us against 64.2 us, 512-instance sweep step
// 239.6 us against 237.6 us; the group kernels are then held to 64 registers, 32 resident
// one-warp blocks per SM, by their launch bounds).
//
// 32 queued long or wrapping runs (one per lane) through the general fill.
static __device__ __noinline__ void drain_run_queue(const int2 *wq, uint32_t *vball, int words,
                                                    int rv) {
    const int lane = threadIdx.x & 31;
    const int2 r = wq[lane];
    raster_projection(vball + (r.y >> kGroupTagShift) * words, rv, r.x,
                      r.y & ((1 << kGroupTagShift) - 1));
}

// Double-float re-decision and rasterisation of the deferred pairs qe[0 .. cnt) (one per lane;
// equal radii R; TORUS: the minimal image on the W x H torus); returns the ballot of the pairs
// with a re-decided boundary within 1e-9 rad of their edge angle.
template <bool TORUS>
__device__ __forceinline__ unsigned drain_deferred_body(const FocalDev *fd,
                                                        const QEntry<false> *qe, int cnt,
                                                        uint32_t *vball, const float *x,
                                                        const float *y, float R, dfl W, dfl H,
                                                        GridDev g) {
    const int lane = threadIdx.x & 31;
    bool near = false;
    if (lane < cnt) {
        const int tag = qe[lane].j();
        const int dg = (int)((unsigned)tag >> kGroupTagShift);
        const int j = tag & ((1 << kGroupTagShift) - 1);
        const FocalDev &f = fd[dg];
        const float xj = __ldg(x + j), yj = __ldg(y + j);
        float dx, dy;
        pair_offset<TORUS, false>(f, xj, yj, R, W, H, dx, dy);
        const PairEst de = estimate_pair<false>(f, dx, dy, R, f.invr, g);
        dfl ex, ey;
        exact_offset<TORUS, false>(f, xj, yj, R, W, H, ex, ey);
        const int3 th = resolve_pair(f.cd, f.sd, ex, ey, R, resolve_grid(g), de.unc_t, de.unc_h,
                                     de.u, de.ps2, de.t, de.h);
        const int ds = th.x - th.y, dn = th.x + th.y;
        if (projection_visible(g, ds, dn)) raster_fast(vball + dg * g.words, g.rv, ds, dn);
        near = th.z != 0;
    }
    return __ballot_sync(ABM_FULL_MASK, near);
}

static __device__ __noinline__ unsigned drain_deferred(const FocalDev *fd, const QEntry<false> *qe,
                                                       int cnt, uint32_t *vball, const float *x,
                                                       const float *y, float R, GridDev g) {
    const dfl z = {0.f, 0.f};
    return drain_deferred_body<false>(fd, qe, cnt, vball, x, y, R, z, z, g);
}

static __device__ __noinline__ unsigned drain_deferred_torus(const FocalDev *fd,
                                                             const QEntry<false> *qe, int cnt,
                                                             uint32_t *vball, const float *x,
                                                             const float *y, float R, dfl W,
                                                             dfl H, GridDev g) {
    return drain_deferred_body<true>(fd, qe, cnt, vball, x, y, R, W, H, g);
}

// The minimal torus image (vf_supcalc.py:70-83) of two FP32 offsets d = fl(v - f) along one
// axis of length L, a float (its double-float low part is zero); the result is the wrapped
// exact offset rounded once, as the double-float offset gives it.  The exact offset is d + e
// (e: the two-sum error).  It wraps iff it lies beyond +-L/2: L/2 is a float, d - L/2 is exact
// wherever the sign of the sum is in doubt (Sterbenz), so fl(fl(d -+ L/2) + e) has the sign of
// the exact comparison.  A wrapped offset is fl(fl(d -+ L) + e), exact up to the last rounding
// for |d| <= 2L (the caller takes positions farther apart through the double-float offset).
// An offset that does not wrap stays d, since fl(d + e) = d.  The wrap k in {-1, 0, 1} comes
// from two compares as floats and d - kL from one fused multiply-add (kL is exact), which keeps
// the selects off the ALU pipe.
__device__ __forceinline__ float2 torus_image2(float2 d, float2 v, float f, float L) {
    const float2 nb = __fadd2_rn(v, make_float2(-d.x, -d.y));   // v - d
    const float2 t = __fadd2_rn(d, nb);                          // d - (d - v)
    const float2 e = __fadd2_rn(__fadd2_rn(v, make_float2(-t.x, -t.y)),
                                __fadd2_rn(make_float2(-f, -f), nb));
    const float h = 0.5f * L;
    const float2 up = __fadd2_rn(__fadd2_rn(d, make_float2(-h, -h)), e);
    const float2 dn = __fadd2_rn(__fadd2_rn(d, make_float2(h, h)), e);
    const float2 k = __fadd2_rn(make_float2(up.x > 0.f ? 1.f : 0.f, up.y > 0.f ? 1.f : 0.f),
                                make_float2(dn.x < 0.f ? -1.f : 0.f, dn.y < 0.f ? -1.f : 0.f));
    return __fadd2_rn(__ffma2_rn(make_float2(-L, -L), k, d), e);
}

// Whether a neighbour lies within 1.5 L (per axis) of every focal agent of a group: then every
// offset of the group's pairs is at most 1.5 L < 2L, as torus_image2 needs (the window's
// bounds are rounded inwards, so the test never admits a position outside it).  NaN positions
// fail it.
struct TorusWindow {
    float xlo, xhi, ylo, yhi;
    __device__ __forceinline__ bool holds(float x, float y) const {
        return x >= xlo && x <= xhi && y >= ylo && y <= yhi;
    }
};

__device__ __forceinline__ TorusWindow torus_window(const FocalDev *fd, int G, float W, float H) {
    float x0 = fd[0].x, x1 = x0, y0 = fd[0].y, y1 = y0;
    for (int g = 1; g < G; ++g) {
        x0 = fminf(x0, fd[g].x);
        x1 = fmaxf(x1, fd[g].x);
        y0 = fminf(y0, fd[g].y);
        y1 = fmaxf(y1, fd[g].y);
    }
    return {__fadd_ru(x1, -1.5f * W), __fadd_rd(x0, 1.5f * W), __fadd_ru(y1, -1.5f * H),
            __fadd_rd(y0, 1.5f * H)};
}

// The offsets of the two neighbours (xv, yv) from focal agent f through the double-float
// minimal image (the rare far offsets of torus_image2), as the one-block form computes them.
static __device__ __noinline__ float4 torus_offsets_exact(const FocalDev *fd, int g, float2 xv,
                                                          float2 yv, dfl W, dfl H) {
    const FocalDev &f = fd[g];
    float4 r;
    pair_offset<true, false>(f, xv.x, yv.x, f.r, W, H, r.x, r.z);
    pair_offset<true, false>(f, xv.y, yv.y, f.r, W, H, r.y, r.w);
    return r;
}

// Phase B of one (agent slot, neighbour) candidate per lane (`have`: the lane holds one; e: its
// offset, d^2 and tagged neighbour index): FP32 decisions, rasterisation of short runs, long and
// wrapping runs to the run queue, guard-band pairs to the double-float queue (each drained 32
// at a time).  FULLFOV: the field of view is the whole circle, so every projection is visible.
// TORUS: the offsets are minimal torus images (the deferred pairs recompute theirs).
template <bool FULLFOV, bool TORUS = false>
__device__ __forceinline__ void group_candidate(const FocalDev *fd, const QEntry<false> &e,
                                                bool have, QEntry<false> *q2, int &q2n, int2 *wq,
                                                int &wqn, uint32_t *vball, const StepArgs &a,
                                                unsigned *counters) {
    const int lane = threadIdx.x & 31;
    const int words = a.g.words;
    const int g = (int)((unsigned)e.j() >> kGroupTagShift);
    const FastEst est = estimate_fast(fd[g], e.v.x, e.v.y, e.v.z, a.radius0,
                                      a.radius0 * a.radius0, a.g);
    const bool unc = have && est.unc;
    const int s = est.t - est.h, en = est.t + est.h;
    const bool vis = have && !est.unc && (FULLFOV || projection_visible(a.g, s, en));
    const unsigned len = (unsigned)(en - s);
    const bool short_run = s >= 0 && en < a.g.rv && len <= 32u;
    {   // short runs: two shared ORs on every lane, without a branch (lanes with nothing to
        // raster OR zero into their own spare words after the block's counters; measured 3 %
        // faster steps than predicated ORs)
        const bool rs = vis && short_run;
        uint32_t *vb = rs ? vball + g * words + (s >> 5) : counters + kCounters + lane;
        const uint32_t m = rs ? __funnelshift_rc(ABM_FULL_MASK, 0u, 32u - len) : 0u;
        const int sh = s & 31;
        atomicOr(vb, m << sh);
        atomicOr(vb + 1, __funnelshift_l(m, 0u, sh));   // may name the next agent's word 0
    }
    const unsigned lt = (1u << lane) - 1u;
    // one vote for the rare cases: a long or wrapping run, or a guard-band decision
    const bool lng = vis && !short_run;
    if (__ballot_sync(ABM_FULL_MASK, lng || unc)) {
        const unsigned wm = __ballot_sync(ABM_FULL_MASK, lng);
        if (wm) {   // long and wrapping runs wait in the run queue (slot in the top byte)
            if (lng) wq[wqn + __popc(wm & lt)] = make_int2(s, en | (g << kGroupTagShift));
            wqn += __popc(wm);
            __syncwarp();
            if (wqn >= 32) {
                wqn -= 32;
                drain_run_queue(wq + wqn, vball, words, a.g.rv);
                __syncwarp();
            }
        }
        const unsigned um = __ballot_sync(ABM_FULL_MASK, unc);
        if (um) {   // defer the uncertain ones to the double-float queue
            if (unc) q2[q2n + __popc(um & lt)] = e;
            q2n += __popc(um);
        }
        __syncwarp();
        if (q2n >= 32) {   // drain 32 deferred pairs (warp-uniform)
            q2n -= 32;
            unsigned nm;
            if constexpr (TORUS)
                nm = drain_deferred_torus(fd, q2 + q2n, 32, vball, a.x, a.y, a.radius0, a.W, a.H,
                                          a.g);
            else
                nm = drain_deferred(fd, q2 + q2n, 32, vball, a.x, a.y, a.radius0, a.g);
            if (lane == 0) {
                atomicAdd(&counters[0], 32u);
                if (nm) atomicAdd(&counters[1], (unsigned)__popc(nm));
            }
            __syncwarp();
        }
    }
}

// Phase B of up to 32 queued candidates (lane < cnt holds one).
template <bool FULL, bool FULLFOV, bool TORUS = false>
__device__ __forceinline__ void group_batch(const FocalDev *fd, const QEntry<false> *q, int cnt,
                                            QEntry<false> *q2, int &q2n, int2 *wq, int &wqn,
                                            uint32_t *vball, const StepArgs &a,
                                            unsigned *counters) {
    const int lane = threadIdx.x & 31;
    const bool have = FULL || lane < cnt;
    const QEntry<false> e = (FULL || have) ? q[lane] : QEntry<false>::make(1.f, 0.f, 1.f, 0);
    group_candidate<FULLFOV, TORUS>(fd, e, have, q2, q2n, wq, wqn, vball, a, counters);
}

// The group form for one swarm: the group is 4 consecutive agents, the neighbours the block's
// chunk.  TORUS: the minimal images on a torus whose width and height are floats (N=4096 torus
// step 166.6 -> 102.8 us against the l1 form, bit-identical).
template <bool FULLFOV, bool TORUS = false>
__global__ void __launch_bounds__(32, 32) vpf_pairs_group_kernel(const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x;
    const int words = a.g.words;
    const bool split = a.vbits != nullptr;
    wait_primary_grid();   // the previous step's state (programmatic launch)
    int grp, j0 = 0, n = a.n;   // neighbours are [j0, n)
    if (a.chunk_rounds) {   // round-major plan: round r's chunk of every group, r = 0, 1, ...
        const int r = (int)(blockIdx.x / (unsigned)a.groups);
        grp = (int)blockIdx.x - r * a.groups;
        j0 = a.chunk_off[r];
        n = a.chunk_off[r + 1];
    } else {
        grp = (int)(blockIdx.x >> a.chunk_shift);
        if (split) {
            j0 = (int)(blockIdx.x & ((1u << a.chunk_shift) - 1u)) * a.chunk_len;
            n = min(n, j0 + a.chunk_len);
        }
    }
    const int i0 = grp * kGroup;
    const int G = min(kGroup, a.n - i0);
    uint32_t *vball = reinterpret_cast<uint32_t *>(smem);
    size_t off = ((size_t)kGroup * words * 4 + 15) & ~size_t(15);
    FocalDev *fd = reinterpret_cast<FocalDev *>(smem + off);
    off += ((size_t)kGroup * sizeof(FocalDev) + 15) & ~size_t(15);
    QEntry<false> *q = reinterpret_cast<QEntry<false> *>(smem + off);
    QEntry<false> *q2 = q + kQueue;
    off += (size_t)(kQueue + kQueue2) * sizeof(QEntry<false>);
    int2 *wq = reinterpret_cast<int2 *>(smem + off);
    off += (size_t)kQueueW * sizeof(int2);
    unsigned *counters = reinterpret_cast<unsigned *>(smem + off);

    // the bitmasks, 16 bytes per store (their region is padded to 16 bytes)
    for (int w4 = lane; 4 * w4 < G * words; w4 += 32)
        reinterpret_cast<uint4 *>(vball)[w4] = make_uint4(0u, 0u, 0u, 0u);
    if (lane < 4) counters[lane] = 0u;
    allow_dependent_launch();
    if (lane < G) fd[lane] = load_focal<false>(a, i0 + lane);   // the group's agents at once
    __syncwarp();
    const float cull_r2 = a.radius0 * a.radius0 * a.g.cull;
    TorusWindow tw{};
    if constexpr (TORUS) tw = torus_window(fd, G, a.W.hi, a.H.hi);

    int qn = 0, q2n = 0, wqn = 0;
    const unsigned lt = (1u << lane) - 1u;
    // two adjacent neighbours per lane, 64 per round: one 8-byte load per coordinate when the
    // state is 8-byte aligned (the pairs start at an even index)
    const bool pl = a.pair_loads != 0;
    auto load2 = [&](int jj, float2 &xv, float2 &yv) {
        if (pl && jj + 1 < n) {
            xv = __ldg(reinterpret_cast<const float2 *>(a.x + jj));
            yv = __ldg(reinterpret_cast<const float2 *>(a.y + jj));
        } else {
            xv = make_float2(jj < n ? __ldg(a.x + jj) : 0.f, jj + 1 < n ? __ldg(a.x + jj + 1) : 0.f);
            yv = make_float2(jj < n ? __ldg(a.y + jj) : 0.f, jj + 1 < n ? __ldg(a.y + jj + 1) : 0.f);
        }
    };
    const int jb0 = j0 & ~1;
    float2 xn2, yn2;
    load2(jb0 + 2 * lane, xn2, yn2);
    for (int jb = jb0; jb < n; jb += 64) {
        const float2 xv = xn2, yv = yn2;
        const int jj = jb + 2 * lane;
        load2(jb + 64 + 2 * lane, xn2, yn2);   // prefetch the next round through L1
        const bool v0 = jj >= j0 && jj < n, v1 = jj + 1 >= j0 && jj + 1 < n;
        bool far = false, anyfar = false;   // neighbours outside the group's torus window
        if constexpr (TORUS) {
            far = (v0 && !tw.holds(xv.x, yv.x)) || (v1 && !tw.holds(xv.y, yv.y));
            anyfar = __any_sync(ABM_FULL_MASK, far);
        }
        for (int g = 0; g < G; ++g) {   // warp-uniform
            const float fx = fd[g].x, fy = fd[g].y;
            float2 dx = __fadd2_rn(xv, make_float2(-fx, -fx));
            float2 dy = __fadd2_rn(yv, make_float2(-fy, -fy));
            if constexpr (TORUS) {
                dx = torus_image2(dx, xv, fx, a.W.hi);
                dy = torus_image2(dy, yv, fy, a.H.hi);
                if (anyfar && far) {
                    const float4 o = torus_offsets_exact(fd, g, xv, yv, a.W, a.H);
                    dx = make_float2(o.x, o.y);
                    dy = make_float2(o.z, o.w);
                }
            }
            const float2 d2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
            const bool live0 = v0 && d2.x > 0.f && d2.x <= cull_r2;
            const bool live1 = v1 && d2.y > 0.f && d2.y <= cull_r2;
            const unsigned lm0 = __ballot_sync(ABM_FULL_MASK, live0);
            const unsigned lm1 = __ballot_sync(ABM_FULL_MASK, live1);
            const int c0 = __popc(lm0);
            const int tag = jj | (g << kGroupTagShift);
            if (live0) q[qn + __popc(lm0 & lt)] = QEntry<false>::make(dx.x, dy.x, d2.x, tag);
            if (live1)
                q[qn + c0 + __popc(lm1 & lt)] = QEntry<false>::make(dx.y, dy.y, d2.y, tag + 1);
            qn += c0 + __popc(lm1);
            __syncwarp();
            while (qn >= 32) {   // warp-uniform; at most two batches
                qn -= 32;
                group_batch<true, FULLFOV, TORUS>(fd, q + qn, 32, q2, q2n, wq, wqn, vball, a,
                                                  counters);
            }
        }
    }
    if (qn > 0)
        group_batch<false, FULLFOV, TORUS>(fd, q, qn, q2, q2n, wq, wqn, vball, a, counters);
    if (lane < wqn) {   // the last long or wrapping runs
        const int2 r = wq[lane];
        raster_projection(vball + (r.y >> kGroupTagShift) * words, a.g.rv, r.x,
                          r.y & ((1 << kGroupTagShift) - 1));
    }
    __syncwarp();
    // the last (< 32) deferred pairs
    unsigned nm = 0u;
    if (q2n) {
        if constexpr (TORUS)
            nm = drain_deferred_torus(fd, q2, q2n, vball, a.x, a.y, a.radius0, a.W, a.H, a.g);
        else
            nm = drain_deferred(fd, q2, q2n, vball, a.x, a.y, a.radius0, a.g);
    }
    if (lane == 0 && q2n) {
        counters[0] += (unsigned)q2n;
        counters[1] += (unsigned)__popc(nm);
    }
    __syncwarp();
    if (split) {   // the group's partial bitmasks (consecutive agents) into the workspace
        uint32_t *gb = a.vbits + (size_t)i0 * words;
        for (int w = lane; w < G * words; w += 32) {
            const uint32_t v = vball[w];
            if (v) atomicOr(gb + w, v);
        }
    } else {       // integrals of each agent (the drained queues hold its transition list)
        for (int g = 0; g < G; ++g)
            finish_agent(a, i0 + g, vball + g * words, reinterpret_cast<uint32_t *>(q),
                         kListCap<false>);
    }
    if (lane == 0) flush_counters(a, counters);
}

// Integrals of a batched group's agents at once (the loop form of warp_integrals_loop): the
// LPA = 32 / kSegGroup lanes LPA g .. LPA g + LPA - 1 take agent g's words w = lane % LPA,
// w + LPA, ..., each visiting its words' transitions, and a reduction over the agent's lanes
// gives its sums (exact fixed point, so the same sums as one agent at a time over 32 lanes).
// agents: the group's agent ids; also copies each agent's bitmask to a.bits when requested.
__device__ __forceinline__ void group_finish_loop(const StepArgs &a, const int *agents, int G,
                                                  const uint32_t *vball) {
    const int lane = threadIdx.x & 31;
    constexpr int LPA = 32 / kSegGroup;
    const int g = lane / LPA, sub = lane % LPA;
    const int rv = a.g.rv, words = a.g.words;
    const bool act = g < G;
    const uint32_t *vb = vball + (act ? g : 0) * words;
    const uint32_t v0 = vb[0] & 1u;
    const uint32_t vl = (vb[(rv - 1) >> 5] >> ((rv - 1) & 31)) & 1u;
    const int bwd = (v0 == 1u && vl == 0u) ? 1 : 0;
    long long bc = 0, bs = 0, ec = 0, es = 0;
    if (act) {
        for (int w = sub; w < words; w += LPA) {
            const uint32_t cur = vb[w];
            const uint32_t prev = (w > 0) ? (vb[w - 1] >> 31) : (cur & 1u);
            uint32_t D = cur ^ ((cur << 1) | prev);
            if (w == words - 1 && (rv & 31)) D &= (1u << (rv & 31)) - 1u;
            while (D) {
                const int b = __ffs(D) - 1;
                D &= D - 1u;
                const int j = (w << 5) + b;
                const longlong2 qv = a.g.q[j];
                if ((cur >> b) & 1u) {   // run starts at j
                    bc -= qv.x;
                    bs -= qv.y;
                } else {                 // run ends at j
                    bc += qv.x;
                    bs += qv.y;
                }
                const longlong2 cv = a.g.cpt[j - 1 + bwd];
                ec += cv.x;
                es += cv.y;
            }
        }
    }
#pragma unroll
    for (int o = LPA / 2; o > 0; o >>= 1) {   // within each agent's lanes
        bc += __shfl_xor_sync(ABM_FULL_MASK, bc, o);
        bs += __shfl_xor_sync(ABM_FULL_MASK, bs, o);
        ec += __shfl_xor_sync(ABM_FULL_MASK, ec, o);
        es += __shfl_xor_sync(ABM_FULL_MASK, es, o);
    }
    if (!act) return;
    const int i = agents[g];
    if (sub == 0) {
        if (vl) {
            bc += a.g.qc_total;
            bs += a.g.qs_total;
        }
        if (v0 != vl) {   // the circular edge between pixels Rv-1 and 0
            const longlong2 cv = a.g.cpt[bwd ? 0 : rv - 1];
            ec += cv.x;
            es += cv.y;
        }
        longlong2 *sp = reinterpret_cast<longlong2 *>(a.sums) + 2 * (size_t)i;
        sp[0] = make_longlong2(bc, bs);
        sp[1] = make_longlong2(ec, es);
    }
    if (a.bits) {
        uint32_t *dst = a.bits + (size_t)i * words;
        for (int w = sub; w < words; w += LPA) dst[w] = vb[w];
    }
}

// The group form for a batched sweep: the group is kSegGroup consecutive entries of the
// schedule, and each distinct neighbour range of its agents (a group may straddle instances)
// is scanned once for the agents that share it.  (A separate kernel: folding this into the
// single-swarm kernel measured 1.3 us slower per step at N=4096.)  DIRECT: the arena lies
// within the cull radius, so (almost) every pair is live and phase B takes the candidates
// straight from the scan, without the queue that compacts the live ones.  TORUS: the minimal
// images on a torus whose width and height are floats, as in the single-swarm kernel.
template <bool FULLFOV, bool DIRECT, bool TORUS = false>
__global__ void __launch_bounds__(32, 32) vpf_pairs_group_seg_kernel(const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_agent[kSegGroup], s_j0[kSegGroup], s_j1[kSegGroup];
    const int lane = threadIdx.x;
    const int words = a.g.words;
    wait_primary_grid();   // the previous step's state (programmatic launch)
    // the group: positions [p0, p0 + G) of the schedule
    const int p0 = (int)blockIdx.x * kSegGroup;
    const int G = min(kSegGroup, a.n - p0);
    uint32_t *vball = reinterpret_cast<uint32_t *>(smem);
    size_t off = ((size_t)kSegGroup * words * 4 + 15) & ~size_t(15);
    FocalDev *fd = reinterpret_cast<FocalDev *>(smem + off);
    off += ((size_t)kSegGroup * sizeof(FocalDev) + 15) & ~size_t(15);
    QEntry<false> *q = reinterpret_cast<QEntry<false> *>(smem + off);
    QEntry<false> *q2 = q + kQueue;
    off += (size_t)(kQueue + kQueue2) * sizeof(QEntry<false>);
    int2 *wq = reinterpret_cast<int2 *>(smem + off);
    off += (size_t)kQueueW * sizeof(int2);
    unsigned *counters = reinterpret_cast<unsigned *>(smem + off);

    // the bitmasks, 16 bytes per store (their region is padded to 16 bytes)
    for (int w4 = lane; 4 * w4 < G * words; w4 += 32)
        reinterpret_cast<uint4 *>(vball)[w4] = make_uint4(0u, 0u, 0u, 0u);
    if (lane < 4) counters[lane] = 0u;
    allow_dependent_launch();
    if (lane < G) {   // the group's agents at once
        const int i = a.order ? a.order[p0 + lane] : p0 + lane;
        s_agent[lane] = i;
        s_j0[lane] = a.seg_begin[i];
        s_j1[lane] = a.seg_end[i];
        fd[lane] = load_focal<false>(a, i);
    }
    __syncwarp();
    const float cull_r2 = a.radius0 * a.radius0 * a.g.cull;
    TorusWindow tw{};
    if constexpr (TORUS) tw = torus_window(fd, G, a.W.hi, a.H.hi);

    int qn = 0, q2n = 0, wqn = 0;
    const unsigned lt = (1u << lane) - 1u;
    // one scan of a neighbour range [j0, n) for the group's agents in `members`: two
    // neighbours per lane, 64 per round -- j0 + 64 r + lane and j0 + 64 r + 32 + lane in round
    // r (two coalesced loads per coordinate), so that a range's last round skips its second
    // half when that holds no neighbour (sweep step 237.7 -> 233.4 us against adjacent pairs)
    auto scan = [&](const int j0, const int n, const unsigned members) {
        auto load2 = [&](int jb, float2 &xv, float2 &yv) {
            const int ja = jb + lane, jc = jb + 32 + lane;
            xv = make_float2(ja < n ? __ldg(a.x + ja) : 0.f, jc < n ? __ldg(a.x + jc) : 0.f);
            yv = make_float2(ja < n ? __ldg(a.y + ja) : 0.f, jc < n ? __ldg(a.y + jc) : 0.f);
        };
        float2 xn2, yn2;
        load2(j0, xn2, yn2);
        for (int jb = j0; jb < n; jb += 64) {
            const float2 xv = xn2, yv = yn2;
            const int ja = jb + lane, jc = jb + 32 + lane;
            load2(jb + 64, xn2, yn2);   // prefetch the next round through L1
            const bool v0 = ja < n, v1 = jc < n;
            const bool second = jb + 32 < n;   // warp-uniform
            bool far = false, anyfar = false;   // neighbours outside the group's torus window
            if constexpr (TORUS) {
                far = (v0 && !tw.holds(xv.x, yv.x)) || (v1 && !tw.holds(xv.y, yv.y));
                anyfar = __any_sync(ABM_FULL_MASK, far);
            }
            for (int g = 0; g < G; ++g) {   // warp-uniform
                if (!((members >> g) & 1u)) continue;
                const float fx = fd[g].x, fy = fd[g].y;
                float2 dx = __fadd2_rn(xv, make_float2(-fx, -fx));
                float2 dy = __fadd2_rn(yv, make_float2(-fy, -fy));
                if constexpr (TORUS) {
                    dx = torus_image2(dx, xv, fx, a.W.hi);
                    dy = torus_image2(dy, yv, fy, a.H.hi);
                    if (anyfar && far) {
                        const float4 o = torus_offsets_exact(fd, g, xv, yv, a.W, a.H);
                        dx = make_float2(o.x, o.y);
                        dy = make_float2(o.z, o.w);
                    }
                }
                const float2 d2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
                const bool live0 = v0 && d2.x > 0.f && d2.x <= cull_r2;
                const bool live1 = v1 && d2.y > 0.f && d2.y <= cull_r2;
                const int gt = g << kGroupTagShift;
                if constexpr (DIRECT) {   // phase B on the lanes' own candidates
                    group_candidate<FULLFOV, TORUS>(
                        fd, QEntry<false>::make(dx.x, dy.x, d2.x, ja | gt), live0, q2, q2n, wq,
                        wqn, vball, a, counters);
                    if (second)
                        group_candidate<FULLFOV, TORUS>(
                            fd, QEntry<false>::make(dx.y, dy.y, d2.y, jc | gt), live1, q2, q2n,
                            wq, wqn, vball, a, counters);
                } else {
                    const unsigned lm0 = __ballot_sync(ABM_FULL_MASK, live0);
                    const unsigned lm1 = __ballot_sync(ABM_FULL_MASK, live1);
                    const int c0 = __popc(lm0);
                    if (live0)
                        q[qn + __popc(lm0 & lt)] = QEntry<false>::make(dx.x, dy.x, d2.x, ja | gt);
                    if (live1)
                        q[qn + c0 + __popc(lm1 & lt)] =
                            QEntry<false>::make(dx.y, dy.y, d2.y, jc | gt);
                    qn += c0 + __popc(lm1);
                    __syncwarp();
                    while (qn >= 32) {   // warp-uniform; at most two batches
                        qn -= 32;
                        group_batch<true, FULLFOV, TORUS>(fd, q + qn, 32, q2, q2n, wq, wqn,
                                                          vball, a, counters);
                    }
                }
            }
        }
    };
    // one scan per distinct neighbour range (a group may straddle instances)
    unsigned todo = (1u << G) - 1u;
    while (todo) {
        const int gr = __ffs(todo) - 1;
        const int j0 = s_j0[gr], n = s_j1[gr];
        unsigned members = 0u;
        for (int g = 0; g < G; ++g)
            if (s_j0[g] == j0 && s_j1[g] == n) members |= 1u << g;
        todo &= ~members;
        scan(j0, n, members);
    }
    if (qn > 0)
        group_batch<false, FULLFOV, TORUS>(fd, q, qn, q2, q2n, wq, wqn, vball, a, counters);
    if (lane < wqn) {   // the last long or wrapping runs
        const int2 r = wq[lane];
        raster_projection(vball + (r.y >> kGroupTagShift) * words, a.g.rv, r.x,
                          r.y & ((1 << kGroupTagShift) - 1));
    }
    __syncwarp();
    // the last (< 32) deferred pairs
    unsigned nm = 0u;
    if (q2n) {
        if constexpr (TORUS)
            nm = drain_deferred_torus(fd, q2, q2n, vball, a.x, a.y, a.radius0, a.W, a.H, a.g);
        else
            nm = drain_deferred(fd, q2, q2n, vball, a.x, a.y, a.radius0, a.g);
    }
    if (lane == 0 && q2n) {
        counters[0] += (unsigned)q2n;
        counters[1] += (unsigned)__popc(nm);
    }
    __syncwarp();
    // integrals of each agent (the whole neighbour ranges were scanned)
    group_finish_loop(a, s_agent, G, vball);
    if (lane == 0) flush_counters(a, counters);
}

// ---------------------------------------------------------------------------- tiled form
// Several focal warps per block; neighbour tiles staged in shared memory by the TMA bulk
// engine (double-buffered when the swarm spans more than one tile).
static int tile_buffers(int n, int tile) { return n > tile ? 2 : 1; }

static size_t tiled_smem_bytes(int warps, int tile, int words, bool hetero, int nbuf) {
    const int nf = hetero ? 3 : 2;
    const size_t qe = sizeof(QEntry<false>);
    size_t b = 16 + (size_t)nbuf * nf * tile * sizeof(float);
    b += (size_t)warps * words * sizeof(uint32_t);
    b = (b + 15) & ~size_t(15);
    b += (size_t)warps * ((kQueue + kQueue2) * qe + kQueueW * sizeof(int2));
    b += 16;  // block counters
    return b;
}

template <bool TORUS, bool HETERO, bool TMA>
__global__ void __launch_bounds__(1024) vpf_pairs_tiled_kernel(const StepArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const int tile = a.tile, n = a.n, words = a.g.words;
    constexpr int NF = HETERO ? 3 : 2;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    float *buf0 = reinterpret_cast<float *>(smem + 16);
    const int nbuf = n > tile ? 2 : 1;   // tile_buffers()
    uint32_t *vball = reinterpret_cast<uint32_t *>(buf0 + nbuf * NF * tile);
    uint32_t *vb = vball + warp * words;
    size_t off = 16 + (size_t)nbuf * NF * tile * sizeof(float) + (size_t)nw * words * 4;
    off = (off + 15) & ~size_t(15);
    QEntry<HETERO> *q = reinterpret_cast<QEntry<HETERO> *>(smem + off) + warp * (kQueue + kQueue2);
    QEntry<HETERO> *q2 = q + kQueue;
    off += (size_t)nw * (kQueue + kQueue2) * sizeof(QEntry<HETERO>);
    int2 *wq = reinterpret_cast<int2 *>(smem + off) + warp * kQueueW;
    off += (size_t)nw * kQueueW * sizeof(int2);
    unsigned *counters = reinterpret_cast<unsigned *>(smem + off);

    const int i = blockIdx.x * nw + warp;
    const bool active = i < n;
    wait_primary_grid();   // the previous step's state (programmatic launch)
    allow_dependent_launch();
    if (tid < 4) counters[tid] = 0u;
    for (int w = lane; w < words; w += 32) vb[w] = 0u;
    if (TMA && tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
    }
    const FocalDev f = load_focal<HETERO>(a, active ? i : blockIdx.x * nw);
    const float cull_r2 = f.r * f.r * a.g.cull;
    __syncthreads();

    const int ntiles = (n + tile - 1) / tile;
    auto issue = [&](int k) {
        const int base = k * tile;
        const int tn = min(tile, n - base);
        const int tn4 = tn & ~3;
        if (tn4 > 0) {
            float *dst = buf0 + (k & 1) * (nbuf - 1) * NF * tile;
            const uint32_t bytes = (uint32_t)tn4 * 4u;
            fence_proxy_async();
            mbar_expect_tx(&bars[k & 1], bytes * NF);
            bulk_g2s(dst, a.x + base, bytes, &bars[k & 1]);
            bulk_g2s(dst + tile, a.y + base, bytes, &bars[k & 1]);
            if (HETERO) bulk_g2s(dst + 2 * tile, a.radius + base, bytes, &bars[k & 1]);
        }
    };
    if (TMA && tid == 0) issue(0);

    int qn = 0, q2n = 0, wqn = 0;
    for (int k = 0; k < ntiles; ++k) {
        const int base = k * tile;
        const int tn = min(tile, n - base);
        int tn_s;
        const float *cur = buf0 + (k & 1) * (nbuf - 1) * NF * tile;
        if (TMA) {
            if (tid == 0 && k + 1 < ntiles) issue(k + 1);
            tn_s = tn & ~3;
            const bool ok = tn_s <= 0 || mbar_wait(&bars[k & 1], (uint32_t)((k >> 1) & 1));
            if (__syncthreads_or(!ok)) {
                // The tile did not arrive within the poll limit: record it, wait (bounded
                // again) for this block's copies still in flight -- tile k and, when issued,
                // tile k + 1 -- so none lands after the block exits, and leave without
                // results; abm_vpf_status reports the timeout to the host.
                if (tid == 0) {
                    counters[2] += 1u;
                    atomicOr(&g_kernel_status, kStatusWaitTimeout);
                    if (k + 1 < ntiles && (min(tile, n - base - tile) & ~3) > 0)
                        mbar_wait(&bars[(k + 1) & 1], (uint32_t)(((k + 1) >> 1) & 1));
                    if (tn_s > 0) mbar_wait(&bars[k & 1], (uint32_t)((k >> 1) & 1));
                    flush_counters(a, counters);
                }
                return;
            }
        } else {
            float *w = buf0 + (k & 1) * (nbuf - 1) * NF * tile;
            for (int qi = tid; qi < tn; qi += blockDim.x) {
                w[qi] = a.x[base + qi];
                w[tile + qi] = a.y[base + qi];
                if (HETERO) w[2 * tile + qi] = a.radius[base + qi];
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
                phase_a<TORUS, HETERO>(f, xj, yj, rj, base + jj, valid, cull_r2, q, qn, q2, q2n,
                                       wq, wqn, vb, a, counters);
            }
        }
        __syncthreads();
    }
    if (active) {
        if (qn > 0) process_candidates<TORUS, HETERO>(f, q, qn, q2, q2n, wq, wqn, vb, a,
                                                      &counters[0], &counters[1]);
        flush_runs(wq, wqn, vb, a.g.rv);
        drain_deferred<TORUS, HETERO>(f, q2, q2n, vb, a, &counters[0], &counters[1]);
        __syncwarp();
        finish_agent(a, i, vb, reinterpret_cast<uint32_t *>(q), kListCap<HETERO>);
    }
    __syncthreads();
    if (tid == 0) flush_counters(a, counters);
}

// ---------------------------------------------------------------------------- update kernel
// New state, optional terms and the non-finite count of agent k.
__device__ __forceinline__ void store_update(const StepArgs &a, int k, const UpdateOut &o) {
    a.xo[k] = o.x;
    a.yo[k] = o.y;
    a.tho[k] = o.th;
    a.vo[k] = o.v;
    if (a.terms) {
        double *t = a.terms + 6 * (size_t)k;
        for (int m = 0; m < 6; ++m) t[m] = (double)o.terms[m].hi + (double)o.terms[m].lo;
    }
    if (a.diag && !(isfinite(o.x) && isfinite(o.y) && isfinite(o.th) && isfinite(o.v)))
        atomicAdd(&a.diag[ABM_DIAG_NONFINITE], 1ull);
}

// The reference's update of every agent from its sums, one thread per agent.
template <bool HETERO>
__global__ void __launch_bounds__(64) vpf_update_kernel(const StepArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = k < a.n;
    // inputs of the step (not written by the pair kernel): loaded before the wait
    float x = 0.f, y = 0.f, th = 0.f, v = 0.f, R = a.radius0;
    dfl alp0 = a.ud.alp0, bet0 = a.ud.bet0, v0 = a.ud.v0;
    if (live) {
        x = a.x[k];
        y = a.y[k];
        th = a.th[k];
        v = a.v[k];
        if (HETERO) R = a.radius[k];
        if (a.alp0) alp0 = dfl{a.alp0[k], 0.f};
        if (a.bet0) bet0 = dfl{a.bet0[k], 0.f};
        if (a.v0) v0 = dfl{a.v0[k], 0.f};
    }
    wait_primary_grid();
    allow_dependent_launch();   // the next step's pair kernel waits for this one's end
    if (!live) return;
    const longlong2 *sp = reinterpret_cast<const longlong2 *>(a.sums) + 2 * (size_t)k;
    const longlong2 s0 = __ldcg(sp), s1 = __ldcg(sp + 1);
    const UpdateOut o = update_agent_df(a.ud, a.sctab, x, y, th, v, R, s0.x, s0.y, s1.x, s1.y,
                                        alp0, bet0, v0);
    store_update(a, k, o);
}

// ---------------------------------------------------------------------------- finish kernel
// After the split l1 form: one warp per agent stages the agent's bitmask in shared memory,
// clears the global copy for the next step, writes the optional bitmask output and reduces
// the VSWRM sums; warp 0 then applies the update to the block's agents, one lane each.
constexpr int kFinishWarps = 8;
constexpr int kFinishList = 256;   // transition-list entries per warp

struct FinishInputs {   // one agent's update inputs, parked in shared memory
    float x, y, th, v, R, alp0, bet0, v0;
};

template <bool HETERO>
__global__ void __launch_bounds__(32 * kFinishWarps) vpf_finish_kernel(const StepArgs a) {
    extern __shared__ __align__(16) unsigned char fsmem[];
    __shared__ longlong2 sums[kFinishWarps][2];
    __shared__ FinishInputs uin[kFinishWarps];
    // the integral tables and the update's double-float sincos table (constant inputs) into
    // L2 while the pair kernel still runs (staging the sincos table in shared memory in every
    // block measured 0.4 us slower per step at N=4096)
    prefetch_table_l2(a.g.q, sizeof(longlong2) * (size_t)(a.g.rv + 1));
    prefetch_table_l2(a.g.cpt, sizeof(longlong2) * (size_t)a.g.rv);
    prefetch_table_l2(a.sctab, sizeof(float4) * kSinCosTab);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, words = a.g.words;
    const int k = blockIdx.x * kFinishWarps + warp;
    const int ku = blockIdx.x * kFinishWarps + lane;
    const bool updater = warp == 0 && lane < kFinishWarps && ku < a.n;
    if (k < a.n) {
        // warp 0 also loads the block's update inputs, so that their latency overlaps the
        // bitmask loads; they wait in shared memory until the sums are ready
        FinishInputs in{};
        if (updater) {
            in.x = a.x[ku];
            in.y = a.y[ku];
            in.th = a.th[ku];
            in.v = a.v[ku];
            in.R = HETERO ? a.radius[ku] : a.radius0;
            in.alp0 = a.alp0 ? a.alp0[ku] : 0.f;
            in.bet0 = a.bet0 ? a.bet0[ku] : 0.f;
            in.v0 = a.v0 ? a.v0[ku] : 0.f;
        }
        wait_primary_grid();
        allow_dependent_launch();   // the next step's pair kernel waits for this one's end
        uint32_t *vb = reinterpret_cast<uint32_t *>(fsmem) + warp * words;
        uint32_t *gb = a.vbits + (size_t)k * words;
        for (int base = 0; base < words; base += 128) {   // loads first: one latency
            uint32_t t[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int w = base + 32 * u + lane;
                t[u] = w < words ? __ldcg(gb + w) : 0u;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int w = base + 32 * u + lane;
                if (w < words) {
                    vb[w] = t[u];
                    gb[w] = 0u;
                }
            }
        }
        if (updater) uin[lane] = in;
        __syncwarp();
        uint32_t *list = reinterpret_cast<uint32_t *>(fsmem) + kFinishWarps * words +
                         warp * kFinishList;
        long long bc, bs, ec, es;
        warp_integrals<8, 4>(vb, a.g, list, kFinishList, bc, bs, ec, es);
        if (a.bits) {
            uint32_t *dst = a.bits + (size_t)k * words;
            for (int w = lane; w < words; w += 32) dst[w] = vb[w];
        }
        if (lane == 0) {
            sums[warp][0] = make_longlong2(bc, bs);
            sums[warp][1] = make_longlong2(ec, es);
        }
    }
    __syncthreads();
    if (!updater) return;
    const FinishInputs in = uin[lane];
    const longlong2 s0 = sums[lane][0], s1 = sums[lane][1];
    const dfl alp0 = a.alp0 ? dfl{in.alp0, 0.f} : a.ud.alp0;
    const dfl bet0 = a.bet0 ? dfl{in.bet0, 0.f} : a.ud.bet0;
    const dfl v0 = a.v0 ? dfl{in.v0, 0.f} : a.ud.v0;
    const UpdateOut o = update_agent_df(a.ud, a.sctab, in.x, in.y, in.th, in.v, in.R, s0.x,
                                        s0.y, s1.x, s1.y, alp0, bet0, v0);
    store_update(a, ku, o);
}

// Copies the four state arrays (addressable host memory) into one device staging buffer.
__global__ void gather_state_kernel(const float *x, const float *y, const float *th,
                                    const float *v, float *dst, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        dst[k] = x[k];
        dst[(size_t)n + k] = y[k];
        dst[2 * (size_t)n + k] = th[k];
        dst[3 * (size_t)n + k] = v[k];
    }
}

// Polarisation of each instance (one block per instance): |sum (cos, sin)| / N.
__global__ void __launch_bounds__(256) polarisation_kernel(const float *theta, int n_total,
                                                           const int *offsets, double *out,
                                                           int capacity, int *step) {
    __shared__ double sx[8], sy[8];
    const int k = blockIdx.x;
    const int a0 = offsets ? offsets[k] : 0, a1 = offsets ? offsets[k + 1] : n_total;
    double cx = 0.0, cy = 0.0;
    for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        float s, c;
        sincosf(theta[i], &s, &c);
        cx += c;
        cy += s;
    }
    for (int o = 16; o > 0; o >>= 1) {
        cx += __shfl_xor_sync(ABM_FULL_MASK, cx, o);
        cy += __shfl_xor_sync(ABM_FULL_MASK, cy, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sx[warp] = cx;
        sy[warp] = cy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tx = 0.0, ty = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            tx += sx[w];
            ty += sy[w];
        }
        const int t = step[k];
        if (t < capacity && a1 > a0) out[(size_t)k * capacity + t] = sqrt(tx * tx + ty * ty) / (a1 - a0);
        step[k] = t + 1;
    }
}

// One column of a visual-flocking recording.  Every block reads the column before it arrives
// at the counter rec.step[1]; the last block to arrive advances rec.step[0] and clears step[1],
// so no block can see the advanced column within the launch (no block waits on another).
__global__ void __launch_bounds__(256) vf_record_kernel(abm_swarm_state s, int n,
                                                        const uint32_t *bits, int words,
                                                        abm_vf_recording rec) {
    const int t = __ldcg(rec.step);
    if (t < rec.capacity) {
        const size_t cap = (size_t)rec.capacity;
        const int stride = gridDim.x * blockDim.x;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const size_t o = (size_t)i * cap + t;
            rec.posx[o] = (int)s.x[i];   // Python int(): truncation toward zero
            rec.posy[o] = (int)s.y[i];
            rec.orientation[o] = s.theta[i];
            rec.velocity[o] = s.v[i];
        }
        if (rec.vpf_bits) {
            const size_t total = (size_t)n * words;
            for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total;
                 q += stride) {
                const size_t i = q / words, w = q % words;
                rec.vpf_bits[(i * cap + t) * words + w] = bits[q];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(rec.step + 1, 1) == (int)gridDim.x - 1) {
            rec.step[1] = 0;
            rec.step[0] = t + 1;
        }
    }
}

// Evaluates the in-kernel double-float cos/sin (verification hook for the tests).
__global__ void check_sincos_kernel(const float *theta, int n, double *out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dfl c, s;
    df_sincos(theta[k], c_sincos, c, s);
    out[2 * k] = (double)c.hi + (double)c.lo;
    out[2 * k + 1] = (double)s.hi + (double)s.lo;
}

// Test hook of the bounded wait: an mbarrier armed for 16 bytes that no copy delivers (no bulk
// copy is issued, so nothing is in flight when the block exits), then `polls` try_wait rounds.
// result[0] = 1 if the wait saw the phase complete, 0 if it gave up; a give-up is counted and
// raises the timeout status like the tiled kernel's.
__global__ void wait_timeout_probe_kernel(int polls, unsigned long long *diag, int *result) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_expect_tx(&bar, 16);
    __syncthreads();
    const bool ok = mbar_wait(&bar, 0, polls);
    const bool gave_up = __syncthreads_or(!ok);
    if (threadIdx.x == 0) {
        result[0] = ok ? 1 : 0;
        if (gave_up) {
            if (diag) atomicAdd(&diag[ABM_DIAG_TIMEOUTS], 1ull);
            atomicOr(&g_kernel_status, kStatusWaitTimeout);
        }
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bar)) : "memory");
    }
}

__global__ void clear_status_kernel(unsigned bits) { atomicAnd(&g_kernel_status, ~bits); }

// Launch of the step's second kernel after the pair kernel with programmatic stream
// serialisation (it may start while the pair kernel drains; it waits in griddepcontrol.wait).
static cudaError_t launch_dependent(void (*kern)(StepArgs), int blocks, int threads, size_t smem,
                                    cudaStream_t s, const StepArgs &a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

// Resident blocks per SM of a kernel at a given block size and dynamic shared memory, times
// the SM count (cached per device and configuration).
static int resident_slots(const void *kern, int threads, size_t smem) {
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, int, size_t>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(dev, kern, threads, smem);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int bps = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, threads, smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return cache[key] = bps * sms;
}

// l1 form.  With a.vbits set (a single swarm, bitmask workspace available) each agent's
// neighbours are split into `split` chunks (0: enough chunks that the blocks fill the GPU about
// three times over, so the block scheduler balances the SMs' work; chunks of at least 256
// neighbours); *chunks returns the number used (1: one block per agent, a.vbits unused).
template <bool TORUS, bool HETERO>
static int launch_l1(StepArgs a, int wpa, int split, cudaStream_t stream, int *chunks) {
    const size_t smem = l1_smem_bytes(wpa, a.g.words, HETERO);
    const void *kern = wpa == 1   ? (const void *)vpf_pairs_l1_kernel<TORUS, HETERO, 1>
                       : wpa == 2 ? (const void *)vpf_pairs_l1_kernel<TORUS, HETERO, 2>
                                  : (const void *)vpf_pairs_l1_kernel<TORUS, HETERO, 4>;
    int c = 1;
    if (a.vbits) {
        if (split > 0) {
            c = split;
        } else {
            const long slots = resident_slots(kern, 32 * wpa, smem);
            while (c < 16 && (long)a.n * c < 3 * slots && a.n / (2 * c) >= 256) c *= 2;
        }
    }
    int shift = 0;
    while ((1 << shift) < c) ++shift;
    a.chunk_shift = shift;
    a.chunk_len = c > 1 ? ((a.n + c - 1) / c + 31) / 32 * 32 : a.n;
    if (c == 1) a.vbits = nullptr;
    *chunks = c;
    const unsigned blocks = (unsigned)a.n << shift;
    // programmatic launch: scheduled while the previous step's last kernel drains
    cudaError_t e;
    if (wpa == 1) e = launch_pdl(vpf_pairs_l1_kernel<TORUS, HETERO, 1>, blocks, 32, smem, stream, a);
    else if (wpa == 2) e = launch_pdl(vpf_pairs_l1_kernel<TORUS, HETERO, 2>, blocks, 64, smem, stream, a);
    else e = launch_pdl(vpf_pairs_l1_kernel<TORUS, HETERO, 4>, blocks, 128, smem, stream, a);
    return check_cuda(e, "vpf_pairs_l1_kernel launch");
}

// Round-major chunk plan of the single-swarm group form with c chunks per group: round r takes
// a share 2 (c - r) + 1 of every group's neighbours (rounded up to multiples of 64), so the
// blocks dispatched last are the shortest and the SMs run out of work together.  Measured at
// N=4096 (8 rounds, 8192 blocks, L2 flushed, three alternating runs): 75.3 us per step with
// equal chunks in group-major or round-major order, 71.1-71.3 us with decreasing shares (the
// ramp, and {12,11,10,9,8,6,5,3}/64 or {10,10,10,9,8,7,6,4}/64); 10 rounds 72.1 us, 5 rounds
// 75.6 us.  Returns the number of rounds and fills off[0..rounds].
static int chunk_plan(int n, int c, int *off) {
    c = std::min(c, kMaxChunkRounds);
    const long long total = (long long)c * c + 2LL * c;   // sum of 2 (c - r) + 1
    long long acc = 0;
    int r = 0, at = 0;
    off[0] = 0;
    for (int k = 0; k < c && at < n; ++k) {
        acc += 2LL * (c - k) + 1;
        int e = k + 1 == c ? n : (int)std::min<long long>(n, (n * acc / total + 63) / 64 * 64);
        if (e <= at) continue;
        off[++r] = e;
        at = e;
    }
    return r;
}

// group form (equal radii): chunks as in launch_l1, counted in groups.
static int launch_group(StepArgs a, int split, double arena_w, double arena_h,
                        cudaStream_t stream, int *chunks) {
    const int gsz = a.seg_begin ? kSegGroup : kGroup;
    const size_t smem = group_smem_bytes(a.g.words, gsz);
    const int groups = (a.n + gsz - 1) / gsz;
    int c = 1;
    long slots = 0;
    if (a.vbits) {
        if (split > 0) {
            c = split;
        } else {
            // about two waves of resident blocks (measured best at N=4096: 8 chunks, 8192
            // blocks; 4 chunks and 16 chunks were 2 us and 4 us slower per step)
            slots = resident_slots((const void *)vpf_pairs_group_kernel<true>, 32, smem);
            while (c < 16 && (long)groups * 2 * c <= 2 * slots && a.n / (2 * c) >= 256) c *= 2;
        }
    }
    int shift = 0;
    while ((1 << shift) < c) ++shift;
    a.chunk_shift = shift;
    a.chunk_len = c > 1 ? ((a.n + c - 1) / c + 63) / 64 * 64 : a.n;
    if (c == 1) a.vbits = nullptr;
    *chunks = c;
    unsigned blocks = (unsigned)groups << shift;
    a.chunk_rounds = 0;
    // automatic chunks over more than one wave of resident blocks: the decreasing round-major
    // plan (in a single wave equal chunks are best: the longest block sets the kernel time;
    // N=1024, 1024 blocks: 37.3 us equal, 40.6 us with the plan)
    if (c > 1 && split <= 0 && !a.seg_begin && (long)groups * c > slots) {
        const int rounds = chunk_plan(a.n, c, a.chunk_off);
        a.chunk_rounds = rounds;
        a.groups = groups;
        blocks = (unsigned)groups * (unsigned)rounds;
    }
    const bool ff = a.g.full_fov != 0;
    cudaError_t e;
    if (a.seg_begin) {
        // direct phase B when every offset between agents inside the arena (on the torus: every
        // minimal image, at most half the extent) lies within the cull radius; any state is
        // still handled exactly, only more slowly
        const bool torus = a.ud.torus != 0;
        double ext2 = (double)arena_w * arena_w + (double)arena_h * arena_h;
        if (torus) ext2 *= 0.25;
        const bool direct = ext2 <= (double)a.radius0 * a.radius0 * a.g.cull;
        void (*kern)(StepArgs);
        if (!torus)
            kern = ff ? (direct ? vpf_pairs_group_seg_kernel<true, true, false>
                                : vpf_pairs_group_seg_kernel<true, false, false>)
                      : (direct ? vpf_pairs_group_seg_kernel<false, true, false>
                                : vpf_pairs_group_seg_kernel<false, false, false>);
        else
            kern = ff ? (direct ? vpf_pairs_group_seg_kernel<true, true, true>
                                : vpf_pairs_group_seg_kernel<true, false, true>)
                      : (direct ? vpf_pairs_group_seg_kernel<false, true, true>
                                : vpf_pairs_group_seg_kernel<false, false, true>);
        e = launch_pdl(kern, blocks, 32, smem, stream, a);
    } else {
        const bool torus = a.ud.torus != 0;
        if (ff && !torus) e = launch_pdl(vpf_pairs_group_kernel<true, false>, blocks, 32, smem, stream, a);
        else if (!torus) e = launch_pdl(vpf_pairs_group_kernel<false, false>, blocks, 32, smem, stream, a);
        else if (ff) e = launch_pdl(vpf_pairs_group_kernel<true, true>, blocks, 32, smem, stream, a);
        else e = launch_pdl(vpf_pairs_group_kernel<false, true>, blocks, 32, smem, stream, a);
    }
    return check_cuda(e, "vpf_pairs_group_kernel launch");
}

template <bool TORUS, bool HETERO, bool TMA>
static int launch_tiled(const StepArgs &a, int warps, cudaStream_t stream) {
    auto kern = vpf_pairs_tiled_kernel<TORUS, HETERO, TMA>;
    int st = allow_dynamic_smem((const void *)kern, 200 * 1024, "vpf_pairs_tiled_kernel smem");
    if (st) return st;
    const size_t smem = tiled_smem_bytes(warps, a.tile, a.g.words, HETERO,
                                         tile_buffers(a.n, a.tile));
    const int blocks = (a.n + warps - 1) / warps;
    return check_cuda(launch_pdl(kern, (unsigned)blocks, (unsigned)(warps * 32), smem, stream, a),
                      "vpf_pairs_tiled_kernel launch");
}

static bool aligned16(const void *p) { return p == nullptr || ((uintptr_t)p & 15u) == 0; }

static dfl split_d(double v) { return {(float)v, (float)(v - (double)(float)v)}; }

UpdateDf make_update_df(const abm_vf_params *p, int phi_ok) {
    UpdateDf u;
    u.gam = split_d(p->gam);
    u.v0 = split_d(p->v0);
    u.alp0 = split_d(p->alp0);
    u.alp1 = split_d(p->alp1);
    u.bet0 = split_d(p->bet0);
    u.bet1 = split_d(p->bet1);
    u.max_vel = split_d(p->max_vel);
    u.max_th = split_d(p->max_th);
    u.dt = split_d(p->dt);
    u.bx0 = split_d(p->window_pad);
    u.bx1 = split_d(p->window_pad + p->width);
    u.by0 = split_d(p->window_pad);
    u.by1 = split_d(p->window_pad + p->height);
    u.limit = p->limit_movement != 0;
    u.torus = p->boundary == ABM_BOUNDARY_INFINITE;
    u.phi_ok = phi_ok;
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
        int3 th = resolve_pair(f.cd, f.sd, ex, ey, rj, resolve_grid(g), unc_t, unc_h, u, ps2, t,
                               h);
        t = th.x;
        h = th.y;
        if (a.diag) {
            atomicAdd(&a.diag[ABM_DIAG_PAIRS_RESOLVED], 1ull);
            if (th.z) atomicAdd(&a.diag[ABM_DIAG_NEAR_BOUNDARY], 1ull);
        }
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

constexpr int kVswrmWarps = 8;

__global__ void __launch_bounds__(32 * kVswrmWarps) vswrm_kernel(const VswrmArgs a) {
    __shared__ uint32_t lists[kVswrmWarps][256];
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= a.n) return;
    const uint32_t *vb = a.bits + (size_t)warp * a.g.words;
    long long bc, bs, ec, es;
    warp_integrals<8, 4>(vb, a.g, lists[threadIdx.x >> 5], 256, bc, bs, ec, es);
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

// ---------------------------------------------------------------------------- multi-step runs
// `steps` steps of one(in, out) between the states a and b: one eager step a -> b (it builds
// the grid tables and the stream's workspace, which no graph capture may do), then whole
// chunks of `chunk` (even) steps replayed from a graph captured on the stream, then the rest
// eagerly.  The final state is in a after an even number of steps, in b after an odd one.
// A legacy default stream (NULL) cannot be captured: every step is then launched eagerly.
template <class StepFn>
static int run_steps(abm_swarm_state *a, abm_swarm_state *b, int steps, int chunk,
                     cudaStream_t s, StepFn one, const char *fn) {
    if (steps < 0 || chunk < 0)
        return set_error(ABM_ERR_INVALID_ARG, "%s: steps=%d graph_chunk=%d", fn, steps, chunk);
    if (steps == 0) return ABM_OK;
    int warn = one(a, b);
    if (warn < 0) return warn;
    int done = 1;
    chunk &= ~1;
    if (s != nullptr && chunk >= 2 && steps - done >= chunk) {
        int st = check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                            "cudaStreamBeginCapture");
        if (st) return st;
        int step_st = ABM_OK;
        for (int k = 0; k < chunk && step_st >= 0; ++k) step_st = (k % 2 == 0) ? one(b, a) : one(a, b);
        cudaGraph_t graph = nullptr;
        st = check_cuda(cudaStreamEndCapture(s, &graph), "cudaStreamEndCapture");
        if (step_st < 0 || st) {
            if (graph) cudaGraphDestroy(graph);
            return step_st < 0 ? step_st : st;
        }
        cudaGraphExec_t exec = nullptr;
        st = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(graph);
        if (st) return st;
        while (steps - done >= chunk && !st) {   // b -> ... -> b
            st = check_cuda(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
            done += chunk;
        }
        cudaGraphExecDestroy(exec);   // freed once its launches complete
        if (st) return st;
    }
    for (; done < steps; ++done) {
        const int st = (done % 2 == 1) ? one(b, a) : one(a, b);
        if (st < 0) return st;
    }
    return warn;
}

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

int abm_vpf_set_step_mode(int32_t mode, int32_t warps_per_agent) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    if (mode < 0 || mode > 3) return set_error(ABM_ERR_INVALID_ARG, "mode=%d", mode);
    if (warps_per_agent && warps_per_agent != 1 && warps_per_agent != 2 && warps_per_agent != 4)
        return set_error(ABM_ERR_INVALID_ARG, "warps_per_agent=%d", warps_per_agent);
    g_mode = mode;
    if (warps_per_agent) g_wpa = warps_per_agent;
    return ABM_OK;
}

int abm_vpf_set_step_split(int32_t chunks) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    if (chunks < 0 || chunks > 16 || (chunks & (chunks - 1)))
        return set_error(ABM_ERR_INVALID_ARG, "chunks=%d", chunks);
    g_split = chunks;
    return ABM_OK;
}

int abm_vpf_get_step_split(int32_t *chunks) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    if (chunks) *chunks = g_split;
    return ABM_OK;
}

int abm_vpf_get_step_mode(int32_t *mode, int32_t *warps_per_agent) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    if (mode) *mode = g_mode;
    if (warps_per_agent) *warps_per_agent = g_wpa;
    return ABM_OK;
}

// Launch of one step given the grid tables and the sincos table; shared by
// abm_vpf_flock_step, abm_vpf_flock_batched and abm_vpf_flock_step_noalloc.
static int step_launch(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                       const abm_vf_params *p, const abm_agent_overrides *ov,
                       uint32_t *vpf_bits_dev, double *terms_dev, unsigned long long *diag_dev,
                       cudaStream_t s, const GridDev *g, const float4 *sctab,
                       const Workspace &ws, const char *fn, const int *seg_begin = nullptr, const int *seg_end = nullptr,
                       const int *order = nullptr) {
    int st;
    int warps, tile, mode, wpa, split;
    abm_vpf_get_step_config(&warps, &tile);
    abm_vpf_get_step_mode(&mode, &wpa);
    abm_vpf_get_step_split(&split);
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
    a.radius0 = (float)p->radius;
    a.bits = vpf_bits_dev;
    a.terms = terms_dev;
    a.diag = diag_dev;
    a.W = {(float)p->width, (float)(p->width - (double)(float)p->width)};
    a.H = {(float)p->height, (float)(p->height - (double)(float)p->height)};
    a.ud = make_update_df(p, g->phi_ok);
    a.sctab = sctab;
    a.sums = ws.sums;
    a.vbits = seg_begin ? nullptr : ws.vbits;
    a.pair_loads = ((uintptr_t)in->x % 8 == 0 && (uintptr_t)in->y % 8 == 0) ? 1 : 0;
    a.g = *g;
    a.seg_begin = seg_begin;
    a.seg_end = seg_end;
    a.order = order;
    const bool torus = p->boundary == ABM_BOUNDARY_INFINITE;
    const bool hetero = a.radius != nullptr;
    // auto: the l1 form while the positions fit comfortably in L1, tiled beyond; segmented
    // (batched) swarms always use the l1 form
    // the group form: equal radii; on a torus, width and height exact in float32
    const bool group_ok = !hetero && n < (1 << kGroupTagShift) &&
                          (!torus || (a.W.lo == 0.f && a.H.lo == 0.f));
    if (mode == 3 && !group_ok)
        return set_error(ABM_ERR_UNSUPPORTED,
                         "%s: the group form needs equal radii (on a torus: width and height "
                         "exact in float32)", fn);
    // automatic: the group form for one swarm up to 16384 agents and for batched sweeps
    const bool use_group = group_ok && (mode == 3 || (mode == 0 && (seg_begin || n <= 16384)));
    const bool use_l1 = !use_group && (seg_begin || mode == 1 || (mode == 0 && n <= 16384));
    int chunks = 1;
    if (use_group) {
        st = launch_group(a, split, p->width, p->height, s, &chunks);
    } else if (use_l1) {
        if (!torus && !hetero) st = launch_l1<false, false>(a, wpa, split, s, &chunks);
        else if (!torus && hetero) st = launch_l1<false, true>(a, wpa, split, s, &chunks);
        else if (torus && !hetero) st = launch_l1<true, false>(a, wpa, split, s, &chunks);
        else st = launch_l1<true, true>(a, wpa, split, s, &chunks);
    } else {
        a.tile = std::min(tile, ((n + 31) / 32) * 32);
        const long per = (hetero ? 3L : 2L) * 4L;   // bytes per staged neighbour
        const long room = (long)(200 * 1024) - (long)tiled_smem_bytes(warps, 0, g->words, hetero, 1);
        if (room < 2 * 32 * per)
            return set_error(ABM_ERR_UNSUPPORTED, "%s: rv=%d too large for %d warps per block",
                             fn, p->rv, warps);
        int t = a.tile;
        if (t >= n && (long)t * per > room) t = (int)((room / per) / 32 * 32);
        if (t < n && 2L * t * per > room) t = (int)((room / (2 * per)) / 32 * 32);
        a.tile = t;
        const bool tma = aligned16(a.x) && aligned16(a.y) && aligned16(a.radius);
        if (!torus && !hetero) st = tma ? launch_tiled<false, false, true>(a, warps, s)
                                         : launch_tiled<false, false, false>(a, warps, s);
        else if (!torus && hetero) st = tma ? launch_tiled<false, true, true>(a, warps, s)
                                             : launch_tiled<false, true, false>(a, warps, s);
        else if (torus && !hetero) st = tma ? launch_tiled<true, false, true>(a, warps, s)
                                             : launch_tiled<true, false, false>(a, warps, s);
        else st = tma ? launch_tiled<true, true, true>(a, warps, s)
                      : launch_tiled<true, true, false>(a, warps, s);
    }
    if (st) return st;
    if (chunks > 1) {
        const int blocks = (n + kFinishWarps - 1) / kFinishWarps;
        const size_t smem = (size_t)kFinishWarps * (g->words + kFinishList) * sizeof(uint32_t);
        st = check_cuda(launch_dependent(hetero ? vpf_finish_kernel<true>
                                                : vpf_finish_kernel<false>,
                                         blocks, 32 * kFinishWarps, smem, s, a),
                        "vpf_finish_kernel launch");
    } else {
        constexpr int kUpd = 64;
        st = check_cuda(launch_dependent(hetero ? vpf_update_kernel<true>
                                                : vpf_update_kernel<false>,
                                         (n + kUpd - 1) / kUpd, kUpd, 0, s, a),
                        "vpf_update_kernel launch");
    }
    if (st) return st;
    return g->phi_ok ? ABM_OK : ABM_WARN_PHI_MISMATCH;
}

static int step_validate(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                         const abm_vf_params *p, const char *fn) {
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
    return ABM_OK;
}

int abm_vpf_flock_step(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                       const abm_vf_params *p, const abm_agent_overrides *ov,
                       uint32_t *vpf_bits_dev, double *terms_dev,
                       unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_flock_step";
    int st = step_validate(in, out, n, p, fn);
    if (st || n == 0) return st;
    const GridDev *g = grid_for(p->rv, p->fov0, p->fov1, &st);
    if (!g) return st;
    if ((st = ensure_sincos_table())) return st;
    const float4 *sctab = sincos_table_dev(&st);
    if (!sctab) return st;
    const Workspace ws = workspace((cudaStream_t)stream, n, g->words, &st);
    if (!ws.sums) return st;
    return step_launch(in, out, n, p, ov, vpf_bits_dev, terms_dev, diag_dev,
                       (cudaStream_t)stream, g, sctab, ws, fn);
}

int abm_vpf_flock_step_host(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                            const abm_vf_params *p, const abm_agent_overrides *ov,
                            void *stream) {
    const char *fn = "abm_vpf_flock_step_host";
    int st = step_validate(in, out, n, p, fn);
    if (st || n == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const GridDev *g = grid_for(p->rv, p->fov0, p->fov1, &st);
    if (!g) return st;
    if ((st = ensure_sincos_table())) return st;
    const float4 *sctab = sincos_table_dev(&st);
    if (!sctab) return st;
    const Workspace ws = workspace(s, n, g->words, &st);
    if (!ws.sums) return st;
    float *stage = host_staging(s, n, &st);
    if (!stage) return st;
    const float *hin[4] = {in->x, in->y, in->theta, in->v};
    float *hout[4] = {out->x, out->y, out->theta, out->v};
    const float *din[4];
    float *dout[4];
    bool zin = true, zout = true;
    for (int k = 0; k < 4; ++k) {
        din[k] = (const float *)device_view(hin[k]);
        dout[k] = (float *)device_view(hout[k]);
        zin = zin && din[k];
        zout = zout && dout[k];
    }
    const size_t bytes = sizeof(float) * (size_t)n;
    if (zin) {
        const int blocks = std::min((n + 255) / 256, 4 * 152);
        gather_state_kernel<<<blocks, 256, 0, s>>>(din[0], din[1], din[2], din[3], stage, n);
        st = check_cuda(cudaGetLastError(), "gather_state_kernel launch");
    } else {
        for (int k = 0; k < 4 && !st; ++k)
            st = check_cuda(cudaMemcpyAsync(stage + k * (size_t)n, hin[k], bytes,
                                            cudaMemcpyHostToDevice, s),
                            "cudaMemcpyAsync(state to device)");
    }
    if (st) return st;
    abm_swarm_state sin{stage, stage + n, stage + 2 * (size_t)n, stage + 3 * (size_t)n};
    float *so = stage + 4 * (size_t)n;
    abm_swarm_state sout = zout ? abm_swarm_state{dout[0], dout[1], dout[2], dout[3]}
                                : abm_swarm_state{so, so + n, so + 2 * (size_t)n,
                                                  so + 3 * (size_t)n};
    const int r = step_launch(&sin, &sout, n, p, ov, nullptr, nullptr, nullptr, s, g, sctab, ws,
                              fn);
    if (r < 0 || zout) return r;
    const float *src[4] = {sout.x, sout.y, sout.theta, sout.v};
    for (int k = 0; k < 4 && !st; ++k)
        st = check_cuda(cudaMemcpyAsync(hout[k], src[k], bytes, cudaMemcpyDeviceToHost, s),
                        "cudaMemcpyAsync(state to host)");
    return st ? st : r;
}

int abm_vpf_flock_batched(const abm_swarm_state *in, abm_swarm_state *out, int32_t n_total,
                          const int32_t *seg_begin_dev, const int32_t *seg_end_dev,
                          const int32_t *order_dev, const abm_vf_params *p,
                          const abm_agent_overrides *ov, uint32_t *vpf_bits_dev,
                          double *terms_dev, unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_flock_batched";
    int st = step_validate(in, out, n_total, p, fn);
    if (st || n_total == 0) return st;
    if (!seg_begin_dev || !seg_end_dev)
        return set_error(ABM_ERR_INVALID_ARG, "%s: segment arrays are NULL", fn);
    const GridDev *g = grid_for(p->rv, p->fov0, p->fov1, &st);
    if (!g) return st;
    if ((st = ensure_sincos_table())) return st;
    const float4 *sctab = sincos_table_dev(&st);
    if (!sctab) return st;
    const Workspace ws = workspace((cudaStream_t)stream, n_total, g->words, &st);
    if (!ws.sums) return st;
    return step_launch(in, out, n_total, p, ov, vpf_bits_dev, terms_dev, diag_dev,
                       (cudaStream_t)stream, g, sctab, ws, fn, seg_begin_dev,
                       seg_end_dev, order_dev);
}

int abm_vpf_flock_run(abm_swarm_state *a, abm_swarm_state *b, int32_t n,
                      const abm_vf_params *p, const abm_agent_overrides *ov, int32_t steps,
                      int32_t graph_chunk, unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_flock_run";
    if (!a || !b) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL state", fn);
    auto one = [&](abm_swarm_state *in, abm_swarm_state *out) {
        return abm_vpf_flock_step(in, out, n, p, ov, nullptr, nullptr, diag_dev, stream);
    };
    return run_steps(a, b, steps, graph_chunk, (cudaStream_t)stream, one, fn);
}

int abm_vpf_flock_run_recorded(abm_swarm_state *a, abm_swarm_state *b, int32_t n,
                               const abm_vf_params *p, const abm_agent_overrides *ov,
                               int32_t steps, int32_t graph_chunk, uint32_t *vpf_bits_dev,
                               abm_vf_recording *rec, unsigned long long *diag_dev,
                               void *stream) {
    const char *fn = "abm_vpf_flock_run_recorded";
    if (!a || !b || !rec) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    if (rec->vpf_bits && n > 0 && !vpf_bits_dev)
        return set_error(ABM_ERR_INVALID_ARG, "%s: VPF series without a VPF buffer", fn);
    uint32_t *bits = rec->vpf_bits ? vpf_bits_dev : nullptr;
    auto one = [&](abm_swarm_state *in, abm_swarm_state *out) {
        const int st = abm_vpf_flock_step(in, out, n, p, ov, bits, nullptr, diag_dev, stream);
        if (st < 0) return st;
        const int rs = abm_vpf_record(out, n, bits, p->rv, rec, stream);
        return rs < 0 ? rs : st;
    };
    return run_steps(a, b, steps, graph_chunk, (cudaStream_t)stream, one, fn);
}

int abm_vpf_flock_batched_run(abm_swarm_state *a, abm_swarm_state *b, int32_t n_total,
                              const int32_t *seg_begin_dev, const int32_t *seg_end_dev,
                              const int32_t *order_dev, const abm_vf_params *p,
                              const abm_agent_overrides *ov, int32_t steps, int32_t graph_chunk,
                              unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_flock_batched_run";
    if (!a || !b) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL state", fn);
    auto one = [&](abm_swarm_state *in, abm_swarm_state *out) {
        return abm_vpf_flock_batched(in, out, n_total, seg_begin_dev, seg_end_dev, order_dev, p,
                                     ov, nullptr, nullptr, diag_dev, stream);
    };
    return run_steps(a, b, steps, graph_chunk, (cudaStream_t)stream, one, fn);
}

int abm_vpf_flock_step_noalloc(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                               const abm_vf_params *p, const abm_agent_overrides *ov,
                               uint32_t *vpf_bits_dev, double *terms_dev,
                               unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_vpf_flock_step_noalloc";
    int st = step_validate(in, out, n, p, fn);
    if (st || n == 0) return st;
    if (n > kNoAllocMaxAgents)
        return set_error(ABM_ERR_INVALID_ARG, "%s: n=%d exceeds the no-alloc maximum of %d agents",
                         fn, n, kNoAllocMaxAgents);
    if (p->rv > kNoAllocMaxRv)
        return set_error(ABM_ERR_RV, "%s: rv=%d exceeds the no-alloc maximum of %d pixels", fn,
                         p->rv, kNoAllocMaxRv);
    NoAllocDevice *d = noalloc_device(&st);
    if (!d) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // one host thread at a time per device, from the state check through the launches
    std::lock_guard<std::mutex> lk(d->mu);
    const bool need_grid =
        !d->grid_loaded || d->rv != p->rv || d->fov0 != p->fov0 || d->fov1 != p->fov1;
    if (!d->base || !d->sincos_loaded || need_grid) {
        // set-up copies from host memory: refused while the stream is being captured, since a
        // captured copy would read host memory that is gone when the graph runs
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        st = check_cuda(cudaStreamIsCapturing(s, &cap), "cudaStreamIsCapturing");
        if (st) return st;
        if (cap != cudaStreamCaptureStatusNone)
            return set_error(ABM_ERR_INVALID_ARG,
                             "%s: the first call on a device and the first call for a grid "
                             "(rv=%d, fov=[%g, %g]) copy set-up tables and must not be made "
                             "during stream capture", fn, p->rv, p->fov0, p->fov1);
    }
    if (!d->base) {
        void *ptr = nullptr;
        st = check_cuda(cudaGetSymbolAddress(&ptr, g_noalloc_scratch),
                        "cudaGetSymbolAddress(g_noalloc_scratch)");
        if (st) return st;
        d->base = (unsigned char *)ptr;
    }
    if ((st = ensure_sincos_table())) return st;
    if (!d->sincos_loaded) {   // set-up: the double-float sincos table into the array
        std::vector<float> tab;
        sincos_table_host(tab);
        st = check_cuda(cudaMemcpy(d->base + kNaSin, tab.data(), tab.size() * sizeof(float),
                                   cudaMemcpyHostToDevice),
                        "cudaMemcpy(no-alloc sincos table)");
        if (st) return st;
        d->sincos_loaded = true;
    }
    if (need_grid) {
        // (re)load this grid's tables into the array, ordered on the caller's stream; a copy
        // from pageable memory has read its source when it returns
        GridHostTables t;
        build_grid_host(p->rv, p->fov0, p->fov1, t);
        GridDev g = t.g;
        g.mid = (const float4 *)(d->base + kNaMid);
        g.cot2 = (const float2 *)(d->base + kNaCot2);
        g.q = (const longlong2 *)(d->base + kNaQ);
        g.cpt = (const longlong2 *)(d->base + kNaCpt);
        const struct { size_t off; const void *src; size_t bytes; } parts[] = {
            {kNaMid, t.mid.data(), t.mid.size() * sizeof(float)},
            {kNaCot2, t.cot2.data(), t.cot2.size() * sizeof(float)},
            {kNaQ, t.q.data(), t.q.size() * sizeof(long long)},
            {kNaCpt, t.cpt.data(), t.cpt.size() * sizeof(long long)}};
        d->grid_loaded = false;
        for (const auto &pt : parts) {
            st = check_cuda(cudaMemcpyAsync(d->base + pt.off, pt.src, pt.bytes,
                                            cudaMemcpyHostToDevice, s),
                            "cudaMemcpyAsync(no-alloc tables)");
            if (st) return st;
        }
        d->g = g;
        d->rv = p->rv;
        d->fov0 = p->fov0;
        d->fov1 = p->fov1;
        d->grid_loaded = true;
    }
    Workspace na_ws;   // no bitmask workspace: the one-block-per-agent or the tiled form
    na_ws.sums = (long long *)(d->base + kNaSums);
    return step_launch(in, out, n, p, ov, vpf_bits_dev, terms_dev, diag_dev, s, &d->g,
                       (const float4 *)(d->base + kNaSin), na_ws, fn);
}

int abm_vpf_polarisation(const float *theta_dev, int32_t n_total, const int32_t *offsets_dev,
                         int32_t n_instances, double *out_dev, int32_t capacity,
                         int32_t *step_dev, void *stream) {
    const char *fn = "abm_vpf_polarisation";
    if (n_total < 0 || n_instances < 0 || capacity < 0)
        return set_error(ABM_ERR_INVALID_ARG, "%s: negative size", fn);
    if (!offsets_dev && n_instances != 1)
        return set_error(ABM_ERR_INVALID_ARG, "%s: one instance without offsets", fn);
    if (n_instances == 0) return ABM_OK;
    if (!theta_dev || !out_dev || !step_dev)
        return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    polarisation_kernel<<<n_instances, 256, 0, (cudaStream_t)stream>>>(
        theta_dev, n_total, offsets_dev, out_dev, capacity, step_dev);
    return check_cuda(cudaGetLastError(), "polarisation_kernel launch");
}

int abm_vpf_record(const abm_swarm_state *s, int32_t n_total, const uint32_t *vpf_bits_dev,
                   int32_t rv, abm_vf_recording *rec, void *stream) {
    const char *fn = "abm_vpf_record";
    if (!s || !rec) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    if (n_total < 0 || rec->capacity < 0)
        return set_error(ABM_ERR_INVALID_ARG, "%s: negative size", fn);
    if (!rec->step) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL step counter", fn);
    if (n_total > 0 && (!s->x || !s->y || !s->theta || !s->v || !rec->posx || !rec->posy ||
                        !rec->orientation || !rec->velocity))
        return set_error(ABM_ERR_INVALID_ARG, "%s: NULL state or series", fn);
    int words = 0;
    if (rec->vpf_bits) {
        if (rv < 1 || rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "%s: rv=%d", fn, rv);
        if (n_total > 0 && !vpf_bits_dev)
            return set_error(ABM_ERR_INVALID_ARG, "%s: VPF series without the step's VPF", fn);
        words = (rv + 31) / 32;
    }
    const size_t items = (size_t)n_total * (words > 1 ? words : 1);
    const int blocks = (int)std::min<size_t>(std::max<size_t>((items + 255) / 256, 1), 1216);
    vf_record_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(*s, n_total, vpf_bits_dev, words,
                                                               *rec);
    return check_cuda(cudaGetLastError(), "vf_record_kernel launch");
}

int abm_vpf_check_sincos(const float *theta_dev, int32_t n, double *out_dev, void *stream) {
    if (n < 0 || (n > 0 && (!theta_dev || !out_dev)))
        return set_error(ABM_ERR_INVALID_ARG, "abm_vpf_check_sincos: bad arguments");
    if (n == 0) return ABM_OK;
    int st = ensure_sincos_table();
    if (st) return st;
    check_sincos_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(theta_dev, n, out_dev);
    return check_cuda(cudaGetLastError(), "check_sincos_kernel launch");
}

int abm_vpf_status(int32_t clear, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    int st = check_cuda(cudaStreamSynchronize(s), "abm_vpf_status: cudaStreamSynchronize");
    if (st) return st;
    unsigned v = 0;
    st = check_cuda(cudaMemcpyFromSymbol(&v, g_kernel_status, sizeof(v)),
                    "abm_vpf_status: read the status word");
    if (st) return st;
    if (v && clear) {   // clear only the bits read, so a concurrent launch's bit survives
        clear_status_kernel<<<1, 1, 0, s>>>(v);
        st = check_cuda(cudaGetLastError(), "clear_status_kernel launch");
        if (!st) st = check_cuda(cudaStreamSynchronize(s), "abm_vpf_status: clear");
        if (st) return st;
    }
    if (v & kStatusWaitTimeout)
        return set_error(ABM_ERR_TIMEOUT, "abm_vpf_status: a step kernel gave up a bounded wait "
                                          "for its staged neighbour tile; that launch's results "
                                          "are incomplete");
    return ABM_OK;
}

int abm_vpf_debug_wait_timeout(int32_t polls, unsigned long long *diag_dev, int32_t *result_dev,
                               void *stream) {
    if (polls < 1 || polls > (1 << 20) || !result_dev)
        return set_error(ABM_ERR_INVALID_ARG, "abm_vpf_debug_wait_timeout: polls=%d", polls);
    wait_timeout_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(polls, diag_dev, result_dev);
    return check_cuda(cudaGetLastError(), "wait_timeout_probe_kernel launch");
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
    const int threads = 32 * kVswrmWarps;
    const int blocks = (n_fields * 32 + threads - 1) / threads;
    vswrm_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(a);
    return check_cuda(cudaGetLastError(), "vswrm_kernel launch");
}

}  // extern "C"
