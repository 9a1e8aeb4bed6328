// vpf_forage.cu -- the collective-foraging step (abm_forage_step): agent-resource interaction,
// the social visual projection field and the agent update of the reference's foraging
// simulation, for one arena.
//
// Three launches per step on the caller's stream (four with agent-agent collisions, whose
// kernel comes first; see the collisions section):
//  * forage_resource_kernel (one block; small arenas staged in shared memory): which patch (if
//    any) holds each agent's centre; then
//    one warp per patch replays the reference's per-patch loop in agent order (the loop is
//    sequential within a patch: depletion order decides who gets the last units); then the
//    emptied patches are regenerated in patch order and the agents on no patch are notified;
//  * the social channel (abm_vpf_social_fields) on the resulting positions, modes and patches;
//  * forage_update_kernel (one warp per agent, one agent per block): private information,
//    decision processes, mode, random walk / relocation / exploitation stop, move, walls.
// Decision and motion arithmetic is FP64 (the reference's Python floats; cos / sin of the new
// heading and the turn towards a patch centre in double-float, within 1e-13 of FP64);
// positions, orientation and speed are stored as float32, rounded where the step writes them.  Random
// numbers come from a Philox-4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011) keyed by the seed, with one counter
// per agent and per patch slot, so a step is reproducible and graph-replayable.
#include <climits>
#include <cmath>
#include <cstring>

#include "../../include/abm_forage.h"
#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

// ------------------------------------------------------------------------------ Philox
// Round multipliers and Weyl key increments of Philox-4x32 as published.
constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;

__host__ __device__ inline void philox4x32_10(const uint32_t c_in[4], const uint32_t k_in[2],
                                              uint32_t out[4]) {
    uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
    uint32_t k0 = k_in[0], k1 = k_in[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)kPhiloxM0 * c0, p1 = (uint64_t)kPhiloxM1 * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// Uniform double in [0, 1) from two 32-bit words (53 random bits).
__host__ __device__ inline double u01(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Stream tags (counter word 3).
constexpr uint32_t kTagWalk = 0x57414C4Bu;    // random walk of an agent
constexpr uint32_t kTagPatch = 0x50415443u;   // regeneration of a patch slot

__device__ inline void philox_draw(uint64_t seed, uint32_t who, uint64_t count, uint32_t tag,
                                   uint32_t out[4]) {
    const uint32_t c[4] = {who, (uint32_t)count, (uint32_t)(count >> 32), tag};
    const uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    philox4x32_10(c, k, out);
}

// ------------------------------------------------------------------------------ kernels
struct ForageArgs {
    abm_forager_state ag;
    abm_patch_state pt;
    int n, np;
    abm_forage_params p;
    const uint32_t *soc;
    int words;
    int *patch_of;     // scratch: index of the patch holding each agent's centre, or -1
    int *exploit;      // scratch: 1 where the overriding mode is "exploit"
    const double *uniforms;
    unsigned long long *diag;
    const float4 *sctab;   // double-float cos/sin table (global copy)
    // 1 / Rv, 1 / (Rv / 2), 1 / (Rv - Rv / 2) for the social field's means (within one FP64
    // ulp of the divisions), and the linspace pixel step 2 pi / (Rv - 1) (the FP64 division)
    double inv_rv, inv_half, inv_rest, px_step, inv_px_step;
    double inv_vr;   // 1 / vision_range, correctly rounded
};

// Agent.get_mode (agent.py:627-639): the overriding mode, else relocate / explore by w.
__device__ inline int get_mode(const ForageArgs &a, int i) {
    const int o = a.ag.override_mode[i];
    if (o != ABM_MODE_NONE) return o;
    return a.ag.w[i] > a.p.T_w ? ABM_MODE_RELOCATE : ABM_MODE_EXPLORE;
}

// notify_agent (sims.py:29-42).
__device__ inline void notify(const ForageArgs &a, int i, int status, int res_id) {
    const int before = a.ag.env_status[i];
    a.ag.env_status_before[i] = before;
    a.ag.env_status[i] = status;
    const uint32_t mask = a.p.Tau >= 32 ? 0xFFFFFFFFu : ((1u << a.p.Tau) - 1u);
    const uint32_t nov = (status - before) > 0 ? 1u : 0u;
    a.ag.novelty[i] = ((a.ag.novelty[i] << 1) & mask) | nov;   // np.roll(novelty, 1); [0] = nov
    a.ag.pool_success[i] = 1;
    a.ag.patch_id[i] = res_id;
}

// atan2(dy, dx) in double-float on the FP32 pipe: the FP32 angle a0, refined by the angle of
// the offset rotated by -a0 (below 1e-6 rad, so its tangent w / u gives it to ~1e-18).  Within
// ~1e-13 rad of the exact angle; atan2(0, 0) = 0 as in FP64.
__device__ dfl df_atan2(double dy, double dx, const float4 *tab) {
    const float a0 = atan2f((float)dy, (float)dx);
    dfl c0, s0;
    df_sincos_df(dfl{a0, 0.f}, tab, c0, s0);
    const dfl X = df_split(dx), Y = df_split(dy);
    const dfl u = df_add(df_mul(X, c0), df_mul(Y, s0));
    const dfl w = df_sub(df_mul(Y, c0), df_mul(X, s0));
    const float uf = u.hi + u.lo;
    const float delta = uf != 0.f ? (w.hi + w.lo) / uf : 0.f;
    return two_sum(a0, delta);
}

// The sims.py:821-823 notification condition.
__device__ inline bool pooling_done(const ForageArgs &a, int i, int m) {
    return ((m == ABM_MODE_POOL || m == ABM_MODE_RELOCATE) && a.ag.pool_success[i]) ||
           a.p.pooling_time == 0;
}

// Agent loop of one patch (sims.py:800-838), run by one warp.  Its members are the agents whose
// centre is inside the patch, in agent order.  Each member only touches its own state, except
// through the patch's stock: every exploiting member takes want = min(consumption, quality)
// in turn, and the first whose take leaves nothing (!(left > 0)) empties the patch; call it D.
// So the loop reduces to (1) lane 0 replaying the stock's subtractions over the exploiting
// members to find D, then (2) every member applying its own sequence in parallel:
//   before D: [pooling notify(1, id) + teleport] [take want] [notify(-1): D's notify-all]
//   D:        [pooling notify(1, id) + teleport] [take the rest] [notify(-1)]
//   after D:  [notify(-1): D's notify-all] [notify(-1): the destroy branch]
// (without D, members just take their pooling notification and their want).  The turn
// towards the patch centre reads only the agent's own position and orientation and comes
// first for every member.
// bias_agent_towards_res_center (sims.py:544-552) for an agent at (x, y) with orientation th
// on patch k: th + ((atan2 + th) % 2 pi - pi) * 0.02, in double-float (within ~1e-14 of FP64
// before the float32 store).
__device__ float turned_orientation(const ForageArgs &a, int k, float x, float y, float thf) {
    const double R = a.p.agent_radius;
    const double pcx = a.pt.x[k] + a.pt.radius[k], pcy = a.pt.y[k] + a.pt.radius[k];
    const double dx = pcx - ((double)x + R), dy = pcy - ((double)y + R);
    const dfl two_pi = df_split(2.0 * M_PI), pi = df_split(M_PI);
    dfl cl = df_add(df_atan2(dy, dx, a.sctab), dfl{thf, 0.f});
    // Python's % with a positive divisor (collision turns may have left the orientation a
    // little outside [0, 2 pi]: a few wraps at most)
    for (int k2 = 0; k2 < 4 && df_sign(cl) < 0; ++k2) cl = df_add(cl, two_pi);
    for (int k2 = 0; k2 < 4 && df_sign(df_sub(cl, two_pi)) >= 0; ++k2) cl = df_sub(cl, two_pi);
    const dfl tn = df_add(dfl{thf, 0.f}, df_mul(df_sub(cl, pi), df_split(0.02)));
    return (float)((double)tn.hi + (double)tn.lo);
}

// with_turn: the members' turn towards the centre is applied here (otherwise by other warps).
__device__ void patch_loop(const ForageArgs &a, int k, bool *destroyed, int *mq,
                           bool with_turn) {
    const int lane = threadIdx.x & 31;
    const double R = a.p.agent_radius;
    const double want = a.p.consumption > a.pt.quality[k] ? a.pt.quality[k] : a.p.consumption;
    double left = a.pt.left[k];
    int D = INT_MAX;       // agent index of the member that empties the patch
    double take_D = 0.0;
    // (1) the stock, in member order
    for (int base = 0; base < a.n && D == INT_MAX; base += 32) {
        const int j = base + lane;
        const bool member = j < a.n && a.patch_of[j] == k;
        const unsigned ex = __ballot_sync(ABM_FULL_MASK, member && get_mode(a, j) == ABM_MODE_EXPLOIT);
        if (lane == 0) {
            for (unsigned m = ex; m; m &= m - 1u) {   // Rescource.deplete, rescource.py:118-133
                double got;
                if (left >= want) {
                    left -= want;
                    got = want;
                } else {
                    got = left;
                    left = 0.0;
                }
                if (!(left > 0.0)) {
                    D = base + __ffs(m) - 1;
                    take_D = got;
                    break;
                }
            }
        }
        D = __shfl_sync(ABM_FULL_MASK, D, 0);
    }
    take_D = __shfl_sync(ABM_FULL_MASK, take_D, 0);
    left = __shfl_sync(ABM_FULL_MASK, left, 0);
    // (2) every member's own sequence.  The members are queued (ballot compaction, order
    //     free: they are independent given D) and run 32 at a time, so the FP64 turn below is
    //     issued once per 32 members rather than once per 32 agents.
    auto member = [&](int i) {
        if (with_turn) a.ag.theta[i] = turned_orientation(a, k, a.ag.x[i], a.ag.y[i], a.ag.theta[i]);
        if (i > D) {
            notify(a, i, -1, -1);
            notify(a, i, -1, -1);
            return;
        }
        const int mode = get_mode(a, i);
        if (pooling_done(a, i, mode)) {
            notify(a, i, 1, a.pt.id[k]);
            if (a.p.teleport_exploit) {
                a.ag.x[i] = (float)(a.pt.x[k] + a.pt.radius[k] - R);
                a.ag.y[i] = (float)(a.pt.y[k] + a.pt.radius[k] - R);
            }
        }
        if (mode == ABM_MODE_EXPLOIT) {
            a.ag.collected_before[i] = a.ag.collected[i];
            a.ag.collected[i] += i == D ? take_D : want;
        }
        if (D != INT_MAX) notify(a, i, -1, -1);
    };
    int qn = 0;   // warp-uniform
    for (int base = 0; base < a.n; base += 32) {
        const int i = base + lane;
        const bool mem = i < a.n && a.patch_of[i] == k;
        const unsigned mm = __ballot_sync(ABM_FULL_MASK, mem);
        if (mem) mq[qn + __popc(mm & ((1u << lane) - 1u))] = i;
        qn += __popc(mm);
        __syncwarp();
        if (qn >= 32) {
            qn -= 32;
            member(mq[qn + lane]);
            __syncwarp();
        }
    }
    if (lane < qn) member(mq[lane]);
    __syncwarp();
    if (lane == 0) a.pt.left[k] = left;
    *destroyed = D != INT_MAX;
}

// add_new_resource_patch (sims.py:332-374) for slot k, with the slot's random stream: uniform
// integer position and units, uniform quality, retried until the patch overlaps no other
// live patch (pygame collide_circle: centre distance below the sum of the radii).
__device__ bool regenerate(const ForageArgs &a, int k) {
    const double r = a.p.patch_radius, pad = a.p.window_pad;
    double lox, hix, loy, hiy;
    if (a.p.allow_border_patch_overlap) {
        lox = pad - r; hix = a.p.width + pad - r;
        loy = pad - r; hiy = a.p.height + pad - r;
    } else {
        lox = pad; hix = a.p.width + pad - 2 * r;
        loy = pad; hiy = a.p.height + pad - 2 * r;
    }
    uint64_t cnt = a.pt.draws[k];
    for (int tries = 0; tries <= 10000; ++tries) {
        uint32_t w[4];
        philox_draw(a.p.seed, (uint32_t)k, cnt++, kTagPatch, w);
        const double x = lox + floor(u01(w[0], w[1]) * (hix - lox));
        const double y = loy + floor(u01(w[2], w[3]) * (hiy - loy));
        bool clear = true;
        for (int q = 0; q < a.np && clear; ++q) {
            if (q == k || a.pt.id[q] < 0) continue;
            const double dx = (x + r) - (a.pt.x[q] + a.pt.radius[q]);
            const double dy = (y + r) - (a.pt.y[q] + a.pt.radius[q]);
            const double rr = r + a.pt.radius[q];
            clear = dx * dx + dy * dy >= rr * rr;
        }
        if (!clear) continue;
        philox_draw(a.p.seed, (uint32_t)k, cnt++, kTagPatch, w);
        const int span = a.p.max_resc_units - a.p.min_resc_units;
        const double units =
            span > 0 ? (double)(a.p.min_resc_units + (int)floor(u01(w[0], w[1]) * span))
                     : (double)a.p.min_resc_units;
        a.pt.x[k] = x;
        a.pt.y[k] = y;
        a.pt.radius[k] = r;
        a.pt.units[k] = units;
        a.pt.left[k] = units;
        a.pt.quality[k] =
            a.p.min_resc_quality + u01(w[2], w[3]) * (a.p.max_resc_quality - a.p.min_resc_quality);
        a.pt.draws[k] = cnt;
        return true;
    }
    a.pt.draws[k] = cnt;
    return false;
}

constexpr int kResourceThreads = 256;
// Arenas up to these sizes are staged in shared memory for the resource kernel: its phases are
// chains of dependent accesses (membership, each patch's sequential loop, notifications), and
// shared memory turns each global round trip of such a chain into a few cycles.
constexpr int kStageAgents = 2048, kStagePatches = 256;

static size_t resource_smem_bytes(int n, int np) {
    return (size_t)64 * n + (size_t)64 * np + 64;
}

// The agent / patch arrays the resource phases touch, copied into shared memory: `s` gets the
// shared copies in place of the global ones.
__device__ void stage_in(const ForageArgs &a, ForageArgs &s, unsigned char *sm) {
    const int n = a.n, np = a.np, tid = threadIdx.x, nt = blockDim.x;
    double *w = reinterpret_cast<double *>(sm), *col = w + n, *colb = col + n;
    double *px = colb + n, *py = px + np, *pr = py + np, *pu = pr + np, *pl = pu + np,
           *pq = pl + np;
    uint64_t *pdr = reinterpret_cast<uint64_t *>(pq + np);
    float *x = reinterpret_cast<float *>(pdr + np), *y = x + n, *th = y + n;
    int *ovr = reinterpret_cast<int *>(th + n), *env = ovr + n, *envb = env + n,
        *pool = envb + n, *pid = pool + n, *pof = pid + n, *ptid = pof + n;
    uint32_t *nov = reinterpret_cast<uint32_t *>(ptid + np);
    for (int i = tid; i < n; i += nt) {
        w[i] = a.ag.w[i];
        col[i] = a.ag.collected[i];
        colb[i] = a.ag.collected_before[i];
        x[i] = a.ag.x[i];
        y[i] = a.ag.y[i];
        th[i] = a.ag.theta[i];
        ovr[i] = a.ag.override_mode[i];
        env[i] = a.ag.env_status[i];
        envb[i] = a.ag.env_status_before[i];
        pool[i] = a.ag.pool_success[i];
        pid[i] = a.ag.patch_id[i];
        nov[i] = a.ag.novelty[i];
    }
    for (int k = tid; k < np; k += nt) {
        px[k] = a.pt.x[k];
        py[k] = a.pt.y[k];
        pr[k] = a.pt.radius[k];
        pu[k] = a.pt.units[k];
        pl[k] = a.pt.left[k];
        pq[k] = a.pt.quality[k];
        pdr[k] = a.pt.draws[k];
        ptid[k] = a.pt.id[k];
    }
    s.ag.w = w;
    s.ag.collected = col;
    s.ag.collected_before = colb;
    s.ag.x = x;
    s.ag.y = y;
    s.ag.theta = th;
    s.ag.override_mode = ovr;
    s.ag.env_status = env;
    s.ag.env_status_before = envb;
    s.ag.pool_success = pool;
    s.ag.patch_id = pid;
    s.ag.novelty = nov;
    s.patch_of = pof;
    s.pt.x = px;
    s.pt.y = py;
    s.pt.radius = pr;
    s.pt.units = pu;
    s.pt.left = pl;
    s.pt.quality = pq;
    s.pt.draws = pdr;
    s.pt.id = ptid;
}

// Write back what the resource phases may change.
__device__ void stage_out(const ForageArgs &a, const ForageArgs &s) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < a.n; i += nt) {
        a.ag.collected[i] = s.ag.collected[i];
        a.ag.collected_before[i] = s.ag.collected_before[i];
        a.ag.x[i] = s.ag.x[i];
        a.ag.y[i] = s.ag.y[i];
        a.ag.theta[i] = s.ag.theta[i];
        a.ag.env_status[i] = s.ag.env_status[i];
        a.ag.env_status_before[i] = s.ag.env_status_before[i];
        a.ag.pool_success[i] = s.ag.pool_success[i];
        a.ag.patch_id[i] = s.ag.patch_id[i];
        a.ag.novelty[i] = s.ag.novelty[i];
    }
    for (int k = tid; k < a.np; k += nt) {
        a.pt.x[k] = s.pt.x[k];
        a.pt.y[k] = s.pt.y[k];
        a.pt.radius[k] = s.pt.radius[k];
        a.pt.units[k] = s.pt.units[k];
        a.pt.left[k] = s.pt.left[k];
        a.pt.quality[k] = s.pt.quality[k];
        a.pt.draws[k] = s.pt.draws[k];
        a.pt.id[k] = s.pt.id[k];
    }
}

__global__ void __launch_bounds__(kResourceThreads) forage_resource_kernel(ForageArgs a) {
    extern __shared__ __align__(16) unsigned char rsmem[];
    __shared__ int destroyed[ABM_FORAGE_MAX_PATCHES];
    __shared__ int mqueue[kResourceThreads / 32][64];   // per patch warp: queued members
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const bool staged = a.n <= kStageAgents && a.np <= kStagePatches;   // block-uniform
    wait_primary_grid();
    allow_dependent_launch();
    ForageArgs s = a;
    if (staged) {
        stage_in(a, s, rsmem);
        __syncthreads();
    }
    const double R = s.p.agent_radius;
    // FP32 centre and radius of each patch, once (the screen below only needs them to far
    // better than a pixel)
    __shared__ float3 pcf[kStagePatches];
    if (staged) {
        for (int k = tid; k < s.np; k += blockDim.x)
            pcf[k] = make_float3((float)(s.pt.x[k] + s.pt.radius[k]),
                                 (float)(s.pt.y[k] + s.pt.radius[k]), (float)s.pt.radius[k]);
        __syncthreads();
    }
    // 1. the patch holding each agent's centre (refine_ar_overlap_group, sims.py:45-56);
    //    patches never overlap, so there is at most one
    for (int i = tid; i < s.n; i += blockDim.x) {
        const double cx = (double)s.ag.x[i] + R, cy = (double)s.ag.y[i] + R;
        const float cxf = (float)cx, cyf = (float)cy;
        int hit = -1;
        for (int k = 0; k < s.np && hit < 0; ++k) {
            if (s.pt.id[k] < 0) continue;   // a slot whose regeneration failed
            // FP32 screen (error far below the one-pixel margin), FP64 test near the edge
            const float3 c = staged ? pcf[k]
                                    : make_float3((float)(s.pt.x[k] + s.pt.radius[k]),
                                                  (float)(s.pt.y[k] + s.pt.radius[k]),
                                                  (float)s.pt.radius[k]);
            const float rk = c.z;
            const float fx = c.x - cxf;
            const float fy = c.y - cyf;
            const float f2 = fx * fx + fy * fy;
            if (f2 > (rk + 1.f) * (rk + 1.f)) continue;
            if (f2 < (rk - 1.f) * (rk - 1.f) && rk > 1.f) {
                hit = k;
                continue;
            }
            const double dx = (s.pt.x[k] + s.pt.radius[k]) - cx;
            const double dy = (s.pt.y[k] + s.pt.radius[k]) - cy;
            if (sqrt(dx * dx + dy * dy) < s.pt.radius[k]) hit = k;
        }
        s.patch_of[i] = hit;
    }
    for (int k = tid; k < s.np; k += blockDim.x) destroyed[k] = 0;
    __syncthreads();
    // 2. each patch's agents in agent order (one warp per patch: the loop is sequential).
    //    When the state is staged and warps are left over, those warps apply the members'
    //    turn towards the patch centre meanwhile: it reads the positions before any teleport
    //    (still in global memory until the write-back) and only the member's orientation,
    //    which nothing else in this phase touches.
    const bool turn_apart = staged && s.np < nw;   // block-uniform
    if (warp < s.np || !turn_apart) {
        for (int k = warp; k < s.np; k += nw) {
            if (s.pt.id[k] < 0) continue;   // warp-uniform
            bool d = false;
            patch_loop(s, k, &d, mqueue[warp], !turn_apart);
            if (lane == 0) destroyed[k] = d ? 1 : 0;
        }
    } else {
        for (int i = (warp - s.np) * 32 + lane; i < s.n; i += (nw - s.np) * 32) {
            const int k = s.patch_of[i];
            if (k >= 0 && s.pt.id[k] >= 0)
                s.ag.theta[i] = turned_orientation(s, k, a.ag.x[i], a.ag.y[i], s.ag.theta[i]);
        }
    }
    __syncthreads();
    // 3. emptied patches are killed and regenerated in patch order (kill_resource)
    if (tid == 0) {
        for (int k = 0; k < s.np; ++k) {
            if (!destroyed[k]) continue;
            if (!s.p.regenerate_patches) {
                s.pt.id[k] = -1;
                continue;
            }
            if (!regenerate(s, k)) {
                s.pt.id[k] = -1;
                if (s.diag) atomicAdd(&s.diag[ABM_DIAG_CAPACITY], 1ull);
            }
        }
    }
    // 4. agents on no patch (sims.py:848-855), and the exploit flags of the social channel
    for (int i = tid; i < s.n; i += blockDim.x) {
        if (s.patch_of[i] < 0) {
            const int m = get_mode(s, i);
            if (pooling_done(s, i, m) || m == ABM_MODE_EXPLOIT) notify(s, i, -1, -1);
        }
        s.exploit[i] = s.ag.override_mode[i] == ABM_MODE_EXPLOIT ? 1 : 0;
    }
    if (staged) {
        __syncthreads();
        stage_out(a, s);
    }
}

// Agent.prove_orientation (agent.py:605-610).
__device__ inline double prove_orientation(double t) {
    if (t < 0) t = 2 * M_PI + t;
    if (t > M_PI * 2) t = t - 2 * M_PI;
    return t;
}

constexpr int kUpdateWarps = 1;

// One warp per agent: the lanes count the social field's pixels (coalesced word loads), lane 0
// applies the update.
__global__ void __launch_bounds__(32 * kUpdateWarps) forage_update_kernel(ForageArgs a) {
    wait_primary_grid();
    allow_dependent_launch();
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kUpdateWarps + (threadIdx.x >> 5);
    if (i >= a.n) return;   // warp-uniform
    const abm_forage_params &p = a.p;
    // lane 0's state loads are issued first, so their latency overlaps the pixel count
    uint32_t nov = 0;
    double col = 0, colb = 0, w = 0, u = 0, r01u = 0;
    int ovr = 0, mode = 0, env = 0;
    float v0f = 0, th0f = 0, x0f = 0, y0f = 0;
    uint64_t draws = 0;
    if (lane == 0) {
        nov = a.ag.novelty[i];
        col = a.ag.collected[i];
        colb = a.ag.collected_before[i];
        w = a.ag.w[i];
        u = a.ag.u[i];
        ovr = a.ag.override_mode[i];
        mode = a.ag.mode[i];
        env = a.ag.env_status[i];
        v0f = a.ag.v[i];
        th0f = a.ag.theta[i];
        x0f = a.ag.x[i];
        y0f = a.ag.y[i];
        if (a.uniforms) r01u = a.uniforms[i];
        else draws = a.ag.draws[i];
    }
    // social field statistics: mean, and the left / right halves of F_reloc_LR
    const uint32_t *bits = a.soc + (size_t)i * a.words;
    const int rv = p.rv, half = rv / 2;
    int total = 0, left = 0;
    for (int wd = lane; wd < a.words; wd += 32) {
        const uint32_t b = bits[wd];
        total += __popc(b);
        const int lo = wd * 32;
        if (lo + 32 <= half) left += __popc(b);
        else if (lo < half) left += __popc(b & ((1u << (half - lo)) - 1u));
    }
    total = __reduce_add_sync(ABM_FULL_MASK, total);
    left = __reduce_add_sync(ABM_FULL_MASK, left);
    if (lane != 0) return;
    // calc_I_priv (agent.py:180-187): novelty memory and the units collected this step
    const double I_priv = p.F_N * (nov ? 1.0 : 0.0) + p.F_R * (col - colb);
    if (a.ag.ipriv) a.ag.ipriv[i] = I_priv;
    // update_decision_processes (agent.py:194-210)
    const double w_p = w > p.T_w ? w : 0.0;
    const double u_p = u > p.T_u ? u : 0.0;
    const double dw = p.Eps_w * ((double)total * a.inv_rv) - p.g_w * (w - p.B_w) - u_p * p.S_uw;
    const double du = p.Eps_u * I_priv - p.g_u * (u - p.B_u) - w_p * p.S_wu;
    w += dw;
    u += du;
    if (w > p.w_max) w = p.w_max;
    if (w < -p.w_max) w = -p.w_max;
    if (u > p.u_max) u = p.u_max;
    if (u < -p.u_max) u = -p.u_max;
    a.ag.w[i] = w;
    a.ag.u[i] = u;
    // mode and motion increments (agent.py:223-259); tr_u compares u with T_w (agent.py:622)
    const double vel0 = (double)v0f;
    double vel = 0.0, theta = 0.0;
    const int cur = ovr != ABM_MODE_NONE ? ovr : (w > p.T_w ? ABM_MODE_RELOCATE : ABM_MODE_EXPLORE);
    if (cur != ABM_MODE_COLLIDE) {
        const bool tw = w > p.T_w, tu = u > p.T_w;
        const bool on_patch = env == 1;
        int action;   // 0 random walk, 1 relocate, 2 exploit
        if (!tw && !tu) action = 0;
        else if (tw && tu) action = on_patch ? 2 : 1;
        else if (tw) action = 1;
        else action = on_patch ? 2 : 0;
        if (action == 0) {   // supcalc.random_walk(desired_vel=max_exp_vel)
            double r01;
            if (a.uniforms) {
                r01 = r01u;
            } else {
                uint32_t wd[4];
                philox_draw(p.seed, (uint32_t)i, draws, kTagWalk, wd);
                r01 = u01(wd[0], wd[1]);
                a.ag.draws[i] = draws + 1;
            }
            vel = p.exp_vel_max;
            theta = p.exp_theta_min + (p.exp_theta_max - p.exp_theta_min) * r01;
            mode = ABM_MODE_EXPLORE;
            ovr = ABM_MODE_NONE;
        } else if (action == 1) {   // supcalc.F_reloc_LR(v, soc_v_field, max_exp_vel)
            const double le = (double)left * a.inv_half;
            const double re = (double)(total - left) * a.inv_rest;
            vel = p.exp_vel_max - vel0;
            theta = (le - re) * p.reloc_theta_max;
            mode = ABM_MODE_RELOCATE;
            ovr = ABM_MODE_NONE;
        } else {
            vel = -vel0 * p.exp_stop_ratio;
            theta = 0.0;
            mode = ABM_MODE_EXPLOIT;
            ovr = ABM_MODE_EXPLOIT;
        }
    }
    a.ag.mode[i] = mode;
    a.ag.override_mode[i] = ovr;
    // the move (agent.py:263-277), prove_velocity (agent.py:612-620), reflect_from_walls
    double th = prove_orientation((double)th0f + theta);
    double v = vel0 + vel;
    const int after = ovr != ABM_MODE_NONE ? ovr : (w > p.T_w ? ABM_MODE_RELOCATE : ABM_MODE_EXPLORE);
    if (after == ABM_MODE_EXPLORE && fabs(v) > 1.0) v = p.exp_vel_max;
    // cos / sin of the new heading in double-float on the FP32 pipe (within 1e-13 of FP64; the
    // position is stored as float32)
    dfl cd, sd;
    df_sincos_df(df_split(th), a.sctab, cd, sd);
    const double cs = (double)cd.hi + (double)cd.lo, sn = (double)sd.hi + (double)sd.lo;
    double x = (double)x0f + v * cs;
    double y = (double)y0f - v * sn;
    const double R = p.agent_radius, bx0 = p.window_pad, bx1 = p.window_pad + p.width;
    const double by0 = p.window_pad, by1 = p.window_pad + p.height;
    const double cx = x + R, cy = y + R;
    if (cx < bx0) {
        x = bx0 - R;
        if (M_PI / 2 <= th && th < M_PI) th -= M_PI / 2;
        else if (M_PI <= th && th <= 3 * M_PI / 2) th += M_PI / 2;
        th = prove_orientation(th);
    }
    if (cx > bx1) {
        x = bx1 - R - 1;
        if (3 * M_PI / 2 <= th && th < 2 * M_PI) th -= M_PI / 2;
        else if (0 <= th && th <= M_PI / 2) th += M_PI / 2;
        th = prove_orientation(th);
    }
    if (cy < by0) {
        y = by0 - R;
        if (M_PI / 2 <= th && th <= M_PI) th += M_PI / 2;
        else if (0 <= th && th < M_PI / 2) th -= M_PI / 2;
        th = prove_orientation(th);
    }
    if (cy > by1) {
        y = by1 - R - 1;
        if (3 * M_PI / 2 <= th && th <= 2 * M_PI) th += M_PI / 2;
        else if (M_PI <= th && th < 3 * M_PI / 2) th -= M_PI / 2;
        th = prove_orientation(th);
    }
    a.ag.x[i] = (float)x;
    a.ag.y[i] = (float)y;
    a.ag.theta[i] = (float)th;
    a.ag.v[i] = (float)v;
    a.ag.collected_before[i] = col;
    if (a.diag && !(isfinite(x) && isfinite(y) && isfinite(th) && isfinite(v) && isfinite(w) &&
                    isfinite(u)))
        atomicAdd(&a.diag[ABM_DIAG_NONFINITE], 1ull);
}

// ------------------------------------------------------------------------------ collisions
// The agent-agent block of Simulation.start (sims.py:735-784), run before the resource
// interaction when collide_agents is set.  pygame's groupcollide lists, for every agent in
// agent order, the agents whose rect circles overlap its own (collide_circle with the radius
// raised by the proximity distance 2; rects hold int(position), width int(2R)).  Every listed
// agent then makes one proximity manoeuvre (agent_agent_collision_proximity, sims.py:421-474)
// unless ghost mode spares a pair with an exploiting member.  A manoeuvre reads only the
// positions (unchanged in this block) and the manoeuvring agent's own heading, so an agent's
// manoeuvres are its own sequence: as many as the lists that hold it, one after another.
// forage_collide_kernel runs one block per agent: one pass over the other agents counts the
// lists that hold it, decides whether it ends up among the collided agents (sims.py:756-776)
// and collects its vicinity (the agents within 2R + 20); then the manoeuvres -- the proximity
// field (Agent.projection_field with keep_distance_info over the full circle,
// agent.py:457-597), the turn away from the fuller half, the stop when the 200 pixels ahead
// are occupied -- and the collide-mode bookkeeping (sims.py:779-784).  The field's half and
// front means are numpy means, so the sums replay numpy's pairwise summation order exactly;
// the geometry follows the reference's FP64 operation sequence (products and sums rounded
// separately, as numpy does them).  Only the heading changes between manoeuvres, so distance,
// projection width and obstacle direction are computed once.
constexpr int kCollideCap = 1024;          // agents within 2R + 20 of one agent

// collide_circle on the rects: squared centre distance <= (2 (R + 2))^2, all integers (the
// agent radius is an integer).
__device__ inline bool rects_collide(float xa, float ya, float xb, float yb, long long half,
                                     long long rr2) {
    // non-finite or absurd coordinates (no rect) never collide
    if (!(fabsf(xa) < 1e9f && fabsf(ya) < 1e9f && fabsf(xb) < 1e9f && fabsf(yb) < 1e9f))
        return false;
    const long long dx = ((long long)xa + half) - ((long long)xb + half);
    const long long dy = ((long long)ya + half) - ((long long)yb + half);
    return dx * dx + dy * dy <= rr2;
}

struct CollideEntry {
    double d;          // squared centre distance (FP64, products and sum rounded separately)
    double ox, oy;     // offset from the focal centre to the obstacle centre
    double u2x, u2y;   // its unit vector (FP64 route only)
    unsigned long long dkey;   // bits of d: non-negative doubles order like their bits
    float x, y;        // top-left position
    int j;             // agent index (the reference's list order)
    int same;          // same top-left position as the focal agent: skipped (agent.py:500)
    int H, frac;       // proj_size / 2 = H + f: floor, and whether f > 0 (heading-independent)
    double hp;         // proj_size / 2 in FP64 when FP32 could not decide H and f
    int hp_exact;      // hp holds it
    float fox, foy;    // the offset in FP32
    int s0, e0;        // untrimmed int(t - ps/2), int(t + ps/2) under the current heading
    int fov;           // bearing inside (-pi, pi)
    int redo;          // FP32 bearing too close to a decision boundary: FP64 route
    int r0l, r0h, r1l, r1h, r2l, r2h;   // fill ranges: wrap below 0 (1), wrap above Rv (1),
                                         // main run (w), numpy slice bounds
};

// int(t - ps/2), int(t + ps/2) for an integer pixel t (truncation toward zero,
// agent.py:545-548): from ps/2 = H + f with f far from 0 and 1, or from the FP64 value.
__device__ __forceinline__ void proj_interval(int t, const CollideEntry &E, int &s0, int &e0) {
    if (E.hp_exact) {
        s0 = (int)__dsub_rn((double)t, E.hp);
        e0 = (int)__dadd_rn((double)t, E.hp);
    } else {
        s0 = (E.frac && t - E.H >= 1) ? t - E.H - 1 : t - E.H;
        e0 = t + E.H;
    }
}

struct CollideSmem {
    size_t ent, rank, code, val, nodes, total;
};

static __host__ __device__ __forceinline__ size_t collide_align16(size_t b) {
    return (b + 15) & ~size_t(15);
}

constexpr int kCollideMaxLeaves = 3 * 160;   // pairwise leaves of three slices of <= 8192
constexpr int kCollideMaxNodes = 2 * kCollideMaxLeaves;

// Dynamic shared memory of forage_collide_kernel: entries, fill order, pixel codes, the
// pairwise trees' node values, and the node table (leaf start / length, children, level).
static __host__ __device__ __forceinline__ CollideSmem collide_smem(int rv, int cap) {
    CollideSmem l;
    l.ent = 0;
    l.rank = collide_align16((size_t)cap * sizeof(CollideEntry));
    l.code = collide_align16(l.rank + (size_t)cap * sizeof(int));
    l.val = collide_align16(l.code + (size_t)rv);
    // node values, then the per-pixel writer array of the fills
    l.nodes = collide_align16(l.val + (size_t)kCollideMaxNodes * sizeof(double) +
                              (size_t)rv * sizeof(int));
    l.total = collide_align16(l.nodes + (size_t)kCollideMaxNodes * 4 * sizeof(int));
    return l;
}

// numpy slice bounds a[lo:hi] on n elements (negative indices count from the end, clamped).
__device__ __forceinline__ void np_slice_bounds(long long lo, long long hi, int n, int &l, int &h) {
    if (lo < 0) { lo += n; if (lo < 0) lo = 0; }
    if (hi < 0) { hi += n; if (hi < 0) hi = 0; }
    if (lo > n) lo = n;
    if (hi > n) hi = n;
    l = (int)lo;
    h = (int)hi;
}

// supcalc.unit_vector (supcalc.py:14-16): v / np.linalg.norm(v), products and sums rounded
// separately.
__device__ __forceinline__ void unit_vector_f64(double vx, double vy, double &ux, double &uy) {
    const double nrm = __dsqrt_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)));
    ux = __ddiv_rn(vx, nrm);
    uy = __ddiv_rn(vy, nrm);
}

// supcalc.angle_between on unit vectors + the strict closed-angle rule of
// Agent.projection_field (supcalc.py:19-34, agent.py:515-523).  The angle lies in [-pi, pi],
// so numpy's remainder by 2 pi is the angle itself, plus 2 pi when negative.
__device__ __forceinline__ double closed_angle_unit_f64(double u1x, double u1y, double u2x,
                                                        double u2y) {
    double dot = __dadd_rn(__dmul_rn(u1x, u2x), __dmul_rn(u1y, u2y));
    if (dot < -1.0) dot = -1.0;
    if (dot > 1.0) dot = 1.0;
    double ang = acos(dot);
    if (__dsub_rn(__dmul_rn(u1x, u2y), __dmul_rn(u1y, u2x)) < 0) ang = -ang;
    const double tp = 2 * kPi;
    const double c = ang < 0 ? __dadd_rn(ang, tp) : (ang == 0 ? 0.0 : ang);
    return (0 < c && c < kPi) ? -c : __dsub_rn(tp, c);
}

// numpy's pairwise summation tree over [lo, lo + n) (split at half the length rounded down to
// a multiple of 8, leaves of at most 128 elements): leaves get node ids in left-to-right order
// from 0 (n0 = start, n1 = length), internal nodes (n0, n1 = left and right child) ids from
// kCollideMaxLeaves, each after its children; n2 = level (0 for a leaf).  Returns the root id.
__device__ int pw_tree(int lo, int n, int4 *node, int *nleaf, int *nnode) {
    int so[32], sl[32], st[32], sleft[32], sp = 0, ret = -1;
    so[sp] = lo; sl[sp] = n; st[sp++] = 0;
    while (sp) {
        const int t = sp - 1;
        if (sl[t] <= 128) {
            ret = (*nleaf)++;
            node[ret] = make_int4(so[t], sl[t], 0, 0);
            --sp;
            continue;
        }
        int n2 = sl[t] / 2;
        n2 -= n2 % 8;
        if (st[t] == 0) {
            st[t] = 1;
            so[sp] = so[t]; sl[sp] = n2; st[sp++] = 0;
        } else if (st[t] == 1) {
            sleft[t] = ret;
            st[t] = 2;
            so[sp] = so[t] + n2; sl[sp] = sl[t] - n2; st[sp++] = 0;
        } else {
            const int id = (*nnode)++;
            node[id] = make_int4(sleft[t], ret, max(node[sleft[t]].z, node[ret].z) + 1, 0);
            ret = id;
            --sp;
        }
    }
    return ret;
}

constexpr int kCollideBlock = 256;

__global__ void __launch_bounds__(kCollideBlock) forage_collide_kernel(ForageArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_m, s_over, s_cnt, s_any, s_both, s_nleaf, s_nnode, s_maxlv, s_root[3];
    __shared__ int s_redo, s_slow, s_occ, s_cnt6[6];
    __shared__ float s_thf;
    __shared__ double s_w, s_th, s_D, s_u1[2], s_sum[3], s_mean[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nthr = blockDim.x;
    const int i = blockIdx.x;
    wait_primary_grid();
    allow_dependent_launch();
    const int rv = a.p.rv;
    const double R = a.p.agent_radius;
    const bool ghost = a.p.ghost_mode != 0;
    const bool ei = a.ag.override_mode[i] == ABM_MODE_EXPLOIT;
    const int cap = min(a.n, kCollideCap);
    const CollideSmem L = collide_smem(rv, cap);
    CollideEntry *ent = reinterpret_cast<CollideEntry *>(smem + L.ent);
    int *rank = reinterpret_cast<int *>(smem + L.rank);
    unsigned char *code = smem + L.code;
    double *val = reinterpret_cast<double *>(smem + L.val);
    int4 *node = reinterpret_cast<int4 *>(smem + L.nodes);
    if (tid == 0) {
        s_m = 0;
        s_over = 0;
        s_cnt = 0;
        s_any = 0;
        s_both = 0;
        s_redo = 0;
        s_slow = 0;
        s_occ = 0;
        s_D = -1.0;
        for (int q = 0; q < 6; ++q) s_cnt6[q] = 0;
        s_th = (double)a.ag.theta[i];
        s_thf = a.ag.theta[i];
    }
    __syncthreads();
    // ---- one pass over the other agents: the collision lists that hold i (pygame's
    //      groupcollide: rect circles, radius + 2), and the vicinity of the proximity field
    //      (supcalc.distance(agent, agent2) < 2 R + 20, sims.py:446) with what does not depend
    //      on the heading: distance, projection half size, direction
    const long long halfw = (long long)(2 * R) / 2;
    const long long rr2 = (long long)(2 * R + 4) * (long long)(2 * R + 4);
    const float fx = a.ag.x[i], fy = a.ag.y[i];
    const double xi = fx, yi = fy;
    const double c1x = __dadd_rn(xi, R), c1y = __dadd_rn(yi, R);
    const double tp = 2 * kPi;
    {
        int cnt = 0, any = 0, both = 0;
        for (int j = tid; j < a.n; j += nthr) {
            if (j == i) continue;
            const float xj = a.ag.x[j], yj = a.ag.y[j];
            if (rects_collide(fx, fy, xj, yj, halfw, rr2)) {
                const bool ej = a.ag.override_mode[j] == ABM_MODE_EXPLOIT;
                if (!(ghost && (ei || ej))) ++cnt;
                any = 1;
                if (!ei && !ej) both = 1;
            }
            // FP32 screen (the offsets' squares are far from the threshold, or FP64 decides)
            const float fdx = xj - fx, fdy = yj - fy, lim = (float)(2 * R + 20) + 1.f;
            if (fdx * fdx + fdy * fdy > lim * lim) continue;
            const double ddx = __dsub_rn(__dadd_rn((double)xj, R), c1x);
            const double ddy = __dsub_rn(__dadd_rn((double)yj, R), c1y);
            // squared distance: a correctly rounded sqrt is monotone, so d < 2R + 20 and the
            // order of the distances follow from it (up to rounding ties of measure zero);
            // the sqrt itself is needed only for the field weight below
            const double d2 = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
            const double lim_d = 2 * R + 20;
            if (!(d2 < lim_d * lim_d)) continue;
            const int pos = atomicAdd(&s_m, 1);
            if (pos >= cap) {
                s_over = 1;
                continue;
            }
            CollideEntry e;
            e.d = d2;
            e.x = xj;
            e.y = yj;
            e.j = j;
            e.same = xj == fx && yj == fy;
            e.ox = ddx;
            e.oy = ddy;
            e.dkey = (unsigned long long)__double_as_longlong(d2);
            e.fov = 0;
            ent[pos] = e;
        }
        cnt = __reduce_add_sync(ABM_FULL_MASK, cnt);
        any = __reduce_or_sync(ABM_FULL_MASK, any);
        both = __reduce_or_sync(ABM_FULL_MASK, both);
        if (lane == 0) {
            if (cnt) atomicAdd(&s_cnt, cnt);
            if (any) atomicOr(&s_any, 1);
            if (both) atomicOr(&s_both, 1);
        }
    }
    __syncthreads();
    const int cnt = s_cnt;
    // collided_agents (sims.py:756-776): teleport_exploit keeps the non-exploiting members of
    // every colliding pair; otherwise both members, in ghost mode only pairs without exploiter
    const bool coll = a.p.teleport_exploit ? (!ei && s_any) : (!ghost ? s_any != 0 : s_both != 0);
    float v_new = a.ag.v[i];
    if (cnt > 0) {   // block-uniform
        const int h = rv / 2;
        int flo, fhi;
        np_slice_bounds((long long)h - 100, (long long)h + 100, rv, flo, fhi);
        const int m = min(s_m, cap);
        if (tid == 0) {
            s_nleaf = -1;   // the pairwise trees are built on first use
            // `distance` after the obstacle loop: the last non-coincident obstacle in list order
            int jl = -1;
            double dl2 = 0.0;
            for (int e = 0; e < m; ++e) {
                if (!ent[e].same && ent[e].j > jl) {
                    jl = ent[e].j;
                    dl2 = ent[e].d;
                }
            }
            // w = 1 - d / vision_range with the division correctly rounded by Markstein's
            // correction of a reciprocal product (Markstein, "Computation of elementary
            // functions on the IBM RISC System/6000 processor", 1990): q0 = d y, r = d - q0 v
            // (exact), q = q0 + r y, with y = 1/v correctly rounded
            const double dl = __dsqrt_rn(dl2), vr = a.p.vision_range, y = a.inv_vr;
            const double q0 = __dmul_rn(dl, y);
            const double rq = __fma_rn(-q0, vr, dl);
            s_w = __dsub_rn(1.0, __fma_rn(rq, y, q0));
            if (s_over && a.diag) atomicAdd(&a.diag[ABM_DIAG_CAPACITY], 1ull);
        }
        // fill order = the reference's stable sorts (distance ascending, then visual angle
        // descending): ascending (distance, list index); and what does not depend on the
        // heading: ps/2 = (2 atan(R / d) / (2 pi)) * Rv / 2 (agent.py:529-566) matters only
        // through its floor H and whether it has a fraction -- FP32 decides them outside a
        // relative guard of 4e-6 (its error is below 1e-6), the reference's FP64 sequence
        // inside it
        const float hp_scale = (float)((double)rv / tp);
        for (int e = tid; e < m; e += nthr) {
            CollideEntry &E = ent[e];
            if (!E.same) {
                const float hpf = atanf((float)R * rsqrtf((float)E.d)) * hp_scale;
                const float fl = floorf(hpf), fr = hpf - fl, g = 4e-6f * hpf + 1e-6f;
                E.H = (int)fl;
                E.frac = 1;
                E.hp_exact = !(fr > g && fr < 1.f - g);
                if (E.hp_exact) {
                    const double va = __dmul_rn(2.0, atan(__ddiv_rn(R, __dsqrt_rn(E.d))));
                    E.hp = __ddiv_rn(__dmul_rn(__ddiv_rn(va, tp), (double)rv), 2.0);
                }
                E.fox = (float)E.ox;
                E.foy = (float)E.oy;
            }
            const unsigned long long de = E.dkey;
            const int je = E.j;
            int r = 0;
            for (int q = 0; q < m; ++q)
                r += (ent[q].dkey < de) || (ent[q].dkey == de && ent[q].j < je);
            rank[r] = e;
        }
        __syncthreads();
        const double step = a.px_step;
        const float inv_stepf = (float)a.inv_px_step, stepf = (float)step;
        int *writer = reinterpret_cast<int *>(val + kCollideMaxNodes);   // after the node values
        // FP32 bearing guard: the FP32 angle is within 1.5e-6 rad of the exact one (heading
        // rounded to float, sincosf, products, atan2f); decisions closer than this to a pixel
        // boundary or to the field's limits are taken again on the FP64 route
        constexpr float kGuard = 4e-6f;
        for (int it = 0; it < cnt; ++it) {
            // ---- bearing, nearest pixel and untrimmed interval per entry: FP32 first
            {
                float sf, cf;
                sincosf(s_thf, &sf, &cf);
                for (int e = tid; e < m; e += nthr) {
                    CollideEntry &E = ent[e];
                    E.fov = 0;
                    E.redo = 0;
                    if (E.same) continue;
                    const float dx = E.fox, dy = E.foy;
                    // angle_between(v1, v2) with v1 ~ (cos th, -sin th): atan2(cross, dot)
                    const float dot = cf * dx - sf * dy, cross = cf * dy + sf * dx;
                    const float ang = atan2f(cross, dot);
                    const float aa = fabsf(ang);
                    const float u = (-ang + kPiF) * inv_stepf;   // closed angle = -angle
                    const float fr = u - floorf(u);
                    if (aa < kGuard || aa > kPiF - kGuard ||
                        fabsf(fr - 0.5f) * stepf < kGuard) {
                        E.redo = 1;
                        s_redo = 1;
                        if (a.diag) atomicAdd(&a.diag[ABM_DIAG_COLLIDE_FP64], 1ull);
                        continue;
                    }
                    const int t = min(max((int)floorf(u + 0.5f), 0), rv - 1);
                    proj_interval(t, E, E.s0, E.e0);
                    E.fov = 1;
                }
                for (int p = tid; p < rv; p += nthr) writer[p] = -1;
            }
            __syncthreads();
            if (s_redo) {   // block-uniform: the FP64 route of the reference (agent.py:486-571)
                if (tid == 0) {
                    double sn, cs;
                    sincos(s_th, &sn, &cs);
                    const double v1x =
                        __dsub_rn(__dadd_rn(xi, __dmul_rn(__dadd_rn(1.0, cs), R)), c1x);
                    const double v1y =
                        __dsub_rn(__dadd_rn(yi, __dmul_rn(__dsub_rn(1.0, sn), R)), c1y);
                    unit_vector_f64(v1x, v1y, s_u1[0], s_u1[1]);
                }
                __syncthreads();
                const double u1x = s_u1[0], u1y = s_u1[1];
                for (int e = tid; e < m; e += nthr) {
                    CollideEntry &E = ent[e];
                    if (!E.redo) continue;
                    unit_vector_f64(E.ox, E.oy, E.u2x, E.u2y);
                    const double ca = closed_angle_unit_f64(u1x, u1y, E.u2x, E.u2y);
                    if (!(-kPi < ca && ca < kPi)) continue;   // outside the full-circle FOV
                    // supcalc.find_nearest on np.linspace(-pi, pi, rv): argmin, first on ties
                    const double kf = floor((ca + kPi) * a.inv_px_step + 0.5);
                    const int k0 = (int)fmin(fmax(kf, 0.0), (double)(rv - 1));
                    double best = INFINITY;
                    int t = 0;
                    for (int k = max(k0 - 2, 0); k <= min(k0 + 2, rv - 1); ++k) {
                        const double ph =
                            k == rv - 1 ? kPi : __dadd_rn(__dmul_rn((double)k, step), -kPi);
                        const double dd = fabs(__dsub_rn(ph, ca));
                        if (dd < best) {
                            best = dd;
                            t = k;
                        }
                    }
                    proj_interval(t, E, E.s0, E.e0);
                    E.fov = 1;
                }
                __syncthreads();
                if (tid == 0) s_redo = 0;
            }
            // ---- exclusion trimming against the strictly closer entries (agent.py:421-445),
            //      then the entry's fill ranges (agent.py:576-588)
            for (int r = tid; r < m; r += nthr) {
                CollideEntry &F = ent[rank[r]];
                if (!F.fov) continue;
                int sx = F.s0, ex = F.e0;
                if (a.p.visual_exclusion) {
                    for (int q = 0; q < r; ++q) {
                        const CollideEntry &I = ent[rank[q]];
                        if (!I.fov || !(I.dkey < F.dkey)) continue;
                        if (sx <= I.s0 && I.s0 <= ex) ex = I.s0;
                        if (sx <= I.e0 && I.e0 <= ex) sx = I.e0;
                        if (I.s0 <= sx && I.e0 >= ex) {
                            sx = 0;
                            ex = 0;
                        }
                    }
                }
                F.r0l = F.r0h = F.r1l = F.r1h = 0;
                if (sx < 0) {
                    np_slice_bounds((long long)rv + sx, rv, rv, F.r0l, F.r0h);
                    sx = 0;
                }
                if (ex >= rv) {
                    np_slice_bounds(0, (long long)ex - rv, rv, F.r1l, F.r1h);
                    ex = rv - 1;
                }
                np_slice_bounds(sx, ex, rv, F.r2l, F.r2h);
            }
            __syncthreads();
            // ---- the fills in rank order, last write wins: each pixel keeps the largest
            //      (rank, part) that writes it; parts in write order: wrap below 0, wrap above
            //      Rv (both 1), main run (w)
            for (int r = 0; r < m; ++r) {
                const CollideEntry &E = ent[rank[r]];
                if (!E.fov) continue;
                for (int p = E.r0l + tid; p < E.r0h; p += nthr) atomicMax(&writer[p], 4 * r);
                for (int p = E.r1l + tid; p < E.r1h; p += nthr) atomicMax(&writer[p], 4 * r + 1);
                for (int p = E.r2l + tid; p < E.r2h; p += nthr) atomicMax(&writer[p], 4 * r + 2);
            }
            __syncthreads();
            // ---- pixel codes (0 empty, 1 one, 2 w) and their counts in the two halves and the
            //      200 pixels ahead; element k of the stored field is raw pixel rv - 1 - k
            {
                int l1 = 0, l2 = 0, r1 = 0, r2 = 0, f1 = 0, f2 = 0;   // ones / w's per slice
                for (int p = tid; p < rv; p += nthr) {
                    const int wr = writer[p];
                    const unsigned char cd = wr < 0 ? 0 : ((wr & 3) == 2 ? 2 : 1);
                    code[p] = cd;
                    if (cd) {
                        const int k = rv - 1 - p;
                        const int one = cd == 1, ww = cd == 2;
                        if (k < h) { l1 += one; l2 += ww; } else { r1 += one; r2 += ww; }
                        if (flo <= k && k < fhi) { f1 += one; f2 += ww; }
                    }
                }
                const int cs[6] = {l1, l2, r1, r2, f1, f2};
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const int v = __reduce_add_sync(ABM_FULL_MASK, cs[q]);
                    if (lane == 0 && v) atomicAdd(&s_cnt6[q], v);
                }
            }
            __syncthreads();
            // ---- the manoeuvre.  D = np.sign(mean(left) - mean(right)) (0 -> -1) and the
            //      front test mean(ahead) > 0 follow from the exact sums (counts x {1, w}) when
            //      they are farther apart than numpy's rounding can move them (pairwise sums
            //      of <= 8192 terms: < 40 eps relative); otherwise numpy's sums are replayed
            if (tid == 0) {
                const double w = s_w, aw = fabs(w);
                const double cl1 = s_cnt6[0], cl2 = s_cnt6[1], cr1 = s_cnt6[2], cr2 = s_cnt6[3];
                const double cf1 = s_cnt6[4], cf2 = s_cnt6[5];
                int slow = 0;
                double D = -1.0;
                if (cl1 + cl2 + cr1 + cr2 > 0) {
                    const double A = (cl1 + cl2 * w) * (double)(rv - h);
                    const double B = (cr1 + cr2 * w) * (double)h;
                    const double mag = (cl1 + cl2 * aw) * (double)(rv - h) + (cr1 + cr2 * aw) * h;
                    if (fabs(A - B) > 1e-12 * mag) D = A > B ? 1.0 : -1.0;
                    else slow |= 1;
                }
                bool occupied = false;
                if (fhi > flo && cf1 + cf2 > 0) {
                    if (w >= 0 || cf2 == 0) {
                        occupied = cf1 > 0 || w > 0;
                    } else {
                        const double S = cf1 + cf2 * w;
                        if (fabs(S) > 1e-12 * (cf1 + cf2 * aw)) occupied = S > 0;
                        else slow |= 2;
                    }
                }
                s_slow = slow;
                if (slow && a.diag) atomicAdd(&a.diag[ABM_DIAG_COLLIDE_REPLAYS], 1ull);
                s_D = D;
                s_occ = occupied;
                for (int q = 0; q < 6; ++q) s_cnt6[q] = 0;
            }
            __syncthreads();
            if (s_slow) {   // block-uniform: numpy's pairwise sums, replayed exactly
                const bool build = s_nleaf < 0;   // the three slices' pairwise trees, once
                __syncthreads();                  // (every thread has read the flag)
                if (build) {
                    if (tid == 0) {
                        int nl = 0, nn = kCollideMaxLeaves;
                        s_root[0] = pw_tree(0, h, node, &nl, &nn);
                        s_root[1] = pw_tree(h, rv - h, node, &nl, &nn);
                        s_root[2] = fhi > flo ? pw_tree(flo, fhi - flo, node, &nl, &nn) : -1;
                        int mx = 0;
                        for (int q = kCollideMaxLeaves; q < nn; ++q) mx = max(mx, node[q].z);
                        s_nnode = nn;
                        s_maxlv = mx;
                        s_nleaf = nl;
                    }
                    __syncthreads();
                }
                const int nleaf = s_nleaf, nnode = s_nnode, maxlv = s_maxlv;
                // eight lanes per leaf run its eight accumulators (adding 0.0 is skipped: exact)
                const double w = s_w;
                const int g = lane >> 3, jj = lane & 7;
                for (int base = warp * 4; base < nleaf; base += (nthr >> 5) * 4) {
                    const int q = base + g;
                    const bool act = q < nleaf;
                    const int lo = act ? node[q].x : 0, n = act ? node[q].y : 0;
                    double r = 0.0;
                    if (act && n >= 8) {
                        const unsigned char c0 = code[rv - 1 - (lo + jj)];
                        r = c0 == 0 ? 0.0 : (c0 == 1 ? 1.0 : w);
                        for (int k = 8; k < n - (n % 8); k += 8) {
                            const unsigned char c = code[rv - 1 - (lo + k + jj)];
                            if (c) r = __dadd_rn(r, c == 1 ? 1.0 : w);
                        }
                    }
                    // ((r0 + r1) + (r2 + r3)) + ((r4 + r5) + (r6 + r7)): IEEE addition commutes
                    r = __dadd_rn(r, __shfl_xor_sync(ABM_FULL_MASK, r, 1));
                    r = __dadd_rn(r, __shfl_xor_sync(ABM_FULL_MASK, r, 2));
                    r = __dadd_rn(r, __shfl_xor_sync(ABM_FULL_MASK, r, 4));
                    if (act && jj == 0) {
                        int k = n >= 8 ? n - (n % 8) : 0;
                        double res = n >= 8 ? r : 0.0;
                        for (; k < n; ++k) {
                            const unsigned char c = code[rv - 1 - (lo + k)];
                            if (c) res = __dadd_rn(res, c == 1 ? 1.0 : w);
                        }
                        val[q] = res;
                    }
                }
                __syncthreads();
                // the trees' internal nodes level by level (left + right), then the means
                if (warp == 0) {
                    for (int lv = 1; lv <= maxlv; ++lv) {
                        for (int q = kCollideMaxLeaves + lane; q < nnode; q += 32) {
                            const int4 nd = node[q];
                            if (nd.z == lv) val[q] = __dadd_rn(val[nd.x], val[nd.y]);
                        }
                        __syncwarp();
                    }
                    if (lane < 3) {
                        const int root = s_root[lane];
                        // np.mean: (0 + pairwise sum) / n
                        s_sum[lane] = root >= 0 ? __dadd_rn(0.0, val[root]) : 0.0;
                        if (lane < 2)
                            s_mean[lane] = __ddiv_rn(s_sum[lane], (double)(lane == 0 ? h : rv - h));
                    }
                    __syncwarp();
                    if (lane == 0) {
                        if (s_slow & 1) s_D = s_mean[0] > s_mean[1] ? 1.0 : -1.0;
                        if (s_slow & 2) s_occ = fhi > flo && s_sum[2] > 0;
                        s_slow = 0;
                    }
                }
                __syncthreads();
            }
            if (tid == 0) {
                if (!ei) s_th = __dsub_rn(s_th, s_D * 0.2);
                s_thf = (float)s_th;
                if (s_occ) v_new = 0.0f;
                else if (!ei) v_new = (float)a.p.exp_vel_max;
            }
            __syncthreads();
        }
    }
    if (tid != 0) return;
    if (cnt > 0) {
        if (!ei) {
            a.ag.override_mode[i] = ABM_MODE_COLLIDE;
            a.ag.mode[i] = ABM_MODE_COLLIDE;
        }
        a.ag.theta[i] = (float)s_th;
        a.ag.v[i] = v_new;
    }
    // sims.py:779-784: collide mode ends when the agent is not among the collided ones; a
    // collided agent still in collide mode is notified with -1
    const bool in_collide = a.ag.override_mode[i] == ABM_MODE_COLLIDE;
    if (!coll && in_collide) {
        a.ag.override_mode[i] = ABM_MODE_NONE;
        a.ag.mode[i] = ABM_MODE_EXPLORE;
    }
    if (coll && in_collide) notify(a, i, -1, -1);
}

static size_t collide_smem_bytes(int rv, int n) {
    return collide_smem(rv, std::min(n, kCollideCap)).total;
}

// ------------------------------------------------------------------------------ recording
// One block appends column t of every series, then advances the counter.
__global__ void __launch_bounds__(1024) forage_record_kernel(abm_forager_state ag, int n,
                                                             abm_patch_state pt, int np,
                                                             const uint32_t *soc, int words,
                                                             abm_forage_recording rec) {
    const int t = *rec.step;
    if (t < rec.capacity) {
        const size_t cap = (size_t)rec.capacity;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const size_t o = (size_t)i * cap + t;
            rec.posx[o] = (int)ag.x[i];   // Python int(): truncation toward zero
            rec.posy[o] = (int)ag.y[i];
            rec.orientation[o] = ag.theta[i];
            rec.velocity[o] = ag.v[i];
            rec.w[o] = ag.w[i];
            rec.u[o] = ag.u[i];
            rec.ipriv[o] = ag.ipriv ? ag.ipriv[i] : 0.0;
            rec.collected[o] = ag.collected[i];
            const int m = ag.mode[i];   // ifdb.mode_to_int (ifdb.py:197-206)
            rec.mode[o] = m == ABM_MODE_EXPLORE ? 0 : m == ABM_MODE_EXPLOIT ? 1
                        : m == ABM_MODE_RELOCATE ? 2 : m == ABM_MODE_COLLIDE ? 3 : -1;
            rec.patch_id[o] = ag.patch_id[i];
        }
        if (rec.soc_bits && soc) {
            const size_t total = (size_t)n * words;
            for (size_t q = threadIdx.x; q < total; q += blockDim.x) {
                const size_t i = q / words, w = q % words;
                rec.soc_bits[(i * cap + t) * words + w] = soc[q];
            }
        }
        for (int k = threadIdx.x; k < np; k += blockDim.x) {
            const size_t o = (size_t)k * cap + t;
            rec.res_posx[o] = (int)pt.x[k];
            rec.res_posy[o] = (int)pt.y[k];
            rec.res_left[o] = pt.left[k];
            rec.res_quality[o] = pt.quality[k];
            rec.res_id[o] = pt.id[k];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *rec.step = t + 1;
}

static int forage_validate(const abm_forager_state *s, int n, const abm_patch_state *pt, int np,
                           const abm_forage_params *p, const uint32_t *soc, const int *scratch,
                           const char *fn) {
    if (!s || !pt || !p) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    if (n < 0 || np < 0 || np > ABM_FORAGE_MAX_PATCHES)
        return set_error(ABM_ERR_INVALID_ARG, "%s: n=%d n_patches=%d", fn, n, np);
    if (p->Tau < 1 || p->Tau > ABM_FORAGE_MAX_TAU)
        return set_error(ABM_ERR_INVALID_ARG, "%s: Tau=%d (1..%d)", fn, p->Tau,
                         ABM_FORAGE_MAX_TAU);
    if (p->rv < 2 || p->rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "%s: rv=%d", fn, p->rv);
    if (!(p->agent_radius > 0) || !(p->width > 0) || !(p->height > 0))
        return set_error(ABM_ERR_INVALID_ARG, "%s: radius / arena not positive", fn);
    if (p->collide_agents && (p->agent_radius != floor(p->agent_radius) || p->agent_radius > 1e6))
        return set_error(ABM_ERR_INVALID_ARG,
                         "%s: agent collisions need an integer agent_radius (pygame rects)", fn);
    if (n == 0) return ABM_OK;
    const void *need[] = {s->x, s->y, s->theta, s->v, s->w, s->u, s->collected,
                          s->collected_before, s->mode, s->override_mode, s->env_status,
                          s->env_status_before, s->pool_success, s->patch_id, s->novelty,
                          s->draws, soc, scratch};
    for (const void *q : need)
        if (!q) return set_error(ABM_ERR_INVALID_ARG, "%s: a state array is NULL", fn);
    if (np > 0 && (!pt->x || !pt->y || !pt->radius || !pt->units || !pt->left || !pt->quality ||
                   !pt->id || !pt->draws))
        return set_error(ABM_ERR_INVALID_ARG, "%s: a patch array is NULL", fn);
    return ABM_OK;
}

}  // namespace abm

using namespace abm;

extern "C" {

int abm_forage_params_default(abm_forage_params *p) {
    if (!p) return set_error(ABM_ERR_INVALID_ARG, "abm_forage_params_default: NULL");
    memset(p, 0, sizeof(*p));
    p->T_w = 0.5; p->Eps_w = 3; p->g_w = 0.085; p->B_w = 0; p->w_max = 1;
    p->T_u = 0.5; p->Eps_u = 3; p->g_u = 0.085; p->B_u = 0; p->u_max = 1;
    p->S_wu = 0.25; p->S_uw = 0.01; p->F_N = 2; p->F_R = 1; p->Tau = 10;
    p->exp_vel_max = 1; p->exp_theta_min = -0.3; p->exp_theta_max = 0.3;
    p->reloc_theta_max = 0.5; p->exp_stop_ratio = 0.08;
    p->width = 1000; p->height = 1000; p->window_pad = 30; p->agent_radius = 10;
    p->consumption = 1; p->pooling_time = 0; p->teleport_exploit = 1;
    p->regenerate_patches = 1; p->allow_border_patch_overlap = 0;
    p->min_resc_units = 1000; p->max_resc_units = 1000;
    p->min_resc_quality = 1; p->max_resc_quality = 1; p->patch_radius = 30;
    p->rv = 1200; p->fov0 = -M_PI; p->fov1 = M_PI; p->vision_range = 2000;
    p->visual_exclusion = 1; p->patchwise_exclusion = 1; p->seed = 0;
    p->collide_agents = 0; p->ghost_mode = 1;
    return ABM_OK;
}

int abm_forage_record(const abm_forager_state *agents, int32_t n, const abm_patch_state *patches,
                      int32_t n_patches, const uint32_t *soc_bits_dev, int32_t rv,
                      abm_forage_recording *rec, void *stream) {
    const char *fn = "abm_forage_record";
    if (!agents || !patches || !rec || !rec->step)
        return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    if (n < 0 || n_patches < 0 || rec->capacity < 0)
        return set_error(ABM_ERR_INVALID_ARG, "%s: negative size", fn);
    if (rv < 2 || rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "%s: rv=%d", fn, rv);
    if (n > 0 && (!rec->posx || !rec->posy || !rec->orientation || !rec->velocity || !rec->w ||
                  !rec->u || !rec->ipriv || !rec->collected || !rec->mode || !rec->patch_id))
        return set_error(ABM_ERR_INVALID_ARG, "%s: an agent series is NULL", fn);
    if (n_patches > 0 && (!rec->res_posx || !rec->res_posy || !rec->res_left ||
                          !rec->res_quality || !rec->res_id))
        return set_error(ABM_ERR_INVALID_ARG, "%s: a patch series is NULL", fn);
    forage_record_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(*agents, n, *patches, n_patches,
                                                               soc_bits_dev, (rv + 31) / 32,
                                                               *rec);
    return check_cuda(cudaGetLastError(), "forage_record_kernel launch");
}

void abm_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox4x32_10(ctr, key, out);
}

int abm_forage_step(abm_forager_state *agents, int32_t n, abm_patch_state *patches,
                    int32_t n_patches, const abm_forage_params *p, uint32_t *soc_bits_dev,
                    int32_t *scratch_dev, const double *uniforms_dev,
                    unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_forage_step";
    int st = forage_validate(agents, n, patches, n_patches, p, soc_bits_dev, scratch_dev, fn);
    if (st || n == 0) return st;
    cudaStream_t s = (cudaStream_t)stream;
    ForageArgs a;
    memset(&a, 0, sizeof(a));
    a.ag = *agents;
    a.pt = *patches;
    a.n = n;
    a.np = n_patches;
    a.p = *p;
    a.soc = soc_bits_dev;
    a.words = (p->rv + 31) / 32;
    a.patch_of = scratch_dev;
    a.exploit = scratch_dev + n;
    a.uniforms = uniforms_dev;
    a.diag = diag_dev;
    a.sctab = sincos_table_dev(&st);
    if (!a.sctab) return st;
    a.inv_rv = 1.0 / p->rv;
    a.inv_half = 1.0 / (p->rv / 2);
    a.inv_rest = 1.0 / (p->rv - p->rv / 2);
    a.px_step = (kPi - (-kPi)) / (double)(p->rv - 1);   // np.linspace(-pi, pi, Rv) step
    a.inv_px_step = 1.0 / a.px_step;                     // estimates only
    a.inv_vr = 1.0 / p->vision_range;
    if (p->collide_agents) {
        if ((st = allow_dynamic_smem((const void *)forage_collide_kernel, 200 * 1024,
                                     "forage_collide_kernel smem")))
            return st;
        if ((st = check_cuda(launch_pdl(forage_collide_kernel, (unsigned)n, kCollideBlock,
                                        collide_smem_bytes(p->rv, n), s, a),
                             "forage_collide_kernel launch")))
            return st;
    }
    {
        const size_t smem = (n <= kStageAgents && n_patches <= kStagePatches)
                                ? resource_smem_bytes(n, n_patches) : 0;
        if ((st = allow_dynamic_smem((const void *)forage_resource_kernel, 200 * 1024,
                                     "forage_resource_kernel smem")))
            return st;
        if ((st = check_cuda(launch_pdl(forage_resource_kernel, 1u, kResourceThreads, smem, s, a),
                             "forage_resource_kernel launch")))
            return st;
    }
    st = abm_vpf_social_fields(agents->x, agents->y, agents->theta, nullptr, p->agent_radius,
                               a.exploit, agents->patch_id, n, p->vision_range,
                               p->visual_exclusion, p->patchwise_exclusion, p->rv, p->fov0,
                               p->fov1, soc_bits_dev, diag_dev, stream);
    if (st < 0) return st;
    return check_cuda(launch_pdl(forage_update_kernel, (unsigned)((n + kUpdateWarps - 1) /
                                                                  kUpdateWarps),
                                 32 * kUpdateWarps, 0, s, a),
                      "forage_update_kernel launch");
}

int abm_forage_run(abm_forager_state *agents, int32_t n, abm_patch_state *patches,
                   int32_t n_patches, const abm_forage_params *p, uint32_t *soc_bits_dev,
                   int32_t *scratch_dev, int32_t steps, int32_t graph_chunk,
                   abm_forage_recording *rec, unsigned long long *diag_dev, void *stream) {
    const char *fn = "abm_forage_run";
    if (steps < 0 || graph_chunk < 0)
        return set_error(ABM_ERR_INVALID_ARG, "%s: steps=%d graph_chunk=%d", fn, steps,
                         graph_chunk);
    cudaStream_t s = (cudaStream_t)stream;
    auto one = [&]() {
        int st = abm_forage_step(agents, n, patches, n_patches, p, soc_bits_dev, scratch_dev,
                                 nullptr, diag_dev, stream);
        if (st >= 0 && rec)
            st = abm_forage_record(agents, n, patches, n_patches, soc_bits_dev, p->rv, rec,
                                   stream);
        return st;
    };
    if (steps == 0) return ABM_OK;
    int st = one();   // eager: tables and kernel attributes are set up outside any capture
    if (st < 0) return st;
    int done = 1;
    if (s != nullptr && graph_chunk >= 1 && steps - done >= graph_chunk) {
        st = check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                        "cudaStreamBeginCapture");
        if (st) return st;
        int step_st = ABM_OK;
        for (int k = 0; k < graph_chunk && step_st >= 0; ++k) step_st = one();
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
        while (steps - done >= graph_chunk && !st) {
            st = check_cuda(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
            done += graph_chunk;
        }
        cudaGraphExecDestroy(exec);   // freed once its launches complete
        if (st) return st;
    }
    for (; done < steps; ++done) {
        st = one();
        if (st < 0) return st;
    }
    return ABM_OK;
}

}  // extern "C"
