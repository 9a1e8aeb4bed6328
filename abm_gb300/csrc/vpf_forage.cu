// vpf_forage.cu -- the collective-foraging step (abm_forage_step): agent-resource interaction,
// the social visual projection field and the agent update of the reference's foraging
// simulation, for one arena.
//
// Three launches per step on the caller's stream:
//  * forage_resource_kernel (one block): which patch (if any) holds each agent's centre; then
//    one warp per patch replays the reference's per-patch loop in agent order (the loop is
//    sequential within a patch: depletion order decides who gets the last units); then the
//    emptied patches are regenerated in patch order and the agents on no patch are notified;
//  * the social channel (abm_vpf_social_fields) on the resulting positions, modes and patches;
//  * forage_update_kernel (one thread per agent): private information, decision processes,
//    mode, random walk / relocation / exploitation stop, move, walls.
// Decision and motion arithmetic is FP64 (the reference's Python floats); positions,
// orientation and speed are stored as float32, rounded where the step writes them.  Random
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
__device__ void patch_loop(const ForageArgs &a, int k, bool *destroyed) {
    const int lane = threadIdx.x & 31;
    const double R = a.p.agent_radius;
    const double pcx = a.pt.x[k] + a.pt.radius[k], pcy = a.pt.y[k] + a.pt.radius[k];
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
    // (2) every member's own sequence
    for (int base = 0; base < a.n; base += 32) {
        const int i = base + lane;
        if (!(i < a.n && a.patch_of[i] == k)) continue;
        // bias_agent_towards_res_center (sims.py:544-552)
        const double dx = pcx - ((double)a.ag.x[i] + R), dy = pcy - ((double)a.ag.y[i] + R);
        double cl = fmod(atan2(dy, dx) + (double)a.ag.theta[i], 2.0 * M_PI);
        if (cl < 0) cl += 2.0 * M_PI;   // Python's % with a positive divisor
        a.ag.theta[i] = (float)((double)a.ag.theta[i] + (cl - M_PI) * 0.02);
        if (i > D) {
            notify(a, i, -1, -1);
            notify(a, i, -1, -1);
            continue;
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
    }
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

constexpr int kResourceThreads = 1024;

__global__ void __launch_bounds__(kResourceThreads) forage_resource_kernel(ForageArgs a) {
    __shared__ int destroyed[ABM_FORAGE_MAX_PATCHES];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const double R = a.p.agent_radius;
    // 1. the patch holding each agent's centre (refine_ar_overlap_group, sims.py:45-56);
    //    patches never overlap, so there is at most one
    for (int i = tid; i < a.n; i += blockDim.x) {
        const double cx = (double)a.ag.x[i] + R, cy = (double)a.ag.y[i] + R;
        int hit = -1;
        for (int k = 0; k < a.np && hit < 0; ++k) {
            if (a.pt.id[k] < 0) continue;   // a slot whose regeneration failed
            // FP32 screen (error far below the one-pixel margin), FP64 test near the edge
            const float rk = (float)a.pt.radius[k];
            const float fx = (float)(a.pt.x[k] + a.pt.radius[k]) - (float)cx;
            const float fy = (float)(a.pt.y[k] + a.pt.radius[k]) - (float)cy;
            const float f2 = fx * fx + fy * fy;
            if (f2 > (rk + 1.f) * (rk + 1.f)) continue;
            if (f2 < (rk - 1.f) * (rk - 1.f) && rk > 1.f) {
                hit = k;
                continue;
            }
            const double dx = (a.pt.x[k] + a.pt.radius[k]) - cx;
            const double dy = (a.pt.y[k] + a.pt.radius[k]) - cy;
            if (sqrt(dx * dx + dy * dy) < a.pt.radius[k]) hit = k;
        }
        a.patch_of[i] = hit;
    }
    for (int k = tid; k < a.np; k += blockDim.x) destroyed[k] = 0;
    __syncthreads();
    // 2. each patch's agents in agent order (one warp per patch: the loop is sequential)
    for (int k = warp; k < a.np; k += nw) {
        if (a.pt.id[k] < 0) continue;   // warp-uniform
        bool d = false;
        patch_loop(a, k, &d);
        if (lane == 0) destroyed[k] = d ? 1 : 0;
    }
    __syncthreads();
    // 3. emptied patches are killed and regenerated in patch order (kill_resource)
    if (tid == 0) {
        for (int k = 0; k < a.np; ++k) {
            if (!destroyed[k]) continue;
            if (!a.p.regenerate_patches) {
                a.pt.id[k] = -1;
                continue;
            }
            if (!regenerate(a, k)) {
                a.pt.id[k] = -1;
                if (a.diag) atomicAdd(&a.diag[ABM_DIAG_CAPACITY], 1ull);
            }
        }
    }
    // 4. agents on no patch (sims.py:848-855), and the exploit flags of the social channel
    for (int i = tid; i < a.n; i += blockDim.x) {
        if (a.patch_of[i] < 0) {
            const int m = get_mode(a, i);
            if (pooling_done(a, i, m) || m == ABM_MODE_EXPLOIT) notify(a, i, -1, -1);
        }
        a.exploit[i] = a.ag.override_mode[i] == ABM_MODE_EXPLOIT ? 1 : 0;
    }
}

// Agent.prove_orientation (agent.py:605-610).
__device__ inline double prove_orientation(double t) {
    if (t < 0) t = 2 * M_PI + t;
    if (t > M_PI * 2) t = t - 2 * M_PI;
    return t;
}

constexpr int kUpdateWarps = 4;

// One warp per agent: the lanes count the social field's pixels (coalesced word loads), lane 0
// applies the update.
__global__ void __launch_bounds__(32 * kUpdateWarps) forage_update_kernel(ForageArgs a) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kUpdateWarps + (threadIdx.x >> 5);
    if (i >= a.n) return;   // warp-uniform
    const abm_forage_params &p = a.p;
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
    const double I_priv = p.F_N * (a.ag.novelty[i] ? 1.0 : 0.0) +
                          p.F_R * (a.ag.collected[i] - a.ag.collected_before[i]);
    if (a.ag.ipriv) a.ag.ipriv[i] = I_priv;
    // update_decision_processes (agent.py:194-210)
    double w = a.ag.w[i], u = a.ag.u[i];
    const double w_p = w > p.T_w ? w : 0.0;
    const double u_p = u > p.T_u ? u : 0.0;
    const double dw = p.Eps_w * ((double)total / rv) - p.g_w * (w - p.B_w) - u_p * p.S_uw;
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
    int ovr = a.ag.override_mode[i], mode = a.ag.mode[i];
    const double vel0 = (double)a.ag.v[i];
    double vel = 0.0, theta = 0.0;
    const int cur = ovr != ABM_MODE_NONE ? ovr : (w > p.T_w ? ABM_MODE_RELOCATE : ABM_MODE_EXPLORE);
    if (cur != ABM_MODE_COLLIDE) {
        const bool tw = w > p.T_w, tu = u > p.T_w;
        const bool on_patch = a.ag.env_status[i] == 1;
        int action;   // 0 random walk, 1 relocate, 2 exploit
        if (!tw && !tu) action = 0;
        else if (tw && tu) action = on_patch ? 2 : 1;
        else if (tw) action = 1;
        else action = on_patch ? 2 : 0;
        if (action == 0) {   // supcalc.random_walk(desired_vel=max_exp_vel)
            double r01;
            if (a.uniforms) {
                r01 = a.uniforms[i];
            } else {
                uint32_t wd[4];
                philox_draw(p.seed, (uint32_t)i, a.ag.draws[i], kTagWalk, wd);
                r01 = u01(wd[0], wd[1]);
                a.ag.draws[i] += 1;
            }
            vel = p.exp_vel_max;
            theta = p.exp_theta_min + (p.exp_theta_max - p.exp_theta_min) * r01;
            mode = ABM_MODE_EXPLORE;
            ovr = ABM_MODE_NONE;
        } else if (action == 1) {   // supcalc.F_reloc_LR(v, soc_v_field, max_exp_vel)
            const double le = (double)left / half, re = (double)(total - left) / (rv - half);
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
    double th = prove_orientation((double)a.ag.theta[i] + theta);
    double v = vel0 + vel;
    const int after = ovr != ABM_MODE_NONE ? ovr : (w > p.T_w ? ABM_MODE_RELOCATE : ABM_MODE_EXPLORE);
    if (after == ABM_MODE_EXPLORE && fabs(v) > 1.0) v = p.exp_vel_max;
    double sn, cs;
    sincos(th, &sn, &cs);
    double x = (double)a.ag.x[i] + v * cs;
    double y = (double)a.ag.y[i] - v * sn;
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
    a.ag.collected_before[i] = a.ag.collected[i];
    if (a.diag && !(isfinite(x) && isfinite(y) && isfinite(th) && isfinite(v) && isfinite(w) &&
                    isfinite(u)))
        atomicAdd(&a.diag[ABM_DIAG_NONFINITE], 1ull);
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
    forage_resource_kernel<<<1, kResourceThreads, 0, s>>>(a);
    if ((st = check_cuda(cudaGetLastError(), "forage_resource_kernel launch"))) return st;
    st = abm_vpf_social_fields(agents->x, agents->y, agents->theta, nullptr, p->agent_radius,
                               a.exploit, agents->patch_id, n, p->vision_range,
                               p->visual_exclusion, p->patchwise_exclusion, p->rv, p->fov0,
                               p->fov1, soc_bits_dev, diag_dev, stream);
    if (st < 0) return st;
    forage_update_kernel<<<(n + kUpdateWarps - 1) / kUpdateWarps, 32 * kUpdateWarps, 0, s>>>(a);
    return check_cuda(cudaGetLastError(), "forage_update_kernel launch");
}

}  // extern "C"
