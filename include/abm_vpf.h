/*
 * abm_vpf.h -- C ABI of the GB300 visual-projection-field (VPF) + VSWRM flocking library.
 *
 * The library replaces the per-timestep perception and movement path of scioip34/ABM's
 * visual-flocking agents (reference version 1.2.0):
 *
 *   vf_supcalc.projection_field            abm/projects/visual_flocking/vf_agent/vf_supcalc.py:20-138
 *   vf_supcalc.VSWRM_flocking_state_variables          vf_supcalc.py:161-254 (dPhi_V_of :257-277)
 *   VFAgent.calc_soc_v_proj / perform_action / update_agent_position
 *                                           abm/projects/visual_flocking/vf_agent/vf_agent.py:216-327
 *   Agent.reflect_from_walls / VFAgent.teleport_infinite_arena
 *                                           abm/agent/agent.py:347-394, vf_agent.py:188-204
 *   Agent.calc_social_V_proj / projection_field (foraging social channel)
 *                                           abm/agent/agent.py:396-603
 *
 * Conventions
 *   - Every entry point returns an int status: ABM_OK (0), a positive warning, or a negative
 *     error; abm_last_error_string() describes the last non-zero status of the calling thread.
 *   - Array arguments named *_dev are CUDA device pointers; *_host are host pointers.  The
 *     caller owns all of them.  `stream` is a cudaStream_t passed as void* (NULL = legacy
 *     default stream).  Calls are stream-ordered and return without synchronising unless
 *     documented otherwise.
 *   - Agent state is structure-of-arrays float32: x, y are TOP-LEFT positions (the agent's
 *     centre is position + radius), theta in [0, 2 pi] with theta = 0 pointing right and
 *     screen y pointing down, v the scalar speed.  This is the reference's convention.
 *   - VPF bitmasks: words = ceil(Rv / 32) uint32 per agent; bit (k & 31) of word (k >> 5) is
 *     raw pixel k, i.e. the pixel order VSWRM integrates (np.flip of the reference's
 *     returned/stored soc_v_field).  Bits >= Rv are zero.
 *   - The library allocates device memory only for its cached lookup tables (one set per
 *     distinct grid: Rv and field of view) and for a per-stream workspace of about 32 + Rv/8
 *     bytes per agent (the VSWRM sums and the VPF bitmasks handed between the step's kernels); the
 *     first call for a grid, and a call with more agents than the stream's workspace holds,
 *     allocate synchronously, so make such a call before capturing a CUDA graph.  A graph
 *     captured from a stream uses that stream's workspace: do not replay it concurrently with
 *     other calls on the same stream.
 *   - The library's kernels are programmatic dependent launches: each waits for the completion
 *     of the previous work on the stream (griddepcontrol.wait) before it touches memory, and
 *     lets the next kernel be scheduled early.  Ordinary launches of the caller keep plain
 *     stream order; a kernel that the caller itself launches with programmatic stream
 *     serialisation right after a library call must call cudaGridDependencySynchronize()
 *     before it reads the library's results.
 */
#ifndef ABM_VPF_H
#define ABM_VPF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ABM_VPF_ABI_VERSION 1

/* status codes */
#define ABM_OK 0
#define ABM_WARN_PHI_MISMATCH 1      /* len(np.arange(-pi, pi, 2pi/Rv)) != Rv: the reference
                                        skips the VSWRM update (dv = dpsi = 0) with a printed
                                        warning, vf_agent.py:268, :283-284 */
#define ABM_ERR_INVALID_ARG (-1)
#define ABM_ERR_RV (-2)              /* Rv outside [2, ABM_MAX_RV] */
#define ABM_ERR_CUDA (-3)
#define ABM_ERR_TIMEOUT (-4)         /* a bounded device-side wait gave up */
#define ABM_ERR_NONFINITE (-5)       /* NaN / inf in the agent state */
#define ABM_ERR_UNSUPPORTED (-6)
#define ABM_ERR_NO_DEVICE (-7)

#define ABM_MAX_RV 16384

/* boundary conditions (vf_params.BOUNDARY) */
#define ABM_BOUNDARY_WALLS 0
#define ABM_BOUNDARY_INFINITE 1

/*
 * Simulation parameters of one swarm (vf_params.py:12-23 plus the simulation geometry of
 * abm/simulation/sims.py:60-161).  alp2/bet2 multiply a time derivative that the reference
 * fixes at zero (vf_supcalc.py:199) and are accepted for completeness only.  dt scales the
 * heading, speed and position increments; dt = 1 is the reference (it has no dt).
 */
typedef struct abm_vf_params {
    double gam, v0, alp0, alp1, alp2, bet0, bet1, bet2;
    int32_t boundary;        /* ABM_BOUNDARY_WALLS / ABM_BOUNDARY_INFINITE */
    int32_t limit_movement;  /* VF_LIMIT_MOVEMENT */
    double max_vel, max_th;  /* VF_MAX_VEL, VF_MAX_TH */
    double width, height;    /* arena size (ENV_WIDTH, ENV_HEIGHT) */
    double window_pad;       /* walls at [pad, pad + width] x [pad, pad + height] */
    double fov0, fov1;       /* field of view in radians, e.g. (-pi, pi) */
    int32_t rv;              /* VPF resolution in pixels (after any FOV rescale) */
    int32_t reserved0;
    double radius;           /* agent radius when no per-agent radii are given */
    double dt;               /* 1.0 = reference */
} abm_vf_params;

/* Device SoA state of n agents (float32, each array n long). */
typedef struct abm_swarm_state {
    float *x, *y, *theta, *v;
} abm_swarm_state;

/* The same state in double precision (used by the FP64 mode of the edge form). */
typedef struct abm_swarm_state_f64 {
    double *x, *y, *theta, *v;
} abm_swarm_state_f64;

/* Optional per-agent device arrays (any may be NULL): radius (object_sizes / agent radius),
 * and the VFAgent.ALP0 / BET0 / V0 heterogeneity overrides (vf_agent.py:24-26). */
typedef struct abm_agent_overrides {
    const float *radius, *alp0, *bet0, *v0;
} abm_agent_overrides;

/* Diagnostics counters (device uint64 array of ABM_DIAG_COUNT, accumulated, never reset by
 * the library). */
#define ABM_DIAG_PAIRS_RESOLVED 0    /* pairs whose FP32 decision fell in the guard band and
                                        were decided again in double-float */
#define ABM_DIAG_NEAR_BOUNDARY 1     /* of those, pairs whose edge angle lies within 1e-9 rad
                                        of a pixel / width boundary (reported, not excused) */
#define ABM_DIAG_NONFINITE 2         /* agents whose state was NaN / inf */
#define ABM_DIAG_TIMEOUTS 3          /* bounded waits that gave up */
#define ABM_DIAG_CAPACITY 4          /* social fields left empty: more obstacles in range than
                                        the kernel's per-agent capacity (4096) */
#define ABM_DIAG_COLLIDE_FP64 5      /* foraging collisions: proximity-field bearings whose FP32
                                        angle lay within 4e-6 rad of a decision boundary and
                                        were taken on the reference's FP64 route */
#define ABM_DIAG_COLLIDE_REPLAYS 6   /* foraging collisions: manoeuvres whose half / front
                                        comparison lay within numpy's rounding and was decided
                                        by replaying numpy's pairwise sums */
#define ABM_DIAG_COUNT 8

/* ---------------------------------------------------------------- utilities */

int abm_vpf_abi_version(void);
const char *abm_last_error_string(void);

/* Reference defaults (vf_params.py:12-23 with the keys unset, sims.py:60-65): GAM 0.1,
 * V0 1, ALP0 1, ALP1 0.09, BET0 1, BET1 0.09, walls, no limit, MAX_VEL 3, MAX_TH 0.1,
 * width 600, height 480, pad 30, FOV (-pi, pi), Rv 800, radius 10, dt 1. */
int abm_vf_params_default(abm_vf_params *p);

/* np.arange(-pi, pi, 2*pi/rv) exactly as numpy builds it (VFAgent.PHI, vf_agent.py:44).
 * Writes min(length, cap) values to phi_host and returns the length (which is rv + 1 for
 * the Rv values that trigger the reference's mismatch warning), or a negative error. */
int abm_phi_table(int32_t rv, double *phi_host, int32_t cap);

/* Number of uint32 words of one VPF bitmask: ceil(rv / 32). */
int abm_vpf_words(int32_t rv);

/* ---------------------------------------------------------------- hot path */

/*
 * One snapshot (Jacobi) step of a whole swarm: for every agent, the VPF of all other agents
 * (projection_field + calc_soc_v_proj, vf_supcalc.py:20-138 / vf_agent.py:216-237), the VSWRM
 * integrals (vf_supcalc.py:161-277), the heading/speed/position update and the boundary rule
 * (vf_agent.py:289-327, agent.py:347-394, vf_agent.py:188-204).  Replaces the per-agent loop
 * of VFAgent.update (vf_agent.py:52-77) driven by VFSimulation.step_sim (vf_sims.py:291-340);
 * the reference updates agents in place in pygame group order, this call reads `in` and
 * writes `out` (which must not alias `in`).
 *
 * vpf_bits_dev (nullable): n * abm_vpf_words(rv) uint32, the binarised VPF of each agent.
 * terms_dev (nullable): n * 6 doubles {dvel, dpsi, alpha_blob, alpha_edge, beta_blob,
 *   beta_edge} = VSWRM_flocking_state_variables(verbose=True) (vf_supcalc.py:241-254).
 * diag_dev (nullable): ABM_DIAG_COUNT uint64 counters.
 * Returns ABM_WARN_PHI_MISMATCH (after launching) when the reference would skip VSWRM.
 */
int abm_vpf_flock_step(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                       const abm_vf_params *p, const abm_agent_overrides *ov,
                       uint32_t *vpf_bits_dev, double *terms_dev,
                       unsigned long long *diag_dev, void *stream);

/*
 * Batched sweep: one snapshot step of many independent swarms (instances) in one pair launch
 * and one update launch.  The reference runs such sweeps as one simulation per generated .env
 * file, sequentially or as separate processes (metarunner.py:168-254,
 * HPC_run_all_exp_distribute.sh); here the instances' agents are concatenated in one SoA state
 * of n_total agents and agent i sees exactly the agents [seg_begin[i], seg_end[i]) of its own
 * instance (which contain i).  Per-instance ALP0 / BET0 / V0 / radius go in the per-agent
 * override arrays.  order_dev (nullable): a permutation of [0, n_total) giving the order in which
 * agents are scheduled (put the largest instances first for load balance).  All instances share
 * p (Rv, arena, boundary, GAM, ALP1, BET1 ...).  Results per instance are bit-identical to
 * abm_vpf_flock_step on that instance alone.  Uses the group form of the pair kernel (groups
 * of 8 consecutive entries of the order) where it applies (equal radii; walls, or a torus whose
 * width and height are exact in float32) and the L1 form otherwise, unless
 * abm_vpf_set_step_mode selects one.
 */
int abm_vpf_flock_batched(const abm_swarm_state *in, abm_swarm_state *out, int32_t n_total,
                          const int32_t *seg_begin_dev, const int32_t *seg_end_dev,
                          const int32_t *order_dev, const abm_vf_params *p,
                          const abm_agent_overrides *ov, uint32_t *vpf_bits_dev,
                          double *terms_dev, unsigned long long *diag_dev, void *stream);

/*
 * Many steps in one call (the reference's simulation loop over VFSimulation.step_sim,
 * vf_sims.py:291-340, for `steps` timesteps; for a sweep, its per-configuration runs of
 * metarunner.py:240-254 for all configurations at once): the state ping-pongs between a and b,
 * starting from a; after an even number of steps the result is in a, after an odd number in b.
 * The library runs one step eagerly, then replays a CUDA graph of graph_chunk steps (rounded
 * down to an even number; 0 or 1: no graph) captured on `stream`, then the remaining steps
 * eagerly.  Results are those of the same number of abm_vpf_flock_step / _batched calls.  A
 * NULL (legacy default) stream cannot be captured: every step is then launched eagerly.  Call
 * it outside any stream capture of the caller's own.  Status: the first step's (0 or
 * ABM_WARN_PHI_MISMATCH) or an error.
 */
int abm_vpf_flock_run(abm_swarm_state *a, abm_swarm_state *b, int32_t n, const abm_vf_params *p,
                      const abm_agent_overrides *ov, int32_t steps, int32_t graph_chunk,
                      unsigned long long *diag_dev, void *stream);
int abm_vpf_flock_batched_run(abm_swarm_state *a, abm_swarm_state *b, int32_t n_total,
                              const int32_t *seg_begin_dev, const int32_t *seg_end_dev,
                              const int32_t *order_dev, const abm_vf_params *p,
                              const abm_agent_overrides *ov, int32_t steps, int32_t graph_chunk,
                              unsigned long long *diag_dev, void *stream);

/*
 * abm_vpf_flock_step on HOST state (no counterpart in the reference; the call a host-side
 * loop makes once per step): in_host / out_host hold host pointers (x, y, theta, v).  For
 * memory registered with CUDA (page-locked, e.g. cudaHostAlloc or torch pin_memory, or
 * managed), one kernel gathers the input into a per-stream device staging buffer and the
 * step's last kernel writes the new state straight into out_host; other (pageable) memory is
 * copied with cudaMemcpyAsync through the same staging buffer.  Stream-ordered: the
 * caller synchronises the stream before reading out_host.  ov (nullable) holds DEVICE arrays as
 * for abm_vpf_flock_step.  Same status codes.
 */
int abm_vpf_flock_step_host(const abm_swarm_state *in_host, abm_swarm_state *out_host,
                            int32_t n, const abm_vf_params *p, const abm_agent_overrides *ov,
                            void *stream);

/*
 * On-device ensemble statistic (no counterpart in the reference's step; the reference computes
 * it afterwards from recorded orientations, DataLoader.calculate_polarization,
 * abm/loader/data_loader.py:1761-1836): the polarisation |sum_i (cos theta_i, sin theta_i)| / N
 * of every instance of the current state, written to out_dev[k * capacity + step_dev[k]], after
 * which step_dev[k] advances (steps beyond capacity are dropped).  offsets_dev: n_instances + 1
 * int32 agent offsets of the instances (device; NULL: one instance of n_total agents).  One
 * launch, graph-safe (the per-instance column counters live on the device).
 */
int abm_vpf_polarisation(const float *theta_dev, int32_t n_total, const int32_t *offsets_dev,
                         int32_t n_instances, double *out_dev, int32_t capacity,
                         int32_t *step_dev, void *stream);

/*
 * Device-side recording of a visual-flocking run: the per-step values the reference's RAM
 * recorder keeps for each agent (ifdb.save_agent_data_RAM, abm/monitoring/ifdb.py:55-96, called
 * after every step by VFSimulation.step_sim, vf_sims.py:328-331): int() of the top-left
 * position, orientation, velocity and, optionally, the step's VPF whose rising / falling edges
 * the reference stores.  The series are agent-major, (n, capacity) and (n, capacity, words).
 */
typedef struct abm_vf_recording {
    int32_t capacity;          /* steps the series hold; later steps are not recorded */
    int32_t *step;             /* device, two int32: [0] the column of the next record,
                                  [1] launch scratch (zero it together with [0]) */
    int32_t *posx, *posy;      /* int() of x and y: truncation toward zero */
    float *orientation, *velocity;
    uint32_t *vpf_bits;        /* nullable: the bitmask abm_vpf_flock_step wrote for the step
                                  (raw pixel order; the reference's soc_v_field is its flip) */
} abm_vf_recording;

/*
 * Append the state s (and vpf_bits_dev when rec->vpf_bits is set; rv gives its words) to the
 * recording at column rec->step[0], then advance the counter (one launch; graph-safe).  Call it
 * after the step, like the reference records after the agents' update.  For a batched sweep
 * pass the concatenated state: rows follow the agents of the instances in order.
 */
int abm_vpf_record(const abm_swarm_state *s, int32_t n_total, const uint32_t *vpf_bits_dev,
                   int32_t rv, abm_vf_recording *rec, void *stream);

/*
 * abm_vpf_flock_run with the recording of every step (VFSimulation.step_sim with save_in_ram,
 * vf_sims.py:291-331, for `steps` timesteps): each step is abm_vpf_flock_step followed by
 * abm_vpf_record, both inside the library's graph.  vpf_bits_dev: an (n, words) device buffer
 * for the step's VPF, needed when rec->vpf_bits is set (NULL otherwise).  Same state
 * ping-pong, status and stream rules as abm_vpf_flock_run; results and records equal those of
 * the same number of step + record calls.
 */
int abm_vpf_flock_run_recorded(abm_swarm_state *a, abm_swarm_state *b, int32_t n,
                               const abm_vf_params *p, const abm_agent_overrides *ov,
                               int32_t steps, int32_t graph_chunk, uint32_t *vpf_bits_dev,
                               abm_vf_recording *rec, unsigned long long *diag_dev,
                               void *stream);

/*
 * Allocation-free variant of abm_vpf_flock_step (no counterpart in the reference): the same
 * step, arguments, results and status codes, for callers that cannot call cudaMalloc, such as
 * code running inside another framework's memory pool (an allocation outside the pool breaks
 * its accounting) or a process that has reserved all device memory up front.  Its scratch (the
 * per-agent VSWRM sums between the two launches, the lookup tables of one grid and the
 * double-float sincos table) lives in a file-scope device array of about 2.5 MiB that every GPU
 * loading the library holds until the process exits; no cudaMalloc, cudaFree or other
 * allocating routine is called.  Up to 16384 agents it runs the group pair kernel without
 * neighbour chunks (equal radii; walls, or a torus whose width and height are exact in
 * float32) or the one-block-per-agent one, above that the tiled one (none of them needs the
 * bitmask workspace of the split form).
 * Limits: n <= ABM_NOALLOC_MAX_AGENTS and rv <= ABM_NOALLOC_MAX_RV, larger values return
 * ABM_ERR_INVALID_ARG / ABM_ERR_RV with a message.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and copies the sincos table into it, and a call
 * with a different rv or field of view copies that grid's tables into it (from pageable host
 * memory), overwriting the tables that earlier calls used; make the first call, and the first
 * call for each grid, before any stream capture (such a call made during capture returns
 * ABM_ERR_INVALID_ARG).  Every call shares the one array and it keeps the last call's contents
 * (nothing in it needs to start at zero: each launch overwrites the sums it reads); calls that
 * overlap on the GPU race on it, so serialise them.  Host threads are serialised per device.
 */
#define ABM_NOALLOC_MAX_AGENTS 65536
#define ABM_NOALLOC_MAX_RV 8192
int abm_vpf_flock_step_noalloc(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                               const abm_vf_params *p, const abm_agent_overrides *ov,
                               uint32_t *vpf_bits_dev, double *terms_dev,
                               unsigned long long *diag_dev, void *stream);

/*
 * Drop-in twin of vf_supcalc.projection_field (vf_supcalc.py:20-138): the dense per-object
 * rows of one focal agent, flipped like the reference's return value.
 * pos_host: focal top-left (x, y) in double; obj_xy_dev: n_obj * 2 doubles (device);
 * obj_sizes_dev: n_obj doubles or NULL (use radius); vision_range < 0 means None.
 * rows_dev: n_obj * rv doubles (device), overwritten with 0/1.
 */
int abm_vpf_project_rows(const double fov[2], int32_t rv, const double pos_host[2],
                         double radius, double orientation, int32_t n_obj,
                         const double *obj_xy_dev, const double *obj_sizes_dev,
                         int32_t boundary, double width, double height, double vision_range,
                         double *rows_dev, unsigned long long *diag_dev, void *stream);

/*
 * Drop-in twin of VSWRM_flocking_state_variables(verbose=True) (vf_supcalc.py:161-254) for a
 * batch of binary fields given as bitmasks in raw pixel order.  phi_host: the rv values of
 * the integration grid Phi (any strictly increasing grid; the reference passes
 * np.arange(-pi, pi, 2pi/rv)).  vel_dev: n_fields floats.  prm: {GAM, V0, ALP0, ALP1, ALP2,
 * BET0, BET1, BET2}; alp0/bet0/v0_dev optional per-field overrides (NULL = use prm).
 * out_dev: n_fields * 6 doubles.
 */
int abm_vswrm_integrals(int32_t n_fields, int32_t rv, const uint32_t *bits_dev,
                        const double *phi_host, const float *vel_dev, const double prm[8],
                        const float *alp0_dev, const float *bet0_dev, const float *v0_dev,
                        double *out_dev, void *stream);

/*
 * Foraging social channel (Agent.calc_social_V_proj, abm/agent/agent.py:396-419, with
 * Agent.projection_field :457-597 and exlude_V_source_data :421-445): for every agent i, the
 * projection of the exploiting agents within vision_range (social cues: exploit[j] != 0,
 * j != i, patch[j] != -1 and, when patchwise, patch[j] != patch[i]), where every other agent in
 * range occludes them through the reference's distance-ordered interval trimming when
 * visual_exclusion != 0.  Obstacle centres use the focal radius (agent.py:504-505); the range
 * filter uses each agent's own radius (supcalc.py:73-78).  radius_dev may be NULL (all agents
 * have `radius`).  out_bits_dev: n * abm_vpf_words(rv) uint32 in the reference's STORED order
 * of soc_v_field (flipped, and zero where phis < fov0 or phis > fov1).  Requires
 * -pi <= fov0 < fov1 <= pi; at most 4096 obstacles per agent (more: that field is left empty
 * and ABM_DIAG_CAPACITY counts it).
 */
int abm_vpf_social_fields(const float *x_dev, const float *y_dev, const float *theta_dev,
                          const float *radius_dev, double radius, const int32_t *exploit_dev,
                          const int32_t *patch_dev, int32_t n, double vision_range,
                          int32_t visual_exclusion, int32_t patchwise, int32_t rv, double fov0,
                          double fov1, uint32_t *out_bits_dev, unsigned long long *diag_dev,
                          void *stream);

/*
 * Continuum edge form (differentiable; no counterpart in the reference, which only has the
 * pixel form): neighbour j covers the retina arc [b_j - a_j, b_j + a_j] (b_j the closed angle
 * of vf_supcalc.py:142-158, a_j = atan(R/d_j) like vf_supcalc.py:96-99, or asin(R/d_j) when
 * use_asin != 0); with the merged arcs [l, u] of the union the VSWRM integrals are
 * blob_c = -sum(sin u - sin l), blob_s = sum(cos u - cos l), edge_c = sum(cos l + cos u),
 * edge_s = sum(sin l + sin u) (the Rv -> infinity limit of vf_supcalc.py:233-238), and the
 * update is the reference's with increments scaled by p->dt (walls only).  Float32, n <= 2048.
 * abm_vpf_edge_fwd: one step in -> out; terms_dev (nullable) n x 4 floats
 *   {blob_c, blob_s, edge_c, edge_s}.
 * abm_vpf_edge_bwd: the adjoint of that step: given grad_out = d loss / d out, OVERWRITES
 *   grad_in with d loss / d in and ADDS d loss / d (alp0, alp1, bet0, bet1, v0) to the five
 *   doubles of grad_params_dev.  The arc structure is recomputed from `in`.
 * The _f64 variants run the same kernels in double precision.  The edge form is piecewise
 * smooth: merges and splits of arcs are events where the edge terms jump, and over long
 * horizons float32 rounding changes which events happen (a float32 rollout of 256 agents x 200
 * steps at dt = 0.1 drifts by pixels from its FP64 twin), so gradients that must match an FP64
 * reference over such horizons need the _f64 variants.
 */
int abm_vpf_edge_fwd(const abm_swarm_state *in, abm_swarm_state *out, int32_t n,
                     const abm_vf_params *p, int32_t use_asin, float *terms_dev, void *stream);
int abm_vpf_edge_bwd(const abm_swarm_state *in, const abm_swarm_state *grad_out,
                     abm_swarm_state *grad_in, double *grad_params_dev, int32_t n,
                     const abm_vf_params *p, int32_t use_asin, void *stream);
int abm_vpf_edge_fwd_f64(const abm_swarm_state_f64 *in, abm_swarm_state_f64 *out, int32_t n,
                         const abm_vf_params *p, int32_t use_asin, double *terms_dev,
                         void *stream);
int abm_vpf_edge_bwd_f64(const abm_swarm_state_f64 *in, const abm_swarm_state_f64 *grad_out,
                         abm_swarm_state_f64 *grad_in, double *grad_params_dev, int32_t n,
                         const abm_vf_params *p, int32_t use_asin, void *stream);

/* ---------------------------------------------------------------- launch configuration */

/* Warps (focal agents) per block and neighbour-tile length of abm_vpf_flock_step.  0 keeps
 * the current value.  warps_per_block in {1,2,4,8,16,32}; tile in [32, 8192], multiple of 32. */
int abm_vpf_set_step_config(int32_t warps_per_block, int32_t tile);
int abm_vpf_get_step_config(int32_t *warps_per_block, int32_t *tile);

/* Form of the pair kernel of abm_vpf_flock_step: mode 0 = automatic (up to 16384 agents the
 * group form where it applies, else the L1 form; the tiled form beyond), 1 = L1 form (one
 * block per focal agent, neighbours read through the read-only L1 path), 2 = tiled form
 * (warps_per_block focal agents share TMA-staged neighbour tiles), 3 = group form (one warp
 * per group of 4 consecutive focal agents, 8 in a batched sweep, each neighbour read once for
 * the group; equal radii, and on the infinite (torus) arena a width and height exact in
 * float32; otherwise the step returns ABM_ERR_UNSUPPORTED).
 * warps_per_agent in {1, 2, 4} splits one focal agent's neighbours over that many warps in the
 * L1 form; 0 keeps the current value.  All forms give bit-identical results. */
int abm_vpf_set_step_mode(int32_t mode, int32_t warps_per_agent);
int abm_vpf_get_step_mode(int32_t *mode, int32_t *warps_per_agent);

/* Neighbour chunks per focal agent in the L1 and group forms of abm_vpf_flock_step (not the
 * batched or no-alloc calls): with chunks > 1 each agent's neighbours are split over that many
 * blocks,
 * whose partial bitmasks are OR-ed into a per-agent bitmask in the stream's workspace (Rv/8
 * bytes per agent) and reduced by a second kernel, so that the block scheduler can balance the
 * SMs' work when the swarm alone does not fill the GPU several times over.  0 (the default) =
 * automatic (in the group form, when the chunks make more than one wave of resident blocks,
 * the chunks of all groups are dispatched round by round with decreasing lengths, so that the
 * last blocks are the shortest); otherwise 1, 2, 4, 8 or 16 equal chunks.  All values give
 * bit-identical results. */
int abm_vpf_set_step_split(int32_t chunks);
int abm_vpf_get_step_split(int32_t *chunks);

/* One launch configuration of the step and its measured time. */
typedef struct {
    int32_t mode;              /* 1 = L1 form, 2 = tiled form, 3 = group form */
    int32_t warps_per_agent;   /* L1 form: warps sharing one focal agent (1, 2, 4) */
    int32_t chunks;            /* L1 / group form, single swarm: neighbour chunks (1..16) */
    int32_t warps_per_block;   /* tiled form: focal agents per block */
    int32_t tile;              /* tiled form: neighbour tile length */
    float ms_per_step;         /* mean device time of one step; < 0 if the form was refused */
} abm_step_config;

/*
 * Autotuner (no counterpart in the reference): times the step on the caller's own state and
 * stream under every candidate configuration and applies the fastest one through
 * abm_vpf_set_step_mode / _config / _split.  Candidates for a single swarm (seg_begin_dev ==
 * NULL): the group form with automatic chunks (chunks = 0) and with chunks in {1, 2, 4, 8, 16}
 * (refused where it does not apply), the
 * L1 form with warps_per_agent in {1, 2, 4} x chunks in {1, 2, 4, 8, 16}, and the tiled form
 * with warps_per_block in {4, 8, 16} x tile in {1024, 2048, 4096, 8192}; for a
 * batched sweep (segment arrays as for abm_vpf_flock_batched): the group form and the L1 form
 * with warps_per_agent in {1, 2, 4}.  Each candidate runs one untimed step and then `reps` timed
 * steps (CUDA events on `stream`) from `in` into a scratch state allocated by the call.  All
 * configurations give bit-identical results, so tuning changes only the speed.  Synchronises
 * the stream; must not be called during stream capture.  best: the chosen configuration;
 * tried (nullable, room for max_tried entries) and *n_tried (nullable): every candidate.
 */
int abm_vpf_autotune(const abm_swarm_state *in, int32_t n, const int32_t *seg_begin_dev,
                     const int32_t *seg_end_dev, const int32_t *order_dev,
                     const abm_vf_params *p, const abm_agent_overrides *ov, int32_t reps,
                     abm_step_config *best, abm_step_config *tried, int32_t max_tried,
                     int32_t *n_tried, void *stream);

/*
 * Status of the step kernels' bounded waits (no counterpart in the reference, which has no
 * device waits; the nearest analogue is its status-and-skip of vf_agent.py:268, :283-284).
 * The tiled pair kernel waits for each neighbour tile that the TMA bulk engine stages, at most
 * 2^20 polls; a block whose wait gives up waits (bounded) for its own copies still in flight,
 * writes no results, counts the event in ABM_DIAG_TIMEOUTS and sets a device status flag.
 * The step entry points return once their kernels are launched, so such a failure is
 * asynchronous, like CUDA's own kernel errors: abm_vpf_status synchronises `stream`, then
 * returns ABM_ERR_TIMEOUT if any step kernel on the current device gave up a wait since the
 * flag was last cleared (clear != 0 clears it), else ABM_OK.  The launch that gave up left
 * incomplete results.  No allocation.
 */
int abm_vpf_status(int32_t clear, void *stream);

/* Test hook of the bounded wait (no counterpart in the reference): one block arms an mbarrier
 * for 16 bytes that no copy will deliver (no bulk copy is issued) and waits at most `polls`
 * (1 .. 2^20) try_wait rounds; result_dev[0] = 1 if the phase completed, 0 if the wait gave
 * up.  A give-up is counted in diag_dev[ABM_DIAG_TIMEOUTS] (nullable) and sets the status that
 * abm_vpf_status reports, exactly as in the tiled pair kernel. */
int abm_vpf_debug_wait_timeout(int32_t polls, unsigned long long *diag_dev, int32_t *result_dev,
                               void *stream);

/* Verification hook (no counterpart in the reference): evaluates the double-float cos/sin of
 * float32 headings that the pair kernels use for the focal agent's heading vector.
 * out_dev: n x 2 doubles (cos, sin). */
int abm_vpf_check_sincos(const float *theta_dev, int32_t n, double *out_dev, void *stream);

/* ---------------------------------------------------------------- measurement utilities */

/* Pipe-throughput probe (no counterpart in the reference; used for the roofline
 * denominators): kind 0 launches independent FFMA chains, kind 1 independent MUFU.RSQ chains,
 * kind 2 independent packed FP32x2 FFMA2 chains, on blocks x threads threads for `iters`
 * rounds.  *ops_out receives the number of FP32 ops
 * (an FFMA counts 2) or MUFU ops the launch performs; time it with CUDA events on `stream`.
 * sink_dev: >= threads floats of scratch that keeps the chains live. */
int abm_probe_pipe_peak(int32_t kind, int32_t blocks, int32_t threads, int32_t iters,
                        float *sink_dev, double *ops_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ABM_VPF_H */
