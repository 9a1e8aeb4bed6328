/*
 * abm_forage.h -- C ABI of the collective-foraging step (libabm_vpf.so).
 *
 * One timestep of the reference's foraging simulation (abm/simulation/sims.py:734-858, the
 * Simulation.start loop body) for one arena on the GPU:
 *   0. when collide_agents is set, the agent-agent collisions (sims.py:735-784): agents whose
 *      integer pygame rects overlap (collide_circle, radius + 2) make the proximity manoeuvre
 *      of Simulation.agent_agent_collision_proximity (sims.py:421-474: the distance-weighted
 *      projection field of the agents within 2R + 20, a 0.2 rad turn away from the fuller
 *      half, a stop when the 200 pixels ahead are occupied) once per collision list that
 *      holds them (none in ghost mode for pairs with an exploiting agent), enter collide mode
 *      and, when among the collided agents, are notified with -1; agents no longer colliding
 *      leave collide mode;
 *   1. agent-resource interaction (sims.py:789-858): agents whose centre lies inside a patch
 *      are turned towards its centre (bias_agent_towards_res_center, sims.py:544-552), notified
 *      about it (notify_agent, sims.py:29-42; teleported to its centre when teleport_exploit)
 *      and, when exploiting, deplete it (Rescource.deplete, rescource.py:118-133) in agent
 *      order; a patch emptied this step notifies its agents and is regenerated at a random
 *      place (add_new_resource_patch, sims.py:332-374); agents on no patch are notified per
 *      sims.py:848-855;
 *   2. the social visual projection field of every agent (Agent.calc_social_V_proj,
 *      agent.py:396-419), as abm_vpf_social_fields;
 *   3. the agent update (Agent.update, agent.py:213-283): private information, the w/u
 *      decision processes (agent.py:194-210), the behavioural mode, random walk / left-right
 *      relocation / exploitation stop (supcalc.py:38-47, :81-92), prove_velocity, the move
 *      and the wall reflection (agent.py:347-394).
 * Agents are updated from one snapshot (Jacobi); the reference updates them one after another
 * in pygame group order, so long runs are compared by ensemble statistics.
 *
 * Conventions of include/abm_vpf.h apply (device pointers, stream order, status codes).
 */
#ifndef ABM_FORAGE_H
#define ABM_FORAGE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Behavioural modes (Agent.set_mode, agent.py:641-661). */
#define ABM_MODE_EXPLORE 0
#define ABM_MODE_RELOCATE 1
#define ABM_MODE_EXPLOIT 2
#define ABM_MODE_POOL 3
#define ABM_MODE_COLLIDE 4
#define ABM_MODE_NONE (-1) /* no overriding mode */

#define ABM_FORAGE_MAX_TAU 32
#define ABM_FORAGE_MAX_PATCHES 1024

typedef struct {
    /* decision processes (abm/contrib/decision_params.py) */
    double T_w, Eps_w, g_w, B_w, w_max;
    double T_u, Eps_u, g_u, B_u, u_max;
    double S_wu, S_uw, F_N, F_R;
    int32_t Tau; /* novelty memory length, 1..ABM_FORAGE_MAX_TAU */
    /* movement (abm/contrib/movement_params.py) */
    double exp_vel_max, exp_theta_min, exp_theta_max, reloc_theta_max, exp_stop_ratio;
    /* arena and agents (Simulation.__init__, sims.py:60-64) */
    double width, height, window_pad, agent_radius, consumption;
    int32_t pooling_time, teleport_exploit, regenerate_patches, allow_border_patch_overlap;
    /* patch regeneration: units uniform integer in [min, max), quality uniform in [min, max) */
    int32_t min_resc_units, max_resc_units;
    double min_resc_quality, max_resc_quality, patch_radius;
    /* social channel (Agent.calc_social_V_proj) */
    int32_t rv;
    double fov0, fov1, vision_range;
    int32_t visual_exclusion, patchwise_exclusion;
    /* random streams (Philox-4x32-10, keyed by seed; counters per agent / patch) */
    uint64_t seed;
    /* agent-agent collisions (AGENT_AGENT_COLLISION; needs an integer agent_radius) and ghost
     * mode (GHOST_WHILE_EXPLOIT: exploiting agents neither collide nor are collided with) */
    int32_t collide_agents, ghost_mode;
} abm_forage_params;

/* Agent state, n entries per array (device). */
typedef struct {
    float *x, *y, *theta, *v;              /* top-left position, orientation, speed */
    double *w, *u;                         /* decision variables */
    double *collected, *collected_before;  /* collected_r, collected_r_before */
    int32_t *mode;                         /* last set_mode value, ABM_MODE_* */
    int32_t *override_mode;                /* overriding_mode: ABM_MODE_NONE or ABM_MODE_* */
    int32_t *env_status, *env_status_before, *pool_success, *patch_id;
    uint32_t *novelty;                     /* bit k = novelty[k] of the reference's array */
    uint64_t *draws;                       /* random draws taken so far */
    double *ipriv;                         /* nullable: I_priv of the last update (recording) */
} abm_forager_state;

/* Resource patches, n_patches entries per array (device). */
typedef struct {
    double *x, *y;         /* top-left position; centre = position + radius */
    double *radius, *units, *left, *quality;
    int32_t *id;
    uint64_t *draws;       /* random draws taken by regenerations of this slot */
} abm_patch_state;

/*
 * Default parameters: decision_params.py / movement_params.py defaults and the foraging
 * workload's arena (1000 x 1000, pad 30, agent radius 10, 3 patches of radius 30 with 1000
 * units, consumption 1, pooling_time 0, teleport_exploit 1, regeneration on, Rv 1200, full
 * field of view, vision range 2000, visual exclusion on, patchwise exclusion on, collisions
 * off, ghost mode on).
 */
int abm_forage_params_default(abm_forage_params *p);

/*
 * One step (see the file comment).  soc_bits_dev: n * abm_vpf_words(rv) uint32 (device),
 * overwritten with the social fields of this step (stored order, as abm_vpf_social_fields).
 * scratch_dev: 2 * n int32 (device) of working space (contents ignored).  uniforms_dev
 * (nullable): n doubles in [0, 1), the random-walk draw of each agent for this step (replaces
 * the agent's Philox stream; for comparisons with an injected stream).  diag_dev (nullable):
 * as abm_vpf_flock_step, plus ABM_DIAG_CAPACITY when a regeneration found no free place in
 * 10000 tries (the reference raises; the patch then stays empty with id -1).
 */
int abm_forage_step(abm_forager_state *agents, int32_t n, abm_patch_state *patches,
                    int32_t n_patches, const abm_forage_params *p, uint32_t *soc_bits_dev,
                    int32_t *scratch_dev, const double *uniforms_dev,
                    unsigned long long *diag_dev, void *stream);

/*
 * Device-side recording of a run in the layout of the reference's RAM recorder
 * (ifdb.save_agent_data_RAM / save_resource_data_RAM, abm/monitoring/ifdb.py:55-96, :223-260):
 * agent-major series of `capacity` steps (agent i, step t at [i * capacity + t]).
 */
typedef struct {
    int32_t capacity;          /* steps the series hold; later steps are not recorded */
    int32_t *step;             /* device counter: the column of the next record */
    int32_t *posx, *posy;      /* int(position), truncated toward zero */
    float *orientation, *velocity;
    double *w, *u, *ipriv, *collected;
    int32_t *mode;             /* ifdb.mode_to_int: explore 0, exploit 1, relocate 2, collide 3 */
    int32_t *patch_id;         /* exploited_patch_id */
    uint32_t *soc_bits;        /* nullable: n x capacity x abm_vpf_words(rv) social fields */
    int32_t *res_posx, *res_posy;  /* n_patches x capacity: int(position) of the slot's patch */
    double *res_left, *res_quality;
    int32_t *res_id;           /* n_patches x capacity: the slot's patch id (-1: no patch) */
} abm_forage_recording;

/*
 * Append the current state of every agent and patch (and the social fields of the last step)
 * to the recording at column *rec->step, then advance the counter (one launch; graph-safe).
 * Call it after abm_forage_step, like the reference records after the agents' update.
 */
int abm_forage_record(const abm_forager_state *agents, int32_t n, const abm_patch_state *patches,
                      int32_t n_patches, const uint32_t *soc_bits_dev, int32_t rv,
                      abm_forage_recording *rec, void *stream);

/*
 * `steps` foraging steps in one call (the reference's Simulation.start loop for T steps), each
 * followed by abm_forage_record when rec is non-NULL: one step eagerly, then a CUDA graph of
 * graph_chunk steps (0: no graph) captured on `stream` and replayed, then the remaining steps
 * eagerly.  The random walk uses the agents' Philox streams (no injected uniforms).  Same
 * results as the same number of abm_forage_step (+ abm_forage_record) calls.  A NULL (legacy
 * default) stream cannot be captured: every step is then launched eagerly.  Call it outside
 * any stream capture of the caller's own.
 */
int abm_forage_run(abm_forager_state *agents, int32_t n, abm_patch_state *patches,
                   int32_t n_patches, const abm_forage_params *p, uint32_t *soc_bits_dev,
                   int32_t *scratch_dev, int32_t steps, int32_t graph_chunk,
                   abm_forage_recording *rec, unsigned long long *diag_dev, void *stream);

/* Philox-4x32-10 block for (counter, key): the generator of abm_forage_step, exported for
 * the tests (host function, no GPU needed). */
void abm_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif

#endif /* ABM_FORAGE_H */
