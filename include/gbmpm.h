/*
 * gbmpm.h - C ABI of the GB300 MLS/APIC material-point engine.
 *
 * One explicit MLS/APIC substep (quadratic B-spline G2P, return mapping and
 * Kirchhoff stress, P2G, grid update with collider boundary conditions) runs as
 * hand-written sm_103a CUDA kernels behind these entry points. Every pointer in
 * gbmpm_particles / gbmpm_grid is a device pointer owned by the caller (the
 * Python host layer keeps them in PyTorch CUDA tensors and passes data_ptr()).
 * No entry point takes a torch type; all take plain pointers, sizes and a
 * cudaStream_t passed as void*.
 *
 * Reference interface replaced (warpmpm, Python over NVIDIA Warp):
 *   gbmpm_engine_create/destroy   MPM_Simulator_WARP.__init__/initialize
 *                                 (src/warpmpm/kernels/mpm_solver_warp.py:213-504)
 *   gbmpm_bind                    load_initial_data_from_torch + the state struct
 *                                 (mpm_solver_warp.py:565-621, kernels/warp_utils.py:23-157)
 *   gbmpm_set_model               set_parameters_dict / finalize_mu_lam
 *                                 (mpm_solver_warp.py:634-805)
 *   gbmpm_set_colliders           add_surface_collider, set_velocity_on_cuboid,
 *                                 add_revolved_sdf_collider, add_bounding_box,
 *                                 add_sdf_collider and their pose setters
 *                                 (mpm_solver_warp.py:1880-2285, 2287-2380, 2621-2814)
 *   gbmpm_get_colliders           reading back integrated poses (param.point/rot/quat)
 *   gbmpm_tick                    p2g2p_fused_tick / p2g2p (mpm_solver_warp.py:1092-1546)
 *   gbmpm_guard                   Solver._update_grid_box edge guard (core/solver.py:485-518)
 *   gbmpm_wrench / _reset_wrench  cup_wrench, sdf_wrench, tool_force and their resets
 *                                 (core/solver.py:295-313, 348-361, 415-427)
 *   gbmpm_sort_particles          Solver._sort_particles + permute_particles
 *                                 (core/solver.py:454-467, mpm_solver_warp.py:1548-1619)
 *   gbmpm_rebuild_active_blocks   rebuild_active_blocks (mpm_solver_warp.py:989-1026)
 *   gbmpm_compute_R / _cov        compute_R_from_F / compute_cov_from_F
 *                                 (kernels/mpm_utils.py:1234-1285)
 *   gbmpm_profile                 Solver.profile_report timings (core/solver.py:469-483)
 *
 * Return value of every int entry point: GBMPM_OK (0) or a gbmpm_status code;
 * gbmpm_last_error() gives a one-line message for the calling thread.
 */
#ifndef GBMPM_H
#define GBMPM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBMPM_MAX_MATERIALS 16
#define GBMPM_MAX_COLLIDERS 32
#define GBMPM_MAX_SUBSTEPS 8192

typedef enum {
    GBMPM_OK = 0,
    GBMPM_ERR_ARG = 1,          /* bad argument (the Python layer raises ValueError) */
    GBMPM_ERR_CUDA = 2,         /* CUDA runtime error (RuntimeError) */
    GBMPM_ERR_STATE = 3,        /* called before gbmpm_bind / gbmpm_set_model */
    GBMPM_ERR_BOUNDS = 4,       /* a kernel bounds check tripped (RuntimeError) */
    GBMPM_ERR_UNSUPPORTED = 5   /* feature not built (NotImplementedError) */
} gbmpm_status;

/* Device status word bits, set by kernels, read with gbmpm_guard. */
#define GBMPM_FLAG_STENCIL_OOB   1u   /* a particle's 3x3x3 stencil left the grid: access skipped */
#define GBMPM_FLAG_NONFINITE     2u   /* a non-finite particle position was seen */
#define GBMPM_FLAG_LIST_OVERFLOW 4u   /* the active-block list overflowed (cannot happen by size) */

/* Material ids, pinned by the reference (mpm_solver_warp.py:14-19). */
enum {
    GBMPM_MAT_JELLY = 0, GBMPM_MAT_METAL = 1, GBMPM_MAT_SAND = 2, GBMPM_MAT_PLASTICINE = 5,
    GBMPM_MAT_FLUID = 6, GBMPM_MAT_STATIONARY = 7, GBMPM_MAT_RIGID = 8, GBMPM_MAT_MU_I = 9,
    GBMPM_MAT_NEWTONIAN = 10, GBMPM_MAT_MU_I_PHI = 11, GBMPM_MAT_TAB_VISCOUS = 12,
    GBMPM_MAT_TAB_MU_I = 13
};

/* Particle state, reference layout (warp_utils.py:88-135): vec3 = 3 floats,
 * mat33 = 9 floats row-major, one record per particle, contiguous. */
typedef struct {
    int32_t n;
    float *x, *v;                       /* [n][3] */
    float *C, *F, *F_trial, *L, *stress; /* [n][9] */
    float *mass, *vol, *density, *Jp;   /* [n] */
    float *mu, *lam, *yield_stress;     /* [n] per-particle model arrays (mpm_solver_warp.py:277-279) */
    int32_t *material, *selection;      /* [n] */
    float *cov, *init_cov;              /* [n][6] upper triangle xx,xy,xz,yy,yz,zz, or NULL */
    int32_t *cdf_tag;                   /* [n] persisted CPIC side bits (warp_utils.py:124-129), or NULL */
    int32_t *rigid_id;                  /* [n] body of a material-8 particle (mpm_solver_warp.py:366-371), or NULL */
    float *x_ref;                       /* [n][3] body-frame position of a rigid particle, or NULL */
    int32_t *mod_mask;                  /* [n] bit m set: particle modifier m acts on the particle, or NULL */
} gbmpm_particles;

/* Dense n^3 grid, index ((ix*n)+iy)*n+iz (Warp 3-D array order).
 * mv: scatter target, per node {m*vx, m*vy, m*vz, m}; all zero between substeps.
 * v : grid velocity after the update and boundary conditions, {vx, vy, vz, 0}.  */
typedef struct {
    int32_t n_grid;
    float *mv;                          /* [n^3][4] */
    float *v;                           /* [n^3][4] */
} gbmpm_grid;

/* Model: scalars plus per-material-type tables (MPMModelStruct, warp_utils.py:23-85). */
typedef struct {
    int32_t n_grid;
    float grid_lim, dx, inv_dx;
    float gravity[3];
    float rpic_damping;                 /* 0 = APIC, < -0.001 = PIC */
    float grid_v_damping_scale;         /* applied only when < 1 */
    int32_t periodic_x;
    int32_t update_cov_with_F;          /* advect cov each substep (cov_mode "step") */
    uint32_t material_mask;             /* bit i set when any particle may carry material i */
    float E[GBMPM_MAX_MATERIALS], nu[GBMPM_MAX_MATERIALS], bulk[GBMPM_MAX_MATERIALS];
    float hardening[GBMPM_MAX_MATERIALS], xi[GBMPM_MAX_MATERIALS];
    float plastic_viscosity[GBMPM_MAX_MATERIALS], softening[GBMPM_MAX_MATERIALS];
    float alpha[GBMPM_MAX_MATERIALS];
    float muI_mu_s[GBMPM_MAX_MATERIALS], muI_delta_mu[GBMPM_MAX_MATERIALS];
    float muI_I0[GBMPM_MAX_MATERIALS], muI_d[GBMPM_MAX_MATERIALS];
    float muI_rho_s[GBMPM_MAX_MATERIALS], muI_phi_init[GBMPM_MAX_MATERIALS];
    float muI_phi_chi[GBMPM_MAX_MATERIALS];
    const float *eta_table;             /* eta_table_n samples; device pointer for the CUDA library */
    int32_t eta_table_n;
    float eta_table_smin, eta_table_smax;
} gbmpm_model;

/* Collider kinds (grid boundary conditions, applied in list order per node). */
enum {
    GBMPM_COLLIDER_PLANE = 0,   /* add_plane: surface 0 sticky, 1 slip, 2 separable, 11 cut */
    GBMPM_COLLIDER_BOX = 1,     /* add_box: kinematic velocity overwrite + impulse */
    GBMPM_COLLIDER_CUP = 2,     /* add_cup: analytic revolved-SDF glass, force + torque */
    GBMPM_COLLIDER_WALLS = 3,   /* add_domain_walls: 3-cell shells at the six faces */
    GBMPM_COLLIDER_SDF = 4      /* add_sdf_collider: trilinear voxel SDF, force + torque */
};

typedef struct {
    int32_t kind;
    int32_t surface_type;       /* plane / sdf surface type */
    int32_t reset;              /* box legacy reset flag */
    int32_t sdf_res;
    float start_time, end_time;
    float point[3];             /* plane point | box, cup or sdf centre (fp32, as in the Warp struct) */
    float normal[3];            /* plane unit normal */
    float size[3];              /* box half extents */
    float velocity[3];
    float omega[3];
    float rot[9];               /* cup local->world rotation, row-major fp32 */
    float quat[4];              /* sdf body->world rotation, x y z w */
    float friction;
    float outer_radius, inner_radius, half_height, inner_floor_z, fillet_radius;
    float sticky_depth, contact_band;
    float sdf_origin[3];
    float sdf_cell, band;
    const float *sdf_val;       /* [res^3] (device pointer for the CUDA library) */
    const float *sdf_grad;      /* [res^3][3] */
    double rot64[9];            /* cup: float64 rotation shadow (mpm_solver_warp.py:2227-2254) */
} gbmpm_collider;

/* CPIC thin-boundary (CDF) collider lane (CDFCollider, kernels/warp_utils.py:261-285).
 * Up to GBMPM_MAX_CDF lanes; the lane index is the collider handle. */
#define GBMPM_MAX_CDF 4
typedef struct {
    const float *values;        /* [res^3] side-signed distance to the sheet (device pointer for the library) */
    const float *valid;         /* [res^3] 1 where distance and side are trustworthy */
    int32_t res;
    int32_t surface_type;       /* 0 sticky, 1 slip, 2 separable + Coulomb */
    float origin[3];
    float cell;
    float center[3];            /* world position of the body origin */
    float quat[4];              /* body -> world, x y z w */
    float velocity[3];
    float omega[3];
    float band;
    float friction;
    float start_time, end_time;
} gbmpm_cdf;

/* gbmpm_tick flags */
#define GBMPM_TICK_FUSED   1    /* fused G2P2G pipeline (Solver.fused) */
#define GBMPM_TICK_GRAPH   2    /* replay the tick as one captured CUDA graph when possible */
#define GBMPM_TICK_PROFILE 4    /* per-phase CUDA-event timing, live launches */
#define GBMPM_TICK_REORDER 8    /* run the tick on a block-sorted working copy with shared-memory
                                   grid tiles (results equal up to float summation order) */
#define GBMPM_TICK_DETERMINISTIC 16  /* deterministic passes: every operation rounded once, P2G summed
                                        per node in particle order (sorted records, no float atomics);
                                        bit-reproducible; every material law but the rigid bodies',
                                        and the particle modifiers (rigid bodies, CDF lanes:
                                        GBMPM_ERR_UNSUPPORTED) */

#define GBMPM_NUM_PHASES 6      /* stress, p2g, g2p2g_fused, grid_update, g2p, sort+gather/scatter */

typedef struct gbmpm_engine gbmpm_engine;

const char *gbmpm_last_error(void);
const char *gbmpm_phase_name(int32_t phase);

/* Lifecycle. create selects the current CUDA device; destroy frees engine-owned
 * scratch (collider tables, block lists, sort scratch), never caller buffers. */
int gbmpm_engine_create(gbmpm_engine **out);
void gbmpm_engine_destroy(gbmpm_engine *e);

/* Bind caller-owned device buffers. Pointers must stay valid and stable until
 * the next bind (captured CUDA graphs bake them in). */
int gbmpm_bind(gbmpm_engine *e, const gbmpm_particles *p, const gbmpm_grid *g);
int gbmpm_set_model(gbmpm_engine *e, const gbmpm_model *m);

/* Replace the collider list. Wrench accumulators of indices that already
 * existed are kept; new indices start at zero. */
int gbmpm_set_colliders(gbmpm_engine *e, const gbmpm_collider *c, int32_t n);
/* Copy the engine's current collider records (poses integrated by ticks). */
int gbmpm_get_colliders(gbmpm_engine *e, gbmpm_collider *c, int32_t n);

/* Advance `substeps` substeps of size dt. *time is the simulation clock in
 * float64 (Python float in the reference); it advances by dt per substep. */
int gbmpm_tick(gbmpm_engine *e, double *time, double dt, int32_t substeps,
               int32_t flags, void *stream);

/* Edge guard: out = {min x, min y, min z, max x, max y, max z, max |v_i|}
 * over all particles, and *status = the device status word (then cleared).
 * Synchronizes the stream. */
int gbmpm_guard(gbmpm_engine *e, float out[7], uint32_t *status, void *stream);

/* Replace the CDF lanes (add_cdf_collider / set_cdf_pose, mpm_solver_warp.py:2819-2953).
 * A lane whose centre or orientation changed is restamped at the next substep.
 * Scenes with CDF lanes tick with live launches (no graph, no block reorder). */
int gbmpm_set_cdf(gbmpm_engine *e, const gbmpm_cdf *lanes, int32_t n);
/* Current lane records (poses integrated by ticks). */
int gbmpm_get_cdf(gbmpm_engine *e, gbmpm_cdf *lanes, int32_t n);
/* Blocked-deposit reaction of a lane since the last reset: {fx, fy, fz, tx, ty, tz}
 * (cdf_wrench, core/solver.py:401-413); the reset clears every lane. */
int gbmpm_cdf_wrench(gbmpm_engine *e, int32_t lane, double out[6], void *stream);
int gbmpm_reset_cdf_wrench(gbmpm_engine *e, void *stream);
/* Node tag and owner-distance grids of the last stamp (grid_cdf_tag, grid_cdf_d,
 * mpm_solver_warp.py:2906-2915), copied into caller device buffers of n_grid^3
 * entries (either may be NULL), and the number of stamps so far (_cdf_stamp_count). */
int gbmpm_cdf_grids(gbmpm_engine *e, int32_t *tag_out, float *d_out, int64_t *stamps, void *stream);
/* Stamp every CDF lane now, at `time` (MPM_Simulator_WARP._stamp_cdf called
 * directly, mpm_solver_warp.py:3040-3098); the previous grids take the new stamp. */
int gbmpm_cdf_restamp(gbmpm_engine *e, double time, void *stream);
/* on != 0: restamp every lane at every substep instead of only the lanes that moved
 * or changed activity (the _cdf_force_stamp switch, :3046-3052). */
int gbmpm_cdf_force_stamp(gbmpm_engine *e, int32_t on);
/* off != 0: every particle scans its 27 stencil nodes for CPIC tags instead of
 * skipping stencils that touch no tagged 4^3 block (model.cdf_mask_off,
 * kernels/warp_utils.py:84, read at kernels/mpm_utils.py:856, 980). The skip is
 * exact, so results do not change. */
int gbmpm_cdf_mask_off(gbmpm_engine *e, int32_t off);
/* 1 when a captured tick graph is ready for replay, 0 when none is, -1 after a
 * capture failed: ticks then launch live for the rest of the run, as the
 * reference falls back (kernels/mpm_solver_warp.py:1118-1125). */
int32_t gbmpm_graph_state(gbmpm_engine *e);
/* Test hook for failure handling: the next capture is discarded as if it had failed.
 * Nothing invalid reaches the GPU. */
int gbmpm_debug_fail_next_capture(gbmpm_engine *e);

/* Current volume vol0 * J, Cauchy stress = stress / J and J = det(F) per particle
 * (Solver.vol / Solver.cauchy, core/solver.py:559-598) into caller device buffers
 * (any may be NULL). policy 0 warn: |J| (Cauchy divides by max(|J|, 1e-9));
 * 1 nan and 2 raise: NaN for inverted particles. *n_inverted (host, may be NULL:
 * then nothing synchronizes) receives the count of non-finite or non-positive J. */
int gbmpm_compute_cauchy(gbmpm_engine *e, float *cauchy_out, float *vol_out, float *J_out, int32_t policy,
                         int32_t *n_inverted, void *stream);

/* Stress-integral reaction on a kinematic box (box_contact_wrench,
 * coupling/wrench.py:15-46) over the bound particles: out = {fx, fy, fz, tx, ty, tz,
 * contacts, sum of current volume, inverted particles}. layer <= 0 takes
 * 3 mean(vol)^(1/3). Volume and Cauchy stress follow the inversion policy
 * (0 warn: |det F|, 1 nan, 2 raise: GBMPM_ERR_STATE when any particle is inverted;
 * core/solver.py:559-598). The caller zeroes the result when contacts < 3. */
int gbmpm_contact_wrench(gbmpm_engine *e, const double box_center[3], const double box_half[3],
                         double layer, int32_t compressive_only, int32_t policy, double out[9],
                         void *stream);

/* ---- adjoint (no counterpart in the reference) ---------------------------------
 * Adjoints of the particle state (x, v, C, F_trial, yield_stress, L, and Jp, the
 * mu(I)-Phi(I) packing state; device arrays in the particle layout) and accumulated
 * per-particle adjoints of mu, lam and of the Newtonian viscosity (its sum is the
 * gradient of the per-type value).
 * Collider trajectories (optional, NULL to skip): collider_force holds, for every
 * substep of the segment, the adjoint of each collider's force accumulator
 * ([substeps][n_colliders][3]; the reaction that gbmpm_wrench and the reference's
 * tool_force read, core/solver.py:415-427), and collider_velocity accumulates the
 * adjoint of each kinematic cuboid's velocity ([n_colliders][3]; the velocity
 * add_box / set_box give, which moves the box and sets the velocity of the nodes it
 * covers, mpm_solver_warp.py:2053-2096). */
typedef struct gbmpm_adj_grads {
    float *x, *v, *C, *F_trial, *yield_stress;
    float *mu, *lam;
    float *L, *viscosity;
    float *Jp;
    const float *collider_force;
    float *collider_velocity;
} gbmpm_adj_grads;

/* Replays `substeps` split-schedule substeps forward from the bound state (the
 * caller restores a checkpoint first), keeping each substep's starting state, then
 * carries the adjoints in g from the end of the segment back to its start and adds
 * each substep's contribution to g->mu, g->lam and g->viscosity. Leaves the bound
 * state at the segment's end and advances *time. Covers every material law but the
 * rigid bodies' and every grid collider; CDF lanes, rigid bodies, particle
 * modifiers, periodic x and rpic_damping != 0 are GBMPM_ERR_UNSUPPORTED. */
int gbmpm_adjoint_segment(gbmpm_engine *e, double *time, double dt, int32_t substeps,
                          const gbmpm_adj_grads *g, void *stream);

/* The two halves of gbmpm_adjoint_segment, for callers that keep every substep's
 * state instead of replaying the segment: gbmpm_adjoint_forward steps the segment
 * from the bound state (advancing it and *time, as a tick on the split schedule
 * does) and writes each substep's starting state into `states` (device memory,
 * 37 x n floats per substep: x 3, v 3, C 9, F_trial 9, L 9, yield 1, mu 1, lam 1,
 * Jp 1 per particle, field-major); gbmpm_adjoint_reverse runs the reverse
 * substeps of that segment from `states`, with the collider poses and *time of the
 * segment's start (the caller restores them, as for gbmpm_adjoint_segment). */
int gbmpm_adjoint_forward(gbmpm_engine *e, double *time, double dt, int32_t substeps, float *states,
                          void *stream);
int gbmpm_adjoint_reverse(gbmpm_engine *e, double *time, double dt, int32_t substeps, const float *states,
                          const gbmpm_adj_grads *g, void *stream);

/* Reaction impulse accumulated since the last reset: {fx, fy, fz, tx, ty, tz}. */
int gbmpm_wrench(gbmpm_engine *e, int32_t collider, double out[6], void *stream);
int gbmpm_reset_wrench(gbmpm_engine *e, int32_t collider, void *stream);

/* Block-key sort: key = ((bx*nb + by)*nb + bz), b = floor(x/dx - 0.5) >> 2 in
 * float64, nb = (n_grid >> 2) + 2; stable; skipped when keys are already
 * non-decreasing (*sorted_out = 0). On a sort every per-particle array (and
 * perm_out, when not NULL, the int32 permutation) is rewritten in place. */
int gbmpm_sort_particles(gbmpm_engine *e, double dx, int32_t *sorted_out,
                         int32_t *perm_out, void *stream);

/* Active 4^3 blocks: mark (fp32 truncation), dilate by one block, compact.
 * counts = {current, union with previous}. Synchronizes the stream. */
int gbmpm_rebuild_active_blocks(gbmpm_engine *e, int32_t counts[2], void *stream);

/* Exports: R_out[n][9] receives R^T of the polar rotation of F_trial;
 * cov_out[n][6] receives F_trial * init_cov * F_trial^T. */
int gbmpm_compute_R(gbmpm_engine *e, float *R_out, void *stream);
int gbmpm_compute_cov(gbmpm_engine *e, float *cov_out, void *stream);

/* Per-phase device milliseconds accumulated while GBMPM_TICK_PROFILE was set. */
int gbmpm_profile(gbmpm_engine *e, double ms_out[GBMPM_NUM_PHASES],
                  int64_t count_out[GBMPM_NUM_PHASES], int32_t reset);

/* Batched scenes (no counterpart in the reference, whose planners step one
 * Solver at a time): a batch advances many independent engines in one CUDA graph
 * whose branches are the scenes' tick chains, so scenes too small to fill the GPU
 * run concurrently. times[n] are the scenes' clocks. Without GBMPM_TICK_GRAPH the
 * scenes are recorded one after another on the stream (the serial baseline).
 * gbmpm_batch_guard runs every scene's edge guard with one synchronization:
 * out[n][7] and status[n] as in gbmpm_guard. */
typedef struct gbmpm_batch gbmpm_batch;
int gbmpm_batch_create(gbmpm_engine *const *engines, int32_t n, gbmpm_batch **out);
void gbmpm_batch_destroy(gbmpm_batch *b);
int gbmpm_batch_tick(gbmpm_batch *b, double *times, double dt, int32_t substeps, int32_t flags, void *stream);
int gbmpm_batch_guard(gbmpm_batch *b, float *out, uint32_t *status, void *stream);
int64_t gbmpm_batch_launch_count(gbmpm_batch *b);
/* Schedule and launch shape of the batch's fused ticks (no counterpart in the
 * reference, which steps scenes one after another). With single_launch (the
 * default) a tick whose scenes all run the fused schedule on their block-sorted
 * working sets, with no CPIC lanes, rigid bodies or particle modifiers, launches
 * each particle pass and each grid pass once over every scene; otherwise each
 * scene's own tick is a branch of the batch graph. tile_threads (64, 128 or 256
 * particles per CTA) and tile_occ (2 or 3 resident 256-thread equivalents per SM)
 * select the particle-pass kernel; grid_ctas (1 to 8 per SM) sizes the grid pass,
 * shared out over the scenes by particle count. The autotuner
 * (mpm_engine_gb300.autotune) sets these. */
int gbmpm_batch_set_tuning(gbmpm_batch *b, int32_t single_launch, int32_t tile_threads, int32_t tile_occ,
                           int32_t grid_ctas);
/* out = {single_launch, tile_threads, tile_occ, grid_ctas, last captured graph
 * runs the single-launch schedule (0/1)}. */
int gbmpm_batch_get_tuning(gbmpm_batch *b, int32_t out[5]);
/* As gbmpm_graph_state for the batch graph: 1 ready, 0 none, -1 after a failed
 * capture (the scenes then tick live, one after another, for the rest of the run). */
int32_t gbmpm_batch_graph_state(gbmpm_batch *b);
/* Test hook: the batch's next capture is discarded as if it had failed. */
int gbmpm_batch_debug_fail_next_capture(gbmpm_batch *b);

/* Edge-guard reduction that allocates nothing (no counterpart in the reference).
 * For callers that cannot call cudaMalloc: a process whose device memory is owned
 * by another allocator, or a control loop that must not take cudaMalloc's implicit
 * synchronization. Same out[7] as gbmpm_guard, over device arrays x, v of [n][3]
 * floats, plus *nonfinite = 1 when a position is not finite. Scratch is a 33 KB
 * static device array, so n <= 4194304 (larger n: GBMPM_ERR_ARG). Calls that
 * overlap on the GPU race on that array. Every call looks up the array's address
 * in the current context (no cached pointer survives a device reset) and
 * synchronizes the stream. */
int gbmpm_guard_noalloc(const float *x, const float *v, int32_t n, float out[7], int32_t *nonfinite,
                        void *stream);

/* Rigid bodies (MPM_Simulator_WARP.finalize_rigid_bodies / _p2g2p_tail,
 * mpm_solver_warp.py:818-987, 1338-1367; kernels mpm_utils.py:1369-1493). The
 * material-8 particles of body b (particles.rigid_id) move with it: after every
 * G2P the body gathers the grid momentum of its particles, integrates (v_cm = P/M,
 * omega = I_world^-1 L, x_cm += dt v_cm, R re-orthogonalised by polar
 * decomposition), takes restitution impulses from the rigid surfaces (add_plane
 * with restitution > 0; the host loop of _apply_rigid_restitution, here on the
 * device) and writes back x, v = v_cm + omega x r, C = skew(omega), F = I. R and the
 * inverse body inertia are row-major. gbmpm_set_rigid replaces bodies and surfaces;
 * gbmpm_get_rigid reads the bodies back (synchronizing the stream). */
typedef struct gbmpm_rigid_body {
    float x_cm[3], v_cm[3], omega[3];
    float R[9];
    float mass;
    float inv_inertia[9];
} gbmpm_rigid_body;
typedef struct gbmpm_rigid_surface {
    double point[3], normal[3];         /* normal of unit length */
    double friction, restitution;
    double start_time, end_time;
} gbmpm_rigid_surface;
#define GBMPM_MAX_RIGID_SURFACES 8
int gbmpm_set_rigid(gbmpm_engine *e, const gbmpm_rigid_body *bodies, int32_t n_bodies,
                    const gbmpm_rigid_surface *surfaces, int32_t n_surfaces);
int gbmpm_get_rigid(gbmpm_engine *e, gbmpm_rigid_body *bodies, int32_t n_bodies, void *stream);

/* Particle modifiers (add_impulse_on_particles, enforce_particle_velocity_translation,
 * enforce_particle_velocity_rotation; mpm_solver_warp.py:2385-2540), applied to the
 * particles whose particles.mod_mask has bit m set, before the stress and P2G of
 * every substep whose start time t (float32) lies in [start_time, end_time): first
 * every impulse (v += force / m * dt), then every velocity override, each kind in
 * list order. kind 1 sets v = vec; kind 2 sets the rotation field about the axis
 * through `point` along `normal` (rotation_scale, translation_scale, with the
 * reference's horizontal axes axis1, axis2). At most 32 modifiers. */
typedef struct gbmpm_modifier {
    int32_t kind;                       /* 0 impulse, 1 velocity translation, 2 velocity rotation */
    float start_time, end_time;
    float vec[3];                       /* kind 0: force; kind 1: velocity */
    float point[3], normal[3], axis1[3], axis2[3];
    float rotation_scale, translation_scale;
} gbmpm_modifier;
#define GBMPM_MAX_MODIFIERS 32
int gbmpm_set_modifiers(gbmpm_engine *e, const gbmpm_modifier *mods, int32_t n);

/* Mesh -> distance-field searches (warpmpm.geometry.mesh_sdf,
 * src/warpmpm/geometry/mesh_sdf.py), engine-free. Every array is device memory,
 * float64, row-major; work is ordered on `stream`. The query points are either
 * `points` [n][3] or, with points == NULL, the res^3 nodes origin + cell * (i, j, k)
 * of a cubic field grid, i slowest (the meshgrid "ij" order of build_sdf :341-348).
 *
 * gbmpm_field_nearest: per point the nearest of the samples [n_samples][3] (the
 *   cKDTree query of _unsigned_distance :314-326 and build_surface_cdf :451-466):
 *   dist_out[p] = sqrt((dx^2 + dy^2) + dz^2) in float64, index_out[p] the sample,
 *   the lowest index on a tie.
 * gbmpm_field_winding: per point the generalized winding number over the faces
 *   tri [n_faces][3 vertices][3] (_winding_number :210-233). Summed in float32
 *   except where within the float32 error of +-0.5, or everywhere with precise != 0.
 * gbmpm_field_tri_distance: per point the exact distance to the nearest face
 *   (_point_triangle_distance_exact :236-289). */
typedef struct gbmpm_field_points {
    const double *points;   /* device [n][3], or NULL for the grid */
    int64_t n;
    double origin[3];
    double cell;
    int32_t res;
} gbmpm_field_points;
int gbmpm_field_nearest(const gbmpm_field_points *pts, const double *samples, int64_t n_samples, double *dist_out,
                        int64_t *index_out, void *stream);
int gbmpm_field_winding(const gbmpm_field_points *pts, const double *tri, int64_t n_faces, int32_t precise,
                        double *wn_out, void *stream);
int gbmpm_field_tri_distance(const gbmpm_field_points *pts, const double *tri, int64_t n_faces, double *dist_out,
                             void *stream);

/* Number of kernels this engine has launched (graph replays count each node). */
int64_t gbmpm_launch_count(gbmpm_engine *e);
/* Launch shape of one scene's passes (no counterpart in the reference): tile_occ
 * (2 to 4 resident 256-thread equivalents per SM; 4 only for scenes without
 * SVD-based laws) selects the tiled particle kernel, grid_ctas (1 to 8 per SM) the
 * grid-update launch. Set by the autotuner (mpm_engine_gb300.autotune). */
int gbmpm_set_tuning(gbmpm_engine *e, int32_t tile_occ, int32_t grid_ctas);
/* out = {tile_occ, grid_ctas}. */
int gbmpm_get_tuning(gbmpm_engine *e, int32_t out[2]);
/* Re-sorts of the block-sorted working copy inside a tick (no counterpart in the
 * reference, whose particle order changes only through sort_interval): a fused tick
 * sorts its working copy again by the particles' current cells every `substeps`
 * substeps, so the scatter's runs of one cell stay long as particles move; a re-sort
 * that would leave less than half an interval of the tick is skipped. 0 sorts once per tick. GBMPM_RESORT_AUTO (the
 * default) re-sorts ticks of S >= 100 substeps of scenes of 150,000 particles or more
 * every max(50, S / 3) substeps. The caller's particle order never changes. */
#define GBMPM_RESORT_AUTO (-1)
int gbmpm_set_resort(gbmpm_engine *e, int32_t substeps);
/* The re-sort setting (GBMPM_RESORT_AUTO, 0 or an interval; -2 for a null engine). */
int32_t gbmpm_get_resort(gbmpm_engine *e);
/* Test hook (no counterpart in the reference): deposits the current particle state
 * (stored stress, v, C; no stress update) into the grid with the P2G kernel,
 * returns out[4] = {sum m, sum m vx, sum m vy, sum m vz} over every grid node in
 * float64, then clears the grid and the block bookkeeping again. Checks that P2G
 * conserves mass and momentum (the B-spline weights sum to 1, the APIC and stress
 * terms sum to 0). Synchronizes the stream. */
int gbmpm_debug_deposit_sums(gbmpm_engine *e, double dt, double out[4], void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GBMPM_H */
