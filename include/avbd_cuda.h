/*
 * avbd_cuda.h - C ABI of the GB300 AVBD world-step backend.
 *
 * This library is a third backend for the AVBD sandbox's scene graph, next to
 * the f64 CPU engine (`Solver.step()`, src/physics/solver.js:307-493) and the
 * WebGPU engine (`GpuBackend`, src/physics/gpu/backend.js:243). The scene graph
 * (bodies, joints, springs, contact manifolds) crosses this boundary as
 * structure-of-arrays of plain doubles and ints owned by the caller; the
 * context owns all device memory and retains no caller pointer after a call
 * returns.
 *
 * Conventions (from src/math/maths.js:14-22):
 *   vec3  = 3 doubles [x, y, z]
 *   quat  = 4 doubles [x, y, z, w], w the scalar part
 *   mat3  = 9 doubles, row-major
 *   gravity acts on world z (Z-up)
 *
 * Every function returns an int status: AVBD_OK (0) or a negative AVBD_ERR_*.
 * No exception crosses the ABI. `avbd_last_error` gives the text of the most
 * recent failure on a context.
 *
 * Threading: a context is NOT thread-safe; distinct contexts are independent.
 * `avbd_step` is asynchronous on the context's CUDA stream; every read
 * synchronises that stream first.
 */
#ifndef AVBD_CUDA_H
#define AVBD_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define AVBD_OK 0
#define AVBD_ERR_ARG (-1)      /* bad argument or inconsistent scene data     */
#define AVBD_ERR_CAPACITY (-2) /* a device arena overflowed; the step was redone
                                  after regrowing, or could not be             */
#define AVBD_ERR_CUDA (-3)     /* a CUDA runtime call failed                  */
#define AVBD_ERR_TIMEOUT (-4)  /* a bounded device-side wait gave up          */
#define AVBD_ERR_NAN (-5)      /* a non-finite body state was produced/given  */
#define AVBD_ERR_STATE (-6)    /* call made in the wrong state (e.g. no pack) */

/* ---- body shapes (src/physics/rigid.js:32, :125) ------------------------ */
#define AVBD_SHAPE_BOX 0
#define AVBD_SHAPE_SPHERE 1

/* ---- body visit order of the primal sweep (src/physics/solver.js:419-422) */
#define AVBD_ORDER_REFERENCE 0 /* newest body first (oracle only)            */
#define AVBD_ORDER_EXPLICIT 1  /* caller-supplied order (the bodyOrder hook)  */
#define AVBD_ORDER_PRIORITY 2  /* colour order of the integer-priority greedy
                                  colouring of this step's constraint graph:
                                  the GPU schedule                            */

/* ---- overflow bits reported in avbd_stats.overflow ---------------------- */
#define AVBD_OVF_CELLS 0x1u      /* hash-grid insertions                     */
#define AVBD_OVF_PAIRS 0x2u      /* candidate pairs per body / in total      */
#define AVBD_OVF_ADJ 0x4u        /* per-body constraint adjacency            */
#define AVBD_OVF_COLORS 0x8u     /* more than AVBD_MAX_COLORS colours        */
#define AVBD_OVF_TIMEOUT 0x10u   /* bounded grid barrier gave up             */
#define AVBD_ERR_COLORING 0x200u /* an uploaded colouring was not proper     */

#define AVBD_MAX_CONTACTS 8 /* contacts per manifold (src/physics/collide.js:22) */
#define AVBD_MAX_COLORS 1024 /* colours the device colouring can hold: the greedy
                                colouring needs at most the largest number of
                                dynamic neighbours of one body, plus one      */

/*
 * Solver parameters. Field meanings and defaults follow
 * `Solver.defaultParams()` (src/physics/solver.js:92-236); the GPU-only fields
 * at the end have no counterpart there.
 */
typedef struct avbd_params {
  double dt;               /* 1/60                                          */
  double gravity;          /* -10, acts on world z                          */
  int32_t iterations;      /* 10                                            */
  int32_t post_stabilize;  /* 0                                             */
  double beta_lin;         /* 1e4                                           */
  double beta_ang;         /* 100                                           */
  double alpha;            /* 0.95                                          */
  double gamma;            /* 0.999                                         */
  double penalty_min;      /* 1                                             */
  double penalty_max;      /* 1e10                                          */
  double collision_margin; /* 0.01                                          */
  double stick_threshold;  /* 1e-5                                          */
  int32_t rotated_inertia;           /* 1                                   */
  int32_t spring_stiffness_ramp;     /* 0                                   */
  int32_t spring_geometric_stiffness;/* 1                                   */
  int32_t cached_contact_jacobians;  /* 1                                   */
  int32_t broadphase;      /* oracle only: 0 auto, 1 hash, 2 brute force     */
  int32_t hash_threshold;  /* oracle only: 150                              */
  int32_t body_order;      /* AVBD_ORDER_*; the CUDA backend always uses
                              AVBD_ORDER_PRIORITY                           */
  /* Polls before a device wait (grid barrier, neighbour progress) gives up:
     the kernel then returns and avbd_synchronize reports AVBD_ERR_TIMEOUT;
     the context needs avbd_pack again. 0 = default (about a second). */
  int32_t wait_limit;
  /* GPU precision policy. A body whose largest constraint stiffness divided
     by its inertial stiffness m/dt^2 exceeds this ratio is assembled and
     factored in FP64; everything else runs in FP32. <= 0 disables FP64.    */
  double fp64_ratio_threshold;
  /* GPU capacity policy (0 = automatic). */
  int32_t max_pairs_per_body; /* candidate partners with a lower index      */
  int32_t max_adjacency;      /* constraints incident to one dynamic body   */
  /* Lanes per body update: 1, 2, 4, 8, 16 or 32 for every body. 0 =
     automatic: under schedule 0 each body gets the fewest lanes (4..128, up
     to four warps; FP64 bodies at most 32) whose staging of four constraints
     per lane holds all of its constraints; schedule 1 uses 32. */
  int32_t lanes_per_body;
  int32_t blocks_per_sm;      /* 0 = automatic                              */
  /* Schedule of the primal/dual iterations on the device:
     0 = colour phases separated by a grid barrier (default),
     1 = dependency wavefront (each body waits only for its neighbours).
     Both give the same result for the same nonzero lanes_per_body. */
  int32_t schedule;
  int32_t grid_factor;        /* hash-grid arena multiplier (0 = 1)         */
  /* Polls before a neighbour-progress wait (the wavefront schedule, the
     colour-phase schedule's tail segment) gives up; 0 = wait_limit (or its
     default when that is 0 as well). Grid barriers keep wait_limit.        */
  int32_t neighbor_wait_limit;
  /* Colour-phase schedule: colours of at most (solve blocks / tail_div) lane
     chunks run as one dependency-driven tail segment per iteration instead
     of one grid barrier each. 0 (automatic): tail_div 8 for steps of at
     least 16 colours, no tail segment for fewer; > 0: that tail_div every
     step; < 0: no tail segment. Does not change results. */
  int32_t tail_div;
  /* 1: each step is replayed as a CUDA graph (captured on first use, once
     per manifold-arena parity; rebuilt after a pack, an arena regrow, an
     uploaded colouring or avbd_autotune). Profiled steps launch directly.
     Does not change results. */
  int32_t graph;
  /* Contact model. AVBD_CONTACT_CPU (0, default): the CPU engine's - one
     friction coefficient, collision_margin on C0, stick = |C_t| below
     stick_threshold, warm start by feature ID (src/physics/manifold.js).
     AVBD_CONTACT_MATERIALS (1): the WebGPU engine's contact extensions
     (src/physics/gpu/shaders.js:1152-1366, 1772-1849, 2235-2260;
     src/physics/rigid.js:144-214): static and dynamic friction (a contact
     that was static uses the static cone; once outside it is clamped to
     the dynamic one), stick = inside the cone, new contacts start static;
     thresholded restitution (a one-frame bias for new or re-armed impacts);
     C0 on the normal measured to the rest distance (the pair's rest offsets)
     with a speculative gap kept unscaled while the pair's contact offsets
     are positive; warm start by feature ID, then by the nearest old contact
     within the persistence distance, each old contact claimed once, with
     multipliers and penalties transported into the new basis. Contact
     generation stays the CPU collider's (no speculative contacts at a
     positive separation). */
  int32_t contact_model;
  double contact_offset;        /* per-body default, 0.005 (solver.js:151)   */
  double rest_offset;           /* per-body default, -0.005 (solver.js:152)  */
  double restitution_threshold; /* 1.0 m/s (solver.js:155)                   */
  double contact_persistence;   /* 0.002 m (solver.js:162)                   */
} avbd_params;

#define AVBD_CONTACT_CPU 0
#define AVBD_CONTACT_MATERIALS 1

/*
 * Bodies, `Rigid` (src/physics/rigid.js:29-133). Static shape/material fields
 * are inputs of avbd_pack; pos/quat/vel/omega/prev_vel are the dynamic state
 * read and written by avbd_read_state / avbd_write_state.
 */
typedef struct avbd_body_soa {
  int32_t count;
  int32_t *shape;     /* AVBD_SHAPE_*                                        */
  double *size;       /* 3 per body: full widths                             */
  double *mass;       /* 0 makes the body static                             */
  double *moment;     /* 3 per body: body-frame principal moments            */
  double *radius;     /* bounding radius; a sphere's own radius              */
  double *friction;   /* combined pairwise as sqrt(fa*fb)                    */
  double *pos;        /* 3 per body                                          */
  double *quat;       /* 4 per body                                          */
  double *vel;        /* 3 per body                                          */
  double *omega;      /* 3 per body                                          */
  double *prev_vel;   /* 3 per body                                          */
  /* Contact materials of AVBD_CONTACT_MATERIALS (Rigid.setMaterial,
     src/physics/rigid.js:144-214), each optional (NULL = default): static
     and dynamic friction (default: friction; pairs combine as sqrt(a b)),
     restitution in [0, 1] (default 0; pairs take the max), contact and rest
     offsets (defaults: the params'; pairs add them). */
  double *static_friction;
  double *dynamic_friction;
  double *restitution;
  double *contact_offset;
  double *rest_offset;
} avbd_body_soa;

/* Ball-socket joints, `Joint` (src/physics/joint.js:74-113). */
typedef struct avbd_joint_soa {
  int32_t count;
  int32_t *body_a;        /* -1: r_a is a fixed world anchor                 */
  int32_t *body_b;
  double *r_a;            /* 3 per joint                                     */
  double *r_b;            /* 3 per joint                                     */
  double *stiffness_lin;  /* INFINITY = hard                                 */
  double *stiffness_ang;  /* 0 disables the angular rows                     */
  double *fracture;       /* threshold on |lambda_ang|; INFINITY = none      */
  double *penalty_lin;    /* state, 3 per joint                              */
  double *penalty_ang;    /* state, 3 per joint                              */
  double *lambda_lin;     /* state, 3 per joint                              */
  double *lambda_ang;     /* state, 3 per joint                              */
  int32_t *broken;        /* state                                           */
  int32_t *order;         /* optional: position in the global force list     */
} avbd_joint_soa;

/* Distance springs, `Spring` (src/physics/spring.js:414-444). */
typedef struct avbd_spring_soa {
  int32_t count;
  int32_t *body_a;
  int32_t *body_b;
  double *r_a;            /* 3 per spring                                    */
  double *r_b;            /* 3 per spring                                    */
  double *stiffness;
  double *rest;           /* >= 0 (the caller resolves "current length")     */
  double *tear_strain;    /* INFINITY = never tears                          */
  double *penalty;        /* state                                           */
  double *peak_strain;    /* state                                           */
  int32_t *broken;        /* state                                           */
  int32_t *order;         /* optional: position in the global force list     */
} avbd_spring_soa;

/*
 * Persistent contact manifolds, `Manifold` + `Contact`
 * (src/physics/manifold.js:33-69, :164-189). Body A has the HIGHER index of
 * the pair (the broad phase visits (i, j) with j < i,
 * src/physics/broadphase.js:13-16). Contact arrays hold AVBD_MAX_CONTACTS
 * slots per manifold. On read, `count` returns the number of live manifolds
 * and at most `capacity` are written.
 */
typedef struct avbd_manifold_soa {
  int32_t count;
  int32_t capacity;
  int32_t *body_a;
  int32_t *body_b;
  int32_t *num_contacts;
  double *basis;          /* 9 per manifold; row 0 = normal B->A            */
  double *friction;
  uint32_t *feature;      /* 8 per manifold                                  */
  double *r_a;            /* 8*3 per manifold, body-A local                  */
  double *r_b;            /* 8*3 per manifold, body-B local                  */
  double *c0;             /* 8*3 per manifold, C*(x_t) (read only)           */
  double *penalty;        /* 8*3 per manifold                                */
  double *lambda;         /* 8*3 per manifold                                */
  int32_t *stick;         /* 8 per manifold                                  */
  int32_t *order;         /* optional: position in the global force list     */
  double *restitution_bias; /* 8 per manifold, AVBD_CONTACT_MATERIALS only  */
} avbd_manifold_soa;

/*
 * A world: one scene, or a batch of independent scenes laid end to end.
 * Scene s owns bodies [scene_start[s], scene_start[s+1]); constraints may
 * not cross scenes. num_scenes <= 1 with scene_start NULL means one scene.
 */
typedef struct avbd_world {
  avbd_body_soa bodies;
  avbd_joint_soa joints;
  avbd_spring_soa springs;
  avbd_manifold_soa manifolds; /* count 0 on pack = no warm-start contacts   */
  int32_t num_scenes;
  int32_t *scene_start;        /* num_scenes + 1 entries                     */
} avbd_world;

/* Diagnostics, `Solver.stats` (src/physics/solver.js:77-89, :495-528). */
typedef struct avbd_stats {
  int64_t bodies;
  int64_t manifolds;
  int64_t contacts;
  int64_t candidate_pairs;
  int64_t joints_broken;
  int64_t springs_broken;
  int32_t colors;
  int32_t fp64_bodies;
  uint32_t overflow;       /* AVBD_OVF_* bits seen since the last pack       */
  int32_t steps;           /* steps taken since the last pack                */
  double max_constraint_error;
  double max_lambda;
  double max_penalty;
  int64_t graph_steps;     /* steps replayed as a CUDA graph since the pack  */
} avbd_stats;

/* Per-phase device times of the last step, ms (src/physics/gpu/backend.js:58),
   and the work that step did (the counters the phase times are divided by). */
typedef struct avbd_profile {
  double broadphase_ms;
  double narrowphase_ms;
  double prepare_ms;
  double coloring_ms;
  double solve_ms;
  double step_ms;
  int64_t candidate_pairs;    /* pairs the narrow phase tested              */
  int64_t manifolds;          /* manifolds with at least one contact        */
  int64_t contacts;           /* contact points in those manifolds          */
  int32_t colors;
  int32_t fp64_bodies;
  /* narrow-phase work split: box pairs with a certain face / edge winner
     (f32 geometry) and pairs decided by the exact f64 collider */
  int32_t np_face;
  int32_t np_edge;
  int32_t np_exact;
  int32_t lanes_per_body;     /* lanes per body the step's solve used       */
  int32_t via_graph;          /* 1: the step ran as a CUDA graph; only
                                 step_ms is timed then (phases read 0)     */
} avbd_profile;

typedef struct avbd_ctx avbd_ctx;

/* Defaults of Solver.defaultParams() (src/physics/solver.js:92-236). */
void avbd_default_params(avbd_params *out);

/* Replaces `new GpuBackend()` + `init()` (src/physics/gpu/backend.js:243,337-450). */
int avbd_create(const avbd_params *params, avbd_ctx **out);

/* Replaces `destroyBuffers()` (src/physics/gpu/backend.js:471). */
int avbd_destroy(avbd_ctx *ctx);

/* Replaces the topology half of `pack(solver)` (src/physics/gpu/backend.js:662-1301):
   uploads shapes, constraints and state; sizes every arena. */
int avbd_pack(avbd_ctx *ctx, const avbd_world *world);

/* Replaces `step(solver)` (src/physics/gpu/backend.js:1393-1620). Asynchronous. */
int avbd_step(avbd_ctx *ctx, int32_t n_steps);

/* Replaces `idle()` (src/physics/gpu/backend.js:1804). Waits for queued steps and
   reports device-side errors (overflow, timeout). */
int avbd_synchronize(avbd_ctx *ctx);

/* Replaces `readState()` / `syncToCPU(solver)` (src/physics/gpu/backend.js:1984-2039,
   2154): body state, joint and spring state, and (when the manifold arrays are
   non-NULL) the live manifolds in pair order. Fields left NULL are skipped. */
int avbd_read_state(avbd_ctx *ctx, avbd_world *out);

/* CPU-authoritative handover back to the device: overwrite the dynamic state
   (bodies, joint/spring state and, if count > 0, the warm-start manifolds) of
   an already-packed world with the same topology. */
int avbd_write_state(avbd_ctx *ctx, const avbd_world *world);

/*
 * Replaces the identity-preserving repack of `pack(solver)` after a topology
 * edit (src/physics/gpu/backend.js:662-1301; identity runs :107-145): spawn,
 * erase, joints and springs added or removed. `world` is the new scene graph
 * (one scene); old_body[i] is the index body i had in the packed world, or -1
 * for a new body (likewise old_joint, old_spring; a NULL map means nothing of
 * that kind is carried). Carried elements keep their live device state -
 * bodies: position, orientation, velocities; joints: penalties, multipliers,
 * broken; springs: penalty, peak strain, torn - gathered on the device, with
 * no readback; everything else comes from `world` as in avbd_pack. When the
 * carried bodies keep their old relative order (append, erase, order-
 * preserving compaction), the warm-start contacts between two carried bodies
 * survive, renumbered; otherwise the contacts start afresh (the reference
 * starts a fresh generation then). `carried` (optional) returns the number of
 * warm-start manifolds carried. The grab and an uploaded colouring are
 * released, as by avbd_pack. Synchronous.
 */
int avbd_repack(avbd_ctx *ctx, const avbd_world *world, const int32_t *old_body, const int32_t *old_joint,
                const int32_t *old_spring, int64_t *carried);

/* Replaces `readColoring()` (src/physics/gpu/backend.js:2053): colour of every
   body in the last step (-1 for static bodies) and the number of colours. */
int avbd_read_coloring(avbd_ctx *ctx, int32_t *color_of, int32_t *num_colors);

/* Replaces `uploadColoring(entries, offsets, counts)` + `overrideColoring`
   (src/physics/gpu/backend.js:1925, 256-299): the colour of every body
   (n int32, -1 or any value for static bodies) to use instead of the
   device's priority colouring, from the next avbd_step on, until cleared
   with color_of = NULL. Each step checks it against that step's constraint
   graph; where two dynamic neighbours share a colour (or a colour is not
   below AVBD_MAX_COLORS) the step uses its own colouring and
   avbd_synchronize reports AVBD_ERR_ARG. Copied at the call. */
int avbd_set_coloring(avbd_ctx *ctx, const int32_t *color_of);

/* Replaces `updateJointAnchor(joint)` (src/physics/gpu/backend.js:1970-1978):
   set joint `joint`'s anchor on body A (its world point when the joint has no
   body A, as a drag joint) for the following steps, without a repack.
   Ordered on the context's stream after the steps already queued. */
int avbd_update_joint_anchor(avbd_ctx *ctx, int32_t joint, const double r_a[3]);

/* Replaces the mouse grab of `GpuBackend` (src/physics/gpu/backend.js:302-307,
   1330-1334; applied in src/physics/gpu/shaders.js:2119-2161): from the next
   queued step on, body `body` is pulled by a finite ball socket from the
   world point `target` to its body-local point `local`, C = target - (p +
   R local), with penalty fixed at `stiffness` (the app uses max(400,
   900 m), src/app/boot.js:592), no multiplier, in that body's primal only.
   No topology change: no repack, no colouring edge. body = -1 releases it
   (local and target may then be NULL). Ordered on the context's stream. */
int avbd_set_grab(avbd_ctx *ctx, int32_t body, const double local[3], const double target[3], double stiffness);

/* Replaces `getConstraintGpuState()` (src/physics/gpu/backend.js:1950-1967):
   where a renderer or another CUDA consumer on the same device finds the
   live state, without a copy. Valid until the next avbd_pack or
   avbd_destroy; read after avbd_synchronize (the stream's steps write them). */
typedef struct avbd_device_views {
  const double *body_pos;      /* x, y, z, unused: 4 doubles per body (x_t)   */
  const float *body_quat;      /* x, y, z, w: 4 floats per body               */
  int32_t body_count;
  const int32_t *joint_state;  /* per joint: bit 0 = broken                   */
  int32_t joint_count;
  const int32_t *spring_state; /* per spring: bit 0 = broken                  */
  int32_t spring_count;
} avbd_device_views;
int avbd_device_views_get(avbd_ctx *ctx, avbd_device_views *out);

/* Candidate pairs of the last broad phase (body A index, body B index), pair
   order; `count` returns the total, at most `capacity` written. */
int avbd_read_pairs(avbd_ctx *ctx, int32_t *body_a, int32_t *body_b,
                    int64_t capacity, int64_t *count);

/* Replaces `lastStats` (src/physics/gpu/backend.js:309, 1650-1680). */
int avbd_read_stats(avbd_ctx *ctx, avbd_stats *out);

/* Replaces `setProfiling(on)` / `lastProfile` (src/physics/gpu/backend.js:1836-1897).
   When on, each step records CUDA events on the context's stream (per phase,
   or around the whole step when it runs as a graph) and waits for them. */
int avbd_set_profiling(avbd_ctx *ctx, int32_t on);
int avbd_read_profile(avbd_ctx *ctx, avbd_profile *out);

/* Number of device kernels launched since the last pack. */
int avbd_kernel_launches(avbd_ctx *ctx, int64_t *out);

/*
 * Autotuner of the solve's launch configuration: the schedule (colour phases
 * or dependency wavefront), lanes per body, the tail segment's threshold and
 * resident solve blocks per SM. Each candidate runs `trial_steps` steps from
 * the current state (device time by CUDA events); the state is then put back
 * exactly as it was and the fastest configuration is kept for the following
 * steps (and reported in `out`). The per-step counts the choice was made on
 * (bodies, warm-start manifolds) are reported beside it. Configurations of
 * equal lanes per body give identical results; other lane counts change the
 * order of the f32 sums within a body's update. The reference's counterpart
 * is its per-frame choice of encoded colours (src/physics/gpu/backend.js:
 * 1673-1681).
 */
typedef struct avbd_tuning {
  int32_t schedule;
  int32_t lanes_per_body;  /* 0: chosen per body                            */
  int32_t tail_div;
  int32_t blocks_per_sm;
  int32_t candidates;      /* configurations timed                          */
  int32_t trial_steps;
  double default_ms;       /* ms per step of the configuration before       */
  double best_ms;          /* ms per step of the chosen configuration       */
  int64_t bodies;
  int64_t manifolds;       /* warm-start manifold slots of the tuned state  */
} avbd_tuning;
int avbd_autotune(avbd_ctx *ctx, int32_t trial_steps, avbd_tuning *out);

/*
 * The differentiable step (forward-mode tangents through the whole AVBD
 * step; the C5 configuration's gradients). `avbd_adjoint_forward` packs
 * `world` into the context's differentiable step - its own device state, f64
 * values (the f64 engine's discrete decisions: pairs, SAT/clip topology,
 * feature-ID warm start, colouring, clamps, stick) and AVBD_TANGENT_DIMS
 * directional derivatives - seeds the inputs `seeds` name, and runs `steps`
 * steps: every contact point and basis as a function of the poses, the warm
 * start, every primal 6x6 solve and dual update of every iteration, and the
 * BDF1 velocity carry the derivatives. `avbd_adjoint_read` returns the body
 * positions (n x 3), their derivatives (n x 3 x AVBD_TANGENT_DIMS, direction
 * fastest) and the orientations (n x 4). `avbd_adjoint_backward` is the
 * vector-Jacobian product of the run: grad_params[d] = sum over bodies and
 * components of grad_pos[i][k] d pos[i][k] / d theta_d, theta_d the input of
 * direction d - the backward of a torch.autograd.Function whose forward is
 * avbd_adjoint_forward (forward mode carries every seeded direction at once,
 * so nothing is checkpointed and the backward is one contraction).
 * Independent of the context's own (FP32) state and of avbd_pack; one scene.
 * No counterpart in the reference (which has no derivatives); its rows are
 * the reference's step (src/physics/solver.js:307-493).
 */
#define AVBD_TANGENT_DIMS 5
#define AVBD_SEED_VELOCITY 0        /* initial velocity component `comp` of body `index` */
#define AVBD_SEED_FRICTION 1        /* the friction of body `index`                      */
#define AVBD_SEED_PENALTY_MAX 2     /* the penalty cap penalty_max                       */
#define AVBD_SEED_JOINT_STIFFNESS 3 /* the finite stiffnesses of joint `index`           */
typedef struct avbd_tangent_seed {
  int32_t kind;   /* AVBD_SEED_*                                           */
  int32_t index;  /* body or joint                                         */
  int32_t comp;   /* velocity component 0..2                               */
  int32_t dir;    /* direction 0..AVBD_TANGENT_DIMS-1 (seeds may share one) */
} avbd_tangent_seed;
int avbd_adjoint_forward(avbd_ctx *ctx, const avbd_world *world, int32_t steps, const avbd_tangent_seed *seeds,
                         int32_t n_seeds);
int avbd_adjoint_read(avbd_ctx *ctx, double *pos, double *dpos, double *quat);
int avbd_adjoint_backward(avbd_ctx *ctx, const double *grad_pos, double *grad_params);

/* Text of the last error on this context (or, when ctx is NULL, of the last
   failed avbd_create or context-free call). Never NULL. */
const char *avbd_last_error(const avbd_ctx *ctx);

/*
 * Allocation-free bounding-sphere overlap query. No counterpart in the
 * reference: it runs the broad phase's pair kernels (the same f64 sphere test
 * and the same pair order as a step's candidate pairs) on caller-owned device
 * buffers, without a context, and allocates nothing: no cudaMalloc, cudaFree
 * or allocating library routine. Its scratch memory (hash grid, per-body
 * partner rows, scan temporaries) is one file-scope __device__ array of
 * AVBD_STATIC_SCRATCH_BYTES (32 MiB) per device.
 *
 * For callers that must not allocate device memory once they are running:
 * frame loops with a fixed memory budget (cudaFree synchronises the whole
 * device and would stall every other stream of the frame), and hosts whose
 * device memory is reserved up front by another allocator.
 *
 *   n          bodies, 0..AVBD_STATIC_PAIRS_MAX_BODIES (65,000; the
 *              reference's per-scene body cap, src/app/scenes.js:66-75);
 *              more is rejected with AVBD_ERR_CAPACITY
 *   pos        device, n x 3 doubles (x, y, z)
 *   radius     device, n doubles (bounding radius, >= 0)
 *   dynamic    device, n int32 (0 = static; NULL = all dynamic); pairs of
 *              two static bodies are not reported
 *   cell_size  hash-grid cell edge, > 0; bodies with 2 r above it (with a
 *              1e-6 relative pad) are tested against every other body, the
 *              rest through the grid. Any value gives the same pairs; about
 *              twice the largest common radius is fastest.
 *   keys       device, capacity uint64: (a << 32) | b for each pair a > b
 *              with |p_a - p_b|^2 <= (r_a + r_b)^2, ascending
 *   count      device, one int32: the number of pairs (may exceed capacity:
 *              then keys holds an incomplete set and the call must be
 *              repeated with a larger buffer), or -1 when a position is
 *              non-finite or beyond 1e9 cells from the origin
 *   stream     a cudaStream_t (NULL = the legacy default stream)
 *
 * The results are ready when the stream reaches the end of the call. Every
 * call outside a stream capture looks up the scratch array's address
 * (cudaGetSymbolAddress, allocation-free) with the calling context current;
 * a call while its stream is being captured (the call allocates nothing, so
 * it can be captured into a CUDA graph) uses the address of the last call
 * on that device, so make one call outside the capture first, with the
 * context the graph will run in.
 * All calls on a device share the one scratch array, and every call resets
 * the parts that must start at zero: two calls whose executions overlap (on
 * different streams, or from different host threads without ordering) race
 * and corrupt each other's results. Order them on one stream or with events.
 */
#define AVBD_STATIC_PAIRS_MAX_BODIES 65000
#define AVBD_STATIC_SCRATCH_BYTES (32u << 20)
int avbd_overlap_pairs_static(int32_t n, const double *pos, const double *radius, const int32_t *dynamic,
                              double cell_size, uint64_t *keys, int64_t capacity, int32_t *count,
                              void *stream);

#ifdef __cplusplus
}
#endif

#endif /* AVBD_CUDA_H */
