/*
 * gpb.h — C ABI of the GB300-native batched rigid-body step.
 *
 * The library batches the step that gorilla-physics' `simulate` loop runs for
 * one mechanism (src/simulate.rs:20-112) over tens of thousands of independent
 * mechanisms on one GPU:
 *   - forward kinematics and world-frame twists (src/mechanism.rs:153-188,
 *     src/spatial/twist.rs:176-204),
 *   - the CRBA joint-space mass matrix (src/mechanism.rs:592-696),
 *   - point / sphere vs half-space contact forces (src/contact.rs:97-128,
 *     260-338, src/collision/halfspace.rs:39-44),
 *   - the RNEA dynamics bias (src/dynamics.rs:41-251, src/spatial/wrench.rs:96-126),
 *   - the solve for q̈ (src/dynamics.rs:255-276; Cholesky instead of LU),
 *   - semi-implicit Euler / RK2 / RK4 (src/integrators.rs:25-39,177-319).
 *
 * Conventions
 *   - Every entry point returns 0 on success or a negative GPB_E_* code.  The
 *     message of the last failure on the calling thread is gpb_last_error().
 *     Per-instance numerical faults (non-finite state, a mass matrix that is not
 *     positive definite) never abort a call: they are recorded in the per-instance
 *     status array (gpb_batch_status) and that instance is frozen.
 *   - Host buffers passed in are copied; device buffers are owned by the library.
 *   - Body / joint numbering inside one mechanism follows MechanismState
 *     (src/mechanism.rs:37-58): joint i has child body i, bodies are 1-based,
 *     body 0 is the world, and parent(i) < i.
 *   - Per-instance q and v are flattened exactly like the reference's
 *     `to_float_dvec` (src/joint/mod.rs:208-303): revolute / prismatic 1 value,
 *     floating q = [qx,qy,qz,qw,tx,ty,tz], floating v = [ωx,ωy,ωz,vx,vy,vz] in the
 *     body frame, fixed 0 values.  A batch stores instances back to back in the
 *     order they were given; gpb_batch_layout reports each instance's offsets.
 *   - One context drives one CUDA device on one stream and is used from one
 *     host thread at a time.  Several contexts may share a device.
 */
#ifndef GPB_H
#define GPB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPB_ABI_VERSION 1

/* ---- return codes ---------------------------------------------------- */
#define GPB_OK 0
#define GPB_E_INVAL (-1)   /* bad argument / malformed mechanism            */
#define GPB_E_NOMEM (-2)   /* device or host allocation failed              */
#define GPB_E_CUDA (-3)    /* a CUDA runtime call failed                    */
#define GPB_E_TIMEOUT (-4) /* a bounded device wait ran out                 */
#define GPB_E_RANGE (-5)   /* size beyond a documented limit                */
#define GPB_E_STATE (-6)   /* call not valid in the object's current state  */

/* ---- per-instance status bits (gpb_batch_status) ---------------------- */
#define GPB_ST_OK 0
#define GPB_ST_NONFINITE 1 /* q, v, q̈ or a contact force became NaN/Inf   */
#define GPB_ST_CHOL_FAIL 2 /* mass matrix not positive definite            */
#define GPB_ST_COLLISION 4 /* cuboid GJK/EPA met a case the reference panics
                              on, or ran past its loop / storage bounds   */
#define GPB_ST_SOLVER 8    /* velocity stepping: the friction-cone program
                              did not converge (the reference panics on a
                              NaN impulse)                                */

/* ---- enums ------------------------------------------------------------ */
/* Joint kinds of src/joint/mod.rs:21-27. */
enum gpb_joint_type {
  GPB_JOINT_FIXED = 0,
  GPB_JOINT_REVOLUTE = 1,
  GPB_JOINT_PRISMATIC = 2,
  GPB_JOINT_FLOATING = 3
};

/* Integrators of src/integrators.rs:17-23.  GPB_VELOCITY_STEPPING is
 * velocity_stepping (src/integrators.rs:42-51, dynamics_discrete
 * src/dynamics.rs:367-430): v_free = v + dt M⁻¹(τ − c) without contact
 * wrenches, every contact (points and spheres against half-spaces, cuboid
 * pairs) a friction cone (μ = 0.95) of the impulse program
 * min ½λᵀ(J M⁻¹ Jᵀ)λ + (J v_free)ᵀλ (src/dynamics.rs:652-742, solved on the
 * device by a primal-dual interior-point method), v' = v_free + M⁻¹Jᵀλ,
 * q' = q + dt v' (compute_new_q).  FP64 only; at most GPB_MAX_VS_CONTACTS
 * potential contacts per instance (points × half-spaces + cuboid pairs).
 * The CCD variant is not provided. */
enum gpb_integrator {
  GPB_SEMI_IMPLICIT_EULER = 0,
  GPB_RUNGE_KUTTA_2 = 1,
  GPB_RUNGE_KUTTA_4 = 2,
  GPB_VELOCITY_STEPPING = 3
};

/* GPB_FP64: every quantity in FP64 (the drop-in).  GPB_MIXED: sweeps, contact
 * and mass-matrix build in FP32; FP64 position/quaternion accumulator; FP64
 * Cholesky when n > 12.  GPB_MIXED_REFINED: bias forces, mass matrix and
 * Cholesky of one evaluation in FP32 (link coordinates), then iterative
 * refinement whose residual τ − ID(q, q̇, q̈₀) is a link-coordinate
 * Newton–Euler pass in FP64 (a second step only where the first correction
 * exceeds 1e-4 of max(|q̈|, 1)); FP64 position/quaternion accumulator. */
enum gpb_precision { GPB_FP64 = 0, GPB_MIXED = 1, GPB_MIXED_REFINED = 2 };

/* How q̈ is obtained from the dynamics (gpb_batch_set_algorithm).
 * GPB_ALGO_CRBA: the reference's route (src/dynamics.rs:322-364): RNEA bias,
 *   CRBA mass matrix (src/mechanism.rs:592-696), then a Cholesky solve where the
 *   reference uses LU.  The default.
 * GPB_ALGO_ABA: Featherstone's articulated-body algorithm in link coordinates,
 *   O(n) per instance; the same q̈ in exact arithmetic (FP64 results agree with
 *   CRBA to the conditioning bound).  With GPB_MIXED its articulated-inertia
 *   recursion, the body bias forces v ×* I v with their inward recursion and
 *   the 1-DOF q̈ solve run in double-float (pairs of FP32 numbers, about 48
 *   bits, on the FP32 pipes) from the FP32-rounded model, and so do a
 *   floating joint's 6×6 factor and solve; kinematics, velocities and bias
 *   accelerations in FP32; the state in FP64.  A contact mechanism keeps its
 *   world poses, body velocities, penetrations and contact-point velocities
 *   (with their split into approach speed and tangential velocity) in FP64,
 *   and runs the contact force law and wrench in FP32 from them.
 *   GPB_MIXED_REFINED always uses CRBA. */
enum gpb_algorithm { GPB_ALGO_CRBA = 0, GPB_ALGO_ABA = 1 };

/* GPB_HUNT_CROSSLEY: src/contact.rs:260-338 (k = k_p k_h/(k_p+k_h), k_h = 50e3,
 * π = max(λ z^1.5 ż + k z^1.5, 0), λ = 1.5 α k).
 * GPB_LINEAR_SPRING_DAMPER: π = max(k z + c ż, 0) with the same friction. */
enum gpb_contact_model { GPB_HUNT_CROSSLEY = 0, GPB_LINEAR_SPRING_DAMPER = 1 };

/* Device-side control law evaluated before every step. */
enum gpb_control {
  GPB_CONTROL_HOST_TAU = 0,    /* τ given by the caller (constant over the call) */
  GPB_CONTROL_OPEN_LOOP = 1,   /* τ ~ N(0, σ²) per DOF, resampled every R steps  */
  GPB_CONTROL_PD = 2           /* τ = kp (q* − q) − kd v on 1-DOF joints           */
};

/* ---- mechanism tables (flattened structure of arrays) ----------------- */
/*
 * All instances of a batch are described by one gpb_model.  Instance i owns
 * joints/bodies [joint_offset[i], joint_offset[i+1]), contact points
 * [contact_offset[i], contact_offset[i+1]) and half-spaces
 * [halfspace_offset[i], halfspace_offset[i+1]).
 *
 * joint_type[j]     gpb_joint_type
 * joint_parent[j]   parent body number within the instance (0 = world), < own number
 * joint_iso[7j..]   init_iso of the joint: quaternion (qx,qy,qz,qw) then translation
 *                   (transform from the child body frame to the parent frame,
 *                   src/joint/revolute.rs:18-19)
 * joint_axis[3j..]  unit axis in the child frame (revolute / prismatic)
 * joint_spring[2j..] prismatic spring (k, rest length); k == 0 means no spring
 *                   (src/joint/prismatic.rs:12-16, src/dynamics.rs:298-315)
 * body_inertia[10j..] mass, cross_part (m·com, 3), moment about the frame origin
 *                   (Jxx, Jyy, Jzz, Jxy, Jxz, Jyz)  (src/inertia.rs:31-37)
 * contact_body[c]   body number (1-based) the point is fixed to
 * contact_params[6c..] location in the body frame (3), k, radius, damping.
 *                   radius 0 is the reference ContactPoint (src/contact.rs:16-21);
 *                   radius > 0 is a sphere: penetration r − d, applied at the
 *                   sphere point nearest the half-space.
 * halfspace_params[8h..] point (3), outward unit normal (3), alpha, mu
 *                   (src/collision/halfspace.rs:6-11)
 * contact_model[i]  gpb_contact_model of instance i
 * joint_armature[j] reflected rotor inertia of a revolute joint, added to its
 *                   diagonal of the mass matrix (src/joint/revolute.rs:29,
 *                   src/hybrid/articulated/mod.rs:244-247); NULL = none.  The
 *                   reference's continuous path has no such term, so leave it
 *                   NULL for parity with dynamics_continuous.
 * body_cuboid[3j..] cuboid collider of body j centred on its frame and aligned
 *                   with it (Cuboid::new_at_center(w, d, h) in
 *                   RigidBody::add_cuboid_collider, src/rigid_body.rs:197-199;
 *                   the pose follows the body, src/mechanism.rs:257-275):
 *                   w, d, h along x, y, z; all zero (or NULL) = no collider.
 *                   Every pair of cuboid bodies (i < j) is tested with GJK/EPA
 *                   and pushed apart by the collider contact law
 *                   (src/contact.rs:191-242,306-317).  At most GPB_MAX_CUBOIDS
 *                   cuboids per instance.
 */
typedef struct gpb_model {
  int64_t n_instances;
  const int32_t* joint_offset;     /* [n_instances + 1] */
  const int32_t* joint_type;
  const int32_t* joint_parent;
  const double* joint_iso;
  const double* joint_axis;
  const double* joint_spring;
  const double* body_inertia;
  const int32_t* contact_offset;   /* [n_instances + 1] */
  const int32_t* contact_body;
  const double* contact_params;
  const int32_t* halfspace_offset; /* [n_instances + 1] */
  const double* halfspace_params;
  const int32_t* contact_model;    /* [n_instances] */
  const double* joint_armature;    /* [n_joints] or NULL */
  const double* body_cuboid;       /* [3 n_joints] or NULL */
} gpb_model;

/* Limits of one instance. */
#define GPB_MAX_BODIES 64
#define GPB_MAX_DOF 64
#define GPB_MAX_CONTACTS 64
#define GPB_MAX_HALFSPACES 4
#define GPB_MAX_CUBOIDS 8
#define GPB_MAX_VS_CONTACTS 16

/* ---- library / context ------------------------------------------------ */
typedef struct gpb_ctx gpb_ctx;
typedef struct gpb_batch gpb_batch;

int gpb_abi_version(void);
const char* gpb_last_error(void);

/* Creates a context on CUDA device `device` with its own stream. */
int gpb_create(int device, gpb_ctx** out);
int gpb_destroy(gpb_ctx* ctx);

/* ---- batches ----------------------------------------------------------- */
/*
 * Validates and uploads the mechanisms of `model` (one per instance), builds
 * the structure-of-arrays topology tables and allocates per-instance state
 * (initially q = joint zero / identity pose, v = 0, like MechanismState::new,
 * src/mechanism.rs:62-148).  Replaces MechanismState::new for a whole slice.
 */
int gpb_batch_create(gpb_ctx* ctx, const gpb_model* model, gpb_batch** out);
int gpb_batch_destroy(gpb_batch* batch);

/* Per-instance offsets into the flattened q / v vectors ([n+1] each) and the
 * totals.  Any pointer may be NULL. */
int gpb_batch_layout(const gpb_batch* batch, int64_t* q_offset, int64_t* v_offset,
                     int64_t* nq_total, int64_t* nv_total);

/* Replaces MechanismState::update(q, v) (src/mechanism.rs:209-214) for every
 * instance: q and v hold nq_total / nv_total doubles. */
int gpb_set_state(gpb_batch* batch, const double* q, const double* v);
int gpb_get_state(gpb_batch* batch, double* q, double* v);

/* ---- the hot path ------------------------------------------------------ */
/*
 * dynamics_continuous (src/dynamics.rs:322-364) for every instance at its
 * current state: writes q̈ (nv_total doubles) and, if `contact_force` is not
 * NULL, the world-frame force of every contact point (3 per point, summed over
 * half-spaces).  `tau` (nv_total doubles) may be NULL for zero torque
 * (src/simulate.rs:26-37).
 */
int gpb_dynamics(gpb_batch* batch, const double* tau, int precision, double* qdd,
                 double* contact_force);

/*
 * gpb_dynamics_static — no counterpart in the reference.
 *
 * The same q̈ as gpb_dynamics, for callers that cannot allocate device memory
 * when they evaluate the dynamics (a hard real-time control loop, or a host
 * that owns the GPU through its own memory pool and forbids cudaMalloc once
 * running).  Nothing is allocated or freed: q (nq_total), v (nv_total), tau
 * (nv_total, or NULL for zero torque) and qdd (nv_total) are the caller's
 * DEVICE buffers in the flattened user order, and the kernel's working memory
 * is a fixed array of GPB_STATIC_SCRATCH_BYTES compiled into the library — each
 * GPU that loads the library holds it until the process exits.  A batch whose
 * scratch needs more (about 32 KB per instance of a 48-DOF chain, 1 KB for an
 * acrobot) is rejected with GPB_E_RANGE.
 *
 * The kernel runs asynchronously on `stream` (a cudaStream_t; NULL = the
 * batch's context stream); read qdd after synchronising that stream.  The first
 * call on a device looks up the array's device address, so make that first call
 * before any stream capture.  The address is kept for the life of the process:
 * do not call this entry point again on a device after cudaDeviceReset (or any
 * other teardown of that device's primary context).  All calls share the one
 * array: calls whose kernels overlap on the GPU race, so order them on one
 * stream.  No state is carried from one call to the next.
 *
 * The kernel also ORs its per-instance status bits into the batch's status
 * array (gpb_batch_status), on `stream`.  Every other entry point of the batch
 * works on the context stream, so with a non-NULL `stream` the caller must
 * order the two: synchronise `stream` before gpb_batch_status,
 * gpb_batch_clear_status, gpb_step or gpb_simulate on the same batch, and do not
 * let this call overlap one of those.
 *
 * q, v, qdd (and tau when not NULL) must be device (or managed) memory: a host
 * pointer is rejected with GPB_E_INVAL before anything is launched.
 */
#define GPB_STATIC_SCRATCH_BYTES (16u << 20)
int gpb_dynamics_static(gpb_batch* batch, const double* q, const double* v, const double* tau,
                        int precision, double* qdd, void* stream);

/*
 * CollisionDetector::new(A, B) followed by gjk() and epa()
 * (src/collision/mod.rs:48-87; gjk.rs:14-125; epa.rs:108-254) for n
 * independent pairs of cuboids, one GPU thread per pair.  pose_a / pose_b: 7
 * doubles per pair (unit quaternion qx, qy, qz, qw, then the centre tx, ty,
 * tz); size_a / size_b: (w, d, h) per pair.  result[i]: 1 = in collision, with
 * cp_a / cp_b the contact points on A and on B (3 doubles each; cp_b − cp_a is
 * the penetration, from A into B); 0 = no collision (cp = 0); -1 = a case where
 * the reference panics (degenerate simplex, face or edge); -2 = the query ran
 * past the kernel's storage bounds (more than 48 polytope vertices, 160
 * faces, 32 horizon edges or 64 GJK iterations).  The decisions and the
 * contact points are computed in the reference's order of operations with
 * IEEE rounding.
 * gpb_collide_cuboids takes host buffers and returns when the results are
 * written.  gpb_collide_cuboids_device takes device buffers and only enqueues
 * the kernel on `stream` (NULL = the context's stream).
 */
int gpb_collide_cuboids(gpb_ctx* ctx, int64_t n, const double* pose_a, const double* size_a,
                        const double* pose_b, const double* size_b, int32_t* result, double* cp_a,
                        double* cp_b);
int gpb_collide_cuboids_device(gpb_ctx* ctx, int64_t n, const double* pose_a, const double* size_a,
                               const double* pose_b, const double* size_b, int32_t* result,
                               double* cp_a, double* cp_b, void* stream);

/*
 * step (src/simulate.rs:20-83) for every instance: one integrator step of
 * size dt with joint torques `tau` (NULL = zero).  State stays on the device.
 */
int gpb_step(gpb_batch* batch, double dt, const double* tau, int integrator,
             int precision);

/* Device-side control for gpb_simulate. */
typedef struct gpb_control_params {
  int32_t mode;          /* gpb_control */
  uint32_t seed;         /* OPEN_LOOP: stream seed (Philox4x32-10 key word 1) */
  int32_t resample_every;/* OPEN_LOOP: steps between torque draws (≥ 1) */
  double sigma;          /* OPEN_LOOP: standard deviation of τ */
  double kp, kd;         /* PD gains */
  const double* tau;     /* HOST_TAU: nv_total doubles (NULL = zero);
                            PD: per-DOF target q* (nv_total doubles, only the
                            1-DOF joints are used) */
} gpb_control_params;

/*
 * K steps of `simulate` (src/simulate.rs:87-112) for every instance, with the
 * control law evaluated on the device each step.  The step counter `step0` is
 * the global index of the first step (it keys the open-loop torque draws, so a
 * horizon split over several calls draws the same torques).  If `history` is not
 * NULL, q and v after every `record_every`-th step are written to it as
 * [K / record_every][nq_total + nv_total] doubles.
 */
int gpb_simulate(gpb_batch* batch, double dt, int64_t K, int64_t step0,
                 int integrator, int precision, const gpb_control_params* control,
                 int64_t record_every, double* history);

/* Step count of the reference loop `while t < final_time { …; t += dt }`
 * (src/simulate.rs:97-109), float accumulation included. */
int64_t gpb_simulate_steps(double final_time, double dt);

/* Per-instance status words (GPB_ST_* bits), n_instances int32. */
int gpb_batch_status(gpb_batch* batch, int32_t* status);
/* Clears all status words (e.g. after the caller repaired the state). */
int gpb_batch_clear_status(gpb_batch* batch);
/* Steps each instance completed in the last gpb_simulate / gpb_step call
 * (fewer than K for an instance frozen by a status bit), n_instances int64. */
int gpb_batch_steps_done(gpb_batch* batch, int64_t* steps);

/* Waits for all work of the context's stream. */
int gpb_synchronize(gpb_ctx* ctx);

/* ---- kernel mapping ---------------------------------------------------- */
/* One lane steps one instance (a warp steps a pack of 32, the default); for
 * the CRBA route the four warps of a block may share one pack
 * (gpb_batch_set_coop); and a batch of serial chains may give each instance
 * several lanes (gpb_batch_set_mapping).  gpb_batch_autotune picks among them. */

/* Lanes per instance of later GPB_FP64 and GPB_MIXED gpb_simulate / gpb_step
 * calls (velocity stepping excepted): 1 = one lane per instance (the
 * default);
 * 2, 4, 8, 16 or 32 = the body-parallel mapping, where that many lanes of a
 * warp step one instance (32 = one warp per instance, 2 = sixteen instances
 * per warp), each lane owning one or two consecutive bodies; 128 = the same
 * with a 4-warp block per instance (one body per thread, the warps' scan
 * totals combined in shared memory, a block barrier per Cholesky column): the outward and
 * inward sweeps are prefix and suffix scans across the lanes by warp
 * shuffles, and the mass matrix and its Cholesky factor sit in shared memory
 * with their entries dealt to the lanes.  It shortens one instance's step by
 * up to the lane count and pays off when the batch has too few instances to
 * fill the GPU one lane each.  Only for a batch whose every instance is a
 * serial chain (joint k's parent is body k) of revolute, prismatic or fixed
 * joints without cuboid colliders, with at most 2 × lanes bodies; else
 * GPB_E_INVAL.  The mapping builds and factors the mass matrix (the CRBA route)
 * in FP64 whatever gpb_batch_set_algorithm chose (which then selects the
 * one-lane route only) and for GPB_MIXED requests too; its results agree
 * with the one-lane FP64 forms to rounding (the sums run in another order).
 * GPB_MIXED_REFINED keeps one lane per instance. */
int gpb_batch_set_mapping(gpb_batch* batch, int lanes_per_instance);

/* Resident warps per SM of the persistent step kernel (one warp per pack of
 * 32 instances): 0 = as many as the kernel's registers allow (the default),
 * else a multiple of 4 up to 64, capped by that limit.  With 4, each of the
 * SM's four schedulers (each with its own FP64 unit) runs one pack at a time. */
int gpb_batch_set_launch(gpb_batch* batch, int warps_per_sm);

/* Packs whose every instance has at least `min_dof` DOF are stepped by a whole
 * 4-warp block (one warp per scheduler): warp 0 runs the sweeps, the four
 * warps share the mass-matrix fill and the Cholesky factorisation.  Results
 * are bit-identical to the one-warp path; large mechanisms finish sooner, which
 * shortens the critical path of a batch with a wide size range.  -1 = the
 * library's default, 0 = off.  Not used by GPB_MIXED_REFINED. */
int gpb_batch_set_coop(gpb_batch* batch, int min_dof);

/* GPB_ALGO_CRBA (default) or GPB_ALGO_ABA for every later dynamics call. */
int gpb_batch_set_algorithm(gpb_batch* batch, int algorithm);

/* Gravitational acceleration along −z for every later call (default 9.81,
 * src/lib.rs:39; 0 switches gravity off as Articulated::free_velocity's
 * gravity_enabled = false does). */
int gpb_batch_set_gravity(gpb_batch* batch, double g);

/*
 * Articulated::free_velocity (src/hybrid/articulated/mod.rs:124-199) for every
 * instance: v + dt · M⁻¹ (τ − c(q, v)) with the armature on the mass matrix's
 * diagonal and the batch's gravity; no contact points and no prismatic springs
 * (the hybrid engine handles contact itself).  tau: nv_total doubles or NULL;
 * v_free: nv_total doubles in the user order.
 */
int gpb_free_velocity(gpb_batch* batch, double dt, const double* tau, int precision, double* v_free);

/* Autotuner: times `trial_steps` steps of this batch (its own mechanisms,
 * state, step size, integrator, precision and control law) for each launch
 * shape (one lane per instance at 4, 8, 12 or 16 resident warps per SM, as
 * many as the step kernel's registers allow; block-cooperative packs off or
 * from 32 / 40 DOF when the batch has such packs; for GPB_FP64 and GPB_MIXED
 * on a chain batch, the body-parallel mapping at the lane counts that give
 * each lane one or two bodies), keeps the fastest with gpb_batch_set_launch /
 * gpb_batch_set_coop / gpb_batch_set_mapping and reports it (warps_per_sm 0
 * for a body-parallel pick).  The batch's q, v, torques and status words are
 * restored afterwards.  The one-lane shapes compute the same bits; the
 * body-parallel mapping agrees with them to rounding.  Any output pointer may
 * be NULL. */
int gpb_batch_autotune(gpb_batch* batch, double dt, int integrator, int precision,
                       const gpb_control_params* control, int trial_steps, int* warps_per_sm,
                       int* coop_min_dof, int* lanes_per_instance);

/* Number of this library's kernel launches issued by the context so far. */
int64_t gpb_launch_count(const gpb_ctx* ctx);

/* Device time (ms, CUDA events on the context's stream) of the last
 * gpb_simulate / gpb_step kernel; waits for it.  −1 if none ran. */
double gpb_last_launch_ms(gpb_ctx* ctx);

/* ---- synthetic configurations ------------------------------------------ */
/*
 * Seeded builders of the benchmark mechanisms (all draws from Philox4x32-10
 * keyed by (instance, seed)):
 *   0  acrobot: 2 revolute links about y, lengths 1 and 2 m, 1 kg, rod inertia
 *   1  serial revolute chain, n ~ U{2..48}, axes U{x,y,z}, l ~ U(0.2,1), m ~ U(0.5,2)
 *   2  free-floating cube, side U(0.2,1) m, 1000 kg/m³, 8 corner contacts, μ ~ U(0.3,1)
 *   3  quadruped: floating 0.6×0.3×0.15 m torso (10 kg), 4 legs × 3 revolute
 *      joints, 0.25 m / 1 kg links, foot spheres r = 0.02 m
 * gpb_config_sizes returns the table sizes; gpb_config_build fills caller-owned
 * arrays laid out as gpb_model (offsets included) plus the initial q / v and,
 * for config 3, the per-DOF PD targets (`aux`, nv doubles; may be NULL).
 * `contact_model` selects the normal-force law for configs 2 and 3.
 */
int gpb_config_sizes(int config, int64_t n_instances, uint32_t seed, int64_t* n_joints,
                     int64_t* n_contacts, int64_t* n_halfspaces, int64_t* nq, int64_t* nv);
int gpb_config_build(int config, int64_t n_instances, uint32_t seed, int contact_model,
                     int32_t* joint_offset, int32_t* joint_type, int32_t* joint_parent,
                     double* joint_iso, double* joint_axis, double* joint_spring,
                     double* body_inertia, int32_t* contact_offset, int32_t* contact_body,
                     double* contact_params, int32_t* halfspace_offset,
                     double* halfspace_params, int32_t* contact_model_out, double* q0,
                     double* v0, double* aux);

/* The open-loop torque draw for (seed, instance, draw block, dof): the value
 * the device uses, exported so that callers can replay a horizon. */
double gpb_open_loop_tau(uint32_t seed, int64_t instance, int64_t block, int32_t dof,
                         double sigma);

/* ---- serving ------------------------------------------------------------ */
/*
 * No reference counterpart: the reference steps one MechanismState per call
 * (src/simulate.rs:20-112).  A server keeps a pool of lane slots resident on
 * one GPU and runs every admitted request in ticks of at most chunk_steps
 * steps (continuous batching: requests join and leave between ticks, each
 * with its own step size, horizon, integrator and control law).  A request's
 * trajectory does not depend on what else is in the pool: it equals the same
 * request run alone, bit for bit.
 *
 * The pool is divided into slot classes (capacities in bodies, q, v, contacts,
 * half-spaces, and whether the class takes planar chains only).  Each request
 * goes to the smallest class it fits (planar-only classes first for a planar
 * chain); it waits in
 * a FIFO queue until that class has a free slot (the admission limit is the
 * HBM budget the pool was sized to).  A server is single-threaded like its
 * context.
 */
typedef struct gpb_server gpb_server;

typedef struct gpb_slot_class {
  int32_t max_bodies, max_q, max_v, max_contacts, max_halfspaces;
  double weight;  /* share of the budget left after the fixed classes; 0 = fixed */
  int32_t packs;  /* packs of 32 slots of a fixed class (weight 0) */
  int32_t chunk_steps; /* steps per tick of this class's requests (0 = the server's) */
  int32_t max_cuboids; /* cuboid colliders per instance (0..GPB_MAX_CUBOIDS) */
  int32_t planar_only; /* 1: only planar chains (revolute joints about ±x/±y/±z with
                          identity joint rotations, each body the child of the previous,
                          no contacts, colliders or springs); its packs run the
                          articulated-body passes specialised for them.  A planar chain
                          goes to the smallest planar-only class it fits, else to the
                          smallest other class. */
} gpb_slot_class;

typedef struct gpb_server_opts {
  int32_t precision;          /* GPB_FP64, GPB_MIXED or GPB_MIXED_REFINED */
  int32_t chunk_steps;        /* steps per tick, >= 1 */
  int64_t hbm_budget_bytes;   /* device bytes of the pool (weighted classes) */
  int32_t n_classes;          /* 1..16 */
  const gpb_slot_class* classes;
  int32_t max_admit_per_tick; /* 0 = no limit */
  int32_t algorithm;          /* GPB_ALGO_CRBA or GPB_ALGO_ABA */
} gpb_server_opts;

typedef struct gpb_request {
  double dt;
  int64_t steps;            /* horizon K >= 1 */
  int32_t integrator;       /* GPB_SEMI_IMPLICIT_EULER … */
  int32_t control;          /* GPB_CONTROL_* */
  uint32_t seed;            /* open-loop draw seed */
  int32_t resample_every;
  double sigma, kp, kd;
  int32_t key;              /* instance number of the open-loop draw (0 = as a batch of one) */
} gpb_request;

/* steps: instance-steps run so far (exact for retired requests, counted from
 * the chunks launched for running ones). */
typedef struct gpb_server_stats {
  int64_t pending, active, completed, slots, ticks, pool_bytes, steps;
} gpb_server_stats;

/* Host-only sizing: device bytes of one pack of each class and the packs each
 * class gets under opts (weighted share of the budget, or its `packs`). */
int gpb_server_plan(const gpb_server_opts* opts, int32_t* packs_per_class, int64_t* bytes_per_pack);
int gpb_server_create(gpb_ctx* ctx, const gpb_server_opts* opts, gpb_server** out);
int gpb_server_destroy(gpb_server* server);
/* Queues instances first..first+count-1 of m as `count` requests.  q, v (and
 * tau: host torques for GPB_CONTROL_HOST_TAU, PD targets for GPB_CONTROL_PD,
 * or NULL) hold those instances' values concatenated in instance order, as
 * gpb_set_state lays them out.  The server copies everything it needs.
 * ids receives `count` request ids.  GPB_E_RANGE if an instance fits no class. */
int gpb_server_submit(gpb_server* server, const gpb_model* m, int64_t first, int64_t count,
                      const double* q, const double* v, const double* tau,
                      const gpb_request* requests, uint64_t* ids);
/* One tick: admit queued requests into free slots, run ≤ chunk_steps steps of
 * every active request, retire the finished ones.  *completed (nullable) =
 * requests that finished in this tick. */
int gpb_server_tick(gpb_server* server, int32_t* completed);
/* Drains up to `max` ids of finished requests not yet listed. */
int gpb_server_completed(gpb_server* server, uint64_t* ids, int32_t max, int32_t* count);
/* Final q, v (nq / nv doubles), status (GPB_ST_* bits), steps run and the
 * seconds from submission to retirement of a finished request, then forgets
 * it.  GPB_E_STATE if the request has not finished. */
int gpb_server_result(gpb_server* server, uint64_t id, double* q, double* v, int32_t* status,
                      int64_t* steps_done, double* latency_s);
/* Forgets the results of finished requests without reading them. */
int gpb_server_forget(gpb_server* server, const uint64_t* ids, int64_t count);
int gpb_server_stats_get(const gpb_server* server, gpb_server_stats* stats);

/* ---- measurement ------------------------------------------------------- */
/* FMA throughput of the FP64 (GPB_FP64) or FP32 (GPB_MIXED) pipe in TFLOP/s,
 * counting 2 flops per fused multiply-add of the `active_lanes` (1..32) lanes
 * of each warp that issue: the roofline denominator of the batched step. */
int gpb_fma_peak(int device, int precision, int active_lanes, double* tflops);
/* FP32 → FP64 conversion throughput (G conversions/s, all lanes active): on
 * GB300 conversions share the FP64 unit's rate, which decides how a mixed form
 * splits its work. */
int gpb_cvt_peak(int device, double* gops);

#ifdef __cplusplus
}
#endif

#endif /* GPB_H */
