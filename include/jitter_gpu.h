/*
 * jitter_gpu.h — C ABI of the GB300 contact pipeline (narrowphase, contact cache,
 * coloured sequential-impulse solve, integration) for Jitter Physics 2 worlds.
 *
 * All entry points are extern "C", take plain pointers and sizes, return an int
 * status (JG_OK = 0, negative JG_ERR_* on failure) and never throw.  The library
 * owns every device buffer; the caller passes host buffers that are copied in or
 * out.  One host thread drives one jg_world (the reference contract "a World has a
 * single external owner", docfx/docs/documentation/world.md:75-97).
 *
 * Each declaration names the reference code it replaces (paths inside the
 * Jitter2 source tree, src/Jitter2/...).
 */
#ifndef JITTER_GPU_H
#define JITTER_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------------- */
#define JG_OK                 0
#define JG_ERR_INVALID_ARG   -1  /* ArgumentException, World.Step.cs:157-165            */
#define JG_ERR_CAPACITY      -2  /* a device pool is full; grow it and retry            */
#define JG_ERR_NONFINITE     -3  /* NaN/Inf in uploaded or simulated state              */
#define JG_ERR_TIMEOUT       -4  /* a bounded device-side wait gave up                  */
#define JG_ERR_CUDA          -5  /* a CUDA runtime call failed                          */
#define JG_ERR_NOT_SUPPORTED -6  /* feature not available (e.g. no sm_103a device)     */
#define JG_ERR_INVALID_SHAPE -7  /* InvalidCollisionTypeException, World.Detect.cs:29-59 */

/* ---- enumerations mirroring the reference ---------------------------------------- */
/* MotionType, Dynamics/RigidBody.cs:75-95 */
#define JG_MOTION_DYNAMIC   0
#define JG_MOTION_KINEMATIC 1
#define JG_MOTION_STATIC    2

/* Shape kinds: BoxShape, SphereShape, CapsuleShape, CylinderShape, ConeShape,
 * PointCloudShape (VertexSupportMap), TriangleShape (files under Collision/Shapes) */
#define JG_SHAPE_BOX        0
#define JG_SHAPE_SPHERE     1
#define JG_SHAPE_CAPSULE    2
#define JG_SHAPE_CYLINDER   3
#define JG_SHAPE_CONE       4
#define JG_SHAPE_POINTCLOUD 5
#define JG_SHAPE_TRIANGLE   6

/* Body flag bits (RigidBodyData.Flags layout, Dynamics/RigidBody.cs:180-250) */
#define JG_BODY_ACTIVE            (1 << 2)
#define JG_BODY_GYROSCOPIC        (1 << 3)
#define JG_BODY_LOCKS_SHIFT       4       /* 6 bits: locked motion axes (MotionAxes ^ All) */
#define JG_BODY_NO_GRAVITY        (1 << 12)
#define JG_BODY_SPECULATIVE       (1 << 13) /* RigidBody.EnableSpeculativeContacts (RigidBody.cs:877-892) */

/* Warm start of newly created contacts (no counterpart in the reference, which
 * always starts new contacts from zero: Contact.cs:727) */
#define JG_WARMSTART_ZERO   0
#define JG_WARMSTART_CACHED 1   /* reference behaviour: new = 0, cached = previous impulse */
#define JG_WARMSTART_MLP    2   /* cached contacts as reference, new contacts from the MLP */

/* Constraint kinds (Dynamics/Constraints/BallSocket.cs, HingeAngle.cs) */
#define JG_CONSTRAINT_BALLSOCKET 1
#define JG_CONSTRAINT_HINGEANGLE 2
#define JG_CONSTRAINT_DISTANCELIMIT 3   /* Dynamics/Constraints/DistanceLimit.cs */
#define JG_CONSTRAINT_CONELIMIT 4       /* Dynamics/Constraints/ConeLimit.cs     */
#define JG_CONSTRAINT_TWISTANGLE 5      /* Dynamics/Constraints/TwistAngle.cs    */
#define JG_CONSTRAINT_FIXEDANGLE 6      /* Dynamics/Constraints/FixedAngle.cs    */
#define JG_CONSTRAINT_POINTONPLANE 7    /* Dynamics/Constraints/PointOnPlane.cs  */
#define JG_CONSTRAINT_ANGULARMOTOR 8    /* Dynamics/Constraints/AngularMotor.cs  */
#define JG_CONSTRAINT_LINEARMOTOR 9     /* Dynamics/Constraints/LinearMotor.cs   */
#define JG_CONSTRAINT_ANGULARSERVO 10   /* Dynamics/Constraints/AngularServo.cs  */
#define JG_CONSTRAINT_LINEARSERVO 11    /* Dynamics/Constraints/LinearServo.cs   */
#define JG_CONSTRAINT_LINEARAXISSERVO 12 /* Dynamics/Constraints/LinearAxisServo.cs */
#define JG_CONSTRAINT_TWISTSERVO 13     /* Dynamics/Constraints/TwistServo.cs    */
#define JG_CONSTRAINT_POINTONLINE 14    /* Dynamics/Constraints/PointOnLine.cs   */
#define JG_CONSTRAINT_ELLIPTICALCONELIMIT 15 /* Dynamics/Constraints/EllipticalConeLimit.cs */

/* ---- plain data structures ------------------------------------------------------- */

/* World settings (World.cs:333-416, World.Detect.cs:88-122). */
typedef struct jg_world_params {
    float   gravity[3];                 /* default (0,-9.81,0), World.cs:389           */
    int32_t substeps;                   /* SubstepCount, default 1                      */
    int32_t solver_iterations;          /* SolverIterations.solver, default 6, at most 4096 */
    int32_t relax_iterations;           /* SolverIterations.relaxation, default 4       */
    int32_t enable_auxiliary_contacts;  /* EnableAuxiliaryContactPoints, default 1      */
    int32_t persistent_manifold;        /* PersistentContactManifold, default 1         */
    float   speculative_relaxation;     /* SpeculativeRelaxationFactor, default 0.9     */
    int32_t edge_filter;                /* default TriangleEdgeCollisionFilter present  */
    int32_t warm_start_mode;            /* JG_WARMSTART_*                               */
    int32_t max_bodies;                 /* device pool capacities (0 = derive)          */
    int32_t max_shapes;
    int32_t max_pairs;
    int32_t max_arbiters;
    int32_t max_constraints;
    int32_t solver_block;               /* threads per CTA of the solver (0 = tuned)    */
    int32_t solver_ctas_per_sm;         /* persistent CTAs per SM (0 = tuned)           */
    int32_t narrow_tile;                /* lanes per pair in the narrowphase (32)       */
    int32_t use_graph;                  /* capture the step in a CUDA graph             */
    int32_t record_residual;            /* record the per-iteration residual (metric)   */
    int32_t deterministic;              /* sort new arbiters by key every step          */
    int32_t partitioned_solve;          /* 1 (default): spatial tasks in shared memory   */
    float   speculative_threshold;      /* SpeculativeVelocityThreshold, default 10      */
    int32_t allow_deactivation;         /* AllowDeactivation, default 1 (World.cs:333)   */
    float   sched_cells_per_sm;         /* partitioned solve: column cells per grid and SM
                                           (0 = the narrowest cells when they are no more
                                           than the solve's blocks, else about 250 arbiters
                                           per cell; the cells never get narrower than three
                                           times the widest arbiter); a speed knob only     */
} jg_world_params;

/* One rigid body: the fields of RigidBodyData (RigidBody.cs:107-250) plus the
 * per-body settings the per-step update reads (RigidBody.cs:380-409, :716-764). */
typedef struct jg_body_desc {
    float   position[3];
    float   orientation[4];             /* quaternion x,y,z,w                            */
    float   velocity[3];
    float   angular_velocity[3];
    float   delta_velocity[3];          /* DeltaVelocity queued by the last update       */
    float   delta_angular_velocity[3];  /* DeltaAngularVelocity                          */
    float   inv_inertia[6];             /* local inverse inertia M11 M12 M13 M22 M23 M33 */
    float   inv_mass;
    float   friction;                   /* default 0.2                                   */
    float   restitution;                /* default 0                                     */
    float   linear_damping;             /* multiplier, default 0.998                     */
    float   angular_damping;            /* multiplier, default 0.995                     */
    float   force[3];                   /* cleared after each step (RigidBody.cs:760)    */
    float   torque[3];
    int32_t motion_type;                /* JG_MOTION_*                                   */
    int32_t flags;                      /* JG_BODY_* bits                                */
    int32_t world;                      /* world index for batched worlds (0 otherwise)  */
} jg_body_desc;

/* One collision shape attached to a body.  The shape index in the uploaded array is
 * the reference's ShapeId order (World.Detect.cs:141-144 orders pairs by it). */
typedef struct jg_shape_desc {
    int32_t kind;                       /* JG_SHAPE_*                                    */
    int32_t body;                       /* owning body index                             */
    float   dims[4];                    /* box: half extents; sphere: r; capsule: r, half length;
                                           cylinder: r, height; cone: r, height;
                                           pointcloud: shift xyz                         */
    float   center[3];                  /* GetCenter(): point cloud centre of mass       */
    int32_t data_offset;                /* pointcloud: first vertex; triangle: triangle id */
    int32_t data_count;                 /* pointcloud: vertex count                      */
} jg_shape_desc;

/* One triangle of a TriangleMesh (Collision/Shapes/TriangleMesh.cs:194-319): mesh-local
 * vertices, unit normal and the neighbour across edges A (c-b), B (a-c), C (b-a). */
typedef struct jg_triangle_desc {
    float   a[3], b[3], c[3];
    float   normal[3];
    int32_t neighbor[3];                /* triangle ids, -1 for an open edge             */
    int32_t pad;
} jg_triangle_desc;

/* Read-only view of one cached contact point (Contact.cs:585-700). */
typedef struct jg_contact_view {
    int32_t shape1, shape2;             /* ArbiterKey (Arbiter.cs:67-103)                */
    int32_t body1, body2;
    int32_t slot;                       /* 0..3 within the ContactData                   */
    int32_t usage_mask;                 /* ContactData.UsageMask                         */
    int32_t color;                      /* solver colour of the arbiter                  */
    int32_t flags;
    float   normal[3], tangent1[3], tangent2[3];
    float   rel_pos1[3], rel_pos2[3];   /* RelativePosition1/2 (world offsets)           */
    float   pos1_local[3], pos2_local[3];
    float   accumulated[3];             /* normal, tangent1, tangent2 impulses           */
    float   mass[3];
    float   bias, penalty_bias;
    float   friction, restitution;
} jg_contact_view;

/* Per-step counters (SceneBenchmark records pairs/contacts, other/SceneBenchmark/Program.cs:64-71). */
typedef struct jg_counters {
    int64_t pairs;                      /* broadphase pairs                              */
    int64_t colliding;                  /* pairs MPR/EPA reported as colliding           */
    int64_t manifold_points;            /* contact points written by the manifold        */
    int64_t arbiters;                   /* arbiters after the step                       */
    int64_t contacts;                   /* active contact points solved (UsageMask bits) */
    int64_t new_contacts;
    int64_t colors;                     /* solver colours                                */
    int64_t epa_calls;
    int64_t epa_failures;               /* EPA fell back to MPR (NarrowPhase.cs:82-84)   */
    int64_t exact_fallbacks;            /* FP64 orientation/normal evaluations           */
    int64_t status;                     /* JG_ERR_* raised on the device, 0 if none      */
    int64_t created_arbiters;
    int64_t removed_arbiters;
    int64_t kernel_launches;            /* device kernels launched by the last step       */
    int64_t solver_tasks;               /* partitioned solve: tasks (cells) of the step   */
    int64_t task_arbiters;              /* arbiters solved in tasks (rest: global colours) */
    int64_t task_colors;                /* most local colours of one task                 */
    int64_t speculative_contacts;       /* pairs registered by the sweep (World.Detect.cs:168-196) */
} jg_counters;

/* Stage timings in milliseconds (World.DebugTimings buckets, World.Step.cs:44-81). */
typedef struct jg_timings {
    float broadphase, narrowphase, add_arbiter, coloring, solve, update_contacts,
          update_bodies, total;
} jg_timings;

typedef struct jg_world jg_world;
typedef struct jg_batch jg_batch;

/* ---- lifetime ---------------------------------------------------------------------- */

/* Fills defaults equal to a freshly constructed World (World.cs:333-416). */
int jg_default_params(jg_world_params* params);

/* new World(...) (World.cs:166-230); allocates the device pools. */
int jg_create(const jg_world_params* params, jg_world** out_world);
/* World.Dispose (World.cs:281-299). */
int jg_destroy(jg_world* world);

/* The World property setters: SolverIterations (World.cs:346-369), SubstepCount
 * (World.cs:378-391), Gravity (World.cs:397-403), EnableAuxiliaryContactPoints,
 * PersistentContactManifold, SpeculativeRelaxationFactor, SpeculativeVelocityThreshold
 * (World.Detect.cs:88-122), plus the device settings.  The reference's
 * ArgumentOutOfRangeException cases (solver iterations below one, negative relaxation
 * iterations, substeps below one, a non-finite gravity) return JG_ERR_INVALID_ARG, and so does
 * a change of the pool capacities, which are fixed at creation.  jg_get_params reads them. */
int jg_set_params(jg_world* world, const jg_world_params* params);
int jg_get_params(jg_world* world, jg_world_params* out);

/* ---- state upload / download -------------------------------------------------------- */

/* World.CreateRigidBody + RigidBody setters (World.cs:930-965, RigidBody.cs:503-760).
 * An upload with a non-finite body returns JG_ERR_NONFINITE, one with an invalid motion type
 * or world JG_ERR_INVALID_ARG (the lowest-indexed invalid body decides), and leaves the
 * world's state unchanged.  A download returns the last uploaded descriptors with the state a
 * step changes (position, orientation, velocities, delta velocities; force and torque 0). */
int jg_upload_bodies(jg_world* world, const jg_body_desc* bodies, int32_t count);
int jg_download_bodies(jg_world* world, jg_body_desc* bodies, int32_t count);

/* RigidBody.AddShape (RigidBody.cs:1440-1520); vertices for point clouds, triangles
 * for meshes.  Uploading shapes clears the contact cache. */
int jg_upload_shapes(jg_world* world, const jg_shape_desc* shapes, int32_t count,
                     const float* hull_vertices, int32_t hull_vertex_count,
                     const jg_triangle_desc* triangles, int32_t triangle_count);

/* World.ActivateBodyNextStep (World.cs:696-720), RigidBody.SetActivationState(true): the
 * body's sleep time restarts and, when it sleeps and is not static, its island joins the
 * active list at the next step.  Only matters with allow_deactivation. */
int jg_activate_body(jg_world* world, int32_t body);
/* RigidBody.DeactivationTime (RigidBody.cs:476-483, seconds, default 1) and
 * RigidBody.DeactivationThreshold (RigidBody.cs:497-508, angular and linear speeds, default
 * sqrt(0.1) each): a body whose speeds stay below the thresholds for the deactivation time
 * stops keeping its island awake.  Negative or NaN values return JG_ERR_INVALID_ARG.  An upload
 * of a different number of bodies restarts every body's sleep time. */
int jg_set_body_sleep(jg_world* world, int32_t body, float deactivation_time, float linear_threshold,
                      float angular_threshold);

/* RigidBody.Position/Orientation/Velocity setters; field: 0 position, 1 orientation,
 * 2 velocity, 3 angular velocity, 4 force, 5 torque.  Position/orientation follow
 * RigidBody.Move (RigidBody.cs:637-648): the body's contact cache is cleared. */
int jg_set_body(jg_world* world, int32_t body, int32_t field, const float* value);

/* World.CreateConstraint<T> + Initialize (BallSocket.cs:120-138, HingeAngle.cs:84-110,
 * DistanceLimit.cs:92-117, ConeLimit.cs:92-118, TwistAngle.cs:85-128, FixedAngle.cs:72-85,
 * PointOnPlane.cs:89-126, AngularMotor.cs:62-82, LinearMotor.cs:97-115, AngularServo.cs:55-77,
 * LinearServo.cs:60-73, LinearAxisServo.cs:61-78, TwistServo.cs:69-87, PointOnLine.cs:92-121,
 * EllipticalConeLimit.cs:92-126),
 * world-space init:
 *   BallSocket     anchor xyz
 *   HingeAngle     axis xyz, min, max (radians)
 *   DistanceLimit  anchor1 xyz, anchor2 xyz, min, max (offsets from the initial distance;
 *                  min >= max fixes it, LinearLimit.Fixed = (1e-6, -1e-6))
 *   ConeLimit      axis1 xyz, axis2 xyz, min, max (radians, 0 <= min <= max <= pi, not a
 *                  fixed tilt of 0 or pi)
 *   TwistAngle     axis1 xyz, axis2 xyz, min, max (radians, finite)
 *   FixedAngle     nothing read (the current relative rotation is kept)
 *   PointOnPlane   axis xyz (plane normal, fixed in body 1), anchor1 xyz, anchor2 xyz,
 *                  min, max (signed distance; min >= max fixes it)
 *   AngularMotor,  axis1 xyz, axis2 xyz, target velocity, maximum torque (force) >= 0
 *   LinearMotor
 *   AngularServo   target relative orientation xyzw (body 2 in body 1's frame, unit; all
 *                  zero = the current one), maximum torque
 *   LinearServo    anchor1 xyz, anchor2 xyz, target position xyz (body 1's frame), maximum force
 *   LinearAxisServo axis xyz (fixed in body 1), anchor1 xyz, anchor2 xyz, target position,
 *                  maximum force
 *   TwistServo     axis1 xyz, axis2 xyz, target angle (radians, in [-pi, pi]), maximum torque
 *   PointOnLine    axis xyz (the line's direction, fixed in body 1), anchor1 xyz (on the line),
 *                  anchor2 xyz, min, max (position along the line; min >= max fixes it,
 *                  LinearLimit.Fixed = (1e-6, -1e-6))
 *   EllipticalConeLimit axis1 xyz, axis2 xyz, reference xyz (body 1, not along axis1),
 *                  min1, max1 (swing along the reference), min2, max2 (across it), radians:
 *                  0 <= min <= max < pi, max > 0, min1 and min2 both zero or both positive
 * A servo's maximum is >= 0 and may be +inf; 0 (the reference's default) applies no impulse.
 * Invalid arguments return JG_ERR_INVALID_ARG (the reference's ArgumentException). */
int jg_add_constraint(jg_world* world, int32_t kind, int32_t body1, int32_t body2,
                      const float* init, int32_t* out_id);

/* A servo's target and maximum, the TargetRelativeOrientation / TargetPosition / TargetAngle and
 * MaximumTorque / MaximumForce setters (AngularServo.cs:79-98, LinearServo.cs:103-124,
 * LinearAxisServo.cs:131-152, TwistServo.cs:89-112): target is xyzw (AngularServo), xyz
 * (LinearServo) or one value (LinearAxisServo position, TwistServo angle).  A changed target
 * drops the servo's warm start; both wake its inactive dynamic bodies (ServoMath.cs:22-28). */
int jg_set_servo(jg_world* world, int32_t constraint, const float* target, float maximum);

/* A constraint's Bias, Softness, LimitBias and LimitSoftness setters (BallSocket.cs:192-222,
 * HingeAngle.cs:250-312, PointOnLine.cs:308-374, EllipticalConeLimit.cs:226-252 and the like):
 * NaN keeps a value; values are >= 0.  The limit pair exists for HingeAngle and PointOnLine only,
 * and the motors have none of the four (JG_ERR_INVALID_ARG). */
int jg_set_constraint_params(jg_world* world, int32_t constraint, float bias, float softness,
                             float limit_bias, float limit_softness);

/* ---- the step ------------------------------------------------------------------------- */

/* World.Step(dt) from DynamicTree.EnumerateOverlaps through DynamicTree.Update
 * (World.Step.cs:153-296): broadphase, narrowphase + manifold, arbiter merge,
 * colouring, substepped solve + integration, contact and body update. */
int jg_step(jg_world* world, float dt);

/* World.Stabilize (World.Step.cs:318-392): CheckDeactivation, then for each substep the
 * solve (prepare, solver_iterations iterations) and relaxation_iterations relaxation passes
 * over the contacts and constraints already present (restored with jg_import_state, for
 * example), with no collision detection and no integration of forces, velocities or
 * positions.  The reference's ArgumentException cases (dt negative or not finite, solver
 * iterations below one, negative relaxation) return JG_ERR_INVALID_ARG / JG_ERR_NONFINITE.
 * Arbiters left without contact points are dropped here rather than at the next step. */
int jg_stabilize(jg_world* world, float dt, int32_t solver_iterations, int32_t relaxation_iterations);

/* Like jg_step but with the body state taken from and returned to host buffers
 * (copies included), the call a host that keeps its own bodies makes: one copy of the array
 * each way (pinned memory copies fastest), validated as jg_upload_bodies does. */
int jg_step_host(jg_world* world, float dt, jg_body_desc* bodies, int32_t count);

/* ---- inspection ------------------------------------------------------------------------ */

/* Batched NarrowPhase.MprEpa (NarrowPhase.cs:902-927) on the world's shapes at the
 * bodies' current poses: shape_pairs holds 2*count shape indices; results receives 10
 * floats per pair (pointA xyz, pointB xyz, normal xyz, penetration, world frame, the
 * reference's out parameters) and hits the method's return value (1 colliding, 0 not).
 * Host buffers; synchronous.  Device scratch grows on demand with the largest count. */
int jg_collide_pairs(jg_world* world, const int32_t* shape_pairs, int32_t count,
                     float* results, int32_t* hits);

/* No counterpart in the reference.  jg_collide_pairs without any allocation in the call:
 * its device scratch is a fixed array of JG_COLLIDE_NOALLOC_MAX_PAIRS pairs (52 B per
 * pair, 832 KiB per device) built into the library, instead of buffers that
 * jg_collide_pairs grows with cudaMalloc.  For hosts that may not allocate device memory
 * once running: a frame loop under a fixed memory budget, or a thread that must not take
 * cudaMalloc's implicit device-wide synchronisation while other streams work.  Same
 * arguments, results and errors as jg_collide_pairs, plus JG_ERR_CAPACITY when count
 * exceeds JG_COLLIDE_NOALLOC_MAX_PAIRS (split the batch).  Every world of a device shares
 * the one scratch array: calls that overlap on the GPU (from several host threads) race
 * on it, so the caller serialises them.  Nothing in the scratch has to start at zero; the
 * kernel writes every slot of the batch.  The first call on a device looks up the
 * array's address (which loads the library's device code there): make it before any
 * stream capture.  The current device must be the world's. */
#define JG_COLLIDE_NOALLOC_MAX_PAIRS 16384
int jg_collide_pairs_noalloc(jg_world* world, const int32_t* shape_pairs, int32_t count,
                             float* results, int32_t* hits);

/* CollisionManifold.BuildManifold (CollisionManifold.cs:393-566) on the world's shapes at
 * the bodies' current poses, for given witness points: points holds 9 floats per pair
 * (pointA, pointB, normal, world frame, as NarrowPhase.MprEpa returns them); out receives
 * 24 floats per pair (up to four point pairs, A xyz then B xyz) and counts the number of
 * pairs (ManifoldCount).  The step's manifold stage runs the same device function.  Host
 * buffers; synchronous; allocates its device buffers for the call. */
int jg_manifold_pairs(jg_world* world, const int32_t* shape_pairs, int32_t count, const float* points,
                      float* results, int32_t* counts);

/* The broadphase pair list of the last step (DynamicTree.EnumerateOverlaps with the
 * default filter, DynamicTree.cs:266-286, World.cs:447-455): every shape pair with
 * non-disjoint world bounding boxes, on different bodies, at least one active and one
 * dynamic, as 2 shape indices per pair in no particular order.  Writes up to capacity
 * pairs; *out_count receives the number of pairs. */
int jg_get_pairs(jg_world* world, int32_t* pairs, int32_t capacity, int32_t* out_count);

/* Arbiter/ContactData view (World.RawData, World.cs:95-141).  Writes up to capacity
 * entries; *out_count receives the number of active contact points. */
int jg_get_contacts(jg_world* world, jg_contact_view* out, int32_t capacity, int32_t* out_count);
/* Arbiter keys created and removed during the last step (BeginCollide/EndCollide). */
int jg_get_arbiter_events(jg_world* world, int32_t* created_pairs, int32_t created_capacity,
                          int32_t* n_created, int32_t* removed_pairs, int32_t removed_capacity,
                          int32_t* n_removed);
/* Constraint state in creation order: the accumulated impulse (BallSocket.Impulse,
 * BallSocket.cs:221; HingeAngle.Impulse, HingeAngle.cs:311) as 3 floats each (the one-row
 * kinds, DistanceLimit, ConeLimit and TwistAngle, in the first of the three), and
 * the order key of the last step's solve (768 + global colour: constraints sharing a key
 * share no dynamic body). */
int jg_get_constraints(jg_world* world, int32_t* order_keys, float* impulses, int32_t capacity,
                       int32_t* out_count);
int jg_get_counters(jg_world* world, jg_counters* out);
int jg_get_timings(jg_world* world, jg_timings* out);
/* Per-iteration residual of the first substep of the last step (record_residual=1), for up
 * to the first 2048 iterations:
 * r_k = |lambda_k - lambda_{k-1}| / max(|lambda_k|, 1e-12) over all contact rows. */
int jg_get_residuals(jg_world* world, float* out, int32_t capacity, int32_t* out_count);

/* Full state dump for checkpoints and one-step comparisons (no reference counterpart;
 * World.Stabilize, World.Step.cs:318-392, re-solves restored contacts). */
int jg_export_state(jg_world* world, void* buffer, int64_t capacity, int64_t* out_size);
/* Validates the blob (jg_check_state against the world's counts and pools) before it
 * changes anything; a rejected blob leaves the world as it was. */
int jg_import_state(jg_world* world, const void* buffer, int64_t size);
/* Host-only check of a state blob for a world of n_bodies bodies and n_shapes shapes with
 * the given arbiter and constraint pools: its size covers the counts in its header, the
 * counts are not negative, and every arbiter's shapes and bodies and every constraint's
 * kind and bodies lie inside the world.  JG_ERR_INVALID_ARG (or JG_ERR_CAPACITY when
 * the counts exceed the pools) otherwise.  Needs no device. */
int jg_check_state(const void* buffer, int64_t size, int32_t n_bodies, int32_t n_shapes, int32_t arbiter_capacity,
                   int32_t constraint_capacity);

/* ---- learned warm start (no reference counterpart) ---------------------------------------- */

/* Loads MLP weights 24->64->64->3 (BF16 stored, given as float): W1[64x24], b1[64],
 * W2[64x64], b2[64], W3[3x64], b3[3], plus feature mean/scale[24] and output scale[3]. */
int jg_mlp_load(jg_world* world, const float* params, int32_t count);
/* Predicts impulses for n feature rows (24 floats each), writes 3 floats per row. */
int jg_mlp_predict(jg_world* world, const float* features, int32_t n, float* out);
/* One Adam step over a minibatch of (features, targets) held in host memory;
 * returns the mean squared error of the minibatch before the update. */
int jg_mlp_train_step(jg_world* world, const float* features, const float* targets,
                      int32_t n, float learning_rate, float* out_loss);
/* Exports the current float parameters in the jg_mlp_load layout. */
int jg_mlp_export(jg_world* world, float* params, int32_t capacity, int32_t* out_count);
/* Gradients of the minibatch MSE with respect to every parameter (jg_mlp_load layout). */
int jg_mlp_gradients(jg_world* world, const float* features, const float* targets,
                     int32_t n, float* out_grads, int32_t capacity, float* out_loss);
/* Collects (features, converged impulse) training pairs of contacts created during
 * the last step: up to capacity rows of 24 + 3 floats. */
int jg_collect_training(jg_world* world, float* features, float* targets, int32_t capacity,
                        int32_t* out_count);

/* ---- batched worlds (no reference counterpart) ---------------------------------------------- */

/* Many independent worlds stepped by one captured launch sequence.  Bodies, shapes and
 * constraints carry their world index; all worlds share params and dt.  jg_batch_step runs
 * the step as one CUDA-graph launch (captured once per arbiter-buffer parity and dt, and
 * again after uploads that change the world's shape); its timings hold only the total. */
int jg_batch_create(const jg_world_params* params, int32_t n_worlds, jg_world** out_world);
int jg_batch_step(jg_world* world, float dt);
/* Autotunes the solve for this world by timing a few steps of a copy of its state: the
 * solve's form (partitioned tasks or global colours), its launch shape (threads per CTA,
 * CTAs per SM) and, for the partitioned solve, the cell density (sched_cells_per_sm);
 * writes the chosen values into params and keeps them. */
int jg_autotune(jg_world* world, float dt, int32_t steps, jg_world_params* chosen);

/* ---- host utilities ------------------------------------------------------------------------- */

/* Shape mass properties, CalculateMassInertia of each shape (BoxShape.cs:188-199,
 * SphereShape.cs:100-111, CapsuleShape.cs:112-129, CylinderShape.cs:122-133,
 * ConeShape.cs:128-138, ShapeHelper.cs:399-412 for point clouds).  Host only. */
int jg_shape_mass_inertia(const jg_shape_desc* shape, const float* hull_vertices,
                          float* inertia6, float* com3, float* mass);

/* Last CUDA error string of this thread (static storage). */
const char* jg_last_error(void);
/* Library version string. */
const char* jg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* JITTER_GPU_H */
