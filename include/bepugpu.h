/*
 * bepugpu.h -- C ABI of the GB300 velocity solver and integration step for
 * BEPUphysics v1 scenes.
 *
 * The library replaces three stages of the reference's Space pipeline:
 *   ForceUpdater     BEPUphysics/OtherSpaceStages/ForceUpdater.cs:73-92
 *   Solver           BEPUphysics/Constraints/Solver.cs:239-314
 *   PositionUpdater  BEPUphysics/PositionUpdating/ContinuousPositionUpdater.cs:134-154
 * and, for frozen manifold sets, the manifold refresh rule of
 *   ContactRefresher BEPUphysics/CollisionTests/ContactRefresher.cs:18-69.
 *
 * Every function returns a bepugpu_status.  No C++ exception and no CUDA
 * error crosses the ABI; bepugpu_last_error() gives the message of the last
 * failing call on a context.  Host arrays passed in are borrowed for the
 * duration of the call only.  All device memory is owned by the context.
 *
 * Threading: one context is driven by one host thread at a time, like the
 * reference's stage contract (MultithreadedProcessingStage.Update is called
 * from one thread).  The serving entry points (bepugpu_server_*) are the
 * exception: submit and poll may be called from different threads.
 */
#ifndef BEPUGPU_H
#define BEPUGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BEPUGPU_ABI_VERSION 12
#define BEPUGPU_MAX_CONTACTS 4

typedef enum bepugpu_status {
    BEPUGPU_OK = 0,
    BEPUGPU_INVALID_ARGUMENT = 1,   /* reference: ArgumentException (Solver.cs:109,142) */
    BEPUGPU_OUT_OF_MEMORY = 2,
    BEPUGPU_ADMISSION_REFUSED = 3,  /* serving: scene does not fit the device budget */
    BEPUGPU_CUDA_ERROR = 4,
    BEPUGPU_TIMEOUT = 5,            /* a bounded device-side wait ran out */
    BEPUGPU_NAN_DETECTED = 6,
    BEPUGPU_NOT_FOUND = 7,
    BEPUGPU_QUEUE_FULL = 8,
    BEPUGPU_INVALID_OPERATION = 9   /* reference: InvalidOperationException, e.g.
                                       "Cannot constrain two kinematic bodies"
                                       (BallSocketJoint.cs:253) */
} bepugpu_status;

/* Global and per-solver settings.  Each field names the reference setting it
 * mirrors; bepugpu_default_settings() fills the reference defaults. */
typedef struct bepugpu_settings {
    float gravity[3];                      /* ForceUpdater.Gravity (Space default 0,-9.81,0 in the configs) */
    int32_t iteration_limit;               /* Solver.IterationLimit, Solver.cs:15 (10) */
    float minimum_impulse;                 /* SolverSettings.DefaultMinimumImpulse, SolverSettings.cs:62 (.001) */
    int32_t minimum_iteration_count;       /* SolverSettings.DefaultMinimumIterationCount, :70 (1) */
    int32_t maximum_iteration_count;       /* SolverSettings.maximumIterationCount, :15 (int.MaxValue) */
    float softness;                        /* CollisionResponseSettings.Softness, :43 (.001) */
    float penetration_recovery_stiffness;  /* CollisionResponseSettings, :24 (.2) */
    float maximum_penetration_recovery_speed; /* CollisionResponseSettings, :18 (2) */
    float static_friction_velocity_threshold; /* CollisionResponseSettings, :31 (.2) */
    float twist_friction_factor;           /* CollisionResponseSettings, :37 (1) */
    float bounciness_velocity_threshold;   /* CollisionResponseSettings, :12 (1) */
    float allowed_penetration;             /* CollisionDetectionSettings.AllowedPenetration, :74 (.01) */
    float contact_invalidation_length_squared; /* CollisionDetectionSettings, :11 (.01) */
    float maximum_contact_distance;        /* CollisionDetectionSettings, :82 (.1) */
    int32_t use_stabilization;             /* DeactivationManager.UseStabilization,
                                              DeactivationManager.cs:60,67 (1): the force update's
                                              low-velocity damping boost, EntityBase.cs:926-936 */
    float velocity_lower_limit;            /* DeactivationManager.VelocityLowerLimit, :18,28 (.26) */
    float low_velocity_time_minimum;       /* DeactivationManager.LowVelocityTimeMinimum, :20,46 (1) */
    int32_t maximum_deactivation_attempts_per_frame; /* DeactivationManager, :15,89 (100): members of
                                              the islands DeactivateObjects looks at in one step
                                              (scenes with bepugpu_set_islands) */
} bepugpu_settings;

/* Body activity flags: the state of the entity's SimulationIslandMember
 * (DeactivationManagement/SimulationIslandMember.cs) that the step reads and
 * writes.  0 is the reference's default for a new entity. */
#define BEPUGPU_BODY_ALWAYS_ACTIVE        1u  /* IsAlwaysActive (:284-297) */
#define BEPUGPU_BODY_NO_STABILIZATION     2u  /* AllowStabilization = false (:305-315; default true) */
#define BEPUGPU_BODY_SLOWING              4u  /* isSlowing (:19), written by the candidacy update */
#define BEPUGPU_BODY_DEACTIVATION_CANDIDATE 8u /* IsDeactivationCandidate (:171-190), written likewise */

/* One rigid body, as the C# shim reads it from an Entity (EntityBase.cs:35-43,
 * 303-347, 1164-1165) and its activity information.  Kinematic bodies have
 * is_dynamic = 0; their inverse mass and inverse inertia are ignored by the
 * solver, as in the reference.  A kinematic body takes part in the position
 * update while it is active: velocity_time_below_limit <= 0
 * (SimulationIslandMember.IsActive, :225-248).  Every dynamic body's island is
 * awake: the library does not put islands to sleep. */
typedef struct bepugpu_body {
    float position[3];
    float orientation[4];            /* quaternion x, y, z, w */
    float linear_velocity[3];
    float angular_velocity[3];
    float inverse_mass;
    float local_inverse_inertia[9];  /* row-major M11 M12 M13 M21 ... M33 */
    float linear_damping;            /* Entity.LinearDamping (.03) */
    float angular_damping;           /* Entity.AngularDamping (.15) */
    int32_t is_dynamic;
    uint32_t activity;               /* BEPUGPU_BODY_*, in/out */
    float previous_velocity;         /* SimulationIslandMember.previousVelocity (:17), in/out */
    float velocity_time_below_limit; /* SimulationIslandMember.velocityTimeBelowLimit (:18), in/out */
} bepugpu_body;

/* One contact of a manifold (Contact.cs:15-31) together with the
 * ContactSupplementData the refresher reads, the warm-start impulse of its
 * ContactPenetrationConstraint (ContactPenetrationConstraint.cs:21) and, in a
 * NONCONVEX manifold, the state of its ContactFrictionConstraint
 * (ContactFrictionConstraint.cs:49-58: accumulatedImpulse, and linearA, the
 * friction direction a contact keeps while its sliding velocity is zero). */
typedef struct bepugpu_contact {
    float position[3];
    float normal[3];
    float penetration_depth;
    int32_t id;
    float local_offset_a[3];         /* ContactSupplementData.LocalOffsetA */
    float local_offset_b[3];         /* ContactSupplementData.LocalOffsetB */
    float base_penetration_depth;    /* ContactSupplementData.BasePenetrationDepth */
    float penetration_impulse;       /* accumulated impulse, in/out */
    float friction_impulse;          /* NONCONVEX: ContactFrictionConstraint.accumulatedImpulse, in/out */
    float friction_direction[3];     /* NONCONVEX: ContactFrictionConstraint.linearA, in/out */
} bepugpu_contact;

/* Manifold flags. */
#define BEPUGPU_MANIFOLD_ACTIVE      1u  /* SolverUpdateable.IsActive */
#define BEPUGPU_MANIFOLD_SOLVER_RULE 2u  /* pair collision rule < CollisionRule.NoSolver */
/* The narrow phase regenerates this manifold's contacts every step from the
 * two bodies' shapes (bepugpu_upload_shapes), as the reference's pair handlers
 * do: BoxContactManifold.cs:122-196 for two boxes, BoxSphereContactManifold.cs
 * for a box (body_a) and a sphere (body_b), SphereContactManifold.cs for two
 * spheres.  Contacts are matched to the previous step's by id; matched
 * contacts keep their warm-start impulse, new ones start at zero.  The
 * refresher skips such manifolds. */
#define BEPUGPU_MANIFOLD_GENERATED   4u
/* The manifold is a NonConvexContactManifoldConstraint
 * (NonConvexContactManifoldConstraint.cs:12-216): each contact's penetration
 * constraint, in contact-add order, then each contact's
 * ContactFrictionConstraint (ContactFrictionConstraint.cs:95-299) in the same
 * order; no sliding or twist friction (their record fields stay zero).  The
 * reference builds these for sphere-sphere and box-sphere pairs
 * (SpherePairHandler.cs:28, BoxSpherePairHandler.cs:28) and for mesh and
 * terrain pairs.  Without the flag a manifold is a
 * ConvexContactManifoldConstraint. */
#define BEPUGPU_MANIFOLD_NONCONVEX   8u

/* One ContactManifoldConstraint.  Convex (ConvexContactManifoldConstraint.cs:12-212):
 * up to four penetration children in contact-add order, then one
 * SlidingFrictionTwoAxis and one TwistFrictionConstraint.  NONCONVEX: up to
 * four penetration children, then one ContactFrictionConstraint per contact. */
typedef struct bepugpu_manifold {
    int32_t body_a;                  /* index into the body array, -1 = no entity */
    int32_t body_b;
    int32_t contact_count;           /* 0..4 */
    uint32_t flags;                  /* BEPUGPU_MANIFOLD_* */
    float kinetic_friction;          /* InteractionProperties (MaterialManager.cs:77-85) */
    float static_friction;
    float bounciness;
    float sliding_impulse[2];        /* SlidingFrictionTwoAxis.accumulatedImpulse, in/out */
    float sliding_axis[3];           /* SlidingFrictionTwoAxis.linearA row 1, kept between
                                        steps (SlidingFrictionTwoAxis.cs:341-366), in/out */
    float twist_impulse;             /* TwistFrictionConstraint.accumulatedImpulse, in/out */
    int32_t contact_order;           /* GENERATED manifolds: the order of the manifold's own contact
                                        list (ContactManifold.contacts, which removes by moving its
                                        last entry into the gap) as 2-bit indices into contacts[],
                                        entry i in bits 2i..2i+1, xor 0xE4 -- so 0 means the list is
                                        in solver order.  Other manifolds: 0.  In/out. */
    bepugpu_contact contacts[BEPUGPU_MAX_CONTACTS];
} bepugpu_manifold;

/* Two-body joints.  A joint record is one SolverUpdateable of the solver list;
 * a REVOLUTE record is the SolverGroup RevoluteJoint (RevoluteJoint.cs:46-95)
 * with its BallSocketJoint, RevoluteAngularJoint and RevoluteLimit children
 * solved in that order (its RevoluteMotor is inactive and not carried). */
typedef enum bepugpu_joint_type {
    BEPUGPU_JOINT_BALL_SOCKET = 1,      /* BallSocketJoint.cs:210-372 */
    BEPUGPU_JOINT_REVOLUTE_ANGULAR = 2, /* RevoluteAngularJoint.cs:226-365 */
    BEPUGPU_JOINT_SWING_LIMIT = 3,      /* SwingLimit.cs:211-347 */
    BEPUGPU_JOINT_REVOLUTE_LIMIT = 4,   /* RevoluteLimit.cs:285-649 */
    BEPUGPU_JOINT_REVOLUTE = 5,         /* RevoluteJoint group: ball socket + angular + limit */
    BEPUGPU_JOINT_NO_ROTATION = 6,      /* NoRotationJoint.cs:160-262 */
    BEPUGPU_JOINT_WELD = 7,             /* WeldJoint group: ball socket + no rotation (WeldJoint.cs:15-55) */
    BEPUGPU_JOINT_DISTANCE = 8,         /* DistanceJoint.cs:226-380 */
    BEPUGPU_JOINT_DISTANCE_LIMIT = 9,   /* DistanceLimit.cs:260-457 */
    BEPUGPU_JOINT_POINT_ON_PLANE = 10,  /* PointOnPlaneJoint.cs:212-330 */
    BEPUGPU_JOINT_TWIST = 11,           /* TwistJoint.cs:204-365 */
    BEPUGPU_JOINT_POINT_ON_LINE = 12,   /* PointOnLineJoint.cs:247-463 */
    BEPUGPU_JOINT_PRISMATIC = 13,       /* PrismaticJoint group: point on line + no rotation */
    BEPUGPU_JOINT_LINE_SLIDER = 14,     /* LineSliderJoint group: point on line + revolute angular */
    BEPUGPU_JOINT_UNIVERSAL = 15,       /* UniversalJoint group: ball socket + twist */
    BEPUGPU_JOINT_TWIST_LIMIT = 16,     /* TwistLimit.cs:200-383 */
    BEPUGPU_JOINT_LINEAR_AXIS_LIMIT = 17, /* LinearAxisLimit.cs:290-466 */
    BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT = 18, /* EllipseSwingLimit.cs:162-357 */
    BEPUGPU_JOINT_SWIVEL_HINGE_ANGULAR = 19, /* SwivelHingeAngularJoint.cs:193-287 */
    BEPUGPU_JOINT_SWIVEL_HINGE = 20,    /* SwivelHingeJoint group: ball socket + swivel hinge angular */
    BEPUGPU_JOINT_REVOLUTE_MOTOR = 21,  /* RevoluteMotor.cs:243-340 */
    BEPUGPU_JOINT_TWIST_MOTOR = 22,     /* TwistMotor.cs:182-253 */
    BEPUGPU_JOINT_LINEAR_AXIS_MOTOR = 23, /* LinearAxisMotor.cs:244-390 */
    BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED = 24, /* MaximumLinearSpeedConstraint (SingleEntity/MaximumLinearVelocityConstraint.cs:138-199) */
    BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED = 25, /* MaximumAngularSpeedConstraint (SingleEntity/MaximumAngularVelocityConstraint.cs:138-199) */
    BEPUGPU_JOINT_PLANE_SLIDER = 26,    /* PlaneSliderJoint group: point on plane (POINT_ON_PLANE's fields) */
    BEPUGPU_JOINT_ANGULAR_MOTOR = 27,   /* AngularMotor.cs:203-326 */
    BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR = 28, /* SingleEntityAngularMotor.cs:117-226: body_b -1, ANGULAR_MOTOR's fields */
    BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR = 29 /* SingleEntityLinearMotor.cs:180-276: body_b -1 */
} bepugpu_joint_type;
/* A group record holds the group's first children: REVOLUTE its ball socket,
 * angular joint and limit; PRISMATIC and LINE_SLIDER their point on line,
 * angular joint and limit; UNIVERSAL its ball socket and twist joint;
 * SWIVEL_HINGE its ball socket and swivel hinge angular joint; PLANE_SLIDER
 * its point on plane joint.  The limits of REVOLUTE, PRISMATIC and LINE_SLIDER
 * records (a LinearAxisLimit on the line's anchors and direction for the last
 * two) follow BEPUGPU_JOINT_LIMIT_ACTIVE.  The group's other children -- its
 * motors, UniversalJoint's twist limit, SwivelHingeJoint's hinge and twist
 * limits, PlaneSliderJoint's two limits -- are records of their own type
 * (REVOLUTE_MOTOR, TWIST_MOTOR, LINEAR_AXIS_MOTOR, TWIST_LIMIT, REVOLUTE_LIMIT,
 * LINEAR_AXIS_LIMIT) flagged BEPUGPU_JOINT_GROUP_CONTINUATION, right after the
 * group record (and its earlier continuations) in the joint list, with the
 * group's two bodies, in the order the group adds its children
 * (RevoluteJoint.cs:88-91, UniversalJoint.cs:54-57, PrismaticJoint.cs:57-60,
 * LineSliderJoint.cs:55-58, SwivelHingeJoint.cs:96-101,
 * PlaneSliderJoint.cs:64-68).  A child the group leaves inactive (as the
 * constructors leave the motors and these limits) is simply not listed: an
 * inactive child takes no part in the group's steps.  A continuation is solved
 * inside its group's visit, after the group's earlier children, and counts
 * toward the group's activity; it is active when both its own ACTIVE flag and
 * the group's are set.  Allowed: REVOLUTE: REVOLUTE_MOTOR; PRISMATIC and
 * LINE_SLIDER: LINEAR_AXIS_MOTOR; UNIVERSAL: TWIST_LIMIT, TWIST_MOTOR;
 * SWIVEL_HINGE: REVOLUTE_LIMIT, REVOLUTE_MOTOR, TWIST_LIMIT, TWIST_MOTOR;
 * PLANE_SLIDER: LINEAR_AXIS_LIMIT, LINEAR_AXIS_MOTOR; at most four a group. */

#define BEPUGPU_JOINT_ACTIVE        1u  /* SolverUpdateable.IsActive of the joint (or group) */
#define BEPUGPU_JOINT_LIMIT_ACTIVE  2u  /* REVOLUTE, PRISMATIC, LINE_SLIDER: the group's Limit.IsActive */
#define BEPUGPU_JOINT_SERVO         4u  /* motors: MotorMode.Servomechanism (else VelocityMotor) */
#define BEPUGPU_JOINT_GROUP_CONTINUATION 8u /* a further child of the group record before it (see above) */

/* Joint record: the state each reference object keeps between steps.  Body -1
 * is TwoEntityConstraint.WorldEntity (TwoEntityConstraint.cs:17): a kinematic
 * entity at the origin with identity orientation and zero velocity.
 *   anchor_a/b        BallSocketJoint.localAnchorA/B (BALL_SOCKET, REVOLUTE, WELD),
 *                     DistanceJoint / DistanceLimit.localAnchorA/B (DISTANCE, DISTANCE_LIMIT),
 *                     PointOnPlaneJoint.localPlaneAnchor / localPointAnchor (POINT_ON_PLANE),
 *                     PointOnLineJoint.localAxisAnchor / localPoint (POINT_ON_LINE, PRISMATIC, LINE_SLIDER),
 *                     LinearAxisLimit.localAnchorA/B (LINEAR_AXIS_LIMIT; the groups' limits take the line's)
 *   axis_a/b          RevoluteAngularJoint.localAxisA/B (REVOLUTE_ANGULAR, REVOLUTE),
 *                     SwingLimit.localAxisA/B (SWING_LIMIT), TwistJoint.localAxisA/B (TWIST),
 *                     PointOnPlaneJoint.localPlaneNormal (axis_a, POINT_ON_PLANE),
 *                     TwistLimit basis A / basis B local primary axes (TWIST_LIMIT),
 *                     EllipseSwingLimit basis primary / localTwistAxisB (ELLIPSE_SWING_LIMIT),
 *                     SwivelHingeAngularJoint.localHingeAxis (A) / localTwistAxis (B)
 *                     (SWIVEL_HINGE_ANGULAR, SWIVEL_HINGE)
 *   constrained_1/2   RevoluteAngularJoint.localConstrainedAxis1/2, in A's frame;
 *                     TwistJoint.aLocalAxisY / aLocalAxisZ (TWIST, UNIVERSAL);
 *                     TwistLimit basis A local x / y axes (TWIST_LIMIT), EllipseSwingLimit
 *                     basis x / y axes (ELLIPSE_SWING_LIMIT)
 *   basis_primary/x   RevoluteLimit.Basis localPrimaryAxis / localXAxis, in A's frame;
 *                     basis_x: TwistJoint.bLocalAxisY (TWIST, UNIVERSAL), TwistLimit basis B
 *                     local x axis (TWIST_LIMIT); basis_primary: LinearAxisLimit.localAxis
 *                     (LINEAR_AXIS_LIMIT);
 *                     PointOnLineJoint: basis_primary localLineDirection, basis_x / test_axis
 *                     localRestrictedAxis1 / 2 (POINT_ON_LINE, PRISMATIC, LINE_SLIDER)
 *   test_axis         RevoluteLimit.localTestAxis, in B's frame
 *   limit_min         RevoluteLimit.minimumAngle; SwingLimit.minimumCosine;
 *                     DistanceJoint.Distance; DistanceLimit.MinimumLength;
 *                     TwistLimit.MinimumAngle (the setter's wrap applied at upload);
 *                     LinearAxisLimit.Minimum (LINEAR_AXIS_LIMIT, PRISMATIC, LINE_SLIDER);
 *                     EllipseSwingLimit.MaximumAngleX (its setter's clamp applied at upload)
 *   limit_max         RevoluteLimit.maximumAngle; DistanceLimit.MaximumLength;
 *                     TwistLimit.MaximumAngle; LinearAxisLimit.Maximum;
 *                     EllipseSwingLimit.MaximumAngleY
 *   orientation_a/b   NoRotationJoint.InitialOrientationA/B (NO_ROTATION, WELD), quaternions x y z w
 *   margin, bounciness, bounce_velocity_threshold   JointLimit fields (0.005, 0, 1)
 *   max_corrective_velocity   Joint.MaxCorrectiveVelocity (FLT_MAX = unlimited)
 *   spring_stiffness/damping  SpringSettings (600000, 90000)
 * The last three apply to every child of a REVOLUTE record.
 *   impulse           accumulated impulses, in/out: BALL_SOCKET [0..2];
 *                     REVOLUTE_ANGULAR [0..1]; SWING_LIMIT [0]; REVOLUTE_LIMIT [0..1];
 *                     REVOLUTE [0..2] ball socket, [3..4] angular, [5..6] limit;
 *                     NO_ROTATION [0..2]; WELD [0..2] ball socket, [3..5] no rotation;
 *                     DISTANCE [0]; DISTANCE_LIMIT [0]; POINT_ON_PLANE [0]; TWIST [0];
 *                     POINT_ON_LINE [0..1]; PRISMATIC [0..1] point on line, [2..4] no rotation,
 *                     [5] limit; LINE_SLIDER [0..1] point on line, [2..3] angular, [4] limit;
 *                     UNIVERSAL [0..2] ball socket, [3] twist; TWIST_LIMIT [0], and [1] the
 *                     error its last Update left (the sign of the next jacobian follows it,
 *                     TwistLimit.cs:284-312); LINEAR_AXIS_LIMIT [0]; ELLIPSE_SWING_LIMIT [0];
 *                     SWIVEL_HINGE_ANGULAR [0]; SWIVEL_HINGE [0..2] ball socket, [3] angular;
 *                     the motors [0].
 * Motors (REVOLUTE_MOTOR, TWIST_MOTOR, LINEAR_AXIS_MOTOR) take their axes as the
 * limit of the same kind does (REVOLUTE_LIMIT's basis and test axis, TWIST_LIMIT's
 * bases, LINEAR_AXIS_LIMIT's anchors and axis) and their MotorSettings1D from:
 *   limit_min  servo goal          limit_max  velocity motor goal velocity
 *   margin     velocity motor softness (default 0.0001)
 *   bounciness servo base corrective speed (0)
 *   bounce_velocity_threshold  maximum force (FLT_MAX)
 *   max_corrective_velocity    servo max corrective velocity
 *   spring_stiffness/damping   servo spring settings
 *   flags & BEPUGPU_JOINT_SERVO  servomechanism mode.
 * The single-entity speed limits (MAXIMUM_LINEAR_SPEED, MAXIMUM_ANGULAR_SPEED) act on
 * body_a; body_b must be -1.  limit_min = MaximumSpeed, limit_max = MaximumForce
 * (FLT_MAX = unlimited), margin = Softness (0.00001); impulse [0..2] is the
 * accumulated impulse of the current step (no warm start: it starts from zero).
 * An ANGULAR_MOTOR takes its basis from axis_a (primary), constrained_1 (x) and
 * constrained_2 (y) in A's frame, the servo goal (a relative orientation) from
 * orientation_a, the velocity goal (in the basis) from anchor_a, its other
 * MotorSettings as the 1-D motors do; impulse [0..2].  A SINGLE_ENTITY_LINEAR_MOTOR
 * drives the point anchor_a (body_a's frame) at the velocity axis_a or, as a
 * servo, towards the world point anchor_b; impulse [0..2], and [3] the used
 * softness it keeps while the point sits at its goal (SingleEntityLinearMotor.cs:214-241).
 * axis_a/b and constrained_1/2 of a LINE_SLIDER are its RevoluteAngularJoint's;
 * orientation_a/b of a PRISMATIC its NoRotationJoint's. */
typedef struct bepugpu_joint {
    int32_t type;                    /* bepugpu_joint_type */
    int32_t body_a;
    int32_t body_b;
    uint32_t flags;                  /* BEPUGPU_JOINT_* */
    float anchor_a[3];
    float anchor_b[3];
    float axis_a[3];
    float axis_b[3];
    float constrained_1[3];
    float constrained_2[3];
    float basis_primary[3];
    float basis_x[3];
    float test_axis[3];
    float limit_min;
    float limit_max;
    float margin;
    float bounciness;
    float bounce_velocity_threshold;
    float max_corrective_velocity;
    float spring_stiffness;
    float spring_damping;
    float impulse[8];
    float orientation_a[4];
    float orientation_b[4];
} bepugpu_joint;

typedef struct bepugpu_context bepugpu_context;

/* Step flags: which stages bepugpu_step runs. */
#define BEPUGPU_STEP_REFRESH_CONTACTS 1u  /* ContactRefresher on every manifold */
#define BEPUGPU_STEP_FORCES           2u  /* ForceUpdater */
#define BEPUGPU_STEP_SOLVE            4u  /* Solver */
#define BEPUGPU_STEP_POSITIONS        8u  /* PositionUpdater (Discrete) */
#define BEPUGPU_STEP_COLLIDE         16u  /* narrow phase of GENERATED manifolds (NarrowPhase) */
#define BEPUGPU_STEP_DEACTIVATION    32u  /* DeactivationManager.Update's per-member part: every
                                             body's UpdateDeactivationCandidacy
                                             (SimulationIslandMember.cs:53-164), before the forces */
#define BEPUGPU_STEP_ALL              63u

/* Collision shapes, one per body, for the narrow phase. */
#define BEPUGPU_SHAPE_NONE   0
#define BEPUGPU_SHAPE_BOX    1  /* BoxShape.cs: size = HalfWidth, HalfHeight, HalfLength */
#define BEPUGPU_SHAPE_SPHERE 2  /* SphereShape.cs: size[0] = Radius (its collision margin) */
typedef struct bepugpu_shape {
    int32_t type;                    /* BEPUGPU_SHAPE_* */
    float size[3];
} bepugpu_shape;

/* Solve strategies for the one-scene path. */
#define BEPUGPU_MODE_GRAPH      0  /* one launch per colour sweep, captured in a CUDA graph */
#define BEPUGPU_MODE_PERSISTENT 1  /* one cooperative launch, bounded grid barrier per colour */

int32_t bepugpu_abi_version(void);
/* sizeof of the record types, so a binding can check its marshalling:
 * kind 0 settings, 1 body, 2 contact, 3 manifold, 4 joint, 5 body state,
 * 6 manifold state. */
uint32_t bepugpu_record_size(int32_t kind);
void bepugpu_default_settings(bepugpu_settings* out);

bepugpu_status bepugpu_create(int32_t device, const bepugpu_settings* settings,
                              bepugpu_context** out);
void bepugpu_destroy(bepugpu_context* ctx);
const char* bepugpu_last_error(bepugpu_context* ctx);
bepugpu_status bepugpu_set_settings(bepugpu_context* ctx, const bepugpu_settings* settings);
bepugpu_status bepugpu_synchronize(bepugpu_context* ctx);
/* Device memory of the context's scenes: `reserved` the slabs mapped for them,
 * `in_use` the arena and staging blocks of resident scenes.  Slabs that no
 * scene uses go back to the device when their last scene goes, unless a
 * server is live (it keeps them for restores). */
bepugpu_status bepugpu_memory_usage(bepugpu_context* ctx, uint64_t* reserved, uint64_t* in_use);

/* Scenes.  A scene is one Space's body set and solver list.  Capacities are
 * fixed at creation; uploads may use any count up to them. */
bepugpu_status bepugpu_scene_create(bepugpu_context* ctx, uint32_t max_bodies,
                                    uint32_t max_manifolds, uint32_t max_joints,
                                    int32_t* scene_out);
bepugpu_status bepugpu_scene_destroy(bepugpu_context* ctx, int32_t scene);

/* Uploads copy host records to the device.  bepugpu_upload_constraints sets the
 * solver list -- joints first, then manifolds, in array order, the order the
 * reference's Solver.Add calls would have produced -- and colours it. */
bepugpu_status bepugpu_upload_bodies(bepugpu_context* ctx, int32_t scene,
                                     const bepugpu_body* bodies, uint32_t count);
bepugpu_status bepugpu_upload_constraints(bepugpu_context* ctx, int32_t scene,
                                          const bepugpu_manifold* manifolds, uint32_t manifold_count,
                                          const bepugpu_joint* joints, uint32_t joint_count);
/* One shape per body, centred on the body's position and turned with its
 * orientation (a convex entity's collidable, ConvexCollidable.UpdateWorldTransform).
 * Box sizes and sphere radii must be positive and finite.  A GENERATED manifold
 * needs both bodies shaped (box-box, box-sphere with the box as body_a, or
 * sphere-sphere); bepugpu_upload_constraints checks it. */
bepugpu_status bepugpu_upload_shapes(bepugpu_context* ctx, int32_t scene, const bepugpu_shape* shapes,
                                     uint32_t count);

/* Broad phase (the pair set the reference's DynamicHierarchy reports,
 * BroadPhaseSystems/Hierarchies/DynamicHierarchy.cs): every pair of shaped
 * bodies whose bounding boxes overlap, from the bodies' current state.  A
 * body's box is its shape's (BoxShape.GetBoundingBox, BoxShape.cs:149-174;
 * SphereShape.GetBoundingBox, SphereShape.cs:75-86) expanded by its linear
 * velocity times dt (EntityCollidable.ExpandBoundingBox,
 * EntityCollidable.cs:195-216, discrete bodies; dt = 0: no expansion); boxes
 * overlap as BoundingBox.Intersects (BoundingBox.cs:58-66) has it; two
 * kinematic bodies make no pair (the default kinematic group's NoBroadPhase
 * rule, CollisionRules.cs:177); bodies of shape NONE take no part.  Pairs are
 * written as (lower index, higher index) in ascending order, at most
 * max_pairs of them (2 int32 each); *pair_count receives how many there are,
 * which may exceed max_pairs.  Needs bepugpu_upload_shapes.  The hierarchy's
 * own traversal order is not reproduced.  Allocates device buffers on first
 * use and when the pair count grows. */
bepugpu_status bepugpu_broad_phase(bepugpu_context* ctx, int32_t scene, float dt, int32_t* pairs,
                                   uint32_t max_pairs, uint32_t* pair_count);
/* Simulation islands (DeactivationManagement/SimulationIsland.cs,
 * DeactivationManager.cs): the host's island partition and list order, after
 * which steps put islands to sleep and skip their work as the reference's
 * DeactivationManager does.  island_of_body[i] is body i's index in the
 * island list (`islands` entries): >= 0 for every dynamic body, -1 for
 * kinematic ones; every island needs a member, and every constraint's dynamic
 * bodies share one island (a SimulationIslandConnection's members do; merging
 * and splitting islands stays with the host, DeactivationManager.cs:345-700).
 * island_flags[k]: BEPUGPU_ISLAND_* of island k.  deactivation_index is
 * DeactivationManager.deactivationIslandIndex, the island DeactivateObjects
 * looked at last.  Body records are the member list in order
 * (DeactivationManager.simulationIslandMembers).
 *
 * With islands set, BEPUGPU_STEP_DEACTIVATION runs DeactivationManager.Update
 * minus the splits (DeactivationManager.cs:216-224) before the other stages:
 * each member's UpdateDeactivationCandidacy in member order
 * (SimulationIslandMember.cs:53-164; an island woken by an active kinematic
 * body is active, and not allowed to deactivate at its next attempt, from that
 * kinematic member on), then DeactivateObjects (:310-336): from the island
 * after deactivation_index, round robin, TryToDeactivate
 * (SimulationIsland.cs:94-118) on islands until their members add up to
 * maximum_deactivation_attempts_per_frame or every island was looked at.  The
 * connections of a kinematic body are its joints and its manifolds with
 * contacts.  A dynamic body is then active when its island is: the force and
 * position updates skip inactive bodies (ForceUpdater.cs:73-76,
 * ContinuousPositionUpdater.cs:71), a constraint with no active dynamic body
 * is not active in the solver (SolverUpdateable.cs:202-219,
 * ContactManifoldConstraint.cs:125-141) and keeps its impulses, and a manifold
 * neither of whose bodies is active is not refreshed or regenerated
 * (NarrowPhase.cs:300-332; world-anchored ends count as inactive).
 *
 * bepugpu_upload_bodies and bepugpu_upload_constraints clear the islands (the
 * scene is stepped with every island awake until they are set again); so does
 * islands = 0.  Batch and serve take scenes with islands into their batched
 * launches while no kinematic body can wake an island, else step them one
 * at a time. */
#define BEPUGPU_ISLAND_ACTIVE             1u  /* SimulationIsland.isActive */
#define BEPUGPU_ISLAND_ALLOW_DEACTIVATION 2u  /* SimulationIsland.allowDeactivation (default true) */
bepugpu_status bepugpu_set_islands(bepugpu_context* ctx, int32_t scene, const int32_t* island_of_body,
                                   uint32_t body_count, const uint32_t* island_flags, uint32_t islands,
                                   int32_t deactivation_index);
/* The islands' flags and the deactivation index as the last step left them
 * (synchronises the scene's stream). */
bepugpu_status bepugpu_get_islands(bepugpu_context* ctx, int32_t scene, uint32_t* island_flags,
                                   uint32_t islands, int32_t* deactivation_index);

/* The narrow phase's pair bookkeeping on the device (NarrowPhase.cs:143-178
 * adds a pair handler for a new overlap, :254-332 drops one whose bounding
 * boxes stopped overlapping), for scenes whose constraints are all GENERATED
 * manifolds: bepugpu_update_pairs runs the broad phase (as
 * bepugpu_broad_phase) and makes the manifold list follow its pair set with
 * no host round trip.  The records of pairs still reported keep their
 * contacts, impulses and relative order; records of pairs that ended go;
 * each new pair gets an empty GENERATED record after them, in ascending pair
 * order -- ACTIVE | SOLVER_RULE, the box first in a box-sphere pair,
 * NONCONVEX when a sphere takes part, the two bodies' materials blended by
 * product (MaterialManager.cs:77-85) -- exactly the records a host that
 * downloaded, diffed and uploaded them with bepugpu_upload_constraints would
 * give.  The list is then coloured on the device with the same colouring
 * (greedy in list order), and every manifold goes to the colour-sweep path;
 * islands are cleared.  Needs bepugpu_upload_shapes and bepugpu_set_materials
 * (three floats a body: kinetic friction, static friction, bounciness).
 * *manifold_count receives the new record count; more pairs than the scene's
 * manifold capacity return BEPUGPU_INVALID_OPERATION with nothing changed. */
bepugpu_status bepugpu_set_materials(bepugpu_context* ctx, int32_t scene, const float* materials, uint32_t count);
bepugpu_status bepugpu_update_pairs(bepugpu_context* ctx, int32_t scene, float dt, uint32_t* manifold_count);

/* Rewrites manifold records in place without recolouring.  Body pairs and the
 * manifold count must be those of the last bepugpu_upload_constraints (checked
 * on the device before anything changes; INVALID_ARGUMENT otherwise). */
bepugpu_status bepugpu_update_manifolds(bepugpu_context* ctx, int32_t scene,
                                        const bepugpu_manifold* manifolds, uint32_t count);

/* Per-step body update: only position, orientation and velocities may differ
 * from the last bepugpu_upload_bodies (mass, inertia, damping and the dynamic
 * flag are checked on the device before anything changes; INVALID_ARGUMENT
 * otherwise).  The world inverse inertia follows the new orientation as on
 * upload.  No reference counterpart: the reference's entities are the state. */
bepugpu_status bepugpu_update_bodies(bepugpu_context* ctx, int32_t scene, const bepugpu_body* bodies,
                                     uint32_t count);

/* One step on host records in one call, for scenes without joints: the
 * bodies' state and the manifold records go up and are checked on the device
 * as bepugpu_update_bodies / bepugpu_update_manifolds check them (nothing
 * changes when one is refused), the scene steps with `flags`, and whole body
 * and manifold records come back into the same arrays, as the downloads write
 * them.  Two host synchronisations per call instead of one per stage. */
bepugpu_status bepugpu_step_host(bepugpu_context* ctx, int32_t scene, bepugpu_body* bodies, uint32_t body_count,
                                 bepugpu_manifold* manifolds, uint32_t manifold_count, float dt, uint32_t flags);

/* The per-step state of a body: the fields a step reads and writes
 * (Entity position, orientation, linear and angular velocity,
 * EntityBase.cs:35-43, and the SimulationIslandMember activity fields). */
typedef struct bepugpu_body_state {
    float position[3];
    float orientation[4];
    float linear_velocity[3];
    float angular_velocity[3];
    uint32_t activity;
    float previous_velocity;
    float velocity_time_below_limit;
} bepugpu_body_state;

/* The per-step result of a manifold: its contacts' ids and warm-start
 * impulses in the solver's contact order (the penetration constraints'
 * accumulatedImpulse, ContactPenetrationConstraint.cs:21), the sliding and
 * twist friction impulses and the sliding axis (SlidingFrictionTwoAxis.cs,
 * TwistFrictionConstraint.cs) of a convex manifold, and the contacts'
 * friction impulses (ContactFrictionConstraint.accumulatedImpulse) of a
 * NONCONVEX one.  Contact slots at and above contact_count are zero; the
 * NONCONVEX friction directions stay on the device (whole-record downloads
 * carry them). */
typedef struct bepugpu_manifold_state {
    int32_t contact_count;
    int32_t contact_id[4];
    float penetration_impulse[4];
    float sliding_impulse[2];
    float twist_impulse;
    float sliding_axis[3];
    float friction_impulse[4];
    int32_t reserved;
} bepugpu_manifold_state;

/* One step on state records, for a C# host that keeps its records on the
 * host and steps every frame: `bodies` (all of the scene's bodies, in upload
 * order) goes up as the new position, orientation, velocities and activity,
 * the scene steps with `flags`, and the stepped state comes back into the same
 * array.  `manifolds` receives each manifold's state in upload order
 * (manifold_count = the scene's count), or nothing (manifold_count = 0).
 * Everything else -- masses, inertia, damping, the manifold set and its
 * contacts, joints -- stays as the last uploads and the device's own steps
 * left it, so a step moves 64 bytes a body each way and 80 bytes a manifold
 * down, against whole records in bepugpu_step_host.  One host
 * synchronisation.  No reference counterpart: the reference's stages share
 * the entities' memory. */
bepugpu_status bepugpu_step_state(bepugpu_context* ctx, int32_t scene, bepugpu_body_state* bodies,
                                  uint32_t body_count, bepugpu_manifold_state* manifolds, uint32_t manifold_count,
                                  float dt, uint32_t flags);
/* The scene's current body and manifold state without stepping (either
 * count may be 0 to skip that part; otherwise it must be the scene's). */
bepugpu_status bepugpu_download_state(bepugpu_context* ctx, int32_t scene, bepugpu_body_state* bodies,
                                      uint32_t body_count, bepugpu_manifold_state* manifolds,
                                      uint32_t manifold_count);

/* Checks every body's position, orientation and velocities for NaN or
 * infinity (the reference's CHECKMATH validation, Toolbox.Validate, off there
 * by default): NAN_DETECTED with *first_bad set to the lowest such body, else
 * OK with *first_bad = -1.  Waits for the scene's work. */
bepugpu_status bepugpu_check_finite(bepugpu_context* ctx, int32_t scene, int32_t* first_bad);

/* Self-test of the bounded device waits the persistent kernel's grid barrier
 * uses: one thread waits on a device flag that nothing sets, giving up after
 * `spin_limit` polls (64 ns apart) and writing TIMEOUT to a status word the
 * host reads.  Returns that status (TIMEOUT when the wait ran out); the
 * context stays usable.  No reference counterpart. */
bepugpu_status bepugpu_probe_bounded_wait(bepugpu_context* ctx, uint32_t spin_limit);

/* Self-test of the device's float results of the reference's double-precision
 * expressions, which the step computes in double-float FP32 arithmetic and
 * falls back to FP64 only where that cannot decide the rounding:
 * kind 0 (float)(1 / Math.Sqrt(a)) (Vector3.Normalize, Vector3.cs:575-581;
 * Quaternion.Normalize), kind 1 (float)(Math.Sqrt(a) / b) (the stabilization
 * boost, EntityBase.cs:931), kind 2 (float)Math.Pow(a, b) (the damping
 * factors, EntityBase.cs:943,952).  `out` receives n results; `fast` (optional)
 * how many the FP32 path decided.  Allocates device memory for the call.  No
 * reference counterpart. */
bepugpu_status bepugpu_probe_double_rounding(bepugpu_context* ctx, int32_t kind, const float* a, const float* b,
                                             uint32_t n, float* out, uint32_t* fast);

/* Writes whole body records: the fields as last uploaded, with position,
 * orientation and velocities as they are now (one copy of the scene's device
 * copy of the records). */
bepugpu_status bepugpu_download_bodies(bepugpu_context* ctx, int32_t scene,
                                       bepugpu_body* bodies, uint32_t count);
/* Writes whole manifold records, in upload order: the uploaded fields as they
 * were, the state (contacts after refresh, accumulated impulses, sliding axis)
 * as it is now, unused contact slots and `reserved` zero.  Joint records get
 * their accumulated impulses written. */
bepugpu_status bepugpu_download_constraints(bepugpu_context* ctx, int32_t scene,
                                            bepugpu_manifold* manifolds, uint32_t manifold_count,
                                            bepugpu_joint* joints, uint32_t joint_count);

/* Colouring of the solver list: colour per updateable (joints first, then
 * manifolds) and the colour-sorted order the sweeps use.  Reading it is how the
 * oracle's colour-order run is set up. */
bepugpu_status bepugpu_get_colouring(bepugpu_context* ctx, int32_t scene,
                                     int32_t* colour, int32_t* order, uint32_t count,
                                     uint32_t* colour_count);

/* The same colouring on host arrays, without a device: body_a/body_b of each
 * updateable (-1 = none) and is_dynamic per body.  No context is needed. */
bepugpu_status bepugpu_colour_list(const int32_t* body_a, const int32_t* body_b, uint32_t count,
                                   const uint8_t* is_dynamic, uint32_t body_count,
                                   int32_t* colour, int32_t* order, uint32_t* colour_count);

/* Stages.  bepugpu_step runs the flagged stages as one device sequence:
 * refresh -> ForceUpdater -> Solver (prestep, warm start, iterations) ->
 * PositionUpdater.  dt = TimeStepSettings.TimeStepDuration. */
bepugpu_status bepugpu_step(bepugpu_context* ctx, int32_t scene, float dt, uint32_t flags);
bepugpu_status bepugpu_set_solve_mode(bepugpu_context* ctx, int32_t scene, int32_t mode);
/* Island groups.  An island (dynamic bodies connected through constraints)
 * with at most max_bodies bodies and max_manifolds manifolds runs its whole
 * step inside one CTA with its bodies in shared memory; small islands are
 * packed together up to target_manifolds per CTA.  Islands holding joints,
 * larger islands and enabled = 0 use the colour-sweep path.  threads = 0 lets
 * the plan choose the CTA size (else a multiple of 32 up to 256).  Takes
 * effect at the next bepugpu_upload_constraints.  Defaults: 1, 1024, 4096,
 * 64, 0. */
bepugpu_status bepugpu_set_group_policy(bepugpu_context* ctx, int32_t scene, int32_t enabled, int32_t max_bodies,
                                        int32_t max_manifolds, int32_t target_manifolds, int32_t threads);

/* Shared-memory residency threshold of island groups: a group whose bodies and
 * solve lanes need at most `bytes` (96 per body + 400 per manifold) keeps its
 * solve lanes in shared memory; larger groups keep them in global memory.
 * 0 keeps every group's lanes in global memory.  At most 200 KiB (default).
 * Takes effect at the next bepugpu_upload_constraints. */
bepugpu_status bepugpu_set_group_smem_budget(bepugpu_context* ctx, int32_t scene, uint32_t bytes);

/* Where island groups run the first stages of their step (the contact
 * refresh, the candidacy and force updates of their bodies, the manifolds'
 * prestep): 0 inside the group kernel, each CTA over its own group; 1 as two
 * grid-wide launches before it, one thread per manifold or body, the group
 * kernel then copying the solve lanes into shared memory; -1 (default) the
 * grid-wide launches when the groups hold joints and at least 8,192
 * constraints.  The results are the same bit for bit.  Takes effect at the
 * next step.  No reference counterpart: it only chooses how the GPU runs the
 * stages of Space.cs:496-513. */
bepugpu_status bepugpu_set_group_prologue(bepugpu_context* ctx, int32_t scene, int32_t mode);

/* Persistent mode: resident blocks per SM of the cooperative launch (1 or 2). */
bepugpu_status bepugpu_set_persistent_blocks_per_sm(bepugpu_context* ctx, int32_t scene, int32_t blocks);

/* Device time of the last bepugpu_step on this scene, in milliseconds, taken
 * with CUDA events on the scene's stream. */
bepugpu_status bepugpu_last_step_ms(bepugpu_context* ctx, int32_t scene, float* ms);

/* Device time of the phases of the last bepugpu_step (six floats).  [5] is
 * the island-group kernel, which runs first.  Graph mode: the colour-sweep
 * path's phases from events captured into the graph, [0] refresh +
 * ForceUpdater, [1] prestep, [2] warm start, [3] solve iterations, [4]
 * PositionUpdater.  Persistent mode: [3] only, from globaltimer stamps around
 * the solve iterations; [0], [1], [2], [4] are 0. */
bepugpu_status bepugpu_last_step_phase_ms(bepugpu_context* ctx, int32_t scene, float* phase_ms);

/* Number of kernel launches the last bepugpu_step issued (graph nodes count
 * as launches). */
bepugpu_status bepugpu_last_step_launches(bepugpu_context* ctx, int32_t scene, uint32_t* launches);

/* Batched stepping (ParallelSpaceTestDemo.cs:24-64 is the reference's
 * analogue: independent Spaces updated side by side).  Every island group of
 * every listed scene becomes one CTA of one graph-captured launch, and each CTA
 * runs its group's `steps` steps back to back with the group's bodies and
 * solve lanes in shared memory.  A scene joins that launch when its whole step
 * is island groups (no colour-sweep constraints, no joints, no dynamic body
 * outside a group, no moving kinematic body); other listed scenes take their
 * one-scene path after it.  The call returns when every scene has advanced.
 * Results equal `steps` calls of bepugpu_step on each scene.  A scene may be
 * listed once per call. */
bepugpu_status bepugpu_batch_step(bepugpu_context* ctx, const int32_t* scenes, uint32_t count,
                                  float dt, uint32_t steps, uint32_t flags);
/* The same with a step count per scene (0 leaves a scene as it is). */
bepugpu_status bepugpu_batch_step_each(bepugpu_context* ctx, const int32_t* scenes, const uint32_t* steps,
                                       uint32_t count, float dt, uint32_t flags);
/* Threads per CTA of the batched launches: 0 (default) sizes them from the
 * largest colour of the listed groups; else a multiple of 32 in [32, 256].
 * Results do not depend on it. */
bepugpu_status bepugpu_set_batch_threads(bepugpu_context* ctx, int32_t threads);

/* Per-phase device times of one step run as separate launches, each bracketed
 * by CUDA events on the scene's stream (an instrumented copy of bepugpu_step:
 * it advances the scene like bepugpu_step does).  The solve census counts,
 * before each solve sweep, the manifolds still active and their algorithmic
 * bytes 76*d + 136 + 48*c (c contacts, d dynamic bodies). */
typedef struct bepugpu_phase_times {
    float refresh_ms, force_ms, prestep_ms, warm_ms, solve_ms, position_ms;
    uint32_t solve_launches, warm_launches;
    double solve_algorithmic_bytes;   /* sweep path and island groups together */
    double solve_manifold_visits;
    double solve_contact_visits;
    float group_ms;                   /* the island-group kernel (whole steps of small islands) */
    uint32_t groups;                  /* CTAs of that kernel */
    double group_compulsory_bytes;    /* DRAM bytes the group kernel cannot avoid in one step:
                                         every input lane read once, every output lane written
                                         once (136 + 64 c per manifold with its solve lanes in
                                         shared memory, 288 + 112 c with them in global memory,
                                         208 per body) */
    double group_solve_algorithmic_bytes; /* the group kernel's share of solve_algorithmic_bytes */
    double group_solve_manifold_visits;   /* the group kernel's share of solve_manifold_visits */
} bepugpu_phase_times;

bepugpu_status bepugpu_profile_step(bepugpu_context* ctx, int32_t scene, float dt, uint32_t flags,
                                    bepugpu_phase_times* out);

/* Step without allocating.  It has no counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc -- a plugin inside an engine or
 * sandbox that owns the device heap, or code held to a memory budget fixed in
 * advance.  `bodies` and `manifolds` are the caller's records in DEVICE memory
 * (in/out, like upload + step + download of the other entry points); joints are
 * not taken.  All scratch lives in one fixed array of
 * BEPUGPU_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * the process exits, so a call takes at most BEPUGPU_NOALLOC_MAX_BODIES bodies
 * and BEPUGPU_NOALLOC_MAX_MANIFOLDS manifolds and returns
 * BEPUGPU_INVALID_ARGUMENT above that.  The step runs on the current device, on
 * `stream` (a cudaStream_t, NULL = legacy default stream), in one thread block,
 * and the call returns when it is done.  The first call made under a CUDA
 * context (the device's primary context, or one the caller created and made
 * current) looks up the scratch array's address in that context and keeps it
 * for later calls under the same context; make that first call before any
 * stream capture.  Calls share the scratch array: calls whose work overlaps
 * on the GPU (other host threads, other streams) race and must be serialised
 * by the caller.  The manifold list is coloured in the call with at most 128
 * colours (two 64-bit masks per body): a list that needs more returns
 * BEPUGPU_INVALID_OPERATION with the records unchanged, where
 * bepugpu_upload_constraints has no colour limit.  Records whose manifolds
 * name bodies out of range, the same body twice or a contact count outside
 * 0..4, and NONCONVEX manifolds (their contact friction lanes are not in the
 * scratch), return BEPUGPU_INVALID_ARGUMENT, found on the device before
 * anything is written.  Settings are bounded as bepugpu_create bounds them
 * (iteration_limit 0..65535).  Damping factors are the float of the
 * reference's double pow, computed on the device.  There is no narrow
 * phase here: GENERATED manifolds are stepped with the contacts they hold
 * (and not refreshed). */
#define BEPUGPU_NOALLOC_MAX_BODIES 1024
#define BEPUGPU_NOALLOC_MAX_MANIFOLDS 2048
#define BEPUGPU_NOALLOC_SCRATCH_BYTES 1639424
bepugpu_status bepugpu_step_noalloc(const bepugpu_settings* settings, bepugpu_body* bodies,
                                    uint32_t body_count, bepugpu_manifold* manifolds,
                                    uint32_t manifold_count, float dt, uint32_t flags, void* stream);

/* Kernel counters of the last call on the context: launches and device ms. */
bepugpu_status bepugpu_last_call_stats(bepugpu_context* ctx, uint32_t* launches, float* device_ms);

/* ------------------------------------------------------------------ serving --
 * A server steps scenes on request.  A worker thread drains a lock-free
 * submit ring, keeps a FIFO of requests per scene, and launches waves: every
 * scene with a request that is not already on the device joins the next wave
 * (continuous batching), up to `max_wave_scenes`, and up to
 * `max_waves_in_flight` waves overlap on the device on their own streams.  In
 * a batched wave every island group of every scene is one CTA of one launch
 * running that request's steps; scenes whose step is not all island groups
 * (joints, large islands) take their one-scene path in the same wave.  With
 * `batching` 0 every request takes the one-scene path (one graph launch per
 * scene step): the plain baseline.
 * Residency: the device bytes of resident scenes stay within
 * `device_budget_bytes`; to make room the least recently used idle scene is
 * spilled to pinned host memory (its arena, impulses included) and restored
 * when a request needs it; a scene larger than the budget is refused
 * (ADMISSION_REFUSED).  Results are the same bits as stepping each scene with
 * bepugpu_step, whatever the mix and the spills.
 * While a scene is added to a server, the other per-scene calls on it return
 * INVALID_OPERATION; bepugpu_server_release_scene gives it back (resident).
 * Submit and poll may be called from any thread.  No reference counterpart:
 * the reference steps each Space on the caller's thread (Space.Update). */
typedef struct bepugpu_server bepugpu_server;

typedef struct bepugpu_server_config {
    uint64_t device_budget_bytes;
    uint32_t max_wave_scenes;      /* scenes per wave (>= 1) */
    uint32_t max_waves_in_flight;  /* 1..4 */
    uint32_t queue_capacity;       /* submit and completion rings, a power of two >= 2 */
    uint32_t batching;             /* 1 continuous batching, 0 one launch per scene step */
    float dt;
    uint32_t flags;                /* BEPUGPU_STEP_* */
    uint32_t threads;              /* CTA size of the batched waves: 0 from each group plan, else a
                                      multiple of 32 in [32, 256] (bepugpu_set_batch_threads's rule) */
    uint32_t reserved[3];
} bepugpu_server_config;

typedef struct bepugpu_completion {
    uint64_t tag;                  /* as submitted */
    int32_t scene;
    int32_t status;                /* BEPUGPU_OK, NOT_FOUND, ADMISSION_REFUSED, CUDA_ERROR */
    uint32_t steps;
    uint32_t wave;                 /* wave number that ran it */
    double submit_us, start_us, done_us;  /* bepugpu_clock_us() at submit, wave launch, completion seen */
} bepugpu_completion;

typedef struct bepugpu_server_stats {
    uint64_t submitted, completed, waves, wave_scenes, launches, spills, restores;
    uint64_t resident_bytes, peak_resident_bytes, spilled_bytes;
    uint32_t scenes, resident_scenes;
    uint64_t room_waits;        /* times a spilled scene waited a wave for room */
    uint64_t restore_failures;  /* restores that could not get device memory */
    uint64_t spill_us;          /* worker time spent spilling (copies included) */
    uint64_t restore_us;        /* worker time spent restoring (copies included) */
    uint64_t pinned_bytes;      /* pinned host memory the server holds for spill buffers */
} bepugpu_server_stats;

void bepugpu_server_default_config(bepugpu_server_config* out);
bepugpu_status bepugpu_server_create(bepugpu_context* ctx, const bepugpu_server_config* config,
                                     bepugpu_server** out);
/* Waits for waves on the device, drops queued requests, restores spilled scenes
 * and gives every scene back. */
bepugpu_status bepugpu_server_destroy(bepugpu_server* server);
bepugpu_status bepugpu_server_add_scene(bepugpu_server* server, int32_t scene);
/* Waits (up to timeout_ms) until the scene has no queued or running request,
 * restores it if spilled and gives it back. */
bepugpu_status bepugpu_server_release_scene(bepugpu_server* server, int32_t scene, uint32_t timeout_ms);
/* Queues `steps` steps of `scene`; QUEUE_FULL when the submit ring is full. */
bepugpu_status bepugpu_serve_submit(bepugpu_server* server, int32_t scene, uint32_t steps, uint64_t tag);
/* Moves up to `max` completions to `out`; *count receives how many. */
bepugpu_status bepugpu_serve_poll(bepugpu_server* server, bepugpu_completion* out, uint32_t max, uint32_t* count);
/* Waits until every submitted request has completed (TIMEOUT after timeout_ms). */
bepugpu_status bepugpu_server_drain(bepugpu_server* server, uint32_t timeout_ms);
bepugpu_status bepugpu_server_stats_get(bepugpu_server* server, bepugpu_server_stats* out);
const char* bepugpu_server_last_error(bepugpu_server* server);
/* Microseconds of the steady clock the completion times use. */
double bepugpu_clock_us(void);

#ifdef __cplusplus
}
#endif

#endif /* BEPUGPU_H */
