// Device side of the two-body joints: layout and per-joint math.
//
// A joint slot is one SolverUpdateable of the solver list.  Every joint is run
// as a SolverGroup of up to three children -- ball socket, revolute angular,
// limit (swing or revolute) -- in that order: RevoluteJoint is exactly that
// group (SolverGroups/RevoluteJoint.cs:46-95, its motor inactive), and a
// stand-alone joint is a group of one, which has the same activity sequence
// (its own zero-impulse streak and the group's emptiness end it at the same
// visit).  Arithmetic follows the reference classes operation for operation:
//   BallSocketJoint       TwoEntity/Joints/BallSocketJoint.cs:210-372
//   RevoluteAngularJoint  TwoEntity/Joints/RevoluteAngularJoint.cs:226-365
//   SwingLimit            TwoEntity/JointLimits/SwingLimit.cs:211-347
//   RevoluteLimit         TwoEntity/JointLimits/RevoluteLimit.cs:285-649
//   NoRotationJoint       TwoEntity/Joints/NoRotationJoint.cs:160-262 (the angular child of
//                         NO_ROTATION and WELD records; WeldJoint.cs:15-55 is ball socket + it)
//   DistanceJoint         TwoEntity/Joints/DistanceJoint.cs:226-380 (the first child slot)
//   DistanceLimit         TwoEntity/JointLimits/DistanceLimit.cs:260-457 (the first child slot)
//   PointOnPlaneJoint     TwoEntity/Joints/PointOnPlaneJoint.cs:212-330 (the first child slot)
//   TwistJoint            TwoEntity/Joints/TwistJoint.cs:204-365 (the angular child slot)
//   PointOnLineJoint      TwoEntity/Joints/PointOnLineJoint.cs:247-463 (the first child slot)
//   TwistLimit            TwoEntity/JointLimits/TwistLimit.cs:200-383 (the limit slot; its
//                         last error, which picks the next jacobian's sign, in kJACC1.w)
//   EllipseSwingLimit     TwoEntity/JointLimits/EllipseSwingLimit.cs:162-357 (the limit slot)
//   RevoluteMotor, TwistMotor, LinearAxisMotor  TwoEntity/Motors/*.cs (the limit slot)
//   AngularMotor          TwoEntity/Motors/AngularMotor.cs:203-326 (the limit slot)
//   MaximumLinearSpeedConstraint, MaximumAngularSpeedConstraint
//                         SingleEntity/Maximum*VelocityConstraint.cs (the limit slot, body B the world)
//   PlaneSliderJoint      SolverGroups/PlaneSliderJoint.cs: its point on plane joint (its limits
//                         and motors are constructed inactive)
//   SwivelHingeAngularJoint  TwoEntity/Joints/SwivelHingeAngularJoint.cs:193-287 (the angular
//                         slot; SWIVEL_HINGE is the group of a ball socket and it)
//   LinearAxisLimit       TwoEntity/JointLimits/LinearAxisLimit.cs:290-466 (the limit slot;
//                         also the limit child of PRISMATIC and LINE_SLIDER records)
// and the groups PrismaticJoint (point on line + no rotation), LineSliderJoint
// (point on line + revolute angular), UniversalJoint (ball socket + twist).
//   SpringSettings        Constraints/SpringSettings.cs:95-110
// A connection of -1 is TwoEntityConstraint.WorldEntity: kinematic, at the
// origin, identity orientation, zero velocity.  Its zeros go through the same
// arithmetic as a real body's so signed zeros come out as the reference's.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bepugpu.h"
#include "solver_device.cuh"

namespace bepugpu {

// Lanes of a joint slot: lanes[k * capacity + slot].  The first kJSolveLanes
// are the ones warm start and solve touch (impulses and prestep products); a
// group kernel keeps those in shared memory.
enum JointLane : int {
    // accumulated impulses (in/out)
    kJACC0 = 0,  // ball socket xyz, angular x
    kJACC1,      // angular y, limit x (swing: its impulse), limit y
    // prestep products
    kJOA,        // ball worldOffsetA, w = ball softness
    kJOB,        // ball worldOffsetB, w = angular softness
    kJM0,        // ball mass M11 M12 M13 M21
    kJM1,        // ball mass M22 M23 M31 M32
    kJM2,        // ball mass M33, ball bias xyz
    kJW1,        // angular worldConstrainedAxis1, w = angular bias x
    kJW2,        // angular worldConstrainedAxis2, w = angular bias y
    kJE,         // angular effective mass M11 M12 M21 M22
    kJL0,        // limit jacobianMinA (swing: hinge axis), w = limit softness
    kJL1,        // limit jacobianMaxA
    kJL2,        // limit bias x, bias y, velocityToImpulse x, y
    kJSolveLanes,
    // inputs (upload)
    kJLA = kJSolveLanes,  // ball socket localAnchorA, w = spring stiffness
    kJLB,        // ball socket localAnchorB, w = spring damping
    kJAXA,       // angular / swing local axis A, w = max corrective velocity
    kJAXB,       // angular / swing local axis B, w = margin
    kJC1,        // angular localConstrainedAxis1 (A's frame), w = bounciness
    kJC2,        // angular localConstrainedAxis2, w = bounce velocity threshold
    kJBP,        // revolute limit basis local primary axis (A's frame), w = GetDistanceFromMinimum(max)
    kJBX,        // revolute limit basis local x axis, w = swing minimum cosine
    kJTA,        // revolute limit local test axis (B's frame), w = max corrective velocity squared
    kJTRIG,      // sin(min + pi/2), 1 - cos(min + pi/2), sin(max - pi/2), 1 - cos(max - pi/2)
    kJointLanes
};
// Shared memory of one joint in a group kernel: the solve lanes, a state
// word and a ref pair.
constexpr int kJointSmemBytes = 16 * kJSolveLanes + 8 + 8;

// head.z: type (bits 0-7), children present (8-10), children IsActive (11-13),
// joint / group IsActive (14), the record continues the group before it (15),
// the next slot continues this one's group (16).
enum : uint32_t {
    kJChildBall = 1u,
    kJChildAngular = 2u,
    kJChildLimit = 4u,
    kJPresentShift = 8,
    kJChildActiveShift = 11,
    kJGroupIsActive = 1u << 14,
    kJHeadContinuation = 1u << 15,
    kJHeadHasNext = 1u << 16,
};
// State word x: kGroupActive (bit 0), child isActiveInSolver bits 1-3,
// limit minIsActive / maxIsActive bits 4-5 (a linear axis limit: bit 4 =
// violated below its minimum), kDynA / kDynB (bits 7-8), the record type
// (bits 9-13), continuation (14) and has-next (15) as in the head,
// iterations << 16.  Word y: 4-bit zero-impulse streaks of the three
// children.
enum : uint32_t {
    kJMinActive = 1u << 4,
    kJMaxActive = 1u << 5,
    kJTypeShift = 9,
    kJIsContinuation = 1u << 14,
    kJHasNext = 1u << 15,
};
__device__ __forceinline__ int JointType(uint32_t stx) { return (int)((stx >> kJTypeShift) & 31u); }
__device__ __forceinline__ bool IsDistanceType(int type) {
    return type == BEPUGPU_JOINT_DISTANCE || type == BEPUGPU_JOINT_DISTANCE_LIMIT;
}
__device__ __forceinline__ bool IsNoRotationType(int type) {
    return type == BEPUGPU_JOINT_NO_ROTATION || type == BEPUGPU_JOINT_WELD || type == BEPUGPU_JOINT_PRISMATIC;
}
__device__ __forceinline__ bool IsPointOnLineType(int type) {
    return type == BEPUGPU_JOINT_POINT_ON_LINE || type == BEPUGPU_JOINT_PRISMATIC ||
           type == BEPUGPU_JOINT_LINE_SLIDER;
}
__device__ __forceinline__ bool IsTwistType(int type) {
    return type == BEPUGPU_JOINT_TWIST || type == BEPUGPU_JOINT_UNIVERSAL;
}
// Quaternion.Concatenate (BEPUutilities/Quaternion.cs:101-117)
__device__ __forceinline__ float4 JQConcat(float4 a, float4 b) {
    return make_float4(a.w * b.x + a.x * b.w + a.z * b.y - a.y * b.z, a.w * b.y + a.y * b.w + a.x * b.z - a.z * b.x,
                       a.w * b.z + a.z * b.w + a.y * b.x - a.x * b.y, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z);
}
// Quaternion.CreateFromRotationMatrix (BEPUutilities/Quaternion.cs:152-194) of the
// matrix with rows Right r, Up u, Backward k.
__device__ __forceinline__ float4 JQFromRows(float3 r, float3 u, float3 k) {
    const float trace = r.x + u.y + k.z;
    if (trace >= 0) {
        const float S = (float)sqrt((double)trace + 1.0) * 2, inverseS = 1 / S;
        return make_float4((u.z - k.y) * inverseS, (k.x - r.z) * inverseS, (r.y - u.x) * inverseS, 0.25f * S);
    }
    if ((r.x > u.y) & (r.x > k.z)) {
        const float S = (float)sqrt(1.0 + (double)r.x - (double)u.y - (double)k.z) * 2, inverseS = 1 / S;
        return make_float4(0.25f * S, (u.x + r.y) * inverseS, (k.x + r.z) * inverseS, (u.z - k.y) * inverseS);
    }
    if (u.y > k.z) {
        const float S = (float)sqrt(1.0 + (double)u.y - (double)r.x - (double)k.z) * 2, inverseS = 1 / S;
        return make_float4((u.x + r.y) * inverseS, 0.25f * S, (k.y + u.z) * inverseS, (k.x - r.z) * inverseS);
    }
    const float S = (float)sqrt(1.0 + (double)k.z - (double)r.x - (double)u.y) * 2, inverseS = 1 / S;
    return make_float4((k.x + r.z) * inverseS, (k.y + u.z) * inverseS, 0.25f * S, (r.y - u.x) * inverseS);
}
__device__ __forceinline__ bool IsPointOnPlaneType(int type) {
    return type == BEPUGPU_JOINT_POINT_ON_PLANE || type == BEPUGPU_JOINT_PLANE_SLIDER;
}
__device__ __forceinline__ bool IsAngularMotorType(int type) {
    return type == BEPUGPU_JOINT_ANGULAR_MOTOR || type == BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR;
}
__device__ __forceinline__ bool IsSpeedLimitType(int type) {
    return type == BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED || type == BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED;
}
__device__ __forceinline__ bool IsMotorType(int type) {
    return type >= BEPUGPU_JOINT_REVOLUTE_MOTOR && type <= BEPUGPU_JOINT_LINEAR_AXIS_MOTOR;
}
// Math.Sign of a float, as the motors' servo bias multiplies it
__device__ __forceinline__ float JSign(float v) { return v > 0 ? 1.f : (v < 0 ? -1.f : 0.f); }
// RevoluteMotor / TwistMotor.GetDistanceFromGoal (RevoluteMotor.cs:345-371); the
// goal arrives wrapped by MathHelper.WrapAngle.
__device__ __forceinline__ float JDistanceFromGoal(float angle, float goalAngle) {
    float forward;
    if (goalAngle > 0) forward = angle > goalAngle ? angle - goalAngle : 6.28318548f - goalAngle + angle;
    else forward = angle < goalAngle ? 6.28318548f - goalAngle + angle : angle - goalAngle;
    return forward > 3.14159274f ? 6.28318548f - forward : -forward;
}
__device__ __forceinline__ bool IsSwivelType(int type) {
    return type == BEPUGPU_JOINT_SWIVEL_HINGE_ANGULAR || type == BEPUGPU_JOINT_SWIVEL_HINGE;
}
__device__ __forceinline__ bool IsLinearLimitType(int type) {
    return type == BEPUGPU_JOINT_LINEAR_AXIS_LIMIT || type == BEPUGPU_JOINT_PRISMATIC ||
           type == BEPUGPU_JOINT_LINE_SLIDER;
}
// The linear axis limit's three solve lanes (jacobian linear A + softness,
// angular A + bias, angular B + mass): a prismatic joint's no-rotation child
// holds kJL0..kJL2, so its limit takes the revolute angular lanes.
__device__ __forceinline__ int LinearLimitLane(int type) {
    return type == BEPUGPU_JOINT_PRISMATIC ? (int)kJW1 : (int)kJL0;
}

struct JointSoA {
    int4* head;     // body A, body B, type | flags, source record index
    float4* lanes;  // [kJointLanes][capacity]
    uint2* state;
    int count;
    int capacity;
    __device__ __forceinline__ float4& L(int k, int s) const { return lanes[(size_t)k * capacity + s]; }
};

// ------------------------------------------------------------- joint math --
struct JM3 {
    float M11, M12, M13, M21, M22, M23, M31, M32, M33;
};

// Matrix3x3.CreateFromQuaternion (Matrix3x3.cs:1303-1328), as in ForceMath.
__device__ __forceinline__ JM3 JRotation(float4 q) {
    float qX2 = q.x + q.x, qY2 = q.y + q.y, qZ2 = q.z + q.z;
    float XX = qX2 * q.x, YY = qY2 * q.y, ZZ = qZ2 * q.z;
    float XY = qX2 * q.y, XZ = qX2 * q.z, XW = qX2 * q.w;
    float YZ = qY2 * q.z, YW = qY2 * q.w, ZW = qZ2 * q.w;
    JM3 r;
    r.M11 = 1 - YY - ZZ; r.M21 = XY - ZW; r.M31 = XZ + YW;
    r.M12 = XY + ZW; r.M22 = 1 - XX - ZZ; r.M32 = YZ - XW;
    r.M13 = XZ - YW; r.M23 = YZ + XW; r.M33 = 1 - XX - YY;
    return r;
}
// Matrix3x3.Transform (:1071-1082): row vector times matrix.
__device__ __forceinline__ float3 JTransform(float3 v, const JM3& m) {
    return make_float3(v.x * m.M11 + v.y * m.M21 + v.z * m.M31, v.x * m.M12 + v.y * m.M22 + v.z * m.M32,
                       v.x * m.M13 + v.y * m.M23 + v.z * m.M33);
}
// Matrix3x3.Multiply (:766-790)
__device__ __forceinline__ JM3 JMul(const JM3& a, const JM3& b) {
    JM3 r;
    r.M11 = a.M11 * b.M11 + a.M12 * b.M21 + a.M13 * b.M31;
    r.M12 = a.M11 * b.M12 + a.M12 * b.M22 + a.M13 * b.M32;
    r.M13 = a.M11 * b.M13 + a.M12 * b.M23 + a.M13 * b.M33;
    r.M21 = a.M21 * b.M11 + a.M22 * b.M21 + a.M23 * b.M31;
    r.M22 = a.M21 * b.M12 + a.M22 * b.M22 + a.M23 * b.M32;
    r.M23 = a.M21 * b.M13 + a.M22 * b.M23 + a.M23 * b.M33;
    r.M31 = a.M31 * b.M11 + a.M32 * b.M21 + a.M33 * b.M31;
    r.M32 = a.M31 * b.M12 + a.M32 * b.M22 + a.M33 * b.M32;
    r.M33 = a.M31 * b.M13 + a.M32 * b.M23 + a.M33 * b.M33;
    return r;
}
__device__ __forceinline__ JM3 JSub(const JM3& a, const JM3& b) {
    return {a.M11 - b.M11, a.M12 - b.M12, a.M13 - b.M13, a.M21 - b.M21, a.M22 - b.M22,
            a.M23 - b.M23, a.M31 - b.M31, a.M32 - b.M32, a.M33 - b.M33};
}
// Matrix3x3.CreateCrossProduct (:378-389)
__device__ __forceinline__ JM3 JCrossMatrix(float3 v) { return {0, -v.z, v.y, v.z, 0, -v.x, -v.y, v.x, 0}; }
// Matrix3x3.CreateScale
__device__ __forceinline__ JM3 JScale(float s) { return {s, 0, 0, 0, s, 0, 0, 0, s}; }
// Matrix3x3.Invert (:505-534) with Determinant (:1231-1235)
__device__ __forceinline__ JM3 JInvert(const JM3& m) {
    float det = m.M11 * m.M22 * m.M33 + m.M12 * m.M23 * m.M31 + m.M13 * m.M21 * m.M32 -
                m.M31 * m.M22 * m.M13 - m.M32 * m.M23 * m.M11 - m.M33 * m.M21 * m.M12;
    float d = 1 / det;
    JM3 r;
    r.M11 = (m.M22 * m.M33 - m.M23 * m.M32) * d;
    r.M12 = (m.M13 * m.M32 - m.M33 * m.M12) * d;
    r.M13 = (m.M12 * m.M23 - m.M22 * m.M13) * d;
    r.M21 = (m.M23 * m.M31 - m.M21 * m.M33) * d;
    r.M22 = (m.M11 * m.M33 - m.M13 * m.M31) * d;
    r.M23 = (m.M13 * m.M21 - m.M11 * m.M23) * d;
    r.M31 = (m.M21 * m.M32 - m.M22 * m.M31) * d;
    r.M32 = (m.M12 * m.M31 - m.M11 * m.M32) * d;
    r.M33 = (m.M11 * m.M22 - m.M12 * m.M21) * d;
    return r;
}
__device__ __forceinline__ float3 JCross(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float JDot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 JXYZ(float4 v) { return make_float3(v.x, v.y, v.z); }
// Vector3.Normalize (Vector3.cs:81-87): the reciprocal square root in double.
__device__ __forceinline__ float3 JNormalize(float3 v) {
    float inverse = dr::InvSqrtAsDouble(v.x * v.x + v.y * v.y + v.z * v.z);
    return make_float3(v.x * inverse, v.y * inverse, v.z * inverse);
}
__device__ __forceinline__ JM3 JInertia(const BodyState& s) {
    return {s.I11, s.I12, s.I13, s.I21, s.I22, s.I23, s.I31, s.I32, s.I33};
}
// (float)System.Math.Sqrt((double)x) equals the float square root (see SqrtOfFloat).
// SpringSettings.ComputeErrorReductionAndSoftness (SpringSettings.cs:95-110)
__device__ __forceinline__ void JSpring(float stiffness, float damping, float dt, float updateRate, float& erp,
                                        float& softness) {
    float multiplier = 1 / (dt * stiffness + damping);
    erp = stiffness * multiplier;
    softness = updateRate * multiplier;
}
// JointLimit.ComputeBounceVelocity (JointLimit.cs:60-66)
__device__ __forceinline__ float JBounce(float impactVelocity, float threshold, float bounciness) {
    float lowThreshold = threshold * 0.3f;
    float velocityFraction = Clampf((impactVelocity - lowThreshold) / (threshold - lowThreshold + 1e-7f), 0, 1);
    return velocityFraction * impactVelocity * bounciness;
}

// A joint connection: body state plus pose, or the world entity.  Body refs go
// through a body view (GlobalBodies on the sweep path, GroupBodies in island
// groups); ref -1 is the world entity.
struct JointBody {
    BodyState s;
    float3 pos;
    float4 q;
    JM3 R;
    bool dynamic;
};
template <class V>
__device__ __forceinline__ void LoadJointBodyV(const V& bv, int r, JointBody& o) {
    if (r == -1) {
        o.s.vx = o.s.vy = o.s.vz = 0.f; o.s.invMass = 0.f;
        o.s.wx = o.s.wy = o.s.wz = 0.f;
        o.s.I11 = o.s.I12 = o.s.I13 = o.s.I21 = o.s.I22 = o.s.I23 = o.s.I31 = o.s.I32 = o.s.I33 = 0.f;
        o.pos = make_float3(0.f, 0.f, 0.f);
        o.q = make_float4(0.f, 0.f, 0.f, 1.f);
        o.R = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        o.dynamic = false;
        return;
    }
    LoadBodyV(bv, r, o.s);
    float4 p = bv.Pos(r);
    o.pos = make_float3(p.x, p.y, p.z);
    o.q = bv.Quat(r);
    o.R = JRotation(o.q);
    o.dynamic = p.w != 0.f;
}
// A connection's local inverse inertia (the distance joints' effective mass
// reads it, DistanceJoint.cs:301-333); only asked for dynamic connections.
template <class V>
__device__ __forceinline__ JM3 LoadLocalInertiaV(const V& bv, int r) {
    float4 l0, l1;
    float m33;
    bv.LocalInertia(r, l0, l1, m33);
    return {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w, m33};
}
// Quaternion.Multiply (Quaternion.cs)
__device__ __forceinline__ float4 JQMul(float4 a, float4 b) {
    float4 r;
    r.x = a.x * b.w + b.x * a.w + a.y * b.z - a.z * b.y;
    r.y = a.y * b.w + b.y * a.w + a.z * b.x - a.x * b.z;
    r.z = a.z * b.w + b.z * a.w + a.x * b.y - a.y * b.x;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    return r;
}
// Quaternion.GetAxisAngleFromQuaternion (Quaternion.cs:756-787); Math.Acos in double.
__device__ __forceinline__ void JAxisAngle(float4 q, float3& axis, float& angle) {
    float qw = q.w;
    if (qw > 0) {
        axis = make_float3(q.x, q.y, q.z);
    } else {
        axis = make_float3(-q.x, -q.y, -q.z);
        qw = -qw;
    }
    float lengthSquared = axis.x * axis.x + axis.y * axis.y + axis.z * axis.z;
    if (lengthSquared > 1e-14f) {
        float inverse = 1 / SqrtOfFloat(lengthSquared);  // Vector3.Divide
        axis = make_float3(axis.x * inverse, axis.y * inverse, axis.z * inverse);
        angle = 2 * (float)acos((double)Clampf(qw, -1, 1));
    } else {
        axis = make_float3(0.f, 1.f, 0.f);
        angle = 0;
    }
}
// Quaternion.Normalize: the reciprocal square root in double.
__device__ __forceinline__ float4 JQNormalize(float4 q) {
    float inverse = dr::InvSqrtAsDouble(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    return make_float4(q.x * inverse, q.y * inverse, q.z * inverse, q.w * inverse);
}
// Quaternion.GetQuaternionBetweenNormalizedVectors (Quaternion.cs:795-823)
__device__ __forceinline__ float4 JQuatBetween(float3 v1, float3 v2) {
    float dot = JDot(v1, v2);
    float4 q;
    if (dot < -0.9999f) {
        float absX = fabsf(v1.x), absY = fabsf(v1.y), absZ = fabsf(v1.z);
        if (absX < absY && absX < absZ) q = make_float4(0.f, -v1.z, v1.y, 0.f);
        else if (absY < absZ) q = make_float4(-v1.z, 0.f, v1.x, 0.f);
        else q = make_float4(-v1.y, v1.x, 0.f, 0.f);
    } else {
        float3 axis = JCross(v1, v2);
        q = make_float4(axis.x, axis.y, axis.z, dot + 1);
    }
    return JQNormalize(q);
}
// Velocity-only view for the warm start and the solve.
template <class V>
__device__ __forceinline__ void LoadJointVelocityV(const V& bv, int r, BodyState& s) {
    if (r == -1) {
        s.vx = s.vy = s.vz = 0.f; s.invMass = 0.f;
        s.wx = s.wy = s.wz = 0.f;
        s.I11 = s.I12 = s.I13 = s.I21 = s.I22 = s.I23 = s.I31 = s.I32 = s.I33 = 0.f;
        return;
    }
    LoadBodyV(bv, r, s);
}

// PointOnLineJoint's impulse on both connections (SolveIteration and
// ExclusiveUpdate, PointOnLineJoint.cs:318-355, 440-463).  Lanes: kJOA rA,
// kJOB rB, kJM0 / kJM1 the world restricted axes; the angular jacobians are
// their cross products with rA and rB, recomputed as the reference computed them.
__device__ __forceinline__ void ApplyPointOnLine(float4 oa, float4 ob, float4 m0, float4 m1, float x, float y,
                                                 bool dynA, bool dynB, BodyState& A, BodyState& B) {
    const float3 rA = JXYZ(oa), rB = JXYZ(ob), ax1 = JXYZ(m0), ax2 = JXYZ(m1);
    float ix = ax1.x * x + ax2.x * y, iy = ax1.y * x + ax2.y * y, iz = ax1.z * x + ax2.z * y;
    if (dynA) {
        const float3 a1 = JCross(rA, ax1), a2 = JCross(rA, ax2);
        ApplyLinear(A, ix, iy, iz);
        ApplyAngular(A, x * a1.x + y * a2.x, x * a1.y + y * a2.y, x * a1.z + y * a2.z);
    }
    if (dynB) {
        const float3 b1 = JCross(ax1, rB), b2 = JCross(ax2, rB);
        ApplyLinear(B, -ix, -iy, -iz);
        ApplyAngular(B, x * b1.x + y * b2.x, x * b1.y + y * b2.y, x * b1.z + y * b2.z);
    }
}

// ------------------------------------------------------------- prestep --
// Solver.UnsafePrestep (Solver.cs:265-275) of one joint: UpdateSolverActivity,
// then Update of every active child (SolverGroup.cs:94-100).
// Reads the joint's inputs and impulses at (ji, si) and writes its impulses,
// prestep products and state at (jo, so): the same slot on the sweep path, the
// group's shared-memory lanes in a group kernel.  ra, rb: the connections'
// refs in the body view.
template <bool kAdded, class V>
__device__ __forceinline__ void PrestepJointIO(const JointSoA& ji, int si, const JointSoA& jo, int so, const V& bv,
                                               int ra, int rb, const StepParams& p) {
    const JointSoA& j = jo;
    const int s = so;
    const int4 h = ji.head[si];
    const uint32_t present = (h.z >> kJPresentShift) & 7u, childIsActive = (h.z >> kJChildActiveShift) & 7u;
    const int type = h.z & 0xff;
    JointBody A, B;
    LoadJointBodyV(bv, ra, A);
    LoadJointBodyV(bv, rb, B);
    float4 acc0 = ji.L(kJACC0, si), acc1 = ji.L(kJACC1, si);
    j.L(kJACC0, s) = acc0;
    uint32_t st = (A.dynamic ? kDynA : 0u) | (B.dynamic ? kDynB : 0u) | ((uint32_t)type << kJTypeShift) |
                  ((h.z & kJHeadContinuation) ? kJIsContinuation : 0u) | ((h.z & kJHeadHasNext) ? kJHasNext : 0u);
    if (!(h.z & kJGroupIsActive) || !(A.dynamic || B.dynamic)) {
        j.L(kJACC1, s) = acc1;
        j.state[s] = make_uint2(st, 0u);
        return;
    }
    const float4 la = ji.L(kJLA, si), lb = ji.L(kJLB, si), axa = ji.L(kJAXA, si), axb = ji.L(kJAXB, si);
    const float stiffness = la.w, damping = lb.w, maxCorr = axa.w, margin = axb.w;
    const float maxCorrSq = ji.L(kJTA, si).w;
    uint32_t active = present & childIsActive;
    if (kAdded && (active & kJChildBall) && IsPointOnLineType(type)) {
        // PointOnLineJoint.Update (PointOnLineJoint.cs:362-438).  Inputs: kJLA line anchor
        // (A), kJLB point (B), kJBP line direction, kJBX / kJTA restricted axes (A's frame).
        // Lanes: kJOA rA + softness, kJOB.xyz rB, kJM0 axis 1 + M11, kJM1 axis 2 + M12,
        // kJM2 M21 M22 bias x y of the negative effective mass.
        const float3 ax1 = JTransform(JXYZ(ji.L(kJBX, si)), A.R), ax2 = JTransform(JXYZ(ji.L(kJTA, si)), A.R);
        float3 lineAnchor = JTransform(JXYZ(la), A.R);
        lineAnchor = make_float3(lineAnchor.x + A.pos.x, lineAnchor.y + A.pos.y, lineAnchor.z + A.pos.z);
        const float3 lineDir = JTransform(JXYZ(ji.L(kJBP, si)), A.R);
        const float3 rB = JTransform(JXYZ(lb), B.R);
        const float3 point = make_float3(rB.x + B.pos.x, rB.y + B.pos.y, rB.z + B.pos.z);
        float3 off = make_float3(point.x - lineAnchor.x, point.y - lineAnchor.y, point.z - lineAnchor.z);
        const float along = JDot(off, lineDir);
        off = make_float3(lineDir.x * along, lineDir.y * along, lineDir.z * along);
        const float3 nearPoint = make_float3(lineAnchor.x + off.x, lineAnchor.y + off.y, lineAnchor.z + off.z);
        const float3 rA = make_float3(nearPoint.x - A.pos.x, nearPoint.y - A.pos.y, nearPoint.z - A.pos.z);
        const float3 e3 = make_float3(point.x - nearPoint.x, point.y - nearPoint.y, point.z - nearPoint.z);
        const float ex = JDot(e3, ax1), ey = JDot(e3, ax2);
        float erp, softness;
        JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
        const float bias = -erp;
        float bx = bias * ex, by = bias * ey;
        const float length = bx * bx + by * by;
        if (length > maxCorrSq) {
            float multiplier = maxCorr / SqrtOfFloat(length);
            bx *= multiplier; by *= multiplier;
        }
        const float3 a1 = JCross(rA, ax1), b1 = JCross(ax1, rB), a2 = JCross(rA, ax2), b2 = JCross(ax2, rB);
        float m11 = 0, m22 = 0, m1221 = 0;
        if (A.dynamic) {
            const JM3 ia = JInertia(A.s);
            float3 t = JTransform(a1, ia);
            m11 = JDot(t, a1);
            m11 += A.s.invMass;
            m1221 = JDot(t, a2);
            t = JTransform(a2, ia);
            m22 = JDot(t, a2);
            m22 += A.s.invMass;
        }
        if (B.dynamic) {
            const JM3 ib = JInertia(B.s);
            float3 t = JTransform(b1, ib);
            float extra = JDot(t, b1);
            m11 += B.s.invMass + extra;
            extra = JDot(t, b2);
            m1221 += extra;
            t = JTransform(b2, ib);
            extra = JDot(t, b2);
            m22 += B.s.invMass + extra;
        }
        // Matrix2x2.Invert (Matrix2x2.cs:160-174), then Negate (:259-273)
        const float k11 = m11 + softness, k12 = m1221, k21 = m1221, k22 = m22 + softness;
        const float d = 1 / (k11 * k22 - k12 * k21);
        const float i11 = k22 * d, i12 = -k12 * d, i21 = -k21 * d, i22 = k11 * d;
        j.L(kJOA, s) = make_float4(rA.x, rA.y, rA.z, softness);
        j.L(kJOB, s).x = rB.x;
        j.L(kJOB, s).y = rB.y;
        j.L(kJOB, s).z = rB.z;
        j.L(kJM0, s) = make_float4(ax1.x, ax1.y, ax1.z, -i11);
        j.L(kJM1, s) = make_float4(ax2.x, ax2.y, ax2.z, -i12);
        j.L(kJM2, s) = make_float4(-i21, -i22, bx, by);
        st |= 1u << (kChildShift + 0);
    } else if (kAdded && (active & kJChildBall) && IsPointOnPlaneType(type)) {
        // PointOnPlaneJoint.Update (PointOnPlaneJoint.cs:250-306).  Lanes: kJOA rA + softness,
        // kJOB.xyz rB, kJM0 normal + negative effective mass, kJM1 rA x n + bias, kJM2 -(rB x n).
        const float3 n = JTransform(JXYZ(axa), A.R);
        float3 wpa = JTransform(JXYZ(la), A.R);
        wpa = make_float3(wpa.x + A.pos.x, wpa.y + A.pos.y, wpa.z + A.pos.z);
        const float3 rB = JTransform(JXYZ(lb), B.R);
        const float3 wpt = make_float3(rB.x + B.pos.x, rB.y + B.pos.y, rB.z + B.pos.z);
        const float pointDistance = JDot(wpt, n), planeDistance = JDot(wpa, n);
        const float distanceChange = planeDistance - pointDistance;
        float3 closest = make_float3(n.x * distanceChange, n.y * distanceChange, n.z * distanceChange);
        closest = make_float3(closest.x + wpt.x, closest.y + wpt.y, closest.z + wpt.z);
        const float3 rA = make_float3(closest.x - A.pos.x, closest.y - A.pos.y, closest.z - A.pos.z);
        const float3 raxn = JCross(rA, n);
        float3 rbxn = JCross(rB, n);
        rbxn = make_float3(-rbxn.x, -rbxn.y, -rbxn.z);
        const float error = JDot(make_float3(wpt.x - closest.x, wpt.y - closest.y, wpt.z - closest.z), n);
        float erp, softness;
        JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
        const float bias = Clampf(-erp * error, -maxCorr, maxCorr);
        float nem;
        if (A.dynamic && B.dynamic) {
            float angularA = JDot(raxn, JTransform(raxn, JInertia(A.s)));
            float angularB = JDot(rbxn, JTransform(rbxn, JInertia(B.s)));
            nem = A.s.invMass + B.s.invMass + angularA + angularB;
            nem = -1 / (nem + softness);
        } else if (A.dynamic) {
            float angularA = JDot(raxn, JTransform(raxn, JInertia(A.s)));
            nem = A.s.invMass + angularA;
            nem = -1 / (nem + softness);
        } else {
            float angularB = JDot(rbxn, JTransform(rbxn, JInertia(B.s)));
            nem = B.s.invMass + angularB;
            nem = -1 / (nem + softness);
        }
        j.L(kJOA, s) = make_float4(rA.x, rA.y, rA.z, softness);
        j.L(kJOB, s).x = rB.x;
        j.L(kJOB, s).y = rB.y;
        j.L(kJOB, s).z = rB.z;
        j.L(kJM0, s) = make_float4(n.x, n.y, n.z, nem);
        j.L(kJM1, s) = make_float4(raxn.x, raxn.y, raxn.z, bias);
        j.L(kJM2, s) = make_float4(rbxn.x, rbxn.y, rbxn.z, 0.f);
        st |= 1u << (kChildShift + 0);
    } else if (kAdded && (active & kJChildBall) && IsDistanceType(type)) {
        // DistanceJoint.Update (DistanceJoint.cs:275-352) / DistanceLimit.Update (DistanceLimit.cs:312-430).
        // Lanes: kJM0 jLinearA + velocityToImpulse, kJM1 jAngularA + bias, kJM2 jAngularB
        // (jLinearB = -jLinearA); kJOA.w softness.  A limit keeps its last jLinearA in kJBP.
        const bool isLimit = type == BEPUGPU_JOINT_DISTANCE_LIMIT;
        const float3 offA = JTransform(JXYZ(la), A.R), offB = JTransform(JXYZ(lb), B.R);
        const float anx = A.pos.x + offA.x, any = A.pos.y + offA.y, anz = A.pos.z + offA.z;
        const float bnx = B.pos.x + offB.x, bny = B.pos.y + offB.y, bnz = B.pos.z + offB.z;
        const float3 sep = make_float3(bnx - anx, bny - any, bnz - anz);
        const float dist = SqrtOfFloat(sep.x * sep.x + sep.y * sep.y + sep.z * sep.z);
        const float minL = axa.x, maxL = axa.y;
        bool on = true;
        float3 jA, jAngA, jAngB;
        if (isLimit && dist <= maxL && dist >= minL) {
            on = false;
            acc0.x = 0.f;
        } else if (isLimit && dist > maxL) {
            jA = JXYZ(ji.L(kJBP, si));  // a degenerate separation keeps the last jLinearA
            if (dist > 1e-7f) jA = make_float3(sep.x / dist, sep.y / dist, sep.z / dist);
            jAngA = JCross(jA, offA);
            jAngB = JCross(jA, offB);
        } else {
            float3 jB = make_float3(0.f, 0.f, 0.f);
            if (dist > 1e-7f) jB = make_float3(sep.x / dist, sep.y / dist, sep.z / dist);
            jA = make_float3(-jB.x, -jB.y, -jB.z);
            jAngA = JCross(offA, jB);
            jAngB = JCross(offB, jB);
        }
        if (on) {
            if (isLimit) {
                const float4 last = ji.L(kJBP, si);
                ji.L(kJBP, si) = make_float4(jA.x, jA.y, jA.z, last.w);
            }
            const float3 jB = make_float3(-jA.x, -jA.y, -jA.z);
            float vti;
            if (A.dynamic && B.dynamic) {
                float3 aAng = JCross(JTransform(jAngA, LoadLocalInertiaV(bv, ra)), offA);
                float3 bAng = JCross(JTransform(jAngB, LoadLocalInertiaV(bv, rb)), offB);
                aAng = make_float3(aAng.x + bAng.x, aAng.y + bAng.y, aAng.z + bAng.z);
                vti = JDot(aAng, jB);
                vti += A.s.invMass + B.s.invMass;
            } else if (A.dynamic) {
                float3 aAng = JCross(JTransform(jAngA, LoadLocalInertiaV(bv, ra)), offA);
                vti = JDot(aAng, jB);
                vti += A.s.invMass;
            } else {
                float3 bAng = JCross(JTransform(jAngB, LoadLocalInertiaV(bv, rb)), offB);
                vti = JDot(bAng, jB);
                vti += B.s.invMass;
            }
            float erp, softness;
            JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
            vti = 1 / (softness + vti);
            jAngA = make_float3(-jAngA.x, -jAngA.y, -jAngA.z);
            float bias;
            if (!isLimit) {
                float error = minL - dist;  // Distance - currentDistance
                bias = Clampf(error * erp, -maxCorr, maxCorr);
            } else {
                float error = dist > maxL ? Maxf(0, dist - maxL - margin) : Maxf(0, minL - margin - dist);
                bias = Minf(erp * error, maxCorr);
                const float bounciness = ji.L(kJC1, si).w, threshold = ji.L(kJC2, si).w;
                if (bounciness > 0) {
                    float rel = jA.x * A.s.vx + jA.y * A.s.vy + jA.z * A.s.vz;
                    float dot = jAngA.x * A.s.wx + jAngA.y * A.s.wy + jAngA.z * A.s.wz;
                    rel += dot;
                    dot = jB.x * B.s.vx + jB.y * B.s.vy + jB.z * B.s.vz;
                    rel += dot;
                    dot = jAngB.x * B.s.wx + jAngB.y * B.s.wy + jAngB.z * B.s.wz;
                    rel += dot;
                    bias = Maxf(bias, JBounce(-rel, threshold, bounciness));
                }
            }
            j.L(kJOA, s) = make_float4(0.f, 0.f, 0.f, softness);
            j.L(kJM0, s) = make_float4(jA.x, jA.y, jA.z, vti);
            j.L(kJM1, s) = make_float4(jAngA.x, jAngA.y, jAngA.z, bias);
            j.L(kJM2, s) = make_float4(jAngB.x, jAngB.y, jAngB.z, 0.f);
            st |= 1u << (kChildShift + 0);
        }
        j.L(kJACC0, s) = acc0;
    } else if (active & kJChildBall) {
        // BallSocketJoint.Update (BallSocketJoint.cs:210-278)
        float3 offA = JTransform(JXYZ(la), A.R), offB = JTransform(JXYZ(lb), B.R);
        float erp, softness;
        JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
        JM3 rA = JCrossMatrix(offA), rB = JCrossMatrix(offB), k;
        if (A.dynamic && B.dynamic) {
            JM3 lin = JScale(A.s.invMass + B.s.invMass);
            JM3 angA = JMul(rA, JInertia(A.s)), angB = JMul(rB, JInertia(B.s));
            angA = JMul(angA, rA);
            angB = JMul(angB, rB);
            k = JSub(lin, angA);
            k = JSub(k, angB);
        } else if (A.dynamic) {
            JM3 lin = JScale(A.s.invMass);
            JM3 angA = JMul(JMul(rA, JInertia(A.s)), rA);
            k = JSub(lin, angA);
        } else {
            JM3 lin = JScale(B.s.invMass);
            JM3 angB = JMul(JMul(rB, JInertia(B.s)), rB);
            k = JSub(lin, angB);
        }
        k.M11 += softness;
        k.M22 += softness;
        k.M33 += softness;
        JM3 mass = JInvert(k);
        float ex = B.pos.x + offB.x, ey = B.pos.y + offB.y, ez = B.pos.z + offB.z;
        ex = ex - A.pos.x; ey = ey - A.pos.y; ez = ez - A.pos.z;
        ex = ex - offA.x; ey = ey - offA.y; ez = ez - offA.z;
        float nerp = -erp;
        float bx = ex * nerp, by = ey * nerp, bz = ez * nerp;
        float length = bx * bx + by * by + bz * bz;
        if (length > maxCorrSq) {
            float multiplier = maxCorr / SqrtOfFloat(length);
            bx *= multiplier; by *= multiplier; bz *= multiplier;
        }
        j.L(kJOA, s) = make_float4(offA.x, offA.y, offA.z, softness);
        j.L(kJOB, s).x = offB.x;  // w of kJOB belongs to the angular child
        j.L(kJOB, s).y = offB.y;
        j.L(kJOB, s).z = offB.z;
        j.L(kJM0, s) = make_float4(mass.M11, mass.M12, mass.M13, mass.M21);
        j.L(kJM1, s) = make_float4(mass.M22, mass.M23, mass.M31, mass.M32);
        j.L(kJM2, s) = make_float4(mass.M33, bx, by, bz);
        st |= 1u << (kChildShift + 0);
    }
    if (kAdded && (active & kJChildAngular) && IsTwistType(type)) {
        // TwistJoint.Update (TwistJoint.cs:235-300).  Inputs: axes A / B, A's local y and z
        // (kJC1, kJC2) and B's local y (kJBX).  Lanes: kJW1 jacobianB + velocityToImpulse,
        // kJW2.x bias, kJOB.w softness (jacobianA = -jacobianB).
        const float3 worldAxisA = JTransform(JXYZ(axa), A.R);
        const float3 aAxisY = JTransform(JXYZ(ji.L(kJC1, si)), A.R), aAxisZ = JTransform(JXYZ(ji.L(kJC2, si)), A.R);
        const float3 worldAxisB = JTransform(JXYZ(axb), B.R);
        const float3 bAxisY = JTransform(JXYZ(ji.L(kJBX, si)), B.R);
        const float4 rotation = JQuatBetween(worldAxisB, worldAxisA);
        const float3 twistMeasure = QTransform(bAxisY.x, bAxisY.y, bAxisY.z, rotation);
        const float y = JDot(twistMeasure, aAxisZ), x = JDot(twistMeasure, aAxisY);
        const float error = (float)atan2((double)y, (double)x);
        float3 jB = make_float3(worldAxisA.x + worldAxisB.x, worldAxisA.y + worldAxisB.y, worldAxisA.z + worldAxisB.z);
        if (JDot(jB, jB) >= 1e-7f) {  // else the child leaves the solver this step, impulse kept
            jB = JNormalize(jB);
            const float3 jA = make_float3(-jB.x, -jB.y, -jB.z);
            float erp, softness;
            JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
            const float bias = Clampf(-error * erp, -maxCorr, maxCorr);
            const float entryA = A.dynamic ? JDot(JTransform(jA, JInertia(A.s)), jA) : 0.f;
            const float entryB = B.dynamic ? JDot(JTransform(jB, JInertia(B.s)), jB) : 0.f;
            const float vti = 1 / (softness + entryA + entryB);
            j.L(kJOB, s).w = softness;
            j.L(kJW1, s) = make_float4(jB.x, jB.y, jB.z, vti);
            j.L(kJW2, s) = make_float4(bias, 0.f, 0.f, 0.f);
            st |= 1u << (kChildShift + 1);
        }
    } else if (kAdded && (active & kJChildAngular) && IsNoRotationType(type)) {
        // NoRotationJoint.Update (NoRotationJoint.cs:194-243).  Inputs: kJC1 / kJC2 the
        // initial orientations' conjugates; lanes kJL0..kJL2 the 3x3 effective mass and
        // the bias, kJOB.w the softness.
        float4 quaternionA = JQMul(A.q, ji.L(kJC1, si));
        float4 quaternionB = JQMul(B.q, ji.L(kJC2, si));
        quaternionB = make_float4(-quaternionB.x, -quaternionB.y, -quaternionB.z, quaternionB.w);
        float4 intermediate = JQMul(quaternionA, quaternionB);
        float3 axis;
        float angle;
        JAxisAngle(intermediate, axis, angle);
        float ex = axis.x * angle, ey = axis.y * angle, ez = axis.z * angle;
        float erp, softness;
        JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
        erp = -erp;
        float bx = erp * ex, by = erp * ey, bz = erp * ez;
        float length = bx * bx + by * by + bz * bz;
        if (length > maxCorrSq) {
            float multiplier = maxCorr / SqrtOfFloat(length);
            bx *= multiplier; by *= multiplier; bz *= multiplier;
        }
        const JM3 ia = JInertia(A.s), ib = JInertia(B.s);  // Matrix3x3.Add, whatever the connections
        JM3 k = {ia.M11 + ib.M11, ia.M12 + ib.M12, ia.M13 + ib.M13, ia.M21 + ib.M21, ia.M22 + ib.M22,
                 ia.M23 + ib.M23, ia.M31 + ib.M31, ia.M32 + ib.M32, ia.M33 + ib.M33};
        k.M11 += softness;
        k.M22 += softness;
        k.M33 += softness;
        JM3 mass = JInvert(k);
        j.L(kJOB, s).w = softness;
        j.L(kJL0, s) = make_float4(mass.M11, mass.M12, mass.M13, mass.M21);
        j.L(kJL1, s) = make_float4(mass.M22, mass.M23, mass.M31, mass.M32);
        j.L(kJL2, s) = make_float4(mass.M33, bx, by, bz);
        st |= 1u << (kChildShift + 1);
    } else if (kAdded && (active & kJChildAngular) && IsSwivelType(type)) {
        // SwivelHingeAngularJoint.Update (SwivelHingeAngularJoint.cs:222-270).  Inputs: the
        // hinge axis (kJAXA, A's frame) and the twist axis (kJAXB, B's frame).  Lanes: kJW1
        // jacobianA + velocityToImpulse, kJW2.x bias, kJOB.w softness (jacobianB = -jacobianA).
        const float3 hinge = JTransform(JXYZ(axa), A.R), twist = JTransform(JXYZ(axb), B.R);
        const float error = JDot(hinge, twist);
        float erp, softness;
        JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
        const float bias = Clampf(error * erp, -maxCorr, maxCorr);
        float3 jA = JCross(hinge, twist);
        const float length = JDot(jA, jA);
        if (length > 1e-7f) {
            const float inverse = 1 / SqrtOfFloat(length);  // Vector3.Divide (Vector3.cs:175-181)
            jA = make_float3(jA.x * inverse, jA.y * inverse, jA.z * inverse);
        } else {
            jA = make_float3(0.f, 0.f, 0.f);
        }
        const float3 jB = make_float3(-jA.x, -jA.y, -jA.z);
        const float entryA = A.dynamic ? JDot(JTransform(jA, JInertia(A.s)), jA) : 0.f;
        const float entryB = B.dynamic ? JDot(JTransform(jB, JInertia(B.s)), jB) : 0.f;
        const float vti = 1 / (softness + entryA + entryB);
        j.L(kJOB, s).w = softness;
        j.L(kJW1, s) = make_float4(jA.x, jA.y, jA.z, vti);
        j.L(kJW2, s) = make_float4(bias, 0.f, 0.f, 0.f);
        st |= 1u << (kChildShift + 1);
    } else if (active & kJChildAngular) {
        // RevoluteAngularJoint.Update (RevoluteAngularJoint.cs:226-289)
        float3 wA = JTransform(JXYZ(axa), A.R), wB = JTransform(JXYZ(axb), B.R);
        float3 c1 = JTransform(JXYZ(ji.L(kJC1, si)), A.R), c2 = JTransform(JXYZ(ji.L(kJC2, si)), A.R);
        float3 e3 = JCross(wA, wB);
        float errX = JDot(e3, c1), errY = JDot(e3, c2);
        float erp, softness;
        JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
        erp = -erp;
        float bx = erp * errX, by = erp * errY;
        float length = bx * bx + by * by;
        if (length > maxCorrSq) {
            float multiplier = maxCorr / SqrtOfFloat(length);
            bx *= multiplier; by *= multiplier;
        }
        float3 a1, a2;
        if (A.dynamic && B.dynamic) {
            JM3 ia = JInertia(A.s), ib = JInertia(B.s);
            JM3 sum = {ia.M11 + ib.M11, ia.M12 + ib.M12, ia.M13 + ib.M13, ia.M21 + ib.M21, ia.M22 + ib.M22,
                       ia.M23 + ib.M23, ia.M31 + ib.M31, ia.M32 + ib.M32, ia.M33 + ib.M33};
            a1 = JTransform(c1, sum);
            a2 = JTransform(c2, sum);
        } else if (A.dynamic) {
            JM3 ia = JInertia(A.s);
            a1 = JTransform(c1, ia);
            a2 = JTransform(c2, ia);
        } else {
            JM3 ib = JInertia(B.s);
            a1 = JTransform(c1, ib);
            a2 = JTransform(c2, ib);
        }
        float m11 = JDot(a1, c1), m12 = JDot(a1, c2), m21 = JDot(a2, c1), m22 = JDot(a2, c2);
        m11 += softness;
        m22 += softness;
        // Matrix2x2.Invert (Matrix2x2.cs:160-174), then Negate (:259-273)
        float d = 1 / (m11 * m22 - m12 * m21);
        float i11 = m22 * d, i12 = -m12 * d, i21 = -m21 * d, i22 = m11 * d;
        j.L(kJOB, s).w = softness;
        j.L(kJW1, s) = make_float4(c1.x, c1.y, c1.z, bx);
        j.L(kJW2, s) = make_float4(c2.x, c2.y, c2.z, by);
        j.L(kJE, s) = make_float4(-i11, -i12, -i21, -i22);
        st |= 1u << (kChildShift + 1);
    }
    if (active & kJChildLimit) {
        const float bounciness = ji.L(kJC1, si).w, threshold = ji.L(kJC2, si).w;
        float erp, softness;
        bool on = true;
        if (kAdded && type == BEPUGPU_JOINT_TWIST_LIMIT) {
            // TwistLimit.Update (TwistLimit.cs:238-366).  Inputs: basis A primary / x / y
            // (kJAXA, kJC1, kJC2), basis B primary / x (kJAXB, kJBX), kJTRIG.x the minimum
            // angle and .y GetDistanceFromMinimum(maximum).  Lanes: kJL0 jacobianA +
            // softness, kJL2 bias, -, velocityToImpulse; impulse kJACC1.y, error kJACC1.w.
            const float4 trig = ji.L(kJTRIG, si);
            const float minimumAngle = trig.x, distanceFromMaximum = trig.y;
            const float3 pA = JTransform(JXYZ(axa), A.R), xA = JTransform(JXYZ(ji.L(kJC1, si)), A.R);
            const float3 yA = JTransform(JXYZ(ji.L(kJC2, si)), A.R);
            const float3 pB = JTransform(JXYZ(axb), B.R), xB = JTransform(JXYZ(ji.L(kJBX, si)), B.R);
            const float4 rotation = JQuatBetween(pB, pA);
            const float3 twistMeasure = QTransform(xB.x, xB.y, xB.z, rotation);
            const float y = JDot(twistMeasure, yA), x = JDot(twistMeasure, xA);
            const float angle = (float)atan2((double)y, (double)x);
            // GetDistanceFromMinimum (:341-357)
            float distanceFromCurrent;
            if (minimumAngle > 0)
                distanceFromCurrent = angle >= minimumAngle ? angle - minimumAngle : 6.28318548f - minimumAngle + angle;
            else
                distanceFromCurrent = angle < minimumAngle ? 6.28318548f - minimumAngle + angle : angle - minimumAngle;
            if (distanceFromCurrent < distanceFromMaximum) {
                on = false;
                acc1.y = 0.f;
                acc1.w = 0.f;
            } else {
                float3 jv = make_float3(pA.x + pB.x, pA.y + pB.y, pA.z + pB.z);
                if (JDot(jv, jv) < 1e-7f) {
                    on = false;  // aligned axes: impulse and error stay
                } else {
                    jv = JNormalize(jv);
                    const float3 nv = make_float3(-jv.x, -jv.y, -jv.z);
                    const float3 jA = acc1.w > 0 ? nv : jv, jB = acc1.w > 0 ? jv : nv;
                    const float errorFromMin = 6.28318548f - distanceFromCurrent;
                    const float errorFromMax = distanceFromCurrent - distanceFromMaximum;
                    const float error = errorFromMax > errorFromMin ? errorFromMin : -errorFromMax;
                    acc1.w = error;
                    JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
                    float bias = Minf(Maxf(0, fabsf(error) - margin) * erp, maxCorr);
                    if (bounciness > 0) {
                        float rel = A.s.wx * jA.x + A.s.wy * jA.y + A.s.wz * jA.z;
                        const float dot = B.s.wx * jB.x + B.s.wy * jB.y + B.s.wz * jB.z;
                        rel += dot;
                        bias = Maxf(bias, JBounce(-rel, threshold, bounciness));
                    }
                    const float entryA = A.dynamic ? JDot(JTransform(jA, JInertia(A.s)), jA) : 0.f;
                    const float entryB = B.dynamic ? JDot(JTransform(jB, JInertia(B.s)), jB) : 0.f;
                    const float v2i = 1 / (softness + entryA + entryB);
                    j.L(kJL0, s) = make_float4(jA.x, jA.y, jA.z, softness);
                    j.L(kJL2, s) = make_float4(bias, 0.f, v2i, 0.f);
                }
            }
        } else if (kAdded && IsAngularMotorType(type)) {
            // AngularMotor.Update (AngularMotor.cs:248-312); SingleEntityAngularMotor.Update
            // (SingleEntityAngularMotor.cs:150-213) on body A alone: its servo error is
            // goal * conjugate(basis), its corrective velocity positive.  Inputs: basis primary / x / y
            // (kJAXA, kJC1, kJC2), the servo goal kJTA (x y z w), the goal velocity kJLA.xyz,
            // kJTRIG velocity softness, base corrective speed, maximum force, servo max corrective
            // velocity squared; kJAXB.w 1 in servo mode.  Lanes: kJL0..kJL2 the effective mass
            // and the bias velocity, kJOA used softness, maxForceDt, its square.  Impulse kJACC0.xyz.
            const float4 trig = ji.L(kJTRIG, si);
            const bool servo = axb.w != 0.f;
            const float3 primary = JTransform(JXYZ(axa), A.R), xAxis = JTransform(JXYZ(ji.L(kJC1, si)), A.R);
            const float3 yAxis = JTransform(JXYZ(ji.L(kJC2, si)), A.R);
            const float inverseDt = 1 / p.dt;
            float usedSoftness;
            float3 bias;
            const bool single = type == BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR;
            if (servo) {
                const float4 worldBasis = JQFromRows(xAxis, yAxis, primary);
                float4 error;
                if (single) {
                    error = JQMul(ji.L(kJTA, si), make_float4(-worldBasis.x, -worldBasis.y, -worldBasis.z, worldBasis.w));
                } else {
                    const float4 bTarget = JQConcat(ji.L(kJTA, si), worldBasis);
                    const float4 conj = make_float4(-bTarget.x, -bTarget.y, -bTarget.z, bTarget.w);
                    error = JQConcat(conj, B.q);
                }
                JSpring(stiffness, damping, p.dt, inverseDt, erp, usedSoftness);
                float3 axis;
                float angle;
                JAxisAngle(error, axis, angle);
                if (angle > 1e-5f) {
                    float velocity = Minf(trig.y, angle * inverseDt) + angle * erp;
                    if (!single) velocity = -velocity;
                    bias = make_float3(axis.x * velocity, axis.y * velocity, axis.z * velocity);
                    const float length = bias.x * bias.x + bias.y * bias.y + bias.z * bias.z;
                    if (length > trig.w) {
                        const float multiplier = maxCorr / SqrtOfFloat(length);
                        bias = make_float3(bias.x * multiplier, bias.y * multiplier, bias.z * multiplier);
                    }
                } else {
                    bias = make_float3(0.f, 0.f, 0.f);
                }
            } else {
                usedSoftness = trig.x * inverseDt;
                const float3 g = JXYZ(la);
                bias = make_float3(g.x * xAxis.x + g.y * yAxis.x + g.z * primary.x,
                                   g.x * xAxis.y + g.y * yAxis.y + g.z * primary.y,
                                   g.x * xAxis.z + g.y * yAxis.z + g.z * primary.z);
            }
            JM3 k = JInertia(A.s);  // Matrix3x3.Add of both connections' (whatever they are) for two
            if (!single) {
                const JM3 ib = JInertia(B.s);
                k = {k.M11 + ib.M11, k.M12 + ib.M12, k.M13 + ib.M13, k.M21 + ib.M21, k.M22 + ib.M22,
                     k.M23 + ib.M23, k.M31 + ib.M31, k.M32 + ib.M32, k.M33 + ib.M33};
            }
            k.M11 += usedSoftness;
            k.M22 += usedSoftness;
            k.M33 += usedSoftness;
            const JM3 mass = JInvert(k);
            float maxForceDt = 3.40282347e+38f, maxForceDtSquared = 3.40282347e+38f;
            if (trig.z < 3.40282347e+38f) {
                maxForceDt = trig.z * p.dt;
                maxForceDtSquared = maxForceDt * maxForceDt;
            }
            j.L(kJL0, s) = make_float4(mass.M11, mass.M12, mass.M13, mass.M21);
            j.L(kJL1, s) = make_float4(mass.M22, mass.M23, mass.M31, mass.M32);
            j.L(kJL2, s) = make_float4(mass.M33, bias.x, bias.y, bias.z);
            j.L(kJOA, s) = make_float4(usedSoftness, maxForceDt, maxForceDtSquared, 0.f);
        } else if (kAdded && type == BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR) {
            // SingleEntityLinearMotor.Update (SingleEntityLinearMotor.cs:210-268).  Inputs: the
            // local point kJLA, the servo goal kJLB.xyz, the goal velocity kJAXA.xyz, kJTRIG and
            // kJAXB.w as the angular motor's.  Lanes: kJL0..kJL2 effective mass and bias, kJOA
            // used softness, maxForceDt, its square, kJOB.xyz r.  Impulse kJACC0.xyz; the used
            // softness is kept in kJACC1.x (the servo leaves it while the point is at its goal).
            const float4 trig = ji.L(kJTRIG, si);
            const bool servo = axb.w != 0.f;
            const float3 r = JTransform(JXYZ(la), A.R);
            const float3 wp = make_float3(r.x + A.pos.x, r.y + A.pos.y, r.z + A.pos.z);
            const float updateRate = 1 / p.dt;
            float usedSoftness = acc1.x;
            float3 bias;
            if (servo) {
                const float3 goal = JXYZ(lb);
                const float3 error = make_float3(goal.x - wp.x, goal.y - wp.y, goal.z - wp.z);
                const float sep = SqrtOfFloat(error.x * error.x + error.y * error.y + error.z * error.z);
                if (sep > 1e-5f) {
                    JSpring(stiffness, damping, p.dt, updateRate, erp, usedSoftness);
                    const float cs = Minf(trig.y, sep * updateRate) + sep * erp;
                    const float f = cs / sep;
                    bias = make_float3(error.x * f, error.y * f, error.z * f);
                    const float length = bias.x * bias.x + bias.y * bias.y + bias.z * bias.z;
                    if (length > trig.w) {
                        const float multiplier = maxCorr / SqrtOfFloat(length);
                        bias = make_float3(bias.x * multiplier, bias.y * multiplier, bias.z * multiplier);
                    }
                } else {
                    bias = make_float3(0.f, 0.f, 0.f);
                }
            } else {
                usedSoftness = trig.x * updateRate;
                bias = JXYZ(axa);
            }
            acc1.x = usedSoftness;
            float maxForceDt = 3.40282347e+38f, maxForceDtSquared = 3.40282347e+38f;
            if (trig.z < 3.40282347e+38f) {
                maxForceDt = trig.z * p.dt;
                maxForceDtSquared = maxForceDt * maxForceDt;
            }
            const JM3 rx = JCrossMatrix(r);
            JM3 k = JSub(JScale(A.s.invMass), JMul(JMul(rx, JInertia(A.s)), rx));
            k.M11 += usedSoftness;
            k.M22 += usedSoftness;
            k.M33 += usedSoftness;
            const JM3 mass = JInvert(k);
            j.L(kJL0, s) = make_float4(mass.M11, mass.M12, mass.M13, mass.M21);
            j.L(kJL1, s) = make_float4(mass.M22, mass.M23, mass.M31, mass.M32);
            j.L(kJL2, s) = make_float4(mass.M33, bias.x, bias.y, bias.z);
            j.L(kJOA, s) = make_float4(usedSoftness, maxForceDt, maxForceDtSquared, 0.f);
            j.L(kJOB, s) = make_float4(r.x, r.y, r.z, 0.f);
        } else if (kAdded && IsSpeedLimitType(type)) {
            // MaximumLinearSpeedConstraint / MaximumAngularSpeedConstraint.Update
            // (MaximumLinearVelocityConstraint.cs:177-193 and the angular file's).  Inputs: kJTRIG
            // maximum speed, maximum force, softness.  Lanes (linear): kJL0 effective mass, used
            // softness, maxForceDt, its square; kJL1 maximum speed, its square.  (Angular): kJL0
            // used softness, maxForceDt, its square, maximum speed; kJL1 / kJL2 / kJOA.x the
            // effective mass matrix; kJOA.y the maximum speed squared.  Impulse kJACC0.xyz.
            const float4 trig = ji.L(kJTRIG, si);
            const float usedSoftness = trig.z / p.dt;
            float maxForceDt = 3.40282347e+38f, maxForceDtSquared = 3.40282347e+38f;
            if (trig.y < 3.40282347e+38f) {
                maxForceDt = trig.y * p.dt;
                maxForceDtSquared = maxForceDt * maxForceDt;
            }
            const float maxSpeedSquared = trig.x * trig.x;
            if (type == BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED) {
                const float mass = 1 / (A.s.invMass + usedSoftness);
                j.L(kJL0, s) = make_float4(mass, usedSoftness, maxForceDt, maxForceDtSquared);
                j.L(kJL1, s) = make_float4(trig.x, maxSpeedSquared, 0.f, 0.f);
            } else {
                JM3 m = JInertia(A.s);
                m.M11 += usedSoftness;
                m.M22 += usedSoftness;
                m.M33 += usedSoftness;
                const JM3 inv = JInvert(m);
                j.L(kJL0, s) = make_float4(usedSoftness, maxForceDt, maxForceDtSquared, trig.x);
                j.L(kJL1, s) = make_float4(inv.M11, inv.M12, inv.M13, inv.M21);
                j.L(kJL2, s) = make_float4(inv.M22, inv.M23, inv.M31, inv.M32);
                j.L(kJOA, s) = make_float4(inv.M33, maxSpeedSquared, 0.f, 0.f);
            }
        } else if (kAdded && IsMotorType(type)) {
            // RevoluteMotor.Update (RevoluteMotor.cs:243-290), TwistMotor.Update (TwistMotor.cs:182-224),
            // LinearAxisMotor.Update (LinearAxisMotor.cs:285-368).  Inputs: kJTRIG wrapped servo
            // goal (the linear motor's as given), goal velocity, velocity softness, base corrective
            // speed; kJBX.w maximum force; kJAXB.w 1 in servo mode; axes as the limits of the same
            // kind take them.  Lanes: kJL0 jacobian (linear A) + used softness; angular motors
            // kJL2 = signed bias (the revolute motor's negated: its solve subtracts it), -,
            // velocityToImpulse, maxForceDt; the linear motor kJL1 jAngularA + bias, kJL2
            // jAngularB + mass, kJOA.x maxForceDt.  Impulse kJACC1.y.
            const float4 trig = ji.L(kJTRIG, si);
            const bool servo = axb.w != 0.f;
            const float maxForce = ji.L(kJBX, si).w;
            const float updateRate = p.updateRate;
            const float maxForceDt = maxForce < 3.40282347e+38f ? maxForce * p.dt : 3.40282347e+38f;
            auto servoBias = [&](float error, float absErrorOverDt, float errorReduction) {
                float bias = JSign(error) * Minf(trig.w, absErrorOverDt) + error * errorReduction;
                return Clampf(bias, -maxCorr, maxCorr);
            };
            float usedSoftness, bias;
            if (type == BEPUGPU_JOINT_LINEAR_AXIS_MOTOR) {
                const float3 offA = JTransform(JXYZ(la), A.R), offB = JTransform(JXYZ(lb), B.R);
                const float3 anchorA = make_float3(offA.x + A.pos.x, offA.y + A.pos.y, offA.z + A.pos.z);
                const float3 anchorB = make_float3(offB.x + B.pos.x, offB.y + B.pos.y, offB.z + B.pos.z);
                const float3 rA = make_float3(anchorB.x - A.pos.x, anchorB.y - A.pos.y, anchorB.z - A.pos.z);
                const float3 axis = JTransform(JXYZ(ji.L(kJBP, si)), A.R);
                if (servo) {
                    const float3 sep = make_float3(anchorB.x - anchorA.x, anchorB.y - anchorA.y, anchorB.z - anchorA.z);
                    float error = JDot(sep, axis);
                    error = error - trig.x;
                    const float absErrorOverDt = fabsf(error * updateRate);
                    JSpring(stiffness, damping, p.dt, updateRate, erp, usedSoftness);
                    bias = servoBias(error, absErrorOverDt, erp);
                } else {
                    bias = -trig.y;
                    usedSoftness = trig.z * updateRate;
                }
                const float3 jlb = make_float3(-axis.x, -axis.y, -axis.z);
                const float3 jaa = JCross(rA, axis), jab = JCross(offB, jlb);
                float entryA = 0, entryB = 0;
                if (A.dynamic) {
                    entryA = JDot(JTransform(jaa, JInertia(A.s)), jaa);
                    entryA += A.s.invMass;
                }
                if (B.dynamic) {
                    entryB = JDot(JTransform(jab, JInertia(B.s)), jab);
                    entryB += B.s.invMass;
                }
                const float mass = 1 / (entryA + entryB + usedSoftness);
                j.L(kJL0, s) = make_float4(axis.x, axis.y, axis.z, usedSoftness);
                j.L(kJL1, s) = make_float4(jaa.x, jaa.y, jaa.z, bias);
                j.L(kJL2, s) = make_float4(jab.x, jab.y, jab.z, mass);
                j.L(kJOA, s).x = maxForceDt;
            } else {
                float3 jA;
                float signedBias;
                if (type == BEPUGPU_JOINT_REVOLUTE_MOTOR) {
                    const float3 primary = JTransform(JXYZ(ji.L(kJBP, si)), A.R);
                    const float3 xAxis = JTransform(JXYZ(ji.L(kJBX, si)), A.R);
                    const float3 test = JTransform(JXYZ(ji.L(kJTA, si)), B.R);
                    if (servo) {
                        const float3 yAxis = JCross(primary, xAxis);
                        const float y = JDot(test, yAxis), x = JDot(test, xAxis);
                        const float angle = (float)atan2((double)y, (double)x);
                        const float error = JDistanceFromGoal(angle, trig.x);
                        const float absErrorOverDt = fabsf(error * updateRate);
                        JSpring(stiffness, damping, p.dt, updateRate, erp, usedSoftness);
                        bias = servoBias(error, absErrorOverDt, erp);
                    } else {
                        bias = trig.y;
                        usedSoftness = trig.z * updateRate;
                    }
                    jA = primary;
                    signedBias = -bias;
                } else {
                    const float3 pA = JTransform(JXYZ(axa), A.R), xA = JTransform(JXYZ(ji.L(kJC1, si)), A.R);
                    const float3 yA = JTransform(JXYZ(ji.L(kJC2, si)), A.R);
                    const float3 pB = JTransform(JXYZ(axb), B.R), xB = JTransform(JXYZ(ji.L(kJBX, si)), B.R);
                    if (servo) {
                        const float4 rotation = JQuatBetween(pB, pA);
                        const float3 tm = QTransform(xB.x, xB.y, xB.z, rotation);
                        const float y = JDot(tm, yA), x = JDot(tm, xA);
                        const float angle = (float)atan2((double)y, (double)x);
                        const float error = JDistanceFromGoal(angle, trig.x);
                        const float absErrorOverDt = fabsf(error / p.dt);
                        JSpring(stiffness, damping, p.dt, updateRate, erp, usedSoftness);
                        bias = servoBias(error, absErrorOverDt, erp);
                    } else {
                        bias = trig.y;
                        usedSoftness = trig.z / p.dt;
                    }
                    float3 jv = make_float3(pA.x + pB.x, pA.y + pB.y, pA.z + pB.z);
                    if (JDot(jv, jv) < 1e-7f) {
                        on = false;  // aligned axes: the motor leaves the solver this step
                    } else {
                        jv = JNormalize(jv);
                        jA = make_float3(-jv.x, -jv.y, -jv.z);
                    }
                    signedBias = bias;
                }
                if (on) {
                    const float3 jB = make_float3(-jA.x, -jA.y, -jA.z);
                    const float entryA = A.dynamic ? JDot(JTransform(jA, JInertia(A.s)), jA) : 0.f;
                    const float entryB = B.dynamic ? JDot(JTransform(jB, JInertia(B.s)), jB) : 0.f;
                    const float vti = 1 / (usedSoftness + entryA + entryB);
                    j.L(kJL0, s) = make_float4(jA.x, jA.y, jA.z, usedSoftness);
                    j.L(kJL2, s) = make_float4(signedBias, 0.f, vti, maxForceDt);
                }
            }
        } else if (kAdded && type == BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT) {
            // EllipseSwingLimit.Update (EllipseSwingLimit.cs:162-308).  Inputs: basis primary /
            // x / y (kJAXA, kJC1, kJC2, A's frame), B's twist axis (kJAXB), kJTRIG.x / .y the
            // maximum angles.  Lanes: kJL0 jacobianA + softness, kJL2 bias, -,
            // velocityToImpulse; impulse (non-positive) kJACC1.y.
            const float4 trig = ji.L(kJTRIG, si);
            const float3 primary = JTransform(JXYZ(axa), A.R), xAxis = JTransform(JXYZ(ji.L(kJC1, si)), A.R);
            const float3 yAxis = JTransform(JXYZ(ji.L(kJC2, si)), A.R), twistB = JTransform(JXYZ(axb), B.R);
            const float4 rel = JQuatBetween(twistB, primary);
            float3 axis;
            float angle;
            JAxisAngle(rel, axis, angle);
            const float3 axisAngle = make_float3(axis.x * angle, axis.y * angle, axis.z * angle);
            const float angleX = JDot(axisAngle, xAxis), angleY = JDot(axisAngle, yAxis);
            const float maxX2 = trig.x * trig.x, maxY2 = trig.y * trig.y;
            float error = angleX * angleX * maxY2 + angleY * angleY * maxX2 - maxX2 * maxY2;
            if (error < 0) {
                on = false;
                acc1.y = 0.f;
            } else {
                const float tangentX = 2 * angleX / maxX2, tangentY = 2 * angleY / maxY2;
                const float4 conj = make_float4(-rel.x, -rel.y, -rel.z, rel.w);
                const float3 stX = QTransform(xAxis.x, xAxis.y, xAxis.z, conj);
                const float3 stY = QTransform(yAxis.x, yAxis.y, yAxis.z, conj);
                const float3 jA = make_float3(stX.x * tangentX + stY.x * tangentY, stX.y * tangentX + stY.y * tangentY,
                                              stX.z * tangentX + stY.z * tangentY);
                const float3 jB = make_float3(-jA.x, -jA.y, -jA.z);
                JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
                error = error - margin;
                float bias = Minf(Maxf(error, 0) * erp, maxCorr);
                if (bounciness > 0) {
                    float rv = A.s.wx * jA.x + A.s.wy * jA.y + A.s.wz * jA.z;
                    const float dot = B.s.wx * jB.x + B.s.wy * jB.y + B.s.wz * jB.z;
                    rv += dot;
                    bias = Maxf(bias, JBounce(rv, threshold, bounciness));
                }
                const float entryA = A.dynamic ? JDot(JTransform(jA, JInertia(A.s)), jA) : 0.f;
                const float entryB = B.dynamic ? JDot(JTransform(jB, JInertia(B.s)), jB) : 0.f;
                const float v2i = 1 / (softness + entryA + entryB);
                j.L(kJL0, s) = make_float4(jA.x, jA.y, jA.z, softness);
                j.L(kJL2, s) = make_float4(bias, 0.f, v2i, 0.f);
            }
        } else if (kAdded && IsLinearLimitType(type)) {
            // LinearAxisLimit.Update (LinearAxisLimit.cs:338-447).  Inputs: anchors kJLA / kJLB,
            // axis kJBP (A's frame), kJTRIG minimum, maximum, bounciness, bounce velocity
            // threshold.  Lanes at
            // LinearLimitLane: jLinearA + softness, jAngularA + bias, jAngularB + mass;
            // impulse kJACC1.z; state bit kJMinActive when violated below the minimum.
            const float4 trig = ji.L(kJTRIG, si);
            const float limitBounciness = trig.z, limitThreshold = trig.w;
            const float3 offA = JTransform(JXYZ(la), A.R), offB = JTransform(JXYZ(lb), B.R);
            const float3 anchorA = make_float3(offA.x + A.pos.x, offA.y + A.pos.y, offA.z + A.pos.z);
            const float3 anchorB = make_float3(offB.x + B.pos.x, offB.y + B.pos.y, offB.z + B.pos.z);
            const float3 rA = make_float3(anchorB.x - A.pos.x, anchorB.y - A.pos.y, anchorB.z - A.pos.z);
            const float3 axis = JTransform(JXYZ(ji.L(kJBP, si)), A.R);
            const float3 sep = make_float3(anchorB.x - anchorA.x, anchorB.y - anchorA.y, anchorB.z - anchorA.z);
            float u = JDot(sep, axis);
            if (u < trig.x) {
                u = trig.x - u;
            } else if (u > trig.y) {
                u = trig.y - u;
            } else {
                on = false;
                acc1.z = 0.f;
            }
            if (on) {
                u = -u;
                const float error = u > 0 ? Maxf(0, u - margin) : Minf(0, u + margin);  // u is never 0 here
                const float3 jlb = make_float3(-axis.x, -axis.y, -axis.z);
                const float3 jaa = JCross(rA, axis), jab = JCross(offB, jlb);
                JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
                float bias = Clampf(erp * error, -maxCorr, maxCorr);
                if (limitBounciness > 0) {
                    float rel = axis.x * A.s.vx + axis.y * A.s.vy + axis.z * A.s.vz;
                    float dot = jaa.x * A.s.wx + jaa.y * A.s.wy + jaa.z * A.s.wz;
                    rel += dot;
                    dot = jlb.x * B.s.vx + jlb.y * B.s.vy + jlb.z * B.s.vz;
                    rel += dot;
                    dot = jab.x * B.s.wx + jab.y * B.s.wy + jab.z * B.s.wz;
                    rel += dot;
                    if (u > 0 && -rel > limitThreshold)
                        bias = Maxf(bias, JBounce(-rel, limitThreshold, limitBounciness));
                    else if (u < 0 && rel > limitThreshold)
                        bias = Minf(bias, -JBounce(rel, limitThreshold, limitBounciness));
                }
                float entryA = 0, entryB = 0;
                if (A.dynamic) {
                    entryA = JDot(JTransform(jaa, JInertia(A.s)), jaa);
                    entryA += A.s.invMass;
                }
                if (B.dynamic) {
                    entryB = JDot(JTransform(jab, JInertia(B.s)), jab);
                    entryB += B.s.invMass;
                }
                const float mass = 1 / (entryA + entryB + softness);
                const int k0 = LinearLimitLane(type);
                j.L(k0, s) = make_float4(axis.x, axis.y, axis.z, softness);
                j.L(k0 + 1, s) = make_float4(jaa.x, jaa.y, jaa.z, bias);
                j.L(k0 + 2, s) = make_float4(jab.x, jab.y, jab.z, mass);
                if (u < 0) st |= kJMinActive;
            }
        } else if (type == BEPUGPU_JOINT_SWING_LIMIT) {
            // SwingLimit.Update (SwingLimit.cs:249-331)
            float3 wA = JTransform(JXYZ(axa), A.R), wB = JTransform(JXYZ(axb), B.R);
            float dot = JDot(wA, wB);
            const float minimumCosine = ji.L(kJBX, si).w;
            if (dot > minimumCosine) {
                on = false;
                acc1.y = 0.f;
            } else {
                float3 hinge = JCross(wA, wB);
                float lengthSquared = JDot(hinge, hinge);
                if (lengthSquared < 1e-7f) {
                    hinge = JCross(wA, make_float3(0.f, 1.f, 0.f));
                    lengthSquared = JDot(hinge, hinge);
                    if (lengthSquared < 1e-7f) hinge = JCross(wA, make_float3(1.f, 0.f, 0.f));
                }
                JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
                float error = minimumCosine - dot - margin;
                error = error > 0.f ? error : 0.f;  // Math.Max(0, x)
                float bias = Clampf(erp * error, -maxCorr, maxCorr);
                if (bounciness > 0) {
                    float rx = A.s.wx - B.s.wx, ry = A.s.wy - B.s.wy, rz = A.s.wz - B.s.wz;
                    float relativeSpeed = rx * hinge.x + ry * hinge.y + rz * hinge.z;
                    bias = Maxf(bias, JBounce(-relativeSpeed, threshold, bounciness));
                }
                float entryA = 0, entryB = 0;
                if (A.dynamic) entryA = JDot(JTransform(hinge, JInertia(A.s)), hinge);
                if (B.dynamic) entryB = JDot(JTransform(hinge, JInertia(B.s)), hinge);
                float v2i = 1 / (softness + entryA + entryB);
                j.L(kJL0, s) = make_float4(hinge.x, hinge.y, hinge.z, softness);
                j.L(kJL2, s) = make_float4(bias, 0.f, v2i, 0.f);
            }
        } else {
            // RevoluteLimit.Update (RevoluteLimit.cs:285-575)
            float3 primary = JTransform(JXYZ(ji.L(kJBP, si)), A.R), xAxis = JTransform(JXYZ(ji.L(kJBX, si)), A.R);
            float3 test = JTransform(JXYZ(ji.L(kJTA, si)), B.R);
            const float4 trig = ji.L(kJTRIG, si);
            // Matrix3x3.CreateFromAxisAngle (Matrix3x3.cs:1383-1406) with the
            // double sine and cosine of the constant angles taken at upload.
            float xx = primary.x * primary.x, yy = primary.y * primary.y, zz = primary.z * primary.z;
            float xy = primary.x * primary.y, xz = primary.x * primary.z, yz = primary.y * primary.z;
            auto rotate = [&](float sinAngle, float omc) {
                JM3 r;
                r.M11 = 1 + omc * (xx - 1);
                r.M21 = -primary.z * sinAngle + omc * xy;
                r.M31 = primary.y * sinAngle + omc * xz;
                r.M12 = primary.z * sinAngle + omc * xy;
                r.M22 = 1 + omc * (yy - 1);
                r.M32 = -primary.x * sinAngle + omc * yz;
                r.M13 = -primary.y * sinAngle + omc * xz;
                r.M23 = primary.x * sinAngle + omc * yz;
                r.M33 = 1 + omc * (zz - 1);
                return JTransform(xAxis, r);
            };
            float3 minN = rotate(trig.x, trig.y), maxN = rotate(trig.z, trig.w);
            float pMin = JDot(minN, test), pMax = JDot(maxN, test);
            const float span = ji.L(kJBP, si).w;
            float errX = 0, errY = 0;
            bool minOn = false, maxOn = false;
            if (span >= 3.14159274f) {
                if (pMax > 0 || pMin > 0) {
                    on = false;
                } else if (pMax > pMin) {
                    errY = -pMax; acc1.y = 0.f; maxOn = true;
                } else {
                    errX = -pMin; acc1.z = 0.f; minOn = true;
                }
            } else {
                if (pMax > 0 && pMin > 0) {
                    on = false;
                } else if (pMin <= 0 && pMax <= 0) {
                    errX = -pMin; errY = -pMax; minOn = maxOn = true;
                } else if (pMin <= 0) {
                    errX = -pMin; acc1.z = 0.f; minOn = true;
                } else {
                    errY = -pMax; acc1.y = 0.f; maxOn = true;
                }
            }
            if (!on) {
                acc1.y = 0.f;
                acc1.z = 0.f;
            } else {
                JSpring(stiffness, damping, p.dt, p.updateRate, erp, softness);
                float4 l0 = j.L(kJL0, s), l1 = j.L(kJL1, s), l2 = j.L(kJL2, s);
                float3 jMin = JXYZ(l0), jMax = JXYZ(l1);  // kept from earlier steps when a plane is off
                if (minOn) {
                    jMin = JCross(minN, test);
                    if (JDot(jMin, jMin) < 1e-7f) jMin = primary;
                    jMin = JNormalize(jMin);
                }
                if (maxOn) {
                    jMax = JCross(maxN, test);
                    if (JDot(jMax, jMax) < 1e-7f) jMax = primary;
                    jMax = JNormalize(jMax);
                }
                float3 jMinB = make_float3(-jMin.x, -jMin.y, -jMin.z), jMaxB = make_float3(-jMax.x, -jMax.y, -jMax.z);
                float biasX = l2.x, biasY = l2.y;
                if (minOn) {
                    biasX = Minf(Maxf(0, errX - margin) * erp, maxCorr);
                    if (bounciness > 0) {
                        float rel = A.s.wx * jMin.x + A.s.wy * jMin.y + A.s.wz * jMin.z;
                        float dot = B.s.wx * jMinB.x + B.s.wy * jMinB.y + B.s.wz * jMinB.z;
                        rel += dot;
                        biasX = Maxf(biasX, JBounce(-rel, threshold, bounciness));
                    }
                }
                if (maxOn) {
                    biasY = Minf(Maxf(0, errY - margin) * erp, maxCorr);
                    if (bounciness > 0) {
                        float rel = A.s.wx * jMax.x + A.s.wy * jMax.y + A.s.wz * jMax.z;
                        float dot = B.s.wx * jMaxB.x + B.s.wy * jMaxB.y + B.s.wz * jMaxB.z;
                        rel += dot;
                        biasY = Maxf(biasY, JBounce(-rel, threshold, bounciness));
                    }
                }
                float minEA = 0, minEB = 0, maxEA = 0, maxEB = 0;
                if (A.dynamic) {
                    JM3 ia = JInertia(A.s);
                    if (minOn) minEA = JDot(JTransform(jMin, ia), jMin);
                    if (maxOn) maxEA = JDot(JTransform(jMax, ia), jMax);
                }
                if (B.dynamic) {
                    JM3 ib = JInertia(B.s);
                    if (minOn) minEB = JDot(JTransform(jMinB, ib), jMinB);
                    if (maxOn) maxEB = JDot(JTransform(jMaxB, ib), jMaxB);
                }
                float v2iX = 1 / (softness + minEA + minEB);
                float v2iY = 1 / (softness + maxEA + maxEB);
                j.L(kJL0, s) = make_float4(jMin.x, jMin.y, jMin.z, softness);
                j.L(kJL1, s) = make_float4(jMax.x, jMax.y, jMax.z, 0.f);
                j.L(kJL2, s) = make_float4(biasX, biasY, v2iX, v2iY);
                st |= (minOn ? kJMinActive : 0u) | (maxOn ? kJMaxActive : 0u);
            }
        }
        if (on) st |= 1u << (kChildShift + 2);
    }
    j.L(kJACC1, s) = acc1;
    // A continuation's visits belong to its group's record: its own slot never
    // carries kGroupActive, so the sweeps pass over it.  The group's first child
    // is active whenever the group is (the constructors' IsActive = true), so the
    // group record's kGroupActive already stands for the whole group here.
    if ((st & (7u << kChildShift)) && !(st & kJIsContinuation)) st |= kGroupActive;
    j.state[s] = make_uint2(st, 0u);
}

template <bool kAdded>
__device__ __forceinline__ void PrestepJoint(const JointSoA& j, const BodySoA& b, int s, const StepParams& p) {
    const int4 h = j.head[s];
    PrestepJointIO<kAdded>(j, s, j, s, GlobalBodies{b}, h.x, h.y, p);
}

// ---------------------------------------------------------- warm start --
// ExclusiveUpdate of every active child of one record in order.
template <bool kAdded>
__device__ __forceinline__ void WarmJointChildren(const JointSoA& j, int s, BodyState& A, BodyState& B, uint32_t st,
                                                  int type) {
    const bool dynA = st & kDynA, dynB = st & kDynB;
    const float4 acc0 = j.L(kJACC0, s), acc1 = j.L(kJACC1, s);
    if (kAdded && (st & (1u << kChildShift)) && IsPointOnLineType(type)) {
        // PointOnLineJoint.ExclusiveUpdate (PointOnLineJoint.cs:440-463)
        ApplyPointOnLine(j.L(kJOA, s), j.L(kJOB, s), j.L(kJM0, s), j.L(kJM1, s), acc0.x, acc0.y, dynA, dynB, A, B);
    } else if (kAdded && (st & (1u << kChildShift)) && IsPointOnPlaneType(type)) {
        // PointOnPlaneJoint.ExclusiveUpdate (PointOnPlaneJoint.cs:308-328)
        const float4 m0 = j.L(kJM0, s), m1 = j.L(kJM1, s), m2 = j.L(kJM2, s);
        const float a = acc0.x;
        const float ix = m0.x * a, iy = m0.y * a, iz = m0.z * a;
        if (dynA) {
            ApplyLinear(A, ix, iy, iz);
            ApplyAngular(A, m1.x * a, m1.y * a, m1.z * a);
        }
        if (dynB) {
            ApplyLinear(B, -ix, -iy, -iz);
            ApplyAngular(B, m2.x * a, m2.y * a, m2.z * a);
        }
    } else if (kAdded && (st & (1u << kChildShift)) && IsDistanceType(type)) {
        // DistanceJoint / DistanceLimit.ExclusiveUpdate (DistanceJoint.cs:354-380)
        const float4 m0 = j.L(kJM0, s), m1 = j.L(kJM1, s), m2 = j.L(kJM2, s);
        const float a = acc0.x;
        if (dynA) {
            ApplyLinear(A, m0.x * a, m0.y * a, m0.z * a);
            ApplyAngular(A, m1.x * a, m1.y * a, m1.z * a);
        }
        if (dynB) {
            ApplyLinear(B, -m0.x * a, -m0.y * a, -m0.z * a);
            ApplyAngular(B, m2.x * a, m2.y * a, m2.z * a);
        }
    } else if (st & (1u << kChildShift)) {
        // BallSocketJoint.ExclusiveUpdate (BallSocketJoint.cs:285-311)
        const float3 offA = JXYZ(j.L(kJOA, s)), offB = JXYZ(j.L(kJOB, s));
        const float3 acc = make_float3(acc0.x, acc0.y, acc0.z);
        if (dynA) {
            float3 lin = make_float3(-acc.x, -acc.y, -acc.z);
            ApplyLinear(A, lin.x, lin.y, lin.z);
            float3 t = JCross(offA, lin);
            ApplyAngular(A, t.x, t.y, t.z);
        }
        if (dynB) {
            ApplyLinear(B, acc.x, acc.y, acc.z);
            float3 t = JCross(offB, acc);
            ApplyAngular(B, t.x, t.y, t.z);
        }
    }
    if (kAdded && (st & (2u << kChildShift)) && IsTwistType(type)) {
        // TwistJoint.ExclusiveUpdate (TwistJoint.cs:302-317)
        const float4 w1 = j.L(kJW1, s);
        const float a = acc0.w;
        if (dynA) ApplyAngular(A, -w1.x * a, -w1.y * a, -w1.z * a);
        if (dynB) ApplyAngular(B, w1.x * a, w1.y * a, w1.z * a);
    } else if (kAdded && (st & (2u << kChildShift)) && IsNoRotationType(type)) {
        // NoRotationJoint.ExclusiveUpdate (NoRotationJoint.cs:245-259)
        if (dynA) ApplyAngular(A, acc0.w, acc1.x, acc1.y);
        if (dynB) ApplyAngular(B, -acc0.w, -acc1.x, -acc1.y);
    } else if (kAdded && (st & (2u << kChildShift)) && IsSwivelType(type)) {
        // SwivelHingeAngularJoint.ExclusiveUpdate (SwivelHingeAngularJoint.cs:272-287)
        const float4 w1 = j.L(kJW1, s);
        const float a = acc0.w;
        if (dynA) ApplyAngular(A, w1.x * a, w1.y * a, w1.z * a);
        if (dynB) ApplyAngular(B, -w1.x * a, -w1.y * a, -w1.z * a);
    } else if (st & (2u << kChildShift)) {
        // RevoluteAngularJoint.ExclusiveUpdate (RevoluteAngularJoint.cs:291-310)
        const float3 c1 = JXYZ(j.L(kJW1, s)), c2 = JXYZ(j.L(kJW2, s));
        float ix = c1.x * acc0.w + c2.x * acc1.x, iy = c1.y * acc0.w + c2.y * acc1.x,
              iz = c1.z * acc0.w + c2.z * acc1.x;
        if (dynA) ApplyAngular(A, ix, iy, iz);
        if (dynB) ApplyAngular(B, -ix, -iy, -iz);
    }
    if (st & (4u << kChildShift)) {
        const float4 l0 = j.L(kJL0, s);
        if (kAdded && type == BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR) {
            // SingleEntityLinearMotor.ExclusiveUpdate (SingleEntityLinearMotor.cs:270-276)
            const float3 r = JXYZ(j.L(kJOB, s)), a = make_float3(acc0.x, acc0.y, acc0.z);
            ApplyLinear(A, a.x, a.y, a.z);
            const float3 t = JCross(r, a);
            ApplyAngular(A, t.x, t.y, t.z);
        } else if (kAdded && IsAngularMotorType(type)) {
            // AngularMotor.ExclusiveUpdate (AngularMotor.cs:314-326), SingleEntityAngularMotor's
            // (:215-218; B is the world there)
            if (dynA) ApplyAngular(A, acc0.x, acc0.y, acc0.z);
            if (dynB) ApplyAngular(B, -acc0.x, -acc0.y, -acc0.z);
        } else if (kAdded && IsSpeedLimitType(type)) {
            // ExclusiveUpdate (MaximumLinearVelocityConstraint.cs:195-199): no warm start, the
            // accumulated impulse starts the iterations from zero
            j.L(kJACC0, s) = make_float4(0.f, 0.f, 0.f, acc0.w);
        } else if (kAdded && type == BEPUGPU_JOINT_LINEAR_AXIS_MOTOR) {
            // LinearAxisMotor.ExclusiveUpdate (LinearAxisMotor.cs:370-390)
            const float4 jaa = j.L(kJL1, s), jab = j.L(kJL2, s);
            const float a = acc1.y;
            if (dynA) {
                ApplyLinear(A, l0.x * a, l0.y * a, l0.z * a);
                ApplyAngular(A, jaa.x * a, jaa.y * a, jaa.z * a);
            }
            if (dynB) {
                ApplyLinear(B, -l0.x * a, -l0.y * a, -l0.z * a);
                ApplyAngular(B, jab.x * a, jab.y * a, jab.z * a);
            }
        } else if (kAdded && (type == BEPUGPU_JOINT_TWIST_LIMIT || type == BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT ||
                              type == BEPUGPU_JOINT_REVOLUTE_MOTOR || type == BEPUGPU_JOINT_TWIST_MOTOR)) {
            // TwistLimit.ExclusiveUpdate (TwistLimit.cs:368-383), EllipseSwingLimit's (:310-325),
            // RevoluteMotor's (RevoluteMotor.cs:292-307), TwistMotor's (TwistMotor.cs:255-270)
            const float a = acc1.y;
            if (dynA) ApplyAngular(A, l0.x * a, l0.y * a, l0.z * a);
            if (dynB) ApplyAngular(B, -l0.x * a, -l0.y * a, -l0.z * a);
        } else if (kAdded && IsLinearLimitType(type)) {
            // LinearAxisLimit.ExclusiveUpdate (LinearAxisLimit.cs:449-466)
            const int k0 = LinearLimitLane(type);
            const float4 ja = j.L(k0, s), jaa = j.L(k0 + 1, s), jab = j.L(k0 + 2, s);
            const float a = acc1.z;
            if (dynA) {
                ApplyLinear(A, ja.x * a, ja.y * a, ja.z * a);
                ApplyAngular(A, jaa.x * a, jaa.y * a, jaa.z * a);
            }
            if (dynB) {
                ApplyLinear(B, -ja.x * a, -ja.y * a, -ja.z * a);
                ApplyAngular(B, jab.x * a, jab.y * a, jab.z * a);
            }
        } else if (type == BEPUGPU_JOINT_SWING_LIMIT) {
            // SwingLimit.ExclusiveUpdate (SwingLimit.cs:333-347)
            float ix = l0.x * acc1.y, iy = l0.y * acc1.y, iz = l0.z * acc1.y;
            if (dynA) ApplyAngular(A, ix, iy, iz);
            if (dynB) ApplyAngular(B, -ix, -iy, -iz);
        } else {
            // RevoluteLimit.ExclusiveUpdate (RevoluteLimit.cs:577-620)
            const float4 l1 = j.L(kJL1, s);
            const bool minOn = st & kJMinActive, maxOn = st & kJMaxActive;
            if (dynA) {
                float ix = 0.f, iy = 0.f, iz = 0.f;
                if (minOn) { ix = l0.x * acc1.y; iy = l0.y * acc1.y; iz = l0.z * acc1.y; }
                if (maxOn) { ix = ix + l1.x * acc1.z; iy = iy + l1.y * acc1.z; iz = iz + l1.z * acc1.z; }
                ApplyAngular(A, ix, iy, iz);
            }
            if (dynB) {
                float ix = 0.f, iy = 0.f, iz = 0.f;
                if (minOn) { ix = -l0.x * acc1.y; iy = -l0.y * acc1.y; iz = -l0.z * acc1.y; }
                if (maxOn) { ix = ix + -l1.x * acc1.z; iy = iy + -l1.y * acc1.z; iz = iz + -l1.z * acc1.z; }
                ApplyAngular(B, ix, iy, iz);
            }
        }
    }
}

// SolverGroup.ExclusiveUpdate (SolverGroup.cs:103-109) over the group's
// children in Add order: the record's own, then those of its continuation
// records in the slots after it.
template <bool kAdded>
__device__ __forceinline__ void WarmJoint(const JointSoA& j, int s, BodyState& A, BodyState& B, uint32_t st,
                                          int type) {
    WarmJointChildren<kAdded>(j, s, A, B, st, type);
    if (kAdded && (st & kJHasNext))
        for (int u = s + 1;; u++) {
            const uint32_t cst = j.state[u].x;
            WarmJointChildren<kAdded>(j, u, A, B, cst, JointType(cst));
            if (!(cst & kJHasNext)) break;
        }
}

// -------------------------------------------------------------- solve --
// SolverGroup.SolveUpdateable (SolverGroup.cs:117-150) on each active child of
// one record: st / zeros are the record's state words, activeConstraints the
// group's count.  A child's currentIterations equals the group's while the
// child stays active (both restart at the Update, SolverGroup.cs:70-76), so
// the group's iteration check covers the child's.
template <bool kAdded>
__device__ __forceinline__ void SolveJointChildren(const JointSoA& j, int s, BodyState& A, BodyState& B,
                                                   uint32_t& st, uint32_t& zeros, int& activeConstraints, int type,
                                                   const StepParams& p) {
    const bool dynA = st & kDynA, dynB = st & kDynB;
    auto account = [&](int c, float r) {
        uint32_t z = (zeros >> (4 * c)) & 0xfu;
        if (r < p.minimumImpulse) {
            z++;
            if ((int)z > p.minimumIterationCount) st &= ~(1u << (kChildShift + c));
            else activeConstraints++;
        } else {
            z = 0;
            activeConstraints++;
        }
        zeros = (zeros & ~(0xfu << (4 * c))) | ((z & 0xfu) << (4 * c));
    };
    float4 acc0 = j.L(kJACC0, s), acc1 = j.L(kJACC1, s);
    if (kAdded && (st & (1u << kChildShift)) && IsPointOnLineType(type)) {
        // PointOnLineJoint.SolveIteration (PointOnLineJoint.cs:247-355)
        const float4 oa = j.L(kJOA, s), ob = j.L(kJOB, s), m0 = j.L(kJM0, s), m1 = j.L(kJM1, s),
                     m2 = j.L(kJM2, s);
        float ax = A.wy * oa.z - A.wz * oa.y, ay = A.wz * oa.x - A.wx * oa.z, az = A.wx * oa.y - A.wy * oa.x;
        ax = ax + A.vx; ay = ay + A.vy; az = az + A.vz;
        float bx = B.wy * ob.z - B.wz * ob.y, by = B.wz * ob.x - B.wx * ob.z, bz = B.wx * ob.y - B.wy * ob.x;
        bx = bx + B.vx; by = by + B.vy; bz = bz + B.vz;
        const float dvx = ax - bx, dvy = ay - by, dvz = az - bz;
        float lx = dvx * m0.x + dvy * m0.y + dvz * m0.z;
        float ly = dvx * m1.x + dvy * m1.y + dvz * m1.z;
        lx += m2.z + oa.w * acc0.x;
        ly += m2.w + oa.w * acc0.y;
        const float x = lx * m0.w + ly * m2.x, y = lx * m1.w + ly * m2.y;  // Matrix2x2.Transform
        acc0.x = x + acc0.x;
        acc0.y = y + acc0.y;
        ApplyPointOnLine(oa, ob, m0, m1, x, y, dynA, dynB, A, B);
        account(0, fabsf(x) + fabsf(y));
    } else if (kAdded && (st & (1u << kChildShift)) && IsPointOnPlaneType(type)) {
        // PointOnPlaneJoint.SolveIteration (PointOnPlaneJoint.cs:212-243)
        const float4 oa = j.L(kJOA, s), ob = j.L(kJOB, s), m0 = j.L(kJM0, s), m1 = j.L(kJM1, s),
                     m2 = j.L(kJM2, s);
        float ax = A.wy * oa.z - A.wz * oa.y, ay = A.wz * oa.x - A.wx * oa.z, az = A.wx * oa.y - A.wy * oa.x;
        ax = ax + A.vx; ay = ay + A.vy; az = az + A.vz;
        float bx = B.wy * ob.z - B.wz * ob.y, by = B.wz * ob.x - B.wx * ob.z, bz = B.wx * ob.y - B.wy * ob.x;
        bx = bx + B.vx; by = by + B.vy; bz = bz + B.vz;
        const float dvx = ax - bx, dvy = ay - by, dvz = az - bz;
        const float vd = dvx * m0.x + dvy * m0.y + dvz * m0.z;
        const float lambda = m0.w * (vd + m1.w + oa.w * acc0.x);
        acc0.x += lambda;
        const float ix = m0.x * lambda, iy = m0.y * lambda, iz = m0.z * lambda;
        if (dynA) {
            ApplyLinear(A, ix, iy, iz);
            ApplyAngular(A, m1.x * lambda, m1.y * lambda, m1.z * lambda);
        }
        if (dynB) {
            ApplyLinear(B, -ix, -iy, -iz);
            ApplyAngular(B, m2.x * lambda, m2.y * lambda, m2.z * lambda);
        }
        account(0, lambda);  // signed, as the reference returns it
    } else if (kAdded && (st & (1u << kChildShift)) && IsDistanceType(type)) {
        // DistanceJoint.SolveIteration (DistanceJoint.cs:226-268) /
        // DistanceLimit.SolveIteration (DistanceLimit.cs:260-305)
        const float4 m0 = j.L(kJM0, s), m1 = j.L(kJM1, s), m2 = j.L(kJM2, s);
        const float softness = j.L(kJOA, s).w;
        const float bx = -m0.x, by = -m0.y, bz = -m0.z;  // jLinearB
        float lambda = m0.x * A.vx + m0.y * A.vy + m0.z * A.vz;
        float dot = m1.x * A.wx + m1.y * A.wy + m1.z * A.wz;
        lambda += dot;
        dot = bx * B.vx + by * B.vy + bz * B.vz;
        lambda += dot;
        dot = m2.x * B.wx + m2.y * B.wy + m2.z * B.wz;
        lambda += dot;
        lambda = -lambda + m1.w - softness * acc0.x;
        lambda *= m0.w;
        if (type == BEPUGPU_JOINT_DISTANCE) {
            acc0.x += lambda;
        } else {
            float previous = acc0.x;
            acc0.x = Maxf(acc0.x + lambda, 0);
            lambda = acc0.x - previous;
        }
        if (dynA) {
            ApplyLinear(A, m0.x * lambda, m0.y * lambda, m0.z * lambda);
            ApplyAngular(A, m1.x * lambda, m1.y * lambda, m1.z * lambda);
        }
        if (dynB) {
            ApplyLinear(B, bx * lambda, by * lambda, bz * lambda);
            ApplyAngular(B, m2.x * lambda, m2.y * lambda, m2.z * lambda);
        }
        account(0, fabsf(lambda));
    } else if (st & (1u << kChildShift)) {
        // BallSocketJoint.SolveIteration (BallSocketJoint.cs:318-372)
        const float4 oa = j.L(kJOA, s), ob = j.L(kJOB, s), m0 = j.L(kJM0, s), m1 = j.L(kJM1, s),
                     m2 = j.L(kJM2, s);
        const float softness = oa.w;
        float crx = A.wy * oa.z - A.wz * oa.y, cry = A.wz * oa.x - A.wx * oa.z, crz = A.wx * oa.y - A.wy * oa.x;
        float ax = A.vx + crx, ay = A.vy + cry, az = A.vz + crz;
        crx = B.wy * ob.z - B.wz * ob.y; cry = B.wz * ob.x - B.wx * ob.z; crz = B.wx * ob.y - B.wy * ob.x;
        float bx = B.vx + crx, by = B.vy + cry, bz = B.vz + crz;
        float lx = ax - bx + m2.y - softness * acc0.x;
        float ly = ay - by + m2.z - softness * acc0.y;
        float lz = az - bz + m2.w - softness * acc0.z;
        // Matrix3x3.Transform by the mass matrix
        float tx = lx * m0.x + ly * m0.w + lz * m1.z;
        float ty = lx * m0.y + ly * m1.x + lz * m1.w;
        float tz = lx * m0.z + ly * m1.y + lz * m2.x;
        acc0.x = acc0.x + tx;
        acc0.y = acc0.y + ty;
        acc0.z = acc0.z + tz;
        if (dynA) {
            float nx = -tx, ny = -ty, nz = -tz;
            ApplyLinear(A, nx, ny, nz);
            ApplyAngular(A, oa.y * nz - oa.z * ny, oa.z * nx - oa.x * nz, oa.x * ny - oa.y * nx);
        }
        if (dynB) {
            ApplyLinear(B, tx, ty, tz);
            ApplyAngular(B, ob.y * tz - ob.z * ty, ob.z * tx - ob.x * tz, ob.x * ty - ob.y * tx);
        }
        account(0, fabsf(tx) + fabsf(ty) + fabsf(tz));
    }
    if (kAdded && (st & (2u << kChildShift)) && IsTwistType(type)) {
        // TwistJoint.SolveIteration (TwistJoint.cs:204-228)
        const float4 w1 = j.L(kJW1, s), w2 = j.L(kJW2, s);
        const float softness = j.L(kJOB, s).w;
        const float jax = -w1.x, jay = -w1.y, jaz = -w1.z;
        const float velocityA = A.wx * jax + A.wy * jay + A.wz * jaz;
        const float velocityB = B.wx * w1.x + B.wy * w1.y + B.wz * w1.z;
        float lambda = -(velocityA + velocityB) + w2.x - softness * acc0.w;
        lambda *= w1.w;
        acc0.w += lambda;
        if (dynA) ApplyAngular(A, jax * lambda, jay * lambda, jaz * lambda);
        if (dynB) ApplyAngular(B, w1.x * lambda, w1.y * lambda, w1.z * lambda);
        account(1, fabsf(lambda));
    } else if (kAdded && (st & (2u << kChildShift)) && IsNoRotationType(type)) {
        // NoRotationJoint.SolveIteration (NoRotationJoint.cs:160-187)
        const float4 l0 = j.L(kJL0, s), l1 = j.L(kJL1, s), l2 = j.L(kJL2, s);
        const float softness = j.L(kJOB, s).w;
        float lx = B.wx - A.wx, ly = B.wy - A.wy, lz = B.wz - A.wz;
        float sx = acc0.w * softness, sy = acc1.x * softness, sz = acc1.y * softness;
        lx = lx + l2.y; ly = ly + l2.z; lz = lz + l2.w;
        lx = lx - sx; ly = ly - sy; lz = lz - sz;
        // Matrix3x3.Transform by the effective mass (M11 M12 M13 M21 | M22 M23 M31 M32 | M33)
        float tx = lx * l0.x + ly * l0.w + lz * l1.z;
        float ty = lx * l0.y + ly * l1.x + lz * l1.w;
        float tz = lx * l0.z + ly * l1.y + lz * l2.x;
        acc0.w = tx + acc0.w;
        acc1.x = ty + acc1.x;
        acc1.y = tz + acc1.y;
        if (dynA) ApplyAngular(A, tx, ty, tz);
        if (dynB) ApplyAngular(B, -tx, -ty, -tz);
        account(1, fabsf(tx) + fabsf(ty) + fabsf(tz));
    } else if (kAdded && (st & (2u << kChildShift)) && IsSwivelType(type)) {
        // SwivelHingeAngularJoint.SolveIteration (SwivelHingeAngularJoint.cs:193-220)
        const float4 w1 = j.L(kJW1, s), w2 = j.L(kJW2, s);
        const float softness = j.L(kJOB, s).w;
        const float jbx = -w1.x, jby = -w1.y, jbz = -w1.z;
        const float velocityA = A.wx * w1.x + A.wy * w1.y + A.wz * w1.z;
        const float velocityB = B.wx * jbx + B.wy * jby + B.wz * jbz;
        float lambda = -(velocityA + velocityB) - w2.x - softness * acc0.w;
        lambda *= w1.w;
        acc0.w += lambda;
        if (dynA) ApplyAngular(A, w1.x * lambda, w1.y * lambda, w1.z * lambda);
        if (dynB) ApplyAngular(B, jbx * lambda, jby * lambda, jbz * lambda);
        account(1, fabsf(lambda));
    } else if (st & (2u << kChildShift)) {
        // RevoluteAngularJoint.SolveIteration (RevoluteAngularJoint.cs:313-356)
        const float4 w1 = j.L(kJW1, s), w2 = j.L(kJW2, s), e = j.L(kJE, s);
        const float softness = j.L(kJOB, s).w;
        float vx = A.wx - B.wx, vy = A.wy - B.wy, vz = A.wz - B.wz;
        float lx = w1.x * vx + w1.y * vy + w1.z * vz;
        float ly = w2.x * vx + w2.y * vy + w2.z * vz;
        lx = lx + w1.w;
        ly = ly + w2.w;
        float sx = acc0.w * softness, sy = acc1.x * softness;
        lx = lx + sx;
        ly = ly + sy;
        float tx = lx * e.x + ly * e.z;
        float ty = lx * e.y + ly * e.w;
        acc0.w = acc0.w + tx;
        acc1.x = acc1.x + ty;
        float ix = w1.x * tx + w2.x * ty, iy = w1.y * tx + w2.y * ty, iz = w1.z * tx + w2.z * ty;
        if (dynA) ApplyAngular(A, ix, iy, iz);
        if (dynB) ApplyAngular(B, -ix, -iy, -iz);
        account(1, fabsf(tx) + fabsf(ty));
    }
    if (kAdded && (st & (4u << kChildShift)) && IsLinearLimitType(type)) {
        // LinearAxisLimit.SolveIteration (LinearAxisLimit.cs:290-336)
        const int k0 = LinearLimitLane(type);
        const float4 ja = j.L(k0, s), jaa = j.L(k0 + 1, s), jab = j.L(k0 + 2, s);
        const float bx = -ja.x, by = -ja.y, bz = -ja.z;  // jLinearB
        float lambda = ja.x * A.vx + ja.y * A.vy + ja.z * A.vz;
        float dot = jaa.x * A.wx + jaa.y * A.wy + jaa.z * A.wz;
        lambda += dot;
        dot = bx * B.vx + by * B.vy + bz * B.vz;
        lambda += dot;
        dot = jab.x * B.wx + jab.y * B.wy + jab.z * B.wz;
        lambda += dot;
        lambda = -lambda + jaa.w - ja.w * acc1.z;
        lambda *= jab.w;
        const float previous = acc1.z;
        acc1.z = (st & kJMinActive) ? Minf(acc1.z + lambda, 0) : Maxf(acc1.z + lambda, 0);
        lambda = acc1.z - previous;
        if (dynA) {
            ApplyLinear(A, ja.x * lambda, ja.y * lambda, ja.z * lambda);
            ApplyAngular(A, jaa.x * lambda, jaa.y * lambda, jaa.z * lambda);
        }
        if (dynB) {
            ApplyLinear(B, bx * lambda, by * lambda, bz * lambda);
            ApplyAngular(B, jab.x * lambda, jab.y * lambda, jab.z * lambda);
        }
        account(2, fabsf(lambda));
    } else if (st & (4u << kChildShift)) {
        const float4 l0 = j.L(kJL0, s), l2 = j.L(kJL2, s);
        const float softness = l0.w;
        if (kAdded && type == BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR) {
            // SingleEntityLinearMotor.SolveIteration (SingleEntityLinearMotor.cs:180-208)
            const float4 l1 = j.L(kJL1, s), oa = j.L(kJOA, s);
            const float3 r = JXYZ(j.L(kJOB, s));
            float3 l = JCross(r, make_float3(A.wx, A.wy, A.wz));
            l = make_float3(l.x - A.vx, l.y - A.vy, l.z - A.vz);
            l = make_float3(l2.y + l.x, l2.z + l.y, l2.w + l.z);
            l = make_float3(l.x - acc0.x * oa.x, l.y - acc0.y * oa.x, l.z - acc0.z * oa.x);
            const JM3 m = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w, l2.x};
            l = JTransform(l, m);
            const float px = acc0.x, py = acc0.y, pz = acc0.z;
            acc0.x = acc0.x + l.x;
            acc0.y = acc0.y + l.y;
            acc0.z = acc0.z + l.z;
            const float sq = acc0.x * acc0.x + acc0.y * acc0.y + acc0.z * acc0.z;
            if (sq > oa.z) {
                const float f = oa.y / SqrtOfFloat(sq);
                acc0.x = acc0.x * f;
                acc0.y = acc0.y * f;
                acc0.z = acc0.z * f;
                l = make_float3(acc0.x - px, acc0.y - py, acc0.z - pz);
            }
            ApplyLinear(A, l.x, l.y, l.z);
            const float3 t = JCross(r, l);
            ApplyAngular(A, t.x, t.y, t.z);
            account(2, fabsf(l.x) + fabsf(l.y) + fabsf(l.z));
        } else if (kAdded && IsAngularMotorType(type)) {
            // AngularMotor.SolveIteration (AngularMotor.cs:203-246); SingleEntityAngularMotor's
            // (SingleEntityAngularMotor.cs:117-148) adds its bias to -w_A
            const float4 l1 = j.L(kJL1, s), oa = j.L(kJOA, s);
            const float us = oa.x;
            float lx, ly, lz;
            if (type == BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR) {
                lx = -A.wx + l2.y - us * acc0.x;
                ly = -A.wy + l2.z - us * acc0.y;
                lz = -A.wz + l2.w - us * acc0.z;
            } else {
                lx = B.wx - A.wx - l2.y - us * acc0.x;
                ly = B.wy - A.wy - l2.z - us * acc0.y;
                lz = B.wz - A.wz - l2.w - us * acc0.z;
            }
            const JM3 m = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w, l2.x};
            const float3 t = JTransform(make_float3(lx, ly, lz), m);
            lx = t.x; ly = t.y; lz = t.z;
            const float px = acc0.x, py = acc0.y, pz = acc0.z;
            acc0.x += lx;
            acc0.y += ly;
            acc0.z += lz;
            const float sumLengthSquared = acc0.x * acc0.x + acc0.y * acc0.y + acc0.z * acc0.z;
            if (sumLengthSquared > oa.z) {
                const float multiplier = oa.y / SqrtOfFloat(sumLengthSquared);
                acc0.x *= multiplier;
                acc0.y *= multiplier;
                acc0.z *= multiplier;
                lx = acc0.x - px;
                ly = acc0.y - py;
                lz = acc0.z - pz;
            }
            if (dynA) ApplyAngular(A, lx, ly, lz);
            if (dynB) ApplyAngular(B, -lx, -ly, -lz);
            account(2, fabsf(lx) + fabsf(ly) + fabsf(lz));
        } else if (kAdded && IsSpeedLimitType(type)) {
            // MaximumLinearSpeedConstraint / MaximumAngularSpeedConstraint.SolveIteration
            // (MaximumLinearVelocityConstraint.cs:138-175 and the angular file's)
            const bool angular = type == BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED;
            const float4 l1 = j.L(kJL1, s);
            float usedSoftness, maxForceDt, maxForceDtSquared, maxSpeed, maxSpeedSquared;
            if (angular) {
                const float4 oa = j.L(kJOA, s);
                usedSoftness = l0.x; maxForceDt = l0.y; maxForceDtSquared = l0.z; maxSpeed = l0.w;
                maxSpeedSquared = oa.y;
            } else {
                usedSoftness = l0.y; maxForceDt = l0.z; maxForceDtSquared = l0.w; maxSpeed = l1.x;
                maxSpeedSquared = l1.y;
            }
            const float vx = angular ? A.wx : A.vx, vy = angular ? A.wy : A.vy, vz = angular ? A.wz : A.vz;
            float speed = vx * vx + vy * vy + vz * vz;
            float result = 0;
            if (speed > maxSpeedSquared) {
                speed = SqrtOfFloat(speed);
                const float f = -(speed - maxSpeed) / speed;
                float ix = vx * f, iy = vy * f, iz = vz * f;
                ix = ix - acc0.x * usedSoftness;
                iy = iy - acc0.y * usedSoftness;
                iz = iz - acc0.z * usedSoftness;
                if (angular) {
                    const float4 oa = j.L(kJOA, s);
                    const JM3 m = {l1.x, l1.y, l1.z, l1.w, l2.x, l2.y, l2.z, l2.w, oa.x};
                    const float3 t = JTransform(make_float3(ix, iy, iz), m);
                    ix = t.x; iy = t.y; iz = t.z;
                } else {
                    ix *= l0.x; iy *= l0.x; iz *= l0.x;
                }
                const float px = acc0.x, py = acc0.y, pz = acc0.z;
                acc0.x = acc0.x + ix;
                acc0.y = acc0.y + iy;
                acc0.z = acc0.z + iz;
                const float forceMagnitude = acc0.x * acc0.x + acc0.y * acc0.y + acc0.z * acc0.z;
                if (forceMagnitude > maxForceDtSquared) {
                    const float multiplier = maxForceDt / SqrtOfFloat(forceMagnitude);
                    acc0.x *= multiplier;
                    acc0.y *= multiplier;
                    acc0.z *= multiplier;
                    ix = acc0.x - px;
                    iy = acc0.y - py;
                    iz = acc0.z - pz;
                }
                if (angular) ApplyAngular(A, ix, iy, iz);
                else ApplyLinear(A, ix, iy, iz);
                result = fabsf(ix) + fabsf(iy) + fabsf(iz);
            }
            account(2, result);
        } else if (kAdded && type == BEPUGPU_JOINT_LINEAR_AXIS_MOTOR) {
            // LinearAxisMotor.SolveIteration (LinearAxisMotor.cs:244-283)
            const float4 jaa = j.L(kJL1, s), jab = j.L(kJL2, s);
            const float maxForceDt = j.L(kJOA, s).x;
            const float bx = -l0.x, by = -l0.y, bz = -l0.z;  // jLinearB
            float lambda = l0.x * A.vx + l0.y * A.vy + l0.z * A.vz;
            float dot = jaa.x * A.wx + jaa.y * A.wy + jaa.z * A.wz;
            lambda += dot;
            dot = bx * B.vx + by * B.vy + bz * B.vz;
            lambda += dot;
            dot = jab.x * B.wx + jab.y * B.wy + jab.z * B.wz;
            lambda += dot;
            lambda = -lambda + jaa.w - softness * acc1.y;
            lambda *= jab.w;
            const float previous = acc1.y;
            acc1.y = Clampf(acc1.y + lambda, -maxForceDt, maxForceDt);
            lambda = acc1.y - previous;
            if (dynA) {
                ApplyLinear(A, l0.x * lambda, l0.y * lambda, l0.z * lambda);
                ApplyAngular(A, jaa.x * lambda, jaa.y * lambda, jaa.z * lambda);
            }
            if (dynB) {
                ApplyLinear(B, bx * lambda, by * lambda, bz * lambda);
                ApplyAngular(B, jab.x * lambda, jab.y * lambda, jab.z * lambda);
            }
            account(2, fabsf(lambda));
        } else if (kAdded && (type == BEPUGPU_JOINT_REVOLUTE_MOTOR || type == BEPUGPU_JOINT_TWIST_MOTOR)) {
            // RevoluteMotor.SolveIteration (RevoluteMotor.cs:309-340), TwistMotor's (TwistMotor.cs:226-253)
            const float nx = -l0.x, ny = -l0.y, nz = -l0.z;  // jacobianB
            const float velocityA = A.wx * l0.x + A.wy * l0.y + A.wz * l0.z;
            const float velocityB = B.wx * nx + B.wy * ny + B.wz * nz;
            float lambda = -(velocityA + velocityB) + l2.x - softness * acc1.y;
            lambda *= l2.z;
            const float previous = acc1.y;
            acc1.y = Clampf(acc1.y + lambda, -l2.w, l2.w);
            lambda = acc1.y - previous;
            if (dynA) ApplyAngular(A, l0.x * lambda, l0.y * lambda, l0.z * lambda);
            if (dynB) ApplyAngular(B, nx * lambda, ny * lambda, nz * lambda);
            account(2, fabsf(lambda));
        } else if (kAdded && type == BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT) {
            // EllipseSwingLimit.SolveIteration (EllipseSwingLimit.cs:327-357)
            const float nx = -l0.x, ny = -l0.y, nz = -l0.z;  // jacobianB
            const float velocityA = A.wx * l0.x + A.wy * l0.y + A.wz * l0.z;
            const float velocityB = B.wx * nx + B.wy * ny + B.wz * nz;
            float lambda = (-velocityA - velocityB) - l2.x - softness * acc1.y;
            lambda *= l2.z;
            const float previous = acc1.y;
            acc1.y = Minf(acc1.y + lambda, 0);
            lambda = acc1.y - previous;
            if (dynA) ApplyAngular(A, l0.x * lambda, l0.y * lambda, l0.z * lambda);
            if (dynB) ApplyAngular(B, nx * lambda, ny * lambda, nz * lambda);
            account(2, fabsf(lambda));
        } else if (kAdded && type == BEPUGPU_JOINT_TWIST_LIMIT) {
            // TwistLimit.SolveIteration (TwistLimit.cs:200-236)
            const float nx = -l0.x, ny = -l0.y, nz = -l0.z;  // jacobianB
            const float velocityA = A.wx * l0.x + A.wy * l0.y + A.wz * l0.z;
            const float velocityB = B.wx * nx + B.wy * ny + B.wz * nz;
            float lambda = -(velocityA + velocityB) + l2.x - softness * acc1.y;
            lambda *= l2.z;
            const float previous = acc1.y;
            acc1.y = Maxf(acc1.y + lambda, 0);
            lambda = acc1.y - previous;
            if (dynA) ApplyAngular(A, l0.x * lambda, l0.y * lambda, l0.z * lambda);
            if (dynB) ApplyAngular(B, nx * lambda, ny * lambda, nz * lambda);
            account(2, fabsf(lambda));
        } else if (type == BEPUGPU_JOINT_SWING_LIMIT) {
            // SwingLimit.SolveIteration (SwingLimit.cs:211-243)
            float rx = A.wx - B.wx, ry = A.wy - B.wy, rz = A.wz - B.wz;
            float lambda = rx * l0.x + ry * l0.y + rz * l0.z;
            lambda = -lambda + l2.x - softness * acc1.y;
            lambda *= l2.z;
            float previous = acc1.y;
            acc1.y = Maxf(acc1.y + lambda, 0);
            lambda = acc1.y - previous;
            float ix = l0.x * lambda, iy = l0.y * lambda, iz = l0.z * lambda;
            if (dynA) ApplyAngular(A, ix, iy, iz);
            if (dynB) ApplyAngular(B, -ix, -iy, -iz);
            account(2, fabsf(lambda));
        } else {
            // RevoluteLimit.SolveIteration (RevoluteLimit.cs:211-283)
            const float4 l1 = j.L(kJL1, s);
            float lambdaTotal = 0;
            if (st & kJMinActive) {
                float nx = -l0.x, ny = -l0.y, nz = -l0.z;
                float velocityA = A.wx * l0.x + A.wy * l0.y + A.wz * l0.z;
                float velocityB = B.wx * nx + B.wy * ny + B.wz * nz;
                float lambda = -(velocityA + velocityB) + l2.x - softness * acc1.y;
                lambda *= l2.z;
                float previous = acc1.y;
                acc1.y = Maxf(acc1.y + lambda, 0);
                lambda = acc1.y - previous;
                if (dynA) ApplyAngular(A, l0.x * lambda, l0.y * lambda, l0.z * lambda);
                if (dynB) ApplyAngular(B, nx * lambda, ny * lambda, nz * lambda);
                lambdaTotal += fabsf(lambda);
            }
            if (st & kJMaxActive) {
                float nx = -l1.x, ny = -l1.y, nz = -l1.z;
                float velocityA = A.wx * l1.x + A.wy * l1.y + A.wz * l1.z;
                float velocityB = B.wx * nx + B.wy * ny + B.wz * nz;
                float lambda = -(velocityA + velocityB) + l2.y - softness * acc1.z;
                lambda *= l2.w;
                float previous = acc1.z;
                acc1.z = Maxf(acc1.z + lambda, 0);
                lambda = acc1.z - previous;
                if (dynA) ApplyAngular(A, l1.x * lambda, l1.y * lambda, l1.z * lambda);
                if (dynB) ApplyAngular(B, nx * lambda, ny * lambda, nz * lambda);
                lambdaTotal += fabsf(lambda);
            }
            account(2, lambdaTotal);
        }
    }
    j.L(kJACC0, s) = acc0;
    j.L(kJACC1, s) = acc1;
}

// Solver.UnsafeSolveIteration (Solver.cs:285-314) on the joint or group, then
// SolverGroup.SolveIteration (SolverGroup.cs:156-165): the record's children,
// then its continuation records' in the slots after it.
template <bool kAdded>
__device__ __forceinline__ void SolveJoint(const JointSoA& j, int s, BodyState& A, BodyState& B, uint2& state,
                                           int type, const StepParams& p) {
    uint32_t st = state.x, zeros = state.y;
    uint32_t iter = (st >> kIterShift) + 1;
    st = (st & 0xffffu) | (iter << kIterShift);
    if (!((int)iter <= p.iterationLimit && (int)iter <= p.maximumIterationCount)) {
        state = make_uint2(st & ~kGroupActive, zeros);
        return;
    }
    int activeConstraints = 0;
    SolveJointChildren<kAdded>(j, s, A, B, st, zeros, activeConstraints, type, p);
    if (kAdded && (st & kJHasNext))
        for (int u = s + 1;; u++) {
            uint2 cs = j.state[u];
            SolveJointChildren<kAdded>(j, u, A, B, cs.x, cs.y, activeConstraints, JointType(cs.x), p);
            j.state[u] = cs;
            if (!(cs.x & kJHasNext)) break;
        }
    if (activeConstraints <= 0) st &= ~kGroupActive;
    state = make_uint2(st, zeros);
}

}  // namespace bepugpu
