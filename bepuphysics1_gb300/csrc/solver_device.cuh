// Device side of the velocity solver: data layout and per-constraint math.
//
// Layout in HBM (structure of arrays, 16-byte lanes so every field moves as
// one 128-bit load):
//   bodies     pos (xyz, dynamic flag), quat, vlin (v, inverse mass),
//              vang (w, world inverse inertia M33), inv0/inv1 (rest of the
//              world inverse inertia), loc0/loc1/damp (local inverse inertia,
//              damping factors).
//   manifolds  one slot per manifold in colour order; per-contact arrays are
//              [4][capacity] so lane k of consecutive slots is contiguous.
// Every routine restates the reference's arithmetic in its evaluation order;
// the library is compiled with -fmad=false so no multiply-add is fused, as
// C# never fuses them.  Double precision is used exactly where the reference
// calls System.Math.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/bepugpu.h"
#include "double_rounding.cuh"

namespace bepugpu {

// Per-step constants (CollisionResponseSettings, CollisionDetectionSettings,
// SolverSettings defaults, the solver's iteration limit, dt).
struct StepParams {
    float dt;
    float updateRate;        // 1 / dt, as every Update computes it
    float gravityDt[3];      // Vector3.Multiply(gravity, dt), ForceUpdater.cs:87
    int iterationLimit;
    int maximumIterationCount;
    int minimumIterationCount;
    float minimumImpulse;
    float softness, recoveryStiffness, maxRecoverySpeed, staticThreshold, twistFactor;
    float bounceThreshold, allowedPenetration, invalidationLengthSquared, maximumContactDistance;
    // DeactivationManager: useStabilization, velocityLowerLimit (and its square, as the
    // setter computes it), lowVelocityTimeMinimum (DeactivationManager.cs:18-20,36-37,60)
    int useStabilization;
    float velocityLowerLimit, velocityLowerLimitSquared, lowVelocityTimeMinimum;
};

struct BodySoA {
    float4* pos;   // position, w = 1 dynamic / 0 kinematic
    float4* quat;  // orientation x y z w
    float4* vlin;  // linear velocity, w = inverse mass (0 when kinematic)
    float4* vang;  // angular velocity, w = world inverse inertia M33
    float4* inv0;  // world inverse inertia M11 M12 M13 M21
    float4* inv1;  // world inverse inertia M22 M23 M31 M32
    float4* loc0;  // local inverse inertia M11 M12 M13 M21
    float4* loc1;  // local inverse inertia M22 M23 M31 M32
    float4* damp;  // linear damping factor, angular damping factor, local M33, flags
    float4* act;   // activity: previousVelocity, velocityTimeBelowLimit, BEPUGPU_BODY_* bits, 0
    float2* rawDamp;  // LinearDamping, AngularDamping (read when the stabilization boost applies)
    // Simulation islands (islands.cu; null without them): each body's island
    // (-1 kinematic) and the islands' BEPUGPU_ISLAND_* flags.
    const int32_t* islandOf;
    const uint32_t* islandFlags;
    int count;
};

// A dynamic body whose island sleeps (SimulationIslandMember.IsActive,
// SimulationIslandMember.cs:225-248, is its island's state).
__device__ __forceinline__ bool IslandAsleep(const BodySoA& b, int i) {
    if (!b.islandOf) return false;
    const int k = b.islandOf[i];
    return k >= 0 && !(b.islandFlags[k] & 1u);
}

// Activity bits in act.z, the ABI's BEPUGPU_BODY_* values.
enum : uint32_t {
    kAlwaysActive = 1u,
    kNoStabilization = 2u,
    kSlowing = 4u,
    kCandidate = 8u
};

// Manifold state bits (word x of the uint2 state).
enum : uint32_t {
    kGroupActive = 1u << 0,       // ConvexContactManifoldConstraint.isActiveInSolver
    kChildShift = 1,              // bits 1..6: pen0..pen3, sliding, twist isActiveInSolver
    kSlidingBit = 1u << 5,
    kTwistBit = 1u << 6,
    kDynA = 1u << 7,              // entityADynamic as computed in Update
    kDynB = 1u << 8,
    kHasA = 1u << 9,              // entity A is not null
    kHasB = 1u << 10,
    kFricShift = 11,              // NONCONVEX: bits 11..14, contact friction 0..3 isActiveInSolver
    kIterShift = 16               // bits 16..31: group currentIterations
};
// Word y: 4-bit iterationsAtZeroImpulse per child: pen0..3, then sliding and
// twist (convex) or contact friction 0..3 (NONCONVEX).
constexpr uint32_t kManifoldNonConvex = 8u;  // BEPUGPU_MANIFOLD_NONCONVEX, in head.z >> 8

struct ManifoldSoA {
    int4* head;      // body A, body B, contact count | flags << 8, source index
    float4* cpos;    // [4][cap] contact position, w = penetration depth
    float4* cnrm;    // [4][cap] contact normal, w = id (int bits)
    float4* offA;    // [4][cap] local offset A, w = base penetration depth
    float4* offB;    // [4][cap] local offset B
    float4* mat;     // kinetic friction, static friction, bounciness
    float4* penacc;  // accumulated impulse of pen0..pen3
    float4* fricacc; // sliding x, sliding y, twist
    float4* saxis;   // sliding linearA row 1 (kept between steps), w = v2i M12
    // prestep products
    float4* pj0;     // [4][cap] linearA (= -normal), w = bias
    float4* pj1;     // [4][cap] angularA, w = softness
    float4* pj2;     // [4][cap] angularB, w = velocityToImpulse
    float4* s0;      // sliding ra, w = friction
    float4* s1;      // sliding rb, w = v2i M11
    float4* s3;      // sliding linearA row 2, w = v2i M21
    float4* s4;      // sliding angularA row 1, w = v2i M22
    float4* s5;      // sliding angularA row 2, w = twist velocityToImpulse
    float4* s6;      // sliding angularB row 1, w = twist friction
    float4* s7;      // sliding angularB row 2
    float4* lever;   // twist lever arms
    // NONCONVEX manifolds: one ContactFrictionConstraint per contact, in
    // global memory only (a group with such a manifold keeps its lanes there)
    float4* cfr;     // [4][cap] linearA (the friction direction, kept between steps), w = accumulatedImpulse
    float4* cfa;     // [4][cap] prestep: angularA, w = velocityToImpulse
    float4* cfb;     // [4][cap] prestep: angularB, w = friction
    uint2* state;
    int count;
    int capacity;
};

// ------------------------------------------------------------------ bodies --
struct BodyState {
    float vx, vy, vz, invMass;
    float wx, wy, wz;
    float I11, I12, I13, I21, I22, I23, I31, I32, I33;
};

// Body storage views.  A ref names a body; -1 is "no entity".  The global
// path's refs are body indices; a group kernel keeps its bodies in shared
// memory and uses its own refs (GroupBodies in groups.cu).  The constraint
// routines are templated on the view, so both paths run the same arithmetic.
struct GlobalBodies {
    BodySoA b;
    // A sleeping body reads as not dynamic: nothing of the step may move it, and
    // a constraint with no active dynamic body is not active in the solver
    // (SolverUpdateable.cs:202-219, ContactManifoldConstraint.cs:125-141).
    __device__ __forceinline__ float4 Pos(int r) const {
        float4 p = b.pos[r];
        if (b.islandOf && p.w != 0.f && IslandAsleep(b, r)) p.w = 0.f;
        return p;
    }
    __device__ __forceinline__ float4 Quat(int r) const { return b.quat[r]; }
    __device__ __forceinline__ float4 Vlin(int r) const { return b.vlin[r]; }
    __device__ __forceinline__ float4 Vang(int r) const { return b.vang[r]; }
    __device__ __forceinline__ float4 Inv0(int r) const { return b.inv0[r]; }
    __device__ __forceinline__ float4 Inv1(int r) const { return b.inv1[r]; }
    __device__ __forceinline__ void SetVelocity(int r, float4 v, float4 w) const { b.vlin[r] = v; b.vang[r] = w; }
    // local inverse inertia: M11 M12 M13 M21, M22 M23 M31 M32, M33
    __device__ __forceinline__ void LocalInertia(int r, float4& l0, float4& l1, float& m33) const {
        l0 = b.loc0[r]; l1 = b.loc1[r]; m33 = b.damp[r].z;
    }
};

template <class V>
__device__ __forceinline__ void LoadBodyV(const V& bv, int r, BodyState& s) {
    float4 v = bv.Vlin(r), w = bv.Vang(r), a = bv.Inv0(r), c = bv.Inv1(r);
    s.vx = v.x; s.vy = v.y; s.vz = v.z; s.invMass = v.w;
    s.wx = w.x; s.wy = w.y; s.wz = w.z; s.I33 = w.w;
    s.I11 = a.x; s.I12 = a.y; s.I13 = a.z; s.I21 = a.w;
    s.I22 = c.x; s.I23 = c.y; s.I31 = c.z; s.I32 = c.w;
}
template <class V>
__device__ __forceinline__ void StoreVelocityV(const V& bv, int r, const BodyState& s) {
    bv.SetVelocity(r, make_float4(s.vx, s.vy, s.vz, s.invMass), make_float4(s.wx, s.wy, s.wz, s.I33));
}
__device__ __forceinline__ void LoadBody(const BodySoA& b, int i, BodyState& s) { LoadBodyV(GlobalBodies{b}, i, s); }
__device__ __forceinline__ void StoreVelocity(const BodySoA& b, int i, const BodyState& s) {
    StoreVelocityV(GlobalBodies{b}, i, s);
}
// EntityBase.ApplyLinearImpulse (EntityBase.cs:754-761)
__device__ __forceinline__ void ApplyLinear(BodyState& s, float x, float y, float z) {
    s.vx += x * s.invMass;
    s.vy += y * s.invMass;
    s.vz += z * s.invMass;
}
// EntityBase.ApplyAngularImpulse, non-CONSERVE (EntityBase.cs:782-784)
__device__ __forceinline__ void ApplyAngular(BodyState& s, float x, float y, float z) {
    s.wx += x * s.I11 + y * s.I21 + z * s.I31;
    s.wy += x * s.I12 + y * s.I22 + z * s.I32;
    s.wz += x * s.I13 + y * s.I23 + z * s.I33;
}

// SimulationIslandMember.UpdateDeactivationCandidacy (SimulationIslandMember.cs:53-164)
// for a body whose island is awake (every dynamic body's: islands are not put
// to sleep here).  v and w are the body's velocities at the start of the step;
// act holds previousVelocity, velocityTimeBelowLimit and the activity bits and
// is rewritten.  The island bookkeeping of the reference (path compression,
// waking islands next to an active kinematic body) has nothing to do when
// every island is awake.
__device__ __forceinline__ void CandidacyMath(float4 v, float4 w, bool dynamic, float4& act, const StepParams& p,
                                              bool islandActive = true) {
    uint32_t f = __float_as_uint(act.z);
    // velocity = linearVelocity.LengthSquared() + angularVelocity.LengthSquared() (Vector3.cs:64-67)
    float velocity = (v.x * v.x + v.y * v.y + v.z * v.z) + (w.x * w.x + w.y * w.y + w.z * w.z);
    float t = act.y;
    // IsActive (:225-248): the island's state for a dynamic body, the time flag for a kinematic one
    const bool isActive = dynamic ? islandActive : t <= 0.f;
    if (isActive) {
        const bool slowing = velocity <= act.x;
        f = slowing ? (f | kSlowing) : (f & ~kSlowing);
        if (dynamic) {
            if (velocity < p.velocityLowerLimitSquared) t = t + p.dt;
            else t = 0.f;
            if (!(f & kAlwaysActive)) {
                if (!(f & kCandidate)) {
                    if (t > p.lowVelocityTimeMinimum && slowing) f |= kCandidate;
                } else if (t <= p.lowVelocityTimeMinimum) {
                    f &= ~kCandidate;  // the IsDeactivationCandidate setter resets the time (:186-189)
                    t = 0.f;
                }
            } else {
                f &= ~kCandidate;
                t = 0.f;
            }
        } else {
            const bool candidate = velocity == 0.f && !(f & kAlwaysActive);
            if (!candidate) t = 0.f;  // the setter, then the time flag below
            f = candidate ? (f | kCandidate) : (f & ~kCandidate);
            if (candidate) {
                if (t == 0.f) t = 1.f;
                else if (t < 0.f) t = 0.f;
            } else {
                t = -1.f;
            }
        }
    }
    act.x = velocity;
    act.y = t;
    act.z = __uint_as_float(f);
}

// (float)Math.Pow(MathHelper.Clamp(1 - d, 0, 1), dt) of a boosted damping
// (EntityBase.cs:943,952): the float System.Math.Pow's double result rounds to.
__device__ __forceinline__ float BoostedDampingFactor(float d, float dt) {
    float c = 1 - d;
    c = c < 0.f ? 0.f : (c > 1.f ? 1.f : c);
    return dr::PowAsDouble(c, dt);
}

// Entity.UpdateForForces (EntityBase.cs:911-975).  The arithmetic on one
// body's lanes: v and w in/out, world inverse inertia to a (M11 M12 M13 M21),
// c (M22 M23 M31 M32) and w.w (M33).  d.x / d.y are the damping factors of
// the entity's own damping, computed on the host; act carries the activity
// state the stabilization boost reads (:926-936), raw the entity's
// LinearDamping and AngularDamping, read only when the boost applies.
__device__ __forceinline__ void ForceMath(float4& v, float4& w, float4 q, float4 l0, float4 l1, float4 d, float4 act,
                                          const float2* raw, float4& a, float4& c, const StepParams& p) {
    uint32_t flags = __float_as_uint(d.w);
    v.x = p.gravityDt[0] + v.x;
    v.y = p.gravityDt[1] + v.y;
    v.z = p.gravityDt[2] + v.z;
    const uint32_t af = __float_as_uint(act.z);
    bool boosted = false;
    if (p.useStabilization && !(af & kNoStabilization) && ((af & kSlowing) || act.y > p.lowVelocityTimeMinimum)) {
        float energy = (v.x * v.x + v.y * v.y + v.z * v.z) + (w.x * w.x + w.y * w.y + w.z * w.z);
        if (energy < p.velocityLowerLimitSquared) {
            float boost = 1 - dr::SqrtQuotientAsDouble(energy, 2.f * p.velocityLowerLimit);
            const float2 r = *raw;
            // ModifyAngularDamping(boost), then ModifyLinearDamping(boost) (:1205-1221), from zero boosts
            float angularBoost = 0.f + boost * (1 - (r.y + 0.f));
            float linearBoost = 0.f + boost * (1 - (r.x + 0.f));
            float linear = r.x + linearBoost;
            if (linear > 0) {
                float f = BoostedDampingFactor(linear, p.dt);
                v.x = v.x * f; v.y = v.y * f; v.z = v.z * f;
            }
            float angular = r.y + angularBoost;
            if (angular > 0) {
                float f = BoostedDampingFactor(angular, p.dt);
                w.x = w.x * f; w.y = w.y * f; w.z = w.z * f;
            }
            boosted = true;
        }
    }
    if (!boosted) {
        if (flags & 1u) { v.x = v.x * d.x; v.y = v.y * d.x; v.z = v.z * d.x; }
        if (flags & 2u) { w.x = w.x * d.y; w.y = w.y * d.y; w.z = w.z * d.y; }
    }
    // orientationMatrix = Matrix3x3.CreateFromQuaternion(orientation) (Matrix3x3.cs:1303-1328)
    float qX2 = q.x + q.x, qY2 = q.y + q.y, qZ2 = q.z + q.z;
    float XX = qX2 * q.x, YY = qY2 * q.y, ZZ = qZ2 * q.z;
    float XY = qX2 * q.y, XZ = qX2 * q.z, XW = qX2 * q.w;
    float YZ = qY2 * q.z, YW = qY2 * q.w, ZW = qZ2 * q.w;
    float R11 = 1 - YY - ZZ, R21 = XY - ZW, R31 = XZ + YW;
    float R12 = XY + ZW, R22 = 1 - XX - ZZ, R32 = YZ - XW;
    float R13 = XZ - YW, R23 = YZ + XW, R33 = 1 - XX - YY;
    float L11 = l0.x, L12 = l0.y, L13 = l0.z, L21 = l0.w, L22 = l1.x, L23 = l1.y, L31 = l1.z, L32 = l1.w,
          L33 = d.z;
    // multiplied = R^T * L (Matrix3x3.MultiplyTransposed, :866-890)
    float m11 = R11 * L11 + R21 * L21 + R31 * L31;
    float m12 = R11 * L12 + R21 * L22 + R31 * L32;
    float m13 = R11 * L13 + R21 * L23 + R31 * L33;
    float m21 = R12 * L11 + R22 * L21 + R32 * L31;
    float m22 = R12 * L12 + R22 * L22 + R32 * L32;
    float m23 = R12 * L13 + R22 * L23 + R32 * L33;
    float m31 = R13 * L11 + R23 * L21 + R33 * L31;
    float m32 = R13 * L12 + R23 * L22 + R33 * L32;
    float m33 = R13 * L13 + R23 * L23 + R33 * L33;
    // inertiaTensorInverse = multiplied * R (Matrix3x3.Multiply, :766-790)
    a.x = m11 * R11 + m12 * R21 + m13 * R31;
    a.y = m11 * R12 + m12 * R22 + m13 * R32;
    a.z = m11 * R13 + m12 * R23 + m13 * R33;
    a.w = m21 * R11 + m22 * R21 + m23 * R31;
    c.x = m21 * R12 + m22 * R22 + m23 * R32;
    c.y = m21 * R13 + m22 * R23 + m23 * R33;
    c.z = m31 * R11 + m32 * R21 + m33 * R31;
    c.w = m31 * R12 + m32 * R22 + m33 * R32;
    w.w = m31 * R13 + m32 * R23 + m33 * R33;
}
// The body stages of one body at the start of a step: the candidacy update
// (BEPUGPU_STEP_DEACTIVATION, every body) and the force update
// (BEPUGPU_STEP_FORCES, dynamic bodies: ForceUpdater only holds those).
__device__ __forceinline__ void StartBodyStep(const BodySoA& b, int i, const StepParams& p, uint32_t stages) {
    const float4 pos = b.pos[i];
    const bool dynamic = pos.w != 0.f;
    float4 act = b.act[i];
    if (stages & BEPUGPU_STEP_DEACTIVATION) {
        CandidacyMath(b.vlin[i], b.vang[i], dynamic, act, p);
        b.act[i] = act;
    }
    if (!dynamic || !(stages & BEPUGPU_STEP_FORCES) || IslandAsleep(b, i)) return;  // ForceUpdater.cs:73-76
    float4 v = b.vlin[i], w = b.vang[i], q = b.quat[i], l0 = b.loc0[i], l1 = b.loc1[i], d = b.damp[i];
    float4 a, c;
    ForceMath(v, w, q, l0, l1, d, act, b.rawDamp + i, a, c, p);
    b.vlin[i] = v;
    b.vang[i] = w;
    b.inv0[i] = a;
    b.inv1[i] = c;
}

// Entity.PreUpdatePosition, Discrete mode (EntityBase.cs:1124-1160), for an
// active body (the position updater skips inactive ones,
// ContinuousPositionUpdater.cs:71): every dynamic body, and a kinematic body
// while its velocityTimeBelowLimit flag is <= 0 (SimulationIslandMember.cs:225-248).
__device__ __forceinline__ bool BodyActive(float4 pos, float4 act) { return pos.w != 0.f || act.y <= 0.f; }
__device__ __forceinline__ void PositionMath(float4& pos, float4& q, float4 v, float4 w, const StepParams& p) {
    float h = p.dt * .5f;
    float ix = w.x * h, iy = w.y * h, iz = w.z * h;
    // Quaternion.Multiply(multiplier = (ix, iy, iz, 0), orientation) (Quaternion.cs:66-79)
    float x = ix, y = iy, z = iz, ww = 0.f;
    float mx = x * q.w + q.x * ww + y * q.z - z * q.y;
    float my = y * q.w + q.y * ww + z * q.x - x * q.z;
    float mz = z * q.w + q.z * ww + x * q.y - y * q.x;
    float mw = ww * q.w - x * q.x - y * q.y - z * q.z;
    q.x = q.x + mx; q.y = q.y + my; q.z = q.z + mz; q.w = q.w + mw;
    // Quaternion.Normalize (Quaternion.cs:262-269)
    float inverse = dr::InvSqrtAsDouble(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    q.x *= inverse; q.y *= inverse; q.z *= inverse; q.w *= inverse;
    pos.x = pos.x + v.x * p.dt;
    pos.y = pos.y + v.y * p.dt;
    pos.z = pos.z + v.z * p.dt;
}
__device__ __forceinline__ void PositionUpdateBody(const BodySoA& b, int i, const StepParams& p) {
    float4 pos = b.pos[i], q = b.quat[i];
    if (!BodyActive(pos, b.act[i]) || IslandAsleep(b, i)) return;
    PositionMath(pos, q, b.vlin[i], b.vang[i], p);
    b.quat[i] = q;
    b.pos[i] = pos;
}

// -------------------------------------------------------------- manifolds --
__device__ __forceinline__ float Maxf(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float Minf(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float Clampf(float v, float lo, float hi) {
    if (v < lo) return lo;
    else if (v > hi) return hi;
    return v;
}

// (float)System.Math.Sqrt((double)x) for a float x.  Rounding the double
// square root to float gives the correctly rounded float square root, since
// double carries at least 2*24+2 significant bits (Figueroa, "When is double
// rounding innocuous?", 1995); the IEEE single-precision square root therefore
// returns the same bits without using the FP64 pipe.
__device__ __forceinline__ float SqrtOfFloat(float x) { return __fsqrt_rn(x); }

// Quaternion.Transform (Quaternion.cs:509-535)
__device__ __forceinline__ float3 QTransform(float vx, float vy, float vz, float4 r) {
    float x2 = r.x + r.x, y2 = r.y + r.y, z2 = r.z + r.z;
    float xx2 = r.x * x2, xy2 = r.x * y2, xz2 = r.x * z2;
    float yy2 = r.y * y2, yz2 = r.y * z2, zz2 = r.z * z2;
    float wx2 = r.w * x2, wy2 = r.w * y2, wz2 = r.w * z2;
    float3 o;
    o.x = vx * (1.f - yy2 - zz2) + vy * (xy2 - wz2) + vz * (xz2 + wy2);
    o.y = vx * (xy2 + wz2) + vy * (1.f - xx2 - zz2) + vz * (yz2 - wx2);
    o.z = vx * (xz2 - wy2) + vy * (yz2 + wx2) + vz * (1.f - xx2 - yy2);
    return o;
}

// ContactRefresher.ContactRefresh (ContactRefresher.cs:18-69) and the
// order-preserving removal of the contacts it queues.  Removed contacts lose
// their accumulated impulse (ContactPenetrationConstraint.CleanUp, :65-75); a
// manifold left empty clears sliding and twist (ConvexContactManifoldConstraint.cs:148-154).
template <class V>
__device__ __forceinline__ void RefreshManifoldV(const ManifoldSoA& m, const V& bv, int s, int ra, int rb,
                                                 const StepParams& p) {
    int4 h = m.head[s];
    int count = h.z & 0xff;
    // narrow-phase manifolds (flag 4, BEPUGPU_MANIFOLD_GENERATED) are not refreshed
    if (count == 0 || ((h.z >> 8) & 4)) return;
    int cap = m.capacity;
    float4 pa = make_float4(0, 0, 0, 0), qa = make_float4(0, 0, 0, 1);
    float4 pb = pa, qb = qa;
    if (ra != -1) { pa = bv.Pos(ra); qa = bv.Quat(ra); }
    if (rb != -1) { pb = bv.Pos(rb); qb = bv.Quat(rb); }
    float4 acc = m.penacc[s];
    const float accs[4] = {acc.x, acc.y, acc.z, acc.w};
    // All contact loops are unrolled over the four lanes with a count guard so
    // per-contact values stay in registers.
    float4 cp[4], cn[4], oa[4], ob[4];
    bool keep[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        keep[k] = false;
        if (k < count) {
            cn[k] = m.cnrm[k * cap + s];
            oa[k] = m.offA[k * cap + s];
            ob[k] = m.offB[k * cap + s];
            float3 ta = QTransform(oa[k].x, oa[k].y, oa[k].z, qa);
            float3 tb = QTransform(ob[k].x, ob[k].y, ob[k].z, qb);
            float ax = ta.x + pa.x, ay = ta.y + pa.y, az = ta.z + pa.z;  // RigidTransform.Transform
            float bx = tb.x + pb.x, by = tb.y + pb.y, bz = tb.z + pb.z;
            float abx = bx - ax, aby = by - ay, abz = bz - az;
            float dot = abx * cn[k].x + aby * cn[k].y + abz * cn[k].z;
            float tx = cn[k].x * dot, ty = cn[k].y * dot, tz = cn[k].z * dot;
            tx = abx - tx; ty = aby - ty; tz = abz - tz;
            dot = tx * tx + ty * ty + tz * tz;
            if (!(dot > p.invalidationLengthSquared)) {
                dot = abx * cn[k].x + aby * cn[k].y + abz * cn[k].z;
                float depth = oa[k].w - dot;
                if (!(depth < -p.maximumContactDistance)) {
                    float nx = bx + ax, ny = by + ay, nz = bz + az;
                    cp[k] = make_float4(nx * .5f, ny * .5f, nz * .5f, depth);
                    keep[k] = true;
                }
            }
        }
    }
    // Kept contacts move down in order; every input is already in registers.
    int kept = 0;
    float n0 = 0.f, n1 = 0.f, n2 = 0.f, n3 = 0.f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!keep[k]) continue;
        m.cpos[kept * cap + s] = cp[k];
        if (kept != k) {
            m.cnrm[kept * cap + s] = cn[k];
            m.offA[kept * cap + s] = oa[k];
            m.offB[kept * cap + s] = ob[k];
        }
        n0 = kept == 0 ? accs[k] : n0;
        n1 = kept == 1 ? accs[k] : n1;
        n2 = kept == 2 ? accs[k] : n2;
        n3 = kept == 3 ? accs[k] : n3;
        kept++;
    }
    if (kept != count) {
        m.penacc[s] = make_float4(n0, n1, n2, n3);
        h.z = (h.z & ~0xff) | kept;
        m.head[s] = h;
        if (kept == 0) {
            float4 f = m.fricacc[s];
            m.fricacc[s] = make_float4(0.f, 0.f, 0.f, f.w);
        }
        if (((uint32_t)h.z >> 8) & kManifoldNonConvex) {
            // NonConvexContactManifoldConstraint.RemoveContact (:139-166): each
            // removed contact's friction child goes with it (CleanUp: impulse 0,
            // and Setup clears the direction when the slot is reused).
            int q = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (k >= count) break;
                if (!keep[k]) continue;
                if (q != k) m.cfr[q * cap + s] = m.cfr[k * cap + s];
                q++;
            }
            for (int k = kept; k < count; k++) m.cfr[k * cap + s] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}
// An entry of the narrow phase is active (NarrowPhase.cs:300-332 updates a
// pair while one of its entries is): a dynamic body while its island is
// awake, a kinematic one while its time flag is <= 0; no entity is a static
// entry, inactive.  Only asked with islands.
__device__ __forceinline__ bool EntryActive(const BodySoA& b, int r) {
    if (r < 0) return false;
    if (b.pos[r].w != 0.f) return !IslandAsleep(b, r);
    return b.act[r].y <= 0.f;
}
__device__ __forceinline__ void RefreshManifold(const ManifoldSoA& m, const BodySoA& b, int s, const StepParams& p) {
    int4 h = m.head[s];
    if (b.islandOf && !EntryActive(b, h.x) && !EntryActive(b, h.y)) return;
    RefreshManifoldV(m, GlobalBodies{b}, s, h.x, h.y, p);
}

// Reads velocity-relevant body data for the prestep.
struct PrestepBody {
    float px, py, pz;
    float vx, vy, vz, wx, wy, wz;
    float invMass;
    float I11, I12, I13, I21, I22, I23, I31, I32, I33;
    bool dynamic;
};
template <class V>
__device__ __forceinline__ void LoadPrestepBody(const V& bv, int r, PrestepBody& o) {
    float4 p = bv.Pos(r), v = bv.Vlin(r), w = bv.Vang(r), a = bv.Inv0(r), c = bv.Inv1(r);
    o.px = p.x; o.py = p.y; o.pz = p.z; o.dynamic = p.w != 0.f;
    o.vx = v.x; o.vy = v.y; o.vz = v.z; o.invMass = v.w;
    o.wx = w.x; o.wy = w.y; o.wz = w.z; o.I33 = w.w;
    o.I11 = a.x; o.I12 = a.y; o.I13 = a.z; o.I21 = a.w;
    o.I22 = c.x; o.I23 = c.y; o.I31 = c.z; o.I32 = c.w;
}

// Solver.UnsafePrestep on one ConvexContactManifoldConstraint:
// UpdateSolverActivity (ContactManifoldConstraint.cs:128-145), then Update
// (ConvexContactManifoldConstraint.cs:171-177) on each active child.
// Inputs (head, contacts, material, previous sliding axis) are read from
// `mi` at slot `si`; products (Jacobians, friction lanes, state, head) are
// written to `mo` at slot `so`.  The sweep path passes the same arrays twice;
// a group kernel writes its products to shared memory.
template <class V>
__device__ __forceinline__ void PrestepManifoldIO(const ManifoldSoA& mi, int si, const ManifoldSoA& mo, int so,
                                                  const V& bv, int ra, int rb, const StepParams& p) {
    int4 h = mi.head[si];
    if (mo.head != mi.head) mo.head[so] = h;
    int count = h.z & 0xff;
    uint32_t mflags = (uint32_t)h.z >> 8;
    const int cap = mi.capacity, capo = mo.capacity;
    PrestepBody A, B;
    bool hasA = ra != -1, hasB = rb != -1;
    if (hasA) LoadPrestepBody(bv, ra, A); else A.dynamic = false;
    if (hasB) LoadPrestepBody(bv, rb, B); else B.dynamic = false;
    uint32_t st = 0;
    // BEPUGPU_MANIFOLD_ACTIVE = 1, BEPUGPU_MANIFOLD_SOLVER_RULE = 2
    bool groupActive = (mflags & 1u) && (mflags & 2u) && ((hasA && A.dynamic) || (hasB && B.dynamic));
    const bool nonConvex = mflags & kManifoldNonConvex;
    // A manifold the sliding update skips keeps its axis, a NONCONVEX one its
    // contacts' friction state; lanes staged in shared memory must carry them
    // too (they are written back whole).
    auto carryState = [&]() {
        if (nonConvex) {
            if (mo.cfr != mi.cfr)
                for (int k = 0; k < count; k++) mo.cfr[k * capo + so] = mi.cfr[k * cap + si];
        } else if (mo.saxis != mi.saxis) {
            mo.saxis[so] = mi.saxis[si];
        }
    };
    if (!groupActive) {
        mo.state[so] = make_uint2(0u, 0u);
        carryState();
        return;
    }
    st |= kGroupActive;
    for (int k = 0; k < count; k++) st |= 1u << (kChildShift + k);
    if (count > 0) st |= kSlidingBit | kTwistBit;
    bool dynA = hasA && A.dynamic, dynB = hasB && B.dynamic;
    if (dynA) st |= kDynA;
    if (dynB) st |= kDynB;
    if (hasA) st |= kHasA;
    if (hasB) st |= kHasB;
    float4 mat = mi.mat[si];
    const float kinetic = mat.x, staticF = mat.y, bounciness = mat.z;
    float updateRate = p.updateRate;

    // ContactPenetrationConstraint.Update (ContactPenetrationConstraint.cs:114-233)
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k >= count) break;
        float4 cp = mi.cpos[k * cap + si], cn = mi.cnrm[k * cap + si];
        float lx = -cn.x, ly = -cn.y, lz = -cn.z;
        float aAx = 0, aAy = 0, aAz = 0, aBx = 0, aBy = 0, aBz = 0;
        if (hasA) {
            float rx = cp.x - A.px, ry = cp.y - A.py, rz = cp.z - A.pz;
            aAx = (ry * lz) - (rz * ly);
            aAy = (rz * lx) - (rx * lz);
            aAz = (rx * ly) - (ry * lx);
        }
        if (hasB) {
            float rx = cp.x - B.px, ry = cp.y - B.py, rz = cp.z - B.pz;
            aBx = (ly * rz) - (lz * ry);
            aBy = (lz * rx) - (lx * rz);
            aBz = (lx * ry) - (ly * rx);
        }
        float entryA, entryB, tX, tY, tZ;
        if (dynA) {
            tX = aAx * A.I11 + aAy * A.I21 + aAz * A.I31;
            tY = aAx * A.I12 + aAy * A.I22 + aAz * A.I32;
            tZ = aAx * A.I13 + aAy * A.I23 + aAz * A.I33;
            entryA = tX * aAx + tY * aAy + tZ * aAz + A.invMass;
        } else entryA = 0;
        if (dynB) {
            tX = aBx * B.I11 + aBy * B.I21 + aBz * B.I31;
            tY = aBx * B.I12 + aBy * B.I22 + aBz * B.I32;
            tZ = aBx * B.I13 + aBy * B.I23 + aBz * B.I33;
            entryB = tX * aBx + tY * aBy + tZ * aBz + B.invMass;
        } else entryB = 0;
        float effectiveMassInverse = entryA + entryB;
        float softness = p.softness * effectiveMassInverse * updateRate;
        float v2i = -1 / (softness + effectiveMassInverse);
        float depth = cp.w, bias;
        if (depth >= 0) {
            bias = Minf(Maxf(0, depth - p.allowedPenetration) * p.recoveryStiffness * updateRate, p.maxRecoverySpeed);
            if (bounciness > 0) {
                float rv = 0;
                if (hasA) rv = A.vx * lx + A.vy * ly + A.vz * lz + A.wx * aAx + A.wy * aAy + A.wz * aAz;
                if (hasB) rv += -B.vx * lx - B.vy * ly - B.vz * lz + B.wx * aBx + B.wy * aBy + B.wz * aBz;
                float bounceVelocity = -rv;
                if (bounceVelocity > 0) {
                    float lowThreshold = p.bounceThreshold * 0.3f;
                    float velocityFraction =
                        Clampf((bounceVelocity - lowThreshold) / (p.bounceThreshold - lowThreshold + 1e-7f), 0, 1);
                    float bouncinessVelocity = velocityFraction * bounceVelocity * bounciness;
                    bias = Maxf(bouncinessVelocity, bias);
                }
            }
        } else {
            bias = depth * updateRate;
        }
        mo.pj0[k * capo + so] = make_float4(lx, ly, lz, bias);
        mo.pj1[k * capo + so] = make_float4(aAx, aAy, aAz, softness);
        mo.pj2[k * capo + so] = make_float4(aBx, aBy, aBz, v2i);
    }
    if (count == 0) {
        mo.state[so] = make_uint2(st, 0u);
        carryState();
        return;
    }
    if (nonConvex) {
        // NonConvexContactManifoldConstraint.Update (NonConvexContactManifoldConstraint.cs:180-186):
        // after the penetration children, each contact's ContactFrictionConstraint.Update
        // (ContactFrictionConstraint.cs:147-256).  The friction direction and impulse come
        // from mi; they go to mo with the prestep products.
        st &= ~(kSlidingBit | kTwistBit);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k >= count) break;
            const float4 cp = mi.cpos[k * cap + si], cn = mi.cnrm[k * cap + si];
            float4 fr = mi.cfr[k * cap + si];
            float rax = 0, ray = 0, raz = 0, rbx = 0, rby = 0, rbz = 0;  // the penetration child's ra, rb
            float vAx = 0, vAy = 0, vAz = 0, vBx = 0, vBy = 0, vBz = 0;
            if (hasA) {
                rax = cp.x - A.px; ray = cp.y - A.py; raz = cp.z - A.pz;
                vAx = A.wy * raz - A.wz * ray;  // Vector3.Cross(angularVelocity, ra)
                vAy = A.wz * rax - A.wx * raz;
                vAz = A.wx * ray - A.wy * rax;
                vAx = vAx + A.vx; vAy = vAy + A.vy; vAz = vAz + A.vz;
            }
            if (hasB) {
                rbx = cp.x - B.px; rby = cp.y - B.py; rbz = cp.z - B.pz;
                vBx = B.wy * rbz - B.wz * rby;
                vBy = B.wz * rbx - B.wx * rbz;
                vBz = B.wx * rby - B.wy * rbx;
                vBx = vBx + B.vx; vBy = vBy + B.vy; vBz = vBz + B.vz;
            }
            float rvx = vAx - vBx, rvy = vAy - vBy, rvz = vAz - vBz;
            const float nvs = cn.x * rvx + cn.y * rvy + cn.z * rvz;
            rvx -= nvs * cn.x;
            rvy -= nvs * cn.y;
            rvz -= nvs * cn.z;
            float length = rvx * rvx + rvy * rvy + rvz * rvz;
            float friction;
            if (length > 1e-7f) {  // Toolbox.Epsilon
                length = SqrtOfFloat(length);
                fr.x = rvx / length;
                fr.y = rvy / length;
                fr.z = rvz / length;
                friction = length > p.staticThreshold ? kinetic : staticF;
            } else if (fr.x != 0 || fr.y != 0 || fr.z != 0) {
                friction = staticF;  // the previous step's direction
            } else {
                mo.cfr[k * capo + so] = fr;
                continue;  // no direction: isActiveInSolver = false for this step
            }
            st |= 1u << (kFricShift + k);
            const float lx = fr.x, ly = fr.y, lz = fr.z;
            const float aAx = (ray * lz) - (raz * ly), aAy = (raz * lx) - (rax * lz), aAz = (rax * ly) - (ray * lx);
            const float aBx = (ly * rbz) - (lz * rby), aBy = (lz * rbx) - (lx * rbz), aBz = (lx * rby) - (ly * rbx);
            float entryA, entryB, tX, tY, tZ;
            if (dynA) {
                tX = aAx * A.I11 + aAy * A.I21 + aAz * A.I31;
                tY = aAx * A.I12 + aAy * A.I22 + aAz * A.I32;
                tZ = aAx * A.I13 + aAy * A.I23 + aAz * A.I33;
                entryA = tX * aAx + tY * aAy + tZ * aAz + A.invMass;
            } else entryA = 0;
            if (dynB) {
                tX = aBx * B.I11 + aBy * B.I21 + aBz * B.I31;
                tY = aBx * B.I12 + aBy * B.I22 + aBz * B.I32;
                tZ = aBx * B.I13 + aBy * B.I23 + aBz * B.I33;
                entryB = tX * aBx + tY * aBy + tZ * aBz + B.invMass;
            } else entryB = 0;
            mo.cfr[k * capo + so] = fr;
            mo.cfa[k * capo + so] = make_float4(aAx, aAy, aAz, -1 / (entryA + entryB));
            mo.cfb[k * capo + so] = make_float4(aBx, aBy, aBz, friction);
        }
        mo.state[so] = make_uint2(st, 0u);
        return;
    }

    // SlidingFrictionTwoAxis.Update (SlidingFrictionTwoAxis.cs:242-440)
    float4 c0 = mi.cpos[si];
    float mcx, mcy, mcz;
    if (count == 1) {
        mcx = c0.x; mcy = c0.y; mcz = c0.z;
    } else {
        float4 c1 = mi.cpos[cap + si];
        mcx = c0.x + c1.x; mcy = c0.y + c1.y; mcz = c0.z + c1.z;
        if (count == 2) {
            mcx *= .5f; mcy *= .5f; mcz *= .5f;
        } else {
            float4 c2 = mi.cpos[2 * cap + si];
            mcx = c2.x + mcx; mcy = c2.y + mcy; mcz = c2.z + mcz;
            if (count == 3) {
                mcx *= .333333333f; mcy *= .333333333f; mcz *= .333333333f;
            } else {
                float4 c3 = mi.cpos[3 * cap + si];
                mcx = c3.x + mcx; mcy = c3.y + mcy; mcz = c3.z + mcz;
                mcx *= .25f; mcy *= .25f; mcz *= .25f;
            }
        }
    }
    float rax = 0, ray = 0, raz = 0, rbx = 0, rby = 0, rbz = 0;
    float vAx = 0, vAy = 0, vAz = 0, vBx = 0, vBy = 0, vBz = 0;
    if (hasA) {
        rax = mcx - A.px; ray = mcy - A.py; raz = mcz - A.pz;
        vAx = A.wy * raz - A.wz * ray;  // Vector3.Cross(angularVelocity, ra)
        vAy = A.wz * rax - A.wx * raz;
        vAz = A.wx * ray - A.wy * rax;
        vAx = vAx + A.vx; vAy = vAy + A.vy; vAz = vAz + A.vz;
    }
    if (hasB) {
        rbx = mcx - B.px; rby = mcy - B.py; rbz = mcz - B.pz;
        vBx = B.wy * rbz - B.wz * rby;
        vBy = B.wz * rbx - B.wx * rbz;
        vBz = B.wx * rby - B.wy * rbx;
        vBx = vBx + B.vx; vBy = vBy + B.vy; vBz = vBz + B.vz;
    }
    float rvx = vAx - vBx, rvy = vAy - vBy, rvz = vAz - vBz;
    float4 n0 = mi.cnrm[si];
    float nx = n0.x, ny = n0.y, nz = n0.z;
    float normalVelocityScalar = nx * rvx + ny * rvy + nz * rvz;
    rvx -= normalVelocityScalar * nx;
    rvy -= normalVelocityScalar * ny;
    rvz -= normalVelocityScalar * nz;
    float4 axis = mi.saxis[si];
    float l11 = axis.x, l12 = axis.y, l13 = axis.z;
    float friction;
    float length = rvx * rvx + rvy * rvy + rvz * rvz;
    if (length > 1e-7f) {
        length = SqrtOfFloat(length);
        float inverseLength = 1 / length;
        l11 = rvx * inverseLength;
        l12 = rvy * inverseLength;
        l13 = rvz * inverseLength;
        friction = length > p.staticThreshold ? kinetic : staticF;
    } else {
        friction = staticF;
        if (!(l11 != 0 || l12 != 0 || l13 != 0)) {
            // Vector3.Cross(normal, Toolbox.RightVector)
            float x1 = ny * 0.f - nz * 0.f, y1 = nz * 1.f - nx * 0.f, z1 = nx * 0.f - ny * 1.f;
            length = x1 * x1 + y1 * y1 + z1 * z1;
            if (length > 1e-7f) {
                length = SqrtOfFloat(length);
                float inverseLength = 1 / length;
                l11 = x1 * inverseLength; l12 = y1 * inverseLength; l13 = z1 * inverseLength;
            } else {
                // Vector3.Cross(normal, Toolbox.UpVector), then Normalize
                x1 = ny * 0.f - nz * 1.f; y1 = nz * 0.f - nx * 0.f; z1 = nx * 1.f - ny * 0.f;
                float inv = dr::InvSqrtAsDouble(x1 * x1 + y1 * y1 + z1 * z1);
                l11 = x1 * inv; l12 = y1 * inv; l13 = z1 * inv;
            }
        }
    }
    float l21 = (l12 * nz) - (l13 * ny);
    float l22 = (l13 * nx) - (l11 * nz);
    float l23 = (l11 * ny) - (l12 * nx);
    float aA11 = 0, aA12 = 0, aA13 = 0, aA21 = 0, aA22 = 0, aA23 = 0;
    float aB11 = 0, aB12 = 0, aB13 = 0, aB21 = 0, aB22 = 0, aB23 = 0;
    if (hasA) {
        aA11 = (ray * l13) - (raz * l12);
        aA12 = (raz * l11) - (rax * l13);
        aA13 = (rax * l12) - (ray * l11);
        aA21 = (ray * l23) - (raz * l22);
        aA22 = (raz * l21) - (rax * l23);
        aA23 = (rax * l22) - (ray * l21);
    }
    if (hasB) {
        aB11 = (l12 * rbz) - (l13 * rby);
        aB12 = (l13 * rbx) - (l11 * rbz);
        aB13 = (l11 * rby) - (l12 * rbx);
        aB21 = (l22 * rbz) - (l23 * rby);
        aB22 = (l23 * rbx) - (l21 * rbz);
        aB23 = (l21 * rby) - (l22 * rbx);
    }
    float eA11 = 0, eA12 = 0, eA21 = 0, eA22 = 0, eB11 = 0, eB12 = 0, eB21 = 0, eB22 = 0;
    if (dynA) {
        // Matrix2x3.Multiply(angularA, I) (Matrix2x3.cs:94-111)
        float t11 = aA11 * A.I11 + aA12 * A.I21 + aA13 * A.I31;
        float t12 = aA11 * A.I12 + aA12 * A.I22 + aA13 * A.I32;
        float t13 = aA11 * A.I13 + aA12 * A.I23 + aA13 * A.I33;
        float t21 = aA21 * A.I11 + aA22 * A.I21 + aA23 * A.I31;
        float t22 = aA21 * A.I12 + aA22 * A.I22 + aA23 * A.I32;
        float t23 = aA21 * A.I13 + aA22 * A.I23 + aA23 * A.I33;
        // Matrix2x2.Multiply(transform, transpose(angularA)) (Matrix2x2.cs:245-252)
        eA11 = t11 * aA11 + t12 * aA12 + t13 * aA13;
        eA12 = t11 * aA21 + t12 * aA22 + t13 * aA23;
        eA21 = t21 * aA11 + t22 * aA12 + t23 * aA13;
        eA22 = t21 * aA21 + t22 * aA22 + t23 * aA23;
        eA11 += A.invMass;
        eA22 += A.invMass;
    }
    if (dynB) {
        float t11 = aB11 * B.I11 + aB12 * B.I21 + aB13 * B.I31;
        float t12 = aB11 * B.I12 + aB12 * B.I22 + aB13 * B.I32;
        float t13 = aB11 * B.I13 + aB12 * B.I23 + aB13 * B.I33;
        float t21 = aB21 * B.I11 + aB22 * B.I21 + aB23 * B.I31;
        float t22 = aB21 * B.I12 + aB22 * B.I22 + aB23 * B.I32;
        float t23 = aB21 * B.I13 + aB22 * B.I23 + aB23 * B.I33;
        eB11 = t11 * aB11 + t12 * aB12 + t13 * aB13;
        eB12 = t11 * aB21 + t12 * aB22 + t13 * aB23;
        eB21 = t21 * aB11 + t22 * aB12 + t23 * aB13;
        eB22 = t21 * aB21 + t22 * aB22 + t23 * aB23;
        eB11 += B.invMass;
        eB22 += B.invMass;
    }
    float v11 = -eA11 - eB11, v12 = -eA12 - eB12, v21 = -eA21 - eB21, v22 = -eA22 - eB22;
    // Matrix2x2.Invert (Matrix2x2.cs:160-174)
    float det = 1 / (v11 * v22 - v12 * v21);
    float i11 = v22 * det, i12 = -v12 * det, i21 = -v21 * det, i22 = v11 * det;

    // TwistFrictionConstraint.Update (TwistFrictionConstraint.cs:114-175)
    float entryA, entryB, tX, tY, tZ;
    if (dynA) {
        tX = nx * A.I11 + ny * A.I21 + nz * A.I31;
        tY = nx * A.I12 + ny * A.I22 + nz * A.I32;
        tZ = nx * A.I13 + ny * A.I23 + nz * A.I33;
        entryA = tX * nx + tY * ny + tZ * nz + A.invMass;
    } else entryA = 0;
    if (dynB) {
        tX = nx * B.I11 + ny * B.I21 + nz * B.I31;
        tY = nx * B.I12 + ny * B.I22 + nz * B.I32;
        tZ = nx * B.I13 + ny * B.I23 + nz * B.I33;
        entryB = tX * nx + tY * ny + tZ * nz + B.invMass;
    } else entryB = 0;
    float tv2i = -1 / (entryA + entryB);
    float rav = 0;
    if (hasA) rav = A.wx * nx + A.wy * ny + A.wz * nz;
    if (hasB) rav -= B.wx * nx + B.wy * ny + B.wz * nz;
    float tfriction = fabsf(rav) > p.staticThreshold || fabsf(rvx) + fabsf(rvy) + fabsf(rvz) > p.staticThreshold
                          ? kinetic
                          : staticF;
    tfriction *= p.twistFactor;
    float lev[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k >= count) break;
        float4 cp = mi.cpos[k * cap + si];
        float ox = cp.x - mcx, oy = cp.y - mcy, oz = cp.z - mcz;
        lev[k] = SqrtOfFloat(ox * ox + oy * oy + oz * oz);
    }

    mo.s0[so] = make_float4(rax, ray, raz, friction);
    mo.s1[so] = make_float4(rbx, rby, rbz, i11);
    mo.saxis[so] = make_float4(l11, l12, l13, i12);
    mo.s3[so] = make_float4(l21, l22, l23, i21);
    mo.s4[so] = make_float4(aA11, aA12, aA13, i22);
    mo.s5[so] = make_float4(aA21, aA22, aA23, tv2i);
    mo.s6[so] = make_float4(aB11, aB12, aB13, tfriction);
    mo.s7[so] = make_float4(aB21, aB22, aB23, 0.f);
    mo.lever[so] = make_float4(lev[0], lev[1], lev[2], lev[3]);
    mo.state[so] = make_uint2(st, 0u);
}
template <class V>
__device__ __forceinline__ void PrestepManifoldV(const ManifoldSoA& m, const V& bv, int s, int ra, int rb,
                                                 const StepParams& p) {
    PrestepManifoldIO(m, s, m, s, bv, ra, rb, p);
}
__device__ __forceinline__ void PrestepManifold(const ManifoldSoA& m, const BodySoA& b, int s, const StepParams& p) {
    int4 h = m.head[s];
    PrestepManifoldV(m, GlobalBodies{b}, s, h.x, h.y, p);
}

// Warm start: ConvexContactManifoldConstraint.ExclusiveUpdate
// (ConvexContactManifoldConstraint.cs:186-192) with the children's
// ExclusiveUpdate bodies (ContactPenetrationConstraint.cs:240-271,
// SlidingFrictionTwoAxis.cs:447-482, TwistFrictionConstraint.cs:182-204).
template <class Body>
__device__ __forceinline__ void WarmStartManifold(const ManifoldSoA& m, int s, Body& A, Body& B, uint32_t st,
                                                  int count) {
    const int cap = m.capacity;
    bool dynA = st & kDynA, dynB = st & kDynB;
    float4 acc4 = m.penacc[s];
    const float accs[4] = {acc4.x, acc4.y, acc4.z, acc4.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k >= count) break;
        if (!(st & (1u << (kChildShift + k)))) continue;
        float4 j0 = m.pj0[k * cap + s], j1 = m.pj1[k * cap + s], j2 = m.pj2[k * cap + s];
        float acc = accs[k];
        float lx = acc * j0.x, ly = acc * j0.y, lz = acc * j0.z;
        if (dynA) {
            ApplyLinear(A, lx, ly, lz);
            ApplyAngular(A, acc * j1.x, acc * j1.y, acc * j1.z);
        }
        if (dynB) {
            ApplyLinear(B, -lx, -ly, -lz);
            ApplyAngular(B, acc * j2.x, acc * j2.y, acc * j2.z);
        }
    }
    if (st & (0xfu << kFricShift)) {
        // ContactFrictionConstraint.ExclusiveUpdate (ContactFrictionConstraint.cs:258-289)
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k >= count) break;
            if (!(st & (1u << (kFricShift + k)))) continue;
            const float4 fr = m.cfr[k * cap + s];
            const float acc = fr.w;
            const float lx = acc * fr.x, ly = acc * fr.y, lz = acc * fr.z;
            if (dynA) {
                const float4 fa = m.cfa[k * cap + s];
                ApplyLinear(A, lx, ly, lz);
                ApplyAngular(A, acc * fa.x, acc * fa.y, acc * fa.z);
            }
            if (dynB) {
                const float4 fb = m.cfb[k * cap + s];
                ApplyLinear(B, -lx, -ly, -lz);
                ApplyAngular(B, acc * fb.x, acc * fb.y, acc * fb.z);
            }
        }
        return;
    }
    if (count == 0) return;
    float4 f = m.fricacc[s];
    if (st & kSlidingBit) {
        float ax = f.x, ay = f.y;
        float4 L1 = m.saxis[s], L2 = m.s3[s], A1 = m.s4[s], A2 = m.s5[s], B1 = m.s6[s], B2 = m.s7[s];
        float lx = ax * L1.x + ay * L2.x;
        float ly = ax * L1.y + ay * L2.y;
        float lz = ax * L1.z + ay * L2.z;
        if (dynA) {
            float gx = ax * A1.x + ay * A2.x, gy = ax * A1.y + ay * A2.y, gz = ax * A1.z + ay * A2.z;
            ApplyLinear(A, lx, ly, lz);
            ApplyAngular(A, gx, gy, gz);
        }
        if (dynB) {
            float gx = ax * B1.x + ay * B2.x, gy = ax * B1.y + ay * B2.y, gz = ax * B1.z + ay * B2.z;
            ApplyLinear(B, -lx, -ly, -lz);
            ApplyAngular(B, gx, gy, gz);
        }
    }
    if (st & kTwistBit) {
        float4 j0 = m.pj0[s];  // twist axis = contact 0 normal = -linearA of penetration 0
        float nx = -j0.x, ny = -j0.y, nz = -j0.z;
        float t = f.z;
        float gx = t * nx, gy = t * ny, gz = t * nz;
        if (dynA) ApplyAngular(A, gx, gy, gz);
        if (dynB) ApplyAngular(B, -gx, -gy, -gz);
    }
}

// Programmatic dependent launch: a sweep kernel lets the next one start its
// preamble (griddepcontrol.launch_dependents) and waits for the previous one's
// completion and memory (griddepcontrol.wait) before it reads what that one
// writes.  Both are no-ops for a kernel launched without the attribute.
__device__ __forceinline__ void LetDependentsLaunch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void WaitForPrerequisites() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The prestep products a solve visit reads; none of them change during the
// sweeps, so a sweep kernel may load them before the sweep it follows ends.
struct SolveLanes {
    float4 J0[4], J1[4], J2[4];
    float4 S0, S1, L1, L2, A1, A2, B1, B2, LEV;
};
__device__ __forceinline__ void LoadSolveLanes(const ManifoldSoA& m, int s, int count, bool friction,
                                               SolveLanes& L) {
    const int cap = m.capacity;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k < count) {
            L.J0[k] = m.pj0[k * cap + s];
            L.J1[k] = m.pj1[k * cap + s];
            L.J2[k] = m.pj2[k * cap + s];
        }
    }
    if (friction) {
        L.S0 = m.s0[s]; L.S1 = m.s1[s]; L.L1 = m.saxis[s]; L.L2 = m.s3[s];
        L.A1 = m.s4[s]; L.A2 = m.s5[s]; L.B1 = m.s6[s]; L.B2 = m.s7[s];
        L.LEV = m.lever[s];
    }
}

// One solver visit of a manifold: Solver.UnsafeSolveIteration (Solver.cs:285-314)
// -> ConvexContactManifoldConstraint.SolveIteration (:199-212) ->
// SolverGroup.SolveUpdateable (SolverGroup.cs:117-150) on each child.
// Children solve strictly in order: they are a Gauss-Seidel sequence.
// pre: the visit's lanes already loaded (LoadSolveLanes with friction = count > 0), or null.
template <class Body>
__device__ __forceinline__ void SolveManifold(const ManifoldSoA& m, int s, Body& A, Body& B, uint2& state,
                                              int count, const StepParams& p, const SolveLanes* pre = nullptr) {
    const int cap = m.capacity;
    uint32_t st = state.x, zeros = state.y;
    // UnsafeSolveIteration on the group
    uint32_t iter = (st >> kIterShift) + 1;
    st = (st & 0xffffu) | (iter << kIterShift);
    if (!((int)iter <= p.iterationLimit && (int)iter <= p.maximumIterationCount)) {
        state = make_uint2(st & ~kGroupActive, zeros);
        return;
    }
    bool hasA = st & kHasA, hasB = st & kHasB;  // kinematic partners' velocities still enter
    bool dynA = st & kDynA, dynB = st & kDynB;
    int activeConstraints = 0;
    // Every load of the visit is issued before the sequential solves start.
    float4 acc4 = m.penacc[s];
    float accs[4] = {acc4.x, acc4.y, acc4.z, acc4.w};
    SolveLanes Lv;
    if (pre) Lv = *pre;
    else LoadSolveLanes(m, s, count, (st & (kSlidingBit | kTwistBit)) != 0, Lv);
    const float4 *J0 = Lv.J0, *J1 = Lv.J1, *J2 = Lv.J2;
    float4 f = m.fricacc[s];
    const float4 S0 = Lv.S0, S1 = Lv.S1, L1 = Lv.L1, L2 = Lv.L2, A1 = Lv.A1, A2 = Lv.A2, B1 = Lv.B1, B2 = Lv.B2,
                 LEV = Lv.LEV;
    // SolveUpdateable bookkeeping for child c (its zero-impulse nibble) given
    // its |impulse|; `bit` is its activity bit.
    auto accountBit = [&](int c, uint32_t bit, float r) {
        uint32_t z = (zeros >> (4 * c)) & 0xfu;
        if (r < p.minimumImpulse) {
            z++;
            if ((int)z > p.minimumIterationCount) st &= ~bit;
            else activeConstraints++;
        } else {
            z = 0;
            activeConstraints++;
        }
        zeros = (zeros & ~(0xfu << (4 * c))) | ((z & 0xfu) << (4 * c));
    };
    auto account = [&](int c, float r) { accountBit(c, 1u << (kChildShift + c), r); };
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k >= count) break;
        if (!(st & (1u << (kChildShift + k)))) continue;
        // child currentIterations equals the group's here; the cap passed above
        const float4 j0 = J0[k], j1 = J1[k], j2 = J2[k];
        float lx = j0.x, ly = j0.y, lz = j0.z, bias = j0.w, softness = j1.w, v2i = j2.w;
        float rv = 0;
        if (hasA) rv = A.vx * lx + A.vy * ly + A.vz * lz + A.wx * j1.x + A.wy * j1.y + A.wz * j1.z;
        if (hasB) rv += -B.vx * lx - B.vy * ly - B.vz * lz + B.wx * j2.x + B.wy * j2.y + B.wz * j2.z;
        float lambda = (rv - bias + softness * accs[k]) * v2i;
        float prev = accs[k];
        accs[k] = Maxf(0, accs[k] + lambda);
        lambda = accs[k] - prev;
        float ix = lambda * lx, iy = lambda * ly, iz = lambda * lz;
        if (dynA) {
            ApplyLinear(A, ix, iy, iz);
            ApplyAngular(A, lambda * j1.x, lambda * j1.y, lambda * j1.z);
        }
        if (dynB) {
            ApplyLinear(B, -ix, -iy, -iz);
            ApplyAngular(B, lambda * j2.x, lambda * j2.y, lambda * j2.z);
        }
        account(k, fabsf(lambda));
    }
    if (st & (0xfu << kFricShift)) {
        // NONCONVEX: each contact's ContactFrictionConstraint.SolveIteration
        // (ContactFrictionConstraint.cs:95-143), after every penetration child.
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k >= count) break;
            const uint32_t bit = 1u << (kFricShift + k);
            if (!(st & bit)) continue;
            float4 fr = m.cfr[k * cap + s];
            const float4 fa = m.cfa[k * cap + s], fb = m.cfb[k * cap + s];
            float velocity = 0;
            if (hasA)
                velocity += A.vx * fr.x + A.vy * fr.y + A.vz * fr.z + A.wx * fa.x + A.wy * fa.y + A.wz * fa.z;
            if (hasB)
                velocity += -B.vx * fr.x - B.vy * fr.y - B.vz * fr.z + B.wx * fb.x + B.wy * fb.y + B.wz * fb.z;
            float lambda = velocity * fa.w;
            const float prev = fr.w, maxForce = fb.w * accs[k];
            fr.w = Clampf(fr.w + lambda, -maxForce, maxForce);
            lambda = fr.w - prev;
            const float ix = lambda * fr.x, iy = lambda * fr.y, iz = lambda * fr.z;
            if (dynA) {
                ApplyLinear(A, ix, iy, iz);
                ApplyAngular(A, lambda * fa.x, lambda * fa.y, lambda * fa.z);
            }
            if (dynB) {
                ApplyLinear(B, -ix, -iy, -iz);
                ApplyAngular(B, lambda * fb.x, lambda * fb.y, lambda * fb.z);
            }
            accountBit(4 + k, bit, fabsf(lambda));
            m.cfr[k * cap + s] = fr;
        }
    }
    if (st & kSlidingBit) {
        // SlidingFrictionTwoAxis.SolveIteration (SlidingFrictionTwoAxis.cs:155-234)
        float dvx = 0, dvy = 0, dvz = 0;
        if (hasA) {
            dvx = A.vx + (A.wy * S0.z) - (A.wz * S0.y);
            dvy = A.vy + (A.wz * S0.x) - (A.wx * S0.z);
            dvz = A.vz + (A.wx * S0.y) - (A.wy * S0.x);
        }
        if (hasB) {
            dvx += -B.vx - (B.wy * S1.z) + (B.wz * S1.y);
            dvy += -B.vy - (B.wz * S1.x) + (B.wx * S1.z);
            dvz += -B.vz - (B.wx * S1.y) + (B.wy * S1.x);
        }
        float lxv = dvx * L1.x + dvy * L1.y + dvz * L1.z;
        float lyv = dvx * L2.x + dvy * L2.y + dvz * L2.z;
        float x = lxv;
        lxv = x * S1.w + lyv * L2.w;   // M11, M21
        lyv = x * L1.w + lyv * A1.w;   // M12, M22
        float px = f.x, py = f.y;
        f.x += lxv;
        f.y += lyv;
        float length = f.x * f.x + f.y * f.y;
        float maximumFrictionForce = 0;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (k < count) maximumFrictionForce += accs[k];
        maximumFrictionForce *= S0.w;
        if (length > maximumFrictionForce * maximumFrictionForce) {
            length = maximumFrictionForce / SqrtOfFloat(length);
            f.x *= length;
            f.y *= length;
        }
        lxv = f.x - px;
        lyv = f.y - py;
        float gx = lxv * L1.x + lyv * L2.x, gy = lxv * L1.y + lyv * L2.y, gz = lxv * L1.z + lyv * L2.z;
        if (dynA) {
            ApplyLinear(A, gx, gy, gz);
            ApplyAngular(A, lxv * A1.x + lyv * A2.x, lxv * A1.y + lyv * A2.y, lxv * A1.z + lyv * A2.z);
        }
        if (dynB) {
            ApplyLinear(B, -gx, -gy, -gz);
            ApplyAngular(B, lxv * B1.x + lyv * B2.x, lxv * B1.y + lyv * B2.y, lxv * B1.z + lyv * B2.z);
        }
        account(4, fabsf(lxv) + fabsf(lyv));
    }
    if (st & kTwistBit) {
        // TwistFrictionConstraint.SolveIteration (TwistFrictionConstraint.cs:65-107)
        const float4 j0 = J0[0], lev = LEV;
        float v2i = A2.w, friction = B1.w;
        float nx = -j0.x, ny = -j0.y, nz = -j0.z;
        float lambda = 0;
        if (hasA) lambda = A.wx * nx + A.wy * ny + A.wz * nz;
        if (hasB) lambda -= B.wx * nx + B.wy * ny + B.wz * nz;
        lambda *= v2i;
        float prev = f.z;
        const float levs[4] = {lev.x, lev.y, lev.z, lev.w};
        float maximumFrictionForce = 0;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (k < count) maximumFrictionForce += levs[k] * accs[k];
        maximumFrictionForce *= friction;
        f.z = Clampf(f.z + lambda, -maximumFrictionForce, maximumFrictionForce);
        lambda = f.z - prev;
        float gx = lambda * nx, gy = lambda * ny, gz = lambda * nz;
        if (dynA) ApplyAngular(A, gx, gy, gz);
        if (dynB) ApplyAngular(B, -gx, -gy, -gz);
        account(5, fabsf(lambda));
    }
    if (activeConstraints <= 0) st &= ~kGroupActive;
    m.penacc[s] = make_float4(accs[0], accs[1], accs[2], accs[3]);
    m.fricacc[s] = f;
    state = make_uint2(st, zeros);
}

}  // namespace bepugpu
