// Oracle -- test infrastructure only (tests, smoke check, CPU-baseline legs of
// bench.py).  The product library never links this file.
//
// A C++ restatement of the reference's solver path, class for class:
//   Entity                    BEPUphysics/Entities/EntityBase.cs
//   SolverUpdateable/Settings BEPUphysics/Constraints/SolverUpdateable.cs, SolverSettings.cs
//   SolverGroup               BEPUphysics/Constraints/SolverGroups/SolverGroup.cs
//   Contact manifold family   BEPUphysics/Constraints/Collision/*.cs
//   Joints                    oracle/bepu_oracle_joints.inc
//   Solver                    BEPUphysics/Constraints/Solver.cs
//   PermutationMapper         BEPUutilities/PermutationMapper.cs
//   ContactRefresher          BEPUphysics/CollisionTests/ContactRefresher.cs
// Build with -ffp-contract=off so float rounding follows C#'s evaluation.
#include "bepu_oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "bepu_math.h"

namespace oracle {

// ---------------------------------------------------------------- settings --
struct Settings {
    Vec3 gravity;
    int iterationLimit;
    float minimumImpulse;
    int minimumIterationCount;
    int maximumIterationCount;
    float softness, recoveryStiffness, maxRecoverySpeed, staticThreshold, twistFactor,
        bounceThreshold, allowedPenetration, invalidationLengthSquared, maximumContactDistance;
    // DeactivationManager (DeactivationManager.cs:18-20,60)
    bool useStabilization = true;
    float velocityLowerLimit = .26f, velocityLowerLimitSquared = .26f * .26f, lowVelocityTimeMinimum = 1;
    int maximumDeactivationAttemptsPerFrame = 100;  // DeactivationManager.cs:15
};

// ---------------------------------------------------------------- PermutationMapper --
static const long long kPrimes[] = {
#include "permutation_primes.inc"
};
static const int kPrimeCount = (int)(sizeof(kPrimes) / sizeof(kPrimes[0]));

// PermutationMapper.cs:27-44 (PermutationIndex setter) and :124-127.
struct PermutationMapper {
    long long permutationIndex = 0, currentPrime = kPrimes[0], currentOffset = 0;
    void SetIndex(long long value) {
        permutationIndex = value < 0 ? value + LLONG_MAX + 1 : value;
        currentPrime = kPrimes[permutationIndex % kPrimeCount];
        // long multiplication wraps in C#; do it unsigned to keep it defined here.
        currentOffset = (long long)((unsigned long long)currentPrime * (unsigned long long)permutationIndex);
        if (currentOffset < 0) currentOffset = currentOffset + LLONG_MAX + 1;
    }
    long long Map(long long index, int setSize) const {
        return (long long)(((unsigned long long)index * (unsigned long long)currentPrime +
                            (unsigned long long)currentOffset) %
                           (unsigned long long)setSize);
    }
};

// ---------------------------------------------------------------- Entity --
struct SpinLock {
    std::atomic<int> owner{-1};
    void Enter() {
        int expected = -1;
        while (!owner.compare_exchange_weak(expected, 0, std::memory_order_acquire)) {
            expected = -1;
            std::this_thread::yield();
        }
    }
    void Exit() { owner.store(-1, std::memory_order_release); }
};

// SimulationIsland.cs:12-56: the state DeactivateObjects reads and writes.
struct Island {
    bool isActive = true, allowDeactivation = true;
    int memberCount = 0, candidates = 0;  // candidates: members that are deactivation candidates
    int deactivationCandidateCount() const { return candidates; }
};

struct Entity {
    int index = 0;
    Island* island = nullptr;  // SimulationIslandMember.SimulationIsland: null for kinematic bodies
                               // and for every body of a space without islands (all awake)
    Vec3 position;
    Quat orientation;
    Mat3 orientationMatrix;
    Vec3 linearVelocity, angularVelocity;
    float inverseMass = 0;
    Mat3 localInertiaTensorInverse, inertiaTensorInverse;
    float linearDamping = .03f, angularDamping = .15f;
    bool isDynamic = false;
    SpinLock locker;
    // activityInformation (SimulationIslandMember.cs:17-19, 278-312).  Every
    // dynamic body's simulation island is awake here.
    float previousVelocity = 0, velocityTimeBelowLimit = 0;
    bool isSlowing = false, isDeactivationCandidate = false, isAlwaysActive = false, allowStabilization = true;
    float linearDampingBoost = 0, angularDampingBoost = 0;

    // SimulationIslandMember.IsActive (:225-248): the island's state, or the
    // time flag without an island (kinematic bodies).  A dynamic body of a
    // space without islands counts as awake.
    bool IsActive() const {
        if (island) return island->isActive;
        return isDynamic || velocityTimeBelowLimit <= 0;
    }
    // The IsDeactivationCandidate setter (:171-190)
    void SetDeactivationCandidate(bool value) {
        isDeactivationCandidate = value;
        if (!value) velocityTimeBelowLimit = 0;
    }
    // SimulationIslandMember.UpdateDeactivationCandidacy (:53-164).  Returns
    // whether an active kinematic body wakes its connections' islands
    // (:135-159); the caller does the waking.
    bool UpdateDeactivationCandidacy(float dt, const Settings& s) {
        float velocity = LengthSquared(linearVelocity) + LengthSquared(angularVelocity);
        bool isActive = IsActive();
        bool wakes = false;
        if (isActive) {
            isSlowing = velocity <= previousVelocity;
            if (isDynamic) {
                if (velocity < s.velocityLowerLimitSquared) velocityTimeBelowLimit += dt;
                else velocityTimeBelowLimit = 0;
                if (!isAlwaysActive) {
                    if (!isDeactivationCandidate) {
                        if (velocityTimeBelowLimit > s.lowVelocityTimeMinimum && isSlowing)
                            SetDeactivationCandidate(true);
                    } else {
                        if (velocityTimeBelowLimit <= s.lowVelocityTimeMinimum) SetDeactivationCandidate(false);
                    }
                } else {
                    SetDeactivationCandidate(false);
                }
            } else {
                SetDeactivationCandidate(velocity == 0 && !isAlwaysActive);
                if (isDeactivationCandidate) {
                    if (velocityTimeBelowLimit == 0) velocityTimeBelowLimit = 1;
                    else if (velocityTimeBelowLimit < 0) velocityTimeBelowLimit = 0;
                } else {
                    velocityTimeBelowLimit = -1;
                }
                wakes = velocityTimeBelowLimit <= 0;
            }
        }
        previousVelocity = velocity;
        return wakes;
    }
    // EntityBase.ModifyLinearDamping / ModifyAngularDamping (EntityBase.cs:1205-1221)
    void ModifyLinearDamping(float damping) {
        float totalDamping = linearDamping + linearDampingBoost;
        float remainder = 1 - totalDamping;
        linearDampingBoost += damping * remainder;
    }
    void ModifyAngularDamping(float damping) {
        float totalDamping = angularDamping + angularDampingBoost;
        float remainder = 1 - totalDamping;
        angularDampingBoost += damping * remainder;
    }

    // EntityBase.cs:754-761
    void ApplyLinearImpulse(const Vec3& impulse) {
        linearVelocity.X += impulse.X * inverseMass;
        linearVelocity.Y += impulse.Y * inverseMass;
        linearVelocity.Z += impulse.Z * inverseMass;
    }
    // EntityBase.cs:769-786, the non-CONSERVE branch
    void ApplyAngularImpulse(const Vec3& impulse) {
        const Mat3& I = inertiaTensorInverse;
        angularVelocity.X += impulse.X * I.M11 + impulse.Y * I.M21 + impulse.Z * I.M31;
        angularVelocity.Y += impulse.X * I.M12 + impulse.Y * I.M22 + impulse.Z * I.M32;
        angularVelocity.Z += impulse.X * I.M13 + impulse.Y * I.M23 + impulse.Z * I.M33;
    }
    // EntityBase.cs:911-975
    void UpdateForForces(float dt, const Vec3& gravityDt, const Settings& s) {
        linearVelocity = Add(gravityDt, linearVelocity);
        // Boost damping at very low velocities (:926-936).
        if (s.useStabilization && allowStabilization &&
            (isSlowing || velocityTimeBelowLimit > s.lowVelocityTimeMinimum)) {
            float energy = LengthSquared(linearVelocity) + LengthSquared(angularVelocity);
            if (energy < s.velocityLowerLimitSquared) {
                float boost = 1 - (float)(std::sqrt((double)energy) / (double)(2.f * s.velocityLowerLimit));
                ModifyAngularDamping(boost);
                ModifyLinearDamping(boost);
            }
        }
        float linear = linearDamping + linearDampingBoost;
        if (linear > 0)
            linearVelocity = Multiply(linearVelocity, (float)std::pow((double)Clamp(1 - linear, 0, 1), (double)dt));
        float angular = angularDamping + angularDampingBoost;
        if (angular > 0)
            angularVelocity = Multiply(angularVelocity, (float)std::pow((double)Clamp(1 - angular, 0, 1), (double)dt));
        linearDampingBoost = 0;
        angularDampingBoost = 0;
        Mat3 multiplied = MultiplyTransposed(orientationMatrix, localInertiaTensorInverse);
        inertiaTensorInverse = Multiply(multiplied, orientationMatrix);
    }
    // EntityBase.cs:1124-1160, PositionUpdateMode.Discrete
    void PreUpdatePosition(float dt) {
        Vec3 increment = Multiply(angularVelocity, dt * .5f);
        Quat multiplier{increment.X, increment.Y, increment.Z, 0};
        multiplier = QMultiply(multiplier, orientation);
        orientation = QAdd(orientation, multiplier);
        QNormalize(orientation);
        orientationMatrix = CreateFromQuaternion(orientation);
        increment = Multiply(linearVelocity, dt);
        position = Add(position, increment);
    }
};

// ---------------------------------------------------------------- SolverUpdateable --
struct SolverSettings {
    int currentIterations = 0;
    int iterationsAtZeroImpulse = 0;
    int maximumIterationCount = 0x7fffffff;
    int minimumIterationCount = 1;
    float minimumImpulse = .001f;
};

struct Space;

struct SolverUpdateable {
    bool isActive = true;
    bool isActiveInSolver = true;
    SolverSettings solverSettings;
    Space* space = nullptr;
    Entity* involved[2] = {nullptr, nullptr};  // sorted by index for lock order (SolverUpdateable.cs:325-329)
    int involvedCount = 0;

    virtual ~SolverUpdateable() = default;
    // SolverUpdateable.cs:202-219: active while a connected member's island
    // is; islands exist for dynamic entities only.
    virtual void UpdateSolverActivity() {
        if (isActive) {
            for (int i = 0; i < involvedCount; i++)
                if (involved[i]->isDynamic && involved[i]->IsActive()) { isActiveInSolver = true; return; }
        }
        isActiveInSolver = false;
    }
    virtual void Update(float dt) = 0;
    virtual void ExclusiveUpdate() = 0;
    virtual float SolveIteration() = 0;

    void SetInvolved(Entity* a, Entity* b) {
        involvedCount = 0;
        if (a) involved[involvedCount++] = a;
        if (b && b != a) involved[involvedCount++] = b;
        if (involvedCount == 2 && involved[0]->index > involved[1]->index) std::swap(involved[0], involved[1]);
    }
    // SolverUpdateable.cs:151-173
    void EnterLock() {
        for (int i = 0; i < involvedCount; i++)
            if (involved[i]->isDynamic) involved[i]->locker.Enter();
    }
    void ExitLock() {
        for (int i = involvedCount - 1; i >= 0; i--)
            if (involved[i]->isDynamic) involved[i]->locker.Exit();
    }
};

struct Space {
    Settings s;
    std::vector<Entity> entities;
    std::vector<std::unique_ptr<SolverUpdateable>> updateables;  // joints, then manifolds
    std::vector<SolverUpdateable*> list;                          // the solver's list
    PermutationMapper mapper;
    int orderMode = ORACLE_ORDER_IDENTITY;
    std::atomic<long long> childSolves{0};
    bool countSolves = true;  // single-threaded runs only: a shared counter would serialize threads
    size_t jointCount = 0;
    std::vector<bepugpu_shape> shapes;  // one per entity, for GENERATED manifolds
    Entity world;  // TwoEntityConstraint.WorldEntity: kinematic, at the origin, identity orientation
    // DeactivationManager.simulationIslands (in list order) and deactivationIslandIndex;
    // empty: every island awake, no deactivation.
    std::vector<Island> islands;
    int deactivationIslandIndex = 0;
    std::vector<std::vector<SolverUpdateable*>> connectionsOf;  // per entity: the constraints touching it
};

// SolverGroup.cs:52-165
struct SolverGroup : SolverUpdateable {
    std::vector<SolverUpdateable*> children;  // the group's solverUpdateables list

    void UpdateSolverActivity() override {
        if (isActive) {
            isActiveInSolver = false;
            for (auto* c : children) {
                c->UpdateSolverActivity();
                isActiveInSolver |= c->isActiveInSolver;
            }
        } else {
            isActiveInSolver = false;
        }
    }
    static void UpdateUpdateable(SolverUpdateable* item, float dt) {
        item->solverSettings.currentIterations = 0;
        item->solverSettings.iterationsAtZeroImpulse = 0;
        if (item->isActiveInSolver) item->Update(dt);
    }
    static void ExclusiveUpdateUpdateable(SolverUpdateable* item) {
        if (item->isActiveInSolver) item->ExclusiveUpdate();
    }
    void SolveUpdateable(SolverUpdateable* item, int& activeConstraints) {
        if (item->isActiveInSolver) {
            SolverSettings& sub = item->solverSettings;
            sub.currentIterations++;
            if (sub.currentIterations <= space->s.iterationLimit &&
                sub.currentIterations <= sub.maximumIterationCount) {
                if (space->countSolves) space->childSolves.fetch_add(1, std::memory_order_relaxed);
                if (item->SolveIteration() < sub.minimumImpulse) {
                    sub.iterationsAtZeroImpulse++;
                    if (sub.iterationsAtZeroImpulse > sub.minimumIterationCount)
                        item->isActiveInSolver = false;
                    else
                        activeConstraints++;
                } else {
                    sub.iterationsAtZeroImpulse = 0;
                    activeConstraints++;
                }
            } else {
                item->isActiveInSolver = false;
            }
        }
    }
    void Update(float dt) override {
        for (auto* c : children) UpdateUpdateable(c, dt);
    }
    void ExclusiveUpdate() override {
        for (auto* c : children) ExclusiveUpdateUpdateable(c);
    }
    float SolveIteration() override {
        int activeConstraints = 0;
        for (auto* c : children) SolveUpdateable(c, activeConstraints);
        isActiveInSolver = activeConstraints > 0;
        return solverSettings.minimumImpulse + 1;
    }
};

// ---------------------------------------------------------------- contact manifold --
struct ConvexManifold;

struct Contact {
    Vec3 Position, Normal;
    float PenetrationDepth = 0;
    int Id = -1;
    Vec3 LocalOffsetA, LocalOffsetB;  // ContactSupplementData
    float BasePenetrationDepth = 0;
};

// ContactPenetrationConstraint.cs:114-321
struct PenetrationConstraint : SolverUpdateable {
    ConvexManifold* m = nullptr;
    Contact contact;
    float accumulatedImpulse = 0;
    float angularAX = 0, angularAY = 0, angularAZ = 0;
    float angularBX = 0, angularBY = 0, angularBZ = 0;
    float softness = 0, bias = 0;
    float linearAX = 0, linearAY = 0, linearAZ = 0;
    Entity *entityA = nullptr, *entityB = nullptr;
    bool entityADynamic = false, entityBDynamic = false;
    float velocityToImpulse = 0;
    Vec3 ra, rb;

    float RelativeVelocity() const {  // :88-105
        float lambda = 0;
        if (entityA)
            lambda = entityA->linearVelocity.X * linearAX + entityA->linearVelocity.Y * linearAY +
                     entityA->linearVelocity.Z * linearAZ + entityA->angularVelocity.X * angularAX +
                     entityA->angularVelocity.Y * angularAY + entityA->angularVelocity.Z * angularAZ;
        if (entityB)
            lambda += -entityB->linearVelocity.X * linearAX - entityB->linearVelocity.Y * linearAY -
                      entityB->linearVelocity.Z * linearAZ + entityB->angularVelocity.X * angularBX +
                      entityB->angularVelocity.Y * angularBY + entityB->angularVelocity.Z * angularBZ;
        return lambda;
    }
    void Update(float dt) override;
    void ExclusiveUpdate() override {  // :240-271
        Vec3 linear, angular;
        linear.X = accumulatedImpulse * linearAX;
        linear.Y = accumulatedImpulse * linearAY;
        linear.Z = accumulatedImpulse * linearAZ;
        if (entityADynamic) {
            angular.X = accumulatedImpulse * angularAX;
            angular.Y = accumulatedImpulse * angularAY;
            angular.Z = accumulatedImpulse * angularAZ;
            entityA->ApplyLinearImpulse(linear);
            entityA->ApplyAngularImpulse(angular);
        }
        if (entityBDynamic) {
            linear.X = -linear.X; linear.Y = -linear.Y; linear.Z = -linear.Z;
            angular.X = accumulatedImpulse * angularBX;
            angular.Y = accumulatedImpulse * angularBY;
            angular.Z = accumulatedImpulse * angularBZ;
            entityB->ApplyLinearImpulse(linear);
            entityB->ApplyAngularImpulse(angular);
        }
    }
    float SolveIteration() override {  // :278-321
        float lambda = (RelativeVelocity() - bias + softness * accumulatedImpulse) * velocityToImpulse;
        float previousAccumulatedImpulse = accumulatedImpulse;
        accumulatedImpulse = Max(0, accumulatedImpulse + lambda);
        lambda = accumulatedImpulse - previousAccumulatedImpulse;
        Vec3 linear, angular;
        linear.X = lambda * linearAX;
        linear.Y = lambda * linearAY;
        linear.Z = lambda * linearAZ;
        if (entityADynamic) {
            angular.X = lambda * angularAX;
            angular.Y = lambda * angularAY;
            angular.Z = lambda * angularAZ;
            entityA->ApplyLinearImpulse(linear);
            entityA->ApplyAngularImpulse(angular);
        }
        if (entityBDynamic) {
            linear.X = -linear.X; linear.Y = -linear.Y; linear.Z = -linear.Z;
            angular.X = lambda * angularBX;
            angular.Y = lambda * angularBY;
            angular.Z = lambda * angularBZ;
            entityB->ApplyLinearImpulse(linear);
            entityB->ApplyAngularImpulse(angular);
        }
        return std::fabs(lambda);
    }
};

// SlidingFrictionTwoAxis.cs:155-482
struct SlidingFriction : SolverUpdateable {
    ConvexManifold* m = nullptr;
    float accX = 0, accY = 0;  // accumulatedImpulse
    Mat2x3 angularA, angularB, linearA;
    int contactCount = 0;
    float friction = 0;
    Entity *entityA = nullptr, *entityB = nullptr;
    bool entityADynamic = false, entityBDynamic = false;
    Vec3 ra, rb;
    Mat2 velocityToImpulse;
    Vec3 manifoldCenter, relativeVelocity;

    void RelativeVelocity(float& lx, float& ly) const {  // :68-126
        float dvx = 0, dvy = 0, dvz = 0;
        if (entityA) {
            const Vec3& v = entityA->linearVelocity; const Vec3& w = entityA->angularVelocity;
            dvx = v.X + (w.Y * ra.Z) - (w.Z * ra.Y);
            dvy = v.Y + (w.Z * ra.X) - (w.X * ra.Z);
            dvz = v.Z + (w.X * ra.Y) - (w.Y * ra.X);
        }
        if (entityB) {
            const Vec3& v = entityB->linearVelocity; const Vec3& w = entityB->angularVelocity;
            dvx += -v.X - (w.Y * rb.Z) + (w.Z * rb.Y);
            dvy += -v.Y - (w.Z * rb.X) + (w.X * rb.Z);
            dvz += -v.Z - (w.X * rb.Y) + (w.Y * rb.X);
        }
        lx = dvx * linearA.M11 + dvy * linearA.M12 + dvz * linearA.M13;
        ly = dvx * linearA.M21 + dvy * linearA.M22 + dvz * linearA.M23;
    }
    float SolveIteration() override;
    void Update(float dt) override;
    void ExclusiveUpdate() override {  // :447-482
        Vec3 linear, angular;
        linear.X = accX * linearA.M11 + accY * linearA.M21;
        linear.Y = accX * linearA.M12 + accY * linearA.M22;
        linear.Z = accX * linearA.M13 + accY * linearA.M23;
        if (entityADynamic) {
            angular.X = accX * angularA.M11 + accY * angularA.M21;
            angular.Y = accX * angularA.M12 + accY * angularA.M22;
            angular.Z = accX * angularA.M13 + accY * angularA.M23;
            entityA->ApplyLinearImpulse(linear);
            entityA->ApplyAngularImpulse(angular);
        }
        if (entityBDynamic) {
            linear.X = -linear.X; linear.Y = -linear.Y; linear.Z = -linear.Z;
            angular.X = accX * angularB.M11 + accY * angularB.M21;
            angular.Y = accX * angularB.M12 + accY * angularB.M22;
            angular.Z = accX * angularB.M13 + accY * angularB.M23;
            entityB->ApplyLinearImpulse(linear);
            entityB->ApplyAngularImpulse(angular);
        }
    }
};

// TwistFrictionConstraint.cs:65-204
struct TwistFriction : SolverUpdateable {
    ConvexManifold* m = nullptr;
    float leverArms[4] = {0, 0, 0, 0};
    float accumulatedImpulse = 0;
    float angularX = 0, angularY = 0, angularZ = 0;
    int contactCount = 0;
    float friction = 0;
    Entity *entityA = nullptr, *entityB = nullptr;
    bool entityADynamic = false, entityBDynamic = false;
    float velocityToImpulse = 0;

    float RelativeVelocity() const {  // :48-58
        float lambda = 0;
        if (entityA)
            lambda = entityA->angularVelocity.X * angularX + entityA->angularVelocity.Y * angularY +
                     entityA->angularVelocity.Z * angularZ;
        if (entityB)
            lambda -= entityB->angularVelocity.X * angularX + entityB->angularVelocity.Y * angularY +
                      entityB->angularVelocity.Z * angularZ;
        return lambda;
    }
    float SolveIteration() override;
    void Update(float dt) override;
    void ExclusiveUpdate() override {  // :182-204
        Vec3 angular;
        angular.X = accumulatedImpulse * angularX;
        angular.Y = accumulatedImpulse * angularY;
        angular.Z = accumulatedImpulse * angularZ;
        if (entityADynamic) entityA->ApplyAngularImpulse(angular);
        if (entityBDynamic) {
            angular.X = -angular.X; angular.Y = -angular.Y; angular.Z = -angular.Z;
            entityB->ApplyAngularImpulse(angular);
        }
    }
};

// ContactFrictionConstraint.cs:10-299: one per contact of a nonconvex manifold.
struct ContactFriction : SolverUpdateable {
    ConvexManifold* m = nullptr;
    PenetrationConstraint* penetration = nullptr;
    float accumulatedImpulse = 0;
    float angularAX = 0, angularAY = 0, angularAZ = 0;
    float angularBX = 0, angularBY = 0, angularBZ = 0;
    float friction = 0;
    float linearAX = 0, linearAY = 0, linearAZ = 0;
    Entity *entityA = nullptr, *entityB = nullptr;
    bool entityAIsDynamic = false, entityBIsDynamic = false;
    float velocityToImpulse = 0;

    float RelativeVelocity() const {  // :85-97
        float velocity = 0;
        if (entityA)
            velocity += entityA->linearVelocity.X * linearAX + entityA->linearVelocity.Y * linearAY +
                        entityA->linearVelocity.Z * linearAZ + entityA->angularVelocity.X * angularAX +
                        entityA->angularVelocity.Y * angularAY + entityA->angularVelocity.Z * angularAZ;
        if (entityB)
            velocity += -entityB->linearVelocity.X * linearAX - entityB->linearVelocity.Y * linearAY -
                        entityB->linearVelocity.Z * linearAZ + entityB->angularVelocity.X * angularBX +
                        entityB->angularVelocity.Y * angularBY + entityB->angularVelocity.Z * angularBZ;
        return velocity;
    }
    float SolveIteration() override {  // :100-143
        float lambda = RelativeVelocity() * velocityToImpulse;
        float previousAccumulatedImpulse = accumulatedImpulse;
        float maxForce = friction * penetration->accumulatedImpulse;
        accumulatedImpulse = Clamp(accumulatedImpulse + lambda, -maxForce, maxForce);
        lambda = accumulatedImpulse - previousAccumulatedImpulse;
        Vec3 linear, angular;
        linear.X = lambda * linearAX;
        linear.Y = lambda * linearAY;
        linear.Z = lambda * linearAZ;
        if (entityAIsDynamic) {
            angular.X = lambda * angularAX;
            angular.Y = lambda * angularAY;
            angular.Z = lambda * angularAZ;
            entityA->ApplyLinearImpulse(linear);
            entityA->ApplyAngularImpulse(angular);
        }
        if (entityBIsDynamic) {
            linear.X = -linear.X; linear.Y = -linear.Y; linear.Z = -linear.Z;
            angular.X = lambda * angularBX;
            angular.Y = lambda * angularBY;
            angular.Z = lambda * angularBZ;
            entityB->ApplyLinearImpulse(linear);
            entityB->ApplyAngularImpulse(angular);
        }
        return std::fabs(lambda);
    }
    void Update(float dt) override;
    void ExclusiveUpdate() override {  // :258-289
        Vec3 linear, angular;
        linear.X = accumulatedImpulse * linearAX;
        linear.Y = accumulatedImpulse * linearAY;
        linear.Z = accumulatedImpulse * linearAZ;
        if (entityAIsDynamic) {
            angular.X = accumulatedImpulse * angularAX;
            angular.Y = accumulatedImpulse * angularAY;
            angular.Z = accumulatedImpulse * angularAZ;
            entityA->ApplyLinearImpulse(linear);
            entityA->ApplyAngularImpulse(angular);
        }
        if (entityBIsDynamic) {
            linear.X = -linear.X; linear.Y = -linear.Y; linear.Z = -linear.Z;
            angular.X = accumulatedImpulse * angularBX;
            angular.Y = accumulatedImpulse * angularBY;
            angular.Z = accumulatedImpulse * angularBZ;
            entityB->ApplyLinearImpulse(linear);
            entityB->ApplyAngularImpulse(angular);
        }
    }
};

// ConvexContactManifoldConstraint.cs:12-212 over ContactManifoldConstraint.cs:15-174,
// or, with nonConvex, NonConvexContactManifoldConstraint.cs:12-216: one
// ContactFriction per contact in place of the sliding and twist friction.
struct ConvexManifold : SolverGroup {
    Entity *entityA = nullptr, *entityB = nullptr;
    float kineticFriction = 0, staticFriction = 0, bounciness = 0;
    bool solverRule = true;
    PenetrationConstraint pool[4];
    std::vector<PenetrationConstraint*> penetrationConstraints;  // contact-add order
    // ContactManifold.contacts: the same contacts in the manifold's own list
    // order (FastRemoveAt moves the last entry into a removed one's place)
    std::vector<PenetrationConstraint*> contactList;
    bool generated = false;  // contacts come from the narrow phase each step
    SlidingFriction slidingFriction;
    TwistFriction twistFriction;
    bool nonConvex = false;
    ContactFriction fpool[4];
    std::vector<ContactFriction*> frictionConstraints;  // nonConvex: one per contact, in contact-add order
    int sourceIndex = 0;

    ConvexManifold() {
        // ConvexContactManifoldConstraint.cs:75-84: four penetration children,
        // then sliding, then twist, all initially inactive.  The contact
        // friction children (NonConvexContactManifoldConstraint.cs:64-74) stay
        // inactive unless the manifold is nonconvex.
        for (auto& p : pool) { p.isActive = false; p.m = this; children.push_back(&p); }
        slidingFriction.isActive = false; slidingFriction.m = this; children.push_back(&slidingFriction);
        twistFriction.isActive = false; twistFriction.m = this; children.push_back(&twistFriction);
        for (auto& f : fpool) { f.isActive = false; f.m = this; children.push_back(&f); }
    }
    // ContactManifoldConstraint.cs:128-145 with every entity awake
    void UpdateSolverActivity() override {
        if (isActive) {
            isActiveInSolver = solverRule && ((entityA && entityA->isDynamic && entityA->IsActive()) ||
                                              (entityB && entityB->isDynamic && entityB->IsActive()));
            for (auto* c : children) c->isActiveInSolver = c->isActive && isActiveInSolver;
        } else {
            isActiveInSolver = false;
        }
    }
    void Update(float dt) override {  // :171-177; NonConvexContactManifoldConstraint.cs:180-186
        for (auto* p : penetrationConstraints) UpdateUpdateable(p, dt);
        if (nonConvex) {
            for (auto* f : frictionConstraints) UpdateUpdateable(f, dt);
            return;
        }
        UpdateUpdateable(&slidingFriction, dt);
        UpdateUpdateable(&twistFriction, dt);
    }
    void ExclusiveUpdate() override {  // :186-192; NonConvexContactManifoldConstraint.cs:189-195
        for (auto* p : penetrationConstraints) ExclusiveUpdateUpdateable(p);
        if (nonConvex) {
            for (auto* f : frictionConstraints) ExclusiveUpdateUpdateable(f);
            return;
        }
        ExclusiveUpdateUpdateable(&slidingFriction);
        ExclusiveUpdateUpdateable(&twistFriction);
    }
    float SolveIteration() override {  // :199-212; NonConvexContactManifoldConstraint.cs:198-207
        int activeConstraints = 0;
        for (auto* p : penetrationConstraints) SolveUpdateable(p, activeConstraints);
        if (nonConvex) {
            for (auto* f : frictionConstraints) SolveUpdateable(f, activeConstraints);
        } else {
            SolveUpdateable(&slidingFriction, activeConstraints);
            SolveUpdateable(&twistFriction, activeConstraints);
        }
        isActiveInSolver = activeConstraints > 0;
        return solverSettings.minimumImpulse + 1;
    }
    // AddContact (:117-129): the first contact sets up sliding and twist.
    // Nonconvex (NonConvexContactManifoldConstraint.cs:115-126): a penetration
    // and a friction child per contact, the friction child Setup (linearA = 0).
    void AddContact(const Contact& c, float impulse, float frictionImpulse = 0, Vec3 frictionDirection = Vec3()) {
        PenetrationConstraint* p = nullptr;
        for (auto& q : pool)
            if (!q.isActive) { p = &q; break; }
        p->contact = c;
        p->isActive = true;
        p->entityA = entityA; p->entityB = entityB;
        p->accumulatedImpulse = impulse;
        penetrationConstraints.push_back(p);
        contactList.push_back(p);
        if (nonConvex) {
            ContactFriction* f = nullptr;
            for (auto& q : fpool)
                if (!q.isActive) { f = &q; break; }
            f->penetration = p;
            f->isActive = true;
            f->entityA = entityA; f->entityB = entityB;
            f->linearAX = frictionDirection.X; f->linearAY = frictionDirection.Y; f->linearAZ = frictionDirection.Z;
            f->accumulatedImpulse = frictionImpulse;
            frictionConstraints.push_back(f);
            return;
        }
        if (!twistFriction.isActive) {
            twistFriction.isActive = true;
            twistFriction.entityA = entityA; twistFriction.entityB = entityB;
            slidingFriction.isActive = true;
            slidingFriction.entityA = entityA; slidingFriction.entityB = entityB;
            slidingFriction.linearA = Mat2x3();
        }
    }
    // ContactManifold.Remove (ContactManifold.cs:51-57): the manifold's list
    // drops the contact by RawList.FastRemoveAt; the constraint's by RemoveAt.
    void RemoveListAt(int i) {
        PenetrationConstraint* p = contactList[i];
        contactList[i] = contactList.back();
        contactList.pop_back();
        for (int k = 0; k < (int)penetrationConstraints.size(); k++)
            if (penetrationConstraints[k] == p) { RemovePenetrationAt(k); return; }
    }
    void RemoveContactAt(int i) {
        PenetrationConstraint* p = penetrationConstraints[i];
        for (int k = 0; k < (int)contactList.size(); k++)
            if (contactList[k] == p) { RemoveListAt(k); return; }
    }
    // RemoveContact (:135-155): order-preserving removal (RawList.RemoveAt).
    void RemovePenetrationAt(int i) {
        PenetrationConstraint* p = penetrationConstraints[i];
        p->accumulatedImpulse = 0;
        p->isActive = false;
        p->entityA = p->entityB = nullptr;
        penetrationConstraints.erase(penetrationConstraints.begin() + i);
        // NonConvexContactManifoldConstraint.RemoveContact (:139-166): the
        // contact's friction child, found from the end, CleanUp and RemoveAt.
        for (int k = (int)frictionConstraints.size() - 1; k >= 0; k--) {
            ContactFriction* f = frictionConstraints[k];
            if (f->penetration == p) {
                f->accumulatedImpulse = 0;
                f->isActive = false;
                f->penetration = nullptr;
                f->entityA = f->entityB = nullptr;
                frictionConstraints.erase(frictionConstraints.begin() + k);
                break;
            }
        }
        if (penetrationConstraints.empty()) {
            twistFriction.accumulatedImpulse = 0; twistFriction.isActive = false;
            twistFriction.entityA = twistFriction.entityB = nullptr;
            slidingFriction.accX = slidingFriction.accY = 0; slidingFriction.isActive = false;
            slidingFriction.entityA = slidingFriction.entityB = nullptr;
        }
    }
};

void PenetrationConstraint::Update(float dt) {  // ContactPenetrationConstraint.cs:114-233
    const Settings& S = m->space->s;
    entityADynamic = entityA != nullptr && entityA->isDynamic;
    entityBDynamic = entityB != nullptr && entityB->isDynamic;
    linearAX = -contact.Normal.X;
    linearAY = -contact.Normal.Y;
    linearAZ = -contact.Normal.Z;
    if (entityA) {
        ra = Subtract(contact.Position, entityA->position);
        angularAX = (ra.Y * linearAZ) - (ra.Z * linearAY);
        angularAY = (ra.Z * linearAX) - (ra.X * linearAZ);
        angularAZ = (ra.X * linearAY) - (ra.Y * linearAX);
    }
    if (entityB) {
        rb = Subtract(contact.Position, entityB->position);
        angularBX = (linearAY * rb.Z) - (linearAZ * rb.Y);
        angularBY = (linearAZ * rb.X) - (linearAX * rb.Z);
        angularBZ = (linearAX * rb.Y) - (linearAY * rb.X);
    }
    float entryA, entryB, tX, tY, tZ;
    if (entityADynamic) {
        const Mat3& I = entityA->inertiaTensorInverse;
        tX = angularAX * I.M11 + angularAY * I.M21 + angularAZ * I.M31;
        tY = angularAX * I.M12 + angularAY * I.M22 + angularAZ * I.M32;
        tZ = angularAX * I.M13 + angularAY * I.M23 + angularAZ * I.M33;
        entryA = tX * angularAX + tY * angularAY + tZ * angularAZ + entityA->inverseMass;
    } else entryA = 0;
    if (entityBDynamic) {
        const Mat3& I = entityB->inertiaTensorInverse;
        tX = angularBX * I.M11 + angularBY * I.M21 + angularBZ * I.M31;
        tY = angularBX * I.M12 + angularBY * I.M22 + angularBZ * I.M32;
        tZ = angularBX * I.M13 + angularBY * I.M23 + angularBZ * I.M33;
        entryB = tX * angularBX + tY * angularBY + tZ * angularBZ + entityB->inverseMass;
    } else entryB = 0;
    float effectiveMassInverse = entryA + entryB;
    float updateRate = 1 / dt;
    softness = S.softness * effectiveMassInverse * updateRate;
    velocityToImpulse = -1 / (softness + effectiveMassInverse);
    if (contact.PenetrationDepth >= 0) {
        bias = Min(Max(0, contact.PenetrationDepth - S.allowedPenetration) * S.recoveryStiffness * updateRate,
                   S.maxRecoverySpeed);
        if (m->bounciness > 0) {
            float bounceVelocity = -RelativeVelocity();
            if (bounceVelocity > 0) {
                float lowThreshold = S.bounceThreshold * 0.3f;
                float velocityFraction =
                    Clamp((bounceVelocity - lowThreshold) / (S.bounceThreshold - lowThreshold + Epsilon), 0, 1);
                float bouncinessVelocity = velocityFraction * bounceVelocity * m->bounciness;
                bias = Max(bouncinessVelocity, bias);
            }
        }
    } else {
        bias = contact.PenetrationDepth * updateRate;
    }
}

void ContactFriction::Update(float dt) {  // ContactFrictionConstraint.cs:147-256
    (void)dt;
    entityAIsDynamic = entityA != nullptr && entityA->isDynamic;
    entityBIsDynamic = entityB != nullptr && entityB->isDynamic;
    Vec3 velocityA, velocityB;
    const Vec3 ra = penetration->ra, rb = penetration->rb;
    if (entityA) {
        velocityA = Cross(entityA->angularVelocity, ra);
        velocityA = Add(velocityA, entityA->linearVelocity);
    }
    if (entityB) {
        velocityB = Cross(entityB->angularVelocity, rb);
        velocityB = Add(velocityB, entityB->linearVelocity);
    }
    Vec3 relativeVelocity = Subtract(velocityA, velocityB);
    const Vec3 normal = penetration->contact.Normal;
    float normalVelocityScalar =
        normal.X * relativeVelocity.X + normal.Y * relativeVelocity.Y + normal.Z * relativeVelocity.Z;
    relativeVelocity.X -= normalVelocityScalar * normal.X;
    relativeVelocity.Y -= normalVelocityScalar * normal.Y;
    relativeVelocity.Z -= normalVelocityScalar * normal.Z;
    float length = LengthSquared(relativeVelocity);
    if (length > 1e-7f) {  // Toolbox.Epsilon
        length = (float)std::sqrt((double)length);
        linearAX = relativeVelocity.X / length;
        linearAY = relativeVelocity.Y / length;
        linearAZ = relativeVelocity.Z / length;
        friction = length > m->space->s.staticThreshold ? m->kineticFriction : m->staticFriction;
    } else {
        if (linearAX != 0 || linearAY != 0 || linearAZ != 0) {
            friction = m->staticFriction;
        } else {
            isActiveInSolver = false;
            return;
        }
    }
    angularAX = (ra.Y * linearAZ) - (ra.Z * linearAY);
    angularAY = (ra.Z * linearAX) - (ra.X * linearAZ);
    angularAZ = (ra.X * linearAY) - (ra.Y * linearAX);
    angularBX = (linearAY * rb.Z) - (linearAZ * rb.Y);
    angularBY = (linearAZ * rb.X) - (linearAX * rb.Z);
    angularBZ = (linearAX * rb.Y) - (linearAY * rb.X);
    float entryA, entryB, tX, tY, tZ;
    if (entityAIsDynamic) {
        const Mat3& I = entityA->inertiaTensorInverse;
        tX = angularAX * I.M11 + angularAY * I.M21 + angularAZ * I.M31;
        tY = angularAX * I.M12 + angularAY * I.M22 + angularAZ * I.M32;
        tZ = angularAX * I.M13 + angularAY * I.M23 + angularAZ * I.M33;
        entryA = tX * angularAX + tY * angularAY + tZ * angularAZ + entityA->inverseMass;
    } else entryA = 0;
    if (entityBIsDynamic) {
        const Mat3& I = entityB->inertiaTensorInverse;
        tX = angularBX * I.M11 + angularBY * I.M21 + angularBZ * I.M31;
        tY = angularBX * I.M12 + angularBY * I.M22 + angularBZ * I.M32;
        tZ = angularBX * I.M13 + angularBY * I.M23 + angularBZ * I.M33;
        entryB = tX * angularBX + tY * angularBY + tZ * angularBZ + entityB->inverseMass;
    } else entryB = 0;
    velocityToImpulse = -1 / (entryA + entryB);
}

float SlidingFriction::SolveIteration() {  // SlidingFrictionTwoAxis.cs:155-234
    float lx, ly;
    RelativeVelocity(lx, ly);
    float x = lx;
    lx = x * velocityToImpulse.M11 + ly * velocityToImpulse.M21;
    ly = x * velocityToImpulse.M12 + ly * velocityToImpulse.M22;
    float prevX = accX, prevY = accY;
    accX += lx;
    accY += ly;
    float length = accX * accX + accY * accY;  // Vector2.LengthSquared
    float maximumFrictionForce = 0;
    for (int i = 0; i < contactCount; i++) maximumFrictionForce += m->penetrationConstraints[i]->accumulatedImpulse;
    maximumFrictionForce *= friction;
    if (length > maximumFrictionForce * maximumFrictionForce) {
        length = maximumFrictionForce / (float)std::sqrt((double)length);
        accX *= length;
        accY *= length;
    }
    lx = accX - prevX;
    ly = accY - prevY;
    Vec3 linear, angular;
    linear.X = lx * linearA.M11 + ly * linearA.M21;
    linear.Y = lx * linearA.M12 + ly * linearA.M22;
    linear.Z = lx * linearA.M13 + ly * linearA.M23;
    if (entityADynamic) {
        angular.X = lx * angularA.M11 + ly * angularA.M21;
        angular.Y = lx * angularA.M12 + ly * angularA.M22;
        angular.Z = lx * angularA.M13 + ly * angularA.M23;
        entityA->ApplyLinearImpulse(linear);
        entityA->ApplyAngularImpulse(angular);
    }
    if (entityBDynamic) {
        linear.X = -linear.X; linear.Y = -linear.Y; linear.Z = -linear.Z;
        angular.X = lx * angularB.M11 + ly * angularB.M21;
        angular.Y = lx * angularB.M12 + ly * angularB.M22;
        angular.Z = lx * angularB.M13 + ly * angularB.M23;
        entityB->ApplyLinearImpulse(linear);
        entityB->ApplyAngularImpulse(angular);
    }
    return std::fabs(lx) + std::fabs(ly);
}

void SlidingFriction::Update(float dt) {  // SlidingFrictionTwoAxis.cs:242-440
    (void)dt;
    const Settings& S = m->space->s;
    entityADynamic = entityA != nullptr && entityA->isDynamic;
    entityBDynamic = entityB != nullptr && entityB->isDynamic;
    contactCount = (int)m->penetrationConstraints.size();
    auto P = [&](int i) -> const Vec3& { return m->penetrationConstraints[i]->contact.Position; };
    switch (contactCount) {
        case 1: manifoldCenter = P(0); break;
        case 2:
            manifoldCenter = Add(P(0), P(1));
            manifoldCenter.X *= .5f; manifoldCenter.Y *= .5f; manifoldCenter.Z *= .5f;
            break;
        case 3:
            manifoldCenter = Add(P(0), P(1));
            manifoldCenter = Add(P(2), manifoldCenter);
            manifoldCenter.X *= .333333333f; manifoldCenter.Y *= .333333333f; manifoldCenter.Z *= .333333333f;
            break;
        case 4:
            manifoldCenter = Add(P(0), P(1));
            manifoldCenter = Add(P(2), manifoldCenter);
            manifoldCenter = Add(P(3), manifoldCenter);
            manifoldCenter.X *= .25f; manifoldCenter.Y *= .25f; manifoldCenter.Z *= .25f;
            break;
        default: {
            float nv = -3.40282347e+38f;
            manifoldCenter = {nv, nv, nv};
        }
    }
    Vec3 velocityA, velocityB;
    if (entityA) {
        ra = Subtract(manifoldCenter, entityA->position);
        velocityA = Cross(entityA->angularVelocity, ra);
        velocityA = Add(velocityA, entityA->linearVelocity);
    }
    if (entityB) {
        rb = Subtract(manifoldCenter, entityB->position);
        velocityB = Cross(entityB->angularVelocity, rb);
        velocityB = Add(velocityB, entityB->linearVelocity);
    }
    relativeVelocity = Subtract(velocityA, velocityB);
    Vec3 normal = m->penetrationConstraints[0]->contact.Normal;
    float normalVelocityScalar = normal.X * relativeVelocity.X + normal.Y * relativeVelocity.Y + normal.Z * relativeVelocity.Z;
    relativeVelocity.X -= normalVelocityScalar * normal.X;
    relativeVelocity.Y -= normalVelocityScalar * normal.Y;
    relativeVelocity.Z -= normalVelocityScalar * normal.Z;
    float length = LengthSquared(relativeVelocity);
    if (length > Epsilon) {
        length = (float)std::sqrt((double)length);
        float inverseLength = 1 / length;
        linearA.M11 = relativeVelocity.X * inverseLength;
        linearA.M12 = relativeVelocity.Y * inverseLength;
        linearA.M13 = relativeVelocity.Z * inverseLength;
        friction = length > S.staticThreshold ? m->kineticFriction : m->staticFriction;
    } else {
        friction = m->staticFriction;
        if (!(linearA.M11 != 0 || linearA.M12 != 0 || linearA.M13 != 0)) {
            Vec3 axis1 = Cross(normal, Vec3{1, 0, 0});  // Toolbox.RightVector
            length = LengthSquared(axis1);
            if (length > Epsilon) {
                length = (float)std::sqrt((double)length);
                float inverseLength = 1 / length;
                linearA.M11 = axis1.X * inverseLength;
                linearA.M12 = axis1.Y * inverseLength;
                linearA.M13 = axis1.Z * inverseLength;
            } else {
                axis1 = Cross(normal, Vec3{0, 1, 0});  // Toolbox.UpVector
                Normalize(axis1);
                linearA.M11 = axis1.X; linearA.M12 = axis1.Y; linearA.M13 = axis1.Z;
            }
        }
    }
    linearA.M21 = (linearA.M12 * normal.Z) - (linearA.M13 * normal.Y);
    linearA.M22 = (linearA.M13 * normal.X) - (linearA.M11 * normal.Z);
    linearA.M23 = (linearA.M11 * normal.Y) - (linearA.M12 * normal.X);
    if (entityA) {
        angularA.M11 = (ra.Y * linearA.M13) - (ra.Z * linearA.M12);
        angularA.M12 = (ra.Z * linearA.M11) - (ra.X * linearA.M13);
        angularA.M13 = (ra.X * linearA.M12) - (ra.Y * linearA.M11);
        angularA.M21 = (ra.Y * linearA.M23) - (ra.Z * linearA.M22);
        angularA.M22 = (ra.Z * linearA.M21) - (ra.X * linearA.M23);
        angularA.M23 = (ra.X * linearA.M22) - (ra.Y * linearA.M21);
    }
    if (entityB) {
        angularB.M11 = (linearA.M12 * rb.Z) - (linearA.M13 * rb.Y);
        angularB.M12 = (linearA.M13 * rb.X) - (linearA.M11 * rb.Z);
        angularB.M13 = (linearA.M11 * rb.Y) - (linearA.M12 * rb.X);
        angularB.M21 = (linearA.M22 * rb.Z) - (linearA.M23 * rb.Y);
        angularB.M22 = (linearA.M23 * rb.X) - (linearA.M21 * rb.Z);
        angularB.M23 = (linearA.M21 * rb.Y) - (linearA.M22 * rb.X);
    }
    Mat2 entryA, entryB;
    if (entityADynamic) {
        Mat2x3 transform = Multiply(angularA, entityA->inertiaTensorInverse);
        Mat3x2 transpose = Transpose(angularA);
        entryA = Multiply(transform, transpose);
        entryA.M11 += entityA->inverseMass;
        entryA.M22 += entityA->inverseMass;
    }
    if (entityBDynamic) {
        Mat2x3 transform = Multiply(angularB, entityB->inertiaTensorInverse);
        Mat3x2 transpose = Transpose(angularB);
        entryB = Multiply(transform, transpose);
        entryB.M11 += entityB->inverseMass;
        entryB.M22 += entityB->inverseMass;
    }
    velocityToImpulse.M11 = -entryA.M11 - entryB.M11;
    velocityToImpulse.M12 = -entryA.M12 - entryB.M12;
    velocityToImpulse.M21 = -entryA.M21 - entryB.M21;
    velocityToImpulse.M22 = -entryA.M22 - entryB.M22;
    velocityToImpulse = Invert(velocityToImpulse);
}

float TwistFriction::SolveIteration() {  // TwistFrictionConstraint.cs:65-107
    float lambda = RelativeVelocity();
    lambda *= velocityToImpulse;
    float previousAccumulatedImpulse = accumulatedImpulse;
    float maximumFrictionForce = 0;
    for (int i = 0; i < contactCount; i++)
        maximumFrictionForce += leverArms[i] * m->penetrationConstraints[i]->accumulatedImpulse;
    maximumFrictionForce *= friction;
    accumulatedImpulse = Clamp(accumulatedImpulse + lambda, -maximumFrictionForce, maximumFrictionForce);
    lambda = accumulatedImpulse - previousAccumulatedImpulse;
    Vec3 angular;
    angular.X = lambda * angularX;
    angular.Y = lambda * angularY;
    angular.Z = lambda * angularZ;
    if (entityADynamic) entityA->ApplyAngularImpulse(angular);
    if (entityBDynamic) {
        angular.X = -angular.X; angular.Y = -angular.Y; angular.Z = -angular.Z;
        entityB->ApplyAngularImpulse(angular);
    }
    return std::fabs(lambda);
}

void TwistFriction::Update(float dt) {  // TwistFrictionConstraint.cs:114-175
    (void)dt;
    const Settings& S = m->space->s;
    entityADynamic = entityA != nullptr && entityA->isDynamic;
    entityBDynamic = entityB != nullptr && entityB->isDynamic;
    Vec3 normal = m->penetrationConstraints[0]->contact.Normal;
    angularX = normal.X; angularY = normal.Y; angularZ = normal.Z;
    float entryA, entryB, tX, tY, tZ;
    if (entityADynamic) {
        const Mat3& I = entityA->inertiaTensorInverse;
        tX = angularX * I.M11 + angularY * I.M21 + angularZ * I.M31;
        tY = angularX * I.M12 + angularY * I.M22 + angularZ * I.M32;
        tZ = angularX * I.M13 + angularY * I.M23 + angularZ * I.M33;
        entryA = tX * angularX + tY * angularY + tZ * angularZ + entityA->inverseMass;
    } else entryA = 0;
    if (entityBDynamic) {
        const Mat3& I = entityB->inertiaTensorInverse;
        tX = angularX * I.M11 + angularY * I.M21 + angularZ * I.M31;
        tY = angularX * I.M12 + angularY * I.M22 + angularZ * I.M32;
        tZ = angularX * I.M13 + angularY * I.M23 + angularZ * I.M33;
        entryB = tX * angularX + tY * angularY + tZ * angularZ + entityB->inverseMass;
    } else entryB = 0;
    velocityToImpulse = -1 / (entryA + entryB);
    float relativeAngularVelocity = RelativeVelocity();
    const Vec3& rs = m->slidingFriction.relativeVelocity;
    friction = std::fabs(relativeAngularVelocity) > S.staticThreshold ||
                       std::fabs(rs.X) + std::fabs(rs.Y) + std::fabs(rs.Z) > S.staticThreshold
                   ? m->kineticFriction
                   : m->staticFriction;
    friction *= S.twistFactor;
    contactCount = (int)m->penetrationConstraints.size();
    for (int i = 0; i < contactCount; i++) {
        Vec3 contactOffset = Subtract(m->penetrationConstraints[i]->contact.Position, m->slidingFriction.manifoldCenter);
        leverArms[i] = Length(contactOffset);
    }
}

// ContactRefresher.cs:18-69 followed by the order-preserving removal of the
// queued contacts (GeneralConvexContactManifold.Update, RemoveQueuedContacts).
static void RefreshManifold(ConvexManifold& m, const Settings& S) {
    if (m.penetrationConstraints.empty()) return;
    Vec3 posA, posB; Quat qA, qB;
    if (m.entityA) { posA = m.entityA->position; qA = m.entityA->orientation; }
    if (m.entityB) { posB = m.entityB->position; qB = m.entityB->orientation; }
    std::vector<int> toRemove;
    for (int k = 0; k < (int)m.penetrationConstraints.size(); k++) {
        Contact& c = m.penetrationConstraints[k]->contact;
        Vec3 newPosA = Add(QTransform(c.LocalOffsetA, qA), posA);  // RigidTransform.Transform
        Vec3 newPosB = Add(QTransform(c.LocalOffsetB, qB), posB);
        Vec3 ab = Subtract(newPosB, newPosA);
        float dot = Dot(ab, c.Normal);
        Vec3 temp = Multiply(c.Normal, dot);
        temp = Subtract(ab, temp);
        dot = LengthSquared(temp);
        if (dot > S.invalidationLengthSquared) {
            toRemove.push_back(k);
        } else {
            dot = Dot(ab, c.Normal);
            c.PenetrationDepth = c.BasePenetrationDepth - dot;
            if (c.PenetrationDepth < -S.maximumContactDistance) {
                toRemove.push_back(k);
            } else {
                Vec3 newPos = Add(newPosB, newPosA);
                newPos = Multiply(newPos, .5f);
                c.Position = newPos;
            }
        }
    }
    for (int i = (int)toRemove.size() - 1; i >= 0; i--) m.RemoveContactAt(toRemove[i]);
}

#include "bepu_oracle_joints.inc"
#include "bepu_oracle_collide.inc"

// BoxContactManifold.Update, managed branch (BoxContactManifold.cs:122-196):
// match the new contacts to the kept ones by id (the last match in the new
// list wins and is consumed), remove the unmatched kept ones from the highest
// list index down, then add what is left of the new list in its order.
static void UpdateBoxBoxManifold(Space& sp, ConvexManifold& m) {
    const bepugpu_shape &sa = sp.shapes[m.entityA->index], &sb = sp.shapes[m.entityB->index];
    BoxDims a{sa.size[0], sa.size[1], sa.size[2]}, b{sb.size[0], sb.size[1], sb.size[2]};
    float distance;
    Vec3 axis;
    TinyContacts manifold;
    if (AreBoxesColliding(a, b, m.entityA->position, m.entityA->orientation, m.entityB->position,
                          m.entityB->orientation, distance, axis, manifold)) {
        axis = Neg(axis);
        std::vector<int> toRemove;
        for (int i = 0; i < (int)m.contactList.size(); i++) {
            Contact& c = m.contactList[i]->contact;
            bool found = false;
            for (int j = manifold.Count - 1; j >= 0; j--) {
                if (c.Id == manifold.e[j].Id) {
                    found = true;
                    c.Position = manifold.e[j].Position;
                    c.PenetrationDepth = -manifold.e[j].Depth;
                    c.Normal = axis;
                    manifold.RemoveAt(j);
                    break;
                }
            }
            if (!found) toRemove.push_back(i);
        }
        for (int i = (int)toRemove.size() - 1; i >= 0; i--) m.RemoveListAt(toRemove[i]);
        for (int i = 0; i < manifold.Count; i++) {
            Contact c;
            c.Position = manifold.e[i].Position;
            c.PenetrationDepth = -manifold.e[i].Depth;
            c.Normal = axis;
            c.Id = manifold.e[i].Id;
            c.LocalOffsetA = Vec3(); c.LocalOffsetB = Vec3(); c.BasePenetrationDepth = 0;
            m.AddContact(c, 0.f);
        }
    } else {
        for (int i = (int)m.contactList.size() - 1; i >= 0; i--) m.RemoveListAt(i);
    }
}

// SphereContactManifold / BoxSphereContactManifold.Update (:55-83): one
// contact; a first contact is taken only at non-negative depth.
static void UpdateOneContactManifold(ConvexManifold& m, bool colliding, const ContactDataO& cd) {
    bool previouslyColliding = !m.penetrationConstraints.empty();
    if (colliding) {
        if (!previouslyColliding && cd.PenetrationDepth >= 0) {
            Contact c;
            c.Position = cd.Position;
            c.Normal = cd.Normal;
            c.PenetrationDepth = cd.PenetrationDepth;
            c.Id = 0;
            c.LocalOffsetA = Vec3(); c.LocalOffsetB = Vec3(); c.BasePenetrationDepth = 0;
            m.AddContact(c, 0.f);
        } else if (previouslyColliding) {
            Contact& c = m.penetrationConstraints[0]->contact;
            c.Normal = cd.Normal;
            c.PenetrationDepth = cd.PenetrationDepth;
            c.Position = cd.Position;
        }
    } else if (previouslyColliding) {
        m.RemoveListAt(0);
    }
}

static void CollideManifold(Space& sp, ConvexManifold& m) {
    const bepugpu_shape &sa = sp.shapes[m.entityA->index], &sb = sp.shapes[m.entityB->index];
    if (sa.type == BEPUGPU_SHAPE_BOX && sb.type == BEPUGPU_SHAPE_BOX) {
        UpdateBoxBoxManifold(sp, m);
    } else if (sa.type == BEPUGPU_SHAPE_SPHERE && sb.type == BEPUGPU_SHAPE_SPHERE) {
        ContactDataO cd;
        bool hit = AreSpheresColliding(sa.size[0], sb.size[0], m.entityA->position, m.entityB->position,
                                       sp.s.maximumContactDistance, cd);
        UpdateOneContactManifold(m, hit, cd);
    } else {  // box (A) and sphere (B)
        ContactDataO cd;
        BoxDims box{sa.size[0], sa.size[1], sa.size[2]};
        bool hit = AreBoxSphereColliding(box, sb.size[0], m.entityA->position, m.entityA->orientation,
                                         m.entityB->position, sp.s.maximumContactDistance, cd);
        UpdateOneContactManifold(m, hit, cd);
    }
}

// ---------------------------------------------------------------- Solver --
// Solver.cs:265-275
static void UnsafePrestep(SolverUpdateable* u, float dt) {
    u->UpdateSolverActivity();
    if (u->isActiveInSolver) {
        u->solverSettings.currentIterations = 0;
        u->solverSettings.iterationsAtZeroImpulse = 0;
        u->Update(dt);
    }
}
// Solver.cs:285-314
static void UnsafeSolveIteration(Space& sp, SolverUpdateable* u) {
    if (u->isActiveInSolver) {
        SolverSettings& ss = u->solverSettings;
        ss.currentIterations++;
        if (ss.currentIterations <= sp.s.iterationLimit && ss.currentIterations <= ss.maximumIterationCount) {
            if (u->SolveIteration() < ss.minimumImpulse) {
                ss.iterationsAtZeroImpulse++;
                if (ss.iterationsAtZeroImpulse > ss.minimumIterationCount) u->isActiveInSolver = false;
            } else {
                ss.iterationsAtZeroImpulse = 0;
            }
        } else {
            u->isActiveInSolver = false;
        }
    }
}

static long long MappedIndex(Space& sp, long long i, int n) {
    return sp.orderMode == ORACLE_ORDER_PERMUTED ? sp.mapper.Map(i, n) : (i % n);
}

// Solver.cs:239-263
static void SolverUpdateSingleThreaded(Space& sp, float dt) {
    int n = (int)sp.list.size();
    for (int i = 0; i < n; i++) UnsafePrestep(sp.list[i], dt);
    for (int i = 0; i < n; i++)
        if (sp.list[i]->isActiveInSolver) sp.list[i]->ExclusiveUpdate();
    long long total = (long long)sp.s.iterationLimit * n;
    sp.mapper.SetIndex(sp.mapper.permutationIndex + 1);
    if (n == 0) return;
    for (long long i = 0; i < total; i++) UnsafeSolveIteration(sp, sp.list[MappedIndex(sp, i, n)]);
}

// ParallelLooper.ForLoop (BEPUutilities/Threading/ParallelLooper.cs:113-144):
// chunks of iterationsPerSteal claimed with an atomic counter.
template <class F>
static void ForLoop(int threads, long long begin, long long end, F&& body) {
    long long count = end - begin;
    if (count <= 0) return;
    long long tasksPerThread = std::max<long long>(3, count / 80);
    long long subdivisions = (long long)threads * tasksPerThread;
    long long perSteal = std::max<long long>(1, count / subdivisions);
    std::atomic<long long> job{0};
    auto worker = [&]() {
        for (;;) {
            long long j = job.fetch_add(1) + 1;
            long long e = j * perSteal, b = e - perSteal;
            if (b >= count) break;
            for (long long i = b; i < e && i < count; i++) body(begin + i);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
}

// Solver.cs:150-237
static void SolverUpdateMultithreaded(Space& sp, float dt, int threads) {
    int n = (int)sp.list.size();
    ForLoop(threads, 0, n, [&](long long i) {
        auto* u = sp.list[i];
        u->UpdateSolverActivity();
        if (u->isActiveInSolver) {
            u->solverSettings.currentIterations = 0;
            u->solverSettings.iterationsAtZeroImpulse = 0;
            u->Update(dt);
        }
    });
    ForLoop(threads, 0, n, [&](long long i) {
        auto* u = sp.list[i];
        if (u->isActiveInSolver) {
            u->EnterLock();
            u->ExclusiveUpdate();
            u->ExitLock();
        }
    });
    sp.mapper.SetIndex(sp.mapper.permutationIndex + 1);
    if (n == 0) return;
    long long total = (long long)sp.s.iterationLimit * n;
    ForLoop(threads, 0, total, [&](long long i) {
        auto* u = sp.list[MappedIndex(sp, i, n)];
        SolverSettings& ss = u->solverSettings;
        if (u->isActiveInSolver) {
            int incremented = -1;
            u->EnterLock();
            if (u->isActiveInSolver) {
                if (u->SolveIteration() < ss.minimumImpulse) {
                    ss.iterationsAtZeroImpulse++;
                    if (ss.iterationsAtZeroImpulse > ss.minimumIterationCount) u->isActiveInSolver = false;
                } else {
                    ss.iterationsAtZeroImpulse = 0;
                }
                incremented = ss.currentIterations++;
            }
            u->ExitLock();
            if (incremented > sp.s.iterationLimit || incremented > ss.maximumIterationCount)
                u->isActiveInSolver = false;
        }
    });
}

// DeactivationManager.DeactivateObjects (DeactivationManager.cs:310-336) over
// islands that all have members, with SimulationIsland.TryToDeactivate
// (SimulationIsland.cs:94-118).
static void DeactivateObjects(Space& sp) {
    int numberOfEntitiesDeactivated = 0, numberOfIslandsChecked = 0;
    const int originalIslandCount = (int)sp.islands.size();
    while (numberOfEntitiesDeactivated < sp.s.maximumDeactivationAttemptsPerFrame && !sp.islands.empty() &&
           numberOfIslandsChecked < originalIslandCount) {
        sp.deactivationIslandIndex = (sp.deactivationIslandIndex + 1) % (int)sp.islands.size();
        Island& island = sp.islands[sp.deactivationIslandIndex];
        if (island.allowDeactivation) {
            if (island.isActive && island.deactivationCandidateCount() == island.memberCount) island.isActive = false;
        } else {
            island.allowDeactivation = true;
        }
        numberOfEntitiesDeactivated += island.memberCount;
        ++numberOfIslandsChecked;
    }
}

// DeactivationManager.UpdateSingleThreaded (DeactivationManager.cs:216-224)
// without the split flush: the candidacy loop in member order, an active
// kinematic member waking its connections' islands as it goes, then
// DeactivateObjects.  A manifold is a connection while it has contacts (the
// pair handler keeps its constraint in the solver only then).
static void DeactivationUpdate(Space& sp, float dt) {
    for (auto& e : sp.entities) {
        if (!e.UpdateDeactivationCandidacy(dt, sp.s)) continue;
        for (SolverUpdateable* c : sp.connectionsOf[(size_t)e.index]) {
            if (auto* m = dynamic_cast<ConvexManifold*>(c))
                if (m->penetrationConstraints.empty()) continue;
            for (int k = 0; k < c->involvedCount; k++)
                if (Island* isl = c->involved[k]->island) {
                    isl->isActive = true;
                    isl->allowDeactivation = false;
                }
        }
    }
    for (auto& isl : sp.islands) isl.candidates = 0;
    for (auto& e : sp.entities)
        if (e.island && e.isDeactivationCandidate) e.island->candidates++;
    DeactivateObjects(sp);
}

// An entry of the narrow phase is active (NarrowPhase.cs:300-332 updates a pair
// while one of its entries is); a missing entity is a static entry, inactive.
static bool EntryActive(const Entity* e) { return e && e->IsActive(); }

static void StepOnce(Space& sp, float dt, uint32_t flags, int threads) {
    // DeactivationManager.Update comes first (Space.cs:502); the narrow phase
    // and the refresher read poses only, so they run before the force update
    // here (the reference runs them after it, Space.cs:504-513).
    const bool islands = !sp.islands.empty();
    if (flags & BEPUGPU_STEP_DEACTIVATION) {  // DeactivationManager.cs:206-224, the candidacy loop
        if (islands) {
            DeactivationUpdate(sp, dt);  // member order matters: sequential
        } else {
            auto body = [&](long long i) { sp.entities[i].UpdateDeactivationCandidacy(dt, sp.s); };
            if (threads > 1) ForLoop(threads, 0, (long long)sp.entities.size(), body);
            else for (size_t i = 0; i < sp.entities.size(); i++) body((long long)i);
        }
    }
    auto pairActive = [&](const ConvexManifold* m) {
        return !islands || EntryActive(m->entityA) || EntryActive(m->entityB);
    };
    if (flags & BEPUGPU_STEP_COLLIDE) {  // pairs are independent: the narrow phase's pair loop
        auto pair = [&](long long i) {
            auto* m = static_cast<ConvexManifold*>(sp.updateables[sp.jointCount + (size_t)i].get());
            if (m->generated && pairActive(m)) CollideManifold(sp, *m);
        };
        const long long n = (long long)(sp.updateables.size() - sp.jointCount);
        if (threads > 1) ForLoop(threads, 0, n, pair);
        else for (long long i = 0; i < n; i++) pair(i);
    }
    if (flags & BEPUGPU_STEP_REFRESH_CONTACTS) {
        for (size_t i = sp.jointCount; i < sp.updateables.size(); i++) {
            auto* m = static_cast<ConvexManifold*>(sp.updateables[i].get());
            if (!m->generated && pairActive(m)) RefreshManifold(*m, sp.s);
        }
    }
    if (flags & BEPUGPU_STEP_FORCES) {  // ForceUpdater.cs:73-92
        Vec3 gravityDt = Multiply(sp.s.gravity, dt);
        auto body = [&](long long i) {
            Entity& e = sp.entities[i];
            if (e.isDynamic && e.IsActive()) e.UpdateForForces(dt, gravityDt, sp.s);
        };
        if (threads > 1) ForLoop(threads, 0, (long long)sp.entities.size(), body);
        else for (size_t i = 0; i < sp.entities.size(); i++) body((long long)i);
    }
    if (flags & BEPUGPU_STEP_SOLVE) {
        sp.childSolves = 0;
        sp.countSolves = threads <= 1;
        if (threads > 1) SolverUpdateMultithreaded(sp, dt, threads);
        else SolverUpdateSingleThreaded(sp, dt);
    }
    if (flags & BEPUGPU_STEP_POSITIONS) {  // ContinuousPositionUpdater.cs:49-74,134-154, Discrete bodies
        // Active entities only (:71): kinematic ones while their time flag is <= 0
        // (SimulationIslandMember.cs:225-248).
        auto body = [&](long long i) {
            Entity& e = sp.entities[i];
            if (e.IsActive()) e.PreUpdatePosition(dt);
        };
        if (threads > 1) ForLoop(threads, 0, (long long)sp.entities.size(), body);
        else for (size_t i = 0; i < sp.entities.size(); i++) body((long long)i);
    }
}

static Vec3 V3(const float* p) { return {p[0], p[1], p[2]}; }
static void P3(float* p, const Vec3& v) { p[0] = v.X; p[1] = v.Y; p[2] = v.Z; }

}  // namespace oracle

using namespace oracle;

struct oracle_space {
    Space sp;
};

extern "C" {

oracle_space* oracle_create(const bepugpu_settings* st, const bepugpu_body* bodies, int32_t nb,
                            const bepugpu_manifold* manifolds, int32_t nm, const bepugpu_joint* joints,
                            int32_t nj) {
    auto* o = new oracle_space();
    Space& sp = o->sp;
    Settings& S = sp.s;
    S.gravity = V3(st->gravity);
    S.iterationLimit = st->iteration_limit;
    S.minimumImpulse = st->minimum_impulse;
    S.minimumIterationCount = st->minimum_iteration_count;
    S.maximumIterationCount = st->maximum_iteration_count;
    S.softness = st->softness;
    S.recoveryStiffness = st->penetration_recovery_stiffness;
    S.maxRecoverySpeed = st->maximum_penetration_recovery_speed;
    S.staticThreshold = st->static_friction_velocity_threshold;
    S.twistFactor = st->twist_friction_factor;
    S.bounceThreshold = st->bounciness_velocity_threshold;
    S.allowedPenetration = st->allowed_penetration;
    S.invalidationLengthSquared = st->contact_invalidation_length_squared;
    S.maximumContactDistance = st->maximum_contact_distance;
    S.useStabilization = st->use_stabilization != 0;
    S.velocityLowerLimit = std::max(0.f, st->velocity_lower_limit);  // DeactivationManager.cs:36-37
    S.velocityLowerLimitSquared = S.velocityLowerLimit * S.velocityLowerLimit;
    S.lowVelocityTimeMinimum = st->low_velocity_time_minimum;
    S.maximumDeactivationAttemptsPerFrame = st->maximum_deactivation_attempts_per_frame;

    sp.entities = std::vector<Entity>(nb);
    for (int i = 0; i < nb; i++) {
        Entity& e = sp.entities[i];
        const bepugpu_body& b = bodies[i];
        e.index = i;
        e.position = V3(b.position);
        e.orientation = {b.orientation[0], b.orientation[1], b.orientation[2], b.orientation[3]};
        e.orientationMatrix = CreateFromQuaternion(e.orientation);
        e.linearVelocity = V3(b.linear_velocity);
        e.angularVelocity = V3(b.angular_velocity);
        e.isDynamic = b.is_dynamic != 0;
        e.inverseMass = e.isDynamic ? b.inverse_mass : 0.f;
        const float* L = b.local_inverse_inertia;
        e.localInertiaTensorInverse = {L[0], L[1], L[2], L[3], L[4], L[5], L[6], L[7], L[8]};
        if (!e.isDynamic) e.localInertiaTensorInverse = Mat3();
        Mat3 mult = MultiplyTransposed(e.orientationMatrix, e.localInertiaTensorInverse);
        e.inertiaTensorInverse = Multiply(mult, e.orientationMatrix);
        e.linearDamping = b.linear_damping;
        e.angularDamping = b.angular_damping;
        e.previousVelocity = b.previous_velocity;
        e.velocityTimeBelowLimit = b.velocity_time_below_limit;
        e.isAlwaysActive = (b.activity & BEPUGPU_BODY_ALWAYS_ACTIVE) != 0;
        e.allowStabilization = (b.activity & BEPUGPU_BODY_NO_STABILIZATION) == 0;
        e.isSlowing = (b.activity & BEPUGPU_BODY_SLOWING) != 0;
        e.isDeactivationCandidate = (b.activity & BEPUGPU_BODY_DEACTIVATION_CANDIDATE) != 0;
    }
    sp.world.index = -1;
    sp.world.orientationMatrix = CreateFromQuaternion(sp.world.orientation);
    auto ent = [&](int idx) -> Entity* { return idx >= 0 && idx < nb ? &sp.entities[idx] : nullptr; };
    for (int j = 0; j < nj; j++) {
        SolverUpdateable* u;
        if (joints[j].flags & BEPUGPU_JOINT_GROUP_CONTINUATION) {
            int h = j;
            while (h > 0 && (joints[h].flags & BEPUGPU_JOINT_GROUP_CONTINUATION)) h--;
            u = h < j ? CreateContinuation(sp, joints[j], ent(joints[j].body_a), ent(joints[j].body_b),
                                           sp.updateables[h].get())
                      : nullptr;
        } else {
            u = CreateJoint(sp, joints[j], ent(joints[j].body_a), ent(joints[j].body_b));
        }
        if (!u) { delete o; return nullptr; }
        sp.updateables.emplace_back(u);
    }
    sp.jointCount = sp.updateables.size();
    for (int i = 0; i < nm; i++) {
        const bepugpu_manifold& mr = manifolds[i];
        auto* m = new ConvexManifold();
        m->space = &sp;
        m->sourceIndex = i;
        for (auto* c : m->children) c->space = &sp;
        m->entityA = ent(mr.body_a);
        m->entityB = ent(mr.body_b);
        m->SetInvolved(m->entityA, m->entityB);
        m->isActive = (mr.flags & BEPUGPU_MANIFOLD_ACTIVE) != 0;
        m->generated = (mr.flags & BEPUGPU_MANIFOLD_GENERATED) != 0;
        m->nonConvex = (mr.flags & BEPUGPU_MANIFOLD_NONCONVEX) != 0;
        m->solverRule = (mr.flags & BEPUGPU_MANIFOLD_SOLVER_RULE) != 0;
        m->kineticFriction = mr.kinetic_friction;
        m->staticFriction = mr.static_friction;
        m->bounciness = mr.bounciness;
        m->solverSettings.minimumImpulse = S.minimumImpulse;
        m->solverSettings.minimumIterationCount = S.minimumIterationCount;
        m->solverSettings.maximumIterationCount = S.maximumIterationCount;
        for (auto* c : m->children) {
            c->solverSettings.minimumImpulse = S.minimumImpulse;
            c->solverSettings.minimumIterationCount = S.minimumIterationCount;
            c->solverSettings.maximumIterationCount = S.maximumIterationCount;
        }
        int cc = std::max(0, std::min(4, (int)mr.contact_count));
        for (int k = 0; k < cc; k++) {
            const bepugpu_contact& cr = mr.contacts[k];
            Contact c;
            c.Position = V3(cr.position);
            c.Normal = V3(cr.normal);
            c.PenetrationDepth = cr.penetration_depth;
            c.Id = cr.id;
            c.LocalOffsetA = V3(cr.local_offset_a);
            c.LocalOffsetB = V3(cr.local_offset_b);
            c.BasePenetrationDepth = cr.base_penetration_depth;
            m->AddContact(c, cr.penetration_impulse, cr.friction_impulse, V3(cr.friction_direction));
        }
        if (m->generated && cc > 0) {  // the list order carried in contact_order
            std::vector<PenetrationConstraint*> list(cc);
            const uint32_t code = (uint32_t)mr.contact_order ^ 0xE4u;
            for (int k = 0; k < cc; k++) list[k] = m->penetrationConstraints[(code >> (2 * k)) & 3];
            m->contactList = list;
        }
        // The sliding axis is kept whatever the count (CleanUp leaves linearA;
        // Setup clears it when a first contact comes); impulses only with contacts.
        m->slidingFriction.linearA.M11 = mr.sliding_axis[0];
        m->slidingFriction.linearA.M12 = mr.sliding_axis[1];
        m->slidingFriction.linearA.M13 = mr.sliding_axis[2];
        if (cc > 0) {
            m->slidingFriction.accX = mr.sliding_impulse[0];
            m->slidingFriction.accY = mr.sliding_impulse[1];
            m->twistFriction.accumulatedImpulse = mr.twist_impulse;
        }
        sp.updateables.emplace_back(m);
    }
    for (auto& u : sp.updateables) sp.list.push_back(u.get());
    sp.mapper.SetIndex(0);
    return o;
}

void oracle_destroy(oracle_space* s) { delete s; }

int32_t oracle_set_list_order(oracle_space* s, const int32_t* order, int32_t count) {
    Space& sp = s->sp;
    if (count != (int32_t)sp.updateables.size()) return -1;
    std::vector<char> seen(count, 0);
    std::vector<SolverUpdateable*> list(count);
    for (int i = 0; i < count; i++) {
        int k = order[i];
        if (k < 0 || k >= count || seen[k]) return -1;
        seen[k] = 1;
        list[i] = sp.updateables[k].get();
    }
    sp.list.swap(list);
    return 0;
}

void oracle_set_order_mode(oracle_space* s, int32_t mode, int64_t permutation_index) {
    s->sp.orderMode = mode;
    s->sp.mapper.SetIndex(permutation_index);
}

int32_t oracle_step(oracle_space* s, float dt, uint32_t flags, int32_t steps) {
    for (int i = 0; i < steps; i++) StepOnce(s->sp, dt, flags, 1);
    return 0;
}

int32_t oracle_step_multithreaded(oracle_space* s, float dt, uint32_t flags, int32_t steps, int32_t threads) {
    if (threads < 1) threads = 1;
    for (int i = 0; i < steps; i++) StepOnce(s->sp, dt, flags, threads);
    return 0;
}

int64_t oracle_last_child_solves(oracle_space* s) { return s->sp.childSolves.load(); }

// The island list as bepugpu_set_islands takes it: island_of[i] per body (-1
// for kinematic bodies), flags per island.  count 0 clears the islands.
// Returns -1 when a dynamic body has no island, an island has no member or a
// constraint's dynamic bodies lie in two islands.
int32_t oracle_set_islands(oracle_space* s, const int32_t* island_of, const uint32_t* flags, int32_t count,
                           int32_t deactivation_index) {
    Space& sp = s->sp;
    for (auto& e : sp.entities) e.island = nullptr;
    sp.islands.clear();
    sp.connectionsOf.clear();
    if (count <= 0) return 0;
    std::vector<Island> islands((size_t)count);
    for (int k = 0; k < count; k++) {
        islands[k].isActive = (flags[k] & BEPUGPU_ISLAND_ACTIVE) != 0;
        islands[k].allowDeactivation = (flags[k] & BEPUGPU_ISLAND_ALLOW_DEACTIVATION) != 0;
    }
    const int nb = (int)sp.entities.size();
    for (int i = 0; i < nb; i++) {
        const int k = island_of[i];
        if (!sp.entities[i].isDynamic) {
            if (k != -1) return -1;
            continue;
        }
        if (k < 0 || k >= count) return -1;
        islands[k].memberCount++;
    }
    for (auto& isl : islands)
        if (isl.memberCount == 0) return -1;
    sp.connectionsOf.assign((size_t)nb, {});
    for (auto& u : sp.updateables) {
        int shared = -1;
        for (int k = 0; k < u->involvedCount; k++) {
            Entity* e = u->involved[k];
            if (e->index < 0) continue;  // the world entity
            sp.connectionsOf[(size_t)e->index].push_back(u.get());
            if (!e->isDynamic) continue;
            if (shared >= 0 && island_of[e->index] != shared) return -1;
            shared = island_of[e->index];
        }
    }
    sp.islands = std::move(islands);
    for (int i = 0; i < nb; i++)
        if (sp.entities[i].isDynamic) sp.entities[i].island = &sp.islands[(size_t)island_of[i]];
    sp.deactivationIslandIndex = deactivation_index;
    return 0;
}

int32_t oracle_get_islands(oracle_space* s, uint32_t* flags, int32_t count, int32_t* deactivation_index) {
    Space& sp = s->sp;
    if (count != (int32_t)sp.islands.size()) return -1;
    for (int k = 0; k < count; k++)
        flags[k] = (sp.islands[k].isActive ? BEPUGPU_ISLAND_ACTIVE : 0u) |
                   (sp.islands[k].allowDeactivation ? BEPUGPU_ISLAND_ALLOW_DEACTIVATION : 0u);
    if (deactivation_index) *deactivation_index = sp.deactivationIslandIndex;
    return 0;
}

void oracle_get_bodies(oracle_space* s, bepugpu_body* out) {
    Space& sp = s->sp;
    for (size_t i = 0; i < sp.entities.size(); i++) {
        const Entity& e = sp.entities[i];
        bepugpu_body& b = out[i];
        P3(b.position, e.position);
        b.orientation[0] = e.orientation.X; b.orientation[1] = e.orientation.Y;
        b.orientation[2] = e.orientation.Z; b.orientation[3] = e.orientation.W;
        P3(b.linear_velocity, e.linearVelocity);
        P3(b.angular_velocity, e.angularVelocity);
        b.previous_velocity = e.previousVelocity;
        b.velocity_time_below_limit = e.velocityTimeBelowLimit;
        b.activity = (e.isAlwaysActive ? BEPUGPU_BODY_ALWAYS_ACTIVE : 0u) |
                     (e.allowStabilization ? 0u : BEPUGPU_BODY_NO_STABILIZATION) |
                     (e.isSlowing ? BEPUGPU_BODY_SLOWING : 0u) |
                     (e.isDeactivationCandidate ? BEPUGPU_BODY_DEACTIVATION_CANDIDATE : 0u);
    }
}

void oracle_get_constraints(oracle_space* s, bepugpu_manifold* manifolds, bepugpu_joint* joints) {
    Space& sp = s->sp;
    for (size_t j = 0; j < sp.jointCount; j++)
        if (joints) ReadJoint(sp.updateables[j].get(), joints[j]);
    if (!manifolds) return;
    for (size_t i = sp.jointCount; i < sp.updateables.size(); i++) {
        auto* m = static_cast<ConvexManifold*>(sp.updateables[i].get());
        bepugpu_manifold& mr = manifolds[m->sourceIndex];
        int cc = (int)m->penetrationConstraints.size();
        mr.contact_count = cc;
        for (int k = 0; k < cc; k++) {
            const PenetrationConstraint* p = m->penetrationConstraints[k];
            bepugpu_contact& cr = mr.contacts[k];
            P3(cr.position, p->contact.Position);
            P3(cr.normal, p->contact.Normal);
            cr.penetration_depth = p->contact.PenetrationDepth;
            cr.id = p->contact.Id;
            P3(cr.local_offset_a, p->contact.LocalOffsetA);
            P3(cr.local_offset_b, p->contact.LocalOffsetB);
            cr.base_penetration_depth = p->contact.BasePenetrationDepth;
            cr.penetration_impulse = p->accumulatedImpulse;
            cr.friction_impulse = 0;
            cr.friction_direction[0] = cr.friction_direction[1] = cr.friction_direction[2] = 0;
            if (m->nonConvex) {
                const ContactFriction* f = m->frictionConstraints[k];
                cr.friction_impulse = f->accumulatedImpulse;
                cr.friction_direction[0] = f->linearAX;
                cr.friction_direction[1] = f->linearAY;
                cr.friction_direction[2] = f->linearAZ;
            }
        }
        for (int k = cc; k < 4; k++) std::memset(&mr.contacts[k], 0, sizeof(bepugpu_contact));
        mr.sliding_impulse[0] = m->slidingFriction.accX;
        mr.sliding_impulse[1] = m->slidingFriction.accY;
        mr.sliding_axis[0] = m->slidingFriction.linearA.M11;
        mr.sliding_axis[1] = m->slidingFriction.linearA.M12;
        mr.sliding_axis[2] = m->slidingFriction.linearA.M13;
        mr.twist_impulse = m->twistFriction.accumulatedImpulse;
        uint32_t code = 0;
        if (m->generated) {
            for (int k = 0; k < 4; k++) {
                uint32_t at = (uint32_t)k;
                if (k < cc)
                    for (int q = 0; q < cc; q++)
                        if (m->penetrationConstraints[q] == m->contactList[k]) at = (uint32_t)q;
                code |= at << (2 * k);
            }
            code ^= 0xE4u;
        }
        mr.contact_order = (int32_t)code;
    }
}

int32_t oracle_set_shapes(oracle_space* s, const bepugpu_shape* shapes, int32_t count) {
    if (count != (int32_t)s->sp.entities.size()) return -1;
    s->sp.shapes.assign(shapes, shapes + count);
    return 0;
}

int64_t oracle_permutation_map(int64_t permutation_index, int64_t index, int32_t set_size) {
    PermutationMapper pm;
    pm.SetIndex(permutation_index);
    return pm.Map(index, set_size);
}

int32_t oracle_prime_count(void) { return kPrimeCount; }

// PermutationTestDemo.cs:82-127: for `iterations` permutation indices from 0,
// GetMappedIndex over [0, set_size) must be a permutation.  Returns the first
// permutation index that is not one, or -1; *distinct receives how many
// different permutations appeared.
int64_t oracle_permutation_check(int64_t iterations, int32_t set_size, int64_t* distinct) {
    PermutationMapper pm;
    std::vector<int32_t> seen((size_t)set_size, -1);
    std::vector<std::vector<int32_t>> perms;
    std::vector<int32_t> cur((size_t)set_size);
    for (int64_t k = 0; k < iterations; k++) {
        pm.SetIndex(k);
        for (int32_t i = 0; i < set_size; i++) {
            const int64_t m = pm.Map(i, set_size);
            if (m < 0 || m >= set_size || seen[(size_t)m] == (int32_t)(k & 0x7fffffff)) return k;
            seen[(size_t)m] = (int32_t)(k & 0x7fffffff);
            cur[(size_t)i] = (int32_t)m;
        }
        if (distinct) perms.push_back(cur);
    }
    if (distinct) {
        std::sort(perms.begin(), perms.end());
        *distinct = (int64_t)(std::unique(perms.begin(), perms.end()) - perms.begin());
    }
    return -1;
}

// Restatement of the library's colouring (deterministic greedy in list order,
// conflicts only through dynamic bodies; colour-sorted order is stable).  A
// GROUP_CONTINUATION record is solved inside its group's visit: it takes the
// colour of the record before it and claims nothing.
int32_t oracle_colour(const bepugpu_body* bodies, int32_t nb, const bepugpu_manifold* manifolds, int32_t nm,
                      const bepugpu_joint* joints, int32_t nj, int32_t* colour_out, int32_t* order_out) {
    int n = nj + nm;
    std::vector<std::vector<int>> used(nb);  // colours taken at each dynamic body
    int colours = 0;
    for (int u = 0; u < n; u++) {
        if (u > 0 && u < nj && (joints[u].flags & BEPUGPU_JOINT_GROUP_CONTINUATION)) {
            colour_out[u] = colour_out[u - 1];
            continue;
        }
        int a = u < nj ? joints[u].body_a : manifolds[u - nj].body_a;
        int b = u < nj ? joints[u].body_b : manifolds[u - nj].body_b;
        int ends[2] = {a, b};
        std::vector<int> taken;
        for (int e : ends)
            if (e >= 0 && e < nb && bodies[e].is_dynamic)
                taken.insert(taken.end(), used[e].begin(), used[e].end());
        std::sort(taken.begin(), taken.end());
        int c = 0;
        for (int t : taken) {
            if (t == c) c++;
            else if (t > c) break;
        }
        colour_out[u] = c;
        colours = std::max(colours, c + 1);
        for (int e : ends)
            if (e >= 0 && e < nb && bodies[e].is_dynamic) used[e].push_back(c);
    }
    int k = 0;
    for (int c = 0; c < colours; c++)
        for (int u = 0; u < n; u++)
            if (colour_out[u] == c) order_out[k++] = u;
    return colours;
}

}  // extern "C"
