// Host side of the two-body joints: record checks, upload into the scene's
// joint slots (colour order) and download of the accumulated impulses.
//
// The constants a joint's Update takes from System.Math in double -- the sine
// and cosine of RevoluteLimit's plane angles (Matrix3x3.CreateFromAxisAngle,
// Matrix3x3.cs:1392-1393, called at RevoluteLimit.cs:293-296) -- depend only on
// the record, so they are computed here once, with the host's libm, in the
// reference's expression: (float)Math.Sin((double)angle) and
// 1 - (float)Math.Cos((double)angle).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "joints_device.cuh"

namespace bepugpu {

namespace {

constexpr float kHostPi = 3.14159274f, kHostTwoPi = 6.28318548f, kHostPiOver2 = 1.57079637f;  // MathHelper.cs:13-33

// RevoluteLimit.GetDistanceFromMinimum (RevoluteLimit.cs:622-646); TwistLimit's
// (TwistLimit.cs:341-357) is the same function.
float DistanceFromMinimum(float minimumAngle, float angle) {
    if (minimumAngle > 0) {
        if (angle >= minimumAngle) return angle - minimumAngle;
        if (angle > 0) return kHostTwoPi - minimumAngle + angle;
        return kHostTwoPi - minimumAngle + angle;
    }
    if (angle < minimumAngle) return kHostTwoPi - minimumAngle + angle;
    return angle - minimumAngle;
}

uint32_t ChildrenOf(int32_t type) {
    switch (type) {
        case BEPUGPU_JOINT_BALL_SOCKET: return kJChildBall;
        case BEPUGPU_JOINT_REVOLUTE_ANGULAR: return kJChildAngular;
        case BEPUGPU_JOINT_SWING_LIMIT:
        case BEPUGPU_JOINT_REVOLUTE_LIMIT: return kJChildLimit;
        case BEPUGPU_JOINT_REVOLUTE: return kJChildBall | kJChildAngular | kJChildLimit;
        case BEPUGPU_JOINT_NO_ROTATION: return kJChildAngular;
        case BEPUGPU_JOINT_WELD: return kJChildBall | kJChildAngular;
        case BEPUGPU_JOINT_DISTANCE:
        case BEPUGPU_JOINT_DISTANCE_LIMIT:
        case BEPUGPU_JOINT_POINT_ON_PLANE:
        case BEPUGPU_JOINT_PLANE_SLIDER: return kJChildBall;
        case BEPUGPU_JOINT_TWIST: return kJChildAngular;
        case BEPUGPU_JOINT_POINT_ON_LINE: return kJChildBall;
        case BEPUGPU_JOINT_PRISMATIC:
        case BEPUGPU_JOINT_LINE_SLIDER: return kJChildBall | kJChildAngular | kJChildLimit;
        case BEPUGPU_JOINT_UNIVERSAL: return kJChildBall | kJChildAngular;
        case BEPUGPU_JOINT_TWIST_LIMIT:
        case BEPUGPU_JOINT_LINEAR_AXIS_LIMIT:
        case BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT: return kJChildLimit;
        case BEPUGPU_JOINT_SWIVEL_HINGE_ANGULAR: return kJChildAngular;
        case BEPUGPU_JOINT_SWIVEL_HINGE: return kJChildBall | kJChildAngular;
        case BEPUGPU_JOINT_REVOLUTE_MOTOR:
        case BEPUGPU_JOINT_TWIST_MOTOR:
        case BEPUGPU_JOINT_LINEAR_AXIS_MOTOR:
        case BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED:
        case BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED:
        case BEPUGPU_JOINT_ANGULAR_MOTOR:
        case BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR:
        case BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR: return kJChildLimit;
        default: return 0;
    }
}

float4 F4(const float* v, float w) { return make_float4(v[0], v[1], v[2], w); }

// The children a group record may be continued with (BEPUGPU_JOINT_GROUP_CONTINUATION).
bool ContinuationAllowed(int32_t group, int32_t child) {
    switch (group) {
        case BEPUGPU_JOINT_REVOLUTE: return child == BEPUGPU_JOINT_REVOLUTE_MOTOR;
        case BEPUGPU_JOINT_PRISMATIC:
        case BEPUGPU_JOINT_LINE_SLIDER: return child == BEPUGPU_JOINT_LINEAR_AXIS_MOTOR;
        case BEPUGPU_JOINT_UNIVERSAL: return child == BEPUGPU_JOINT_TWIST_LIMIT || child == BEPUGPU_JOINT_TWIST_MOTOR;
        case BEPUGPU_JOINT_SWIVEL_HINGE:
            return child == BEPUGPU_JOINT_REVOLUTE_LIMIT || child == BEPUGPU_JOINT_REVOLUTE_MOTOR ||
                   child == BEPUGPU_JOINT_TWIST_LIMIT || child == BEPUGPU_JOINT_TWIST_MOTOR;
        case BEPUGPU_JOINT_PLANE_SLIDER:
            return child == BEPUGPU_JOINT_LINEAR_AXIS_LIMIT || child == BEPUGPU_JOINT_LINEAR_AXIS_MOTOR;
        default: return false;
    }
}

}  // namespace

bepugpu_status CheckJointRecords(Context* ctx, const bepugpu_joint* joints, uint32_t nj, int32_t bodies) {
    for (uint32_t u = 0; u < nj; u++) {
        const bepugpu_joint& r = joints[u];
        if (!ChildrenOf(r.type)) {
            ctx->SetError("joint %u has unknown type %d", u, r.type);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (r.body_a < -1 || r.body_a >= bodies || r.body_b < -1 || r.body_b >= bodies) {
            ctx->SetError("joint %u references a body outside [-1, %d)", u, bodies);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (r.body_a == r.body_b && r.body_a >= 0) {
            ctx->SetError("joint %u connects body %d to itself", u, r.body_a);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        // SpringSettings.ComputeErrorReductionAndSoftness throws on this (SpringSettings.cs:104-105)
        if (r.spring_stiffness == 0 && r.spring_damping == 0) {
            ctx->SetError("joint %u: constraints cannot have both 0 stiffness and 0 damping", u);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        // DistanceJoint.Distance, DistanceLimit.MinimumLength / MaximumLength setters keep these
        if (r.type == BEPUGPU_JOINT_DISTANCE && !(r.limit_min >= 0)) {
            ctx->SetError("joint %u: distance %g must be non-negative", u, r.limit_min);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if ((r.type == BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED || r.type == BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED ||
             r.type == BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR || r.type == BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR) &&
            r.body_b != -1) {
            ctx->SetError("joint %u: a single-entity constraint acts on body_a alone (body_b must be -1)", u);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (r.type == BEPUGPU_JOINT_DISTANCE_LIMIT && !(r.limit_min >= 0 && r.limit_min <= r.limit_max)) {
            ctx->SetError("joint %u: lengths need 0 <= minimum <= maximum", u);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (r.flags & BEPUGPU_JOINT_GROUP_CONTINUATION) {
            uint32_t g = u, children = 0;
            while (g > 0 && (joints[g].flags & BEPUGPU_JOINT_GROUP_CONTINUATION)) {
                g--;
                children++;
            }
            const bepugpu_joint& head = joints[g];
            if (head.flags & BEPUGPU_JOINT_GROUP_CONTINUATION || !ContinuationAllowed(head.type, r.type)) {
                ctx->SetError("joint %u: a GROUP_CONTINUATION record of type %d does not follow a group that takes it",
                              u, r.type);
                return BEPUGPU_INVALID_ARGUMENT;
            }
            if (children > 4) {
                ctx->SetError("joint %u: a group takes at most four continuation records", u);
                return BEPUGPU_INVALID_ARGUMENT;
            }
            if (r.body_a != head.body_a || r.body_b != head.body_b) {
                ctx->SetError("joint %u: a GROUP_CONTINUATION record connects its group's bodies", u);
                return BEPUGPU_INVALID_ARGUMENT;
            }
        }
    }
    return BEPUGPU_OK;
}

// Records in slot order into the input lanes (kJLA .. kJTRIG), the impulse
// lanes (kJACC0, kJACC1), heads and a cleared state.
bepugpu_status UploadJoints(Context* ctx, Scene* s, const bepugpu_joint* joints, uint32_t nj) {
    s->j.count = (int)nj;
    s->addedJointTypes = false;
    for (uint32_t u = 0; u < nj; u++) s->addedJointTypes |= joints[u].type > BEPUGPU_JOINT_REVOLUTE;
    if (!nj) return BEPUGPU_OK;
    constexpr int kIn = kJointLanes - kJLA;
    std::vector<float4> lanes((size_t)kIn * nj), acc(2 * (size_t)nj);
    std::vector<int4> head(nj);
    auto at = [&](int k, int slot) -> float4& {
        return k >= kJLA ? lanes[(size_t)(k - kJLA) * nj + slot] : acc[(size_t)(k - kJACC0) * nj + slot];
    };
    for (uint32_t u = 0; u < nj; u++) {
        const bepugpu_joint& r = joints[u];
        const int slot = s->hostJointSlotOf[u];
        const uint32_t present = ChildrenOf(r.type);
        uint32_t childIsActive = present;
        const bool groupLimit = r.type == BEPUGPU_JOINT_REVOLUTE || r.type == BEPUGPU_JOINT_PRISMATIC ||
                                r.type == BEPUGPU_JOINT_LINE_SLIDER;
        if (groupLimit && !(r.flags & BEPUGPU_JOINT_LIMIT_ACTIVE)) childIsActive &= ~kJChildLimit;
        // a continuation is active when it and its group are; the group's
        // visit solves it right after the slot before it (same colour, next slot)
        const bool continuation = (r.flags & BEPUGPU_JOINT_GROUP_CONTINUATION) != 0;
        bool isActive = (r.flags & BEPUGPU_JOINT_ACTIVE) != 0;
        if (continuation) {
            uint32_t g = u;
            while (g > 0 && (joints[g].flags & BEPUGPU_JOINT_GROUP_CONTINUATION)) g--;
            isActive = isActive && (joints[g].flags & BEPUGPU_JOINT_ACTIVE);
        }
        const bool hasNext = u + 1 < nj && (joints[u + 1].flags & BEPUGPU_JOINT_GROUP_CONTINUATION);
        if (hasNext && s->hostJointSlotOf[u + 1] != slot + 1) {
            ctx->SetError("joint %u: its continuation record did not get the next slot", u);
            return BEPUGPU_INVALID_OPERATION;
        }
        uint32_t z = (uint32_t)r.type | (present << kJPresentShift) | (childIsActive << kJChildActiveShift) |
                     (isActive ? kJGroupIsActive : 0u) | (continuation ? kJHeadContinuation : 0u) |
                     (hasNext ? kJHeadHasNext : 0u);
        head[slot] = make_int4(r.body_a, r.body_b, (int)z, (int)u);
        // Joint.MaxCorrectiveVelocity setter (Joint.cs:23-36)
        float maxCorr = std::max(0.f, r.max_corrective_velocity);
        float maxCorrSq = maxCorr >= FLT_MAX ? FLT_MAX : maxCorr * maxCorr;
        float minAngle = r.limit_min, maxAngle = r.limit_max;
        float span = DistanceFromMinimum(minAngle, maxAngle);
        float aMin = minAngle + kHostPiOver2, aMax = maxAngle - kHostPiOver2;
        float sinMin = (float)std::sin((double)aMin), omcMin = 1 - (float)std::cos((double)aMin);
        float sinMax = (float)std::sin((double)aMax), omcMax = 1 - (float)std::cos((double)aMax);
        at(kJLA, slot) = F4(r.anchor_a, r.spring_stiffness);
        at(kJLB, slot) = F4(r.anchor_b, r.spring_damping);
        at(kJAXA, slot) = F4(r.axis_a, maxCorr);
        at(kJAXB, slot) = F4(r.axis_b, r.margin);
        at(kJC1, slot) = F4(r.constrained_1, r.bounciness);
        at(kJC2, slot) = F4(r.constrained_2, r.bounce_velocity_threshold);
        at(kJBP, slot) = F4(r.basis_primary, span);
        at(kJBX, slot) = F4(r.basis_x, r.type == BEPUGPU_JOINT_SWING_LIMIT ? r.limit_min : 0.f);
        at(kJTA, slot) = F4(r.test_axis, maxCorrSq);
        at(kJTRIG, slot) = make_float4(sinMin, omcMin, sinMax, omcMax);
        if (r.type == BEPUGPU_JOINT_NO_ROTATION || r.type == BEPUGPU_JOINT_WELD ||
            r.type == BEPUGPU_JOINT_PRISMATIC) {
            // the initial orientations' conjugates (NoRotationJoint.cs:48-63)
            const float* qa = r.orientation_a;
            const float* qb = r.orientation_b;
            at(kJC1, slot) = make_float4(-qa[0], -qa[1], -qa[2], qa[3]);
            at(kJC2, slot) = make_float4(-qb[0], -qb[1], -qb[2], qb[3]);
        }
        if (r.type == BEPUGPU_JOINT_DISTANCE || r.type == BEPUGPU_JOINT_DISTANCE_LIMIT) {
            at(kJAXA, slot) = make_float4(r.limit_min, r.limit_max, 0.f, maxCorr);
            at(kJBP, slot) = make_float4(0.f, 0.f, 0.f, 0.f);  // the limit's last jLinearA
        }
        if (r.type == BEPUGPU_JOINT_TWIST_LIMIT) {
            // MinimumAngle / MaximumAngle setters (TwistLimit.cs:50-75): the maximum's
            // setter wraps the minimum a second time, which changes nothing.
            float minimumAngle = std::fmod(r.limit_min, kHostTwoPi);
            if (minimumAngle > kHostPi) minimumAngle -= kHostTwoPi;
            if (minimumAngle <= -kHostPi) minimumAngle += kHostTwoPi;
            const float maximumAngle = std::fmod(r.limit_max, kHostTwoPi);
            at(kJBX, slot) = F4(r.basis_x, 0.f);
            at(kJTRIG, slot) = make_float4(minimumAngle, DistanceFromMinimum(minimumAngle, maximumAngle), 0.f, 0.f);
        }
        if (r.type == BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT) {
            // MaximumAngleX / Y setters (EllipseSwingLimit.cs:57-68): MathHelper.Clamp to [BigEpsilon, Pi]
            auto clamp = [](float v) { return v < 1e-5f ? 1e-5f : (v > kHostPi ? kHostPi : v); };
            at(kJTRIG, slot) = make_float4(clamp(r.limit_min), clamp(r.limit_max), 0.f, 0.f);
        }
        if (r.type == BEPUGPU_JOINT_ANGULAR_MOTOR || r.type == BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR ||
            r.type == BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR) {
            // MotorSettings3D / ServoSettingsOrientation through their setters (MotorSettings.cs)
            const float softness = r.margin < 0 ? 0.f : r.margin;
            const float base = r.bounciness < 0 ? 0.f : r.bounciness;
            const float maxForce = r.bounce_velocity_threshold >= 0 ? r.bounce_velocity_threshold : 0.f;
            at(kJTRIG, slot) = make_float4(softness, base, maxForce, maxCorrSq);
            at(kJTA, slot) = make_float4(r.orientation_a[0], r.orientation_a[1], r.orientation_a[2],
                                         r.orientation_a[3]);
            at(kJAXB, slot) = F4(r.axis_b, (r.flags & BEPUGPU_JOINT_SERVO) ? 1.f : 0.f);
        }
        if (r.type == BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED || r.type == BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED) {
            // MaximumSpeed, MaximumForce and Softness setters (MaximumLinearVelocityConstraint.cs:32-59)
            const float speed = 0 > r.limit_min ? 0.f : r.limit_min;
            const float force = r.limit_max >= 0 ? r.limit_max : 0.f;
            at(kJTRIG, slot) = make_float4(speed, force, std::max(0.f, r.margin), 0.f);
        }
        if (r.type >= BEPUGPU_JOINT_REVOLUTE_MOTOR && r.type <= BEPUGPU_JOINT_LINEAR_AXIS_MOTOR) {
            // MotorSettings1D through its setters (MotorSettings.cs): the angular motors' goal
            // wrapped by MathHelper.WrapAngle (MathHelper.cs:35-49), as GetDistanceFromGoal does
            float goal = r.limit_min;
            if (r.type != BEPUGPU_JOINT_LINEAR_AXIS_MOTOR) {
                goal = (float)std::remainder((double)goal, (double)kHostTwoPi);
                if (goal < -kHostPi) goal += kHostTwoPi;
                else if (goal >= kHostPi) goal -= kHostTwoPi;
            }
            const float softness = r.margin < 0 ? 0.f : r.margin;
            const float base = r.bounciness < 0 ? 0.f : r.bounciness;
            const float maxForce = r.bounce_velocity_threshold >= 0 ? r.bounce_velocity_threshold : 0.f;
            at(kJTRIG, slot) = make_float4(goal, r.limit_max, softness, base);
            at(kJBX, slot) = F4(r.basis_x, maxForce);
            at(kJAXB, slot) = F4(r.axis_b, (r.flags & BEPUGPU_JOINT_SERVO) ? 1.f : 0.f);
        }
        if (r.type == BEPUGPU_JOINT_LINEAR_AXIS_LIMIT || r.type == BEPUGPU_JOINT_PRISMATIC ||
            r.type == BEPUGPU_JOINT_LINE_SLIDER)
            // a prismatic joint's kJC1 / kJC2 hold orientations: the limit's bounce settings go here
            at(kJTRIG, slot) = make_float4(r.limit_min, r.limit_max, r.bounciness, r.bounce_velocity_threshold);
        // impulses: ball xyz | angular x, angular y | limit x | limit y | twist limit error
        float ball[3] = {0, 0, 0}, ang[2] = {0, 0}, lim[2] = {0, 0}, last = 0;
        switch (r.type) {
            case BEPUGPU_JOINT_BALL_SOCKET: std::memcpy(ball, r.impulse, 12); break;
            case BEPUGPU_JOINT_REVOLUTE_ANGULAR: std::memcpy(ang, r.impulse, 8); break;
            case BEPUGPU_JOINT_SWING_LIMIT: lim[0] = r.impulse[0]; break;
            case BEPUGPU_JOINT_REVOLUTE_LIMIT: std::memcpy(lim, r.impulse, 8); break;
            case BEPUGPU_JOINT_REVOLUTE:
                std::memcpy(ball, r.impulse, 12);
                std::memcpy(ang, r.impulse + 3, 8);
                std::memcpy(lim, r.impulse + 5, 8);
                break;
            case BEPUGPU_JOINT_NO_ROTATION:  // angular x, y and (in the limit's first lane) z
                ang[0] = r.impulse[0]; ang[1] = r.impulse[1]; lim[0] = r.impulse[2];
                break;
            case BEPUGPU_JOINT_WELD:
                std::memcpy(ball, r.impulse, 12);
                ang[0] = r.impulse[3]; ang[1] = r.impulse[4]; lim[0] = r.impulse[5];
                break;
            case BEPUGPU_JOINT_DISTANCE:
            case BEPUGPU_JOINT_DISTANCE_LIMIT:
            case BEPUGPU_JOINT_POINT_ON_PLANE:
            case BEPUGPU_JOINT_PLANE_SLIDER:
                ball[0] = r.impulse[0];
                break;
            case BEPUGPU_JOINT_TWIST:
                ang[0] = r.impulse[0];
                break;
            case BEPUGPU_JOINT_POINT_ON_LINE:
                ball[0] = r.impulse[0]; ball[1] = r.impulse[1];
                break;
            case BEPUGPU_JOINT_PRISMATIC:
                ball[0] = r.impulse[0]; ball[1] = r.impulse[1];
                ang[0] = r.impulse[2]; ang[1] = r.impulse[3]; lim[0] = r.impulse[4];
                lim[1] = r.impulse[5];
                break;
            case BEPUGPU_JOINT_LINE_SLIDER:
                ball[0] = r.impulse[0]; ball[1] = r.impulse[1];
                ang[0] = r.impulse[2]; ang[1] = r.impulse[3];
                lim[1] = r.impulse[4];
                break;
            case BEPUGPU_JOINT_TWIST_LIMIT:
                lim[0] = r.impulse[0];
                last = r.impulse[1];
                break;
            case BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT:
                lim[0] = r.impulse[0];
                break;
            case BEPUGPU_JOINT_SWIVEL_HINGE_ANGULAR:
                ang[0] = r.impulse[0];
                break;
            case BEPUGPU_JOINT_REVOLUTE_MOTOR:
            case BEPUGPU_JOINT_TWIST_MOTOR:
            case BEPUGPU_JOINT_LINEAR_AXIS_MOTOR:
                lim[0] = r.impulse[0];
                break;
            case BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED:
            case BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED:
            case BEPUGPU_JOINT_ANGULAR_MOTOR:
            case BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR:
                std::memcpy(ball, r.impulse, 12);
                break;
            case BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR:  // and the used softness it keeps
                std::memcpy(ball, r.impulse, 12);
                ang[1] = r.impulse[3];
                break;
            case BEPUGPU_JOINT_SWIVEL_HINGE:
                std::memcpy(ball, r.impulse, 12);
                ang[0] = r.impulse[3];
                break;
            case BEPUGPU_JOINT_LINEAR_AXIS_LIMIT:
                lim[1] = r.impulse[0];
                break;
            case BEPUGPU_JOINT_UNIVERSAL:
                std::memcpy(ball, r.impulse, 12);
                ang[0] = r.impulse[3];
                break;
        }
        at(kJACC0, slot) = make_float4(ball[0], ball[1], ball[2], ang[0]);
        at(kJACC1, slot) = make_float4(ang[1], lim[0], lim[1], last);
    }
    cudaError_t e;
    if ((e = cudaMemcpy2DAsync(s->j.lanes + (size_t)kJLA * s->j.capacity, sizeof(float4) * s->j.capacity,
                               lanes.data(), sizeof(float4) * nj, sizeof(float4) * nj, kIn, cudaMemcpyHostToDevice,
                               s->stream)) ||
        (e = cudaMemcpy2DAsync(s->j.lanes + (size_t)kJACC0 * s->j.capacity, sizeof(float4) * s->j.capacity,
                               acc.data(), sizeof(float4) * nj, sizeof(float4) * nj, 2, cudaMemcpyHostToDevice,
                               s->stream)) ||
        (e = cudaMemcpyAsync(s->j.head, head.data(), sizeof(int4) * nj, cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaMemsetAsync(s->j.state, 0, sizeof(uint2) * nj, s->stream)) ||
        (e = cudaMemcpyAsync(s->jointOffsetsDev, s->jointOffsets.data(), sizeof(int32_t) * s->jointOffsets.size(),
                             cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaStreamSynchronize(s->stream))) {
        ctx->SetError("joint upload: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    return BEPUGPU_OK;
}

bepugpu_status DownloadJoints(Context* ctx, Scene* s, bepugpu_joint* joints, uint32_t nj) {
    if (!nj) return BEPUGPU_OK;
    s->hostJointAcc.resize(2 * (size_t)nj);
    cudaError_t e;
    if ((e = cudaMemcpy2DAsync(s->hostJointAcc.data(), sizeof(float4) * nj,
                               s->j.lanes + (size_t)kJACC0 * s->j.capacity, sizeof(float4) * s->j.capacity,
                               sizeof(float4) * nj, 2, cudaMemcpyDeviceToHost, s->stream)) ||
        (e = cudaStreamSynchronize(s->stream))) {
        ctx->SetError("joint download: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    for (uint32_t u = 0; u < nj; u++) {
        bepugpu_joint& r = joints[u];
        const int slot = s->hostJointSlotOf[u];
        const float4 a0 = s->hostJointAcc[slot], a1 = s->hostJointAcc[(size_t)nj + slot];
        switch (r.type) {
            case BEPUGPU_JOINT_BALL_SOCKET:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y; r.impulse[2] = a0.z;
                break;
            case BEPUGPU_JOINT_REVOLUTE_ANGULAR:
                r.impulse[0] = a0.w; r.impulse[1] = a1.x;
                break;
            case BEPUGPU_JOINT_SWING_LIMIT:
                r.impulse[0] = a1.y;
                break;
            case BEPUGPU_JOINT_REVOLUTE_LIMIT:
                r.impulse[0] = a1.y; r.impulse[1] = a1.z;
                break;
            case BEPUGPU_JOINT_REVOLUTE:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y; r.impulse[2] = a0.z;
                r.impulse[3] = a0.w; r.impulse[4] = a1.x;
                r.impulse[5] = a1.y; r.impulse[6] = a1.z;
                break;
            case BEPUGPU_JOINT_NO_ROTATION:
                r.impulse[0] = a0.w; r.impulse[1] = a1.x; r.impulse[2] = a1.y;
                break;
            case BEPUGPU_JOINT_WELD:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y; r.impulse[2] = a0.z;
                r.impulse[3] = a0.w; r.impulse[4] = a1.x; r.impulse[5] = a1.y;
                break;
            case BEPUGPU_JOINT_DISTANCE:
            case BEPUGPU_JOINT_DISTANCE_LIMIT:
            case BEPUGPU_JOINT_POINT_ON_PLANE:
            case BEPUGPU_JOINT_PLANE_SLIDER:
                r.impulse[0] = a0.x;
                break;
            case BEPUGPU_JOINT_TWIST:
                r.impulse[0] = a0.w;
                break;
            case BEPUGPU_JOINT_POINT_ON_LINE:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y;
                break;
            case BEPUGPU_JOINT_PRISMATIC:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y;
                r.impulse[2] = a0.w; r.impulse[3] = a1.x; r.impulse[4] = a1.y;
                r.impulse[5] = a1.z;
                break;
            case BEPUGPU_JOINT_LINE_SLIDER:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y;
                r.impulse[2] = a0.w; r.impulse[3] = a1.x;
                r.impulse[4] = a1.z;
                break;
            case BEPUGPU_JOINT_TWIST_LIMIT:
                r.impulse[0] = a1.y; r.impulse[1] = a1.w;
                break;
            case BEPUGPU_JOINT_LINEAR_AXIS_LIMIT:
                r.impulse[0] = a1.z;
                break;
            case BEPUGPU_JOINT_ELLIPSE_SWING_LIMIT:
                r.impulse[0] = a1.y;
                break;
            case BEPUGPU_JOINT_SWIVEL_HINGE_ANGULAR:
                r.impulse[0] = a0.w;
                break;
            case BEPUGPU_JOINT_REVOLUTE_MOTOR:
            case BEPUGPU_JOINT_TWIST_MOTOR:
            case BEPUGPU_JOINT_LINEAR_AXIS_MOTOR:
                r.impulse[0] = a1.y;
                break;
            case BEPUGPU_JOINT_SINGLE_ENTITY_LINEAR_MOTOR:  // and the used softness it keeps
                r.impulse[0] = a0.x; r.impulse[1] = a0.y; r.impulse[2] = a0.z;
                r.impulse[3] = a1.x;
                break;
            case BEPUGPU_JOINT_MAXIMUM_LINEAR_SPEED:
            case BEPUGPU_JOINT_MAXIMUM_ANGULAR_SPEED:
            case BEPUGPU_JOINT_ANGULAR_MOTOR:
            case BEPUGPU_JOINT_SINGLE_ENTITY_ANGULAR_MOTOR:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y; r.impulse[2] = a0.z;
                break;
            case BEPUGPU_JOINT_SWIVEL_HINGE:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y; r.impulse[2] = a0.z;
                r.impulse[3] = a0.w;
                break;
            case BEPUGPU_JOINT_UNIVERSAL:
                r.impulse[0] = a0.x; r.impulse[1] = a0.y; r.impulse[2] = a0.z;
                r.impulse[3] = a0.w;
                break;
        }
    }
    return BEPUGPU_OK;
}

}  // namespace bepugpu
