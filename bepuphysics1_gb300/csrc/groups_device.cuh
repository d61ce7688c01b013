// Device side of island groups, shared by the one-scene group kernels
// (groups.cu) and the batched kernels (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include "bepugpu_internal.h"
#include "joints_device.cuh"
#include "solver_device.cuh"

namespace bepugpu {

// Body view of a group kernel.  Refs >= 0 are the group's bodies in shared
// memory, -1 is "no entity", refs <= -2 name global body -2 - ref (kinematic
// bodies, read only).
struct GroupBodies {
    float4 *pos, *quat, *vlin, *vang, *inv0, *inv1;
    BodySoA g;
    const int32_t* globalOf;  // the group's bodies' global indices
    __device__ __forceinline__ float4 Pos(int r) const { return r >= 0 ? pos[r] : g.pos[-2 - r]; }
    __device__ __forceinline__ float4 Quat(int r) const { return r >= 0 ? quat[r] : g.quat[-2 - r]; }
    __device__ __forceinline__ float4 Vlin(int r) const { return r >= 0 ? vlin[r] : g.vlin[-2 - r]; }
    __device__ __forceinline__ float4 Vang(int r) const { return r >= 0 ? vang[r] : g.vang[-2 - r]; }
    __device__ __forceinline__ float4 Inv0(int r) const { return r >= 0 ? inv0[r] : g.inv0[-2 - r]; }
    __device__ __forceinline__ float4 Inv1(int r) const { return r >= 0 ? inv1[r] : g.inv1[-2 - r]; }
    __device__ __forceinline__ void SetVelocity(int r, float4 v, float4 w) const {
        if (r >= 0) { vlin[r] = v; vang[r] = w; }  // only a group's own (dynamic) bodies are written
    }
    __device__ __forceinline__ void LocalInertia(int r, float4& l0, float4& l1, float& m33) const {
        const int gi = r >= 0 ? globalOf[r] : -2 - r;
        l0 = g.loc0[gi]; l1 = g.loc1[gi]; m33 = g.damp[gi].z;
    }
};

// Asynchronous global -> shared copies (cp.async), waited for with
// CopyAsyncWait before the block barrier that publishes them.
__device__ __forceinline__ void CopyAsync16(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void CopyAsync8(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void CopyAsyncWait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Shared memory of one CTA: 6 body lanes per body; with kShared also 24 float4
// lanes, a state word and a ref pair per manifold (400 bytes), plus 4 lanes
// when the groups hold NONCONVEX manifolds (nonConvex: 464 bytes); with joints
// the joints' solve lanes, state and refs (kJointSmemBytes each).
__host__ __device__ constexpr int GroupManifoldLanes(bool nonConvex) { return nonConvex ? 29 : 25; }
__host__ __device__ constexpr size_t GroupSmemBytes(bool shared, int bodies, int manifolds, int joints = 0,
                                                    bool nonConvex = false) {
    return 96 * (size_t)bodies + (shared ? 16 * (size_t)GroupManifoldLanes(nonConvex) * (size_t)manifolds : 0) +
           (size_t)kJointSmemBytes * joints;
}

// One step of group g by the calling CTA (the body of the group kernels).
// smem holds GroupSmemBytes(kShared, Bc, Lc) bytes.
// With kJoints the group's joints (slots [jBegin, jEnd)) are prestepped beside
// the manifolds into shared-memory solve lanes (Jc per lane) and swept colour
// by colour with them -- a colour's joints and manifolds share no dynamic
// body -- and their impulses go back to the joint lanes after the sweeps.
// kJoints: 0 no joints, 1 the classic joint types (1-5) only, 2 any type; the
// classic variant leaves the added types' branches out of the kernel.
// nonConvex: the launch's shared lanes have room for NONCONVEX manifolds'
// contact friction lanes (GroupManifoldLanes); a NONCONVEX manifold keeps its
// friction direction and impulse in lanes 12-15 (the sliding lanes it does not
// use), its prestep angular A in lanes 16-19 and angular B in lanes 25-28.
// prestepped: the group's bodies went through the candidacy and force updates
// and its manifolds through the refresh and the prestep in grid-wide launches
// before this one (k_group_refresh_force, k_group_prestep), so the step starts
// by copying bodies and manifold solve lanes into shared memory; the group's
// joints are prestepped here as without it.
template <bool kCensus, bool kShared, int kJoints>
__device__ __forceinline__ void GroupStep(const ManifoldSoA& m, const BodySoA& b, const JointSoA& jt,
                                          const StepParams& p, uint32_t flags, const GroupTables& t,
                                          const GroupDesc& g, int Bc, int Lc, int Jc, float4* smem,
                                          unsigned long long* census, bool nonConvex = false,
                                          bool prestepped = false) {
    const int nLocal = g.bEnd - g.bBegin, nm = g.mEnd - g.mBegin;
    GroupBodies bv;
    bv.pos = smem;
    bv.quat = bv.pos + Bc;
    bv.vlin = bv.quat + Bc;
    bv.vang = bv.vlin + Bc;
    bv.inv0 = bv.vang + Bc;
    bv.inv1 = bv.inv0 + Bc;
    bv.g = b;
    bv.globalOf = t.bodies + g.bBegin;
    // Solve lanes: in shared memory at local slot j, or the global lanes at
    // slot mBegin + j.
    ManifoldSoA ml = m;
    int2* sRefs = nullptr;
    if (kShared) {
        float4* lanes = smem + 6 * Bc;
        ml.pj0 = lanes;
        ml.pj1 = lanes + 4 * Lc;
        ml.pj2 = lanes + 8 * Lc;
        ml.s0 = lanes + 12 * Lc;
        ml.s1 = lanes + 13 * Lc;
        ml.saxis = lanes + 14 * Lc;
        ml.s3 = lanes + 15 * Lc;
        ml.s4 = lanes + 16 * Lc;
        ml.s5 = lanes + 17 * Lc;
        ml.s6 = lanes + 18 * Lc;
        ml.s7 = lanes + 19 * Lc;
        ml.lever = lanes + 20 * Lc;
        ml.penacc = lanes + 21 * Lc;
        ml.fricacc = lanes + 22 * Lc;
        ml.head = (int4*)(lanes + 23 * Lc);
        ml.state = (uint2*)(lanes + 24 * Lc);
        sRefs = (int2*)(ml.state + Lc);
        ml.capacity = Lc;
        ml.cfr = nonConvex ? lanes + 12 * Lc : nullptr;
        ml.cfa = nonConvex ? lanes + 16 * Lc : nullptr;
        ml.cfb = nonConvex ? lanes + 25 * Lc : nullptr;
    }
    // Joint solve lanes after the bodies and manifold lanes.
    JointSoA jl{};
    int2* jRefs = nullptr;
    const int nj = g.jEnd - g.jBegin;
    if (kJoints) {
        float4* jbase = smem + 6 * Bc + (kShared ? GroupManifoldLanes(nonConvex) * Lc : 0);
        jl.lanes = jbase;
        jl.capacity = Jc;
        jl.state = (uint2*)(jbase + kJSolveLanes * Jc);
        jRefs = (int2*)(jl.state + Jc);
        jl.count = nj;
    }
    const int tid = threadIdx.x, T = blockDim.x;
    const int lbase = kShared ? 0 : g.mBegin;  // slot of local manifold 0 in ml

    // Bodies into shared memory, through the candidacy update
    // (SimulationIslandMember.cs:53-164) and the force update (EntityBase.cs:911-975).
    // With islands (the candidacy update ran before this launch) a body of a
    // sleeping island skips the force update and reads as not dynamic for the
    // rest of the step: pos.w = 0 in shared memory.
    int asleepAll = b.islandOf != nullptr;
    if (prestepped) {
        // Bodies, then (shared lanes) every solve lane the prestep wrote, as
        // asynchronous copies; a sleeping body's pos.w is cleared after them.
        for (int i = tid; i < nLocal; i += T) {
            const int gi = t.bodies[g.bBegin + i];
            CopyAsync16(bv.pos + i, b.pos + gi);
            CopyAsync16(bv.quat + i, b.quat + gi);
            CopyAsync16(bv.vlin + i, b.vlin + gi);
            CopyAsync16(bv.vang + i, b.vang + gi);
            CopyAsync16(bv.inv0 + i, b.inv0 + gi);
            CopyAsync16(bv.inv1 + i, b.inv1 + gi);
        }
        if (kShared) {
            const int cap = m.capacity;
            for (int j = tid; j < nm; j += T) {
                const int s = g.mBegin + j;
                const bool nc = nonConvex && ((((uint32_t)m.head[s].z) >> 8) & kManifoldNonConvex);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    CopyAsync16(ml.pj0 + k * Lc + j, m.pj0 + k * cap + s);
                    CopyAsync16(ml.pj1 + k * Lc + j, m.pj1 + k * cap + s);
                    CopyAsync16(ml.pj2 + k * Lc + j, m.pj2 + k * cap + s);
                }
                if (nc) {
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        CopyAsync16(ml.cfr + k * Lc + j, m.cfr + k * cap + s);
                        CopyAsync16(ml.cfa + k * Lc + j, m.cfa + k * cap + s);
                        CopyAsync16(ml.cfb + k * Lc + j, m.cfb + k * cap + s);
                    }
                } else {
                    CopyAsync16(ml.s0 + j, m.s0 + s);
                    CopyAsync16(ml.s1 + j, m.s1 + s);
                    CopyAsync16(ml.saxis + j, m.saxis + s);
                    CopyAsync16(ml.s3 + j, m.s3 + s);
                    CopyAsync16(ml.s4 + j, m.s4 + s);
                    CopyAsync16(ml.s5 + j, m.s5 + s);
                    CopyAsync16(ml.s6 + j, m.s6 + s);
                    CopyAsync16(ml.s7 + j, m.s7 + s);
                }
                CopyAsync16(ml.lever + j, m.lever + s);
                CopyAsync16(ml.penacc + j, m.penacc + s);
                CopyAsync16(ml.fricacc + j, m.fricacc + s);
                CopyAsync16(ml.head + j, m.head + s);
                CopyAsync8(ml.state + j, m.state + s);
                CopyAsync8(sRefs + j, t.refs + s);
                if (kCensus) {  // lanes in global memory: prestep products written once and read once
                    unsigned long long c4 = (unsigned long long)(m.head[s].z & 0xff);
                    atomicAdd(census + 3, 288ull + 112ull * c4);
                }
            }
        } else if (kCensus) {
            for (int j = tid; j < nm; j += T)
                atomicAdd(census + 3, 288ull + 112ull * (unsigned long long)(m.head[g.mBegin + j].z & 0xff));
        }
        CopyAsyncWait();
        for (int i = tid; i < nLocal; i += T) {
            const bool asleep = IslandAsleep(b, t.bodies[g.bBegin + i]);
            asleepAll &= asleep ? 1 : 0;
            if (asleep) bv.pos[i].w = 0.f;
        }
    } else {
        for (int i = tid; i < nLocal; i += T) {
            int gi = t.bodies[g.bBegin + i];
            float4 v = b.vlin[gi], w = b.vang[gi], q = b.quat[gi], a, c;
            float4 act = make_float4(0.f, 0.f, 0.f, 0.f);
            const bool asleep = IslandAsleep(b, gi);
            asleepAll &= asleep ? 1 : 0;
            if (flags & (BEPUGPU_STEP_DEACTIVATION | BEPUGPU_STEP_FORCES)) act = b.act[gi];
            if ((flags & BEPUGPU_STEP_DEACTIVATION) && !b.islandOf) {  // with islands the island stage did it
                CandidacyMath(v, w, true, act, p);  // a group's bodies are dynamic
                b.act[gi] = act;
            }
            if ((flags & BEPUGPU_STEP_FORCES) && !asleep) {
                ForceMath(v, w, q, b.loc0[gi], b.loc1[gi], b.damp[gi], act, b.rawDamp + gi, a, c, p);
            } else {
                a = b.inv0[gi];
                c = b.inv1[gi];
            }
            float4 pos = b.pos[gi];
            if (asleep) pos.w = 0.f;
            bv.pos[i] = pos;
            bv.quat[i] = q;
            bv.vlin[i] = v;
            bv.vang[i] = w;
            bv.inv0[i] = a;
            bv.inv1[i] = c;
        }
    }
    // A group whose islands all sleep has nothing to do: no active constraint,
    // no manifold with an active entry (an active kinematic body touching one
    // of its islands would have woken it), no body to move.
    if (__syncthreads_and(asleepAll)) return;
    // Refresh, lanes in, prestep: a thread keeps the same manifolds throughout.
    if (!prestepped) {
        for (int j = tid; j < nm; j += T) {
            const int s = g.mBegin + j;
            int2 r = t.refs[s];
            // with islands, a pair between two inactive entries is not refreshed (NarrowPhase.cs:300-332)
            auto entryActive = [&](int ref) {
                return ref >= 0 ? bv.pos[ref].w != 0.f : (ref <= -2 && b.act[-2 - ref].y <= 0.f);
            };
            if ((flags & BEPUGPU_STEP_REFRESH_CONTACTS) && (!b.islandOf || entryActive(r.x) || entryActive(r.y)))
                RefreshManifoldV(m, bv, s, r.x, r.y, p);
            if (kShared) {
                ml.penacc[j] = m.penacc[s];  // after the refresh, which may compact them
                ml.fricacc[j] = m.fricacc[s];
                sRefs[j] = r;
            }
            if (flags & BEPUGPU_STEP_SOLVE) PrestepManifoldIO(m, s, ml, lbase + j, bv, r.x, r.y, p);
            if (kCensus) {
                // Compulsory DRAM bytes of the step for this manifold.  Lanes in shared memory:
                // head, refs, 3 input lanes per contact, material, axis and impulses read once,
                // positions, impulses and axis written once: 136 + 64 c.  Lanes in global
                // memory add the prestep products written once: 288 + 112 c.
                unsigned long long c4 = (unsigned long long)(m.head[s].z & 0xff);
                atomicAdd(census + 3, kShared ? 136ull + 64ull * c4 : 288ull + 112ull * c4);
            }
        }
    }
    if (kJoints && (flags & BEPUGPU_STEP_SOLVE))
        for (int q = tid; q < nj; q += T) {
            const int2 r = t.jointRefs[g.jBegin + q];
            jRefs[q] = r;
            PrestepJointIO<kJoints == 2>(jt, g.jBegin + q, jl, q, bv, r.x, r.y, p);
        }
    if (kCensus && tid == 0) atomicAdd(census + 3, 208ull * (unsigned long long)nLocal);  // 7 lanes in, 6 out
    __syncthreads();
    if (flags & BEPUGPU_STEP_SOLVE) {
        const int* co = t.colourOffsets + g.cBegin;
        const int* jco = kJoints ? t.jointColourOffsets + g.jcBegin : nullptr;
        for (int c = 0; c < g.cCount; c++) {
            if (kJoints)
                for (int q = jco[c] + tid; q < jco[c + 1]; q += T) {
                    const uint2 st = jl.state[q];
                    if (!(st.x & kGroupActive)) continue;
                    const int2 r = jRefs[q];
                    BodyState A, B;
                    LoadJointVelocityV(bv, r.x, A);
                    LoadJointVelocityV(bv, r.y, B);
                    WarmJoint<kJoints == 2>(jl, q, A, B, st.x, JointType(st.x));
                    if (st.x & kDynA) StoreVelocityV(bv, r.x, A);
                    if (st.x & kDynB) StoreVelocityV(bv, r.y, B);
                }
            for (int j = co[c] + tid; j < co[c + 1]; j += T) {
                const int sl = lbase + j;
                uint2 st = ml.state[sl];
                if (!(st.x & kGroupActive)) continue;
                int2 r = kShared ? sRefs[j] : t.refs[g.mBegin + j];
                BodyState A, B;
                if (r.x != -1) LoadBodyV(bv, r.x, A);
                if (r.y != -1) LoadBodyV(bv, r.y, B);
                WarmStartManifold(ml, sl, A, B, st.x, ml.head[sl].z & 0xff);
                if (st.x & kDynA) StoreVelocityV(bv, r.x, A);
                if (st.x & kDynB) StoreVelocityV(bv, r.y, B);
            }
            __syncthreads();
        }
        for (int it = 0; it < p.iterationLimit; it++)
            for (int c = 0; c < g.cCount; c++) {
                if (kJoints)
                    for (int q = jco[c] + tid; q < jco[c + 1]; q += T) {
                        uint2 st = jl.state[q];
                        if (!(st.x & kGroupActive)) continue;
                        const int2 r = jRefs[q];
                        BodyState A, B;
                        LoadJointVelocityV(bv, r.x, A);
                        LoadJointVelocityV(bv, r.y, B);
                        SolveJoint<kJoints == 2>(jl, q, A, B, st, JointType(st.x), p);
                        if (st.x & kDynA) StoreVelocityV(bv, r.x, A);
                        if (st.x & kDynB) StoreVelocityV(bv, r.y, B);
                        jl.state[q] = st;
                    }
                for (int j = co[c] + tid; j < co[c + 1]; j += T) {
                    const int sl = lbase + j;
                    uint2 st = ml.state[sl];
                    if (!(st.x & kGroupActive)) continue;
                    int2 r = kShared ? sRefs[j] : t.refs[g.mBegin + j];
                    const int count = ml.head[sl].z & 0xff;
                    BodyState A, B;
                    if (r.x != -1) LoadBodyV(bv, r.x, A);
                    if (r.y != -1) LoadBodyV(bv, r.y, B);
                    if (kCensus) {  // algorithmic bytes of the visit: 76 d + 136 + 48 c
                        int d = ((st.x & kDynA) ? 1 : 0) + ((st.x & kDynB) ? 1 : 0);
                        atomicAdd(census, 76ull * d + 136ull + 48ull * count);
                        atomicAdd(census + 1, 1ull);
                        atomicAdd(census + 2, (unsigned long long)count);
                    }
                    SolveManifold(ml, sl, A, B, st, count, p);
                    if (st.x & kDynA) StoreVelocityV(bv, r.x, A);
                    if (st.x & kDynB) StoreVelocityV(bv, r.y, B);
                    ml.state[sl] = st;
                }
                __syncthreads();
            }
        if (kJoints)  // joint impulses back to the joint lanes
            for (int q = tid; q < nj; q += T) {
                jt.L(kJACC0, g.jBegin + q) = jl.L(kJACC0, q);
                jt.L(kJACC1, g.jBegin + q) = jl.L(kJACC1, q);
            }
        if (kShared) {  // impulses and sliding axis (NONCONVEX: contact friction) back to the manifold records
            for (int j = tid; j < nm; j += T) {
                const int s = g.mBegin + j;
                m.penacc[s] = ml.penacc[j];
                m.fricacc[s] = ml.fricacc[j];
                const int4 h = ml.head[j];
                if (nonConvex && (((uint32_t)h.z >> 8) & kManifoldNonConvex)) {
                    for (int k = 0; k < (h.z & 0xff); k++) m.cfr[k * m.capacity + s] = ml.cfr[k * Lc + j];
                } else {
                    m.saxis[s] = ml.saxis[j];
                }
            }
        }
    }
    // Position update (EntityBase.cs:1124-1160) and write-back; a sleeping
    // body (pos.w = 0 here) is left as it was.
    for (int i = tid; i < nLocal; i += T) {
        int gi = t.bodies[g.bBegin + i];
        float4 pos = bv.pos[i], q = bv.quat[i], v = bv.vlin[i], w = bv.vang[i];
        if (pos.w == 0.f) continue;
        if (flags & BEPUGPU_STEP_POSITIONS) {  // a group's bodies are dynamic, so active
            PositionMath(pos, q, v, w, p);
            b.pos[gi] = pos;
            b.quat[gi] = q;
        }
        b.vlin[gi] = v;
        b.vang[gi] = w;
        b.inv0[gi] = bv.inv0[i];
        b.inv1[gi] = bv.inv1[i];
    }
}


}  // namespace bepugpu
