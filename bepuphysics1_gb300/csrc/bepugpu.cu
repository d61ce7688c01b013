// C ABI of the GB300 solver (include/bepugpu.h): contexts, scenes, uploads,
// colouring and the one-scene step path.
//
// One scene step is the device sequence
//   refresh -> ForceUpdater -> prestep -> warm start (one sweep per colour) ->
//   I x (one sweep per colour) -> PositionUpdater
// run either as one kernel per sweep captured in a CUDA graph
// (BEPUGPU_MODE_GRAPH) or as one cooperative persistent kernel that separates
// the sweeps with a bounded grid barrier (BEPUGPU_MODE_PERSISTENT).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/bepugpu.h"
#include "colouring.h"
#include "solver_device.cuh"
#include "bepugpu_internal.h"

namespace bepugpu {

// ------------------------------------------------------------------ kernels --
__global__ void k_unpack_bodies(const bepugpu_body* __restrict__ rec, int n, BodySoA b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bepugpu_body& r = rec[i];
    bool dyn = r.is_dynamic != 0;
    b.pos[i] = make_float4(r.position[0], r.position[1], r.position[2], dyn ? 1.f : 0.f);
    b.quat[i] = make_float4(r.orientation[0], r.orientation[1], r.orientation[2], r.orientation[3]);
    const float* L = r.local_inverse_inertia;
    float l[9];
    for (int k = 0; k < 9; k++) l[k] = dyn ? L[k] : 0.f;
    b.vlin[i] = make_float4(r.linear_velocity[0], r.linear_velocity[1], r.linear_velocity[2], dyn ? r.inverse_mass : 0.f);
    b.vang[i] = make_float4(r.angular_velocity[0], r.angular_velocity[1], r.angular_velocity[2], 0.f);
    b.loc0[i] = make_float4(l[0], l[1], l[2], l[3]);
    b.loc1[i] = make_float4(l[4], l[5], l[6], l[7]);
    b.inv0[i] = make_float4(0, 0, 0, 0);
    b.inv1[i] = make_float4(0, 0, 0, 0);
    b.act[i] = make_float4(r.previous_velocity, r.velocity_time_below_limit, __uint_as_float(r.activity), 0.f);
}

// World inverse inertia R^T L R of a body with orientation q and local inverse
// inertia L (rows l0.xyz, l0.w l1.xy, l1.zw L33): the first eight entries in
// a, c and the last returned (kept in the angular velocity lane's w).
__device__ __forceinline__ float WorldInertia(float4 q, float4 l0, float4 l1, float L33, float4& a, float4& c) {
    float qX2 = q.x + q.x, qY2 = q.y + q.y, qZ2 = q.z + q.z;
    float XX = qX2 * q.x, YY = qY2 * q.y, ZZ = qZ2 * q.z;
    float XY = qX2 * q.y, XZ = qX2 * q.z, XW = qX2 * q.w;
    float YZ = qY2 * q.z, YW = qY2 * q.w, ZW = qZ2 * q.w;
    float R11 = 1 - YY - ZZ, R21 = XY - ZW, R31 = XZ + YW;
    float R12 = XY + ZW, R22 = 1 - XX - ZZ, R32 = YZ - XW;
    float R13 = XZ - YW, R23 = YZ + XW, R33 = 1 - XX - YY;
    float L11 = l0.x, L12 = l0.y, L13 = l0.z, L21 = l0.w, L22 = l1.x, L23 = l1.y, L31 = l1.z, L32 = l1.w;
    float m11 = R11 * L11 + R21 * L21 + R31 * L31;
    float m12 = R11 * L12 + R21 * L22 + R31 * L32;
    float m13 = R11 * L13 + R21 * L23 + R31 * L33;
    float m21 = R12 * L11 + R22 * L21 + R32 * L31;
    float m22 = R12 * L12 + R22 * L22 + R32 * L32;
    float m23 = R12 * L13 + R22 * L23 + R32 * L33;
    float m31 = R13 * L11 + R23 * L21 + R33 * L31;
    float m32 = R13 * L12 + R23 * L22 + R33 * L32;
    float m33 = R13 * L13 + R23 * L23 + R33 * L33;
    a.x = m11 * R11 + m12 * R21 + m13 * R31;
    a.y = m11 * R12 + m12 * R22 + m13 * R32;
    a.z = m11 * R13 + m12 * R23 + m13 * R33;
    a.w = m21 * R11 + m22 * R21 + m23 * R31;
    c.x = m21 * R12 + m22 * R22 + m23 * R32;
    c.y = m21 * R13 + m22 * R23 + m23 * R33;
    c.z = m31 * R11 + m32 * R21 + m33 * R31;
    c.w = m31 * R12 + m32 * R22 + m33 * R32;
    return m31 * R13 + m32 * R23 + m33 * R33;
}
// World inverse inertia at upload (Entity orientation setter: R^T L R), so a
// solve-only step without the force stage sees the same tensor as the oracle.
__global__ void k_world_inertia(BodySoA b, const float* __restrict__ localM33) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.count) return;
    float4 a, c, w = b.vang[i];
    w.w = WorldInertia(b.quat[i], b.loc0[i], b.loc1[i], localM33[i], a, c);
    b.inv0[i] = a;
    b.inv1[i] = c;
    b.vang[i] = w;
}

// The state fields of the scene's device copy of the caller's body records
// (kept since the upload): the download is then one copy of whole records,
// their other fields exactly as uploaded.
__global__ void k_patch_body_records(BodySoA b, bepugpu_body* __restrict__ rec) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.count) return;
    float4 p = b.pos[i], q = b.quat[i], v = b.vlin[i], w = b.vang[i];
    bepugpu_body& r = rec[i];
    r.position[0] = p.x; r.position[1] = p.y; r.position[2] = p.z;
    r.orientation[0] = q.x; r.orientation[1] = q.y; r.orientation[2] = q.z; r.orientation[3] = q.w;
    r.linear_velocity[0] = v.x; r.linear_velocity[1] = v.y; r.linear_velocity[2] = v.z;
    r.angular_velocity[0] = w.x; r.angular_velocity[1] = w.y; r.angular_velocity[2] = w.z;
    const float4 a = b.act[i];
    r.previous_velocity = a.x;
    r.velocity_time_below_limit = a.y;
    r.activity = __float_as_uint(a.z);
}

// Lowest body with a non-finite position, orientation or velocity.
__device__ __forceinline__ bool Finite4(float4 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w); }
__global__ void k_check_finite(BodySoA b, int* firstBad) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.count) return;
    float4 p = b.pos[i], v = b.vlin[i], w = b.vang[i];
    if (!Finite4(p) || !Finite4(b.quat[i]) || !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z) ||
        !isfinite(w.x) || !isfinite(w.y) || !isfinite(w.z))
        atomicMin(firstBad, i);
}

// A wait on a flag nothing sets, bounded like GridBarrier's: gives up after
// `limit` polls and reports TIMEOUT in *status.
__global__ void k_bounded_wait_probe(volatile unsigned int* flag, unsigned int limit, int* status) {
    unsigned int spins = 0;
    while (*flag == 0u) {
        if (++spins > limit) {
            *status = BEPUGPU_TIMEOUT;
            return;
        }
        __nanosleep(64);
    }
    *status = BEPUGPU_OK;
}

// The device's float results of the reference's double expressions
// (double_rounding.cuh) over n inputs; `fast` counts the inputs the FP32
// path decided.
__global__ void k_probe_double_rounding(int kind, const float* __restrict__ a, const float* __restrict__ b, int n,
                                        float* __restrict__ out, unsigned int* fast) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r = 0.f;
    bool f = false;
    if (kind == 0) {
        f = dr::TryInvSqrt(a[i], r);
        if (!f) r = dr::InvSqrtAsDouble(a[i]);
    } else if (kind == 1) {
        f = dr::TrySqrtQuotient(a[i], b[i], r);
        if (!f) r = dr::SqrtQuotientAsDouble(a[i], b[i]);
    } else {
        f = dr::TryPow(a[i], b[i], r);
        if (!f) r = dr::PowAsDouble(a[i], b[i]);
    }
    out[i] = r;
    if (f) atomicAdd(fast, 1u);
}

// Checks of the update calls, before anything is written: check[0] receives
// the lowest offending record index (stays INT_MAX when none), check[1] the
// KinematicState bits of the kinematic bodies.
__device__ __forceinline__ bool SameWord(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }
__global__ void k_check_body_records(const bepugpu_body* __restrict__ in, const bepugpu_body* __restrict__ kept, int n,
                                     int* check) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bepugpu_body &r = in[i], &k = kept[i];
    bool same = r.is_dynamic == k.is_dynamic && SameWord(r.inverse_mass, k.inverse_mass) &&
                SameWord(r.linear_damping, k.linear_damping) && SameWord(r.angular_damping, k.angular_damping);
    for (int q = 0; q < 9; q++) same = same && SameWord(r.local_inverse_inertia[q], k.local_inverse_inertia[q]);
    if (!same) atomicMin(check, i);
    if (!r.is_dynamic) {
        KinematicState k{};
        k.Add(r.linear_velocity[0] != 0 || r.linear_velocity[1] != 0 || r.linear_velocity[2] != 0 ||
                  r.angular_velocity[0] != 0 || r.angular_velocity[1] != 0 || r.angular_velocity[2] != 0,
              r.activity, r.previous_velocity, r.velocity_time_below_limit);
        const uint32_t bits = k.Bits();
        if (bits) atomicOr(check + 1, (int)bits);
    }
}
// The state fields of checked records into the body lanes and the kept records.
__global__ void k_update_body_state(const bepugpu_body* __restrict__ in, int n, BodySoA b, bepugpu_body* kept) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bepugpu_body& r = in[i];
    bepugpu_body& k = kept[i];
    float4 p = b.pos[i], v = b.vlin[i], w = b.vang[i];
    b.pos[i] = make_float4(r.position[0], r.position[1], r.position[2], p.w);
    b.quat[i] = make_float4(r.orientation[0], r.orientation[1], r.orientation[2], r.orientation[3]);
    b.vlin[i] = make_float4(r.linear_velocity[0], r.linear_velocity[1], r.linear_velocity[2], v.w);
    b.vang[i] = make_float4(r.angular_velocity[0], r.angular_velocity[1], r.angular_velocity[2], w.w);
    b.act[i] = make_float4(r.previous_velocity, r.velocity_time_below_limit, __uint_as_float(r.activity), 0.f);
    k.previous_velocity = r.previous_velocity;
    k.velocity_time_below_limit = r.velocity_time_below_limit;
    k.activity = r.activity;
    for (int q = 0; q < 3; q++) {
        k.position[q] = r.position[q];
        k.linear_velocity[q] = r.linear_velocity[q];
        k.angular_velocity[q] = r.angular_velocity[q];
    }
    for (int q = 0; q < 4; q++) k.orientation[q] = r.orientation[q];
}
// State records cross the host link (records in page-locked host memory are
// read and written in place), so a block moves its records as one contiguous
// run of 16-byte words through shared memory: consecutive threads, consecutive words.
constexpr int kStateBlock = 128;

// State records into the body lanes and the kept records (bepugpu_step_state),
// with the world inverse inertia of the new orientation (k_world_inertia).
__global__ void __launch_bounds__(kStateBlock) k_update_body_state_records(const bepugpu_body_state* __restrict__ in,
                                                                           int n, BodySoA b, bepugpu_body* kept,
                                                                           const float* __restrict__ localM33) {
    __shared__ float4 buf[4 * kStateBlock];
    const int first = blockIdx.x * kStateBlock, rows = min(kStateBlock, n - first);
    const float4* src = (const float4*)(in + first);
    for (int k = threadIdx.x; k < 4 * rows; k += kStateBlock) buf[k] = src[k];
    __syncthreads();
    const int i = first + threadIdx.x;
    if (threadIdx.x >= rows) return;
    const float4* w4 = buf + 4 * threadIdx.x;  // 64-byte records: four 16-byte words
    const float4 r0 = w4[0], r1 = w4[1], r2 = w4[2], r3 = w4[3];
    // r0 = p.xyz q.x, r1 = q.yzw v.x, r2 = v.yz w.xy, r3 = w.z activity previous timeBelow
    const float4 p = b.pos[i], v = b.vlin[i], q = make_float4(r0.w, r1.x, r1.y, r1.z);
    float4 ia, ic;
    const float m33 = WorldInertia(q, b.loc0[i], b.loc1[i], localM33[i], ia, ic);
    b.pos[i] = make_float4(r0.x, r0.y, r0.z, p.w);
    b.quat[i] = q;
    b.vlin[i] = make_float4(r1.w, r2.x, r2.y, v.w);
    b.vang[i] = make_float4(r2.z, r2.w, r3.x, m33);
    b.inv0[i] = ia;
    b.inv1[i] = ic;
    b.act[i] = make_float4(r3.z, r3.w, r3.y, 0.f);
    bepugpu_body& k = kept[i];
    k.position[0] = r0.x; k.position[1] = r0.y; k.position[2] = r0.z;
    k.orientation[0] = r0.w; k.orientation[1] = r1.x; k.orientation[2] = r1.y; k.orientation[3] = r1.z;
    k.linear_velocity[0] = r1.w; k.linear_velocity[1] = r2.x; k.linear_velocity[2] = r2.y;
    k.angular_velocity[0] = r2.z; k.angular_velocity[1] = r2.w; k.angular_velocity[2] = r3.x;
    k.activity = __float_as_uint(r3.y);
    k.previous_velocity = r3.z;
    k.velocity_time_below_limit = r3.w;
}
// Body lanes -> state records (one block's share).
__device__ __forceinline__ void PackBodyState(const BodySoA& b, bepugpu_body_state* __restrict__ out, int block,
                                              float4* buf) {
    const int first = block * kStateBlock, rows = min(kStateBlock, b.count - first);
    const int i = first + threadIdx.x;
    if (threadIdx.x < rows) {
        const float4 p = b.pos[i], q = b.quat[i], v = b.vlin[i], w = b.vang[i], a = b.act[i];
        float4* o = buf + 4 * threadIdx.x;
        o[0] = make_float4(p.x, p.y, p.z, q.x);
        o[1] = make_float4(q.y, q.z, q.w, v.x);
        o[2] = make_float4(v.y, v.z, w.x, w.y);
        o[3] = make_float4(w.z, a.z, a.x, a.y);
    }
    __syncthreads();
    float4* dst = (float4*)(out + first);
    for (int k = threadIdx.x; k < 4 * rows; k += kStateBlock) dst[k] = buf[k];
}
// Manifold slots -> state records, in record order (one block's share).
__device__ __forceinline__ void PackManifoldState(const ManifoldSoA& m, const int32_t* __restrict__ slot_of, int n,
                                                  bepugpu_manifold_state* __restrict__ out, int block, float4* buf) {
    const int first = block * kStateBlock, rows = min(kStateBlock, n - first);
    const int i = first + threadIdx.x;
    if (threadIdx.x < rows) {
    const int s = slot_of[i], cap = m.capacity;
    const int count = m.head[s].z & 0xff;
    const float4 pa = m.penacc[s], f = m.fricacc[s], ax = m.saxis[s];
    int id[4];
    float fi[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        id[k] = k < count ? __float_as_int(m.cnrm[k * cap + s].w) : 0;
        fi[k] = k < count ? m.cfr[k * cap + s].w : 0.f;
    }
    float4* o = buf + 5 * threadIdx.x;
    o[0] = make_float4(__int_as_float(count), __int_as_float(id[0]), __int_as_float(id[1]), __int_as_float(id[2]));
    o[1] = make_float4(__int_as_float(id[3]), count > 0 ? pa.x : 0.f, count > 1 ? pa.y : 0.f, count > 2 ? pa.z : 0.f);
    o[2] = make_float4(count > 3 ? pa.w : 0.f, f.x, f.y, f.z);
    o[3] = make_float4(ax.x, ax.y, ax.z, fi[0]);
    o[4] = make_float4(fi[1], fi[2], fi[3], 0.f);
    }
    __syncthreads();
    float4* dst = (float4*)(out + first);
    for (int k = threadIdx.x; k < 5 * rows; k += kStateBlock) dst[k] = buf[k];
}
// Both downloads in one launch: blocks [0, bodyBlocks) pack body state
// records, the rest manifold state records.
__global__ void __launch_bounds__(kStateBlock) k_pack_state(BodySoA b, bepugpu_body_state* __restrict__ bodies,
                                                            int bodyBlocks, ManifoldSoA m,
                                                            const int32_t* __restrict__ slot_of, int nm,
                                                            bepugpu_manifold_state* __restrict__ manifolds) {
    __shared__ float4 buf[5 * kStateBlock];
    if ((int)blockIdx.x < bodyBlocks) PackBodyState(b, bodies, blockIdx.x, buf);
    else PackManifoldState(m, slot_of, nm, manifolds, blockIdx.x - bodyBlocks, buf);
}
__global__ void k_check_manifold_records(const bepugpu_manifold* __restrict__ rec, const int32_t* __restrict__ slot_of,
                                         int n, ManifoldSoA m, int* check) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bepugpu_manifold& r = rec[i];
    int4 h = m.head[slot_of[i]];
    const uint32_t was = (uint32_t)h.z >> 8;
    bool bad = r.body_a != h.x || r.body_b != h.y || r.contact_count < 0 || r.contact_count > 4 ||
               ((r.flags ^ was) & (BEPUGPU_MANIFOLD_GENERATED | BEPUGPU_MANIFOLD_NONCONVEX));
    if (!bad && (r.flags & BEPUGPU_MANIFOLD_GENERATED)) {  // contact_order: a permutation of the contacts
        const uint32_t code = (uint32_t)r.contact_order ^ 0xE4u;
        uint32_t seen = 0;
        for (int k = 0; k < r.contact_count; k++) seen |= 1u << ((code >> (2 * k)) & 3u);
        bad = seen != (1u << r.contact_count) - 1u;
    }
    if (bad) atomicMin(check, i);
}

// Manifold records -> slots (slot_of[i] is the colour-order slot of record i).
__global__ void k_unpack_manifolds(const bepugpu_manifold* __restrict__ rec, const int32_t* __restrict__ slot_of,
                                   int n, ManifoldSoA m) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bepugpu_manifold& r = rec[i];
    int s = slot_of[i];
    int cap = m.capacity;
    int count = r.contact_count < 0 ? 0 : (r.contact_count > 4 ? 4 : r.contact_count);
    m.head[s] = make_int4(r.body_a, r.body_b, count | (int)(r.flags << 8), i);
    for (int k = 0; k < 4; k++) {
        const bepugpu_contact& c = r.contacts[k];
        m.cpos[k * cap + s] = make_float4(c.position[0], c.position[1], c.position[2], c.penetration_depth);
        m.cnrm[k * cap + s] = make_float4(c.normal[0], c.normal[1], c.normal[2], __int_as_float(c.id));
        m.offA[k * cap + s] = make_float4(c.local_offset_a[0], c.local_offset_a[1], c.local_offset_a[2],
                                          c.base_penetration_depth);
        m.offB[k * cap + s] = make_float4(c.local_offset_b[0], c.local_offset_b[1], c.local_offset_b[2], 0.f);
        // contact friction state: NONCONVEX manifolds only (zero in a convex one's records)
        m.cfr[k * cap + s] = k < count && (r.flags & BEPUGPU_MANIFOLD_NONCONVEX)
                                 ? make_float4(c.friction_direction[0], c.friction_direction[1],
                                               c.friction_direction[2], c.friction_impulse)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float pa[4];
    for (int k = 0; k < 4; k++) pa[k] = k < count ? r.contacts[k].penetration_impulse : 0.f;
    m.penacc[s] = make_float4(pa[0], pa[1], pa[2], pa[3]);
    bool live = count > 0;
    const int order = (r.flags & BEPUGPU_MANIFOLD_GENERATED) ? r.contact_order : 0;
    m.fricacc[s] = make_float4(live ? r.sliding_impulse[0] : 0.f, live ? r.sliding_impulse[1] : 0.f,
                               live ? r.twist_impulse : 0.f, __int_as_float(order));
    m.saxis[s] = make_float4(r.sliding_axis[0], r.sliding_axis[1], r.sliding_axis[2], 0.f);
    m.mat[s] = make_float4(r.kinetic_friction, r.static_friction, r.bounciness, 0.f);
    m.state[s] = make_uint2(0u, 0u);
}

// Whole manifold records in record order (the caller's array), built in
// shared memory and written out as contiguous 8-byte stores: the download
// is then one copy straight into the caller's records.
constexpr int kRecordBlock = 128;
static_assert(sizeof(bepugpu_manifold) % 8 == 0, "manifold records must tile 8-byte stores");
__global__ void __launch_bounds__(kRecordBlock) k_pack_manifold_records(ManifoldSoA m,
                                                                         const int32_t* __restrict__ slot_of, int n,
                                                                         uint2* __restrict__ out) {
    __shared__ __align__(16) bepugpu_manifold recs[kRecordBlock];
    const int first = blockIdx.x * kRecordBlock;
    const int i = first + threadIdx.x;
    if (i < n) {
        const int s = slot_of[i], cap = m.capacity;
        const int4 h = m.head[s];
        const int count = h.z & 0xff;
        bepugpu_manifold& r = recs[threadIdx.x];
        r.body_a = h.x;
        r.body_b = h.y;
        r.contact_count = count;
        r.flags = (uint32_t)h.z >> 8;
        const float4 mat = m.mat[s], pa = m.penacc[s], f = m.fricacc[s], ax = m.saxis[s];
        r.kinetic_friction = mat.x;
        r.static_friction = mat.y;
        r.bounciness = mat.z;
        r.sliding_impulse[0] = f.x;
        r.sliding_impulse[1] = f.y;
        r.sliding_axis[0] = ax.x;
        r.sliding_axis[1] = ax.y;
        r.sliding_axis[2] = ax.z;
        r.twist_impulse = f.z;
        r.contact_order = __float_as_int(f.w);
        const float acc[4] = {pa.x, pa.y, pa.z, pa.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            bepugpu_contact& c = r.contacts[k];
            if (k < count) {
                const float4 cp = m.cpos[k * cap + s], cn = m.cnrm[k * cap + s], oa = m.offA[k * cap + s],
                             ob = m.offB[k * cap + s], fr = m.cfr[k * cap + s];
                c.position[0] = cp.x; c.position[1] = cp.y; c.position[2] = cp.z;
                c.normal[0] = cn.x; c.normal[1] = cn.y; c.normal[2] = cn.z;
                c.penetration_depth = cp.w;
                c.id = __float_as_int(cn.w);
                c.local_offset_a[0] = oa.x; c.local_offset_a[1] = oa.y; c.local_offset_a[2] = oa.z;
                c.local_offset_b[0] = ob.x; c.local_offset_b[1] = ob.y; c.local_offset_b[2] = ob.z;
                c.base_penetration_depth = oa.w;
                c.penetration_impulse = acc[k];
                c.friction_impulse = fr.w;
                c.friction_direction[0] = fr.x; c.friction_direction[1] = fr.y; c.friction_direction[2] = fr.z;
            } else {
                uint32_t* w = (uint32_t*)&c;
                for (int q = 0; q < (int)(sizeof(bepugpu_contact) / 4); q++) w[q] = 0u;
            }
        }
    }
    __syncthreads();
    const int rows = min(kRecordBlock, n - first);
    const int words = rows * (int)(sizeof(bepugpu_manifold) / 8);
    const uint2* src = (const uint2*)recs;
    uint2* dst = out + (size_t)first * (sizeof(bepugpu_manifold) / 8);
    for (int k = threadIdx.x; k < words; k += kRecordBlock) dst[k] = src[k];
}

__global__ void k_refresh(ManifoldSoA m, BodySoA b, StepParams p) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < m.count) RefreshManifold(m, b, s, p);
}
// Refresh and force update in one launch: the refresh reads poses only and the
// force update writes velocities and inertia only.
// Bodies a group kernel steps are skipped by the sweep path's body kernels.
__device__ __forceinline__ bool OwnedByGroup(const BodySoA& b, int i) {
    return __float_as_uint(b.damp[i].w) & kOwnedByGroup;
}
// The body stages at the start of a step (candidacy and force update) touch
// velocities, inertia and activity only, so they share the refresh's launch.
constexpr uint32_t kStartStages = BEPUGPU_STEP_FORCES | BEPUGPU_STEP_DEACTIVATION;
__global__ void k_refresh_force(ManifoldSoA m, BodySoA b, StepParams p, uint32_t flags) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m.count) {
        if (flags & BEPUGPU_STEP_REFRESH_CONTACTS) RefreshManifold(m, b, t, p);
    } else if (t - m.count < b.count && !OwnedByGroup(b, t - m.count)) {
        StartBodyStep(b, t - m.count, p, flags);
    }
}
// Body stages over the bodies no group kernel steps (the scene has groups).
__global__ void k_refresh_force_list(ManifoldSoA m, BodySoA b, StepParams p, const int32_t* __restrict__ list, int n,
                                     uint32_t flags) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m.count) {
        if (flags & BEPUGPU_STEP_REFRESH_CONTACTS) RefreshManifold(m, b, t, p);
    } else if (t - m.count < n) {
        if (flags & kStartStages) StartBodyStep(b, list[t - m.count], p, flags);
    }
}
// The kinematic bodies of a scene whose step is otherwise island groups
// alone, after the group launch: their candidacy update and, while active,
// their position update.  A kinematic body's velocity does not change during
// the step, so its candidacy reads the same values here as at the start.
__global__ void k_kinematic_tail(BodySoA b, StepParams p, const int32_t* __restrict__ list, int n, uint32_t flags) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = list[t];
    if (flags & BEPUGPU_STEP_DEACTIVATION) StartBodyStep(b, i, p, BEPUGPU_STEP_DEACTIVATION);
    if (flags & BEPUGPU_STEP_POSITIONS) PositionUpdateBody(b, i, p);
}
__global__ void k_position_list(BodySoA b, StepParams p, const int32_t* __restrict__ list, int n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) PositionUpdateBody(b, list[t], p);
}
__global__ void k_position(BodySoA b, StepParams p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < b.count && !OwnedByGroup(b, i)) PositionUpdateBody(b, i, p);
}
__global__ void k_prestep(ManifoldSoA m, BodySoA b, StepParams p) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < m.count) PrestepManifold(m, b, s, p);
}

__device__ __forceinline__ void LoadPair(const BodySoA& b, int4 h, BodyState& A, BodyState& B) {
    if (h.x >= 0) LoadBody(b, h.x, A);
    if (h.y >= 0) LoadBody(b, h.y, B);
}
__device__ __forceinline__ void StorePair(const BodySoA& b, int4 h, uint32_t st, const BodyState& A,
                                          const BodyState& B) {
    if (st & kDynA) StoreVelocity(b, h.x, A);
    if (st & kDynB) StoreVelocity(b, h.y, B);
}

__device__ __forceinline__ void WarmSlot(const ManifoldSoA& m, const BodySoA& b, int s) {
    uint2 state = m.state[s];
    if (!(state.x & kGroupActive)) return;
    int4 h = m.head[s];
    BodyState A, B;
    LoadPair(b, h, A, B);
    WarmStartManifold(m, s, A, B, state.x, h.z & 0xff);
    StorePair(b, h, state.x, A, B);
}
__device__ __forceinline__ void SolveSlot(const ManifoldSoA& m, const BodySoA& b, int s, const StepParams& p) {
    uint2 state = m.state[s];
    if (!(state.x & kGroupActive)) return;
    int4 h = m.head[s];
    BodyState A, B;
    LoadPair(b, h, A, B);
    SolveManifold(m, s, A, B, state, h.z & 0xff, p);
    StorePair(b, h, state.x, A, B);
    m.state[s] = state;
}

__global__ void k_warm(ManifoldSoA m, BodySoA b, int begin, int end) {
    int s = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (s < end) WarmSlot(m, b, s);
}
// A colour sweep: the visit's prestep lanes load before the previous sweep
// ends (they do not change during the sweeps); state, impulses and bodies after.
__global__ void k_solve(ManifoldSoA m, BodySoA b, StepParams p, int begin, int end) {
    LetDependentsLaunch();
    const int s = begin + blockIdx.x * blockDim.x + threadIdx.x;
    SolveLanes L;
    int4 h = make_int4(0, 0, 0, 0);
    if (s < end) {
        h = m.head[s];
        const int count = h.z & 0xff;
        LoadSolveLanes(m, s, count, count > 0, L);
    }
    WaitForPrerequisites();
    if (s >= end) return;
    uint2 state = m.state[s];
    if (!(state.x & kGroupActive)) return;
    BodyState A, B;
    LoadPair(b, h, A, B);
    SolveManifold(m, s, A, B, state, h.z & 0xff, p, &L);
    StorePair(b, h, state.x, A, B);
    m.state[s] = state;
}

// Joints (joints_device.cuh).  A colour's joints and manifolds touch different
// dynamic bodies, so one launch runs both: threads [0, joints) take the joints.
// kAdded false builds the variant for scenes whose joints are all of the
// classic types (1-5), without the added types' branches.
template <bool kAdded>
__device__ __forceinline__ void WarmJointSlot(const JointSoA& j, const BodySoA& b, int s) {
    uint2 st = j.state[s];
    if (!(st.x & kGroupActive)) return;
    int4 h = j.head[s];
    BodyState A, B;
    LoadJointVelocityV(GlobalBodies{b}, h.x, A);
    LoadJointVelocityV(GlobalBodies{b}, h.y, B);
    WarmJoint<kAdded>(j, s, A, B, st.x, h.z & 0xff);
    if (st.x & kDynA) StoreVelocity(b, h.x, A);
    if (st.x & kDynB) StoreVelocity(b, h.y, B);
}
template <bool kAdded>
__device__ __forceinline__ void SolveJointSlot(const JointSoA& j, const BodySoA& b, int s, const StepParams& p) {
    uint2 st = j.state[s];
    if (!(st.x & kGroupActive)) return;
    int4 h = j.head[s];
    BodyState A, B;
    LoadJointVelocityV(GlobalBodies{b}, h.x, A);
    LoadJointVelocityV(GlobalBodies{b}, h.y, B);
    SolveJoint<kAdded>(j, s, A, B, st, h.z & 0xff, p);
    if (st.x & kDynA) StoreVelocity(b, h.x, A);
    if (st.x & kDynB) StoreVelocity(b, h.y, B);
    j.state[s] = st;
}
template <bool kAdded>
__global__ void k_prestep_mixed(ManifoldSoA m, BodySoA b, JointSoA j, StepParams p) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < j.count) PrestepJoint<kAdded>(j, b, t, p);
    else if (t - j.count < m.count) PrestepManifold(m, b, t - j.count, p);
}
template <bool kAdded>
__global__ void k_warm_mixed(ManifoldSoA m, BodySoA b, JointSoA j, int mb, int me, int jb, int je) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < je - jb) WarmJointSlot<kAdded>(j, b, jb + t);
    else if (mb + t - (je - jb) < me) WarmSlot(m, b, mb + t - (je - jb));
}
template <bool kAdded>
__global__ void k_solve_mixed(ManifoldSoA m, BodySoA b, JointSoA j, StepParams p, int mb, int me, int jb, int je) {
    LetDependentsLaunch();
    WaitForPrerequisites();
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < je - jb) SolveJointSlot<kAdded>(j, b, jb + t, p);
    else if (mb + t - (je - jb) < me) SolveSlot(m, b, mb + t - (je - jb), p);
}

// Bounded grid barrier for the cooperative kernel.  Thread 0 of each block
// arrives on a counter; the last arrival resets it and bumps the generation.
// A wait that outlives kBarrierSpinLimit polls sets *err and the kernel returns.
constexpr long long kBarrierSpinLimit = 1ll << 24;
__device__ __forceinline__ bool GridBarrier(unsigned int* counter, volatile unsigned int* generation,
                                            unsigned int& localGen, volatile int* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int g = localGen;
        __threadfence();
        unsigned int arrived = atomicAdd(counter, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(counter, 0u);
            __threadfence();
            atomicAdd((unsigned int*)generation, 1u);
        } else {
            long long spins = 0;
            while (*generation == g) {
                if (++spins > kBarrierSpinLimit) {
                    *err = BEPUGPU_TIMEOUT;
                    break;
                }
                if (*err) break;
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    localGen++;
    __syncthreads();
    return *err == 0;
}

struct PersistentArgs {
    ManifoldSoA m;
    BodySoA b;
    JointSoA j;
    StepParams p;
    const int* colourOffsets;  // manifold slots, colours + 1 entries
    const int* jointOffsets;   // joint slots, colours + 1 entries
    int colours;
    uint32_t flags;
    unsigned int* counter;
    unsigned int* generation;
    int* err;
    unsigned long long* stamps;  // globaltimer at solve start and solve end (block 0)
};

__device__ __forceinline__ unsigned long long GlobalTimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <bool kAdded>
__global__ void k_persistent(PersistentArgs a) {
    unsigned int localGen = *(volatile unsigned int*)a.generation;
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    volatile int* err = a.err;
    __syncthreads();
    // The refresh reads poses only and the force update writes velocities and
    // inertia only, so the two share one phase.
    if (a.flags & (BEPUGPU_STEP_REFRESH_CONTACTS | kStartStages)) {
        if (a.flags & BEPUGPU_STEP_REFRESH_CONTACTS)
            for (int s = tid; s < a.m.count; s += stride) RefreshManifold(a.m, a.b, s, a.p);
        if (a.flags & kStartStages)
            for (int i = tid; i < a.b.count; i += stride)
                if (!OwnedByGroup(a.b, i)) StartBodyStep(a.b, i, a.p, a.flags);
        if (!GridBarrier(a.counter, a.generation, localGen, err)) return;
    }
    if (a.flags & BEPUGPU_STEP_SOLVE) {
        for (int s = tid; s < a.j.count; s += stride) PrestepJoint<kAdded>(a.j, a.b, s, a.p);
        for (int s = tid; s < a.m.count; s += stride) PrestepManifold(a.m, a.b, s, a.p);
        if (!GridBarrier(a.counter, a.generation, localGen, err)) return;
        for (int c = 0; c < a.colours; c++) {
            if (a.j.count)
                for (int s = a.jointOffsets[c] + tid; s < a.jointOffsets[c + 1]; s += stride) WarmJointSlot<kAdded>(a.j, a.b, s);
            for (int s = a.colourOffsets[c] + tid; s < a.colourOffsets[c + 1]; s += stride) WarmSlot(a.m, a.b, s);
            if (!GridBarrier(a.counter, a.generation, localGen, err)) return;
        }
        if (tid == 0) a.stamps[0] = GlobalTimer();
        for (int it = 0; it < a.p.iterationLimit; it++)
            for (int c = 0; c < a.colours; c++) {
                if (a.j.count)
                    for (int s = a.jointOffsets[c] + tid; s < a.jointOffsets[c + 1]; s += stride)
                        SolveJointSlot<kAdded>(a.j, a.b, s, a.p);
                for (int s = a.colourOffsets[c] + tid; s < a.colourOffsets[c + 1]; s += stride)
                    SolveSlot(a.m, a.b, s, a.p);
                if (!GridBarrier(a.counter, a.generation, localGen, err)) return;
            }
        if (tid == 0) a.stamps[1] = GlobalTimer();
    }
    if (a.flags & BEPUGPU_STEP_POSITIONS) {
        for (int i = tid; i < a.b.count; i += stride)
            if (!OwnedByGroup(a.b, i)) PositionUpdateBody(a.b, i, a.p);
    }
}


// Census before a solve sweep: active manifolds of the sweep and their
// algorithmic bytes 76*d + 136 + 48*c.
__global__ void k_census(ManifoldSoA m, int begin, int end, unsigned long long* acc) {
    int s = begin + blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long bytes = 0, visits = 0, contacts = 0;
    if (s < end) {
        uint2 st = m.state[s];
        if (st.x & kGroupActive) {
            int c = m.head[s].z & 0xff;
            int d = ((st.x & kDynA) ? 1 : 0) + ((st.x & kDynB) ? 1 : 0);
            bytes = 76ull * d + 136ull + 48ull * c;
            visits = 1;
            contacts = (unsigned long long)c;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        bytes += __shfl_down_sync(0xffffffffu, bytes, o);
        visits += __shfl_down_sync(0xffffffffu, visits, o);
        contacts += __shfl_down_sync(0xffffffffu, contacts, o);
    }
    if ((threadIdx.x & 31) == 0 && visits) {
        atomicAdd(acc, bytes);
        atomicAdd(acc + 1, visits);
        atomicAdd(acc + 2, contacts);
    }
}

// ------------------------------------------------------------------ host side --
static inline int Blocks(int n, int t) { return (n + t - 1) / t; }

void Context::SetError(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    lastError = buf;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            ctx->SetError("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return BEPUGPU_CUDA_ERROR;                                                        \
        }                                                                                     \
    } while (0)

static size_t Align(size_t x) { return (x + 255) & ~(size_t)255; }

Scene::~Scene() {
    if (graphExec) cudaGraphExecDestroy(graphExec);
    if ((arena || staging) && stream) cudaStreamSynchronize(stream);  // no work reads the blocks any more
    if (heap) {
        heap->Free(arena);
        heap->Free(staging);
    }
    if (spillHost && !spillHostBorrowed) cudaFreeHost(spillHost);
    if (evSpill) cudaEventDestroy(evSpill);
    if (evRestore) cudaEventDestroy(evRestore);
    if (counter) cudaFree(counter);
    if (evStart) cudaEventDestroy(evStart);
    if (evStop) cudaEventDestroy(evStop);
    for (auto e : evPhase)
        if (e) cudaEventDestroy(e);
    for (auto e : evGroup)
        if (e) cudaEventDestroy(e);
    ReleaseBroadPhase(this);
    ReleaseIslands(this);
    ReleasePairs(this);
    if (stream) cudaStreamDestroy(stream);
}

StepParams MakeParams(const bepugpu_settings& s, float dt) {
    StepParams p;
    p.dt = dt;
    p.updateRate = 1 / dt;
    p.gravityDt[0] = s.gravity[0] * dt;
    p.gravityDt[1] = s.gravity[1] * dt;
    p.gravityDt[2] = s.gravity[2] * dt;
    p.iterationLimit = s.iteration_limit < 0 ? 0 : s.iteration_limit;
    p.maximumIterationCount = s.maximum_iteration_count;
    p.minimumIterationCount = s.minimum_iteration_count;
    p.minimumImpulse = s.minimum_impulse;
    p.softness = s.softness;
    p.recoveryStiffness = s.penetration_recovery_stiffness;
    p.maxRecoverySpeed = s.maximum_penetration_recovery_speed;
    p.staticThreshold = s.static_friction_velocity_threshold;
    p.twistFactor = s.twist_friction_factor;
    p.bounceThreshold = s.bounciness_velocity_threshold;
    p.allowedPenetration = s.allowed_penetration;
    p.invalidationLengthSquared = s.contact_invalidation_length_squared;
    p.maximumContactDistance = s.maximum_contact_distance;
    p.useStabilization = s.use_stabilization != 0 ? 1 : 0;
    p.velocityLowerLimit = s.velocity_lower_limit;
    p.velocityLowerLimitSquared = s.velocity_lower_limit * s.velocity_lower_limit;
    p.lowVelocityTimeMinimum = s.low_velocity_time_minimum;
    return p;
}

// (float)Math.Pow(MathHelper.Clamp(1 - d, 0, 1), dt) (EntityBase.cs:943,952),
// computed on the host in double like System.Math.Pow.
static float DampingFactor(float d, float dt) {
    float c = 1 - d;
    c = c < 0 ? 0 : (c > 1 ? 1 : c);
    return (float)std::pow((double)c, (double)dt);
}

bepugpu_status Scene::RefreshDamping(Context* ctx, float dt) {
    if (!dampDirty && dt == dampDt) return BEPUGPU_OK;
    int n = b.count;
    float lastD = NAN, lastF = 0, lastA = NAN, lastG = 0;
    for (int i = 0; i < n; i++) {
        float ld = hostLinDamp[i], ad = hostAngDamp[i];
        float lin = ld + 0.f, ang = ad + 0.f;
        uint32_t flags = (lin > 0 ? 1u : 0u) | (ang > 0 ? 2u : 0u) |
                         ((size_t)i < hostOwned.size() && hostOwned[i] ? kOwnedByGroup : 0u);
        if (!(ld == lastD)) { lastD = ld; lastF = DampingFactor(lin, dt); }
        if (!(ad == lastA)) { lastA = ad; lastG = DampingFactor(ang, dt); }
        float fbits;
        std::memcpy(&fbits, &flags, 4);
        hostDamp[i] = make_float4(lastF, lastG, hostLocalM33[i], fbits);
    }
    CK(cudaMemcpyAsync(b.damp, hostDamp.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, stream));
    dampDirty = false;
    dampDt = dt;
    return BEPUGPU_OK;
}

bepugpu_status Scene::Allocate(Context* ctx, uint32_t nb, uint32_t nm, uint32_t nj) {
    maxBodies = nb; maxManifolds = nm; maxJoints = nj;
    size_t B = nb ? nb : 1, M = nm ? nm : 1, J = nj ? nj : 1;
    size_t bytes = 0;
    auto take = [&](size_t n) { size_t o = bytes; bytes += Align(n); return o; };
    ArenaLayout& L = layout;
    L.pos = take(16 * B); L.quat = take(16 * B); L.vlin = take(16 * B); L.vang = take(16 * B);
    L.inv0 = take(16 * B); L.inv1 = take(16 * B); L.loc0 = take(16 * B); L.loc1 = take(16 * B);
    L.damp = take(16 * B); L.m33 = take(4 * B); L.act = take(16 * B); L.rawDamp = take(8 * B);
    L.head = take(16 * M); L.cpos = take(64 * M); L.cnrm = take(64 * M); L.offA = take(64 * M);
    L.offB = take(64 * M); L.mat = take(16 * M); L.pen = take(16 * M); L.fric = take(16 * M);
    L.axis = take(16 * M); L.pj0 = take(64 * M); L.pj1 = take(64 * M); L.pj2 = take(64 * M);
    L.s0 = take(16 * M); L.s1 = take(16 * M); L.s3 = take(16 * M); L.s4 = take(16 * M); L.s5 = take(16 * M);
    L.s6 = take(16 * M); L.s7 = take(16 * M); L.lev = take(16 * M);
    L.cfr = take(64 * M); L.cfa = take(64 * M); L.cfb = take(64 * M); L.state = take(8 * M);
    L.slot = take(4 * M); L.offs = take(4 * (M + J + 2));
    L.jhead = take(16 * J); L.jlanes = take(16 * (size_t)kJointLanes * J); L.jstate = take(8 * J);
    L.joffs = take(4 * (M + J + 2));
    // a group holds at least one manifold or joint: at most M + J groups
    L.groups = take(sizeof(GroupDesc) * (M + J)); L.groupBodies = take(4 * B); L.groupRefs = take(8 * M);
    // colour offset tables of groups: cCount + 1 entries a group, and a group's
    // colours are at most its members, so 2 (M + J) + 2 entries suffice
    L.groupOffsets = take(4 * (2 * (M + J) + 2)); L.sweepBodies = take(4 * B);
    L.groupJointRefs = take(8 * J); L.groupJointOffsets = take(4 * (2 * (M + J) + 2));
    L.bodyRecords = take(sizeof(bepugpu_body) * B);
    L.shape = take(16 * B); L.genSlots = take(4 * M);
    arenaBytes = bytes;
    // The arena and the staging buffer are blocks of the context's heap, like
    // the ones a restore takes after a spill.
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    cudaError_t e = heap->Alloc(bytes, &arena);
    if (e != cudaSuccess) {
        arena = nullptr;
        ctx->SetError("scene arena of %zu bytes: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? BEPUGPU_OUT_OF_MEMORY : BEPUGPU_CUDA_ERROR;
    }
    b.count = 0;
    m.count = 0;
    m.capacity = (int)M;
    j.count = 0;
    j.capacity = (int)J;
    Rebase();
    CK(cudaMemsetAsync(arena, 0, bytes, stream));
    // body records, then manifold records: bepugpu_step_host stages both at once
    stagingManifoldsAt = Align(sizeof(bepugpu_body) * B);
    stagingBytes = stagingManifoldsAt + sizeof(bepugpu_manifold) * M;
    CK(heap->Alloc(stagingBytes, &staging));
    CK(cudaStreamSynchronize(stream));
    CK(cudaMalloc(&counter, kScratchBytes));
    CK(cudaMemset(counter, 0, kScratchBytes));
    CK(cudaEventCreate(&evStart));
    CK(cudaEventCreate(&evStop));
    for (auto& e : evPhase) CK(cudaEventCreate(&e));
    for (auto& e : evGroup) CK(cudaEventCreate(&e));
    return BEPUGPU_OK;
}

// Every device pointer of the scene from the arena base and the layout.
void Scene::Rebase() {
    char* base = (char*)arena;
    const ArenaLayout& L = layout;
    b.pos = (float4*)(base + L.pos); b.quat = (float4*)(base + L.quat); b.vlin = (float4*)(base + L.vlin);
    b.vang = (float4*)(base + L.vang); b.inv0 = (float4*)(base + L.inv0); b.inv1 = (float4*)(base + L.inv1);
    b.loc0 = (float4*)(base + L.loc0); b.loc1 = (float4*)(base + L.loc1); b.damp = (float4*)(base + L.damp);
    b.act = (float4*)(base + L.act); b.rawDamp = (float2*)(base + L.rawDamp);
    ApplyIslandViews(this);
    localM33 = (float*)(base + L.m33);
    m.head = (int4*)(base + L.head); m.cpos = (float4*)(base + L.cpos); m.cnrm = (float4*)(base + L.cnrm);
    m.offA = (float4*)(base + L.offA); m.offB = (float4*)(base + L.offB); m.mat = (float4*)(base + L.mat);
    m.penacc = (float4*)(base + L.pen); m.fricacc = (float4*)(base + L.fric); m.saxis = (float4*)(base + L.axis);
    m.pj0 = (float4*)(base + L.pj0); m.pj1 = (float4*)(base + L.pj1); m.pj2 = (float4*)(base + L.pj2);
    m.s0 = (float4*)(base + L.s0); m.s1 = (float4*)(base + L.s1); m.s3 = (float4*)(base + L.s3);
    m.s4 = (float4*)(base + L.s4); m.s5 = (float4*)(base + L.s5); m.s6 = (float4*)(base + L.s6);
    m.s7 = (float4*)(base + L.s7); m.lever = (float4*)(base + L.lev); m.state = (uint2*)(base + L.state);
    m.cfr = (float4*)(base + L.cfr); m.cfa = (float4*)(base + L.cfa); m.cfb = (float4*)(base + L.cfb);
    slotOf = (int32_t*)(base + L.slot);
    colourOffsetsDev = (int32_t*)(base + L.offs);
    groupDescDev = (GroupDesc*)(base + L.groups);
    groupBodiesDev = (int32_t*)(base + L.groupBodies);
    groupRefsDev = (int2*)(base + L.groupRefs);
    groupColourOffsetsDev = (int32_t*)(base + L.groupOffsets);
    sweepBodiesDev = (int32_t*)(base + L.sweepBodies);
    groupJointRefsDev = (int2*)(base + L.groupJointRefs);
    groupJointColourOffsetsDev = (int32_t*)(base + L.groupJointOffsets);
    j.head = (int4*)(base + L.jhead);
    j.lanes = (float4*)(base + L.jlanes);
    j.state = (uint2*)(base + L.jstate);
    jointOffsetsDev = (int32_t*)(base + L.joffs);
    bodyRecords = (bepugpu_body*)(base + L.bodyRecords);
    shape = (float4*)(base + L.shape);
    genSlotsDev = (int32_t*)(base + L.genSlots);
}

// Moves the arena to pinned host memory and gives the scene's heap blocks
// back (all of its device memory but the 1 KiB scratch block).  The scene's
// step graph is dropped: it holds device addresses.
// Neither call synchronises the device with other scenes' work, and without
// `wait` neither blocks: the spill's copy is ordered on the scene's stream and
// marked by evSpill, and its blocks become reusable once that copy is done; a
// restore takes blocks from the heap, waits for the mark on the stream it is
// given, copies there, and the scene's stream waits for the copy (evRestore).  `host` (optional) is a pinned buffer of arenaBytes
// for the first spill, owned by the caller.
bepugpu_status Scene::Spill(Context* ctx, bool wait, void* host) {
    if (!arena) return BEPUGPU_OK;
    if (!spillHost) {
        if (host) {
            spillHost = host;
            spillHostBorrowed = true;
        } else {
            CK(cudaMallocHost(&spillHost, arenaBytes));
            spillHostBorrowed = false;
        }
    }
    if (!evSpill) CK(cudaEventCreateWithFlags(&evSpill, cudaEventDisableTiming));
    CK(cudaMemcpyAsync(spillHost, arena, arenaBytes, cudaMemcpyDeviceToHost, stream));
    CK(heap->FreeAfter(arena, stream));
    arena = nullptr;
    if (staging) CK(heap->FreeAfter(staging, stream));
    staging = nullptr;
    CK(cudaEventRecord(evSpill, stream));
    if (wait) CK(cudaStreamSynchronize(stream));
    if (graphExec) cudaGraphExecDestroy(graphExec);
    graphExec = nullptr;
    asyncPending = false;
    return BEPUGPU_OK;
}

bepugpu_status Scene::Restore(Context* ctx, cudaStream_t q, bool wait) {
    if (arena) return BEPUGPU_OK;
    if (!q) q = stream;
    cudaError_t e = heap->Alloc(arenaBytes, &arena);
    if (e == cudaSuccess) {
        e = heap->Alloc(stagingBytes, &staging);
        if (e != cudaSuccess) {
            heap->Free(arena);
            arena = nullptr;
            staging = nullptr;
        }
    } else {
        arena = nullptr;
    }
    if (e != cudaSuccess) {
        ctx->SetError("scene restore of %zu bytes: %s", arenaBytes + stagingBytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? BEPUGPU_OUT_OF_MEMORY : BEPUGPU_CUDA_ERROR;
    }
    Rebase();
    if (evSpill) CK(cudaStreamWaitEvent(q, evSpill, 0));
    CK(cudaMemcpyAsync(arena, spillHost, arenaBytes, cudaMemcpyHostToDevice, q));
    if (q != stream) {
        if (!evRestore) CK(cudaEventCreateWithFlags(&evRestore, cudaEventDisableTiming));
        CK(cudaEventRecord(evRestore, q));
        CK(cudaStreamWaitEvent(stream, evRestore, 0));
    }
    if (wait) CK(cudaStreamSynchronize(q));
    version++;
    return BEPUGPU_OK;
}

// Gives up a borrowed spill buffer (its owner frees it); the next spill takes
// another.  Only while resident: a spilled scene's data lives there.
void Scene::DropBorrowedSpillBuffer() {
    if (arena && spillHostBorrowed) {
        spillHost = nullptr;
        spillHostBorrowed = false;
    }
}

// A spilled scene whose borrowed buffer's owner goes away moves its data to a
// pinned buffer of its own.  False if that allocation fails.
bool Scene::OwnSpillBuffer() {
    if (arena || !spillHostBorrowed) return true;
    if (stream) cudaStreamSynchronize(stream);  // the spill copy has landed
    void* own = nullptr;
    if (cudaMallocHost(&own, arenaBytes) != cudaSuccess) return false;
    std::memcpy(own, spillHost, arenaBytes);
    spillHost = own;
    spillHostBorrowed = false;
    return true;
}

// The bodies the sweep path's body stages handle once groups exist: every
// body no group kernel steps.
bepugpu_status Scene::RebuildSweepBodies(Context* ctx) {
    std::vector<int32_t> list;
    list.reserve(b.count);
    sweepDynamicCount = 0;
    for (int32_t e = 0; e < b.count; e++)
        if (!((size_t)e < hostOwned.size() && hostOwned[e])) {
            list.push_back(e);
            if ((size_t)e < hostDynamic.size() && hostDynamic[e]) sweepDynamicCount++;
        }
    sweepBodyCount = (uint32_t)list.size();
    if (!list.empty())
        CK(cudaMemcpyAsync(sweepBodiesDev, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice,
                           stream));
    CK(cudaStreamSynchronize(stream));
    version++;
    return BEPUGPU_OK;
}

// A sweep launch that may start while the sweep before it finishes: the
// kernel waits for it (griddepcontrol.wait) before reading its results.
template <typename... KArgs, typename... Args>
static cudaError_t LaunchAfterSweep(void (*kernel)(KArgs...), int grid, int block, cudaStream_t q, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.stream = q;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

bepugpu_status Scene::BuildGraph(Context* ctx, const StepParams& p, uint32_t flags) {
    if (graphExec) { cudaGraphExecDestroy(graphExec); graphExec = nullptr; }
    const int T = 128;
    launchesPerStep = 0;
    const uint32_t requested = flags;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    // DeactivationManager.Update before everything else (Space.cs:502): the
    // narrow phase, the refresher and the body stages read the islands' state.
    graphWakes = islands && IslandWakesPossible(this);
    if (islands && (flags & BEPUGPU_STEP_DEACTIVATION)) {
        cudaError_t ie = LaunchIslandStage(this, p, ctx->settings.maximum_deactivation_attempts_per_frame, stream);
        if (ie != cudaSuccess) {
            cudaGraph_t dropped;
            cudaStreamEndCapture(stream, &dropped);
            if (dropped) cudaGraphDestroy(dropped);
            ctx->SetError("island stage launch: %s", cudaGetErrorString(ie));
            return BEPUGPU_CUDA_ERROR;
        }
    }
    flags = StageFlags(flags);
    // The narrow phase first: it rewrites the GENERATED manifolds' contacts
    // from the poses the rest of the step starts from.
    if ((flags & BEPUGPU_STEP_COLLIDE) && generatedCount) {
        cudaError_t ce = LaunchCollide(this, p, stream);
        if (ce != cudaSuccess) {
            cudaGraph_t dropped;
            cudaStreamEndCapture(stream, &dropped);
            if (dropped) cudaGraphDestroy(dropped);
            ctx->SetError("narrow phase launch: %s", cudaGetErrorString(ce));
            return BEPUGPU_CUDA_ERROR;
        }
        launchesPerStep++;
    }
    // Island groups next: one CTA per group runs the group's whole step.
    // They share only kinematic bodies (read only) with the sweep path, whose
    // position update of moving kinematic bodies therefore has to follow.
    CK(cudaEventRecordWithFlags(evGroup[0], stream, cudaEventRecordExternal));
    if (!groupPlan.groups.empty()) {
        int groupLaunches = 0;
        bepugpu_status gs = LaunchGroups(ctx, this, p, flags, false, &groupLaunches);
        if (gs != BEPUGPU_OK) {
            cudaGraph_t dropped;
            cudaStreamEndCapture(stream, &dropped);
            if (dropped) cudaGraphDestroy(dropped);
            return gs;
        }
        launchesPerStep += groupLaunches;
    }
    CK(cudaEventRecordWithFlags(evGroup[1], stream, cudaEventRecordExternal));
    const ManifoldSoA ms = SweepManifolds();
    const int colours = SweepColours();
    int nm = ms.count, nb = b.count;
    // A scene whose whole step is island groups has nothing left for the sweep
    // path: no sweep manifolds or joints, no dynamic body outside the groups,
    // no moving kinematic body.  Its graph is the group launch alone.
    phaseEvents = !SweepEmpty();
    graphTail = false;
    if (!phaseEvents) {
        // the kinematic bodies' candidacy and position stages, while they change anything
        if (kin.Needed(flags) && sweepBodyCount) {
            k_kinematic_tail<<<Blocks((int)sweepBodyCount, T), T, 0, stream>>>(b, p, sweepBodiesDev,
                                                                               (int)sweepBodyCount, flags);
            launchesPerStep++;
            graphTail = true;
        }
        cudaGraph_t graph;
        cudaError_t e = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess) {
            ctx->SetError("graph capture: %s", cudaGetErrorString(e));
            return BEPUGPU_CUDA_ERROR;
        }
        e = cudaGraphInstantiate(&graphExec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            graphExec = nullptr;
            ctx->SetError("graph instantiate: %s", cudaGetErrorString(e));
            return BEPUGPU_CUDA_ERROR;
        }
        graphDt = p.dt;
        graphFlags = requested;
        graphVersion = version;
        graphIterations = p.iterationLimit;
        return BEPUGPU_OK;
    }
    // Phase events become event-record nodes of the graph: their elapsed times
    // are the device time of each phase of every launched step.
    CK(cudaEventRecordWithFlags(evPhase[0], stream, cudaEventRecordExternal));
    bool refresh = (flags & BEPUGPU_STEP_REFRESH_CONTACTS) && nm, force = (flags & kStartStages) && nb;
    const bool listed = !groupPlan.groups.empty();  // body stages over the sweep path's own bodies
    const int nl = (int)sweepBodyCount;
    if (listed) {
        if ((refresh || force) && nm + nl > 0) {
            k_refresh_force_list<<<Blocks(nm + nl, T), T, 0, stream>>>(ms, b, p, sweepBodiesDev, nl, flags);
            launchesPerStep++;
        }
    } else if (refresh && force) {
        k_refresh_force<<<Blocks(nm + nb, T), T, 0, stream>>>(ms, b, p, flags); launchesPerStep++;
    } else if (refresh) {
        k_refresh<<<Blocks(nm, T), T, 0, stream>>>(ms, b, p); launchesPerStep++;
    } else if (force) {
        ManifoldSoA none = ms;
        none.count = 0;
        k_refresh_force<<<Blocks(nb, T), T, 0, stream>>>(none, b, p, flags & kStartStages); launchesPerStep++;
    }
    CK(cudaEventRecordWithFlags(evPhase[1], stream, cudaEventRecordExternal));
    const JointSoA js = SweepJoints();
    const int nj = js.count;
    bool solve = (flags & BEPUGPU_STEP_SOLVE) && (nm || nj);
    const auto prestepMixed = addedJointTypes ? k_prestep_mixed<true> : k_prestep_mixed<false>;
    const auto warmMixed = addedJointTypes ? k_warm_mixed<true> : k_warm_mixed<false>;
    const auto solveMixed = addedJointTypes ? k_solve_mixed<true> : k_solve_mixed<false>;
    if (solve) {
        if (nj) prestepMixed<<<Blocks(nm + nj, T), T, 0, stream>>>(ms, b, js, p);
        else k_prestep<<<Blocks(nm, T), T, 0, stream>>>(ms, b, p);
        launchesPerStep++;
    }
    CK(cudaEventRecordWithFlags(evPhase[2], stream, cudaEventRecordExternal));
    if (solve) {
        for (int c = 0; c < colours; c++) {
            int b0 = manifoldOffsets[c], b1 = manifoldOffsets[c + 1];
            int j0 = nj ? jointOffsets[c] : 0, j1 = nj ? jointOffsets[c + 1] : 0;
            if (j1 > j0) {
                warmMixed<<<Blocks(b1 - b0 + j1 - j0, T), T, 0, stream>>>(ms, b, js, b0, b1, j0, j1);
                launchesPerStep++;
            } else if (b1 > b0) {
                k_warm<<<Blocks(b1 - b0, T), T, 0, stream>>>(ms, b, b0, b1);
                launchesPerStep++;
            }
        }
    }
    CK(cudaEventRecordWithFlags(evPhase[3], stream, cudaEventRecordExternal));
    if (solve) {
        for (int it = 0; it < p.iterationLimit; it++)
            for (int c = 0; c < colours; c++) {
                int b0 = manifoldOffsets[c], b1 = manifoldOffsets[c + 1];
                int j0 = nj ? jointOffsets[c] : 0, j1 = nj ? jointOffsets[c + 1] : 0;
                if (j1 > j0) {
                    CK(LaunchAfterSweep(solveMixed, Blocks(b1 - b0 + j1 - j0, T), T, stream, ms, b, js, p, b0, b1, j0, j1));
                    launchesPerStep++;
                } else if (b1 > b0) {
                    CK(LaunchAfterSweep(k_solve, Blocks(b1 - b0, T), T, stream, ms, b, p, b0, b1));
                    launchesPerStep++;
                }
            }
    }
    CK(cudaEventRecordWithFlags(evPhase[4], stream, cudaEventRecordExternal));
    if (listed) {
        if ((flags & BEPUGPU_STEP_POSITIONS) && nl > 0) {
            k_position_list<<<Blocks(nl, T), T, 0, stream>>>(b, p, sweepBodiesDev, nl); launchesPerStep++;
        }
    } else if ((flags & BEPUGPU_STEP_POSITIONS) && nb) {
        k_position<<<Blocks(nb, T), T, 0, stream>>>(b, p); launchesPerStep++;
    }
    CK(cudaEventRecordWithFlags(evPhase[5], stream, cudaEventRecordExternal));
    cudaGraph_t graph;
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
    if (e != cudaSuccess) {
        ctx->SetError("graph capture: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    e = cudaGraphInstantiate(&graphExec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        graphExec = nullptr;
        ctx->SetError("graph instantiate: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    graphDt = p.dt;
    graphFlags = requested;
    graphVersion = version;
    graphIterations = p.iterationLimit;
    return BEPUGPU_OK;
}

bepugpu_status Scene::RunPersistent(Context* ctx, const StepParams& p, uint32_t flags) {
    const int T = 256;
    void* kernel = addedJointTypes ? (void*)k_persistent<true> : (void*)k_persistent<false>;
    if (persistentBlocks == 0 || persistentAdded != addedJointTypes) {
        int perSm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, T, 0));
        if (perSm < 1) {
            ctx->SetError("persistent kernel cannot be resident");
            return BEPUGPU_CUDA_ERROR;
        }
        persistentBlocks = std::min(perSm, persistentBlocksPerSm) * ctx->smCount;
        persistentAdded = addedJointTypes;
    }
    launchesPerStep = 0;
    if (islands && (flags & BEPUGPU_STEP_DEACTIVATION))
        CK(LaunchIslandStage(this, p, ctx->settings.maximum_deactivation_attempts_per_frame, stream));
    flags = StageFlags(flags);
    if ((flags & BEPUGPU_STEP_COLLIDE) && generatedCount) {
        CK(LaunchCollide(this, p, stream));
        launchesPerStep++;
    }
    CK(cudaEventRecord(evGroup[0], stream));
    if (!groupPlan.groups.empty()) {
        int groupLaunches = 0;
        bepugpu_status gs = LaunchGroups(ctx, this, p, flags, false, &groupLaunches);
        if (gs != BEPUGPU_OK) return gs;
        launchesPerStep += groupLaunches;
    }
    CK(cudaEventRecord(evGroup[1], stream));
    PersistentArgs a;
    a.m = SweepManifolds(); a.b = b; a.j = SweepJoints(); a.p = p;
    a.colourOffsets = colourOffsetsDev;
    a.jointOffsets = jointOffsetsDev;
    a.colours = SweepColours();
    a.flags = flags;
    a.counter = BarrierCounter();
    a.generation = BarrierGeneration();
    a.err = ErrorWord();
    a.stamps = Stamps();
    // A barrier abandoned by an earlier timed-out launch must not count here.
    CK(cudaMemsetAsync(BarrierCounter(), 0, sizeof(unsigned int), stream));
    CK(cudaMemsetAsync(ErrorWord(), 0, sizeof(int), stream));
    void* args[] = {&a};
    CK(cudaLaunchCooperativeKernel(kernel, dim3(persistentBlocks), dim3(T), args, 0, stream));
    launchesPerStep++;
    return BEPUGPU_OK;
}

bepugpu_status Scene::Step(Context* ctx, float dt, uint32_t flags) {
    NvtxRange range("bepugpu_step");
    if (!(dt > 0) || !std::isfinite(dt)) {
        ctx->SetError("dt must be positive and finite");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (maxBodyReferenced >= b.count) {
        ctx->SetError("constraints reference body %d but the scene holds %d bodies", maxBodyReferenced, b.count);
        return BEPUGPU_INVALID_OPERATION;
    }
    if (planStale) {
        ctx->SetError("bodies changed between dynamic and kinematic: upload the constraints again to recolour");
        return BEPUGPU_INVALID_OPERATION;
    }
    if (generatedCount && (flags & BEPUGPU_STEP_COLLIDE) && hostShapes.size() != (size_t)b.count) {
        ctx->SetError("the body count changed since the shapes were uploaded: upload the shapes again");
        return BEPUGPU_INVALID_OPERATION;
    }
    bepugpu_status st = RefreshDamping(ctx, dt);
    if (st != BEPUGPU_OK) return st;
    StepParams p = MakeParams(ctx->settings, dt);
    CK(cudaEventRecord(evStart, stream));
    if (mode == BEPUGPU_MODE_PERSISTENT) {
        st = RunPersistent(ctx, p, flags);
        if (st != BEPUGPU_OK) return st;
    } else {
        const bool tail = SweepEmpty() && kin.Needed(StageFlags(flags)) && sweepBodyCount;
        const bool wakes = islands && IslandWakesPossible(this);
        if (!graphExec || graphDt != dt || graphFlags != flags || graphVersion != version ||
            graphIterations != p.iterationLimit || graphTail != tail || graphWakes != wakes) {
            st = BuildGraph(ctx, p, flags);
            if (st != BEPUGPU_OK) return st;
        }
        CK(cudaGraphLaunch(graphExec, stream));
    }
    CK(cudaEventRecord(evStop, stream));
    kin.Advance(flags);
    stepped = true;
    asyncPending = true;
    return BEPUGPU_OK;
}

}  // namespace bepugpu

namespace bepugpu {
// Copies `n` records to the device, runs `check` over them and returns the
// offending index (-1 when none) and the flag word.
template <class Launch>
bepugpu_status CheckRecords(Context* ctx, Scene* s, const void* rec, size_t bytes, Launch launch, int& bad,
                                   int& flag) {
    int* check = s->CheckWords();
    CK(cudaMemcpyAsync(s->staging, rec, bytes, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(check, 0x7f, sizeof(int), s->stream));
    CK(cudaMemsetAsync(check + 1, 0, sizeof(int), s->stream));
    launch(check);
    CK(cudaGetLastError());
    int h[2];
    CK(cudaMemcpyAsync(h, check, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    bad = h[0] == 0x7f7f7f7f ? -1 : h[0];
    flag = h[1];
    return BEPUGPU_OK;
}

}  // namespace bepugpu

// ================================================================== C ABI ==
using namespace bepugpu;

#define CTX_CHECK(ctx)                               \
    do {                                             \
        if (!(ctx)) return BEPUGPU_INVALID_ARGUMENT; \
        cudaSetDevice((ctx)->device);                \
    } while (0)

// A scene of this context that no server owns (a served scene's device
// state belongs to the server's worker until it is released).
Scene* bepugpu::FindScene(Context* ctx, int32_t id) {
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) {
        ctx->SetError("scene %d does not exist", id);
        return nullptr;
    }
    if (it->second->server) {
        ctx->SetError("scene %d is served; release it from its server first", id);
        return nullptr;
    }
    return it->second.get();
}
bepugpu_status bepugpu::SceneMissing(Context* ctx, int32_t id) {
    auto it = ctx->scenes.find(id);
    return it != ctx->scenes.end() && it->second->server ? BEPUGPU_INVALID_OPERATION : BEPUGPU_NOT_FOUND;
}

extern "C" {

int32_t bepugpu_abi_version(void) { return BEPUGPU_ABI_VERSION; }

uint32_t bepugpu_record_size(int32_t kind) {
    switch (kind) {
        case 0: return sizeof(bepugpu_settings);
        case 1: return sizeof(bepugpu_body);
        case 2: return sizeof(bepugpu_contact);
        case 3: return sizeof(bepugpu_manifold);
        case 4: return sizeof(bepugpu_joint);
        case 5: return sizeof(bepugpu_body_state);
        case 6: return sizeof(bepugpu_manifold_state);
        default: return 0;
    }
}

void bepugpu_default_settings(bepugpu_settings* s) {
    std::memset(s, 0, sizeof(*s));
    s->gravity[0] = 0.f; s->gravity[1] = -9.81f; s->gravity[2] = 0.f;
    s->iteration_limit = 10;
    s->minimum_impulse = .001f;
    s->minimum_iteration_count = 1;
    s->maximum_iteration_count = 0x7fffffff;
    s->softness = .001f;
    s->penetration_recovery_stiffness = .2f;
    s->maximum_penetration_recovery_speed = 2.f;
    s->static_friction_velocity_threshold = .2f;
    s->twist_friction_factor = 1.f;
    s->bounciness_velocity_threshold = 1.f;
    s->allowed_penetration = .01f;
    s->contact_invalidation_length_squared = .01f;
    s->maximum_contact_distance = .1f;
    s->use_stabilization = 1;
    s->velocity_lower_limit = .26f;
    s->low_velocity_time_minimum = 1.f;
    s->maximum_deactivation_attempts_per_frame = 100;
}

static bepugpu_status ValidateSettings(Context* ctx, const bepugpu_settings* s) {
    if (s->iteration_limit < 0 || s->iteration_limit > 65535) {
        ctx->SetError("iteration_limit must be in [0, 65535]");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->minimum_iteration_count < 0 || s->minimum_iteration_count > 14) {
        ctx->SetError("minimum_iteration_count must be in [0, 14]");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    // DeactivationManager.VelocityLowerLimit clamps to >= 0 and LowVelocityTimeMinimum
    // throws ArgumentException for values <= 0 (DeactivationManager.cs:36,54-55).
    if (!(s->velocity_lower_limit >= 0) || !std::isfinite(s->velocity_lower_limit)) {
        ctx->SetError("velocity_lower_limit must be finite and >= 0");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (!(s->low_velocity_time_minimum > 0)) {
        ctx->SetError("low_velocity_time_minimum must be positive");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->maximum_deactivation_attempts_per_frame < 0) {
        ctx->SetError("maximum_deactivation_attempts_per_frame must be >= 0");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_create(int32_t device, const bepugpu_settings* settings, bepugpu_context** out) {
    if (!out) return BEPUGPU_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return BEPUGPU_CUDA_ERROR;
    auto* ctx = new Context();
    ctx->device = device;
    ctx->heap = std::make_unique<DeviceHeap>();
    if (settings) ctx->settings = *settings;
    else bepugpu_default_settings(&ctx->settings);
    if (ValidateSettings(ctx, &ctx->settings) != BEPUGPU_OK) { delete ctx; return BEPUGPU_INVALID_ARGUMENT; }
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return BEPUGPU_CUDA_ERROR; }
    cudaDeviceGetAttribute(&ctx->smCount, cudaDevAttrMultiProcessorCount, device);
    *out = reinterpret_cast<bepugpu_context*>(ctx);
    return BEPUGPU_OK;
}

void bepugpu_destroy(bepugpu_context* c) {
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    ShutdownServers(ctx);  // their workers step these scenes
    ctx->batch.reset();
    ctx->scenes.clear();
    delete ctx;
}

bepugpu_status bepugpu_memory_usage(bepugpu_context* c, uint64_t* reserved, uint64_t* in_use) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    if (!reserved || !in_use) return BEPUGPU_INVALID_ARGUMENT;
    *reserved = ctx->heap->Reserved();
    *in_use = ctx->heap->InUse();
    return BEPUGPU_OK;
}

const char* bepugpu_last_error(bepugpu_context* c) {
    auto* ctx = reinterpret_cast<Context*>(c);
    return ctx ? ctx->lastError.c_str() : "null context";
}

bepugpu_status bepugpu_set_settings(bepugpu_context* c, const bepugpu_settings* s) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    if (!s) return BEPUGPU_INVALID_ARGUMENT;
    bepugpu_status st = ValidateSettings(ctx, s);
    if (st != BEPUGPU_OK) return st;
    ctx->settings = *s;
    for (auto& kv : ctx->scenes) kv.second->version++;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_synchronize(bepugpu_context* c) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    CK(cudaDeviceSynchronize());
    for (auto& kv : ctx->scenes) {
        Scene& s = *kv.second;
        if (s.mode == BEPUGPU_MODE_PERSISTENT && s.counter) {
            int err = 0;
            CK(cudaMemcpy(&err, s.ErrorWord(), sizeof(int), cudaMemcpyDeviceToHost));
            if (err) {
                CK(cudaMemset(s.ErrorWord(), 0, sizeof(int)));
                ctx->SetError("persistent step: a grid barrier wait ran out");
                return BEPUGPU_TIMEOUT;
            }
        }
    }
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_scene_create(bepugpu_context* c, uint32_t nb, uint32_t nm, uint32_t nj, int32_t* out) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    if (!out) return BEPUGPU_INVALID_ARGUMENT;
    if (nb > (1u << 30) || nm > (1u << 28) || nj > (1u << 28)) {
        ctx->SetError("scene capacity too large");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    auto s = std::make_unique<Scene>();
    s->heap = ctx->heap.get();
    bepugpu_status st = s->Allocate(ctx, nb, nm, nj);
    if (st != BEPUGPU_OK) return st;
    int32_t id = ctx->nextScene++;
    s->id = id;
    ctx->scenes[id] = std::move(s);
    *out = id;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_scene_destroy(bepugpu_context* c, int32_t id) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    if (!FindScene(ctx, id)) return SceneMissing(ctx, id);
    ctx->scenes.erase(id);
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_upload_bodies(bepugpu_context* c, int32_t id, const bepugpu_body* bodies, uint32_t n) {
    NvtxRange range("bepugpu_upload_bodies");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (n > s->maxBodies || (n && !bodies)) {
        ctx->SetError("body count %u exceeds scene capacity %u", n, s->maxBodies);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->islands || s->pairs) {  // islands and materials are set again for the new bodies
        if (s->asyncPending) CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
        ReleaseIslands(s);
        ReleasePairs(s);
        s->version++;
    }
    s->hostLinDamp.resize(n); s->hostAngDamp.resize(n); s->hostLocalM33.resize(n); s->hostDamp.resize(n);
    bool dynamicChanged = s->hostDynamic.size() != n;
    s->hostDynamic.resize(n);
    s->hostRawDamp.resize(n);
    s->kin.Clear();
    s->hostKinematic.clear();
    for (uint32_t i = 0; i < n; i++) {
        if (!dynamicChanged && s->hostDynamic[i] != (bodies[i].is_dynamic ? 1 : 0)) dynamicChanged = true;
        if (!bodies[i].is_dynamic) {
            s->hostKinematic.push_back((int32_t)i);
            const float* v = bodies[i].linear_velocity;
            const float* w = bodies[i].angular_velocity;
            s->kin.Add(v[0] != 0 || v[1] != 0 || v[2] != 0 || w[0] != 0 || w[1] != 0 || w[2] != 0,
                       bodies[i].activity, bodies[i].previous_velocity, bodies[i].velocity_time_below_limit);
        }
        s->hostRawDamp[i] = make_float2(bodies[i].linear_damping, bodies[i].angular_damping);
        s->hostLinDamp[i] = bodies[i].linear_damping;
        s->hostAngDamp[i] = bodies[i].angular_damping;
        s->hostDynamic[i] = bodies[i].is_dynamic ? 1 : 0;
        s->hostLocalM33[i] = bodies[i].is_dynamic ? bodies[i].local_inverse_inertia[8] : 0.f;
    }
    const bool resized = n != (uint32_t)s->b.count;
    if (resized) s->version++;
    // The colouring and the island groups depend on which bodies are dynamic.
    if (dynamicChanged && (s->m.count || s->jointCount)) s->planStale = true;
    s->b.count = (int)n;
    s->dampDirty = true;
    if (resized && !s->groupPlan.groups.empty()) {
        bepugpu_status lst = s->RebuildSweepBodies(ctx);
        if (lst != BEPUGPU_OK) return lst;
    }
    if (n) {
        CK(cudaMemcpyAsync(s->bodyRecords, bodies, sizeof(bepugpu_body) * n, cudaMemcpyHostToDevice, s->stream));
        k_unpack_bodies<<<Blocks(n, 256), 256, 0, s->stream>>>(s->bodyRecords, (int)n, s->b);
        CK(cudaMemcpyAsync(s->localM33, s->hostLocalM33.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->b.rawDamp, s->hostRawDamp.data(), sizeof(float2) * n, cudaMemcpyHostToDevice,
                           s->stream));
        k_world_inertia<<<Blocks(n, 256), 256, 0, s->stream>>>(s->b, s->localM33);
        CK(cudaGetLastError());
        // The staging buffer and host vectors are reused by the next call: wait.
        CK(cudaStreamSynchronize(s->stream));
    }
    return BEPUGPU_OK;
}

static bepugpu_status UploadManifoldRecords(Context* ctx, Scene* s, const bepugpu_manifold* rec, uint32_t n,
                                            bool staged = false) {
    if (!n) return BEPUGPU_OK;
    if (!staged)
        CK(cudaMemcpyAsync(s->staging, rec, sizeof(bepugpu_manifold) * n, cudaMemcpyHostToDevice, s->stream));
    k_unpack_manifolds<<<Blocks(n, 256), 256, 0, s->stream>>>((const bepugpu_manifold*)s->staging, s->slotOf,
                                                               (int)n, s->m);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_upload_constraints(bepugpu_context* c, int32_t id, const bepugpu_manifold* man, uint32_t nm,
                                          const bepugpu_joint* joints, uint32_t nj) {
    NvtxRange range("bepugpu_upload_constraints");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (nm > s->maxManifolds || nj > s->maxJoints || (nm && !man) || (nj && !joints)) {
        ctx->SetError("constraint counts exceed scene capacity");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->islands) {  // the islands are set again for the new connections
        if (s->asyncPending) CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
        ReleaseIslands(s);
    }
    int nb = s->b.count;
    if (nj) {
        bepugpu_status jst = CheckJointRecords(ctx, joints, nj, nb);
        if (jst != BEPUGPU_OK) return jst;
    }
    std::vector<int32_t> a(nm + nj), bb(nm + nj);
    std::vector<uint8_t> nonConvex(nm), follows(nm + nj, 0);
    for (uint32_t u = 0; u < nj; u++) {
        a[u] = joints[u].body_a;
        bb[u] = joints[u].body_b;
        follows[u] = (joints[u].flags & BEPUGPU_JOINT_GROUP_CONTINUATION) != 0;
    }
    for (uint32_t i = 0; i < nm; i++) {
        a[nj + i] = man[i].body_a;
        bb[nj + i] = man[i].body_b;
        nonConvex[i] = (man[i].flags & BEPUGPU_MANIFOLD_NONCONVEX) != 0;
        if (man[i].contact_count < 0 || man[i].contact_count > 4) {
            ctx->SetError("manifold %u has contact_count %d (0..4 allowed)", i, man[i].contact_count);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (man[i].body_a == man[i].body_b && man[i].body_a >= 0) {
            ctx->SetError("manifold %u connects body %d to itself", i, man[i].body_a);
            return BEPUGPU_INVALID_ARGUMENT;
        }
    }
    if (!ColourSolverList(a.data(), bb.data(), (int32_t)(nm + nj), s->hostDynamic.data(), nb, s->colouring,
                          follows.data())) {
        ctx->SetError("a constraint references a body outside [0, %d)", nb);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    // Manifold and joint slots: the colour-sweep part in colour-major order,
    // then the island groups (groups.cu); the persistent mode keeps everything
    // on the sweep path.
    GroupPolicy pol = s->policy;
    if (s->mode == BEPUGPU_MODE_PERSISTENT) pol.enabled = false;
    // kind of an entry for the slot order inside a colour: a joint's record
    // type, a manifold's nonconvex flag and contact count
    std::vector<int32_t> kind(nm + nj);
    for (uint32_t u = 0; u < nj; u++) kind[u] = joints[u].type;
    for (uint32_t i = 0; i < nm; i++) kind[nj + i] = 64 + (nonConvex[i] ? 8 : 0) + std::max(0, man[i].contact_count);
    PlanGroups(pol, a.data(), bb.data(), s->colouring.colour.data(), (int32_t)nj, (int32_t)nm,
               s->hostDynamic.data(), nb, s->colouring.colours, s->groupPlan, nonConvex.data(), kind.data(),
               follows.data());
    const GroupPlan& plan = s->groupPlan;
    s->manifoldOffsets = plan.globalOffsets;
    s->jointOffsets = plan.jointGlobalOffsets;
    s->hostJointSlotOf = plan.jointSlotOf;
    s->hostOwned.assign(nb, 0);
    for (int32_t e = 0; e < nb && e < (int32_t)plan.localOf.size(); e++) s->hostOwned[e] = plan.localOf[e] >= 0;
    {
        bepugpu_status lst = s->RebuildSweepBodies(ctx);
        if (lst != BEPUGPU_OK) return lst;
    }
    s->dampDirty = true;
    s->planStale = false;
    s->m.count = (int)nm;
    s->jointCount = nj;
    s->version++;
    if (nm) {
        CK(cudaMemcpyAsync(s->slotOf, plan.slotOf.data(), sizeof(int32_t) * nm, cudaMemcpyHostToDevice, s->stream));
    }
    CK(cudaMemcpyAsync(s->colourOffsetsDev, s->manifoldOffsets.data(), sizeof(int32_t) * s->manifoldOffsets.size(),
                       cudaMemcpyHostToDevice, s->stream));
    {
        bepugpu_status gst = s->UploadGroups(ctx);
        if (gst != BEPUGPU_OK) return gst;
    }
    s->hostSlotOf = plan.slotOf;
    s->maxBodyReferenced = -1;
    for (uint32_t u = 0; u < nm + nj; u++) s->maxBodyReferenced = std::max(s->maxBodyReferenced, std::max(a[u], bb[u]));
    {
        bepugpu_status jst = UploadJoints(ctx, s, joints, nj);
        if (jst != BEPUGPU_OK) return jst;
    }
    {
        bepugpu_status gst = PrepareGenerated(ctx, s, man, nm, s->hostSlotOf);
        if (gst != BEPUGPU_OK) return gst;
    }
    return UploadManifoldRecords(ctx, s, man, nm);
}

bepugpu_status bepugpu_update_manifolds(bepugpu_context* c, int32_t id, const bepugpu_manifold* man, uint32_t n) {
    NvtxRange range("bepugpu_update_manifolds");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (n != (uint32_t)s->m.count || (n && !man)) {
        ctx->SetError("update_manifolds needs the %d manifolds of the last upload", s->m.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (!n) return BEPUGPU_OK;
    // The colouring is kept, so every manifold must still join the same bodies:
    // checked on the device against the stored slots before anything changes.
    int bad = -1, flag = 0;
    bepugpu_status st = CheckRecords(ctx, s, man, sizeof(bepugpu_manifold) * n, [&](int* check) {
        k_check_manifold_records<<<Blocks(n, 256), 256, 0, s->stream>>>((const bepugpu_manifold*)s->staging,
                                                                         s->slotOf, (int)n, s->m, check);
    }, bad, flag);
    if (st != BEPUGPU_OK) return st;
    if (bad >= 0) {
        ctx->SetError("manifold %d changed its bodies or its GENERATED or NONCONVEX flag, has a contact count outside "
                      "0..4 or a contact_order that is no permutation; use bepugpu_upload_constraints", bad);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    return UploadManifoldRecords(ctx, s, man, n, true);
}

bepugpu_status bepugpu_step_host(bepugpu_context* c, int32_t id, bepugpu_body* bodies, uint32_t nb,
                                 bepugpu_manifold* man, uint32_t nm, float dt, uint32_t flags) {
    NvtxRange range("bepugpu_step_host");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (nb != (uint32_t)s->b.count || nm != (uint32_t)s->m.count || (nb && !bodies) || (nm && !man)) {
        ctx->SetError("step_host needs the %d bodies and %d manifolds of the last uploads", s->b.count, s->m.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->jointCount) {
        ctx->SetError("step_host takes scenes without joints; use the update, step and download calls");
        return BEPUGPU_INVALID_OPERATION;
    }
    if (!(dt > 0) || !std::isfinite(dt)) {
        ctx->SetError("dt must be positive and finite");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->asyncPending) {  // an earlier step may still read the staging buffer's neighbours
        CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
    }
    // Both record arrays up, both checked on the device; one round trip for
    // the verdict, so nothing changes when a record is refused.
    bepugpu_body* sb = (bepugpu_body*)s->staging;
    bepugpu_manifold* sm = (bepugpu_manifold*)((char*)s->staging + s->stagingManifoldsAt);
    int* check = s->CheckWords();
    if (nb) CK(cudaMemcpyAsync(sb, bodies, sizeof(bepugpu_body) * nb, cudaMemcpyHostToDevice, s->stream));
    if (nm) CK(cudaMemcpyAsync(sm, man, sizeof(bepugpu_manifold) * nm, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(check, 0x7f, sizeof(int), s->stream));
    CK(cudaMemsetAsync(check + 1, 0, sizeof(int), s->stream));
    CK(cudaMemsetAsync(check + 2, 0x7f, sizeof(int), s->stream));
    if (nb) k_check_body_records<<<Blocks(nb, 256), 256, 0, s->stream>>>(sb, s->bodyRecords, (int)nb, check);
    if (nm) k_check_manifold_records<<<Blocks(nm, 256), 256, 0, s->stream>>>(sm, s->slotOf, (int)nm, s->m, check + 2);
    CK(cudaGetLastError());
    int h[3];
    CK(cudaMemcpyAsync(h, check, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (h[0] != 0x7f7f7f7f) {
        ctx->SetError("body %d changed more than its state (position, orientation, velocities); use "
                      "bepugpu_upload_bodies", h[0]);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (h[2] != 0x7f7f7f7f) {
        ctx->SetError("manifold %d changed its bodies or its GENERATED or NONCONVEX flag, has a contact count "
                      "outside 0..4 or a contact_order that is no permutation; use bepugpu_upload_constraints", h[2]);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (nb) {
        k_update_body_state<<<Blocks(nb, 256), 256, 0, s->stream>>>(sb, (int)nb, s->b, s->bodyRecords);
        k_world_inertia<<<Blocks(nb, 256), 256, 0, s->stream>>>(s->b, s->localM33);
    }
    if (nm) k_unpack_manifolds<<<Blocks(nm, 256), 256, 0, s->stream>>>(sm, s->slotOf, (int)nm, s->m);
    CK(cudaGetLastError());
    s->kin.FromBits((uint32_t)h[1]);
    bepugpu_status st = s->Step(ctx, dt, flags & BEPUGPU_STEP_ALL);
    if (st != BEPUGPU_OK) return st;
    // whole records back into the caller's arrays
    if (nb) {
        k_patch_body_records<<<Blocks(nb, 256), 256, 0, s->stream>>>(s->b, s->bodyRecords);
        CK(cudaMemcpyAsync(bodies, s->bodyRecords, sizeof(bepugpu_body) * nb, cudaMemcpyDeviceToHost, s->stream));
    }
    if (nm) {
        k_pack_manifold_records<<<Blocks(nm, kRecordBlock), kRecordBlock, 0, s->stream>>>(s->m, s->slotOf, (int)nm,
                                                                                        (uint2*)sm);
        CK(cudaMemcpyAsync(man, sm, sizeof(bepugpu_manifold) * nm, cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    s->asyncPending = false;
    return BEPUGPU_OK;
}

namespace {
// Argument checks shared by bepugpu_step_state and bepugpu_download_state.
bepugpu_status CheckStateArrays(Context* ctx, Scene* s, const void* bodies, uint32_t nb, bool bodiesRequired,
                                const void* man, uint32_t nm) {
    if ((bodiesRequired || nb) && (nb != (uint32_t)s->b.count || (nb && !bodies))) {
        ctx->SetError("state calls take the %d bodies of the last upload", s->b.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (nm && (nm != (uint32_t)s->m.count || !man)) {
        ctx->SetError("state calls take all %d manifolds of the last upload, or none", s->m.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    return BEPUGPU_OK;
}
// The device's address of a page-locked host array (cudaHostAlloc or
// cudaHostRegister memory is mapped into the device's address space), or
// null for pageable memory.  Kernels then read and write the caller's array
// over the host link themselves (NVLink-C2C on Grace), with no staging copy.
void* PinnedDeviceAddress(const void* p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Packs the scene's state into the caller's arrays (asynchronous on the
// scene's stream): straight into page-locked arrays, else through the
// staging buffer and a copy.
bepugpu_status QueueStateDownload(Context* ctx, Scene* s, bepugpu_body_state* bodies, uint32_t nb,
                                  bepugpu_manifold_state* man, uint32_t nm) {
    auto* sb = (bepugpu_body_state*)s->staging;
    auto* sm = (bepugpu_manifold_state*)((char*)s->staging + s->stagingManifoldsAt);
    auto* db = nb ? (bepugpu_body_state*)PinnedDeviceAddress(bodies) : nullptr;
    auto* dm = nm ? (bepugpu_manifold_state*)PinnedDeviceAddress(man) : nullptr;
    const int bodyBlocks = nb ? Blocks(nb, kStateBlock) : 0, manifoldBlocks = nm ? Blocks(nm, kStateBlock) : 0;
    if (bodyBlocks + manifoldBlocks)
        k_pack_state<<<bodyBlocks + manifoldBlocks, kStateBlock, 0, s->stream>>>(s->b, db ? db : sb, bodyBlocks, s->m,
                                                                                 s->slotOf, (int)nm, dm ? dm : sm);
    if (nb && !db)
        CK(cudaMemcpyAsync(bodies, sb, sizeof(bepugpu_body_state) * nb, cudaMemcpyDeviceToHost, s->stream));
    if (nm && !dm)
        CK(cudaMemcpyAsync(man, sm, sizeof(bepugpu_manifold_state) * nm, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaGetLastError());
    return BEPUGPU_OK;
}
}  // namespace

static_assert(sizeof(bepugpu_body_state) == 64 && sizeof(bepugpu_manifold_state) == 80,
              "state records are four and five 16-byte words");

bepugpu_status bepugpu_step_state(bepugpu_context* c, int32_t id, bepugpu_body_state* bodies, uint32_t nb,
                                  bepugpu_manifold_state* man, uint32_t nm, float dt, uint32_t flags) {
    NvtxRange range("bepugpu_step_state");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    bepugpu_status st = CheckStateArrays(ctx, s, bodies, nb, true, man, nm);
    if (st != BEPUGPU_OK) return st;
    if (!(dt > 0) || !std::isfinite(dt)) {
        ctx->SetError("dt must be positive and finite");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->asyncPending) {  // an earlier step may still read the staging buffer
        CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
    }
    // What the kinematic bodies' stages have to do, from their new state on
    // the host (the rest of their records cannot change here).
    s->kin.Clear();
    for (int32_t i : s->hostKinematic) {
        const bepugpu_body_state& r = bodies[i];
        const float* v = r.linear_velocity;
        const float* w = r.angular_velocity;
        s->kin.Add(v[0] != 0 || v[1] != 0 || v[2] != 0 || w[0] != 0 || w[1] != 0 || w[2] != 0, r.activity,
                   r.previous_velocity, r.velocity_time_below_limit);
    }
    auto* sb = (bepugpu_body_state*)s->staging;
    if (nb) {
        // page-locked caller arrays are read in place, others through the staging buffer
        auto* in = (const bepugpu_body_state*)PinnedDeviceAddress(bodies);
        if (!in) {
            CK(cudaMemcpyAsync(sb, bodies, sizeof(bepugpu_body_state) * nb, cudaMemcpyHostToDevice, s->stream));
            in = sb;
        }
        k_update_body_state_records<<<Blocks(nb, kStateBlock), kStateBlock, 0, s->stream>>>(in, (int)nb, s->b,
                                                                                          s->bodyRecords, s->localM33);
        CK(cudaGetLastError());
    }
    st = s->Step(ctx, dt, flags & BEPUGPU_STEP_ALL);
    if (st != BEPUGPU_OK) {
        cudaStreamSynchronize(s->stream);  // the caller may reuse its arrays after an error
        s->asyncPending = false;
        return st;
    }
    st = QueueStateDownload(ctx, s, bodies, nb, man, nm);
    CK(cudaStreamSynchronize(s->stream));
    s->asyncPending = false;
    return st;
}

bepugpu_status bepugpu_download_state(bepugpu_context* c, int32_t id, bepugpu_body_state* bodies, uint32_t nb,
                                      bepugpu_manifold_state* man, uint32_t nm) {
    NvtxRange range("bepugpu_download_state");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    bepugpu_status st = CheckStateArrays(ctx, s, bodies, nb, false, man, nm);
    if (st != BEPUGPU_OK) return st;
    if (s->asyncPending) {
        CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
    }
    st = QueueStateDownload(ctx, s, bodies, nb, man, nm);
    CK(cudaStreamSynchronize(s->stream));
    return st;
}

bepugpu_status bepugpu_update_bodies(bepugpu_context* c, int32_t id, const bepugpu_body* bodies, uint32_t n) {
    NvtxRange range("bepugpu_update_bodies");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (n != (uint32_t)s->b.count || (n && !bodies)) {
        ctx->SetError("update_bodies needs the %d bodies of the last upload", s->b.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (!n) return BEPUGPU_OK;
    int bad = -1, moving = 0;  // moving: the kinematic bodies' KinematicState bits
    bepugpu_status st = CheckRecords(ctx, s, bodies, sizeof(bepugpu_body) * n, [&](int* check) {
        k_check_body_records<<<Blocks(n, 256), 256, 0, s->stream>>>((const bepugpu_body*)s->staging,
                                                                     s->bodyRecords, (int)n, check);
    }, bad, moving);
    if (st != BEPUGPU_OK) return st;
    if (bad >= 0) {
        ctx->SetError("body %d changed more than its state (position, orientation, velocities); use "
                      "bepugpu_upload_bodies", bad);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    k_update_body_state<<<Blocks(n, 256), 256, 0, s->stream>>>((const bepugpu_body*)s->staging, (int)n, s->b,
                                                                 s->bodyRecords);
    k_world_inertia<<<Blocks(n, 256), 256, 0, s->stream>>>(s->b, s->localM33);
    CK(cudaGetLastError());
    s->kin.FromBits((uint32_t)moving);
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_probe_double_rounding(bepugpu_context* c, int32_t kind, const float* a, const float* b,
                                             uint32_t n, float* out, uint32_t* fast) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    if (kind < 0 || kind > 2 || (n && (!a || !out || (kind > 0 && !b))) || n > (1u << 26)) {
        ctx->SetError("probe_double_rounding: kind 0..2, inputs and output given, at most 2^26 values");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (fast) *fast = 0;
    if (!n) return BEPUGPU_OK;
    float *da = nullptr, *db = nullptr, *dout = nullptr;
    unsigned int* dfast = nullptr;
    auto release = [&]() {
        cudaFree(da);
        cudaFree(db);
        cudaFree(dout);
        cudaFree(dfast);
    };
    cudaError_t e;
    if ((e = cudaMalloc(&da, 4ull * n)) || (e = cudaMalloc(&db, 4ull * n)) || (e = cudaMalloc(&dout, 4ull * n)) ||
        (e = cudaMalloc(&dfast, 4)) || (e = cudaMemcpy(da, a, 4ull * n, cudaMemcpyHostToDevice)) ||
        (e = cudaMemset(db, 0, 4ull * n)) || (kind > 0 && (e = cudaMemcpy(db, b, 4ull * n, cudaMemcpyHostToDevice))) ||
        (e = cudaMemset(dfast, 0, 4))) {
        release();
        ctx->SetError("probe_double_rounding: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    k_probe_double_rounding<<<Blocks((int)n, 256), 256>>>(kind, da, db, (int)n, dout, dfast);
    unsigned int h = 0;
    if ((e = cudaGetLastError()) || (e = cudaMemcpy(out, dout, 4ull * n, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(&h, dfast, 4, cudaMemcpyDeviceToHost))) {
        release();
        ctx->SetError("probe_double_rounding: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    release();
    if (fast) *fast = h;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_check_finite(bepugpu_context* c, int32_t id, int32_t* firstBad) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (!firstBad) return BEPUGPU_INVALID_ARGUMENT;
    *firstBad = -1;
    if (!s->b.count) return BEPUGPU_OK;
    int* check = s->CheckWords();
    CK(cudaMemsetAsync(check, 0x7f, sizeof(int), s->stream));
    k_check_finite<<<Blocks(s->b.count, 256), 256, 0, s->stream>>>(s->b, check);
    CK(cudaGetLastError());
    int h = 0;
    CK(cudaMemcpyAsync(&h, check, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->asyncPending = false;
    if (h == 0x7f7f7f7f) return BEPUGPU_OK;
    *firstBad = h;
    ctx->SetError("body %d has a non-finite position, orientation or velocity", h);
    return BEPUGPU_NAN_DETECTED;
}

bepugpu_status bepugpu_probe_bounded_wait(bepugpu_context* c, uint32_t limit) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    void* words = nullptr;  // [0] the flag nothing sets, [1] the status
    CK(cudaMalloc(&words, 2 * sizeof(int)));
    cudaError_t e = cudaMemset(words, 0, 2 * sizeof(int));
    int status = BEPUGPU_CUDA_ERROR;
    if (e == cudaSuccess) {
        k_bounded_wait_probe<<<1, 1>>>((volatile unsigned int*)words, limit, (int*)words + 1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&status, (int*)words + 1, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(words);
    if (e != cudaSuccess) {
        ctx->SetError("bounded wait probe: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    if (status == BEPUGPU_TIMEOUT) ctx->SetError("the bounded wait ran out after %u polls", limit);
    return (bepugpu_status)status;
}

bepugpu_status bepugpu_download_bodies(bepugpu_context* c, int32_t id, bepugpu_body* bodies, uint32_t n) {
    NvtxRange range("bepugpu_download_bodies");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (n != (uint32_t)s->b.count || (n && !bodies)) {
        ctx->SetError("download_bodies needs exactly %d records", s->b.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (!n) return BEPUGPU_OK;
    k_patch_body_records<<<Blocks(n, 256), 256, 0, s->stream>>>(s->b, s->bodyRecords);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(bodies, s->bodyRecords, sizeof(bepugpu_body) * n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_download_constraints(bepugpu_context* c, int32_t id, bepugpu_manifold* man, uint32_t nm,
                                            bepugpu_joint* joints, uint32_t nj) {
    NvtxRange range("bepugpu_download_constraints");
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (nm != (uint32_t)s->m.count || nj != s->jointCount || (nm && !man) || (nj && !joints)) {
        ctx->SetError("download_constraints needs %d manifolds and %u joints", s->m.count, s->jointCount);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    {
        bepugpu_status jst = DownloadJoints(ctx, s, joints, nj);
        if (jst != BEPUGPU_OK) return jst;
    }
    if (!nm) return BEPUGPU_OK;
    // Whole records are rebuilt on the device in record order and copied
    // straight into the caller's array (their fields are the uploaded ones,
    // the state fields current; `reserved` comes back 0).
    k_pack_manifold_records<<<Blocks(nm, kRecordBlock), kRecordBlock, 0, s->stream>>>(s->m, s->slotOf, (int)nm,
                                                                                    (uint2*)s->staging);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(man, s->staging, sizeof(bepugpu_manifold) * nm, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_get_colouring(bepugpu_context* c, int32_t id, int32_t* colour, int32_t* order, uint32_t n,
                                     uint32_t* colours) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (n != s->colouring.colour.size()) {
        ctx->SetError("colouring has %zu entries", s->colouring.colour.size());
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (colour && n) std::memcpy(colour, s->colouring.colour.data(), 4 * n);
    if (order && n) std::memcpy(order, s->colouring.order.data(), 4 * n);
    if (colours) *colours = (uint32_t)s->colouring.colours;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_colour_list(const int32_t* a, const int32_t* b, uint32_t n, const uint8_t* dynamic,
                                   uint32_t nb, int32_t* colour, int32_t* order, uint32_t* colours) {
    if ((n && (!a || !b || !colour || !order)) || (nb && !dynamic)) return BEPUGPU_INVALID_ARGUMENT;
    Colouring col;
    if (!ColourSolverList(a, b, (int32_t)n, dynamic, (int32_t)nb, col)) return BEPUGPU_INVALID_ARGUMENT;
    if (n) {
        std::memcpy(colour, col.colour.data(), 4 * n);
        std::memcpy(order, col.order.data(), 4 * n);
    }
    if (colours) *colours = (uint32_t)col.colours;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_set_solve_mode(bepugpu_context* c, int32_t id, int32_t mode) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (mode != BEPUGPU_MODE_GRAPH && mode != BEPUGPU_MODE_PERSISTENT) return BEPUGPU_INVALID_ARGUMENT;
    s->mode = mode;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_set_group_policy(bepugpu_context* c, int32_t id, int32_t enabled, int32_t maxBodies,
                                        int32_t maxManifolds, int32_t target, int32_t threads) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    // 96 bytes of shared memory per body must fit a CTA's 227 KB
    if (maxBodies < 1 || maxBodies > 2400 || maxManifolds < 1 || target < 1 || threads < 0 || threads > 256 ||
        threads % 32) {
        ctx->SetError("group policy out of range (bodies 1..2400, manifolds >= 1, threads 0 or 32..256 by 32)");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    s->policy.enabled = enabled != 0;
    s->policy.maxGroupBodies = maxBodies;
    s->policy.maxGroupManifolds = maxManifolds;
    s->policy.targetGroupManifolds = target;
    s->groupThreadsOverride = threads;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_set_group_smem_budget(bepugpu_context* c, int32_t id, uint32_t bytes) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (bytes > kGroupSmemBudget) {
        ctx->SetError("shared-lane budget above %zu bytes", kGroupSmemBudget);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    s->policy.sharedLanesBudget = bytes;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_set_group_prologue(bepugpu_context* c, int32_t id, int32_t mode) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (mode < -1 || mode > 1) {
        ctx->SetError("group prologue mode must be -1, 0 or 1");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->groupPrologue != mode && s->graphExec) {  // the step graph holds the launches
        cudaGraphExecDestroy(s->graphExec);
        s->graphExec = nullptr;
    }
    s->groupPrologue = mode;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_set_persistent_blocks_per_sm(bepugpu_context* c, int32_t id, int32_t blocks) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (blocks < 1 || blocks > 2) {
        ctx->SetError("persistent blocks per SM must be 1 or 2");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    s->persistentBlocksPerSm = blocks;
    s->persistentBlocks = 0;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_step(bepugpu_context* c, int32_t id, float dt, uint32_t flags) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    return s->Step(ctx, dt, flags & BEPUGPU_STEP_ALL);
}

bepugpu_status bepugpu_last_step_ms(bepugpu_context* c, int32_t id, float* ms) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (!ms || !s->stepped) return BEPUGPU_INVALID_ARGUMENT;
    CK(cudaEventSynchronize(s->evStop));
    CK(cudaEventElapsedTime(ms, s->evStart, s->evStop));
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_last_step_phase_ms(bepugpu_context* c, int32_t id, float* phase_ms) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (!phase_ms || !s->stepped) {
        ctx->SetError("phase times exist after a step");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    CK(cudaEventSynchronize(s->evStop));
    CK(cudaEventElapsedTime(&phase_ms[5], s->evGroup[0], s->evGroup[1]));
    if (s->mode == BEPUGPU_MODE_PERSISTENT) {
        // globaltimer stamps taken by block 0 around the solve iterations
        unsigned long long t[2];
        CK(cudaMemcpy(t, s->Stamps(), sizeof(t), cudaMemcpyDeviceToHost));
        for (int k = 0; k < 5; k++) phase_ms[k] = 0.f;
        phase_ms[3] = t[1] > t[0] ? (float)((double)(t[1] - t[0]) * 1e-6) : 0.f;
        return BEPUGPU_OK;
    }
    if (!s->phaseEvents) {  // the step was the group launch alone
        for (int k = 0; k < 5; k++) phase_ms[k] = 0.f;
        return BEPUGPU_OK;
    }
    for (int k = 0; k < 5; k++) CK(cudaEventElapsedTime(&phase_ms[k], s->evPhase[k], s->evPhase[k + 1]));
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_last_step_launches(bepugpu_context* c, int32_t id, uint32_t* launches) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (!launches) return BEPUGPU_INVALID_ARGUMENT;
    *launches = s->launchesPerStep;
    return BEPUGPU_OK;
}


bepugpu_status bepugpu_profile_step(bepugpu_context* c, int32_t id, float dt, uint32_t flags,
                                    bepugpu_phase_times* out) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (!out || !(dt > 0)) return BEPUGPU_INVALID_ARGUMENT;
    if (s->maxBodyReferenced >= s->b.count) {
        ctx->SetError("constraints reference body %d but the scene holds %d bodies", s->maxBodyReferenced, s->b.count);
        return BEPUGPU_INVALID_OPERATION;
    }
    bepugpu_status st = s->RefreshDamping(ctx, dt);
    if (st != BEPUGPU_OK) return st;
    StepParams p = MakeParams(ctx->settings, dt);
    std::memset(out, 0, sizeof(*out));
    const int T = 128;
    cudaStream_t q = s->stream;
    std::vector<cudaEvent_t> ev;
    auto mark = [&]() -> cudaEvent_t {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, q);
        ev.push_back(e);
        return e;
    };
    struct Span { cudaEvent_t a, b; float* dst; };
    std::vector<Span> spans;
    unsigned long long* acc = s->Census();
    CK(cudaMemsetAsync(acc, 0, 8 * sizeof(unsigned long long), q));
    if (s->islands && (flags & BEPUGPU_STEP_DEACTIVATION)) {  // the island stage first, timed with the forces
        cudaEvent_t a = mark();
        CK(LaunchIslandStage(s, p, ctx->settings.maximum_deactivation_attempts_per_frame, q));
        spans.push_back({a, mark(), &out->force_ms});
    }
    flags = s->StageFlags(flags);
    if (!s->groupPlan.groups.empty()) {  // the census variant of the group kernel counts its visits
        cudaEvent_t a = mark();
        bepugpu_status gs = LaunchGroups(ctx, s, p, flags, true);
        if (gs != BEPUGPU_OK) return gs;
        spans.push_back({a, mark(), &out->group_ms});
        out->groups = (uint32_t)s->groupPlan.groups.size();
        // the groups' own share of the visit census
        CK(cudaMemcpyAsync(acc + 4, acc, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, q));
    }
    const ManifoldSoA ms = s->SweepManifolds();
    const int colours = s->SweepColours();
    int nm = ms.count, nb = s->b.count;
    if ((flags & BEPUGPU_STEP_REFRESH_CONTACTS) && nm) {
        cudaEvent_t a = mark(); k_refresh<<<Blocks(nm, T), T, 0, q>>>(ms, s->b, p); spans.push_back({a, mark(), &out->refresh_ms});
    }
    if ((flags & kStartStages) && nb) {
        ManifoldSoA none = ms;
        none.count = 0;
        cudaEvent_t a = mark();
        k_refresh_force<<<Blocks(nb, T), T, 0, q>>>(none, s->b, p, flags & kStartStages);
        spans.push_back({a, mark(), &out->force_ms});
    }
    const JointSoA js = s->SweepJoints();
    const int nj = js.count;
    if ((flags & BEPUGPU_STEP_SOLVE) && (nm || nj)) {
        cudaEvent_t a = mark();
        const bool added = s->addedJointTypes;
        (added ? k_prestep_mixed<true> : k_prestep_mixed<false>)<<<Blocks(nm + nj, T), T, 0, q>>>(ms, s->b, js, p);
        spans.push_back({a, mark(), &out->prestep_ms});
        for (int cc = 0; cc < colours; cc++) {
            int b0 = s->manifoldOffsets[cc], b1 = s->manifoldOffsets[cc + 1];
            int j0 = nj ? s->jointOffsets[cc] : 0, j1 = nj ? s->jointOffsets[cc + 1] : 0;
            if (b1 - b0 + j1 - j0 <= 0) continue;
            cudaEvent_t e0 = mark();
            (added ? k_warm_mixed<true> : k_warm_mixed<false>)<<<Blocks(b1 - b0 + j1 - j0, T), T, 0, q>>>(
                ms, s->b, js, b0, b1, j0, j1);
            spans.push_back({e0, mark(), &out->warm_ms});
            out->warm_launches++;
        }
        for (int it = 0; it < p.iterationLimit; it++)
            for (int cc = 0; cc < colours; cc++) {
                int b0 = s->manifoldOffsets[cc], b1 = s->manifoldOffsets[cc + 1];
                int j0 = nj ? s->jointOffsets[cc] : 0, j1 = nj ? s->jointOffsets[cc + 1] : 0;
                if (b1 - b0 + j1 - j0 <= 0) continue;
                if (b1 > b0) k_census<<<Blocks(b1 - b0, T), T, 0, q>>>(ms, b0, b1, acc);
                cudaEvent_t e0 = mark();
                (added ? k_solve_mixed<true> : k_solve_mixed<false>)<<<Blocks(b1 - b0 + j1 - j0, T), T, 0, q>>>(
                    ms, s->b, js, p, b0, b1, j0, j1);
                spans.push_back({e0, mark(), &out->solve_ms});
                out->solve_launches++;
            }
    }
    if ((flags & BEPUGPU_STEP_POSITIONS) && nb) {
        cudaEvent_t a = mark(); k_position<<<Blocks(nb, T), T, 0, q>>>(s->b, p); spans.push_back({a, mark(), &out->position_ms});
    }
    CK(cudaGetLastError());
    unsigned long long h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, q));
    CK(cudaStreamSynchronize(q));
    for (auto& sp : spans) {
        float ms = 0;
        cudaEventElapsedTime(&ms, sp.a, sp.b);
        *sp.dst += ms;
    }
    for (auto e : ev) cudaEventDestroy(e);
    out->solve_algorithmic_bytes = (double)h[0];
    out->solve_manifold_visits = (double)h[1];
    out->solve_contact_visits = (double)h[2];
    out->group_compulsory_bytes = (double)h[3];
    out->group_solve_algorithmic_bytes = (double)h[4];
    out->group_solve_manifold_visits = (double)h[5];
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_last_call_stats(bepugpu_context* c, uint32_t* launches, float* ms) {
    auto* ctx = reinterpret_cast<Context*>(c);
    CTX_CHECK(ctx);
    if (launches) *launches = ctx->lastLaunches;
    if (ms) *ms = ctx->lastMs;
    return BEPUGPU_OK;
}

}  // extern "C"
