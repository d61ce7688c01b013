// bepugpu_step_noalloc: one solver step of a small scene without any device
// allocation.
//
// Who needs it: hosts that cannot call cudaMalloc -- a plugin running inside
// an engine or a sandbox that owns the device heap and hands out only the
// buffers it allocated itself, or code that must stay inside a memory budget
// fixed before it starts.  Such a caller owns its body and manifold records in
// device memory and passes their addresses; everything else the step needs
// (the structure-of-arrays state, the prestep products, the colouring) lives
// in one fixed array in this file, g_stepScratch, sized for at most
// BEPUGPU_NOALLOC_MAX_BODIES bodies and BEPUGPU_NOALLOC_MAX_MANIFOLDS
// manifolds.  Every GPU that loads the library holds that array until the
// process exits.
//
// The step runs in one CTA: it validates and colours the manifold list
// (greedy, in list order, conflicts through dynamic bodies -- the same
// colouring as bepugpu_upload_constraints), then runs refresh, force update,
// prestep, warm start, the colour sweeps and the position update with block
// barriers between them, and writes the state fields back into the caller's
// records, as bepugpu_download_bodies / bepugpu_download_constraints do.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "solver_device.cuh"

namespace {

using namespace bepugpu;

constexpr int kMaxBodies = BEPUGPU_NOALLOC_MAX_BODIES;
constexpr int kMaxManifolds = BEPUGPU_NOALLOC_MAX_MANIFOLDS;
constexpr int kMaxColours = 128;  // two 64-bit colour masks per body
constexpr int kThreads = 256;

// Byte layout of the scratch array.
constexpr size_t A(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kBodyArray = A(16 * (size_t)kMaxBodies);       // one float4 per body
constexpr size_t kLaneArray = A(16 * (size_t)kMaxManifolds);    // one float4 per manifold
constexpr size_t kLane4Array = A(64 * (size_t)kMaxManifolds);   // four float4 per manifold
constexpr size_t kBodiesAt = 0;                                  // 11 body arrays
constexpr size_t kHeadAt = kBodiesAt + 11 * kBodyArray;
constexpr size_t kLane4At = kHeadAt + kLaneArray;               // cpos cnrm offA offB pj0 pj1 pj2
constexpr size_t kLaneAt = kLane4At + 7 * kLane4Array;          // mat penacc fricacc saxis s0 s1 s3..s7 lever
constexpr size_t kStateAt = kLaneAt + 14 * kLaneArray;
constexpr size_t kSlotAt = kStateAt + A(8 * (size_t)kMaxManifolds);
constexpr size_t kColourAt = kSlotAt + A(4 * (size_t)kMaxManifolds);
constexpr size_t kMaskAt = kColourAt + A(4 * (size_t)kMaxManifolds);
constexpr size_t kOffsetsAt = kMaskAt + A(16 * (size_t)kMaxBodies);
constexpr size_t kStepErrorAt = kOffsetsAt + A(4 * (size_t)(kMaxColours + 1));
constexpr size_t kScratchBytes = kStepErrorAt + 256;
static_assert(kScratchBytes == BEPUGPU_NOALLOC_SCRATCH_BYTES, "keep the header's stated size in step");

// The scratch.  Host code must not pass this name to a kernel: on the host it
// is only a stand-in symbol, so its device address is looked up once per
// device with cudaGetSymbolAddress.  Every call shares it: two calls whose
// kernels overlap on the GPU race on it.
static __device__ __align__(256) unsigned char g_stepScratch[kScratchBytes];

struct Views {
    BodySoA b;
    ManifoldSoA m;
    int32_t* slotOf;
    int32_t* colour;
    unsigned long long* masks;
    int32_t* offsets;
    int32_t* error;
};

__device__ Views Carve(unsigned char* s, int nb, int nm) {
    Views v;
    float4* body[11];
    for (int k = 0; k < 11; k++) body[k] = (float4*)(s + kBodiesAt + k * kBodyArray);
    v.b.pos = body[0]; v.b.quat = body[1]; v.b.vlin = body[2]; v.b.vang = body[3]; v.b.inv0 = body[4];
    v.b.inv1 = body[5]; v.b.loc0 = body[6]; v.b.loc1 = body[7]; v.b.damp = body[8]; v.b.act = body[9];
    v.b.rawDamp = (float2*)body[10];
    v.b.islandOf = nullptr;  // every island awake
    v.b.islandFlags = nullptr;
    v.b.count = nb;
    float4* l4[7];
    for (int k = 0; k < 7; k++) l4[k] = (float4*)(s + kLane4At + k * kLane4Array);
    float4* l1[14];
    for (int k = 0; k < 14; k++) l1[k] = (float4*)(s + kLaneAt + k * kLaneArray);
    v.m.head = (int4*)(s + kHeadAt);
    v.m.cpos = l4[0]; v.m.cnrm = l4[1]; v.m.offA = l4[2]; v.m.offB = l4[3];
    v.m.pj0 = l4[4]; v.m.pj1 = l4[5]; v.m.pj2 = l4[6];
    v.m.mat = l1[0]; v.m.penacc = l1[1]; v.m.fricacc = l1[2]; v.m.saxis = l1[3];
    v.m.s0 = l1[4]; v.m.s1 = l1[5]; v.m.s3 = l1[6]; v.m.s4 = l1[7]; v.m.s5 = l1[8]; v.m.s6 = l1[9];
    v.m.s7 = l1[10]; v.m.lever = l1[11];
    v.m.cfr = v.m.cfa = v.m.cfb = nullptr;  // NONCONVEX manifolds are refused
    v.m.state = (uint2*)(s + kStateAt);
    v.m.count = nm;
    v.m.capacity = kMaxManifolds;
    v.slotOf = (int32_t*)(s + kSlotAt);
    v.colour = (int32_t*)(s + kColourAt);
    v.masks = (unsigned long long*)(s + kMaskAt);
    v.offsets = (int32_t*)(s + kOffsetsAt);
    v.error = (int32_t*)(s + kStepErrorAt);
    return v;
}

// (float)Math.Pow(Clamp(1 - d, 0, 1), dt) (EntityBase.cs:943,952), here on
// the device: the float the double result rounds to.
__device__ float DeviceDampingFactor(float d, float dt) {
    float c = 1 - d;
    c = c < 0 ? 0 : (c > 1 ? 1 : c);
    return dr::PowAsDouble(c, dt);
}

__global__ void __launch_bounds__(kThreads) k_step_noalloc(bepugpu_body* bodies, int nb, bepugpu_manifold* man,
                                                           int nm, StepParams p, uint32_t flags,
                                                           unsigned char* scratch) {
    Views v = Carve(scratch, nb, nm);
    __shared__ int sErr;
    __shared__ int sColours;
    const int t = threadIdx.x;
    // Validate before any indexed access; clear the error word of an earlier call.
    if (t == 0) {
        int err = BEPUGPU_OK;
        for (int i = 0; i < nm && !err; i++) {
            int a = man[i].body_a, b = man[i].body_b, c = man[i].contact_count;
            if (a < -1 || a >= nb || b < -1 || b >= nb || (a >= 0 && a == b) || c < 0 || c > 4 ||
                (man[i].flags & BEPUGPU_MANIFOLD_NONCONVEX))
                err = BEPUGPU_INVALID_ARGUMENT;
        }
        sErr = err;
        *v.error = err;
    }
    __syncthreads();
    if (sErr) return;

    // Bodies: records -> structure of arrays, world inverse inertia R^T L R.
    for (int i = t; i < nb; i += kThreads) {
        const bepugpu_body& r = bodies[i];
        bool dyn = r.is_dynamic != 0;
        const float* L = r.local_inverse_inertia;
        float l[9];
        for (int k = 0; k < 9; k++) l[k] = dyn ? L[k] : 0.f;
        v.b.pos[i] = make_float4(r.position[0], r.position[1], r.position[2], dyn ? 1.f : 0.f);
        float4 q = make_float4(r.orientation[0], r.orientation[1], r.orientation[2], r.orientation[3]);
        v.b.quat[i] = q;
        v.b.vlin[i] = make_float4(r.linear_velocity[0], r.linear_velocity[1], r.linear_velocity[2],
                                  dyn ? r.inverse_mass : 0.f);
        v.b.loc0[i] = make_float4(l[0], l[1], l[2], l[3]);
        v.b.loc1[i] = make_float4(l[4], l[5], l[6], l[7]);
        float lin = r.linear_damping + 0.f, ang = r.angular_damping + 0.f;
        uint32_t dflags = (lin > 0 ? 1u : 0u) | (ang > 0 ? 2u : 0u);
        v.b.damp[i] = make_float4(DeviceDampingFactor(lin, p.dt), DeviceDampingFactor(ang, p.dt), l[8],
                                  __uint_as_float(dflags));
        v.b.rawDamp[i] = make_float2(r.linear_damping, r.angular_damping);
        v.b.act[i] = make_float4(r.previous_velocity, r.velocity_time_below_limit, __uint_as_float(r.activity), 0.f);
        // Matrix3x3.CreateFromQuaternion then MultiplyTransposed / Multiply, as in the force update.
        float qX2 = q.x + q.x, qY2 = q.y + q.y, qZ2 = q.z + q.z;
        float XX = qX2 * q.x, YY = qY2 * q.y, ZZ = qZ2 * q.z;
        float XY = qX2 * q.y, XZ = qX2 * q.z, XW = qX2 * q.w;
        float YZ = qY2 * q.z, YW = qY2 * q.w, ZW = qZ2 * q.w;
        float R11 = 1 - YY - ZZ, R21 = XY - ZW, R31 = XZ + YW;
        float R12 = XY + ZW, R22 = 1 - XX - ZZ, R32 = YZ - XW;
        float R13 = XZ - YW, R23 = YZ + XW, R33 = 1 - XX - YY;
        float m11 = R11 * l[0] + R21 * l[3] + R31 * l[6];
        float m12 = R11 * l[1] + R21 * l[4] + R31 * l[7];
        float m13 = R11 * l[2] + R21 * l[5] + R31 * l[8];
        float m21 = R12 * l[0] + R22 * l[3] + R32 * l[6];
        float m22 = R12 * l[1] + R22 * l[4] + R32 * l[7];
        float m23 = R12 * l[2] + R22 * l[5] + R32 * l[8];
        float m31 = R13 * l[0] + R23 * l[3] + R33 * l[6];
        float m32 = R13 * l[1] + R23 * l[4] + R33 * l[7];
        float m33 = R13 * l[2] + R23 * l[5] + R33 * l[8];
        v.b.inv0[i] = make_float4(m11 * R11 + m12 * R21 + m13 * R31, m11 * R12 + m12 * R22 + m13 * R32,
                                  m11 * R13 + m12 * R23 + m13 * R33, m21 * R11 + m22 * R21 + m23 * R31);
        v.b.inv1[i] = make_float4(m21 * R12 + m22 * R22 + m23 * R32, m21 * R13 + m22 * R23 + m23 * R33,
                                  m31 * R11 + m32 * R21 + m33 * R31, m31 * R12 + m32 * R22 + m33 * R32);
        v.b.vang[i] = make_float4(r.angular_velocity[0], r.angular_velocity[1], r.angular_velocity[2],
                                  m31 * R13 + m32 * R23 + m33 * R33);
        v.masks[2 * i] = 0ull;  // colour masks start empty on every call
        v.masks[2 * i + 1] = 0ull;
    }
    __syncthreads();

    // Colouring: greedy first fit in list order, then a stable colour sort.
    if (t == 0) {
        int colours = 0, err = BEPUGPU_OK;
        for (int i = 0; i < nm; i++) {
            int ends[2] = {man[i].body_a, man[i].body_b};
            unsigned long long taken0 = 0, taken1 = 0;
            for (int e : ends)
                if (e >= 0 && bodies[e].is_dynamic) { taken0 |= v.masks[2 * e]; taken1 |= v.masks[2 * e + 1]; }
            int c = taken0 != ~0ull ? __ffsll((long long)~taken0) - 1
                                    : (taken1 != ~0ull ? 64 + __ffsll((long long)~taken1) - 1 : -1);
            if (c < 0) { err = BEPUGPU_INVALID_OPERATION; break; }
            v.colour[i] = c;
            colours = c + 1 > colours ? c + 1 : colours;
            for (int e : ends)
                if (e >= 0 && bodies[e].is_dynamic) v.masks[2 * e + (c >> 6)] |= 1ull << (c & 63);
        }
        if (!err) {
            // offsets[c] .. offsets[c + 1] is colour c's slot range
            for (int c = 0; c <= colours; c++) v.offsets[c] = 0;
            for (int i = 0; i < nm; i++) v.offsets[v.colour[i] + 1]++;
            for (int c = 0; c < colours; c++) v.offsets[c + 1] += v.offsets[c];
            // the colour masks are spent: reuse them as per-colour cursors
            int32_t* cursor = (int32_t*)v.masks;
            for (int c = 0; c < colours; c++) cursor[c] = v.offsets[c];
            for (int i = 0; i < nm; i++) v.slotOf[i] = cursor[v.colour[i]]++;
        }
        sColours = colours;
        sErr = err;
        *v.error = err;
    }
    __syncthreads();
    if (sErr) return;
    const int colours = sColours;

    // Manifolds: records -> slots.
    for (int i = t; i < nm; i += kThreads) {
        const bepugpu_manifold& r = man[i];
        int s = v.slotOf[i], cap = kMaxManifolds, count = r.contact_count;
        v.m.head[s] = make_int4(r.body_a, r.body_b, count | (int)(r.flags << 8), i);
        for (int k = 0; k < 4; k++) {
            const bepugpu_contact& c = r.contacts[k];
            v.m.cpos[k * cap + s] = make_float4(c.position[0], c.position[1], c.position[2], c.penetration_depth);
            v.m.cnrm[k * cap + s] = make_float4(c.normal[0], c.normal[1], c.normal[2], __int_as_float(c.id));
            v.m.offA[k * cap + s] = make_float4(c.local_offset_a[0], c.local_offset_a[1], c.local_offset_a[2],
                                                c.base_penetration_depth);
            v.m.offB[k * cap + s] = make_float4(c.local_offset_b[0], c.local_offset_b[1], c.local_offset_b[2], 0.f);
        }
        float pa[4];
        for (int k = 0; k < 4; k++) pa[k] = k < count ? r.contacts[k].penetration_impulse : 0.f;
        v.m.penacc[s] = make_float4(pa[0], pa[1], pa[2], pa[3]);
        bool live = count > 0;
        v.m.fricacc[s] = make_float4(live ? r.sliding_impulse[0] : 0.f, live ? r.sliding_impulse[1] : 0.f,
                                     live ? r.twist_impulse : 0.f, 0.f);
        v.m.saxis[s] = make_float4(r.sliding_axis[0], r.sliding_axis[1], r.sliding_axis[2], 0.f);
        v.m.mat[s] = make_float4(r.kinetic_friction, r.static_friction, r.bounciness, 0.f);
        v.m.state[s] = make_uint2(0u, 0u);
    }
    __syncthreads();

    if (flags & BEPUGPU_STEP_REFRESH_CONTACTS)
        for (int s = t; s < nm; s += kThreads) RefreshManifold(v.m, v.b, s, p);
    if (flags & (BEPUGPU_STEP_FORCES | BEPUGPU_STEP_DEACTIVATION))
        for (int i = t; i < nb; i += kThreads) StartBodyStep(v.b, i, p, flags);
    __syncthreads();
    if (flags & BEPUGPU_STEP_SOLVE) {
        for (int s = t; s < nm; s += kThreads) PrestepManifold(v.m, v.b, s, p);
        __syncthreads();
        for (int c = 0; c < colours; c++) {
            for (int s = v.offsets[c] + t; s < v.offsets[c + 1]; s += kThreads) {
                uint2 st = v.m.state[s];
                if (!(st.x & kGroupActive)) continue;
                int4 h = v.m.head[s];
                BodyState A, B;
                if (h.x >= 0) LoadBody(v.b, h.x, A);
                if (h.y >= 0) LoadBody(v.b, h.y, B);
                WarmStartManifold(v.m, s, A, B, st.x, h.z & 0xff);
                if (st.x & kDynA) StoreVelocity(v.b, h.x, A);
                if (st.x & kDynB) StoreVelocity(v.b, h.y, B);
            }
            __syncthreads();
        }
        for (int it = 0; it < p.iterationLimit; it++)
            for (int c = 0; c < colours; c++) {
                for (int s = v.offsets[c] + t; s < v.offsets[c + 1]; s += kThreads) {
                    uint2 st = v.m.state[s];
                    if (!(st.x & kGroupActive)) continue;
                    int4 h = v.m.head[s];
                    BodyState A, B;
                    if (h.x >= 0) LoadBody(v.b, h.x, A);
                    if (h.y >= 0) LoadBody(v.b, h.y, B);
                    SolveManifold(v.m, s, A, B, st, h.z & 0xff, p);
                    if (st.x & kDynA) StoreVelocity(v.b, h.x, A);
                    if (st.x & kDynB) StoreVelocity(v.b, h.y, B);
                    v.m.state[s] = st;
                }
                __syncthreads();
            }
    }
    if (flags & BEPUGPU_STEP_POSITIONS)
        for (int i = t; i < nb; i += kThreads) PositionUpdateBody(v.b, i, p);
    __syncthreads();

    // State fields back into the caller's records.
    for (int i = t; i < nb; i += kThreads) {
        float4 ps = v.b.pos[i], q = v.b.quat[i], lv = v.b.vlin[i], av = v.b.vang[i];
        bepugpu_body& r = bodies[i];
        r.position[0] = ps.x; r.position[1] = ps.y; r.position[2] = ps.z;
        r.orientation[0] = q.x; r.orientation[1] = q.y; r.orientation[2] = q.z; r.orientation[3] = q.w;
        r.linear_velocity[0] = lv.x; r.linear_velocity[1] = lv.y; r.linear_velocity[2] = lv.z;
        r.angular_velocity[0] = av.x; r.angular_velocity[1] = av.y; r.angular_velocity[2] = av.z;
        const float4 a = v.b.act[i];
        r.previous_velocity = a.x;
        r.velocity_time_below_limit = a.y;
        r.activity = __float_as_uint(a.z);
    }
    for (int i = t; i < nm; i += kThreads) {
        int s = v.slotOf[i], cap = kMaxManifolds;
        bepugpu_manifold& r = man[i];
        int count = v.m.head[s].z & 0xff;
        float4 pa = v.m.penacc[s], f = v.m.fricacc[s], ax = v.m.saxis[s];
        float acc[4] = {pa.x, pa.y, pa.z, pa.w};
        r.contact_count = count;
        for (int k = 0; k < 4; k++) {
            bepugpu_contact& c = r.contacts[k];
            if (k < count) {
                float4 cp = v.m.cpos[k * cap + s], cn = v.m.cnrm[k * cap + s];
                float4 oa = v.m.offA[k * cap + s], ob = v.m.offB[k * cap + s];
                c.position[0] = cp.x; c.position[1] = cp.y; c.position[2] = cp.z; c.penetration_depth = cp.w;
                c.normal[0] = cn.x; c.normal[1] = cn.y; c.normal[2] = cn.z; c.id = __float_as_int(cn.w);
                c.local_offset_a[0] = oa.x; c.local_offset_a[1] = oa.y; c.local_offset_a[2] = oa.z;
                c.base_penetration_depth = oa.w;
                c.local_offset_b[0] = ob.x; c.local_offset_b[1] = ob.y; c.local_offset_b[2] = ob.z;
                c.penetration_impulse = acc[k];
            } else {
                float* z = (float*)&c;
                for (int w = 0; w < (int)(sizeof(bepugpu_contact) / 4); w++) z[w] = 0.f;
            }
        }
        r.sliding_impulse[0] = f.x; r.sliding_impulse[1] = f.y; r.twist_impulse = f.z;
        r.sliding_axis[0] = ax.x; r.sliding_axis[1] = ax.y; r.sliding_axis[2] = ax.z;
    }
}

// Device address of g_stepScratch in each CUDA context that has called: the
// first call made under a context (the device's primary context, or a
// context the caller created and made current) looks the address up with
// cudaGetSymbolAddress, which loads the library's module into that context.
// An address is valid only in the context it was looked up in, so the cache
// is keyed by the current context (cuCtxGetCurrent, reached through
// cudaGetDriverEntryPointByVersion so the library does not link the driver).
typedef int (*CtxGetCurrentFn)(void**);
std::mutex g_setupLock;
CtxGetCurrentFn g_ctxGetCurrent = nullptr;
bool g_ctxLookedUp = false;
struct ScratchEntry {
    void* context;
    void* address;
};
ScratchEntry g_scratchAddress[64];
int g_scratchEntries = 0;

void* CurrentContext() {
    void* c = nullptr;
    if (g_ctxGetCurrent && g_ctxGetCurrent(&c) != 0) c = nullptr;
    return c;
}

// The scratch array's address in the current context (null on failure).
void* ScratchAddress() {
    std::lock_guard<std::mutex> lock(g_setupLock);
    if (!g_ctxLookedUp) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctxGetCurrent = (CtxGetCurrentFn)fn;
        g_ctxLookedUp = true;
    }
    void* ctx = CurrentContext();
    if (ctx)
        for (int i = 0; i < g_scratchEntries; i++)
            if (g_scratchAddress[i].context == ctx) return g_scratchAddress[i].address;
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_stepScratch) != cudaSuccess || !ptr) return nullptr;
    ctx = CurrentContext();  // the runtime has made its context current if none was
    if (ctx) {
        if (g_scratchEntries == 64) g_scratchEntries = 0;  // a full table starts over
        g_scratchAddress[g_scratchEntries++] = {ctx, ptr};
    }
    return ptr;
}

}  // namespace

extern "C" bepugpu_status bepugpu_step_noalloc(const bepugpu_settings* settings, bepugpu_body* bodies,
                                               uint32_t body_count, bepugpu_manifold* manifolds,
                                               uint32_t manifold_count, float dt, uint32_t flags,
                                               void* stream) {
    if (!settings || (body_count && !bodies) || (manifold_count && !manifolds)) return BEPUGPU_INVALID_ARGUMENT;
    if (body_count > (uint32_t)kMaxBodies || manifold_count > (uint32_t)kMaxManifolds)
        return BEPUGPU_INVALID_ARGUMENT;  // beyond the fixed scratch: at most 1024 bodies, 2048 manifolds
    if (!(dt > 0) || !std::isfinite(dt)) return BEPUGPU_INVALID_ARGUMENT;
    // the bounds bepugpu_create and bepugpu_set_settings apply
    if (settings->iteration_limit < 0 || settings->iteration_limit > 65535 ||
        settings->minimum_iteration_count < 0 || settings->minimum_iteration_count > 14 ||
        !(settings->velocity_lower_limit >= 0) || !std::isfinite(settings->velocity_lower_limit) ||
        !(settings->low_velocity_time_minimum > 0))
        return BEPUGPU_INVALID_ARGUMENT;
    void* scratch = ScratchAddress();
    if (!scratch) return BEPUGPU_CUDA_ERROR;
    cudaStream_t s = (cudaStream_t)stream;
    StepParams p = MakeParams(*settings, dt);
    k_step_noalloc<<<1, kThreads, 0, s>>>(bodies, (int)body_count, manifolds, (int)manifold_count, p,
                                         flags & BEPUGPU_STEP_ALL, (unsigned char*)scratch);
    if (cudaGetLastError() != cudaSuccess) return BEPUGPU_CUDA_ERROR;
    int32_t err = 0;
    if (cudaMemcpyAsync(&err, (unsigned char*)scratch + kStepErrorAt, sizeof(err), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return BEPUGPU_CUDA_ERROR;
    return (bepugpu_status)err;
}
