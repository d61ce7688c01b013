// Narrow phase: shapes, the GENERATED manifold list and the collide kernel.
//
// The reference's NarrowPhase updates every pair handler's manifold
// (NarrowPhaseSystems/NarrowPhase.cs, Pairs/*PairHandler.cs) after the force
// update and before the solver; here one thread per GENERATED manifold runs
// the pair's tester and manifold update (collide_device.cuh) as the first
// launch of the step.  The shapes sit in the scene arena (one float4 per
// body), so spills and restores carry them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "collide_device.cuh"

namespace bepugpu {

// 64-thread blocks: the pair count (65,536 on the pile) fills only about a
// fifth of the SMs' warp slots, so smaller blocks spread it more evenly.
__global__ void __launch_bounds__(64) k_collide(ManifoldSoA m, BodySoA b, const float4* __restrict__ shape,
                                                 const int32_t* __restrict__ slots, int n, StepParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (b.islandOf) {  // with islands, a pair between two inactive entries keeps its contacts (NarrowPhase.cs:300-332)
        const int4 h = m.head[slots[i]];
        if (!EntryActive(b, h.x) && !EntryActive(b, h.y)) return;
    }
    nphase::CollideManifold(m, b, shape, slots[i], p);
}

cudaError_t LaunchCollide(Scene* s, const StepParams& p, cudaStream_t stream) {
    const int n = s->generatedCount;
    if (n <= 0) return cudaSuccess;
    const int T = 64;
    k_collide<<<(n + T - 1) / T, T, 0, stream>>>(s->m, s->b, s->shape, s->genSlotsDev, n, p);
    return cudaGetLastError();
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            ctx->SetError("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return BEPUGPU_CUDA_ERROR;                                                        \
        }                                                                                     \
    } while (0)

namespace {

bool PairShapesFit(const bepugpu_shape& a, const bepugpu_shape& b) {
    if (a.type == BEPUGPU_SHAPE_BOX) return b.type == BEPUGPU_SHAPE_BOX || b.type == BEPUGPU_SHAPE_SPHERE;
    return a.type == BEPUGPU_SHAPE_SPHERE && b.type == BEPUGPU_SHAPE_SPHERE;
}

}  // namespace

bepugpu_status PrepareGenerated(Context* ctx, Scene* s, const bepugpu_manifold* man, uint32_t nm,
                                const std::vector<int32_t>& slotOf) {
    std::vector<int32_t> slots;
    std::vector<int2> pairs;
    for (uint32_t i = 0; i < nm; i++) {
        const bepugpu_manifold& r = man[i];
        if (!(r.flags & BEPUGPU_MANIFOLD_GENERATED)) continue;
        if (s->hostShapes.size() != (size_t)s->b.count) {
            ctx->SetError("manifold %u is GENERATED but the scene has no shapes for its %d bodies "
                          "(bepugpu_upload_shapes)", i, s->b.count);
            return BEPUGPU_INVALID_OPERATION;
        }
        if (r.body_a < 0 || r.body_b < 0) {
            ctx->SetError("GENERATED manifold %u needs two bodies", i);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        const bepugpu_shape &sa = s->hostShapes[r.body_a], &sb = s->hostShapes[r.body_b];
        if (!PairShapesFit(sa, sb)) {
            ctx->SetError("GENERATED manifold %u pairs shapes %d and %d (box-box, box-sphere with the box as "
                          "body_a, or sphere-sphere)", i, sa.type, sb.type);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        const uint32_t code = (uint32_t)r.contact_order ^ 0xE4u;
        uint32_t seen = 0;
        for (int k = 0; k < r.contact_count; k++) seen |= 1u << ((code >> (2 * k)) & 3u);
        if (seen != (1u << r.contact_count) - 1u) {
            ctx->SetError("GENERATED manifold %u: contact_order is not a permutation of its %d contacts", i,
                          r.contact_count);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (sb.type == BEPUGPU_SHAPE_SPHERE && r.contact_count > 1) {
            ctx->SetError("GENERATED manifold %u holds %d contacts; a sphere pair holds at most one", i,
                          r.contact_count);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        slots.push_back(slotOf[i]);
        pairs.push_back(make_int2(r.body_a, r.body_b));
    }
    s->hostGenPairs = pairs;
    std::sort(slots.begin(), slots.end());  // ascending slots: neighbouring threads read neighbouring lanes
    s->generatedCount = (int32_t)slots.size();
    if (!slots.empty()) {
        CK(cudaMemcpyAsync(s->genSlotsDev, slots.data(), sizeof(int32_t) * slots.size(), cudaMemcpyHostToDevice,
                           s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return BEPUGPU_OK;
}

}  // namespace bepugpu

using namespace bepugpu;

extern "C" bepugpu_status bepugpu_upload_shapes(bepugpu_context* c, int32_t id, const bepugpu_shape* shapes,
                                                uint32_t count) {
    NvtxRange range("bepugpu_upload_shapes");
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (count != (uint32_t)s->b.count || (count && !shapes)) {
        ctx->SetError("upload_shapes needs one shape for each of the %d bodies", s->b.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    std::vector<float4> lane(count);
    for (uint32_t i = 0; i < count; i++) {
        const bepugpu_shape& sh = shapes[i];
        const int n = sh.type == BEPUGPU_SHAPE_BOX ? 3 : (sh.type == BEPUGPU_SHAPE_SPHERE ? 1 : 0);
        if (sh.type != BEPUGPU_SHAPE_NONE && n == 0) {
            ctx->SetError("shape %u has unknown type %d", i, sh.type);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        for (int k = 0; k < n; k++)
            if (!(sh.size[k] > 0) || !std::isfinite(sh.size[k])) {
                ctx->SetError("shape %u: sizes must be positive and finite", i);
                return BEPUGPU_INVALID_ARGUMENT;
            }
        float typeBits;
        std::memcpy(&typeBits, &sh.type, sizeof(float));
        lane[i] = make_float4(sh.size[0], sh.size[1], sh.size[2], typeBits);
    }
    // Shapes of bodies the GENERATED manifolds join must keep fitting them.
    if (s->generatedCount) {
        for (size_t i = 0; i < s->hostGenPairs.size(); i++) {
            const int2 pr = s->hostGenPairs[i];
            if (!PairShapesFit(shapes[pr.x], shapes[pr.y])) {
                ctx->SetError("shape change breaks GENERATED manifold between bodies %d and %d", pr.x, pr.y);
                return BEPUGPU_INVALID_ARGUMENT;
            }
        }
    }
    if (s->asyncPending) {
        CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
    }
    if (count) {
        CK(cudaMemcpyAsync(s->shape, lane.data(), sizeof(float4) * count, cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    s->hostShapes.assign(shapes, shapes + count);
    return BEPUGPU_OK;
}
