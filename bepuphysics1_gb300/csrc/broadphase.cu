// Broad phase of a scene's shaped bodies: every pair whose bounding boxes
// overlap.
//
// The reference keeps its entities' bounding boxes in a DynamicHierarchy
// (BroadPhaseSystems/Hierarchies/DynamicHierarchy.cs) and reports the
// overlapping pairs to the narrow phase.  The pair *set* follows from the
// bounding boxes alone: each collidable's box is its shape's
// (BoxShape.cs:149-174 from the orientation matrix, SphereShape.cs:75-86 the
// centre plus the radius) expanded by its linear velocity times dt
// (EntityCollidable.ExpandBoundingBox, EntityCollidable.cs:195-216, discrete
// bodies), two boxes overlap as BoundingBox.Intersects has it
// (BoundingBox.cs:58-66), and two kinematic bodies make no pair (the default
// kinematic collision group's NoBroadPhase rule, CollisionRules.cs:177).  The
// hierarchy's traversal order is not reproduced: the pairs come back sorted.
//
// Device side, a uniform grid whose cell is twice the mean box extent:
//   1. one thread per body computes its box;
//   2. a body no wider than a cell enters every cell its box touches (at most
//      eight) as a 64-bit key (cell code, body); wider bodies go to a short
//      list;
//   3. the keys are sorted (bitonic, the low 2048-element stages in shared
//      memory), so each cell's bodies are contiguous;
//   4. a thread per key tests its body against the later keys of the same
//      cell, and reports a pair only in the cell that holds the largest
//      corner of the two boxes' minima -- a point of both boxes, so exactly
//      one cell of each overlapping pair reports it;
//   5. a thread per (wide body, body) tests the wide bodies against all;
//   6. the pairs, as 64-bit keys, are sorted and copied back.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"

namespace bepugpu {
namespace {

constexpr int kSortBlock = 1024;            // threads of the shared-memory sort stages
constexpr int kSortTile = 2 * kSortBlock;   // keys per shared-memory tile
constexpr unsigned long long kNoKey = ~0ull;

// Scalars of one call: [0] sum of box extents (float bits, atomics), [1]
// bodies with a box, [2] wide-body count, [3] pair count, [4] cell entries.
enum : int { kWExtent = 0, kWShaped, kWWide, kWPairs, kWEntries, kWords = 8 };

// The bounding box of body i: lo.w = 0 (no shape), 1 (kinematic), 2 (dynamic).
__device__ __forceinline__ float BoxOf(const BodySoA& b, const float4* __restrict__ shape, float dt, int i,
                                       float4* __restrict__ lo, float4* __restrict__ hi) {
    const float4 sh = shape[i];
    const int type = __float_as_int(sh.w);
    const float4 p = b.pos[i];
    float mnx, mny, mnz, mxx, mxy, mxz;
    if (type == BEPUGPU_SHAPE_BOX) {
        // Matrix3x3.CreateFromQuaternion, then the extreme points of the
        // signed half extents (BoxShape.GetBoundingBox, TransformLocalExtremePoints)
        const float4 q = b.quat[i];
        const float qX2 = q.x + q.x, qY2 = q.y + q.y, qZ2 = q.z + q.z;
        const float XX = qX2 * q.x, YY = qY2 * q.y, ZZ = qZ2 * q.z;
        const float XY = qX2 * q.y, XZ = qX2 * q.z, XW = qX2 * q.w;
        const float YZ = qY2 * q.z, YW = qY2 * q.w, ZW = qZ2 * q.w;
        const float M11 = 1 - YY - ZZ, M12 = XY + ZW, M13 = XZ - YW;
        const float M21 = XY - ZW, M22 = 1 - XX - ZZ, M23 = YZ + XW;
        const float M31 = XZ + YW, M32 = YZ - XW, M33 = 1 - XX - YY;
        auto sgn = [](float v) { return v > 0 ? 1.f : (v < 0 ? -1.f : 0.f); };  // Math.Sign
        const float hw = sh.x, hh = sh.y, hl = sh.z;
        const float rx = sgn(M11) * hw, ry = sgn(M21) * hh, rz = sgn(M31) * hl;
        const float ux = sgn(M12) * hw, uy = sgn(M22) * hh, uz = sgn(M32) * hl;
        const float bx = sgn(M13) * hw, by = sgn(M23) * hh, bz = sgn(M33) * hl;
        const float ox = rx * M11 + ry * M21 + rz * M31;
        const float oy = ux * M12 + uy * M22 + uz * M32;
        const float oz = bx * M13 + by * M23 + bz * M33;
        mxx = p.x + ox; mxy = p.y + oy; mxz = p.z + oz;
        mnx = p.x - ox; mny = p.y - oy; mnz = p.z - oz;
    } else if (type == BEPUGPU_SHAPE_SPHERE) {
        const float r = sh.x;
        mnx = p.x - r; mny = p.y - r; mnz = p.z - r;
        mxx = p.x + r; mxy = p.y + r; mxz = p.z + r;
    } else {
        lo[i] = make_float4(0, 0, 0, __int_as_float(0));
        hi[i] = make_float4(0, 0, 0, 0);
        return -1.f;
    }
    if (dt > 0) {
        const float4 v = b.vlin[i];
        if (v.x > 0) mxx += v.x * dt * 1.f; else mnx += v.x * dt * 1.f;
        if (v.y > 0) mxy += v.y * dt * 1.f; else mny += v.y * dt * 1.f;
        if (v.z > 0) mxz += v.z * dt * 1.f; else mnz += v.z * dt * 1.f;
    }
    lo[i] = make_float4(mnx, mny, mnz, __int_as_float(p.w != 0.f ? 2 : 1));
    hi[i] = make_float4(mxx, mxy, mxz, 0.f);
    return fmaxf(mxx - mnx, fmaxf(mxy - mny, mxz - mnz));
}
__global__ void k_bp_boxes(BodySoA b, const float4* __restrict__ shape, float dt, float4* __restrict__ lo,
                           float4* __restrict__ hi, unsigned* __restrict__ words) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float extent = i < b.count ? BoxOf(b, shape, dt, i, lo, hi) : -1.f;
    // the cell size follows the mean extent (any cell size gives the same
    // pairs); every lane reaches the warp sums
    const bool shaped = extent >= 0.f && isfinite(extent);
    float sum = shaped ? extent : 0.f;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    const unsigned count = __reduce_add_sync(0xffffffffu, shaped ? 1u : 0u);
    if ((threadIdx.x & 31) == 0 && count) {
        atomicAdd((float*)(words + kWExtent), sum);
        atomicAdd(words + kWShaped, count);
    }
}

__device__ __forceinline__ float CellSize(const unsigned* words) {
    const unsigned shaped = words[kWShaped];
    const float mean = shaped ? __uint_as_float(words[kWExtent]) / (float)shaped : 1.f;
    return mean > 0.f && isfinite(mean) ? 2.f * mean : 1.f;
}
__device__ __forceinline__ int CellOf(float x, float inv) { return (int)floorf(x * inv); }
// 10 bits per axis, wrapping: distinct cells far apart may share a code; the
// overlap test keeps that from making pairs, and a box spans at most two
// cells per axis, so it never meets the same code twice.
__device__ __forceinline__ unsigned CellCode(int x, int y, int z) {
    return ((unsigned)(x & 1023) << 20) | ((unsigned)(y & 1023) << 10) | (unsigned)(z & 1023);
}

// Cell entries of the bodies no wider than a cell; the wider ones to a list.
__global__ void k_bp_cells(const float4* __restrict__ lo, float4* __restrict__ hi, int n,
                           unsigned* __restrict__ words, unsigned long long* __restrict__ keys, unsigned keyCap,
                           int* __restrict__ wide, unsigned wideCap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 l = lo[i];
    float4 h = hi[i];
    if (__float_as_int(l.w) == 0) return;
    const float inv = 1.f / CellSize(words);
    const int x0 = CellOf(l.x, inv), x1 = CellOf(h.x, inv), y0 = CellOf(l.y, inv), y1 = CellOf(h.y, inv);
    const int z0 = CellOf(l.z, inv), z1 = CellOf(h.z, inv);
    // wide: more than two cells along an axis (or a box too far out for int cells)
    const bool inRange = fabsf(l.x * inv) < 1e9f && fabsf(l.y * inv) < 1e9f && fabsf(l.z * inv) < 1e9f &&
                         fabsf(h.x * inv) < 1e9f && fabsf(h.y * inv) < 1e9f && fabsf(h.z * inv) < 1e9f;
    if (!inRange || x1 - x0 > 1 || y1 - y0 > 1 || z1 - z0 > 1) {
        h.w = 1.f;  // marks the body wide for k_bp_wide_pairs
        hi[i] = h;
        const unsigned at = atomicAdd(words + kWWide, 1u);
        if (at < wideCap) wide[at] = i;
        return;
    }
    const int count = (x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1);
    unsigned at = atomicAdd(words + kWEntries, (unsigned)count);
    for (int x = x0; x <= x1; x++)
        for (int y = y0; y <= y1; y++)
            for (int z = z0; z <= z1; z++, at++)
                if (at < keyCap) keys[at] = ((unsigned long long)CellCode(x, y, z) << 32) | (unsigned)i;
}

__global__ void k_fill_keys(unsigned long long* __restrict__ keys, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = kNoKey;
}

// Bitonic stages with partner distance j >= kSortTile, one pair per thread.
__global__ void k_bitonic_global(unsigned long long* __restrict__ keys, int j, int k) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;  // pair index
    const unsigned i = 2 * t - (t & (j - 1));                   // lower element of the pair
    const unsigned l = i + j;
    const bool up = (i & k) == 0;
    const unsigned long long a = keys[i], b = keys[l];
    if ((a > b) == up) { keys[i] = b; keys[l] = a; }
}
// The stages of one k with j < kSortTile (all of them when k <= kSortTile: a
// whole tile sort), in shared memory; each block owns one tile.
__global__ void __launch_bounds__(kSortBlock) k_bitonic_tile(unsigned long long* __restrict__ keys, int kFrom,
                                                             int kTo, int jFrom) {
    __shared__ unsigned long long s[kSortTile];
    const unsigned base = blockIdx.x * kSortTile;
    const unsigned t = threadIdx.x;
    s[t] = keys[base + t];
    s[t + kSortBlock] = keys[base + t + kSortBlock];
    __syncthreads();
    for (int k = kFrom; k <= kTo; k <<= 1) {
        for (int j = (k == kFrom ? jFrom : k >> 1); j > 0; j >>= 1) {
            const unsigned i = 2 * t - (t & (j - 1));
            const unsigned l = i + j;
            const bool up = ((base + i) & k) == 0;
            const unsigned long long a = s[i], b = s[l];
            if ((a > b) == up) { s[i] = b; s[l] = a; }
            __syncthreads();
        }
    }
    keys[base + t] = s[t];
    keys[base + t + kSortBlock] = s[t + kSortBlock];
}

}  // namespace

// The power of two at or above n, at least one tile.
size_t PaddedSize(size_t n) {
    size_t p = kSortTile;
    while (p < n) p <<= 1;
    return p;
}

// Ascending bitonic sort of `padded` keys (a power of two, at least one
// tile): each tile sorted in shared memory, then for every larger k the wide
// stages in global memory and the narrow ones in shared memory.
void SortKeys(unsigned long long* keys, size_t padded, cudaStream_t st) {
    k_bitonic_tile<<<(unsigned)(padded / kSortTile), kSortBlock, 0, st>>>(keys, 2, kSortTile, 1);
    for (size_t k = 2 * kSortTile; k <= padded; k <<= 1) {
        for (size_t j = k >> 1; j >= kSortTile; j >>= 1)
            k_bitonic_global<<<(unsigned)(padded / 2 / 256), 256, 0, st>>>(keys, (int)j, (int)k);
        k_bitonic_tile<<<(unsigned)(padded / kSortTile), kSortBlock, 0, st>>>(keys, (int)k, (int)k, kSortTile / 2);
    }
}

// keys[0, n) set to the largest key (sorts last).
void FillKeys(unsigned long long* keys, size_t n, cudaStream_t st) {
    if (n) k_fill_keys<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(keys, n);
}

namespace {

// BoundingBox.Intersects (BoundingBox.cs:58-66) and the NoBroadPhase rule of
// two kinematic bodies.
__device__ __forceinline__ bool MakesPair(float4 la, float4 ha, float4 lb, float4 hb) {
    if (__float_as_int(la.w) == 1 && __float_as_int(lb.w) == 1) return false;
    if (lb.x > ha.x || lb.y > ha.y || lb.z > ha.z) return false;
    if (la.x > hb.x || la.y > hb.y || la.z > hb.z) return false;
    return true;
}
__device__ __forceinline__ void Report(int a, int b, unsigned long long* __restrict__ pairs, unsigned capacity,
                                       unsigned* __restrict__ count) {
    const unsigned at = atomicAdd(count, 1u);
    if (at < capacity) pairs[at] = ((unsigned long long)min(a, b) << 32) | (unsigned)max(a, b);
}

// One thread per sorted cell entry: the later entries of the same cell.
__global__ void k_bp_cell_pairs(const unsigned long long* __restrict__ keys, unsigned entries,
                                const float4* __restrict__ lo, const float4* __restrict__ hi,
                                const unsigned* __restrict__ words, unsigned long long* __restrict__ pairs,
                                unsigned capacity, unsigned* __restrict__ count) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= entries) return;
    const unsigned long long ki = keys[i];
    const unsigned code = (unsigned)(ki >> 32);
    const int a = (int)(ki & 0xffffffffu);
    const float4 la = lo[a], ha = hi[a];
    const float inv = 1.f / CellSize(words);
    for (unsigned j = i + 1; j < entries; j++) {
        const unsigned long long kj = keys[j];
        if ((unsigned)(kj >> 32) != code) break;
        const int b = (int)(kj & 0xffffffffu);
        const float4 lb = lo[b], hb = hi[b];
        if (!MakesPair(la, ha, lb, hb)) continue;
        // report in the cell of the largest corner of the minima only
        const unsigned home = CellCode(CellOf(fmaxf(la.x, lb.x), inv), CellOf(fmaxf(la.y, lb.y), inv),
                                       CellOf(fmaxf(la.z, lb.z), inv));
        if (home == code) Report(a, b, pairs, capacity, count);
    }
}

// One thread per (wide body, body): wide bodies against every other body
// (a pair of two wide bodies from the lower one only).
__global__ void k_bp_wide_pairs(const int* __restrict__ wide, unsigned wideCount, int n,
                                const float4* __restrict__ lo, const float4* __restrict__ hi,
                                const unsigned* __restrict__ words, unsigned long long* __restrict__ pairs,
                                unsigned capacity, unsigned* __restrict__ count) {
    const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (unsigned long long)wideCount * n) return;
    const int w = wide[t / n], b = (int)(t % n);
    if (b == w) return;
    const float4 lb = lo[b], hb = hi[b];
    if (__float_as_int(lb.w) == 0) return;
    const float4 la = lo[w], ha = hi[w];
    if (hb.w != 0.f && b < w) return;  // two wide bodies: from the lower one
    if (MakesPair(la, ha, lb, hb)) Report(w, b, pairs, capacity, count);
}

}  // namespace

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            ctx->SetError("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return BEPUGPU_CUDA_ERROR;                                                        \
        }                                                                                     \
    } while (0)

// Device buffers of a scene's broad phase, grown as needed.
struct BroadPhaseBuffers {
    float4 *lo = nullptr, *hi = nullptr;
    int* wide = nullptr;
    unsigned long long* keys = nullptr;   // cell entries
    unsigned long long* pairs = nullptr;  // (lower << 32) | higher, then sorted
    unsigned* words = nullptr;
    size_t bodyCap = 0, keyCap = 0, pairCap = 0;
    ~BroadPhaseBuffers() {
        cudaFree(lo);
        cudaFree(hi);
        cudaFree(wide);
        cudaFree(keys);
        cudaFree(pairs);
        cudaFree(words);
    }
};

void ReleaseBroadPhase(Scene* s) {
    delete s->broadPhase;
    s->broadPhase = nullptr;
}

namespace {
template <class T>
cudaError_t Grow(T*& p, size_t& cap, size_t want) {
    if (cap >= want) return cudaSuccess;
    cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * want);
    if (e == cudaSuccess) cap = want;
    return e;
}
}  // namespace

}  // namespace bepugpu

using namespace bepugpu;

namespace bepugpu {
// The broad phase of scene s into s->broadPhase->pairs: `found` keys
// (lower << 32 | higher), ascending.  The stream is synchronised.
bepugpu_status RunBroadPhase(Context* ctx, Scene* s, float dt, unsigned& found) {
    found = 0;
    const int n = s->b.count;
    if ((size_t)n != s->hostShapes.size()) {
        ctx->SetError("broad_phase needs one shape for each of the %d bodies (bepugpu_upload_shapes)", n);
        return BEPUGPU_INVALID_OPERATION;
    }
    if (n < 2) return BEPUGPU_OK;
    if (s->asyncPending) {
        CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
    }
    if (!s->broadPhase) s->broadPhase = new BroadPhaseBuffers();
    BroadPhaseBuffers& bp = *s->broadPhase;
    size_t wideCap = bp.bodyCap;
    if (bp.bodyCap < (size_t)n) {
        size_t c1 = bp.bodyCap, c2 = bp.bodyCap, c3 = bp.bodyCap;
        CK(Grow(bp.lo, c1, (size_t)n));
        CK(Grow(bp.hi, c2, (size_t)n));
        CK(Grow(bp.wide, c3, (size_t)n));
        bp.bodyCap = n;
        wideCap = n;
    }
    size_t wordsCap = bp.words ? kWords : 0;
    CK(Grow(bp.words, wordsCap, (size_t)kWords));
    CK(Grow(bp.keys, bp.keyCap, PaddedSize((size_t)8 * n)));  // at most eight cells a body
    CK(Grow(bp.pairs, bp.pairCap, PaddedSize((size_t)4 * n)));
    const cudaStream_t st = s->stream;
    CK(cudaMemsetAsync(bp.words, 0, sizeof(unsigned) * kWords, st));
    k_bp_boxes<<<(n + 255) / 256, 256, 0, st>>>(s->b, s->shape, dt, bp.lo, bp.hi, bp.words);
    k_bp_cells<<<(n + 255) / 256, 256, 0, st>>>(bp.lo, bp.hi, n, bp.words, bp.keys, (unsigned)bp.keyCap, bp.wide,
                                               (unsigned)wideCap);
    unsigned w[kWords];
    CK(cudaMemcpyAsync(w, bp.words, sizeof(w), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const unsigned entries = w[kWEntries], wideCount = std::min<unsigned>(w[kWWide], (unsigned)wideCap);
    const size_t sortedEntries = PaddedSize(entries);
    if (entries < sortedEntries)
        k_fill_keys<<<(unsigned)((sortedEntries - entries + 255) / 256), 256, 0, st>>>(bp.keys + entries,
                                                                                    sortedEntries - entries);
    SortKeys(bp.keys, sortedEntries, st);
    CK(cudaGetLastError());
    for (int attempt = 0; attempt < 2; attempt++) {
        CK(cudaMemsetAsync(bp.words + kWPairs, 0, sizeof(unsigned), st));
        if (entries)
            k_bp_cell_pairs<<<(entries + 127) / 128, 128, 0, st>>>(bp.keys, entries, bp.lo, bp.hi, bp.words,
                                                                  bp.pairs, (unsigned)bp.pairCap,
                                                                  bp.words + kWPairs);
        const unsigned long long wideWork = (unsigned long long)wideCount * n;
        if (wideWork)
            k_bp_wide_pairs<<<(unsigned)((wideWork + 255) / 256), 256, 0, st>>>(
                bp.wide, wideCount, n, bp.lo, bp.hi, bp.words, bp.pairs, (unsigned)bp.pairCap, bp.words + kWPairs);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&found, bp.words + kWPairs, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (PaddedSize(found) <= bp.pairCap) break;
        CK(Grow(bp.pairs, bp.pairCap, PaddedSize(found)));  // too many pairs for the buffer: grow, test again
    }
    // the pairs in ascending order: pad with the largest key and sort
    const size_t sortedPairs = PaddedSize(found);
    if (found) {
        if (sortedPairs > found)
            k_fill_keys<<<(unsigned)((sortedPairs - found + 255) / 256), 256, 0, st>>>(bp.pairs + found,
                                                                                      sortedPairs - found);
        SortKeys(bp.pairs, sortedPairs, st);
        CK(cudaGetLastError());
    }
    return BEPUGPU_OK;
}

const unsigned long long* BroadPhasePairs(const Scene* s) { return s->broadPhase ? s->broadPhase->pairs : nullptr; }
}  // namespace bepugpu

extern "C" bepugpu_status bepugpu_broad_phase(bepugpu_context* c, int32_t id, float dt, int32_t* pairs,
                                              uint32_t max_pairs, uint32_t* pair_count) {
    NvtxRange range("bepugpu_broad_phase");
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (!pair_count || (max_pairs && !pairs) || !(dt >= 0) || !std::isfinite(dt)) {
        ctx->SetError("broad_phase: pair_count is required, pairs when max_pairs > 0, and dt >= 0 finite");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    *pair_count = 0;
    unsigned found = 0;
    bepugpu_status bst = RunBroadPhase(ctx, s, dt, found);
    if (bst != BEPUGPU_OK) return bst;
    if (!found) return BEPUGPU_OK;
    const cudaStream_t st = s->stream;
    BroadPhaseBuffers& bp = *s->broadPhase;
    const uint32_t nw = std::min<uint32_t>(found, max_pairs);
    std::vector<unsigned long long> host(nw);
    if (nw) {
        CK(cudaMemcpyAsync(host.data(), bp.pairs, sizeof(unsigned long long) * nw, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    for (uint32_t k = 0; k < nw; k++) {
        pairs[2 * k] = (int32_t)(host[k] >> 32);
        pairs[2 * k + 1] = (int32_t)(host[k] & 0xffffffffu);
    }
    *pair_count = found;
    return BEPUGPU_OK;
}
