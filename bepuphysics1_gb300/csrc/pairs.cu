// The narrow phase's pair bookkeeping on the device: the manifold list of a
// scene follows the broad phase's pair set without a host round trip, as the
// reference's NarrowPhase keeps a pair handler per overlap
// (NarrowPhaseSystems/NarrowPhase.cs:143-178 adds one for a new overlap,
// :254-332 drops a pair whose boxes stopped overlapping), and the solver list
// is recoloured on the device.
//
//   1. the broad phase leaves the pair keys sorted in device memory;
//   2. each record looks its pair up in them (kept or dropped), each pair
//      looks itself up in the sorted old keys (kept or new);
//   3. prefix sums give the new list: the kept records in their order, then
//      the new pairs ascending;
//   4. the colouring -- the smallest colour no earlier entry sharing a dynamic
//      body took, the host's greedy colouring in list order -- runs as rounds
//      of Jones-Plassmann with the list index as priority: an entry takes its
//      colour once the entries before it at each of its dynamic bodies have
//      theirs, which is exactly the greedy choice;
//   5. slots follow the colour-major order (a sort of (colour, index) keys) and
//      the records' lanes move to them, new records start empty.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "scan_device.cuh"
#include "solver_device.cuh"

namespace bepugpu {

// Device buffers of bepugpu_update_pairs, grown as needed.
struct PairBuffers {
    float4* material = nullptr;  // per body: kinetic, static friction, bounciness
    int32_t materialCount = 0;
    void* block = nullptr;
    size_t blockBytes = 0;
    ~PairBuffers() {
        cudaFree(material);
        cudaFree(block);
    }
};

void ReleasePairs(Scene* s) {
    delete s->pairs;
    s->pairs = nullptr;
}

namespace {

constexpr int kScanBlock = 256, kScanItems = 4, kScanTile = kScanBlock * kScanItems;
constexpr int kLanes = 25;  // head, cpos x4, cnrm x4, offA x4, offB x4, mat, penacc, fricacc, saxis, cfr x4

// Exclusive scan of one tile per block; tile totals to sums.
__global__ void k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, int n, int* __restrict__ sums) {
    __shared__ int warpSums[32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems], t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        t += v[k];
    }
    const int incl = BlockInclusiveSum(t, warpSums);
    int run = incl - t;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == blockDim.x - 1) sums[blockIdx.x] = incl;
}
__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ sums) {
    const int i = blockIdx.x * kScanTile + threadIdx.x;
    const int add = sums[blockIdx.x];
    for (int k = 0; k < kScanItems; k++) {
        const int j = i + k * kScanBlock;
        if (j < n) out[j] += add;
    }
}

// 64-bit key of a pair: lower body << 32 | higher body.
__device__ __forceinline__ unsigned long long PairKey(int a, int b) {
    const int lo = min(a, b), hi = max(a, b);
    return ((unsigned long long)(unsigned)lo << 32) | (unsigned)hi;
}
__device__ __forceinline__ bool Contains(const unsigned long long* __restrict__ keys, int n, unsigned long long k) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && keys[lo] == k;
}

// Old records: their keys in record order and a copy to sort.
__global__ void k_old_keys(ManifoldSoA m, const int32_t* __restrict__ slotOf, int n, unsigned long long* key,
                           unsigned long long* sorted) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int4 h = m.head[slotOf[r]];
    key[r] = sorted[r] = PairKey(h.x, h.y);
}
// kept[r]: record r's pair is still reported; fresh[p]: pair p is new.
__global__ void k_membership(const unsigned long long* __restrict__ oldKey, int nOld,
                             const unsigned long long* __restrict__ oldSorted, const unsigned long long* __restrict__ pairs,
                             int nPairs, int* kept, int* fresh) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nOld) kept[t] = Contains(pairs, nPairs, oldKey[t]) ? 1 : 0;
    if (t < nPairs) fresh[t] = Contains(oldSorted, nOld, pairs[t]) ? 0 : 1;
}

// The new list: record i's bodies (A, B as the record keeps them), its flags
// and its old slot (-1 for a new pair).
struct NewRecords {
    int2* ends;
    uint32_t* flags;
    int32_t* oldSlot;
};
__global__ void k_list_kept(ManifoldSoA m, const int32_t* __restrict__ slotOf, int nOld, const int* __restrict__ kept,
                            const int* __restrict__ keptAt, NewRecords out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nOld || !kept[r]) return;
    const int s = slotOf[r], i = keptAt[r];
    const int4 h = m.head[s];
    out.ends[i] = make_int2(h.x, h.y);
    out.flags[i] = (uint32_t)h.z >> 8;
    out.oldSlot[i] = s;
}
// A new pair's record: the box first in a box-sphere pair (BoxSpherePairHandler),
// NONCONVEX for a pair with a sphere (SpherePairHandler.cs:28, BoxSpherePairHandler.cs:28).
__global__ void k_list_fresh(const unsigned long long* __restrict__ pairs, int nPairs, const int* __restrict__ fresh,
                             const int* __restrict__ freshAt, int kept, const float4* __restrict__ shape,
                             NewRecords out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs || !fresh[p]) return;
    int a = (int)(pairs[p] >> 32), b = (int)(pairs[p] & 0xffffffffu);
    const int ta = __float_as_int(shape[a].w), tb = __float_as_int(shape[b].w);
    if (ta == BEPUGPU_SHAPE_SPHERE && tb == BEPUGPU_SHAPE_BOX) {
        const int t = a;
        a = b;
        b = t;
    }
    const bool sphere = ta == BEPUGPU_SHAPE_SPHERE || tb == BEPUGPU_SHAPE_SPHERE;
    const int i = kept + freshAt[p];
    out.ends[i] = make_int2(a, b);
    out.flags[i] = BEPUGPU_MANIFOLD_ACTIVE | BEPUGPU_MANIFOLD_SOLVER_RULE | BEPUGPU_MANIFOLD_GENERATED |
                   (sphere ? BEPUGPU_MANIFOLD_NONCONVEX : 0u);
    out.oldSlot[i] = -1;
}

// Colouring.  entries: (dynamic body << 32 | entry) for each dynamic end of
// each entry, sorted; at[i]: the entry's positions there for its ends A and
// B, -1 for an end without a dynamic body.
__global__ void k_colour_entries(const int2* __restrict__ ends, int n, BodySoA b, unsigned long long* entries,
                                 int* colour) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 e = ends[i];
    const bool da = e.x >= 0 && b.pos[e.x].w != 0.f, db = e.y >= 0 && b.pos[e.y].w != 0.f;
    entries[2 * i] = da ? ((unsigned long long)(unsigned)e.x << 32) | (unsigned)i : ~0ull;
    entries[2 * i + 1] = db ? ((unsigned long long)(unsigned)e.y << 32) | (unsigned)i : ~0ull;
    colour[i] = -1;
}
__global__ void k_colour_positions(const unsigned long long* __restrict__ entries, int count, const int2* __restrict__ ends,
                                   int2* at) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const unsigned long long key = entries[k];
    if (key == ~0ull) return;
    const int body = (int)(key >> 32), i = (int)(key & 0xffffffffu);
    if (ends[i].x == body) at[i].x = k;
    else at[i].y = k;
}
// One round: an entry whose predecessors at both dynamic bodies are coloured
// takes the smallest colour none of its predecessors has.
__global__ void k_colour_round(const unsigned long long* __restrict__ entries, const int2* __restrict__ at, int n,
                               int* colour, int* waiting) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || colour[i] >= 0) return;
    const int2 pos = at[i];
    const int ks[2] = {pos.x, pos.y};
    for (int e = 0; e < 2; e++) {
        const int k = ks[e];
        if (k <= 0) continue;
        if ((entries[k - 1] >> 32) != (entries[k] >> 32)) continue;
        if (((volatile int*)colour)[(int)(entries[k - 1] & 0xffffffffu)] < 0) {
            atomicAdd(waiting, 1);
            return;
        }
    }
    for (int base = 0;; base += 64) {
        unsigned long long used = 0;
        for (int e = 0; e < 2; e++) {
            const int k = ks[e];
            if (k < 0) continue;
            const unsigned long long body = entries[k] >> 32;
            for (int q = k - 1; q >= 0 && (entries[q] >> 32) == body; q--) {
                const int c = colour[(int)(entries[q] & 0xffffffffu)] - base;
                if (c >= 0 && c < 64) used |= 1ull << c;
            }
        }
        if (used != ~0ull) {
            colour[i] = base + __ffsll((long long)~used) - 1;
            return;
        }
    }
}
__global__ void k_colour_count(const int* __restrict__ colour, int n, int* counts, int* maxColour) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicAdd(counts + colour[i], 1);
    atomicMax(maxColour, colour[i]);
}
__global__ void k_slot_keys(const int* __restrict__ colour, int n, unsigned long long* keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = ((unsigned long long)(unsigned)colour[i] << 32) | (unsigned)i;
}
__global__ void k_slots(const unsigned long long* __restrict__ keys, int n, int* slotOf, int* order) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = (int)(keys[k] & 0xffffffffu);
    slotOf[i] = k;
    order[k] = i;
}

// A record's input lanes at its new slot of the scratch copy (capacity n):
// a kept record's lanes as a download and upload would carry them, a new
// record's empty with the blended material (MaterialManager.cs:77-85).
__global__ void k_move_lanes(ManifoldSoA m, NewRecords rec, const int* __restrict__ newSlot, int n,
                             const float4* __restrict__ material, float4* scratch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int ns = newSlot[i], os = rec.oldSlot[i], cap = m.capacity;
    const int2 e = rec.ends[i];
    const uint32_t flags = rec.flags[i];
    float4* L = scratch;
    auto at = [&](int lane) -> float4& { return L[(size_t)lane * n + ns]; };
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    if (os < 0) {
        at(0) = make_float4(__int_as_float(e.x), __int_as_float(e.y), __int_as_float((int)(flags << 8)),
                            __int_as_float(i));
        for (int lane = 1; lane < kLanes; lane++) at(lane) = zero;
        const float4 ma = material[e.x], mb = material[e.y];
        at(17) = make_float4(ma.x * mb.x, ma.y * mb.y, ma.z * mb.z, 0.f);
        return;
    }
    const int4 h = m.head[os];
    const int count = h.z & 0xff;
    at(0) = make_float4(__int_as_float(h.x), __int_as_float(h.y), __int_as_float(h.z), __int_as_float(i));
    const bool nonConvex = flags & BEPUGPU_MANIFOLD_NONCONVEX;
    for (int k = 0; k < 4; k++) {
        const bool live = k < count;
        const float4 ob = m.offB[k * cap + os];
        at(1 + k) = live ? m.cpos[k * cap + os] : zero;
        at(5 + k) = live ? m.cnrm[k * cap + os] : zero;
        at(9 + k) = live ? m.offA[k * cap + os] : zero;
        at(13 + k) = live ? make_float4(ob.x, ob.y, ob.z, 0.f) : zero;
        at(21 + k) = live && nonConvex ? m.cfr[k * cap + os] : zero;
    }
    const float4 mat = m.mat[os], pa = m.penacc[os], f = m.fricacc[os], ax = m.saxis[os];
    at(17) = make_float4(mat.x, mat.y, mat.z, 0.f);
    at(18) = make_float4(count > 0 ? pa.x : 0.f, count > 1 ? pa.y : 0.f, count > 2 ? pa.z : 0.f,
                         count > 3 ? pa.w : 0.f);
    at(19) = make_float4(count > 0 ? f.x : 0.f, count > 0 ? f.y : 0.f, count > 0 ? f.z : 0.f, f.w);
    at(20) = make_float4(ax.x, ax.y, ax.z, 0.f);
}
// The scratch copy back into the scene's lanes, slots [0, n).
__global__ void k_lanes_back(ManifoldSoA m, const float4* __restrict__ scratch, int n, int32_t* genSlots) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int cap = m.capacity;
    auto L = [&](int lane) { return scratch[(size_t)lane * n + s]; };
    const float4 h = L(0);
    m.head[s] = make_int4(__float_as_int(h.x), __float_as_int(h.y), __float_as_int(h.z), __float_as_int(h.w));
    for (int k = 0; k < 4; k++) {
        m.cpos[k * cap + s] = L(1 + k);
        m.cnrm[k * cap + s] = L(5 + k);
        m.offA[k * cap + s] = L(9 + k);
        m.offB[k * cap + s] = L(13 + k);
        m.cfr[k * cap + s] = L(21 + k);
    }
    m.mat[s] = L(17);
    m.penacc[s] = L(18);
    m.fricacc[s] = L(19);
    m.saxis[s] = L(20);
    m.state[s] = make_uint2(0u, 0u);
    genSlots[s] = s;
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

namespace {

// Exclusive scan of n ints (in and out may not alias); *total receives the sum.
bepugpu_status ExclusiveScan(Context* ctx, const int* in, int* out, int n, int* scratch, int* total, cudaStream_t st) {
    if (n <= 0) {
        CK(cudaMemsetAsync(total, 0, sizeof(int), st));
        return BEPUGPU_OK;
    }
    const int tiles = (n + kScanTile - 1) / kScanTile;
    int* sums = scratch;
    k_scan_tiles<<<tiles, kScanBlock, 0, st>>>(in, out, n, sums);
    CK(cudaGetLastError());
    if (tiles == 1) {
        CK(cudaMemcpyAsync(total, sums, sizeof(int), cudaMemcpyDeviceToDevice, st));
        return BEPUGPU_OK;
    }
    int* scanned = sums + tiles;
    bepugpu_status r = ExclusiveScan(ctx, sums, scanned, tiles, scanned + tiles, total, st);
    if (r != BEPUGPU_OK) return r;
    k_scan_add<<<tiles, kScanBlock, 0, st>>>(out, n, scanned);
    CK(cudaGetLastError());
    return BEPUGPU_OK;
}

// Bump allocator over one block of device memory.
struct Carve {
    char* base;
    size_t used = 0;
    template <class T>
    T* take(size_t count) {
        T* p = (T*)(base + used);
        used += (count * sizeof(T) + 255) & ~(size_t)255;
        return p;
    }
};

}  // namespace

// The colouring of n entries with ends[] (host-side greedy rule, on the
// device): colour[i], order (colour-major, list order inside a colour),
// per-colour offsets into order.  Needs the buffers of one call.
struct DeviceColouring {
    int* colour;
    int* order;
    int* slotOf;
    int colours = 0;
    std::vector<int32_t> offsets;
};

static bepugpu_status ColourOnDevice(Context* ctx, Scene* s, const int2* ends, int n, Carve& c, DeviceColouring& out) {
    const cudaStream_t st = s->stream;
    const int T = 256;
    out.colour = c.take<int>(n);
    out.order = c.take<int>(n);
    out.slotOf = c.take<int>(n);
    out.colours = 0;
    out.offsets.assign(1, 0);
    if (n == 0) return BEPUGPU_OK;
    const size_t padded = PaddedSize((size_t)2 * n);
    auto* entries = c.take<unsigned long long>(padded);
    auto* at = c.take<int2>(n);
    int* counters = c.take<int>(64);
    k_colour_entries<<<(n + T - 1) / T, T, 0, st>>>(ends, n, s->b, entries, out.colour);
    FillKeys(entries + 2 * (size_t)n, padded - 2 * (size_t)n, st);
    SortKeys(entries, padded, st);
    CK(cudaMemsetAsync(at, 0xff, sizeof(int2) * n, st));
    k_colour_positions<<<(int)((2 * (size_t)n + T - 1) / T), T, 0, st>>>(entries, 2 * n, ends, at);
    CK(cudaGetLastError());
    // Rounds in batches of 16.  An entry still waiting counts itself; a round
    // with none waiting leaves every entry coloured (the ready ones took their
    // colours in it), so a batch whose last count is zero ends the loop.
    // Each round colours at least the lowest uncoloured entry: n rounds suffice.
    constexpr int kBatch = 16;
    for (int round = 0;; round += kBatch) {
        if (round > n + kBatch) {
            ctx->SetError("update_pairs: the colouring did not finish");
            return BEPUGPU_CUDA_ERROR;
        }
        CK(cudaMemsetAsync(counters, 0, sizeof(int) * kBatch, st));
        for (int k = 0; k < kBatch; k++)
            k_colour_round<<<(n + T - 1) / T, T, 0, st>>>(entries, at, n, out.colour, counters + k);
        CK(cudaGetLastError());
        int waiting = 0;
        CK(cudaMemcpyAsync(&waiting, counters + kBatch - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (waiting == 0) break;
    }
    // colour counts and offsets
    int* counts = c.take<int>(n + 1);
    int* maxColour = counters + 32;
    CK(cudaMemsetAsync(counts, 0, sizeof(int) * (n + 1), st));
    CK(cudaMemsetAsync(maxColour, 0, sizeof(int), st));
    k_colour_count<<<(n + T - 1) / T, T, 0, st>>>(out.colour, n, counts, maxColour);
    int top = 0;
    CK(cudaMemcpyAsync(&top, maxColour, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    out.colours = top + 1;
    std::vector<int32_t> hc(out.colours);
    CK(cudaMemcpyAsync(hc.data(), counts, sizeof(int) * out.colours, cudaMemcpyDeviceToHost, st));
    // slots: (colour, entry) keys sorted
    const size_t paddedSlots = PaddedSize((size_t)n);
    auto* keys = c.take<unsigned long long>(paddedSlots);
    k_slot_keys<<<(n + T - 1) / T, T, 0, st>>>(out.colour, n, keys);
    FillKeys(keys + n, paddedSlots - n, st);
    SortKeys(keys, paddedSlots, st);
    k_slots<<<(n + T - 1) / T, T, 0, st>>>(keys, n, out.slotOf, out.order);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    out.offsets.assign(out.colours + 1, 0);
    for (int k = 0; k < out.colours; k++) out.offsets[k + 1] = out.offsets[k] + hc[k];
    return BEPUGPU_OK;
}

}  // namespace bepugpu

using namespace bepugpu;

extern "C" bepugpu_status bepugpu_set_materials(bepugpu_context* c, int32_t id, const float* materials,
                                                uint32_t count) {
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (count != (uint32_t)s->b.count || (count && !materials)) {
        ctx->SetError("set_materials: three floats for each of the %d bodies", s->b.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (!s->pairs) s->pairs = new PairBuffers();
    PairBuffers& P = *s->pairs;
    if (P.materialCount < (int32_t)count) {
        cudaFree(P.material);
        P.material = nullptr;
        P.materialCount = 0;
        CK(cudaMalloc(&P.material, sizeof(float4) * std::max<uint32_t>(count, 1)));
        P.materialCount = (int32_t)count;
    }
    std::vector<float4> h(count);
    for (uint32_t i = 0; i < count; i++) h[i] = make_float4(materials[3 * i], materials[3 * i + 1], materials[3 * i + 2], 0.f);
    if (count) CK(cudaMemcpyAsync(P.material, h.data(), sizeof(float4) * count, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return BEPUGPU_OK;
}

extern "C" bepugpu_status bepugpu_update_pairs(bepugpu_context* c, int32_t id, float dt, uint32_t* manifold_count) {
    NvtxRange range("bepugpu_update_pairs");
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (!(dt >= 0) || !std::isfinite(dt)) {
        ctx->SetError("update_pairs: dt must be >= 0 and finite");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (s->jointCount != 0 || s->generatedCount != s->m.count) {
        ctx->SetError("update_pairs: the scene's constraints must all be GENERATED manifolds");
        return BEPUGPU_INVALID_OPERATION;
    }
    if (!s->pairs || s->pairs->materialCount < s->b.count) {
        ctx->SetError("update_pairs: set the bodies' materials first (bepugpu_set_materials)");
        return BEPUGPU_INVALID_OPERATION;
    }
    unsigned found = 0;
    bepugpu_status st0 = RunBroadPhase(ctx, s, dt, found);
    if (st0 != BEPUGPU_OK) return st0;
    const int nPairs = (int)found, nOld = s->m.count;
    if ((uint32_t)nPairs > s->maxManifolds) {
        ctx->SetError("update_pairs: %d pairs exceed the scene's capacity of %u manifolds", nPairs, s->maxManifolds);
        return BEPUGPU_INVALID_OPERATION;
    }
    const unsigned long long* pairs = BroadPhasePairs(s);
    const cudaStream_t st = s->stream;
    PairBuffers& P = *s->pairs;
    // scratch: keys, flags and scans, the new list, the colouring, the moved lanes
    const int nMax = std::max(std::max(nPairs, nOld), 1);
    const size_t want = 256 * 64 + sizeof(unsigned long long) * (2 * (size_t)nMax + PaddedSize(nMax) +
                                                               PaddedSize(2 * (size_t)nMax) + PaddedSize(nMax)) +
                        sizeof(int) * (14 * (size_t)nMax + 64) + sizeof(float4) * kLanes * (size_t)nMax +
                        sizeof(int2) * 2 * (size_t)nMax;
    if (P.blockBytes < want) {
        cudaFree(P.block);
        P.block = nullptr;
        P.blockBytes = 0;
        const size_t bytes = want + want / 4;
        cudaError_t e = cudaMalloc(&P.block, bytes);
        if (e != cudaSuccess) {
            ctx->SetError("update_pairs: %zu bytes of scratch: %s", bytes, cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? BEPUGPU_OUT_OF_MEMORY : BEPUGPU_CUDA_ERROR;
        }
        P.blockBytes = bytes;
    }
    Carve cv{(char*)P.block};
    const int T = 256;
    auto* oldKey = cv.take<unsigned long long>(nMax);
    const size_t paddedOld = PaddedSize(nMax);
    auto* oldSorted = cv.take<unsigned long long>(paddedOld);
    int* kept = cv.take<int>(nMax);
    int* keptAt = cv.take<int>(nMax);
    int* fresh = cv.take<int>(nMax);
    int* freshAt = cv.take<int>(nMax);
    int* scanScratch = cv.take<int>(2 * (size_t)nMax + 64);
    int* totals = cv.take<int>(2);
    NewRecords rec{cv.take<int2>(nMax), cv.take<uint32_t>(nMax), cv.take<int32_t>(nMax)};
    if (nOld) {
        k_old_keys<<<(nOld + T - 1) / T, T, 0, st>>>(s->m, s->slotOf, nOld, oldKey, oldSorted);
        FillKeys(oldSorted + nOld, paddedOld - nOld, st);
        SortKeys(oldSorted, paddedOld, st);
    }
    const int nt = std::max(nOld, nPairs);
    if (nt) k_membership<<<(nt + T - 1) / T, T, 0, st>>>(oldKey, nOld, oldSorted, pairs, nPairs, kept, fresh);
    CK(cudaGetLastError());
    bepugpu_status sr = ExclusiveScan(ctx, kept, keptAt, nOld, scanScratch, totals, st);
    if (sr != BEPUGPU_OK) return sr;
    sr = ExclusiveScan(ctx, fresh, freshAt, nPairs, scanScratch, totals + 1, st);
    if (sr != BEPUGPU_OK) return sr;
    int tot[2] = {0, 0};
    CK(cudaMemcpyAsync(tot, totals, sizeof(tot), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const int nKept = tot[0], n = tot[0] + tot[1];
    if (n != nPairs) {
        ctx->SetError("update_pairs: %d kept and %d new records for %d pairs", tot[0], tot[1], nPairs);
        return BEPUGPU_CUDA_ERROR;
    }
    if (nOld) k_list_kept<<<(nOld + T - 1) / T, T, 0, st>>>(s->m, s->slotOf, nOld, kept, keptAt, rec);
    if (nPairs)
        k_list_fresh<<<(nPairs + T - 1) / T, T, 0, st>>>(pairs, nPairs, fresh, freshAt, nKept, s->shape, rec);
    CK(cudaGetLastError());
    DeviceColouring col;
    sr = ColourOnDevice(ctx, s, rec.ends, n, cv, col);
    if (sr != BEPUGPU_OK) return sr;
    auto* scratch = cv.take<float4>((size_t)kLanes * nMax);
    if (cv.used > P.blockBytes) {
        ctx->SetError("update_pairs: scratch overrun (%zu of %zu bytes)", cv.used, P.blockBytes);
        return BEPUGPU_CUDA_ERROR;
    }
    if (n) {
        k_move_lanes<<<(n + T - 1) / T, T, 0, st>>>(s->m, rec, col.slotOf, n, P.material, scratch);
        k_lanes_back<<<(n + T - 1) / T, T, 0, st>>>(s->m, scratch, n, s->genSlotsDev);
        CK(cudaMemcpyAsync(s->slotOf, col.slotOf, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    }
    CK(cudaGetLastError());
    // the scene's bookkeeping: every manifold on the colour-sweep path
    if (s->islands) ReleaseIslands(s);
    const bool hadGroups = !s->groupPlan.groups.empty();
    GroupPlan& plan = s->groupPlan;
    plan = GroupPlan();
    plan.globalOffsets = col.offsets;
    plan.globalCount = n;
    plan.jointGlobalOffsets.assign(col.colours + 1, 0);
    plan.slotOf.resize(n);
    plan.jointSlotOf.clear();
    s->colouring.colours = col.colours;
    s->colouring.colour.resize(n);
    s->colouring.order.resize(n);
    s->colouring.offsets = col.offsets;
    if (n) {
        CK(cudaMemcpyAsync(s->colouring.colour.data(), col.colour, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(s->colouring.order.data(), col.order, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(plan.slotOf.data(), col.slotOf, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    }
    s->manifoldOffsets = col.offsets;
    s->jointOffsets.assign(col.colours + 1, 0);
    s->hostSlotOf = plan.slotOf;
    s->m.count = n;
    s->generatedCount = n;
    s->hostGenPairs.clear();  // the shapes' pair check of bepugpu_upload_shapes applies to uploaded records only
    CK(cudaMemcpyAsync(s->colourOffsetsDev, col.offsets.data(), sizeof(int32_t) * col.offsets.size(),
                       cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    if (hadGroups) {  // the bodies groups stepped go back to the sweep path's body stages
        s->hostOwned.assign(s->b.count, 0);
        s->dampDirty = true;
        bepugpu_status rs = s->RebuildSweepBodies(ctx);
        if (rs != BEPUGPU_OK) return rs;
    }
    s->version++;
    if (manifold_count) *manifold_count = (uint32_t)n;
    return BEPUGPU_OK;
}
