// Island groups: whole steps of small simulation islands inside one CTA.
//
// An island is a set of dynamic bodies connected through constraints
// (kinematic bodies do not connect, as in the reference's simulation islands,
// DeactivationManagement/SimulationIslandMember.cs).  Constraints of different
// islands never share a dynamic body, so the solver's colour-ordered sequence
// restricted to one island is that island's own Gauss-Seidel sequence and
// islands can run in any interleaving.  Islands small enough to keep their
// bodies in shared memory are packed into groups; one CTA runs a group's whole
// step -- refresh, force update, prestep, warm start, every colour sweep of
// every iteration, position update -- with block barriers between sweeps
// instead of grid-wide ones.  When the group's solve lanes (Jacobians,
// friction lanes, impulses, state) fit too, the prestep writes them to shared
// memory and the sweeps never touch global memory for them.  Larger islands
// stay on the colour-sweep path.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "solver_device.cuh"

namespace bepugpu {

// Body view of a group kernel.  Refs >= 0 are the group's bodies in shared
// memory, -1 is "no entity", refs <= -2 name global body -2 - ref (kinematic
// bodies, read only).
struct GroupBodies {
    float4 *pos, *quat, *vlin, *vang, *inv0, *inv1;
    BodySoA g;
    __device__ __forceinline__ float4 Pos(int r) const { return r >= 0 ? pos[r] : g.pos[-2 - r]; }
    __device__ __forceinline__ float4 Quat(int r) const { return r >= 0 ? quat[r] : g.quat[-2 - r]; }
    __device__ __forceinline__ float4 Vlin(int r) const { return r >= 0 ? vlin[r] : g.vlin[-2 - r]; }
    __device__ __forceinline__ float4 Vang(int r) const { return r >= 0 ? vang[r] : g.vang[-2 - r]; }
    __device__ __forceinline__ float4 Inv0(int r) const { return r >= 0 ? inv0[r] : g.inv0[-2 - r]; }
    __device__ __forceinline__ float4 Inv1(int r) const { return r >= 0 ? inv1[r] : g.inv1[-2 - r]; }
    __device__ __forceinline__ void SetVelocity(int r, float4 v, float4 w) const {
        if (r >= 0) { vlin[r] = v; vang[r] = w; }  // only a group's own (dynamic) bodies are written
    }
};

// Shared memory of one CTA: 6 body lanes per body; with kShared also 24 float4
// lanes, a state word and a ref pair per manifold (400 bytes).
__host__ __device__ constexpr size_t GroupSmemBytes(bool shared, int bodies, int manifolds) {
    return 96 * (size_t)bodies + (shared ? 400 * (size_t)manifolds : 0);
}

template <bool kCensus, bool kShared>
__global__ void k_groups(ManifoldSoA m, BodySoA b, StepParams p, uint32_t flags, GroupTables t, int groupBase,
                         int Bc, int Lc, unsigned long long* census) {
    extern __shared__ float4 smem[];
    const GroupDesc g = t.groups[groupBase + blockIdx.x];
    const int nLocal = g.bEnd - g.bBegin, nm = g.mEnd - g.mBegin;
    GroupBodies bv;
    bv.pos = smem;
    bv.quat = bv.pos + Bc;
    bv.vlin = bv.quat + Bc;
    bv.vang = bv.vlin + Bc;
    bv.inv0 = bv.vang + Bc;
    bv.inv1 = bv.inv0 + Bc;
    bv.g = b;
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
    }
    const int tid = threadIdx.x, T = blockDim.x;
    const int lbase = kShared ? 0 : g.mBegin;  // slot of local manifold 0 in ml

    // Bodies into shared memory, through the force update (EntityBase.cs:911-975).
    for (int i = tid; i < nLocal; i += T) {
        int gi = t.bodies[g.bBegin + i];
        float4 v = b.vlin[gi], w = b.vang[gi], q = b.quat[gi], a, c;
        if (flags & BEPUGPU_STEP_FORCES) {
            ForceMath(v, w, q, b.loc0[gi], b.loc1[gi], b.damp[gi], a, c, p);
        } else {
            a = b.inv0[gi];
            c = b.inv1[gi];
        }
        bv.pos[i] = b.pos[gi];
        bv.quat[i] = q;
        bv.vlin[i] = v;
        bv.vang[i] = w;
        bv.inv0[i] = a;
        bv.inv1[i] = c;
    }
    __syncthreads();
    // Refresh, lanes in, prestep: a thread keeps the same manifolds throughout.
    for (int j = tid; j < nm; j += T) {
        const int s = g.mBegin + j;
        int2 r = t.refs[s];
        if (flags & BEPUGPU_STEP_REFRESH_CONTACTS) RefreshManifoldV(m, bv, s, r.x, r.y, p);
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
    if (kCensus && tid == 0) atomicAdd(census + 3, 208ull * (unsigned long long)nLocal);  // 7 lanes in, 6 out
    __syncthreads();
    if (flags & BEPUGPU_STEP_SOLVE) {
        const int* co = t.colourOffsets + g.cBegin;
        for (int c = 0; c < g.cCount; c++) {
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
        if (kShared) {  // impulses and sliding axis back to the manifold records
            for (int j = tid; j < nm; j += T) {
                const int s = g.mBegin + j;
                m.penacc[s] = ml.penacc[j];
                m.fricacc[s] = ml.fricacc[j];
                m.saxis[s] = ml.saxis[j];
            }
        }
    }
    // Position update (EntityBase.cs:1124-1160) and write-back.
    for (int i = tid; i < nLocal; i += T) {
        int gi = t.bodies[g.bBegin + i];
        float4 pos = bv.pos[i], q = bv.quat[i], v = bv.vlin[i], w = bv.vang[i];
        if (flags & BEPUGPU_STEP_POSITIONS) {
            if (PositionMath(pos, q, v, w, p)) {
                b.pos[gi] = pos;
                b.quat[gi] = q;
            }
        }
        b.vlin[gi] = v;
        b.vang[gi] = w;
        b.inv0[gi] = bv.inv0[i];
        b.inv1[gi] = bv.inv1[i];
    }
}

// ------------------------------------------------------------------ host side --
namespace {
struct UnionFind {
    std::vector<int32_t> parent;
    explicit UnionFind(int n) : parent(n) { std::iota(parent.begin(), parent.end(), 0); }
    int32_t Find(int32_t x) {
        while (parent[x] != x) {
            parent[x] = parent[parent[x]];
            x = parent[x];
        }
        return x;
    }
    void Join(int32_t a, int32_t b) {
        a = Find(a);
        b = Find(b);
        if (a != b) parent[std::max(a, b)] = std::min(a, b);
    }
};
}  // namespace

// Splits the manifold list into the colour-sweep part and island groups and
// assigns every manifold its slot.  colour[u] is the solver-list colouring
// (joints first).  The sweep part takes slots [0, globalCount) in colour-major
// order; each group takes a contiguous range in colour-major order.
void PlanGroups(const GroupPolicy& pol, const int32_t* a, const int32_t* b, const int32_t* colour, int32_t nj,
                int32_t nm, const uint8_t* dynamic, int32_t nb, GroupPlan& plan) {
    plan = GroupPlan();
    const int32_t* mc = colour + nj;  // manifold colours
    std::vector<int32_t> groupOfManifold(nm, -1);
    std::vector<std::vector<int32_t>> gBodies;
    plan.localOf.assign(nb, -1);
    if (pol.enabled && nm > 0) {
        UnionFind uf(nb);
        for (int32_t u = 0; u < nj + nm; u++)
            if (a[u] >= 0 && b[u] >= 0 && dynamic[a[u]] && dynamic[b[u]]) uf.Join(a[u], b[u]);
        std::vector<int32_t> idOfRoot(nb, -1), manifolds, bodiesCount, islandOf(nm, -1);
        std::vector<uint8_t> jointTouched(nb, 0);
        for (int32_t u = 0; u < nj; u++)  // islands holding a joint stay on the sweep path
            for (int32_t e : {a[u], b[u]})
                if (e >= 0 && dynamic[e]) jointTouched[uf.Find(e)] = 1;
        for (int32_t i = 0; i < nm; i++) {
            int32_t ea = a[nj + i], eb = b[nj + i];
            int32_t e = ea >= 0 && dynamic[ea] ? ea : (eb >= 0 && dynamic[eb] ? eb : -1);
            if (e < 0) continue;  // no dynamic body: never active, sweep path
            int32_t root = uf.Find(e);
            if (jointTouched[root]) continue;
            if (idOfRoot[root] < 0) {
                idOfRoot[root] = (int32_t)manifolds.size();
                manifolds.push_back(0);
                bodiesCount.push_back(0);
            }
            islandOf[i] = idOfRoot[root];
            manifolds[islandOf[i]]++;
        }
        for (int32_t e = 0; e < nb; e++)
            if (dynamic[e] && idOfRoot[uf.Find(e)] >= 0) bodiesCount[idOfRoot[uf.Find(e)]]++;
        // islands too large for one CTA stay on the sweep path
        std::vector<uint8_t> small(manifolds.size());
        for (size_t k = 0; k < manifolds.size(); k++)
            small[k] = bodiesCount[k] <= pol.maxGroupBodies && manifolds[k] <= pol.maxGroupManifolds;
        // pack small islands into groups in island order
        std::vector<int32_t> groupOfIsland(manifolds.size(), -1);
        int32_t gm = 0, gb = 0, groups = 0;
        for (size_t k = 0; k < manifolds.size(); k++) {
            if (!small[k]) continue;
            if (groups == 0 || gm + manifolds[k] > pol.targetGroupManifolds ||
                gb + bodiesCount[k] > pol.maxGroupBodies) {
                groups++;
                gm = gb = 0;
            }
            groupOfIsland[k] = groups - 1;
            gm += manifolds[k];
            gb += bodiesCount[k];
        }
        gBodies.resize(groups);
        for (int32_t e = 0; e < nb; e++) {
            if (!dynamic[e]) continue;
            int32_t id = idOfRoot[uf.Find(e)];
            if (id < 0 || groupOfIsland[id] < 0) continue;
            plan.localOf[e] = (int32_t)gBodies[groupOfIsland[id]].size();
            gBodies[groupOfIsland[id]].push_back(e);
        }
        for (int32_t i = 0; i < nm; i++)
            if (islandOf[i] >= 0) groupOfManifold[i] = groupOfIsland[islandOf[i]];
    }
    const int32_t G = (int32_t)gBodies.size();
    std::vector<std::vector<int32_t>> members(G);
    for (int32_t i = 0; i < nm; i++)
        if (groupOfManifold[i] >= 0) members[groupOfManifold[i]].push_back(i);
    // groups whose solve lanes fit shared memory run the shared variant; they come first
    std::vector<int32_t> order(G);
    std::iota(order.begin(), order.end(), 0);
    std::vector<uint8_t> fits(G);
    for (int32_t gId = 0; gId < G; gId++)
        fits[gId] = GroupSmemBytes(true, (int)gBodies[gId].size(), (int)members[gId].size()) <= kGroupSmemBudget;
    std::stable_partition(order.begin(), order.end(), [&](int32_t gId) { return fits[gId] != 0; });

    // Slots: the sweep part, then the groups in launch order.
    int32_t colours = 0;
    for (int32_t i = 0; i < nm; i++) colours = std::max(colours, mc[i] + 1);
    plan.slotOf.assign(nm, -1);
    plan.globalOffsets.assign(colours + 1, 0);
    int32_t slot = 0;
    {
        std::vector<std::vector<int32_t>> byColour(colours);
        for (int32_t i = 0; i < nm; i++)
            if (groupOfManifold[i] < 0) byColour[mc[i]].push_back(i);
        for (int32_t c = 0; c < colours; c++) {
            plan.globalOffsets[c] = slot;
            for (int32_t i : byColour[c]) plan.slotOf[i] = slot++;
        }
        plan.globalOffsets[colours] = slot;
        plan.globalCount = slot;
    }
    plan.refs.assign(nm, make_int2(-1, -1));
    plan.groupOfManifold.assign(nm, -1);
    plan.groups.resize(G);
    for (int32_t k = 0; k < G; k++) {
        const int32_t gId = order[k];
        GroupDesc& d = plan.groups[k];
        GroupClass& cls = fits[gId] ? plan.shared : plan.global;
        if (cls.end == cls.begin) cls.begin = cls.end = k;
        cls.end = k + 1;
        d.bBegin = (int32_t)plan.groupBodies.size();
        plan.groupBodies.insert(plan.groupBodies.end(), gBodies[gId].begin(), gBodies[gId].end());
        d.bEnd = (int32_t)plan.groupBodies.size();
        cls.maxLocal = std::max(cls.maxLocal, d.bEnd - d.bBegin);
        cls.maxManifolds = std::max(cls.maxManifolds, (int32_t)members[gId].size());
        int32_t gc = 0;
        for (int32_t i : members[gId]) gc = std::max(gc, mc[i] + 1);
        std::vector<std::vector<int32_t>> byColour(gc);
        for (int32_t i : members[gId]) byColour[mc[i]].push_back(i);
        d.mBegin = slot;
        d.cBegin = (int32_t)plan.colourOffsets.size();
        d.cCount = gc;
        for (int32_t c = 0; c < gc; c++) {
            plan.colourOffsets.push_back(slot - d.mBegin);
            cls.maxColourMembers = std::max(cls.maxColourMembers, (int32_t)byColour[c].size());
            for (int32_t i : byColour[c]) {
                plan.slotOf[i] = slot;
                plan.groupOfManifold[i] = k;
                auto ref = [&](int32_t e) -> int32_t {
                    if (e < 0) return -1;
                    return dynamic[e] ? plan.localOf[e] : -2 - e;
                };
                plan.refs[slot] = make_int2(ref(a[nj + i]), ref(b[nj + i]));
                slot++;
            }
        }
        plan.colourOffsets.push_back(slot - d.mBegin);
        d.mEnd = slot;
    }
}

bepugpu_status Scene::UploadGroups(Context* ctx) {
    const GroupPlan& g = groupPlan;
    size_t G = g.groups.size();
    if (G == 0) return BEPUGPU_OK;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(groupDescDev, g.groups.data(), sizeof(GroupDesc) * G, cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(groupBodiesDev, g.groupBodies.data(), sizeof(int32_t) * g.groupBodies.size(),
                             cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(groupRefsDev, g.refs.data(), sizeof(int2) * g.refs.size(), cudaMemcpyHostToDevice,
                             stream)) ||
        (e = cudaMemcpyAsync(groupColourOffsetsDev, g.colourOffsets.data(), sizeof(int32_t) * g.colourOffsets.size(),
                             cudaMemcpyHostToDevice, stream)) ||
        (e = cudaStreamSynchronize(stream))) {
        ctx->SetError("group tables: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    return BEPUGPU_OK;
}

namespace {
int ClassThreads(const GroupClass& c, int override_) {
    if (override_ > 0) return override_;
    int t = ((c.maxColourMembers + 31) / 32) * 32;
    return std::min(std::max(t, 32), 256);
}

template <bool kShared>
bepugpu_status LaunchClass(Context* ctx, Scene* s, const GroupClass& c, const StepParams& p, uint32_t flags,
                           bool count, GroupTables t) {
    if (c.end <= c.begin) return BEPUGPU_OK;
    const int Bc = std::max(c.maxLocal, 1), Lc = std::max(c.maxManifolds, 1);
    size_t smemBytes = GroupSmemBytes(kShared, Bc, Lc);
    cudaError_t e = cudaSuccess;
    if (smemBytes > 48 * 1024) {
        e = cudaFuncSetAttribute(k_groups<false, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_groups<true, kShared>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smemBytes);
        if (e != cudaSuccess) {
            ctx->SetError("group kernel shared memory %zu bytes: %s", smemBytes, cudaGetErrorString(e));
            return BEPUGPU_CUDA_ERROR;
        }
    }
    const int threads = ClassThreads(c, s->groupThreadsOverride);
    const unsigned blocks = (unsigned)(c.end - c.begin);
    if (count)
        k_groups<true, kShared><<<blocks, threads, smemBytes, s->stream>>>(s->m, s->b, p, flags, t, c.begin, Bc, Lc,
                                                                            s->Census());
    else
        k_groups<false, kShared><<<blocks, threads, smemBytes, s->stream>>>(s->m, s->b, p, flags, t, c.begin, Bc, Lc,
                                                                             nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->SetError("group kernel launch: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    return BEPUGPU_OK;
}
}  // namespace

int GroupLaunchCount(const GroupPlan& g) {
    return (g.shared.end > g.shared.begin ? 1 : 0) + (g.global.end > g.global.begin ? 1 : 0);
}

bepugpu_status LaunchGroups(Context* ctx, Scene* s, const StepParams& p, uint32_t flags, bool count) {
    const GroupPlan& g = s->groupPlan;
    if (g.groups.empty()) return BEPUGPU_OK;
    GroupTables t;
    t.groups = s->groupDescDev;
    t.bodies = s->groupBodiesDev;
    t.refs = s->groupRefsDev;
    t.colourOffsets = s->groupColourOffsetsDev;
    bepugpu_status st = LaunchClass<true>(ctx, s, g.shared, p, flags, count, t);
    if (st != BEPUGPU_OK) return st;
    return LaunchClass<false>(ctx, s, g.global, p, flags, count, t);
}

}  // namespace bepugpu
