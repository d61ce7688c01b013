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
#include "groups_device.cuh"
#include "solver_device.cuh"

namespace bepugpu {

template <bool kCensus, bool kShared>
__global__ void k_groups(ManifoldSoA m, BodySoA b, StepParams p, uint32_t flags, GroupTables t, int groupBase,
                         int Bc, int Lc, unsigned long long* census) {
    extern __shared__ float4 smem[];
    const GroupDesc g = t.groups[groupBase + blockIdx.x];
    GroupStep<kCensus, kShared>(m, b, p, flags, t, g, Bc, Lc, smem, census);
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
        fits[gId] = GroupSmemBytes(true, (int)gBodies[gId].size(), (int)members[gId].size()) <=
                    std::min<size_t>(pol.sharedLanesBudget, kGroupSmemBudget);
    std::stable_partition(order.begin(), order.end(), [&](int32_t gId) { return fits[gId] != 0; });

    // Slots: the sweep part, then the groups in launch order.
    int32_t colours = 0;  // the sweep covers every colour of the list (joints sweep too)
    for (int32_t u = 0; u < nj + nm; u++) colours = std::max(colours, colour[u] + 1);
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
