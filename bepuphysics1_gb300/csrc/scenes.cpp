// Seeded synthetic scenes and their contact manifolds (host only).
//
// Bodies are axis-aligned boxes and spheres resting in settled stacks.  Every
// touching or near pair (gap <= contact_distance) becomes one convex manifold:
// box-box pairs get the corners of their face overlap rectangle (up to four
// contacts, ids 0..3), pairs with a sphere get one contact.  The normal points
// from body A to body B, the convention of ContactPenetrationConstraint.cs:121-146
// (A receives the impulse along -normal).  Supplement data for the refresher
// (ContactRefresher.cs:18-69) is the contact position in each body's frame and
// the depth at creation.
#include "../../include/bepuscenes.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace {

// Splitmix64: a platform-independent seeded stream (std distributions are not
// specified bit-for-bit across standard libraries).
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x1234567ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
    float uniform(float a, float b) { return a + (b - a) * uniform(); }
    int range(int lo, int hi) { return lo + (int)(next() % (uint64_t)(hi - lo + 1)); }
};

enum Shape { kBox = 0, kSphere = 1 };

struct Body {
    int shape;
    float c[3];     // centre
    float h[3];     // half extents (box) / radius in h[0] (sphere)
    float mass;     // 0 = static
    float friction;
};

// Matrix3x3.Invert of a diagonal inertia tensor (Matrix3x3.cs:505-534), the
// full-matrix case EntityBase's AdaptiveInvert takes for a nonsingular tensor.
void InverseDiagonalInertia(float a, float b, float c, float out[9]) {
    float det = a * b * c + 0.f * 0.f * 0.f + 0.f * 0.f * 0.f - 0.f * b * 0.f - 0.f * 0.f * a - c * 0.f * 0.f;
    float d = 1 / det;
    std::memset(out, 0, 9 * sizeof(float));
    out[0] = (b * c - 0.f * 0.f) * d;
    out[4] = (a * c - 0.f * 0.f) * d;
    out[8] = (a * b - 0.f * 0.f) * d;
}

bepugpu_body MakeRecord(const Body& b) {
    bepugpu_body r;
    std::memset(&r, 0, sizeof(r));
    for (int k = 0; k < 3; k++) r.position[k] = b.c[k];
    r.orientation[3] = 1.f;
    r.linear_damping = .03f;   // EntityBase.cs:1165
    r.angular_damping = .15f;  // EntityBase.cs:1164
    if (b.mass > 0) {
        r.is_dynamic = 1;
        r.inverse_mass = 1.f / b.mass;
        const float scale = b.mass * 2.5f;  // InertiaHelper.InertiaTensorScale (InertiaHelper.cs:20)
        float i0, i1, i2;
        if (b.shape == kBox) {  // BoxShape.cs:120-131
            float w = 2 * b.h[0], h = 2 * b.h[1], l = 2 * b.h[2];
            const float inv12 = 1 / 12.f;
            i0 = (h * h + l * l) * inv12 * scale;
            i1 = (w * w + l * l) * inv12 * scale;
            i2 = (w * w + h * h) * inv12 * scale;
        } else {  // SphereShape.cs:55-60: 2/5 r^2
            float r2 = b.h[0] * b.h[0];
            i0 = i1 = i2 = r2 * .4f * scale;
        }
        InverseDiagonalInertia(i0, i1, i2, r.local_inverse_inertia);
    }
    return r;
}

struct Generator {
    std::vector<Body> bodies;
    std::vector<bepugpu_manifold> manifolds;
    std::vector<bepugpu_joint> joints;
    float contactDistance = .1f;

    void AddContact(bepugpu_manifold& m, const float p[3], const float n[3], float depth, int id) {
        bepugpu_contact& c = m.contacts[m.contact_count++];
        const Body& A = bodies[m.body_a];
        const Body& B = bodies[m.body_b];
        for (int k = 0; k < 3; k++) {
            c.position[k] = p[k];
            c.normal[k] = n[k];
            c.local_offset_a[k] = p[k] - A.c[k];
            c.local_offset_b[k] = p[k] - B.c[k];
        }
        c.penetration_depth = depth;
        c.base_penetration_depth = depth;
        c.id = id;
        c.penetration_impulse = 0.f;
    }

    bepugpu_manifold NewManifold(int a, int b) {
        bepugpu_manifold m;
        std::memset(&m, 0, sizeof(m));
        m.body_a = a;
        m.body_b = b;
        m.flags = BEPUGPU_MANIFOLD_ACTIVE | BEPUGPU_MANIFOLD_SOLVER_RULE;
        float f = bodies[a].friction * bodies[b].friction;  // MaterialManager.cs:77-85
        m.kinetic_friction = f;
        m.static_friction = f;
        m.bounciness = 0.f;
        return m;
    }

    void BoxBox(int a, int b) {
        const Body &A = bodies[a], &B = bodies[b];
        float o[3];
        for (int k = 0; k < 3; k++) o[k] = (A.h[k] + B.h[k]) - std::fabs(A.c[k] - B.c[k]);
        int ax = 0;
        for (int k = 1; k < 3; k++)
            if (o[k] < o[ax]) ax = k;
        if (o[ax] < -contactDistance) return;
        int u = (ax + 1) % 3, v = (ax + 2) % 3;
        if (o[u] <= .05f || o[v] <= .05f) return;  // edge, corner or sliver touch: no face patch
        float s = B.c[ax] >= A.c[ax] ? 1.f : -1.f;
        float n[3] = {0, 0, 0};
        n[ax] = s;
        float u0 = std::max(A.c[u] - A.h[u], B.c[u] - B.h[u]), u1 = std::min(A.c[u] + A.h[u], B.c[u] + B.h[u]);
        float v0 = std::max(A.c[v] - A.h[v], B.c[v] - B.h[v]), v1 = std::min(A.c[v] + A.h[v], B.c[v] + B.h[v]);
        float plane = .5f * ((A.c[ax] + s * A.h[ax]) + (B.c[ax] - s * B.h[ax]));
        bepugpu_manifold m = NewManifold(a, b);
        const float cu[4] = {u0, u1, u1, u0}, cv[4] = {v0, v0, v1, v1};
        for (int i = 0; i < 4; i++) {
            float p[3];
            p[ax] = plane; p[u] = cu[i]; p[v] = cv[i];
            AddContact(m, p, n, o[ax], i);
        }
        manifolds.push_back(m);
    }

    void WithSphere(int a, int b) {
        const Body &A = bodies[a], &B = bodies[b];
        float p[3], n[3], depth;
        if (A.shape == kSphere && B.shape == kSphere) {
            float d[3], len2 = 0;
            for (int k = 0; k < 3; k++) { d[k] = B.c[k] - A.c[k]; len2 += d[k] * d[k]; }
            float len = std::sqrt(len2);
            if (len < 1e-6f) return;
            depth = A.h[0] + B.h[0] - len;
            if (depth < -contactDistance) return;
            for (int k = 0; k < 3; k++) {
                n[k] = d[k] / len;
                p[k] = .5f * ((A.c[k] + n[k] * A.h[0]) + (B.c[k] - n[k] * B.h[0]));
            }
        } else {
            bool sphereIsB = B.shape == kSphere;
            const Body& box = sphereIsB ? A : B;
            const Body& sph = sphereIsB ? B : A;
            float q[3], d[3], len2 = 0;
            for (int k = 0; k < 3; k++) {
                q[k] = std::min(std::max(sph.c[k], box.c[k] - box.h[k]), box.c[k] + box.h[k]);
                d[k] = sph.c[k] - q[k];
                len2 += d[k] * d[k];
            }
            float len = std::sqrt(len2);
            if (len < 1e-6f) return;  // centre inside the box: not produced by these scenes
            depth = sph.h[0] - len;
            if (depth < -contactDistance) return;
            float sign = sphereIsB ? 1.f : -1.f;  // normal from A to B
            for (int k = 0; k < 3; k++) {
                float dirBoxToSphere = d[k] / len;
                n[k] = sign * dirBoxToSphere;
                p[k] = .5f * (q[k] + (sph.c[k] - dirBoxToSphere * sph.h[0]));
            }
        }
        bepugpu_manifold m = NewManifold(a, b);
        AddContact(m, p, n, depth, 0);
        manifolds.push_back(m);
    }

    // Uniform-grid broad phase over all bodies except the ground (index 0,
    // tested against every body it can reach).
    void Collide(float groundTop) {
        float cell = 0;
        for (size_t i = 1; i < bodies.size(); i++)
            for (int k = 0; k < 3; k++) cell = std::max(cell, 2 * bodies[i].h[bodies[i].shape == kBox ? k : 0]);
        cell += contactDistance;
        auto key = [&](int x, int y, int z) -> uint64_t {
            return ((uint64_t)(uint32_t)(x + (1 << 20)) << 42) ^ ((uint64_t)(uint32_t)(y + (1 << 20)) << 21) ^
                   (uint64_t)(uint32_t)(z + (1 << 20));
        };
        std::unordered_map<uint64_t, std::vector<int>> grid;
        grid.reserve(bodies.size() * 2);
        auto cellOf = [&](const Body& b, int k) { return (int)std::floor(b.c[k] / cell); };
        for (size_t i = 1; i < bodies.size(); i++)
            grid[key(cellOf(bodies[i], 0), cellOf(bodies[i], 1), cellOf(bodies[i], 2))].push_back((int)i);
        for (size_t i = 1; i < bodies.size(); i++) {
            const Body& b = bodies[i];
            float ext = b.shape == kBox ? b.h[1] : b.h[0];
            if (b.c[1] - ext - groundTop <= contactDistance) Pair(0, (int)i);
            std::vector<int> near;
            int cx = cellOf(b, 0), cy = cellOf(b, 1), cz = cellOf(b, 2);
            for (int dx = -1; dx <= 1; dx++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dz = -1; dz <= 1; dz++) {
                        auto it = grid.find(key(cx + dx, cy + dy, cz + dz));
                        if (it == grid.end()) continue;
                        for (int j : it->second)
                            if (j > (int)i) near.push_back(j);
                    }
            std::sort(near.begin(), near.end());
            for (int j : near) Pair((int)i, j);
        }
    }

    void Pair(int a, int b) {
        if (bodies[a].shape == kBox && bodies[b].shape == kBox) BoxBox(a, b);
        else WithSphere(a, b);
    }
};

}  // namespace

struct bepuscene {
    std::vector<bepugpu_body> bodies;
    std::vector<bepugpu_manifold> manifolds;
    std::vector<bepugpu_joint> joints;
};

static bepuscene* Finish(Generator& g) {
    auto* s = new bepuscene();
    s->bodies.reserve(g.bodies.size());
    for (const Body& b : g.bodies) s->bodies.push_back(MakeRecord(b));
    s->manifolds = std::move(g.manifolds);
    s->joints = std::move(g.joints);
    return s;
}

extern "C" {

void bepuscene_default_pile(bepuscene_pile_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->nx = 10; p->ny = 10; p->nz = 10;
    p->spacing = 1.05f;
    p->size_min = p->size_max = 1.f;
    p->density = 0.f;
    p->mass = 1.f;
    p->jitter = .05f;
    p->friction_min = p->friction_max = .6f;
    p->ground_friction = .6f;
    p->ground_size[0] = 100.f; p->ground_size[1] = 1.f; p->ground_size[2] = 100.f;
    p->settle_penetration = .02f;
    p->contact_distance = .1f;
    p->seed = 1234;
}

void bepuscene_default_tower(bepuscene_tower_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->body_count = 64;
    p->tower_min = 4; p->tower_max = 32;
    p->sphere_fraction = .3f;
    p->friction = .6f;
    p->tower_spacing = 2.f;
    p->settle_penetration = .02f;
    p->seed = 1;
}

void bepuscene_default_chain(bepuscene_chain_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->chains = 8192; p->links = 16;
    p->capsule_radius = .1f; p->capsule_length = .4f; p->link_mass = 1.f;
    p->swing_limit = 0.78539816f;
    p->loose_bodies = 20000;
    p->region[0] = 200.f; p->region[1] = 50.f; p->region[2] = 200.f;
    p->seed = 3;
}

int32_t bepuscene_make_pile(const bepuscene_pile_params* p, bepuscene** out) {
    if (!p || !out || p->nx <= 0 || p->ny <= 0 || p->nz <= 0) return BEPUGPU_INVALID_ARGUMENT;
    Rng rng(p->seed);
    Generator g;
    g.contactDistance = p->contact_distance;
    Body ground{kBox, {0, -.5f * p->ground_size[1], 0},
                {.5f * p->ground_size[0], .5f * p->ground_size[1], .5f * p->ground_size[2]}, 0.f, p->ground_friction};
    g.bodies.push_back(ground);
    float x0 = -.5f * p->spacing * (p->nx - 1), z0 = -.5f * p->spacing * (p->nz - 1);
    for (int ix = 0; ix < p->nx; ix++)
        for (int iz = 0; iz < p->nz; iz++) {
            float top = 0.f;  // ground top
            for (int iy = 0; iy < p->ny; iy++) {
                Body b;
                b.shape = kBox;
                for (int k = 0; k < 3; k++) b.h[k] = .5f * rng.uniform(p->size_min, p->size_max);
                b.c[0] = x0 + ix * p->spacing + rng.uniform(-p->jitter, p->jitter);
                b.c[2] = z0 + iz * p->spacing + rng.uniform(-p->jitter, p->jitter);
                float pen = rng.uniform(0.f, p->settle_penetration);
                b.c[1] = top + b.h[1] - pen;
                top = b.c[1] + b.h[1];
                b.mass = p->density > 0 ? p->density * (8.f * b.h[0] * b.h[1] * b.h[2]) : p->mass;
                b.friction = rng.uniform(p->friction_min, p->friction_max);
                g.bodies.push_back(b);
            }
        }
    g.Collide(0.f);
    *out = Finish(g);
    return BEPUGPU_OK;
}

int32_t bepuscene_make_tower(const bepuscene_tower_params* p, bepuscene** out) {
    if (!p || !out || p->body_count <= 0 || p->tower_min <= 0 || p->tower_max < p->tower_min)
        return BEPUGPU_INVALID_ARGUMENT;
    Rng rng(p->seed);
    Generator g;
    std::vector<int> heights;
    for (int left = p->body_count; left > 0;) {
        int h = std::min(left, rng.range(p->tower_min, p->tower_max));
        heights.push_back(h);
        left -= h;
    }
    int side = (int)std::ceil(std::sqrt((double)heights.size()));
    float extent = side * p->tower_spacing + 2.f;
    Body ground{kBox, {0, -.5f, 0}, {.5f * extent, .5f, .5f * extent}, 0.f, p->friction};
    g.bodies.push_back(ground);
    float origin = -.5f * p->tower_spacing * (side - 1);
    for (size_t t = 0; t < heights.size(); t++) {
        float cx = origin + (float)(t % side) * p->tower_spacing;
        float cz = origin + (float)(t / side) * p->tower_spacing;
        float top = 0.f;
        for (int i = 0; i < heights[t]; i++) {
            Body b;
            b.shape = rng.uniform() < p->sphere_fraction ? kSphere : kBox;
            b.h[0] = b.h[1] = b.h[2] = .5f;
            b.c[0] = cx + rng.uniform(-.02f, .02f);
            b.c[2] = cz + rng.uniform(-.02f, .02f);
            float pen = rng.uniform(0.f, p->settle_penetration);
            b.c[1] = top + .5f - pen;
            top = b.c[1] + .5f;
            b.mass = 1.f;
            b.friction = p->friction;
            g.bodies.push_back(b);
        }
    }
    g.Collide(0.f);
    *out = Finish(g);
    return BEPUGPU_OK;
}

int32_t bepuscene_make_chain(const bepuscene_chain_params* p, bepuscene** out) {
    (void)p; (void)out;
    return BEPUGPU_INVALID_OPERATION;
}

void bepuscene_counts(const bepuscene* s, int32_t* nb, int32_t* nm, int32_t* nj) {
    if (nb) *nb = (int32_t)s->bodies.size();
    if (nm) *nm = (int32_t)s->manifolds.size();
    if (nj) *nj = (int32_t)s->joints.size();
}

void bepuscene_copy(const bepuscene* s, bepugpu_body* b, bepugpu_manifold* m, bepugpu_joint* j) {
    if (b && !s->bodies.empty()) std::memcpy(b, s->bodies.data(), s->bodies.size() * sizeof(bepugpu_body));
    if (m && !s->manifolds.empty()) std::memcpy(m, s->manifolds.data(), s->manifolds.size() * sizeof(bepugpu_manifold));
    if (j && !s->joints.empty()) std::memcpy(j, s->joints.data(), s->joints.size() * sizeof(bepugpu_joint));
}

void bepuscene_free(bepuscene* s) { delete s; }

}  // extern "C"
