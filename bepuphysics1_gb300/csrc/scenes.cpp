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
#include <cfloat>
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

enum Shape { kBox = 0, kSphere = 1, kCapsule = 2 };

struct Body {
    int shape;
    float c[3];     // centre
    float h[3];     // half extents (box) / radius in h[0] (sphere, capsule), capsule half length in h[1]
    float mass;     // 0 = static
    float friction;
    float q[4] = {0.f, 0.f, 0.f, 1.f};  // orientation (capsules only; boxes and spheres are axis aligned)
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
    for (int k = 0; k < 4; k++) r.orientation[k] = b.q[k];
    r.linear_damping = .03f;   // EntityBase.cs:1165
    r.angular_damping = .15f;  // EntityBase.cs:1164
    if (b.mass > 0) {
        r.is_dynamic = 1;
        // Dynamic bodies are always active, as DeterminismTestDemo.cs:84 makes its
        // boxes: no island of them would go to sleep in the reference either.  The
        // static bodies keep the default and go inactive after their first step.
        r.activity = BEPUGPU_BODY_ALWAYS_ACTIVE;
        r.inverse_mass = 1.f / b.mass;
        const float scale = b.mass * 2.5f;  // InertiaHelper.InertiaTensorScale (InertiaHelper.cs:20)
        float i0, i1, i2;
        if (b.shape == kBox) {  // BoxShape.cs:120-131
            float w = 2 * b.h[0], h = 2 * b.h[1], l = 2 * b.h[2];
            const float inv12 = 1 / 12.f;
            i0 = (h * h + l * l) * inv12 * scale;
            i1 = (w * w + l * l) * inv12 * scale;
            i2 = (w * w + h * h) * inv12 * scale;
        } else if (b.shape == kSphere) {  // SphereShape.cs:55-60: 2/5 r^2
            float r2 = b.h[0] * b.h[0];
            i0 = i1 = i2 = r2 * .4f * scale;
        } else {  // CapsuleShape.cs:76-92: cylindrical approximation, axis along local y
            float radius = b.h[0], length = 2 * b.h[1];
            float effectiveLength = length + radius / 2;
            float diagValue = (.0833333333f * effectiveLength * effectiveLength + .25f * radius * radius);
            i0 = diagValue * scale;
            i1 = .5f * radius * radius * scale;
            i2 = diagValue * scale;
        }
        InverseDiagonalInertia(i0, i1, i2, r.local_inverse_inertia);
    }
    return r;
}

// ---- small vector helpers for the joint scenes (BEPUutilities conventions) --
struct V3 {
    float x, y, z;
};
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 Cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 Normalized(V3 v) {  // Vector3.Normalize (Vector3.cs:575-581)
    float inverse = (float)(1 / std::sqrt((double)(v.x * v.x + v.y * v.y + v.z * v.z)));
    return {v.x * inverse, v.y * inverse, v.z * inverse};
}
struct M3 {
    float m[3][3];  // row-major M11..M33
};
M3 RotationOf(const float q[4]) {  // Matrix3x3.CreateFromQuaternion (Matrix3x3.cs:1303-1328)
    float qX2 = q[0] + q[0], qY2 = q[1] + q[1], qZ2 = q[2] + q[2];
    float XX = qX2 * q[0], YY = qY2 * q[1], ZZ = qZ2 * q[2];
    float XY = qX2 * q[1], XZ = qX2 * q[2], XW = qX2 * q[3];
    float YZ = qY2 * q[2], YW = qY2 * q[3], ZW = qZ2 * q[3];
    M3 r;
    r.m[0][0] = 1 - YY - ZZ; r.m[1][0] = XY - ZW; r.m[2][0] = XZ + YW;
    r.m[0][1] = XY + ZW; r.m[1][1] = 1 - XX - ZZ; r.m[2][1] = YZ - XW;
    r.m[0][2] = XZ - YW; r.m[1][2] = YZ + XW; r.m[2][2] = 1 - XX - YY;
    return r;
}
V3 TransformTranspose(V3 v, const M3& r) {  // Matrix3x3.TransformTranspose (Matrix3x3.cs:1113-1123)
    return {v.x * r.m[0][0] + v.y * r.m[0][1] + v.z * r.m[0][2], v.x * r.m[1][0] + v.y * r.m[1][1] + v.z * r.m[1][2],
            v.x * r.m[2][0] + v.y * r.m[2][1] + v.z * r.m[2][2]};
}
// Rotation of v about unit axis n by angle a (Rodrigues), in double.
V3 Rotate(V3 v, V3 n, double a) {
    double c = std::cos(a), sn = std::sin(a), d = (double)v.x * n.x + (double)v.y * n.y + (double)v.z * n.z;
    double cx = (double)n.y * v.z - (double)n.z * v.y, cy = (double)n.z * v.x - (double)n.x * v.z,
           cz = (double)n.x * v.y - (double)n.y * v.x;
    V3 r{(float)(v.x * c + cx * sn + n.x * d * (1 - c)), (float)(v.y * c + cy * sn + n.y * d * (1 - c)),
         (float)(v.z * c + cz * sn + n.z * d * (1 - c))};
    return Normalized(r);
}
// Quaternion.GetQuaternionBetweenNormalizedVectors(Up, d) (Quaternion.cs:795-825)
void QuaternionFromUp(V3 d, float q[4]) {
    V3 up{0, 1, 0};
    float dot = Dot(up, d);
    if (dot < -0.9999f) {
        q[0] = -up.y; q[1] = up.x; q[2] = 0; q[3] = 0;
    } else {
        V3 axis = Cross(up, d);
        q[0] = axis.x; q[1] = axis.y; q[2] = axis.z; q[3] = dot + 1;
    }
    float inverse = (float)(1 / std::sqrt((double)(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])));
    for (int k = 0; k < 4; k++) q[k] *= inverse;
}

struct Generator {
    std::vector<Body> bodies;
    std::vector<bepugpu_manifold> manifolds;
    std::vector<bepugpu_joint> joints;
    float contactDistance = .1f;
    bool narrowPhase = false;  // emit empty GENERATED manifolds for candidate pairs

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
        if (SpherePairIsNonConvex(A, B)) m.flags |= BEPUGPU_MANIFOLD_NONCONVEX;
        AddContact(m, p, n, depth, 0);
        manifolds.push_back(m);
    }

    // The reference's sphere-sphere and box-sphere pair handlers carry a
    // NonConvexContactManifoldConstraint (SpherePairHandler.cs:28,
    // BoxSpherePairHandler.cs:28); pairs with a capsule are convex pairs.
    static bool SpherePairIsNonConvex(const Body& A, const Body& B) {
        return (A.shape == kSphere && (B.shape == kSphere || B.shape == kBox)) ||
               (B.shape == kSphere && A.shape == kBox);
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

    // An empty GENERATED manifold for a pair whose bounding boxes come within
    // the contact distance: the library's narrow phase fills it.
    void Candidate(int a, int b) {
        const Body &A = bodies[a], &B = bodies[b];
        for (int k = 0; k < 3; k++) {
            float ea = A.shape == kBox ? A.h[k] : A.h[0], eb = B.shape == kBox ? B.h[k] : B.h[0];
            if (std::fabs(A.c[k] - B.c[k]) > ea + eb + contactDistance) return;
        }
        if (A.shape == kSphere && B.shape == kBox) std::swap(a, b);  // box-sphere pairs put the box first
        bepugpu_manifold m = NewManifold(a, b);
        m.flags |= BEPUGPU_MANIFOLD_GENERATED;
        if (SpherePairIsNonConvex(bodies[a], bodies[b])) m.flags |= BEPUGPU_MANIFOLD_NONCONVEX;
        manifolds.push_back(m);
    }

    void Pair(int a, int b) {
        const bool collidable = bodies[a].shape != kCapsule && bodies[b].shape != kCapsule;
        if (narrowPhase && collidable) Candidate(a, b);
        else if (bodies[a].shape == kBox && bodies[b].shape == kBox) BoxBox(a, b);
        else WithSphere(a, b);
    }
};

}  // namespace

struct bepuscene {
    std::vector<float> friction;  // per body
    std::vector<bepugpu_shape> shapes;
    std::vector<bepugpu_body> bodies;
    std::vector<bepugpu_manifold> manifolds;
    std::vector<bepugpu_joint> joints;
};

static bepuscene* Finish(Generator& g) {
    auto* s = new bepuscene();
    s->bodies.reserve(g.bodies.size());
    for (const Body& b : g.bodies) {
        s->bodies.push_back(MakeRecord(b));
        s->friction.push_back(b.friction);
        bepugpu_shape sh;
        std::memset(&sh, 0, sizeof(sh));
        if (b.shape == kBox) {
            sh.type = BEPUGPU_SHAPE_BOX;
            for (int k = 0; k < 3; k++) sh.size[k] = b.h[k];
        } else if (b.shape == kSphere) {
            sh.type = BEPUGPU_SHAPE_SPHERE;
            sh.size[0] = b.h[0];
        }
        s->shapes.push_back(sh);
    }
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
    g.narrowPhase = p->narrow_phase != 0;
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
                if (p->drop_spacing > 0) {
                    b.c[1] = .05f + .5f * p->size_max + iy * p->drop_spacing;
                } else {
                    b.c[1] = top + b.h[1] - pen;
                    top = b.c[1] + b.h[1];
                }
                b.mass = p->density > 0 ? p->density * (8.f * b.h[0] * b.h[1] * b.h[2]) : p->mass;
                b.friction = rng.uniform(p->friction_min, p->friction_max);
                g.bodies.push_back(b);
            }
        }
    if (!(p->drop_spacing > 0)) g.Collide(0.f);
    *out = Finish(g);
    return BEPUGPU_OK;
}

int32_t bepuscene_make_tower(const bepuscene_tower_params* p, bepuscene** out) {
    if (!p || !out || p->body_count <= 0 || p->tower_min <= 0 || p->tower_max < p->tower_min)
        return BEPUGPU_INVALID_ARGUMENT;
    Rng rng(p->seed);
    Generator g;
    g.narrowPhase = p->narrow_phase != 0;
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

namespace {

bepugpu_joint NewJoint(int32_t type, int a, int b) {
    bepugpu_joint j;
    std::memset(&j, 0, sizeof(j));
    j.type = type;
    j.body_a = a;
    j.body_b = b;
    j.flags = BEPUGPU_JOINT_ACTIVE;
    j.margin = .005f;                   // JointLimit.cs:22
    j.bounce_velocity_threshold = 1.f;  // JointLimit.cs:14
    j.max_corrective_velocity = FLT_MAX;
    j.spring_stiffness = 600000.f;      // SpringSettings.cs:58-59
    j.spring_damping = 90000.f;
    return j;
}

// Pose of body i, or the world entity for -1.
struct Pose {
    V3 c;
    M3 R;
    float q[4];
};
Pose PoseOf(const std::vector<Body>& bodies, int i) {
    Pose p;
    if (i < 0) {
        p.c = {0, 0, 0};
        p.q[0] = p.q[1] = p.q[2] = 0; p.q[3] = 1;
    } else {
        const Body& b = bodies[i];
        p.c = {b.c[0], b.c[1], b.c[2]};
        for (int k = 0; k < 4; k++) p.q[k] = b.q[k];
    }
    p.R = RotationOf(p.q);
    return p;
}
void Put(float* dst, V3 v) { dst[0] = v.x; dst[1] = v.y; dst[2] = v.z; }

// BallSocketJoint(connectionA, connectionB, anchor) (BallSocketJoint.cs:40-50):
// OffsetA/B = anchor - position, stored in each body's frame.
void SetBallSocket(bepugpu_joint& j, const Pose& A, const Pose& B, V3 anchor) {
    Put(j.anchor_a, TransformTranspose(anchor - A.c, A.R));
    Put(j.anchor_b, TransformTranspose(anchor - B.c, B.R));
}

}  // namespace

// Articulated chains of capsules.  Chain c hangs from a static anchor (a ball
// socket to the world entity) with its links bent by seeded angles of up to
// 70 degrees, so that part of the limits start beyond their 45 degrees; links
// alternate BallSocketJoint + SwingLimit and RevoluteJoint with its limit
// active.  Chains that reach the ground are lifted to rest on it and get
// capsule-ground contacts.  Loose spheres and boxes stand in two-body stacks
// on a jittered grid covering the region.
int32_t bepuscene_make_chain(const bepuscene_chain_params* p, bepuscene** out) {
    if (!p || !out || p->chains < 0 || p->links < 1 || p->loose_bodies < 0 || p->capsule_radius <= 0 ||
        p->capsule_length <= 0 || p->link_mass <= 0)
        return BEPUGPU_INVALID_ARGUMENT;
    Rng rng(p->seed);
    Generator g;
    const float half = .5f * std::max(p->region[0], p->region[2]) + 5.f;
    g.bodies.push_back(Body{kBox, {0, -.5f, 0}, {half, .5f, half}, 0.f, .6f});
    // loose bodies: two per grid column
    const int columns = (p->loose_bodies + 1) / 2;
    const int side = (int)std::ceil(std::sqrt((double)std::max(columns, 1)));
    const float spacing = std::max(p->region[0], p->region[2]) / (float)std::max(side, 1);
    int placed = 0;
    for (int col = 0; col < columns && placed < p->loose_bodies; col++) {
        float cx = -.5f * p->region[0] + (col % side + .5f) * spacing + rng.uniform(-.1f, .1f);
        float cz = -.5f * p->region[2] + (col / side + .5f) * spacing + rng.uniform(-.1f, .1f);
        float top = 0.f;
        for (int k = 0; k < 2 && placed < p->loose_bodies; k++, placed++) {
            Body b;
            if (rng.uniform() < .5f) {
                b.shape = kSphere;
                float r = rng.uniform(.3f, .7f);
                b.h[0] = b.h[1] = b.h[2] = r;
            } else {
                b.shape = kBox;
                for (int a = 0; a < 3; a++) b.h[a] = rng.uniform(.25f, .6f);
            }
            b.c[0] = cx + rng.uniform(-.05f, .05f);
            b.c[2] = cz + rng.uniform(-.05f, .05f);
            float pen = rng.uniform(0.f, .02f);
            b.c[1] = top + b.h[1] - pen;
            top = b.c[1] + b.h[1];
            b.mass = b.shape == kSphere ? 4.18879f * b.h[0] * b.h[0] * b.h[0] : 8.f * b.h[0] * b.h[1] * b.h[2];
            b.friction = rng.uniform(.4f, .8f);
            g.bodies.push_back(b);
        }
    }
    g.Collide(0.f);
    // chains
    const float r = p->capsule_radius, hl = .5f * p->capsule_length, tip = hl + r;
    const double kLimit = (double)p->swing_limit;
    const double kMaxBend = 70.0 * 3.14159265358979323846 / 180.0;
    std::vector<V3> dirs(p->links), axes(p->links), centres(p->links);
    for (int c = 0; c < p->chains; c++) {
        V3 root{rng.uniform(-.5f * p->region[0], .5f * p->region[0]), rng.uniform(2.f, p->region[1]),
                rng.uniform(-.5f * p->region[2], .5f * p->region[2])};
        auto randomPerpendicular = [&](V3 d) {
            V3 t{rng.uniform(-1.f, 1.f), rng.uniform(-1.f, 1.f), rng.uniform(-1.f, 1.f)};
            V3 n = Cross(d, t);
            if (Dot(n, n) < 1e-4f) n = Cross(d, V3{1, 0, 0});
            return Normalized(n);
        };
        V3 up{0, 1, 0};
        dirs[0] = Rotate(up, randomPerpendicular(up), rng.uniform() * (kMaxBend / 2));
        centres[0] = root - dirs[0] * tip;
        for (int k = 1; k < p->links; k++) {
            axes[k - 1] = randomPerpendicular(dirs[k - 1]);
            dirs[k] = Rotate(dirs[k - 1], axes[k - 1], rng.uniform() * kMaxBend);
            V3 anchor = centres[k - 1] - dirs[k - 1] * tip;
            centres[k] = anchor - dirs[k] * tip;
        }
        float lowest = 1e30f;
        for (int k = 0; k < p->links; k++)
            for (float sgn : {-1.f, 1.f}) lowest = std::min(lowest, centres[k].y + sgn * dirs[k].y * hl - r);
        float lift = lowest < 0.f ? -lowest - rng.uniform(0.f, .01f) : 0.f;
        root.y += lift;
        const int first = (int)g.bodies.size();
        for (int k = 0; k < p->links; k++) {
            Body b;
            b.shape = kCapsule;
            b.h[0] = r; b.h[1] = hl; b.h[2] = r;
            b.c[0] = centres[k].x; b.c[1] = centres[k].y + lift; b.c[2] = centres[k].z;
            QuaternionFromUp(dirs[k], b.q);
            b.mass = p->link_mass;
            b.friction = .6f;
            g.bodies.push_back(b);
        }
        // capsule-ground contacts: endpoint spheres within reach of the ground top (y = 0)
        for (int k = 0; k < p->links; k++) {
            const int bi = first + k;
            bepugpu_manifold m = g.NewManifold(0, bi);
            const Body& cap = g.bodies[bi];
            int id = 0;
            for (float sgn : {-1.f, 1.f}) {
                V3 e{cap.c[0] + sgn * dirs[k].x * hl, cap.c[1] + sgn * dirs[k].y * hl, cap.c[2] + sgn * dirs[k].z * hl};
                float depth = r - e.y;
                if (-depth > g.contactDistance) { id++; continue; }
                float pos[3] = {e.x, .5f * (e.y - r), e.z}, n[3] = {0, 1, 0};
                bepugpu_contact& ct = m.contacts[m.contact_count++];
                M3 Rc = RotationOf(cap.q);
                V3 offB = TransformTranspose(V3{pos[0] - cap.c[0], pos[1] - cap.c[1], pos[2] - cap.c[2]}, Rc);
                for (int a = 0; a < 3; a++) {
                    ct.position[a] = pos[a];
                    ct.normal[a] = n[a];
                    ct.local_offset_a[a] = pos[a] - g.bodies[0].c[a];
                }
                Put(ct.local_offset_b, offB);
                ct.penetration_depth = depth;
                ct.base_penetration_depth = depth;
                ct.id = id++;
            }
            if (m.contact_count) g.manifolds.push_back(m);
        }
        // joints: the root socket, then links alternating ball socket + swing limit and revolute
        {
            bepugpu_joint j = NewJoint(BEPUGPU_JOINT_BALL_SOCKET, -1, first);
            SetBallSocket(j, PoseOf(g.bodies, -1), PoseOf(g.bodies, first), root);
            g.joints.push_back(j);
        }
        for (int k = 0; k + 1 < p->links; k++) {
            const int a = first + k, b = first + k + 1;
            const Pose A = PoseOf(g.bodies, a), B = PoseOf(g.bodies, b);
            V3 anchor = A.c - dirs[k] * tip;
            if (k % 2 == 0) {
                bepugpu_joint j = NewJoint(BEPUGPU_JOINT_BALL_SOCKET, a, b);
                SetBallSocket(j, A, B, anchor);
                g.joints.push_back(j);
                // SwingLimit(A, B, axisA, axisB, maximumAngle) (SwingLimit.cs:30-38): the
                // axes kept in each body's frame; minimumCosine = (float)Math.Cos(angle)
                bepugpu_joint s = NewJoint(BEPUGPU_JOINT_SWING_LIMIT, a, b);
                Put(s.axis_a, TransformTranspose(Normalized(dirs[k]), A.R));
                Put(s.axis_b, TransformTranspose(Normalized(dirs[k + 1]), B.R));
                s.limit_min = (float)std::cos((double)std::min(std::max((float)kLimit, 0.f), 3.14159274f));
                g.joints.push_back(s);
            } else {
                // RevoluteJoint(A, B, anchor, freeAxis) (RevoluteJoint.cs:46-95) with Limit.IsActive
                bepugpu_joint j = NewJoint(BEPUGPU_JOINT_REVOLUTE, a, b);
                j.flags |= BEPUGPU_JOINT_LIMIT_ACTIVE;
                SetBallSocket(j, A, B, anchor);
                V3 freeAxis = Normalized(axes[k]);
                // RevoluteAngularJoint: free axis in both frames, restricted axes from A's
                // (RevoluteAngularJoint.cs:56-93)
                V3 la = TransformTranspose(freeAxis, A.R);
                Put(j.axis_a, la);
                Put(j.axis_b, TransformTranspose(freeAxis, B.R));
                V3 c1 = Cross(V3{0, 1, 0}, la);
                if (Dot(c1, c1) < .001f) c1 = Cross(V3{1, 0, 0}, la);
                V3 c2 = Cross(la, c1);
                Put(j.constrained_1, Normalized(c1));
                Put(j.constrained_2, Normalized(c2));
                // limit basis: free axis and the anchor direction from A, test axis toward B
                V3 baseAxis = anchor - A.c;
                baseAxis = baseAxis - freeAxis * Dot(baseAxis, freeAxis);
                Put(j.basis_primary, TransformTranspose(freeAxis, A.R));
                Put(j.basis_x, TransformTranspose(Normalized(baseAxis), A.R));
                V3 testAxis = B.c - anchor;
                testAxis = testAxis - freeAxis * Dot(testAxis, freeAxis);
                Put(j.test_axis, TransformTranspose(Normalized(testAxis), B.R));
                j.limit_min = std::fmod(-(float)kLimit, 6.28318548f);
                j.limit_max = std::fmod((float)kLimit, 6.28318548f);
                g.joints.push_back(j);
            }
        }
    }
    *out = Finish(g);
    return BEPUGPU_OK;
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

uint32_t bepuscene_params_size(int32_t kind) {
    switch (kind) {
        case 0: return sizeof(bepuscene_pile_params);
        case 1: return sizeof(bepuscene_tower_params);
        case 2: return sizeof(bepuscene_chain_params);
        default: return 0;
    }
}

void bepuscene_body_friction(const bepuscene* s, float* friction) {
    if (friction && !s->friction.empty()) std::memcpy(friction, s->friction.data(), s->friction.size() * sizeof(float));
}

void bepuscene_shapes(const bepuscene* s, bepugpu_shape* shapes) {
    if (shapes && !s->shapes.empty()) std::memcpy(shapes, s->shapes.data(), s->shapes.size() * sizeof(bepugpu_shape));
}

void bepuscene_free(bepuscene* s) { delete s; }

}  // extern "C"
