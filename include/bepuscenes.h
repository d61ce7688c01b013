/*
 * bepuscenes.h -- seeded synthetic scenes for the solver: body sets and the
 * convex contact manifolds a narrow phase would hand the solver.
 *
 * The reference's narrow phase (BoxBoxCollider.cs, BoxContactManifold.cs) is
 * not part of the accelerated path, so solver input comes from this contact
 * source: settled stacks of boxes and spheres whose touching pairs get
 * face-patch manifolds of up to four contacts (Contact.cs:15-31 layout) with
 * the supplement data ContactRefresher.cs:18-69 reads.  Speculative contacts
 * (negative depth down to -maximum_contact_distance) are generated for pairs
 * that are close but apart, as the reference's margins do.
 */
#ifndef BEPUSCENES_H
#define BEPUSCENES_H

#include <stdint.h>
#include "bepugpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bepuscene bepuscene;

/* Box pile: nx * nz columns of ny boxes, stacked and settled on a static ground
 * box.  Box sizes per axis uniform in [size_min, size_max]; mass = density *
 * volume when density > 0, else `mass`.  Column spacing `spacing`, horizontal
 * jitter uniform in +-jitter.  Per-body friction uniform in
 * [friction_min, friction_max] (static = kinetic); the ground uses
 * ground_friction.  Pair friction is the product blend (MaterialManager.cs:77-85). */
typedef struct bepuscene_pile_params {
    int32_t nx, ny, nz;
    float spacing;
    float size_min, size_max;
    float density;
    float mass;
    float jitter;
    float friction_min, friction_max;
    float ground_friction;
    float ground_size[3];
    float settle_penetration;  /* each resting contact penetrates uniform [0, this] */
    float contact_distance;    /* speculative contacts for gaps up to this */
    uint64_t seed;
    int32_t narrow_phase;      /* nonzero: every pair whose boxes are within contact_distance gets an
                                  empty BEPUGPU_MANIFOLD_GENERATED manifold (box first in box-sphere
                                  pairs) for the library's narrow phase to fill, instead of contacts */
    float drop_spacing;        /* > 0: boxes not stacked but on a 3D grid, layer iy's centres at
                                  drop_spacing * iy above the first layer, which starts 0.05 above the
                                  ground, all at rest in the air and without manifolds (a pile to settle) */
} bepuscene_pile_params;

/* Towers: one scene of `body_count` bodies (boxes and spheres, 1 m, 1 kg) in
 * towers of height uniform in [tower_min, tower_max] on a static ground. */
typedef struct bepuscene_tower_params {
    int32_t body_count;
    int32_t tower_min, tower_max;
    float sphere_fraction;
    float friction;
    float tower_spacing;
    float settle_penetration;
    uint64_t seed;
    int32_t narrow_phase;      /* as in bepuscene_pile_params */
} bepuscene_tower_params;

/* Chains: `chains` articulated chains of `links` capsules joined alternately by
 * a ball socket with a swing limit and by a revolute joint with its limit,
 * hanging from static anchors, plus `loose_bodies` spheres and boxes resting on
 * a ground.  Joint parameters per bepugpu_joint. */
typedef struct bepuscene_chain_params {
    int32_t chains, links;
    float capsule_radius, capsule_length, link_mass;
    float swing_limit;           /* radians */
    int32_t loose_bodies;
    float region[3];
    uint64_t seed;
} bepuscene_chain_params;

void bepuscene_default_pile(bepuscene_pile_params* p);
void bepuscene_default_tower(bepuscene_tower_params* p);
void bepuscene_default_chain(bepuscene_chain_params* p);

int32_t bepuscene_make_pile(const bepuscene_pile_params* p, bepuscene** out);
int32_t bepuscene_make_tower(const bepuscene_tower_params* p, bepuscene** out);
int32_t bepuscene_make_chain(const bepuscene_chain_params* p, bepuscene** out);
void bepuscene_counts(const bepuscene* s, int32_t* bodies, int32_t* manifolds, int32_t* joints);
void bepuscene_copy(const bepuscene* s, bepugpu_body* bodies, bepugpu_manifold* manifolds,
                    bepugpu_joint* joints);
/* sizeof of the parameter structs (kind 0 pile, 1 tower, 2 chain), so a
 * binding can check its layout. */
uint32_t bepuscene_params_size(int32_t kind);
/* One collision shape per body: boxes and spheres; capsules have none. */
void bepuscene_shapes(const bepuscene* s, bepugpu_shape* shapes);
/* Each body's friction coefficient (static = kinetic), which a manifold between
 * two bodies blends as their product (MaterialManager.cs:77-85). */
void bepuscene_body_friction(const bepuscene* s, float* friction);
void bepuscene_free(bepuscene* s);

#ifdef __cplusplus
}
#endif

#endif /* BEPUSCENES_H */
