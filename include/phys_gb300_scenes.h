/*
 * Seeded synthetic workloads for phys-engine-gb300 (benchmarks and parity tests).
 *
 * Counterpart in the reference: benchmarks/bench_scenes.cpp:11-93
 * (makeMixedField / makeSphereField), which builds scenes directly into a
 * PhysicsWorld.  Here a scene is returned as plain arrays of body-creation
 * records so the same scene can be loaded into the GPU world, the CPU oracle
 * and the reference itself through their own public creation calls.
 */
#ifndef PHYS_GB300_SCENES_H
#define PHYS_GB300_SCENES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PE_SCENE_SPHERES_ON_FLOOR = 1,   /* n spheres r~U[.25,.5] in 20x40x20 m over a floor */
    PE_SCENE_MIXED_VOLUME = 2,       /* n mixed spheres/boxes, N(0,1) velocities, no floor */
    PE_SCENE_PYRAMIDS = 3,           /* n x n box pyramids (base 20) + convex hulls */
    PE_SCENE_PYRAMIDS_BOXES_ONLY = 4,/* the same pyramids without hulls */
    PE_SCENE_BOXES_ON_PLANE = 5      /* n boxes resting on a floor slab */
};

/* Per body (count entries): shape 0 sphere / 1 box / 2 hull; dims = radius or
   full box size (hull: ellipsoid semi-axes, informational); pos; density g/cm^3;
   is_static; restitution; friction; linvel; spin (orientation idiom vector);
   hull_id, mass, inv_inertia (hulls only).  Hull vertices of hull h are
   hull_vertices[3*hull_offsets[h] .. 3*hull_offsets[h+1]). */
typedef struct pe_scene {
    uint32_t count;
    uint8_t *shape;
    uint8_t *is_static;
    float *dims;
    float *pos;
    float *density;
    float *restitution;
    float *friction;
    float *linvel;
    float *spin;
    int32_t *hull_id;
    float *mass;
    float *inv_inertia;
    uint32_t hull_count;
    uint32_t *hull_offsets;
    float *hull_vertices;
} pe_scene;

int pe_scene_generate(int kind, uint32_t n, uint32_t seed, pe_scene *out);
void pe_scene_free(pe_scene *scene);

#ifdef __cplusplus
}
#endif

#endif
