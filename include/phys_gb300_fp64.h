/*
 * phys-engine-gb300 — FP64 CPU reference of the differentiable rollout.
 *
 * The GPU rollout (pe_rollout_* in phys_gb300.h) runs in FP32 on the device.
 * This library evaluates the same forward step and the same hand-written
 * adjoint in double precision on the host, from the same source, so that the
 * GPU gradients can be compared with an FP64 evaluation of one world.  It is a
 * checking tool: the GPU entry points never call it.  No reference
 * counterpart (the reference has no differentiation).
 */
#ifndef PHYS_GB300_FP64_H
#define PHYS_GB300_FP64_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mass and diagonal local inverse inertia exactly as RigidBody::createSphere /
   createBox compute them (src/dynamics/rigid_body.cpp:25-91, in float):
   shape 0 sphere (dims[0] = radius) or 1 box (dims = full width, height,
   depth).  Returns 0, or 1 for an invalid body (message in err). */
int pe_fp64_body_properties(int shape, const float *dims, float density, int is_static, float *mass,
                            float *inv_inertia, char *err, int err_len);

/* One world of n bodies stepped `steps` times (PhysicsWorld::step(dt), SAP
   pair set, graph-colour solve order, `iterations` velocity iterations) in
   double precision, starting from an empty warm-start cache.
   half_extents: radius in [0] for spheres, half extents for boxes (3 per body).
   State arrays: positions / linear / angular velocity 3 per body, rotations
   4 per body (x, y, z, w).  When d_final_* are given (any may be NULL = zero),
   also runs the adjoint and writes the gradients of
   sum(d_final . final state) with respect to the initial state, the masses,
   the frictions and the restitutions (any output may be NULL).
   Returns 0, or a nonzero status with a message in err. */
int pe_fp64_rollout(uint32_t n, const uint8_t *shape, const uint8_t *is_static, const double *half_extents,
                    const double *inv_inertia, const double *gravity, double dt, int iterations, uint32_t steps,
                    const double *x0, const double *q0, const double *v0, const double *w0, const double *mass,
                    const double *friction, const double *restitution, double *x_final, double *q_final,
                    double *v_final, double *w_final, const double *d_final_x, const double *d_final_q,
                    const double *d_final_v, const double *d_final_w, double *d_x0, double *d_q0, double *d_v0,
                    double *d_w0, double *d_mass, double *d_friction, double *d_restitution, char *err, int err_len);

#ifdef __cplusplus
}
#endif

#endif
