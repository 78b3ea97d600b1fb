// Differentiable batched rollout on the GPU: many independent worlds stepped
// `steps` times by one persistent kernel (one thread block per world at a time,
// worlds taken from a queue), with checkpoints every `checkpointEvery` steps;
// the adjoint kernel recomputes each segment from its checkpoint, recording the
// tape, and runs the hand-written reverse step by step (ad_world.cuh).
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "pe_engine.h"
#include "world.h"

namespace pe {

// Largest world of a rollout (bodies); the batched engine has the same limit.
constexpr uint32_t kRolloutMaxBodies = 8192;

class Rollout {
  public:
    explicit Rollout(int device);
    ~Rollout();
    Rollout(const Rollout &) = delete;
    Rollout &operator=(const Rollout &) = delete;

    // Per body: shape (0 sphere, 1 box), static flag, radius / half extents (3),
    // diagonal local inverse inertia (3).
    void create(const std::vector<uint32_t> &worldBodies, const std::vector<uint8_t> &shape,
                const std::vector<uint8_t> &isStatic, const std::vector<float> &halfExtents,
                const std::vector<float> &invInertia, uint32_t steps, float dt, int iterations,
                uint32_t checkpointEvery);
    float gravity[3] = {0.0f, -9.81f, 0.0f};

    // Device pointers, all worlds' bodies back to back.
    void forward(const float *x0, const float *q0, const float *v0, const float *w0, const float *mass,
                 const float *friction, const float *restitution, float *xT, float *qT, float *vT, float *wT,
                 cudaStream_t s);
    // Gradients of sum(d_final . final state) for the last forward call.
    void backward(const float *gx, const float *gq, const float *gv, const float *gw, float *gx0, float *gq0,
                  float *gv0, float *gw0, float *gmass, float *gfriction, float *grestitution, cudaStream_t s);

    // Manifold capacity per body (default 2: boxes resting on one another);
    // sparse worlds need far less.  A world that outgrows it fails the call.
    void setManifoldCapacity(float perBody);

    uint64_t bodyCount() const { return nb_; }
    uint32_t worldCount() const { return (uint32_t)worldBodies_.size(); }
    uint32_t steps() const { return steps_; }
    double lastForwardMs() const { return fwdMs_; }
    double lastBackwardMs() const { return bwdMs_; }
    size_t deviceBytes() const { return bytes_; }
    int threads = 128;

  private:
    void checkErrors(cudaStream_t s, const char *what);
    void ensureArena();
    uint32_t quarterPerBody_ = 8;

    int device_;
    uint64_t nb_ = 0;
    uint32_t steps_ = 0, ckEvery_ = 10, nMax_ = 0, nCk_ = 0;
    float dt_ = 1.0f / 120.0f;
    int iterations_ = 10;
    bool haveForward_ = false;
    std::vector<uint32_t> worldBodies_;
    double fwdMs_ = 0, bwdMs_ = 0;
    size_t bytes_ = 0;
    cudaEvent_t e0_ = nullptr, e1_ = nullptr;
    uint32_t *hostErr_ = nullptr;
    // per body
    DeviceArray<uint32_t> bodyStart_;
    DeviceArray<uint8_t> shape_, static_;
    DeviceArray<float> dims_, iinv_, mass_, mu_, rest_;
    // per world slots, each sized by its world's body count
    DeviceArray<unsigned char> arena_;
    DeviceArray<unsigned long long> worldOff_;
    DeviceArray<uint32_t> order_;
    DeviceArray<uint32_t> queue_, err_;
};

} // namespace pe
