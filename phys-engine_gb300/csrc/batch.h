// Batched worlds: thousands of independent worlds of uneven size stepped by one
// persistent kernel per size bucket.  Each world is exactly a PhysicsWorld of
// sphere/box bodies with one collider each (body i owns collider i), stepped as
// PhysicsWorld::step (src/world/physics_world.cpp:518-782) with the SAP
// broadphase and the graph-colour solve order; a world's results equal those of
// the single-world engine on the same bodies.
#pragma once
#include <string>
#include <vector>

#include "pe_engine.h"
#include "pe_stages.h"
#include "world.h"

namespace pe {

// One world's slice of the batch arrays.
struct WorldDesc {
    uint32_t bodyStart, bodyCount;
    uint32_t pairBase, pairCap;    // pair-key slice; pairCap is a power of two
    uint32_t mBase, mCap;          // manifold slice (points at 4 * mBase)
    uint32_t cacheBase, cacheCap;  // warm-start cache slice (cacheCap = 4 * mCap)
};

// Everything one bucket launch needs (passed by value).
struct BatchView {
    BodyState state[2];
    const float4 *force;  // nullable
    const float4 *mat, *iinv;
    const uint32_t *bflags, *bgen;
    const uint32_t *cbody, *cbgen, *cflags;
    const float4 *cshape;
    float4 *aabbMin, *aabbMax;
    unsigned long long *pairKeys;
    ManifoldView mv;
    SolverBuffers sb;  // block-path fields; per-world slices are taken in the kernel
    CacheView cache[2];
    uint32_t *cacheCount;  // [2 * worlds]
    unsigned long long *epoch;  // [worlds]
    uint32_t *colorCount;  // [worlds * kMaxColors]
    DevStats *stats;       // [worlds]
    const WorldDesc *worlds;
    const uint32_t *queue;  // world ids of this bucket, largest first
    uint32_t queueLen;
    uint32_t *queueHead;    // work counter of this bucket (zeroed before the launch)
    uint32_t *batchErr;     // OR of all worlds' error bits
    uint32_t worldCount;
    uint32_t maxM;          // shared-memory manifold capacity of this launch
    uint32_t maxN;          // largest world of this bucket (shared-memory SAP keys)
    int iterations;
    uint32_t parity;        // state[parity] is read, state[parity ^ 1] written
    float gx, gy, gz, dt;
};

// Kernel variants the autotuner chooses from: threads per block and the
// minimum resident blocks per SM the register allocation is built for (more
// blocks = fewer registers per thread).
struct BatchVariant {
    int threads, minBlocks;
};
constexpr BatchVariant kBatchVariants[] = {{128, 1}, {128, 4}, {256, 1}, {256, 2}, {512, 1}};
constexpr int kBatchVariantCount = 5;
// Dynamic shared memory of a launch: SAP keys of the largest world or the
// solver's manifold arrays, whichever is larger.
size_t batchSharedBytes(uint32_t maxN, uint32_t maxM);
// Resident blocks over the whole GPU for a variant (also sets its shared-memory limit).
uint32_t batchMaxBlocks(int variant, size_t smem);
void launchBatchBucket(const BatchView &b, int variant, uint32_t blocks, cudaStream_t s);

struct BatchBucket {
    uint32_t lo = 0, hi = 0;        // body-count range [lo, hi]
    std::vector<uint32_t> worlds;   // largest first
    uint32_t queueOff = 0;          // offset of this bucket's worlds in the device queue
    uint32_t maxN = 0, maxM = 0;
    int variant = 2;
    uint32_t blocks = 0;
    double tunedMs = 0;             // autotuner's best time per launch (0 = not tuned)
    std::vector<double> candidateMs;
};

class Batch {
  public:
    explicit Batch(int device);
    ~Batch();
    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;

    // bodies[i] / colliders[i] concatenated world by world; colliders[i].body
    // is the body index within its world.
    void create(const std::vector<uint32_t> &worldBodies, const std::vector<HostBody> &bodies,
                const std::vector<HostCollider> &colliders);

    float gravity[3] = {0.0f, -9.81f, 0.0f};
    int iterations = 8;

    uint32_t worldCount() const { return (uint32_t)desc_.size(); }
    uint64_t bodyCount() const { return nb_; }
    const std::vector<uint32_t> &worldBodies() const { return worldBodies_; }
    const std::vector<BatchBucket> &buckets() const { return buckets_; }

    void step(float dt);
    // Times every kernel variant on each bucket (`reps` launches each, from the
    // current state, which they leave unchanged) and keeps the fastest.
    void autotune(float dt, int reps);
    void setGraphsEnabled(bool on) {
        graphsDisabled_ = !on;
        dropGraphs();
    }
    const std::string &graphError() const { return graphError_; }
    // Settings captured in the graphs (gravity, iterations) changed.
    void invalidateGraphs() { dropGraphs(); }

    void readBodies(float *pos, float *rot, float *lin, float *ang);
    void writeBodies(const float *pos, const float *rot, const float *lin, const float *ang);
    void writeForces(const float *forces);
    void readPoses(float *pos, float *rot);
    void worldCounters(uint32_t w, StepCounters &c);
    uint32_t worldPairs(uint32_t w, uint32_t *pairs, uint32_t capacity);
    uint32_t worldManifolds(uint32_t w, void *records, uint32_t capacity);
    double lastStepMs() const { return lastMs_; }
    uint64_t kernelLaunches() const { return lastLaunches_; }
    bool lastGraphed() const { return lastGraphed_; }
    cudaStream_t stream() const { return stream_; }
    uint64_t stepsTaken() const { return steps_; }
    size_t deviceBytes() const { return deviceBytes_; }

  private:
    void layout(const std::vector<uint32_t> &pairCap, const std::vector<uint32_t> &mCap, bool keepCaches);
    void makeBuckets();
    BatchView view(const BatchBucket &bk, float dt, uint32_t parity) const;
    void launchAll(float dt, uint32_t parity);
    bool finishStep();
    void dropGraphs();

    int device_;
    cudaStream_t stream_ = nullptr;
    std::vector<cudaStream_t> side_;
    std::vector<cudaEvent_t> joins_;
    cudaEvent_t fork_ = nullptr, t0_ = nullptr, t1_ = nullptr;
    uint64_t nb_ = 0;
    uint32_t parity_ = 0;
    uint64_t steps_ = 0;
    bool forces_ = false;
    std::vector<uint32_t> worldBodies_;
    std::vector<WorldDesc> desc_;
    std::vector<BatchBucket> buckets_;

    // bodies (two state copies), colliders
    DeviceArray<float4> pos_[2], rot_[2], lin_[2], ang_[2];
    DeviceArray<float4> force_, mat_, iinv_, cshape_, aabbMin_, aabbMax_;
    DeviceArray<uint32_t> bflags_, bgen_, cbody_, cbgen_, cflags_;
    // pairs, manifolds, solver, caches
    DeviceArray<unsigned long long> pairKeys_;
    DeviceArray<uint32_t> mBodyA_, mGenA_, mBodyB_, mGenB_, mCount_, mFeature_;
    DeviceArray<float4> mNormal_, mAnchorA_, mAnchorB_, mImpulse_;
    DeviceArray<float> mRest_;
    DeviceArray<unsigned long long> bodyBest_, bodyUsed_, epoch_;
    DeviceArray<uint32_t> color_, dyn_, colorCount_, order_, colorStart_;
    DeviceArray<float4> pm_, pmInertia_, pp_, pimp_, pn_;
    DeviceArray<uint2> pbody_;
    DeviceArray<uint32_t> pcount_;
    DeviceArray<unsigned long long> cacheKey_[2], cacheGens_[2];
    DeviceArray<float4> cacheA_[2], cacheB_[2];
    DeviceArray<float> cacheT2_[2];
    DeviceArray<uint32_t> cacheCount_;
    DeviceArray<DevStats> stats_;
    DeviceArray<WorldDesc> descDev_;
    DeviceArray<uint32_t> queue_, queueHead_, batchErr_;
    uint32_t *hostErr_ = nullptr;
    DeviceArray<float> xfer_;  // forces in / poses out when the caller's arrays are pageable
    uint64_t pairTotal_ = 0, mTotal_ = 0, cacheTotal_ = 0;
    size_t deviceBytes_ = 0;

    // one graph per (state parity, forces pending for this step)
    cudaGraphExec_t graph_[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    float graphDt_ = 0.0f;
    bool graphsDisabled_ = false;
    std::string graphError_;
    double lastMs_ = 0;
    uint64_t lastLaunches_ = 0;
    bool lastGraphed_ = false;
};

} // namespace pe
