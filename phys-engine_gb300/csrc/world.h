// Host side of a GPU world: the reference's slot/generation storage
// (src/world/physics_world.cpp:162-339) kept as a host mirror, device
// structure-of-arrays state, and the step pipeline.
#pragma once
#include <utility>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "pe_engine.h"
#include "pe_stages.h"

namespace pe {

template <class T> struct DeviceArray {
    T *ptr = nullptr;
    size_t count = 0;
    DeviceArray() = default;
    DeviceArray(const DeviceArray &) = delete;
    DeviceArray &operator=(const DeviceArray &) = delete;
    ~DeviceArray() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
    void swap(DeviceArray &o) {
        std::swap(ptr, o.ptr);
        std::swap(count, o.count);
    }
    // Grows to at least n elements (contents are not kept); zero-filled.
    void reserve(size_t n) {
        if (n <= count && ptr) return;
        release();
        size_t c = n ? n : 1;
        PE_CHECK(cudaMalloc(&ptr, c * sizeof(T)));
        PE_CHECK(cudaMemset(ptr, 0, c * sizeof(T)));
        PE_CHECK(cudaDeviceSynchronize());
        count = c;
    }
};

struct HostBody {
    float mass = 0, restitution = 0, friction = 0;
    bool isStatic = false;
    float pos[3] = {0, 0, 0};
    float rot[4] = {0, 0, 0, 1};
    float lin[3] = {0, 0, 0};
    float ang[3] = {0, 0, 0};
    float force[3] = {0, 0, 0};
    float iinv[3] = {0, 0, 0};  // diagonal local inverse inertia
    uint32_t generation = 0;
    bool alive = false;
    // RigidBody::sleeping / wakeRequested (rigid_body.hpp:132-133) and the
    // body's quiet time (SleepState::quietTime)
    bool sleeping = false;
    bool wakeRequested = true;
    float quiet = 0.0f;
    // State at the end of the last step (SleepState pose, mass, material,
    // static flag): host edits since then wake the body at the next step
    // (PhysicsWorld::prepareSleeping, physics_world.cpp:434-452).
    bool snapValid = false;
    bool snapStatic = false;
    float snapPos[3] = {0, 0, 0}, snapRot[4] = {0, 0, 0, 1};
    float snapMass = 0, snapRestitution = 0, snapFriction = 0;
    void wakeUp() {
        sleeping = false;
        wakeRequested = true;
    }
    bool isSleeping() const { return !isStatic && sleeping; }
};

struct HostCollider {
    uint32_t body = 0, bodyGeneration = 0;
    float lpos[3] = {0, 0, 0};
    float lrot[4] = {0, 0, 0, 1};
    uint32_t shape = 0;
    float dims[3] = {0, 0, 0};  // radius or half extents
    uint32_t hull = 0;
    uint32_t generation = 0;
    bool alive = false;
};

struct StepCounters {
    uint64_t possiblePairs = 0, candidatePairs = 0, contactCount = 0, solvedContactCount = 0;
    uint64_t awakeBodyCount = 0, sleepingBodyCount = 0, xWindow = 0, aabbPairs = 0, gridComparisons = 0, gridEntries = 0,
             gridOverflow = 0;
    double cellSize = 0;
    uint64_t npCandidates[4] = {0, 0, 0, 0}, npContacts[4] = {0, 0, 0, 0};
    uint64_t preparedPoints = 0, warmComparisons = 0, warmMatches = 0, velocityPointVisits = 0;
    uint64_t colors = 0, colorRounds = 0, epaFailures = 0, points = 0;
    double gpuMs = 0;
    // device time per stage (CUDA events on the world's stream)
    double integrateMs = 0, broadphaseMs = 0, narrowphaseMs = 0, solverMs = 0, poseMs = 0;
    uint64_t kernelLaunches = 0;
    bool graphed = false;  // the step ran from a captured CUDA graph
    // device time of the one-cluster solver's phases (ms; zero when it did not
    // run): prepare, island union, island lists, plan + staging (or colouring),
    // sweeps, write-back, cache rebuild
    double solverPhaseMs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

// Copies M manifolds of a device manifold view into pe_contact_manifold records.
void downloadManifoldRecords(const ManifoldView &mv, uint32_t M, void *records);

class World {
  public:
    explicit World(int device);
    ~World();
    World(const World &) = delete;
    World &operator=(const World &) = delete;

    // configuration (PhysicsWorld::gravity, broadPhaseAlgorithm; solver
    // iteration count and order are additions)
    float gravity[3] = {0.0f, -9.81f, 0.0f};
    int algorithm = 0;        // 0 SAP, 1 uniform grid, 2 dynamic tree (unsupported)
    double cellSize = 0.0;    // grid: <= 0 median (reference), > 0 fixed
    int iterations = 8;
    int orderMode = 1;        // 0 manifold order (serial), 1 graph-colour order
    bool sleepingEnabled = false;  // PhysicsWorld::setSleepingEnabled

    // host mirror (bodies / colliders by slot)
    std::vector<HostBody> bodies;
    std::vector<uint32_t> freeBodies;
    std::vector<HostCollider> colliders;
    std::vector<uint32_t> freeColliders;
    std::vector<float> hullVerts;          // xyz per vertex
    std::vector<uint32_t> hullOffsets{0};

    uint32_t addBody(const HostBody &b, uint32_t &generation);
    uint32_t addCollider(const HostCollider &c, uint32_t &generation);
    void removeBody(uint32_t index, uint32_t generation);
    void removeCollider(uint32_t index, uint32_t generation);
    HostBody *body(uint32_t index, uint32_t generation);
    HostCollider *collider(uint32_t index, uint32_t generation);
    // A write through the reference's public Collider fields: body, shape and
    // local transform of a live collider.  Returns false for a stale handle.
    bool setCollider(uint32_t index, uint32_t generation, uint32_t body, uint32_t bodyGeneration, uint32_t shape,
                     const float *dims, const float *lpos, const float *lrot);
    int addHull(const float *verts, uint32_t count);

    // Host-mirror access: pull() refreshes it from the device, touch() marks it
    // modified so the next step uploads it.
    void pull();
    void touch() { hostDirty_ = true; }
    // PhysicsWorld::setSleepingEnabled (physics_world.cpp:341-351).
    void setSleepingEnabled(bool enabled);
    // The PhysicsWorld copy constructor (physics_world.cpp:74-93): bodies,
    // colliders, contacts, warm-start cache, step counters and sleep state.
    std::unique_ptr<World> clone();

    void step(float dt);
    // Bulk per-step I/O: set the accumulated force of bodies [0, n) (xyz each),
    // and read the current poses (positions xyz, rotations xyzw).
    void writeForces(const float *forces, uint32_t n);
    void readPoses(float *positions, float *rotations);
    // writeForces + step + readPoses with one synchronisation (any pointer may
    // be null).
    void stepIO(const float *forces, uint32_t n, float dt, float *positions, float *rotations);
    // Standalone stages (BroadPhase::findCandidatePairs, solve on explicit manifolds).
    void broadphaseOnly(const float *mins, const float *maxs, uint32_t n, int algo, double cell,
                        std::vector<uint32_t> &pairs, StepCounters &c);
    void solveOnly(std::vector<float> &manifoldRecords, uint32_t count, float dt, int iterations, int mode);

    const StepCounters &counters() const { return counters_; }
    uint32_t manifoldCount() const { return lastManifolds_; }
    uint32_t pairCount() const { return lastPairs_; }
    void downloadPairs(uint32_t *pairs);
    // Manifold fields in the pe_contact_manifold layout (see capi).
    void downloadManifolds(void *records, uint32_t count);
    void downloadOrder(uint32_t *order, uint32_t *colors);
    uint32_t statusBits() const { return lastErr_; }
    int device() const { return device_; }
    cudaStream_t stream() const { return stream_; }
    uint64_t stepsTaken() const { return steps_; }
    // CUDA graphs for the step (on by default; off runs the same launches directly).
    const std::string &graphError() const { return graphError_; }
    void setGraphsEnabled(bool on) {
        graphsDisabled_ = !on;
        dropGraphs();
    }
    void syncDevice();

  private:
    void push();
    void ensureCapacity();
    void ensureScratch(uint32_t maxN);
    WorldView view(float dt);
    ManifoldView manifoldView();
    CacheView cacheView(int which);
    void runPipeline(float dt);
    void runStep(float dt, const float *forces, uint32_t nForces, float *positions, float *rotations);
    void stageForces(const float *forces, uint32_t n);
    void enqueuePoses(int which, float *positions, float *rotations);
    bool finishStep();
    void computePossiblePairs();
    // PhysicsWorld::wakeContacts (physics_world.cpp:353-371) on the host mirror
    // from the last step's contacts.
    void wakeContacts(uint32_t index, uint32_t generation);

    int device_;
    int smCount_ = 0;
    cudaStream_t stream_ = nullptr;
    bool hostDirty_ = true;
    bool deviceNewer_ = false;
    bool dense_ = true;
    bool forces_ = false;
    bool localIdentity_ = true;
    uint32_t nb_ = 0, nc_ = 0, nin_ = 0;
    int cur_ = 0;
    int cache_ = 0;
    uint64_t steps_ = 0;
    uint32_t lastErr_ = 0;
    uint32_t lastPairs_ = 0, lastManifolds_ = 0, lastMEstimate_ = 0, lastRawEstimate_ = 0;
    // the last step needed more than kMaxColors solver colours: solve on the
    // multi-kernel path (the cluster solver's colour ranges hold kMaxColors)
    bool wideColors_ = false;
    uint32_t gridKeyBits_ = 64;
    uint64_t possiblePairs_ = 0, dynamicAlive_ = 0;
    StepCounters counters_;

    // body state (two copies), static body data, colliders
    DeviceArray<float4> pos_[2], rot_[2], lin_[2], ang_[2];
    DeviceArray<float4> force_, mat_, iinv_;
    DeviceArray<float> xfer3_;  // 3 floats per body: caller forces in, positions out
    DeviceArray<float> posOut_;  // 3 floats per body: positions written by the step for the caller
    // this step reads the caller's forces from xfer3_ (force3n bodies) and
    // writes packed positions to posOut_ (set per step by runStep)
    bool rawForces_ = false, packPoses_ = false;
    uint32_t force3n_ = 0;
    DeviceArray<uint32_t> poseDone_;  // arrival counter of the pose kernel's blocks
    DeviceArray<uint32_t> bflags_, bgen_;
    // sleeping: flags and quiet times (two copies, like the body state), the
    // island scratch, and the warm-start merge buffers
    DeviceArray<uint32_t> sleep_[2];
    DeviceArray<float> quiet_[2];
    DeviceArray<uint32_t> sParent_, sIsland_, sQuietMin_, sleepErr_;
    DeviceArray<unsigned long long> tKey_, tGens_;
    DeviceArray<float4> tA_, tB_;
    DeviceArray<float> tT2_;
    DeviceArray<uint32_t> tCount_, carry_, carryPos_, carryTotal_;
    uint32_t cacheNeed_ = 0;   // warm-start capacity asked for by a carry overflow
    bool wakeCheck_ = false;   // host edits since the last step: run the wake pass first
    bool solveSkipped_ = false;  // the last step solved nothing: every body asleep
    float sleepGravity_[3] = {0, 0, 0};  // PhysicsWorld::sleepGravity
    DeviceArray<uint32_t> cbody_, cbgen_, cflags_;
    DeviceArray<float4> cshape_, clpos_, clrot_, aabbMin_, aabbMax_, npRec_;
    DeviceArray<uint32_t> hullOffset_;
    DeviceArray<float4> hullVerts_;
    // broadphase input compaction
    DeviceArray<uint32_t> collectFlags_, collectPos_, inSlot_;
    DeviceArray<float4> inMin_, inMax_;
    DeviceArray<uint32_t> sapKeys_, sapVals_, sapKeyOf_, sapWords_;  // words: unsorted flag, sort count
    // broadphase / pairs
    BroadBuffers bb_{};
    DeviceArray<uint32_t> bbBucketHead_, bbEntryNext_;
    DeviceArray<uint4> bbEntryRec_;
    DeviceArray<float4> bbCand_;
    DeviceArray<uint32_t> bbKeyTmp32_, bbValTmp_, bbIdx_, bbLen_, bbOff_, bbCellCount_, bbOverflow_, bbEntryOff_,
        bbEntryVals_, bbEntryValsTmp_, bbCounters_;
    DeviceArray<float> bbMinX_, bbMaxX_;
    DeviceArray<float4> bbYZ_;
    DeviceArray<unsigned long long> bbWidth_, bbWidthTmp_, bbEntryKeys_, bbEntryKeysTmp_;
    DeviceArray<int4> bbFirst_;
    DeviceArray<uint8_t> bbInGrid_;
    uint32_t entryCap_ = 0;
    // DynamicTree: linear BVH (allocated when the selector is first used)
    LbvhBuffers lb_{};
    DeviceArray<unsigned long long> lbKeys_, lbKeysTmp_;
    DeviceArray<uint32_t> lbChildL_, lbChildR_, lbParent_, lbLeafParent_, lbRangeMax_, lbVisit_, lbBox_;
    DeviceArray<float4> lbLeafMn_, lbLeafMx_, lbNodeMn_, lbNodeMx_;
    void ensureLbvh();
    PairBuffers pb_{};
    DeviceArray<unsigned long long> pairKeys_, pairKeysTmp_;
    DeviceArray<uint32_t> pairFlags_, pairPos_, pairA_, pairB_, pairCounters_;
    uint32_t pairCap_ = 0;
    // manifolds
    uint32_t mcap_ = 0;
    DeviceArray<uint32_t> mBodyA_, mGenA_, mBodyB_, mGenB_, mCount_, mFeature_;
    DeviceArray<float4> mNormal_, mAnchorA_, mAnchorB_, mImpulse_;
    DeviceArray<float> mRest_;
    // solver
    SolverBuffers sb_{};
    DeviceArray<unsigned long long> sBest_, sUsed_, sEpoch_, sCacheKeys_, sCacheKeysTmp_;
    DeviceArray<uint32_t> sColor_, sDyn_, sColorCount_, sColorStart_, sOrderKeys_, sOrderKeysTmp_, sOrder_, sOrderTmp_, sPcount_,
        sCacheVals_, sCacheValsTmp_, sCacheCounts_, sCacheOff_, sBar_, sCounters_, sStageBody_, sIslandList_;
    DeviceArray<uint32_t> sIslPar_, sIslOff_, sIslRoot_, sIslSlot_, sIslList_, sIslRoots_, sIslLone_, sIslCounters_;
    DeviceArray<uint32_t> sIslLink_, sIslSize_, sPathHint_;
    DeviceArray<uint4> sIslandRec_;
    DeviceArray<unsigned long long> sIslKeys_, sIslKeysTmp_, sIslSort_;
    DeviceArray<float4> sPm_, sPmI_, sPp_, sPimp_, sPn_;
    DeviceArray<uint2> sPbody_, sStageSlot_;
    // warm-start caches (two copies)
    DeviceArray<unsigned long long> cKey_[2], cGens_[2];
    DeviceArray<float4> cA_[2], cB_[2];
    DeviceArray<float> cT2_[2];
    DeviceArray<uint32_t> cCount_;  // [2]
    uint32_t cacheCap_ = 0;
    // scratch and stats
    Scratch ws_{};
    DeviceArray<unsigned long long> wsScan_;
    DeviceArray<uint32_t> wsSortHist_, wsSortState_;
    uint32_t scratchN_ = 0;
    DeviceArray<DevStats> stats_;
    DevStats *hostStats_ = nullptr;
    // Captured step pipelines, one per ping-pong parity, valid for graphKey_.
    struct GraphKey {
        uint32_t nb, nc, pairCap, entryCap, mcap, cacheCap;
        float dt, gx, gy, gz;
        int algorithm, iterations, orderMode, coopBlocks;
        bool blockSolver, blockPairs, bodyPairs, hashed;
        uint32_t blockM;
        uint32_t pairBits, gridKeyBits;
        double cellSize;
        bool dense, localIdentity, forces, identityColliders, sleeping, rawForces, packPoses, ioMode;
        uint32_t force3n;
        bool operator==(const GraphKey &o) const;
    };
    cudaGraphExec_t graph_[2] = {nullptr, nullptr};
    GraphKey graphKey_[2] = {};
    unsigned long long graphLaunches_[2] = {0, 0};
    bool graphsDisabled_ = false;
    bool lastGraphed_ = false;
    std::string graphError_;
    int coopBlocks_ = 1;
    bool blockSolver_ = true;
    uint32_t blockM_ = kBlockMaxManifolds;  // manifold capacity of the single-block solver launch
    bool bodyPairs_ = true;
    bool hashGrid_ = true;  // fixed-cell grid through hashed buckets (off after a cell left its range)
    bool identityColliders_ = false;  // collider i is body i for every slot (unique body pair per manifold)  // grid pairs per body (off after a body overflowed its partner list)
    GraphKey currentKey(float dt) const;
    void dropGraphs();
    unsigned long long launchStep(float dt);
    float4 *pinned_ = nullptr;
    size_t pinnedCount_ = 0;
    float4 *pinnedBuffer(size_t n);
    // Step I/O descriptor in mapped pinned memory (host and device addresses);
    // ioMode_: this step reads and writes the caller's arrays through it.
    StepIo *ioHost_ = nullptr;
    StepIo *ioDev_ = nullptr;
    bool ioMode_ = false;
    void *deviceAddress(const void *p, size_t align) const;
};

} // namespace pe
