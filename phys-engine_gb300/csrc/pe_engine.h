// Internal declarations of the GB300 engine: device-side views of a world,
// scratch memory, and the stage launchers used by the step pipeline.
#pragma once
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <cuda_runtime.h>

namespace pe {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define PE_CHECK(expr)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            throw ::pe::CudaError(std::string(#expr) + ": " + cudaGetErrorString(e_));             \
    } while (0)

// Every kernel launch of the engine is followed by PE_LAUNCHED(): it checks the
// launch and counts it (the count is reported per step).
extern unsigned long long g_kernelLaunches;

// Iteration limit of the bounded waits on the current device (0 = the
// default); each setSpinLimit* writes one translation unit's copy.
void setSpinLimit(uint32_t limit);
void setSpinLimitPrims(uint32_t limit);
void setSpinLimitBroad(uint32_t limit);
void setSpinLimitNarrow(uint32_t limit);
void setSpinLimitSleep(uint32_t limit);
void setSpinLimitSolve(uint32_t limit);
void setSpinLimitIslands(uint32_t limit);

// Streaming multiprocessors of the current device (queried once per device and
// cached); launch sizes of the persistent and grid-stride kernels scale with it.
int smCount();

// The device address of a caller's array when kernels on `device` can read and
// write it in place — pinned host memory (mapped into every device's address
// space under unified addressing; on GB300 reached over NVLink-C2C) or memory
// of that device — aligned to `align` bytes; nullptr otherwise (pageable host
// memory goes through copies).
void *deviceAddress(const void *p, size_t align, int device);
#define PE_LAUNCHED()                                                                               \
    do {                                                                                            \
        PE_CHECK(cudaGetLastError());                                                               \
        ++::pe::g_kernelLaunches;                                                                   \
    } while (0)

// Error bits shared by all kernels (written to the step's status word).
enum : uint32_t {
    kErrTimeout = 1u,
    kErrPairCapacity = 2u,
    kErrManifoldCapacity = 4u,
    kErrColors = 8u,
    kErrEntryCapacity = 16u,
    kErrEpa = 32u,
    kErrSmallPath = 64u,  // a single-block path saw more work than it holds: re-run on the full path
    kErrBodyPairs = 128u, // a body had more grid partners than the per-body pair path holds
    kErrHashRange = 256u, // a grid cell lies outside the hashed grid's coordinate range
    kErrCacheCapacity = 512u, // the warm-start cache with carried sleeping entries exceeds its capacity
    kErrTreeDepth = 1024u,    // a BVH traversal outgrew its stack
};

// Body flag bits (bflags) and collider flag layout (cflags).  kBodySleeping
// is derived data the step writes for the solver: the body sleeps this step
// (after the contact wake pass).
enum : uint32_t { kBodyAlive = 1u, kBodyStatic = 2u, kBodySleeping = 4u };
// Per-body sleep flags (PhysicsWorld sleeping, physics_world.cpp:341-516):
// RigidBody::sleeping, RigidBody::wakeRequested, and the per-step record of
// whether gravity was integrated (SleepState::integratedVelocity).
enum : uint32_t { kSleepAsleep = 1u, kSleepWake = 2u, kSleepIntegrated = 4u };
// A body that moves under impulses: alive, not static, not sleeping.
__host__ __device__ inline bool bodyMoves(uint32_t bflags) {
    return (bflags & (kBodyAlive | kBodyStatic | kBodySleeping)) == kBodyAlive;
}
enum : uint32_t { kColliderAlive = 1u };
__host__ __device__ inline uint32_t colliderShape(uint32_t cflags) { return (cflags >> 8) & 0xFFu; }
enum : uint32_t { kShapeSphere = 0, kShapeBox = 1, kShapeHull = 2 };

// Feature-id kinds (bits 24-31 of a contact feature id).
enum : uint32_t { kFeatSphereSphere = 1, kFeatSphereBox = 2, kFeatBoxFace = 3, kFeatBoxFallback = 4, kFeatHull = 5 };

// One copy of the integrated body state (the step reads one and writes the
// other, so a step can be re-run from the untouched copy).
struct BodyState {
    float4 *pos;  // xyz
    float4 *rot;  // quaternion xyzw
    float4 *lin;  // xyz
    float4 *ang;  // xyz
};

// Device counters of one step (copied to pinned host memory after the step).
struct DevStats {
    unsigned long long xWindow;
    unsigned long long aabbPairs;
    unsigned long long gridComparisons;
    unsigned long long gridEntries;
    unsigned long long gridOverflow;
    unsigned long long npCandidates[4];
    unsigned long long npContacts[4];
    unsigned long long preparedPoints;
    unsigned long long warmComparisons;
    unsigned long long warmMatches;
    unsigned long long epaFailures;
    double cellSize;
    uint32_t err;
    uint32_t inputCount;     // bounds handed to the broadphase
    uint32_t rawPairs;       // pairs emitted before dedup (capacity check)
    uint32_t uniquePairs;
    uint32_t pairs;          // candidate pairs after the same-body filter
    uint32_t manifolds;
    uint32_t points;         // contact points over all manifolds
    uint32_t colors;
    uint32_t gridEntryCount; // grid entries (capacity check)
    uint32_t overflowCount;
    uint32_t colorRounds;
    uint32_t sel;            // radix-sort buffer selector (device-side pass skipping)
    uint32_t windowWork;     // SAP flattened window work
    uint32_t solved;         // manifolds whose bodies are valid (prepared)
    uint32_t cellKeyBits;    // bits of the packed grid cell key this step needed
    uint32_t awakeBodies;    // sleeping on: live dynamic bodies awake / asleep after the step
    uint32_t sleepingBodies;
    uint32_t carried;        // sleeping on: warm-start entries carried for sleeping contacts
    uint32_t awakeInStep;    // sleeping on: live dynamic bodies awake after the contact wake pass
    uint32_t solveCount;     // sleeping on: manifolds handed to the solver (0 when no body is awake)
    uint32_t islandRefused;  // one-cluster solver: the island path cannot take this step
    int32_t cellLo[3];
    int32_t cellHi[3];
    // Phase boundaries of the one-cluster solver (global timer, ns; zero when
    // it did not run): prepare kernel start, its end (last block), cluster
    // kernel start, island lists done, planned (coloured) and staged, sweeps
    // done (island path: with the results and the cache, on the last rank),
    // then on the colour-phase path results written, cache rebuilt.
    unsigned long long solverStamp[8];
    // Stage boundaries (global timer, ns), written by the stage kernels
    // themselves instead of event nodes in the step graph: integrate start,
    // integrate end (latest block), narrowphase start, narrowphase end (last
    // tile), pose start, pose end (latest block).  Not cleared per step: the
    // "latest block" entries are maxima of an increasing clock.
    unsigned long long stamp[6];
};
static_assert(sizeof(DevStats) % 8 == 0, "DevStats is copied in 8-byte words");

// A step's I/O in the caller's own memory (pinned host or device memory, which
// the kernels address directly: on GB300 the host arrays are read and written
// over NVLink-C2C inside the step, with no copy operations).  The host rewrites
// it before each step; the step reads it at run time, so one captured graph
// serves every call.
struct StepIo {
    const float *force3;  // xyz per body for bodies [0, force3n), zero beyond (null: none)
    float *pos3;          // xyz per body, written by the pose kernel (null: none)
    float4 *rot4;         // quaternion per body, written by the pose kernel (null: none)
    uint32_t force3n;
    uint32_t pad;
};

struct WorldView {
    uint32_t nb, nc;
    BodyState cur, nxt;
    const StepIo *io;        // nullable: the step's I/O descriptor (in place of force3 / pos3)
    const float4 *force;     // nullable: all forces zero
    // nullable: the caller's forces as they were handed over (xyz for bodies
    // [0, force3n), zero beyond), read in place of `force`
    const float *force3;
    uint32_t force3n;
    // nullable: positions also written here as xyz per body by the pose kernel
    float *pos3;
    const float4 *mat;       // invMass, restitution, friction, mass
    const float4 *iinv;      // diagonal local inverse inertia (xyz)
    const uint32_t *bflags;
    const uint32_t *bgen;
    const uint32_t *cbody;
    const uint32_t *cbgen;
    const uint32_t *cflags;
    const float4 *cshape;    // sphere: radius in x; box: half extents; hull: hull index in w (as uint bits)
    const float4 *clpos;     // nullable: all local positions zero
    const float4 *clrot;     // nullable: all local rotations identity
    const uint32_t *hullOffset;
    const float4 *hullVerts;
    float4 *aabbMin;
    float4 *aabbMax;
    // nullable: per collider slot c, the narrowphase's view of the collider in
    // one 64-byte line, written with its box by the integrate kernel:
    // [4c] world position, dims.x; [4c+1] world rotation; [4c+2] dims.y,
    // dims.z, dims.w (hull index bits), collider flags (bits); [4c+3] the
    // body's restitution, friction, body index (bits), body generation (bits)
    float4 *npRec;
    float gx, gy, gz, dt;
    // Sleeping (zero / null when off).  Sleep flags and quiet times are read
    // from the step's input copy and written to its output copy; parent,
    // island and quietMin are per-body scratch of the island pass.
    uint32_t sleepMode;
    const uint32_t *sleepIn;
    uint32_t *sleepOut;
    const float *quietIn;
    float *quietOut;
    uint32_t *sleepParent;
    uint32_t *sleepIsland;
    uint32_t *sleepQuietMin;
};

// Contact manifolds (structure of arrays; manifold m owns points 4m..4m+3).
struct ManifoldView {
    uint32_t *bodyA, *genA, *bodyB, *genB;
    float4 *normalFriction;  // normal xyz, friction
    float *restitution;
    uint32_t *pointCount;
    float4 *anchorA;         // xyz, penetration
    float4 *anchorB;         // xyz
    float4 *impulse;         // normal, tangent1, tangent2
    uint32_t *feature;
};

// Warm-start cache (sorted by (bodyA index, bodyB index); generations checked).
struct CacheView {
    unsigned long long *key;  // bodyA index << 32 | bodyB index
    unsigned long long *gens; // bodyA gen << 32 | bodyB gen
    float4 *anchorA;          // xyz, normal impulse
    float4 *anchorB;          // xyz, tangent impulse 1
    float *tangent2;
};

struct Scratch {
    unsigned long long *scanState = nullptr;
    uint32_t *sortHist = nullptr;
    uint32_t *sortState = nullptr;
};

void launchScanExclusive(const uint32_t *in, uint32_t *out, const uint32_t *d_n, uint32_t max_n, uint32_t *d_total,
                         Scratch &ws, uint32_t *d_err, cudaStream_t s);
template <class K>
void launchRadixSort(K *keys, K *keys_tmp, uint32_t *vals, uint32_t *vals_tmp, const uint32_t *d_n, uint32_t max_n,
                    int bit_begin, int bit_end, Scratch &ws, uint32_t *d_err, cudaStream_t s);
void launchClamp(const uint32_t *src, uint32_t cap, uint32_t *dst, cudaStream_t s);
size_t scratchBytesScan(uint32_t max_n);
size_t scratchBytesSort(uint32_t max_n);

} // namespace pe
