// Buffers and launchers of the step stages (broadphase, narrowphase, solver).
#pragma once
#include "pe_engine.h"

namespace pe {

struct BroadInput {
    const float4 *mn;
    const float4 *mx;
    const uint32_t *d_n;  // live count on the device
    uint32_t maxN;        // launch bound
};

// Fewest items per tile of any single-pass kernel with a tile look-back
// (scratch holds one state word per tile).
constexpr uint32_t kMinLookbackTile = 64;

struct BroadBuffers {
    // SAP
    uint32_t *keyTmp32, *valTmp;
    float *sMinX, *sMaxX;
    float4 *sYZ;
    uint32_t *sIdx, *len, *off;
    // grid
    unsigned long long *widthKeys, *widthTmp;
    int4 *firstCell;
    uint32_t *cellCount;
    uint8_t *inGrid;
    uint32_t *overflow, *entryOff;
    unsigned long long *entryKeys, *entryKeysTmp;
    uint32_t *entryVals, *entryValsTmp;
    uint32_t entryCap;
    uint32_t keyBits;    // cell-key bits sorted this step (from the previous step's cell range)
    uint32_t *counters;  // [4] device scratch counters
    // hashed grid (fixed cell size): per bucket (a hash of the cell key) a list
    // of entries; entryNext[e] links entry e to the bucket's next entry
    uint32_t *bucketHead;  // [1 << logBuckets]
    uint32_t *entryNext;   // [entryCap]
    // set per launch by the step pipeline: the bucket heads were cleared by
    // the integrate kernel; the insert kernel zeroes nZeroState look-back
    // words at zeroState (the pair and narrowphase tiles' states)
    bool headsCleared;
    unsigned long long *zeroState;
    uint32_t nZeroState;
    uint32_t logBuckets;
    bool hashed;
    // hashed grid, packed for the pair walk: entry e = (cell key low, cell key
    // high, body, next entry) in one 16-byte record; body i's candidate record
    // = (min.xyz, first-cell key low) and (max.xyz, first-cell key high), one
    // 32-byte sector
    uint4 *entryRec;   // [entryCap]
    float4 *cand;      // [2 * maxN]
};

// Linear BVH of the DynamicTree selector (k_lbvh.cu), sized for maxN leaves.
struct LbvhBuffers {
    unsigned long long *keys, *keysTmp;   // Morton code << index bits | index
    uint32_t *childL, *childR, *parent;   // internal nodes (leaf children flagged)
    uint32_t *leafParent, *rangeMax, *visit;
    float4 *leafMn, *leafMx;              // leaf bounds in sorted order
    float4 *nodeMn, *nodeMx;              // internal node bounds
    uint32_t *box;                        // [6] ordered-float bounds of the centres
};

struct PairBuffers {
    unsigned long long *keys, *keysTmp;
    uint32_t cap;
    uint32_t bits;         // pair key = (first << bits) | second
    bool blockPath;        // single-block finalize (raw pairs <= kBlockMaxPairs)
    bool bodyPath;         // grid: pairs emitted per body in final order (no sort / finalize)
    uint32_t *flags, *pos;
    uint32_t *a, *b;       // candidate pairs (collider slots), lexicographic
    uint32_t *counters;    // [4]
};

struct SolverBuffers {
    uint32_t mcap;
    // colouring
    unsigned long long *bodyBest;   // [nb] round-stamped max priority
    unsigned long long *bodyUsed;   // [2 * nb] colour masks of the current window of kMaxColors colours
    unsigned long long *epoch;      // [1] persistent round stamp
    uint32_t *color;                // [mcap]
    uint32_t *dyn;                  // [mcap] bit0 A dynamic, bit1 B dynamic
    uint32_t *colorCount;           // [kMaxColors]
    uint32_t *colorStart;           // [mcap] steps with more than kMaxColors colours: first solve index
                                    // (block paths), or counts then fill cursors (multi-kernel path) per colour
    uint32_t *orderKeys, *orderKeysTmp, *order, *orderTmp;  // [mcap]
    // prepared data, in solve order k (structure of arrays)
    float4 *pm;                     // [mcap] invMassA, staticA, invMassB, staticB
    float4 *pmInertia;              // [6 * mcap] rows of the world inverse inertia (A: 3, B: 3)
    float4 *pp;                     // [kPreparedVec4 * 4 * mcap] prepared contact points
    float4 *pimp;                   // [4 * mcap] normal, tangent1, tangent2 impulse, warm-start match flag
    float4 *pn;                     // [mcap] normal, friction
    uint2 *pbody;                   // [mcap] body A, body B
    uint32_t *pcount;               // [mcap] point count
    // cache rebuild
    unsigned long long *cacheKeys, *cacheKeysTmp;
    uint32_t *cacheVals, *cacheValsTmp;
    uint32_t *cacheCounts, *cacheOff;
    uint32_t *bar;                  // grid barrier [2]
    uint32_t *counters;             // [4]
    // cluster solver: staging slots by solve index and the body of each slot
    // (colour-phase path); the manifolds of each island, kIslandMax entries
    // per root body (island path)
    uint2 *stageSlot;               // [mcap]
    uint32_t *stageBody;            // [2 * mcap + 64]
    uint32_t *islandList;           // [kIslandMax * nb]
    // island sweeps of the multi-kernel path (k_solve_islands.cu)
    uint32_t *islPar;               // [2 * nb] union-find parents, then per-root manifold counts
    uint32_t *islOff;               // [nb] list offset of each root's island
    uint32_t *islRoot, *islSlot;    // [mcap] island root and slot of each solved manifold
    uint32_t *islList;              // [mcap] manifolds island by island
    uint32_t *islRoots, *islLone;   // [mcap] island roots; solved manifolds without a dynamic body
    unsigned long long *islKeys, *islKeysTmp;  // [mcap] island queue (as u32), spare
    unsigned long long *islSort;    // [2 * mcap] sort scratch of large islands
    uint32_t *islCounters;          // [kIslCounterWords] islands, lone manifolds, work queue, listed manifolds,
                                    // queue fills; large islands' manifolds per colour and fill cursors
    // island path of the cluster solver: union-find links stored as parent XOR
    // body (0 at a root, so the zero-filled array is every body on its own) and
    // the manifolds listed at each root; the solver returns both to zero before
    // it ends.  islandRec: kIslandMax records per root body, one per manifold
    // {manifold | flags << 13 | points << 16, body A, body B, spare}.
    uint32_t *islLink;              // [nb]
    uint32_t *islSize;              // [nb]
    uint4 *islandRec;               // [kIslandMax * nb]
    // [1] steps in which the cluster solver goes straight to its colour-phase
    // path without the island attempt (set when an attempt was refused; kept
    // by the device across steps, zero in a new world)
    uint32_t *pathHint;
};
// Steps the cluster solver skips the island attempt after one was refused (a
// pile persists for many steps; the attempt is retried when this runs out).
constexpr uint32_t kPathHintSteps = 16;

constexpr int kMaxColors = 128;
constexpr uint32_t kBlockMaxPairs = 8192;
// The single-block finalize (keys sorted in registers up to 4,096, a
// shared-memory merge sort above) — or, for the one-block SAP sweep, the
// sweep's own finalize — is chosen while the expected raw pair count is at
// most this.
constexpr uint32_t kBlockPreferredPairs = 6144;
constexpr int kPreparedVec4 = 10;

void launchStepInit(DevStats *st, uint32_t inputCount, cudaStream_t s);
void launchSetManifoldCount(DevStats *st, uint32_t count, cudaStream_t s);
void launchSapKeys(const BroadInput &in, uint32_t *keys, uint32_t *vals, cudaStream_t s);
// st != nullptr: also initialises the step's counters (in place of launchStepInit).
void launchIntegrateAabb(const WorldView &w, uint32_t *sapKeys, uint32_t *sapVals, DevStats *st, uint32_t inputCount,
                         cudaStream_t s, uint32_t *fill = nullptr,
                         uint32_t nFill = 0);
void launchCollect(const WorldView &w, uint32_t *flags, uint32_t *pos, float4 *inMin, float4 *inMax, uint32_t *inSlot,
                   uint32_t *sapKeys, uint32_t *sapVals, uint32_t *d_count, Scratch &ws, uint32_t *d_err,
                   cudaStream_t s);
// hostOut (nullable): pinned host memory the counters are copied to by the
// kernel's last block (done: a zeroed arrival counter).
void launchIntegratePose(const WorldView &w, cudaStream_t s, DevStats *st = nullptr, DevStats *hostOut = nullptr,
                         uint32_t *done = nullptr);
// Host-facing transfers: caller forces (3 floats per body) into the force
// array with static / dead bodies masked; positions packed to 3 floats.
// sleep (nullable): the committed sleep flags; a nonzero force wakes its body
// (RigidBody::applyForce, rigid_body.hpp:77-85).
void launchExpandForces(const float *f3, const uint32_t *bflags, float4 *force, uint32_t n, cudaStream_t s,
                        uint32_t *sleep = nullptr);
// Sleeping (k_sleep.cu).  launchSleepWake: the wake pass of prepareSleeping
// over the last step's M contacts, on the committed sleep flags and quiet
// times (run before a step that follows host edits).  launchSleepContacts: the
// wake pass after the narrowphase inside the step (also writes the solver's
// sleeping bit into bflags).  launchSleepFinish: finishSleeping's sleep
// decision and counts after the pose kernel.  launchCacheCarry: the next
// warm-start cache from the carried sleeping entries of the old cache and
// the solver's entries (written to tmp).
struct SolveArgs;
// The multi-kernel path's sweeps island by island (after k_color and prepare):
// a thread, a warp or a block per island by its size; once an island is too
// large for a block, every island in grid-wide colour sweeps (a cooperative
// launch of at most coopBlocks blocks).
constexpr uint32_t kIslCounterWords = 10 + 2 * kMaxColors;
void launchSolveIslands(const SolveArgs &a, int coopBlocks, Scratch &ws, cudaStream_t s);
void launchSleepWake(const WorldView &w, const ManifoldView &mv, uint32_t Mhost, uint32_t mcap, uint32_t *flags,
                     float *quiet, uint32_t *err, cudaStream_t s);
void launchSleepContacts(const WorldView &w, const ManifoldView &mv, DevStats *st, uint32_t mcap, uint32_t *bflags,
                         cudaStream_t s);
void launchSleepFinish(const WorldView &w, DevStats *st, DevStats *hostOut, uint32_t *done, cudaStream_t s);
void launchSleepBits(const WorldView &w, const uint32_t *flags, uint32_t *bflags, DevStats *st, cudaStream_t s);
void launchCacheCarry(const WorldView &w, const CacheView &oldCache, const uint32_t *oldCount, const CacheView &tmp,
                      const uint32_t *tmpCount, const CacheView &newCache, uint32_t *newCount, uint32_t cap,
                      uint32_t *carry, uint32_t *carryPos, uint32_t *carryTotal, DevStats *st, Scratch &ws,
                      cudaStream_t s);
void launchPackPositions(const float4 *pos, float *p3, uint32_t n, cudaStream_t s);
// SAP order kept from step to step: keyOf[i] = min.x key of input i (written
// by the integrate kernel), unsorted / sortCount = device words.
struct SapCoherence {
    const uint32_t *keyOf;
    uint32_t *unsorted;
    uint32_t *sortCount;
};
// Collider slot of each broadphase input (null: the input index is the slot)
// and the body / generation of each slot, for the pair finalize.
struct PairMapping {
    const uint32_t *inSlot, *cbody, *cbgen;
};
// Returns true when the sweep also finalized the pairs (one-block sweep with
// `finalize` given and the raw pairs expected to fit it): the caller then
// launches no separate finalize.
bool launchSap(const BroadInput &in, uint32_t *sapKeys, uint32_t *sapVals, BroadBuffers &bb, PairBuffers &pb,
               DevStats *st, Scratch &ws, cudaStream_t s, const SapCoherence *coh = nullptr,
               const PairMapping *finalize = nullptr);
void launchGrid(const BroadInput &in, double fixedCell, BroadBuffers &bb, PairBuffers &pb, DevStats *st, Scratch &ws,
                cudaStream_t s);
// DynamicTree: every overlapping pair through a linear BVH (pair keys for
// launchPairsFinalize).
void launchLbvh(const BroadInput &in, const LbvhBuffers &lb, PairBuffers &pb, DevStats *st, Scratch &ws,
                cudaStream_t s);
// Grid pairs emitted body by body in lexicographic order, mapped to slots and
// filtered (replaces the per-cell pairs and the finalize when pb.bodyPath).
void launchGridBodyPairs(const BroadInput &in, const BroadBuffers &bb, PairBuffers &pb, const uint32_t *inSlot,
                         const uint32_t *cbody, const uint32_t *cbgen, DevStats *st, Scratch &ws, cudaStream_t s,
                         bool stateCleared = false);
void launchPairsFinalize(const uint32_t *inSlot, const uint32_t *cbody, const uint32_t *cbgen, PairBuffers &pb,
                         DevStats *st, Scratch &ws, cudaStream_t s);
void launchNarrowphase(const WorldView &w, const PairBuffers &pb, const ManifoldView &mv, uint32_t mcap, DevStats *st,
                       Scratch &ws, cudaStream_t s, unsigned long long *state = nullptr, bool stateCleared = false);
void launchSolver(const WorldView &w, const ManifoldView &mv, const CacheView &oldCache, const uint32_t *oldCacheCount,
                  const CacheView &newCache, uint32_t *newCacheCount, uint32_t cacheCap, SolverBuffers &sb,
                  int iterations, int orderMode, int coopBlocks, bool blockPath, uint32_t blockM, bool pairOrderCache,
                  DevStats *st, Scratch &ws, cudaStream_t s);
// Largest manifold count the single-block solver handles, and the largest
// body index it can key (bodies < 2^20).
constexpr uint32_t kBlockMaxManifolds = 4096;

// Cluster solver: ranks per cluster, dynamic shared memory per rank, and the
// per-rank layout (byte offsets into the dynamic shared memory).
// Islands (manifolds joined by shared dynamic bodies) of at most this many
// manifolds are solved by one thread each; a larger one sends the step to the
// colour-phase path.
constexpr uint32_t kIslandMax = 16;
constexpr uint32_t kClusterRanks = 8;
constexpr uint32_t kClusterSmemMax = 224 * 1024;
struct ClusterSolveLayout {
    uint32_t blockM, stageSlots;   // capacities of the single-block front (rank 0)
    uint32_t localCap, pointCap;   // manifolds / prepared points held per rank
    uint32_t islandBodies;         // island path: body slots per rank
    uint32_t offVel, offPm, offPn, offSlot, offM, offCnt, offOff, offPt;
    uint32_t offCacheOff;          // island path: warm-start cache offset of every manifold [blockM]
    uint32_t offPtL;               // island path: local manifold of every staged point [pointCap]
    uint32_t smemBytes;
};
constexpr uint32_t kBlockMaxBodies = 1u << 20;
int maxCooperativeBlocks(int smCount);
// Co-resident blocks per SM of the large islands' cooperative sweep kernel.
int solveIslandsBlocksPerSm();
void launchGeneratePairs(const float4 *in, float4 *out, uint32_t n, cudaStream_t s);

} // namespace pe
