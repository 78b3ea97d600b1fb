// Narrowphase: one candidate pair per thread; manifolds are compacted in pair
// order in the same pass (block scan of hit flags + decoupled look-back), so
// manifold order equals the reference's (src/world/physics_world.cpp:692-736).
// Per pair this is the world's generateContact lambda
// (physics_world.cpp:645-691): collider world transforms, shape dispatch with
// the box-sphere swap (src/collision/narrowphase.cpp:353-365), anchors moved
// from collider space to body space, restitution = max, friction =
// sqrt(max(fa,0) * max(fb,0)).
#include "pe_kernels.cuh"
#include "pe_narrow.cuh"
#include "pe_stages.h"

namespace pe {

// Small tiles spread the few candidate pairs of a step over many SMs: each
// pair is a long dependent chain of arithmetic, so latency, not issue rate,
// bounds a tile.
constexpr int kNarrowThreads = 64;
static_assert(kNarrowThreads >= (int)kMinLookbackTile, "look-back scratch is sized for kMinLookbackTile");

__global__ void __launch_bounds__(kNarrowThreads)
k_narrowphase(WorldView w, const uint32_t *__restrict__ pairA, const uint32_t *__restrict__ pairB,
              const uint32_t *d_pairs, ManifoldView out, uint32_t mcap, DevStats *st, unsigned long long *state,
              uint32_t *counter) {
    __shared__ uint32_t s_tile, s_scan[9], s_prefix, s_abort;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->stamp[2] = globalNs();
    const uint32_t P = min(*d_pairs, mcap);
    const uint32_t ntiles = max((P + kNarrowThreads - 1) / kNarrowThreads, 1u);
    for (;;) {
    const uint32_t tile = takeTile(counter, &s_tile);
    if (tile >= ntiles) return;
    const uint32_t p = tile * kNarrowThreads + threadIdx.x;

    LocalManifold lm;
    lm.count = 0;
    bool hit = false;
    uint32_t ca = 0, cb = 0, ba = 0, bb = 0, ga = 0, gb = 0, category = 0;
    float restitution = 0.0f, friction = 0.0f;
    if (p < P) {
        ca = pairA[p];
        cb = pairB[p];
        bool epaFailed;
        if (w.npRec) {
            // both colliders' packed records: one 64-byte line each
            float4 ra[4], rb[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                ra[k] = w.npRec[4 * (size_t)ca + k];
                rb[k] = w.npRec[4 * (size_t)cb + k];
            }
            ba = __float_as_uint(ra[3].z);
            bb = __float_as_uint(rb[3].z);
            ga = __float_as_uint(ra[3].w);
            gb = __float_as_uint(rb[3].w);
            hit = narrowphasePairRec(w, ca, cb, ra, rb, lm, restitution, friction, category, epaFailed);
        } else {
            ba = w.cbody[ca];
            bb = w.cbody[cb];
            ga = w.cbgen[ca];
            gb = w.cbgen[cb];
            hit = narrowphasePair(w, ca, cb, ba, bb, lm, restitution, friction, category, epaFailed);
        }
        if (epaFailed) atomicAdd(&st->epaFailures, 1ull);
        aggregatedCount(st->npCandidates, category);
        if (hit) aggregatedCount(st->npContacts, category);
    }
    uint32_t total;
    const uint32_t local = blockExclusiveScan(hit ? 1u : 0u, total, s_scan);
    if (threadIdx.x < 32) {
        bool timedOut;
        const uint32_t pre = lookbackExclusiveWarp(state, tile, total, &st->err, &timedOut);
        if (threadIdx.x == 0) {
            s_prefix = pre;
            s_abort = timedOut ? 1u : 0u;
        }
    }
    __syncthreads();
    if (s_abort) return;  // a bounded wait ran out: nothing of this tile is written
    const uint32_t m = s_prefix + local;
    if (hit) {
        if (m < mcap) storeManifoldGen(out, m, ba, ga, bb, gb, lm, restitution, friction);
        aggregatedAdd32(&st->points, (uint32_t)lm.count);
    }
    if (threadIdx.x == 0 && tile + 1 == ntiles) {
        st->manifolds = s_prefix + total;
        st->stamp[3] = globalNs();
    }
    __syncthreads();
    }
}

void launchNarrowphase(const WorldView &w, const PairBuffers &pb, const ManifoldView &mv, uint32_t mcap, DevStats *st,
                       Scratch &ws, cudaStream_t s, unsigned long long *state, bool stateCleared) {
    uint32_t tiles = (pb.cap + kNarrowThreads - 1) / kNarrowThreads;
    if (tiles == 0) tiles = 1;
    if (!state) state = ws.scanState;
    if (!stateCleared) PE_CHECK(cudaMemsetAsync(state, 0, sizeof(unsigned long long) * (tiles + 1), s));
    const uint32_t maxGrid = 8u * (uint32_t)smCount();
    const uint32_t grid = tiles < maxGrid ? tiles : maxGrid;
    k_narrowphase<<<grid, kNarrowThreads, 0, s>>>(w, pb.a, pb.b, &st->pairs, mv, mcap, st, state,
                                                   (uint32_t *)(state + tiles));
    PE_LAUNCHED();
}

} // namespace pe

namespace pe {

// NarrowPhase::generateContact on explicit transforms (sphere / box only):
// in[6k..6k+5] = dims A (w = shape), pos A, rot A, dims B (w = shape), pos B, rot B;
// out[11k..] = normal (w = hit, point count in bits), 4 x anchorA (w = depth),
// 4 x anchorB, features as uint bits in two float4.
__global__ void k_generate_pairs(const float4 *in, float4 *out, uint32_t n) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 da = in[6 * k], pa = in[6 * k + 1], ra = in[6 * k + 2];
    const float4 db = in[6 * k + 3], pb = in[6 * k + 4], rb = in[6 * k + 5];
    const uint32_t sa = (uint32_t)da.w, sb = (uint32_t)db.w;
    Tf tA{f4xyz(pa), f4q(ra)}, tB{f4xyz(pb), f4q(rb)};
    LocalManifold lm;
    lm.count = 0;
    bool hit;
    if (sa == kShapeSphere && sb == kShapeSphere) hit = sphereSphere(da.x, tA, db.x, tB, lm);
    else if (sa == kShapeSphere) hit = sphereBox(da.x, tA, V3{db.x, db.y, db.z}, tB, lm);
    else if (sb == kShapeSphere) {
        hit = sphereBox(db.x, tB, V3{da.x, da.y, da.z}, tA, lm);
        if (hit) {
            lm.normal = -lm.normal;
            for (uint32_t i = 0; i < lm.count; ++i) {
                V3 t = lm.anchorA[i];
                lm.anchorA[i] = lm.anchorB[i];
                lm.anchorB[i] = t;
            }
        }
    } else hit = boxBox(V3{da.x, da.y, da.z}, tA, V3{db.x, db.y, db.z}, tB, lm);
    float4 *o = out + 11 * k;
    o[0] = make_float4(lm.normal.x, lm.normal.y, lm.normal.z, hit ? (float)lm.count : -1.0f);
    for (uint32_t i = 0; i < 4; ++i) {
        bool live = hit && i < lm.count;
        o[1 + i] = live ? make4(lm.anchorA[i], lm.depth[i]) : make_float4(0, 0, 0, 0);
        o[5 + i] = live ? make4(lm.anchorB[i], 0.0f) : make_float4(0, 0, 0, 0);
    }
    uint32_t f[4];
    for (uint32_t i = 0; i < 4; ++i) f[i] = (hit && i < lm.count) ? lm.feature[i] : 0u;
    o[9] = make_float4(__uint_as_float(f[0]), __uint_as_float(f[1]), __uint_as_float(f[2]), __uint_as_float(f[3]));
    o[10] = make_float4(0, 0, 0, 0);
}

void launchGeneratePairs(const float4 *in, float4 *out, uint32_t n, cudaStream_t s) {
    if (!n) return;
    k_generate_pairs<<<(n + 127) / 128, 128, 0, s>>>(in, out, n);
    PE_LAUNCHED();
}

void setSpinLimitNarrow(uint32_t limit) { setSpinLimitOfUnit(limit); }

} // namespace pe
