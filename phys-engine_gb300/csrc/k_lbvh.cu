// BroadPhaseAlgorithm::DynamicTree on the device: a linear BVH rebuilt every
// step.  The reference keeps an incremental AABB tree with fattened node bounds
// (src/collision/dynamic_aabb_tree.cpp) and reports every leaf pair whose tight
// bounds overlap, sorted lexicographically (:276-327) — the same pair set as
// sweep-and-prune, so only the way it is found differs here:
//
//   k_lbvh_bounds : bounds of the AABB centres (ordered-float atomics)
//   k_lbvh_codes  : 30-bit Morton code of each centre, key = code << b | index
//                   (unique keys), then a radix sort of the keys
//   k_lbvh_build  : binary radix tree over the sorted keys (Karras, "Maximizing
//                   Parallelism in the Construction of BVHs, Octrees, and k-d
//                   Trees", HPG 2012): one thread per internal node finds its
//                   range and split from common-prefix lengths
//   k_lbvh_refit  : node bounds bottom-up (the second child to arrive at a node
//                   unites both children and climbs on)
//   k_lbvh_pairs  : one thread per leaf walks the tree with its AABB and emits
//                   the overlapping leaves after it in sorted order (each pair
//                   once), touching counting as overlap (Aabb::overlaps)
//
// The emitted pair keys go through the common finalize (sort, mapping to
// collider slots, same-body filter), exactly like the other broadphases.
#include "pe_kernels.cuh"
#include "pe_math.cuh"
#include "pe_prims.cuh"
#include "pe_stages.h"

namespace pe {

namespace {

constexpr int kLbvhThreads = 256;
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kLbvhStack = 64;

inline int lbvhGrid(uint32_t n) {
    uint32_t b = (n + kLbvhThreads - 1) / kLbvhThreads;
    const uint32_t maxGrid = 8u * (uint32_t)smCount();
    return (int)(b ? (b < maxGrid ? b : maxGrid) : 1u);
}

__device__ __forceinline__ float orderedFloatDecode(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    return __uint_as_float(u);
}

// Spreads the low 10 bits of v to every third bit.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    uint32_t r = 0;
#pragma unroll
    for (int b = 0; b < 10; ++b) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}

__device__ __forceinline__ bool boxOverlap(const float4 &amn, const float4 &amx, const float4 &bmn, const float4 &bmx) {
    // Aabb::overlaps (include/phys/collision/aabb.hpp:15-19)
    return amn.x <= bmx.x && amx.x >= bmn.x && amn.y <= bmx.y && amx.y >= bmn.y && amn.z <= bmx.z && amx.z >= bmn.z;
}

// Common-prefix length of sorted keys i and j; -1 outside [0, n).
__device__ __forceinline__ int prefixLen(const unsigned long long *keys, uint32_t n, int i, int j) {
    if (j < 0 || j >= (int)n) return -1;
    return __clzll(keys[i] ^ keys[j]);
}

} // namespace

// box[0..2] = ordered-float minima of the centres, box[3..5] maxima.
__global__ void k_lbvh_init(uint32_t *box) {
    if (threadIdx.x < 3) box[threadIdx.x] = 0xFFFFFFFFu;
    else if (threadIdx.x < 6) box[threadIdx.x] = 0u;
}

__global__ void k_lbvh_bounds(BroadInput in, uint32_t *box) {
    const uint32_t n = *in.d_n;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = in.mn[i], b = in.mx[i];
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], c[k]);
            hi[k] = fmaxf(hi[k], c[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0 && lo[0] <= hi[0]) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(&box[k], orderedFloatKey(lo[k]));
            atomicMax(&box[3 + k], orderedFloatKey(hi[k]));
        }
    }
}

// Morton key of each centre (10 bits per axis) above the index bits.
__global__ void k_lbvh_codes(BroadInput in, const uint32_t *box, unsigned long long *keys, uint32_t indexBits) {
    const uint32_t n = *in.d_n;
    float lo[3], scale[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = orderedFloatDecode(box[k]);
        const float ext = orderedFloatDecode(box[3 + k]) - lo[k];
        scale[k] = ext > 0.0f ? 1024.0f / ext : 0.0f;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = in.mn[i], b = in.mx[i];
        const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        uint32_t q[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float t = fminf(fmaxf((c[k] - lo[k]) * scale[k], 0.0f), 1023.0f);  // NaN -> 0
            q[k] = (uint32_t)t;
        }
        const uint32_t code = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
        keys[i] = ((unsigned long long)code << indexBits) | i;
    }
}

// Internal node i of n - 1: children (leaf children flagged with kLeafBit),
// parents, the last sorted leaf it covers, and the sorted leaves' bounds.
__global__ void k_lbvh_build(BroadInput in, const unsigned long long *keys, uint32_t indexBits, uint32_t *childL,
                             uint32_t *childR, uint32_t *parent, uint32_t *leafParent, uint32_t *rangeMax,
                             uint32_t *visit, float4 *leafMn, float4 *leafMx) {
    const uint32_t n = *in.d_n;
    const unsigned long long idxMask = (1ull << indexBits) - 1ull;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t idx = (uint32_t)(keys[t] & idxMask);
        leafMn[t] = in.mn[idx];
        leafMx[t] = in.mx[idx];
        if (t + 1 >= n) continue;
        const int i = (int)t;
        visit[i] = 0u;
        const int d = prefixLen(keys, n, i, i + 1) - prefixLen(keys, n, i, i - 1) > 0 ? 1 : -1;
        const int dmin = prefixLen(keys, n, i, i - d);
        int lmax = 2;
        while (prefixLen(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int s = lmax >> 1; s >= 1; s >>= 1)
            if (prefixLen(keys, n, i, i + (l + s) * d) > dmin) l += s;
        const int j = i + l * d;
        const int dnode = prefixLen(keys, n, i, j);
        int split = 0;
        for (int s = (l + 1) >> 1;; s = (s + 1) >> 1) {
            if (prefixLen(keys, n, i, i + (split + s) * d) > dnode) split += s;
            if (s == 1) break;
        }
        const int gamma = i + split * d + (d < 0 ? -1 : 0);
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        const uint32_t left = lo == gamma ? (kLeafBit | (uint32_t)gamma) : (uint32_t)gamma;
        const uint32_t right = hi == gamma + 1 ? (kLeafBit | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
        childL[i] = left;
        childR[i] = right;
        rangeMax[i] = (uint32_t)hi;
        if (left & kLeafBit) leafParent[gamma] = (uint32_t)i;
        else parent[gamma] = (uint32_t)i;
        if (right & kLeafBit) leafParent[gamma + 1] = (uint32_t)i;
        else parent[gamma + 1] = (uint32_t)i;
    }
}

// Node bounds from the leaves up; the second arrival at a node unites both
// children (their bounds are published before the arrival counter moves).
__global__ void k_lbvh_refit(const uint32_t *d_n, const uint32_t *childL, const uint32_t *childR,
                             const uint32_t *parent, const uint32_t *leafParent, uint32_t *visit, const float4 *leafMn,
                             const float4 *leafMx, float4 *nodeMn, float4 *nodeMx) {
    const uint32_t n = *d_n;
    if (n < 2) return;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        uint32_t node = leafParent[t];
        for (uint32_t depth = 0; depth < n; ++depth) {
            __threadfence();
            if (atomicAdd(&visit[node], 1u) == 0u) break;  // the sibling finishes this node
            __threadfence();
            const uint32_t c[2] = {childL[node], childR[node]};
            float4 mn = make_float4(INFINITY, INFINITY, INFINITY, 0.0f), mx = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                float4 a, b;
                if (c[k] & kLeafBit) {
                    a = leafMn[c[k] & ~kLeafBit];
                    b = leafMx[c[k] & ~kLeafBit];
                } else {
                    a = __ldcg(&nodeMn[c[k]]);
                    b = __ldcg(&nodeMx[c[k]]);
                }
                mn = make_float4(fminf(mn.x, a.x), fminf(mn.y, a.y), fminf(mn.z, a.z), 0.0f);
                mx = make_float4(fmaxf(mx.x, b.x), fmaxf(mx.y, b.y), fmaxf(mx.z, b.z), 0.0f);
            }
            __stcg(&nodeMn[node], mn);
            __stcg(&nodeMx[node], mx);
            if (node == 0) break;
            node = parent[node];
        }
    }
}

// Leaf t's AABB against the tree; pairs with the sorted leaves after t.
__global__ void __launch_bounds__(kLbvhThreads)
k_lbvh_pairs(const uint32_t *d_n, const unsigned long long *keys, uint32_t indexBits, const uint32_t *childL,
             const uint32_t *childR, const uint32_t *rangeMax, const float4 *leafMn, const float4 *leafMx,
             const float4 *nodeMn, const float4 *nodeMx, unsigned long long *pkeys, uint32_t cap, uint32_t bits,
             DevStats *st) {
    const uint32_t n = *d_n;
    if (n < 2) return;
    const unsigned long long idxMask = (1ull << indexBits) - 1ull;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const float4 qmn = leafMn[t], qmx = leafMx[t];
        const uint32_t qi = (uint32_t)(keys[t] & idxMask);
        uint32_t stack[kLbvhStack];
        int sp = 0;
        stack[sp++] = 0u;
        // a tree visits each of its n - 1 internal nodes at most once
        for (uint32_t pops = 0; sp > 0; ++pops) {
            if (pops >= n) {
                atomicOr(&st->err, kErrTreeDepth);
                break;
            }
            const uint32_t node = stack[--sp];
            const uint32_t c[2] = {childL[node], childR[node]};
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (c[k] & kLeafBit) {
                    const uint32_t l = c[k] & ~kLeafBit;
                    if (l > t && boxOverlap(qmn, qmx, leafMn[l], leafMx[l])) {
                        const uint32_t oi = (uint32_t)(keys[l] & idxMask);
                        const uint32_t lo = qi < oi ? qi : oi, hi = qi < oi ? oi : qi;
                        const uint32_t slot = aggregatedAppend(&st->rawPairs);
                        if (slot < cap) pkeys[slot] = ((unsigned long long)lo << bits) | hi;
                    }
                } else if (rangeMax[c[k]] > t && boxOverlap(qmn, qmx, nodeMn[c[k]], nodeMx[c[k]])) {
                    if (sp < kLbvhStack) stack[sp++] = c[k];
                    else atomicOr(&st->err, kErrTreeDepth);
                }
            }
        }
    }
}

void launchLbvh(const BroadInput &in, const LbvhBuffers &lb, PairBuffers &pb, DevStats *st, Scratch &ws,
                cudaStream_t s) {
    uint32_t indexBits = 1;
    while (indexBits < 32 && (1ull << indexBits) < (unsigned long long)(in.maxN > 2 ? in.maxN : 2)) ++indexBits;
    const int g = lbvhGrid(in.maxN);
    k_lbvh_init<<<1, 32, 0, s>>>(lb.box);
    PE_LAUNCHED();
    k_lbvh_bounds<<<g, kLbvhThreads, 0, s>>>(in, lb.box);
    PE_LAUNCHED();
    k_lbvh_codes<<<g, kLbvhThreads, 0, s>>>(in, lb.box, lb.keys, indexBits);
    PE_LAUNCHED();
    // The index bits are already ascending (keys are laid out by index) and the
    // sort is stable, so sorting the 30 code bits orders the whole keys.
    launchRadixSort<unsigned long long>(lb.keys, lb.keysTmp, nullptr, nullptr, in.d_n, in.maxN, (int)indexBits,
                                        (int)indexBits + 30, ws, &st->err, s);
    k_lbvh_build<<<g, kLbvhThreads, 0, s>>>(in, lb.keys, indexBits, lb.childL, lb.childR, lb.parent, lb.leafParent,
                                            lb.rangeMax, lb.visit, lb.leafMn, lb.leafMx);
    PE_LAUNCHED();
    k_lbvh_refit<<<g, kLbvhThreads, 0, s>>>(in.d_n, lb.childL, lb.childR, lb.parent, lb.leafParent, lb.visit,
                                            lb.leafMn, lb.leafMx, lb.nodeMn, lb.nodeMx);
    PE_LAUNCHED();
    k_lbvh_pairs<<<g, kLbvhThreads, 0, s>>>(in.d_n, lb.keys, indexBits, lb.childL, lb.childR, lb.rangeMax, lb.leafMn,
                                            lb.leafMx, lb.nodeMn, lb.nodeMx, pb.keys, pb.cap, pb.bits, st);
    PE_LAUNCHED();
}

} // namespace pe
