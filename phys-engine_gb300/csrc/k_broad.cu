// Broadphase kernels.  Both algorithms emit every AABB-overlapping pair of
// input indices exactly as BroadPhase::findCandidatePairs does
// (src/collision/broadphase.cpp:186-291): inclusive (touching) overlap on all
// three axes, (min, max) index order; the pair list is then put into the
// reference's lexicographic order by a radix sort of 64-bit pair keys
// (first << 32 | second), deduplicated, mapped to collider slots and filtered
// of same-body pairs (src/world/physics_world.cpp:623-633).
#include "pe_block.cuh"
#include "pe_kernels.cuh"
#include "pe_stages.h"

namespace pe {

__device__ __forceinline__ bool overlapYZ(const float4 &f, const float4 &s) {
    // f, s = (min.y, max.y, min.z, max.z); broadphase.cpp:233-236
    return f.x <= s.y && f.y >= s.x && f.z <= s.w && f.w >= s.z;
}
__device__ __forceinline__ bool overlaps(const float4 &amn, const float4 &amx, const float4 &bmn, const float4 &bmx) {
    // Aabb::overlaps (include/phys/collision/aabb.hpp:15-19)
    return amn.x <= bmx.x && amx.x >= bmn.x && amn.y <= bmx.y && amx.y >= bmn.y && amn.z <= bmx.z && amx.z >= bmn.z;
}
// Pair key = (first << bits) | second with first < second, so a plain integer
// sort gives the reference's lexicographic order (broadphase.cpp:18-60).
__device__ __forceinline__ void emitPair(uint32_t a, uint32_t b, unsigned long long *keys, uint32_t cap,
                                         uint32_t *count, uint32_t bits) {
    uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
    uint32_t slot = aggregatedAppend(count);
    if (slot < cap) keys[slot] = ((unsigned long long)lo << bits) | hi;
}

__global__ void k_step_init(DevStats *st, uint32_t inputCount) {
    if (threadIdx.x == 0 && blockIdx.x == 0) initStepStats(st, inputCount);
}

// ---------------------------------------------------------------- SAP ------
// Temporal coherence of the SAP order: the last step's sorted order (sapVals)
// is kept; its keys are refreshed and checked to still be strictly increasing
// in (min.x key, index) — the order the sort defines — in which case the sort
// is skipped (sortCount = 0), else the keys are laid out in index order and
// sorted as usual.  Either way the sorted arrays are the same.
__global__ void k_sap_presort(const uint32_t *d_n, const uint32_t *keyOf, uint32_t *keys, const uint32_t *vals,
                              uint32_t *unsorted) {
    const uint32_t n = *d_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = vals[i];
        bool bad = p >= n;
        if (!bad) {
            const uint32_t k = keyOf[p];
            keys[i] = k;
            if (i + 1 < n) {
                const uint32_t q = vals[i + 1];
                bad = q >= n || !(k < keyOf[q] || (k == keyOf[q] && p < q));
            }
        }
        if (bad) atomicOr(unsorted, 1u);
    }
}

__global__ void k_sap_order(const uint32_t *d_n, const uint32_t *keyOf, uint32_t *keys, uint32_t *vals,
                            const uint32_t *unsorted, uint32_t *sortCount) {
    const uint32_t n = *d_n;
    const bool redo = *unsorted != 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) *sortCount = redo ? n : 0u;
    if (!redo) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = keyOf[i];
        vals[i] = i;
    }
}

__global__ void k_sap_gather(BroadInput in, const uint32_t *sortedVals, float *sMinX, float *sMaxX, float4 *sYZ,
                             uint32_t *sIdx, uint32_t *unsorted) {
    if (unsorted && blockIdx.x == 0 && threadIdx.x == 0) *unsorted = 0u;  // for the next step's check
    const uint32_t n = *in.d_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t idx = sortedVals[i];
        float4 mn = in.mn[idx], mx = in.mx[idx];
        sMinX[i] = mn.x;
        sMaxX[i] = mx.x;
        sYZ[i] = make_float4(mn.y, mx.y, mn.z, mx.z);
        sIdx[i] = idx;
    }
}

// Window of sorted entry i: entries i+1 .. e-1 with min.x <= max.x(i), the
// reference's sweep break (broadphase.cpp:228-231).
__global__ void k_sap_window(const uint32_t *d_n, const float *sMinX, const float *sMaxX, uint32_t *len,
                             DevStats *st) {
    const uint32_t n = *d_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = sMaxX[i];
        uint32_t lo = i + 1, hi = n;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (sMinX[mid] > x) hi = mid;
            else lo = mid + 1;
        }
        uint32_t l = lo - i - 1;
        len[i] = l;
        aggregatedAdd64(&st->xWindow, l);
    }
}

// Load-balanced sweep over the flattened windows: each thread owns kSweepChunk
// consecutive (entry, partner) items.
constexpr uint32_t kSweepChunk = 16;
__global__ void k_sap_emit(const uint32_t *d_n, const uint32_t *off, const uint32_t *len, const float4 *sYZ,
                           const uint32_t *sIdx, unsigned long long *keys, uint32_t cap, uint32_t bits,
                           DevStats *st) {
    const uint32_t n = *d_n;
    const uint32_t W = st->windowWork;
    // The flattened window work is indexed in 32 bits; beyond that the sweep
    // refuses (error flag) instead of walking wrapped offsets.
    if (st->xWindow > 0xFFFFFFFFull) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&st->err, kErrPairCapacity | kErrEntryCapacity);
        return;
    }
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kSweepChunk;
    for (uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kSweepChunk; w0 < W; w0 += stride) {
        // i = last entry with off[i] <= w0 (it has a non-empty window)
        uint32_t lo = 0, hi = n;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (off[mid] > w0) hi = mid;
            else lo = mid + 1;
        }
        uint32_t i = lo - 1;
        uint32_t j = i + 1 + (uint32_t)(w0 - off[i]);
        uint32_t end = i + 1 + len[i];
        float4 f = sYZ[i];
        uint32_t fi = sIdx[i];
        uint64_t wEnd = w0 + kSweepChunk < W ? w0 + kSweepChunk : W;
        for (uint64_t w = w0; w < wEnd; ++w) {
            if (j >= n) {
                atomicOr(&st->err, kErrEntryCapacity);
                break;
            }
            if (overlapYZ(f, sYZ[j])) emitPair(fi, sIdx[j], keys, cap, &st->rawPairs, bits);
            if (++j == end && w + 1 < wEnd) {
                do { ++i; } while (i + 1 < n && len[i] == 0);
                j = i + 1;
                end = i + 1 + len[i];
                f = sYZ[i];
                fi = sIdx[i];
            }
        }
    }
}

// ------------------------------------------------------ SAP, one block ------
// The whole sweep of a small world in one thread block: the (min.x key,
// index) keys sorted in registers (blockRegisterSort), each sorted entry's
// window by binary search, the windows flattened by a block scan and dealt out
// in equal chunks (a floor box's window holds every body: one thread per entry
// would walk it alone).  The sorted order, the windows, the window and pair
// counters and the pair keys are those of the multi-kernel sweep above (one
// launch instead of a dozen; at a thousand boxes the launches, not the work,
// set the sweep's time).
//
// With `finalize` set the block also does what k_pairs_block does for the
// step: the raw pairs stay in shared memory as 32-bit keys (first << bits |
// second, 2 bits <= 32) and are put in order by their first index (counts per
// first index taken during the sweep, a scan, a scatter), then each first
// index's partners by second index (a thread per short list, a warp and a
// bitmap of the second indices per long one: a floor box's list holds every
// body); then mapped to collider slots, filtered of same-body pairs and
// written in order.  The sweep emits each overlapping pair once, so there are
// no duplicates to drop.  More raw pairs than kSapBlockPairs raise
// kErrSmallPath (the step is re-run with the separate finalize).
constexpr uint32_t kSapBlockMax = 4096;
constexpr uint32_t kSapBlockPairs = 8192;
constexpr int kSapBlockThreads = (int)kRegSortThreads;
// Shared memory: two sort buffers of kSapBlockMax u64 keys (the second also
// holds the pair flags of the finalize), y/z bounds, min.x, max.x, entry
// index, window offsets, then kSapBlockPairs u32 pair keys.
constexpr size_t kSapBlockSmem = (size_t)kSapBlockMax * (8 + 8 + 16 + 4 + 4 + 4 + 4) + (size_t)kSapBlockPairs * 4;
static_assert(kSapBlockPairs * 4 <= kSapBlockMax * 8, "pair flags fit one key buffer");

template <int E>
__device__ __forceinline__ void sapSortKeys(const BroadInput &in, uint32_t n, unsigned long long *bufA,
                                            unsigned long long *bufB, uint32_t *sapKeys, uint32_t *sapVals,
                                            float *sMinX, float *sMaxX, float4 *sYZ, uint32_t *sIdx) {
    const uint32_t tid = threadIdx.x;
    unsigned long long v[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const uint32_t i = tid * E + r;
        v[r] = i < n ? ((unsigned long long)orderedFloatKey(in.mn[i].x) << 32 | i) : ~0ull;
    }
    blockRegisterSort<unsigned long long, E>(v, bufA, bufB);
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const uint32_t i = tid * E + r;
        if (i >= n) continue;
        const uint32_t idx = (uint32_t)v[r];
        const float4 mn = in.mn[idx], mx = in.mx[idx];
        sMinX[i] = mn.x;
        sMaxX[i] = mx.x;
        sYZ[i] = make_float4(mn.y, mx.y, mn.z, mx.z);
        sIdx[i] = idx;
        sapKeys[i] = (uint32_t)(v[r] >> 32);
        sapVals[i] = idx;
    }
}

__global__ void __launch_bounds__(kSapBlockThreads)
k_sap_block(BroadInput in, uint32_t *sapKeys, uint32_t *sapVals, uint32_t *unsorted, unsigned long long *keys,
            uint32_t cap, uint32_t bits, DevStats *st, int finalize, const uint32_t *inSlot, const uint32_t *cbody,
            const uint32_t *cbgen, uint32_t *pairA, uint32_t *pairB) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long *bufA = reinterpret_cast<unsigned long long *>(smem);
    unsigned long long *bufB = bufA + kSapBlockMax;
    float4 *sYZ = reinterpret_cast<float4 *>(bufB + kSapBlockMax);
    float *sMinX = reinterpret_cast<float *>(sYZ + kSapBlockMax);
    float *sMaxX = sMinX + kSapBlockMax;
    uint32_t *sIdx = reinterpret_cast<uint32_t *>(sMaxX + kSapBlockMax);
    uint32_t *sOff = sIdx + kSapBlockMax;  // window lengths, then their exclusive scan
    uint32_t *sPairs = sOff + kSapBlockMax;
    __shared__ uint32_t s_count, s_scan[40];
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t n = min(*in.d_n, kSapBlockMax);  // the host launches this for at most kSapBlockMax boxes
    if (tid == 0) {
        s_count = 0;
        if (unsorted) *unsorted = 0u;  // as after the multi-kernel sweep
    }
    if (n <= kRegSortThreads) sapSortKeys<1>(in, n, bufA, bufB, sapKeys, sapVals, sMinX, sMaxX, sYZ, sIdx);
    else if (n <= 2 * kRegSortThreads) sapSortKeys<2>(in, n, bufA, bufB, sapKeys, sapVals, sMinX, sMaxX, sYZ, sIdx);
    else sapSortKeys<4>(in, n, bufA, bufB, sapKeys, sapVals, sMinX, sMaxX, sYZ, sIdx);
    __syncthreads();
    uint32_t *sCnt = reinterpret_cast<uint32_t *>(bufA);  // pairs per first index (finalize), n entries
    if (finalize)
        for (uint32_t i = tid; i < n; i += nt) sCnt[i] = 0u;
    for (uint32_t i = tid; i < n; i += nt) {
        // window: entries i+1 .. lo-1 with min.x <= max.x(i) (k_sap_window)
        const float x = sMaxX[i];
        uint32_t lo = i + 1, hi = n;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (sMinX[mid] > x) hi = mid;
            else lo = mid + 1;
        }
        sOff[i] = lo - i - 1;
    }
    __syncthreads();
    const uint32_t W = blockExclusiveScanArray(sOff, n, s_scan);  // ends with a barrier
    // thread t: flattened items [t C, (t + 1) C) of the windows, in order
    const uint32_t C = (W + nt - 1) / nt;
    const uint32_t w0 = tid * C, wEnd = min(W, w0 + C);
    const uint32_t pairCap = finalize ? kSapBlockPairs : cap;
    if (w0 < wEnd) {
        uint32_t lo = 0, hi = n;  // i = last entry with off[i] <= w0
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (sOff[mid] > w0) hi = mid;
            else lo = mid + 1;
        }
        uint32_t i = lo - 1;
        uint32_t j = i + 1 + (w0 - sOff[i]);
        uint32_t end = i + 1 + ((i + 1 < n ? sOff[i + 1] : W) - sOff[i]);  // i has a non-empty window
        float4 f = sYZ[i];
        uint32_t fi = sIdx[i];
        for (uint32_t w = w0; w < wEnd; ++w) {
            if (overlapYZ(f, sYZ[j])) {
                const uint32_t b = sIdx[j];
                const uint32_t lo2 = fi < b ? fi : b, hi2 = fi < b ? b : fi;
                const uint32_t slot = aggregatedAppend(&s_count);
                if (slot < pairCap) {
                    if (finalize) {
                        sPairs[slot] = lo2 << bits | hi2;
                        atomicAdd(&sCnt[lo2], 1u);
                    } else {
                        keys[slot] = ((unsigned long long)lo2 << bits) | hi2;
                    }
                }
            }
            if (++j == end && w + 1 < wEnd) {
                do {
                    ++i;
                } while (i + 1 < n && (sOff[i + 1] - sOff[i]) == 0);
                j = i + 1;
                end = i + 1 + ((i + 1 < n ? sOff[i + 1] : W) - sOff[i]);
                f = sYZ[i];
                fi = sIdx[i];
            }
        }
    }
    __syncthreads();
    const uint32_t P = s_count;
    if (tid == 0) {
        atomicAdd(&st->xWindow, (unsigned long long)W);
        st->windowWork = W;
        atomicAdd(&st->rawPairs, P);
    }
    if (!finalize) return;
    if (P > kSapBlockPairs) {
        if (tid == 0) atomicOr(&st->err, kErrSmallPath);
        return;
    }
    const uint32_t mask = (1u << bits) - 1u;
    // Pairs in order of their first index: list offsets, then a scatter with
    // the counters as cursors (afterwards sCnt[f] is the end of f's list).
    uint32_t *sSec = reinterpret_cast<uint32_t *>(bufB);      // second indices by list
    uint32_t *sLong = sOff;                                   // first indices with long lists
    uint32_t *sBits = reinterpret_cast<uint32_t *>(sYZ);      // a bitmap of kSapBlockMax bits per warp
    blockExclusiveScanArray(sCnt, n, s_scan);  // ends with a barrier
    if (tid == 0) s_count = 0;                 // now counts the long lists
    for (uint32_t k = tid; k < P; k += nt) {
        const uint32_t key = sPairs[k];
        sSec[atomicAdd(&sCnt[key >> bits], 1u)] = key & mask;
    }
    __syncthreads();
    // Short lists: one thread sorts its list (insertion) and writes the full
    // keys back in order; long ones are queued for a warp.
    constexpr uint32_t kShortList = 32;
    for (uint32_t f = tid; f < n; f += nt) {
        const uint32_t begin = f ? sCnt[f - 1] : 0u, end = sCnt[f];
        if (end - begin > kShortList) {
            sLong[aggregatedAppend(&s_count)] = f;
            continue;
        }
        for (uint32_t x = begin + 1; x < end; ++x) {
            const uint32_t v = sSec[x];
            uint32_t y = x;
            for (; y > begin && sSec[y - 1] > v; --y) sSec[y] = sSec[y - 1];
            sSec[y] = v;
        }
        for (uint32_t x = begin; x < end; ++x) sPairs[x] = f << bits | sSec[x];
    }
    __syncthreads();
    {
        const uint32_t lane = tid & 31, warp = tid >> 5, nLong = s_count;
        constexpr uint32_t kWords = kSapBlockMax / 32, kPerLane = kWords / 32;
        uint32_t *bm = sBits + warp * kWords;
        for (uint32_t q = warp; q < nLong; q += nt / 32) {
            const uint32_t f = sLong[q];
            const uint32_t begin = f ? sCnt[f - 1] : 0u, end = sCnt[f];
#pragma unroll
            for (uint32_t r = 0; r < kPerLane; ++r) bm[lane * kPerLane + r] = 0u;
            __syncwarp();
            for (uint32_t x = begin + lane; x < end; x += 32) atomicOr(&bm[sSec[x] >> 5], 1u << (sSec[x] & 31u));
            __syncwarp();
            // lane l owns words [l kPerLane, (l + 1) kPerLane): its set bits
            // come after those of the lanes before it
            uint32_t words[kPerLane], cnt = 0;
#pragma unroll
            for (uint32_t r = 0; r < kPerLane; ++r) {
                words[r] = bm[lane * kPerLane + r];
                cnt += __popc(words[r]);
            }
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl += t;
            }
            uint32_t out = begin + incl - cnt;
#pragma unroll
            for (uint32_t r = 0; r < kPerLane; ++r)
                for (uint32_t wbits = words[r]; wbits; wbits &= wbits - 1u)
                    sPairs[out++] = f << bits | ((lane * kPerLane + r) * 32u + (uint32_t)(__ffs(wbits) - 1));
            __syncwarp();
        }
    }
    __syncthreads();
    // slot mapping, same-body filter, compaction (k_pairs_block)
    uint32_t *sFlag = reinterpret_cast<uint32_t *>(bufB);
    uint32_t unique = 0;
    for (uint32_t k = tid; k < P; k += nt) {
        const uint32_t key = sPairs[k];
        bool keep = !(k > 0 && sPairs[k - 1] == key);
        if (keep) {
            ++unique;
            uint32_t a = key >> bits, b = key & mask;
            if (inSlot) {
                a = inSlot[a];
                b = inSlot[b];
            }
            if (cbody && cbody[a] == cbody[b] && cbgen[a] == cbgen[b]) keep = false;
        }
        sFlag[k] = keep ? 1u : 0u;
    }
    if (unique) atomicAdd(&st->uniquePairs, unique);
    __syncthreads();
    const uint32_t total = blockExclusiveScanArray(sFlag, P, s_scan);
    for (uint32_t k = tid; k < P; k += nt) {
        const uint32_t next = k + 1 < P ? sFlag[k + 1] : total;
        if (next == sFlag[k]) continue;
        const uint32_t key = sPairs[k];
        uint32_t a = key >> bits, b = key & mask;
        if (inSlot) {
            a = inSlot[a];
            b = inSlot[b];
        }
        pairA[sFlag[k]] = a;
        pairB[sFlag[k]] = b;
    }
    if (tid == 0) st->pairs = total;
}

// --------------------------------------------------------------- grid ------
// Widths for the median cell size (broadphase.cpp:94-110).
__global__ void k_grid_widths(BroadInput in, unsigned long long *keys, uint32_t *count) {
    const uint32_t n = *in.d_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 mn = in.mn[i], mx = in.mx[i];
        double wx = (double)mx.x - (double)mn.x, wy = (double)mx.y - (double)mn.y, wz = (double)mx.z - (double)mn.z;
        double w = wx;
        if (w < wy) w = wy;
        if (w < wz) w = wz;
        bool ok = w > 0.0 && isfinite(w);
        keys[i] = ok ? (unsigned long long)__double_as_longlong(w) : ~0ull;
        if (ok) aggregatedAppend(count);
    }
}

__global__ void k_grid_cellsize(const unsigned long long *sortedWidths, const uint32_t *count, double fixedCell,
                                DevStats *st) {
    double cell = 1.0;
    const uint32_t c = *count, n = st->inputCount;
    if (fixedCell > 0.0) cell = fixedCell;
    else if (c > 0 && c <= n) cell = __longlong_as_double((long long)sortedWidths[c / 2]);
    st->cellSize = cell;
}

// floor((double)x / cell) exactly as the reference computes it
// (broadphase.cpp:66-71).  The float product q = x * invf (invf = 1/cell
// rounded to float) is within 2^-23 (relative) of the exact quotient; when q
// lies farther than 1e-6 (relative) from both neighbouring integers, the exact
// quotient and its double rounding floor to the same integer as q, so the
// double division only runs near cell boundaries and for |q| >= 2^20.
__device__ __forceinline__ double cellFloor(float x, double cell, float invf) {
    const float q = x * invf;
    if (fabsf(q) < 1048576.0f) {
        const float f = floorf(q);
        const float tol = 1e-6f * fmaxf(1.0f, fabsf(q));
        if (q - f > tol && (f + 1.0f) - q > tol) return (double)f;
    }
    return floor((double)x / cell);
}

// gridRange (broadphase.cpp:62-88) per input box.
// fixedCell > 0: the cell size is given (no k_grid_cellsize launch); this
// kernel records it.
__global__ void k_grid_range(BroadInput in, DevStats *st, int4 *firstCell, uint32_t *cellCount, uint8_t *inGrid,
                             uint32_t *overflow, double fixedCell) {
    const uint32_t n = *in.d_n;
    if (fixedCell > 0.0 && blockIdx.x == 0 && threadIdx.x == 0) st->cellSize = fixedCell;
    const double cell = fixedCell > 0.0 ? fixedCell : st->cellSize;
    const float inv = (float)(1.0 / cell);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 mn = in.mn[i], mx = in.mx[i];
        double lower[3] = {cellFloor(mn.x, cell, inv), cellFloor(mn.y, cell, inv), cellFloor(mn.z, cell, inv)};
        double upper[3] = {cellFloor(mx.x, cell, inv), cellFloor(mx.y, cell, inv), cellFloor(mx.z, cell, inv)};
        uint64_t total = 1;
        int32_t first[3];
        int counts[3];
        bool ok = true;
        for (int a = 0; a < 3 && ok; ++a) {
            if (!isfinite(lower[a]) || !isfinite(upper[a]) || lower[a] < -2147483648.0 || upper[a] > 2147483647.0 ||
                lower[a] > upper[a]) {
                ok = false;
                break;
            }
            int64_t c = (int64_t)upper[a] - (int64_t)lower[a] + 1;
            if (c > (int64_t)(64 / total)) {
                ok = false;
                break;
            }
            first[a] = (int32_t)lower[a];
            counts[a] = (int)c;
            total *= (uint64_t)c;
        }
        if (ok) {
            firstCell[i] = make_int4(first[0], first[1], first[2], counts[0] | (counts[1] << 8) | (counts[2] << 16));
            cellCount[i] = (uint32_t)total;
            inGrid[i] = 1;
            namespace cg = cooperative_groups;
            cg::coalesced_group g = cg::coalesced_threads();
            for (int a = 0; a < 3; ++a) {
                int lo = cg::reduce(g, first[a], cg::less<int>());
                int hi = cg::reduce(g, first[a] + counts[a] - 1, cg::greater<int>());
                if (g.thread_rank() == 0) {
                    atomicMin(&st->cellLo[a], lo);
                    atomicMax(&st->cellHi[a], hi);
                }
            }
        } else {
            cellCount[i] = 0;
            inGrid[i] = 0;
            uint32_t k = aggregatedAppend(&st->overflowCount);
            overflow[k] = i;
        }
    }
}

__device__ __forceinline__ uint32_t bitsFor(uint32_t range) { return range ? 32u - __clz(range) : 0u; }

// Cell (x, y, z) as offsets from the lowest cell, packed x | y | z.
__device__ __forceinline__ unsigned long long packCell(int x, int y, int z, const DevStats *st, uint32_t by,
                                                       uint32_t bz) {
    const unsigned long long dx = (uint32_t)(x - st->cellLo[0]);
    const unsigned long long dy = (uint32_t)(y - st->cellLo[1]);
    const unsigned long long dz = (uint32_t)(z - st->cellLo[2]);
    return (dx << (by + bz)) | (dy << bz) | dz;
}

// One entry per covered cell; key = packed cell offsets from the lowest cell,
// so equal cells are adjacent after the sort (cell order is irrelevant: the
// reference only groups entries by cell before the final pair sort).
__global__ void k_grid_entries(BroadInput in, const int4 *firstCell, const uint8_t *inGrid, const uint32_t *entryOff,
                               unsigned long long *keys, uint32_t *vals, uint32_t cap, uint32_t sortBits,
                               DevStats *st) {
    const uint32_t n = *in.d_n;
    // No box in the grid: the bounds keep their sentinels and there is nothing to write.
    if (st->cellLo[0] > st->cellHi[0]) return;
    const uint32_t bx = bitsFor((uint32_t)(st->cellHi[0] - st->cellLo[0]));
    const uint32_t by = bitsFor((uint32_t)(st->cellHi[1] - st->cellLo[1]));
    const uint32_t bz = bitsFor((uint32_t)(st->cellHi[2] - st->cellLo[2]));
    if (blockIdx.x == 0 && threadIdx.x == 0) st->cellKeyBits = bx + by + bz;
    if (bx + by + bz > sortBits) {
        // Wider than this launch sorts: the host re-runs the step with the width recorded above.
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&st->err, bx + by + bz > 64 ? kErrEntryCapacity : kErrSmallPath);
        return;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!inGrid[i]) continue;
        int4 f = firstCell[i];
        int cx = f.w & 0xFF, cy = (f.w >> 8) & 0xFF, cz = (f.w >> 16) & 0xFF;
        uint32_t e = entryOff[i];
        for (int x = 0; x < cx; ++x)
            for (int y = 0; y < cy; ++y)
                for (int z = 0; z < cz; ++z, ++e) {
                    if (e >= cap) continue;
                    keys[e] = packCell(f.x + x, f.y + y, f.z + z, st, by, bz);
                    vals[e] = i;
                }
    }
}

// Per-cell all pairs (broadphase.cpp:152-160): entry e against every later
// entry of its cell.
// An overlapping pair is emitted only from the lowest cell both boxes cover, so
// the list is already free of the duplicates the reference removes with
// sort + unique (broadphase.cpp:169-172); every check is still counted.
__global__ void k_grid_cell_pairs(const uint32_t *d_entries, uint32_t ecap, const unsigned long long *ekeys,
                                  const uint32_t *evals, const int4 *firstCell, BroadInput in,
                                  unsigned long long *pkeys, uint32_t cap, uint32_t bits, DevStats *st) {
    // Entries were not written this attempt (key width refused): nothing to scan.
    if (st->err & (kErrSmallPath | kErrEntryCapacity)) return;
    const uint32_t E = min(*d_entries, ecap);
    const uint32_t by = bitsFor((uint32_t)(st->cellHi[1] - st->cellLo[1]));
    const uint32_t bz = bitsFor((uint32_t)(st->cellHi[2] - st->cellLo[2]));
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        const unsigned long long key = ekeys[e];
        const uint32_t a = evals[e];
        const float4 amn = in.mn[a], amx = in.mx[a];
        const int4 fa = firstCell[a];
        uint64_t cmp = 0;
        for (uint32_t f = e + 1; f < E && ekeys[f] == key; ++f) {
            ++cmp;
            const uint32_t b = evals[f];
            if (!overlaps(amn, amx, in.mn[b], in.mx[b])) continue;
            const int4 fb = firstCell[b];
            const unsigned long long low = packCell(max(fa.x, fb.x), max(fa.y, fb.y), max(fa.z, fb.z), st, by, bz);
            if (low == key) emitPair(a, b, pkeys, cap, &st->rawPairs, bits);
        }
        aggregatedAdd64(&st->gridComparisons, cmp);
    }
}

// Overflow boxes against all others (broadphase.cpp:162-166).
__global__ void k_grid_overflow_pairs(BroadInput in, const uint32_t *overflow, const uint8_t *inGrid,
                                      unsigned long long *pkeys, uint32_t cap, uint32_t bits, DevStats *st) {
    const uint32_t n = *in.d_n;
    const uint32_t F = st->overflowCount;
    const uint64_t total = (uint64_t)F * n;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = (uint32_t)(t / n), s = (uint32_t)(t % n);
        const uint32_t f = overflow[k];
        if (f == s || !(inGrid[s] || f < s)) continue;
        aggregatedAdd64(&st->gridComparisons, 1ull);
        if (overlaps(in.mn[f], in.mx[f], in.mn[s], in.mx[s])) emitPair(f, s, pkeys, cap, &st->rawPairs, bits);
    }
}

// Per-body pair emission (grid): body a gathers its partners b > a from the
// cells it covers (its own entry in each cell is found by a binary search on
// (cell, index); the later entries of the cell are exactly the partners with a
// higher index), keeps a pair in its lowest shared cell only, adds overflow
// partners, sorts its few partners and writes them in body order (block scan +
// decoupled look-back).  The result equals the reference's sorted, unique pair
// list (broadphase.cpp:144-172) after the slot mapping and same-body filter
// (physics_world.cpp:623-633), so no pair sort or finalize is needed.  The
// comparison counter gets the per-cell comparisons (sum of n(n-1)/2 over cells)
// and the overflow comparisons, as the reference counts them.
constexpr uint32_t kBodyPartners = 32;
constexpr int kBodyPairThreads = 256;

__global__ void __launch_bounds__(kBodyPairThreads)
k_grid_body_pairs(BroadInput in, const int4 *firstCell, const uint8_t *inGrid, const uint32_t *overflow,
                  const uint32_t *d_entries, uint32_t ecap, const unsigned long long *ekeys, const uint32_t *evals,
                  const uint32_t *inSlot, const uint32_t *cbody, const uint32_t *cbgen, uint32_t *pairA,
                  uint32_t *pairB, uint32_t cap, DevStats *st, unsigned long long *state, uint32_t *counter) {
    __shared__ uint32_t s_tile, s_scan[9], s_prefix, s_abort;
    // Entries were not written this attempt (key width refused): nothing to scan.
    if (st->err & (kErrSmallPath | kErrEntryCapacity)) return;
    const uint32_t n = *in.d_n;
    const uint32_t E = min(*d_entries, ecap);
    const uint32_t F = st->overflowCount;
    const uint32_t by = bitsFor((uint32_t)(st->cellHi[1] - st->cellLo[1]));
    const uint32_t bz = bitsFor((uint32_t)(st->cellHi[2] - st->cellLo[2]));
    if (blockIdx.x == 0 && threadIdx.x == 0 && F)
        atomicAdd(&st->gridComparisons, (unsigned long long)F * (n - F) + (unsigned long long)F * (F - 1) / 2);
    const uint32_t ntiles = max((n + kBodyPairThreads - 1) / kBodyPairThreads, 1u);
    for (;;) {
        const uint32_t tile = takeTile(counter, &s_tile);
        if (tile >= ntiles) return;
        const uint32_t a = tile * kBodyPairThreads + threadIdx.x;
        uint32_t part[kBodyPartners];
        uint32_t cnt = 0;
        uint32_t cmp = 0;
        if (a < n) {
            const float4 amn = in.mn[a], amx = in.mx[a];
            auto add = [&](uint32_t b) {
                if (cnt < kBodyPartners) part[cnt] = b;
                ++cnt;
            };
            if (inGrid[a]) {
                const int4 fa = firstCell[a];
                const int cx = fa.w & 0xFF, cy = (fa.w >> 8) & 0xFF, cz = (fa.w >> 16) & 0xFF;
                for (int x = 0; x < cx; ++x)
                    for (int y = 0; y < cy; ++y)
                        for (int z = 0; z < cz; ++z) {
                            const unsigned long long key = packCell(fa.x + x, fa.y + y, fa.z + z, st, by, bz);
                            uint32_t lo = 0, hi = E;
                            while (lo < hi) {
                                const uint32_t mid = (lo + hi) >> 1;
                                const unsigned long long k2 = ekeys[mid];
                                if (k2 < key || (k2 == key && evals[mid] < a)) lo = mid + 1;
                                else hi = mid;
                            }
                            for (uint32_t f = lo + 1; f < E && ekeys[f] == key; ++f) {
                                ++cmp;
                                const uint32_t b = evals[f];
                                if (!overlaps(amn, amx, in.mn[b], in.mx[b])) continue;
                                const int4 fb = firstCell[b];
                                if (packCell(max(fa.x, fb.x), max(fa.y, fb.y), max(fa.z, fb.z), st, by, bz) != key)
                                    continue;
                                add(b);
                            }
                        }
                for (uint32_t k = 0; k < F; ++k) {
                    const uint32_t o = overflow[k];
                    if (o > a && overlaps(amn, amx, in.mn[o], in.mx[o])) add(o);
                }
            } else {
                for (uint32_t b = a + 1; b < n; ++b)
                    if (overlaps(amn, amx, in.mn[b], in.mx[b])) add(b);
            }
            if (cnt > kBodyPartners) atomicOr(&st->err, kErrBodyPairs);
            const uint32_t m = min(cnt, kBodyPartners);
            for (uint32_t i = 1; i < m; ++i) {
                const uint32_t v = part[i];
                uint32_t j = i;
                while (j > 0 && part[j - 1] > v) {
                    part[j] = part[j - 1];
                    --j;
                }
                part[j] = v;
            }
        }
        const uint32_t m = min(cnt, kBodyPartners);
        const uint32_t sa = a < n ? (inSlot ? inSlot[a] : a) : 0u;
        uint32_t kept = 0;
        for (uint32_t j = 0; j < m; ++j) {
            const uint32_t sb = inSlot ? inSlot[part[j]] : part[j];
            if (cbody && cbody[sa] == cbody[sb] && cbgen[sa] == cbgen[sb]) continue;
            ++kept;
        }
        {
            // one atomic per warp and counter
            const uint32_t wc = __reduce_add_sync(0xffffffffu, cnt);
            const uint32_t wm = __reduce_add_sync(0xffffffffu, cmp);
            if ((threadIdx.x & 31) == 0) {
                if (wc) {
                    atomicAdd(&st->rawPairs, wc);  // no duplicates: raw = unique
                    atomicAdd(&st->uniquePairs, wc);
                }
                if (wm) atomicAdd(&st->gridComparisons, (unsigned long long)wm);
            }
        }
        uint32_t total;
        const uint32_t local = blockExclusiveScan(kept, total, s_scan);
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
        uint32_t o = s_prefix + local;
        for (uint32_t j = 0; j < m; ++j) {
            const uint32_t sb = inSlot ? inSlot[part[j]] : part[j];
            if (cbody && cbody[sa] == cbody[sb] && cbgen[sa] == cbgen[sb]) continue;
            if (o < cap) {
                pairA[o] = sa;
                pairB[o] = sb;
            }
            ++o;
        }
        if (threadIdx.x == 0 && tile + 1 == ntiles) st->pairs = s_prefix + total;
        __syncthreads();
    }
}

// ------------------------------------------------------------ hashed grid --
// With a fixed cell size the grid needs no global cell range: a cell is keyed
// by its exact coordinates (21 bits each) and entries are grouped by a hash of
// the key (counting pass, scan, fill).  Each body then gathers its partners
// from the buckets of its cells, keeping the entries with its exact cell key,
// as the sorted grid does.  Cells, overflow boxes, pairs, their order and the
// comparison / entry / overflow counters are those of the reference's grid
// (broadphase.cpp:62-182).
__device__ __forceinline__ bool cellKey21(int x, int y, int z, unsigned long long &key) {
    const int lim = 1 << 20;
    if (x < -lim || x >= lim || y < -lim || y >= lim || z < -lim || z >= lim) return false;
    key = ((unsigned long long)(x + lim) << 42) | ((unsigned long long)(y + lim) << 21) | (unsigned long long)(z + lim);
    return true;
}
__device__ __forceinline__ uint32_t bucketOf(unsigned long long key, uint32_t logB) {
    return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - logB));
}

constexpr uint32_t kNoEntry = 0xFFFFFFFFu;

// Cell range per box (as k_grid_range) and one entry per covered cell, pushed
// onto its bucket's list: entry e holds (cell key, body) and the bucket's
// previous head.  Entry slots come from one counter (a warp scan of the boxes'
// cell counts, one atomic per warp), so entry order varies from run to run;
// nothing downstream depends on it (each body sorts its partners).
__device__ __forceinline__ bool cellFloorFast(float x, float invf, int &cellOut) {
    const float q = x * invf;
    if (!(fabsf(q) < 1048576.0f)) return false;
    const float f = floorf(q);
    const float tol = 1e-6f * fmaxf(1.0f, fabsf(q));
    if (!(q - f > tol && (f + 1.0f) - q > tol)) return false;
    cellOut = (int)f;
    return true;
}

__global__ void __launch_bounds__(256)
k_hgrid_insert(BroadInput in, DevStats *st, int4 *firstCell, uint8_t *inGrid, uint32_t *overflow, double cell,
               float inv, uint32_t *bucketHead, uint32_t logB, uint4 *entryRec, float4 *cand, uint32_t ecap,
               unsigned long long *zeroState, uint32_t nZeroState) {
    __shared__ uint32_t s_scan[9], s_base;
    const uint32_t n = *in.d_n;
    // look-back states of the kernels that follow (cleared here, not by memsets)
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nZeroState; j += gridDim.x * blockDim.x)
        zeroState[j] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->cellSize = cell;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        uint32_t total = 0;
        int32_t first[3] = {0, 0, 0};
        int counts[3] = {0, 0, 0};
        if (i < n) {
            const float4 mn = in.mn[i], mx = in.mx[i];
            int lo[3], hi[3];
            bool ok = cellFloorFast(mn.x, inv, lo[0]) && cellFloorFast(mn.y, inv, lo[1]) &&
                      cellFloorFast(mn.z, inv, lo[2]) && cellFloorFast(mx.x, inv, hi[0]) &&
                      cellFloorFast(mx.y, inv, hi[1]) && cellFloorFast(mx.z, inv, hi[2]);
            uint32_t cells = 1;
            if (ok) {
                // all six floors exact from the float products (|cell| < 2^20)
                for (int a2 = 0; a2 < 3 && ok; ++a2) {
                    const int c = hi[a2] - lo[a2] + 1;
                    if (lo[a2] > hi[a2] || c > (int)(64 / cells)) {
                        ok = false;
                        break;
                    }
                    first[a2] = lo[a2];
                    counts[a2] = c;
                    cells *= (uint32_t)c;
                }
            } else {
                // gridRange in double (broadphase.cpp:62-88)
                const double lower[3] = {cellFloor(mn.x, cell, inv), cellFloor(mn.y, cell, inv),
                                         cellFloor(mn.z, cell, inv)};
                const double upper[3] = {cellFloor(mx.x, cell, inv), cellFloor(mx.y, cell, inv),
                                         cellFloor(mx.z, cell, inv)};
                ok = true;
                for (int a2 = 0; a2 < 3 && ok; ++a2) {
                    if (!isfinite(lower[a2]) || !isfinite(upper[a2]) || lower[a2] < -2147483648.0 ||
                        upper[a2] > 2147483647.0 || lower[a2] > upper[a2]) {
                        ok = false;
                        break;
                    }
                    const int64_t c = (int64_t)upper[a2] - (int64_t)lower[a2] + 1;
                    if (c > (int64_t)(64 / cells)) {
                        ok = false;
                        break;
                    }
                    first[a2] = (int32_t)lower[a2];
                    counts[a2] = (int)c;
                    cells *= (uint32_t)c;
                }
            }
            unsigned long long k0, k1;
            if (!ok) {
                inGrid[i] = 0;
                overflow[aggregatedAppend(&st->overflowCount)] = i;
            } else if (!cellKey21(first[0], first[1], first[2], k0) ||
                       !cellKey21(first[0] + counts[0] - 1, first[1] + counts[1] - 1, first[2] + counts[2] - 1, k1)) {
                atomicOr(&st->err, kErrHashRange);
                inGrid[i] = 0;
            } else {
                firstCell[i] = make_int4(first[0], first[1], first[2], counts[0] | (counts[1] << 8) | (counts[2] << 16));
                inGrid[i] = 1;
                total = cells;
                cand[2 * i] = make_float4(mn.x, mn.y, mn.z, __uint_as_float((uint32_t)k0));
                cand[2 * i + 1] = make_float4(mx.x, mx.y, mx.z, __uint_as_float((uint32_t)(k0 >> 32)));
            }
        }
        // entry slots: block scan of the cell counts, one atomic per block
        uint32_t blockTotal;
        const uint32_t local = blockExclusiveScan(total, blockTotal, s_scan);
        if (threadIdx.x == 0) s_base = blockTotal ? atomicAdd(&st->gridEntryCount, blockTotal) : 0u;
        __syncthreads();
        uint32_t e = s_base + local;
        __syncthreads();
        for (int x = 0; x < counts[0] && total; ++x)
            for (int y = 0; y < counts[1]; ++y)
                for (int z = 0; z < counts[2]; ++z, ++e) {
                    if (e >= ecap) continue;  // the host re-runs the step with more entry slots
                    unsigned long long key;
                    cellKey21(first[0] + x, first[1] + y, first[2] + z, key);
                    const uint32_t nx = atomicExch(&bucketHead[bucketOf(key, logB)], e);
                    entryRec[e] = make_uint4((uint32_t)key, (uint32_t)(key >> 32), i, nx);
                }
    }
}

// Per-body pairs from the buckets (the counterpart of k_grid_body_pairs).
__global__ void __launch_bounds__(kBodyPairThreads)
k_hgrid_pairs(BroadInput in, const int4 *firstCell, const uint8_t *inGrid, const uint32_t *overflow,
              const uint32_t *bucketHead, uint32_t logB, uint32_t ecap, const uint4 *__restrict__ entryRec,
              const float4 *__restrict__ cand, const uint32_t *inSlot, const uint32_t *cbody, const uint32_t *cbgen,
              uint32_t *pairA, uint32_t *pairB, uint32_t cap, DevStats *st, unsigned long long *state,
              uint32_t *counter) {
    __shared__ uint32_t s_tile, s_scan[9], s_prefix, s_abort;
    // Out-of-range cells or too few entry slots: the host re-runs the step.
    if ((st->err & kErrHashRange) || st->gridEntryCount > ecap) return;
    const uint32_t n = *in.d_n;
    const uint32_t F = st->overflowCount;
    if (blockIdx.x == 0 && threadIdx.x == 0 && F)
        atomicAdd(&st->gridComparisons, (unsigned long long)F * (n - F) + (unsigned long long)F * (F - 1) / 2);
    const uint32_t ntiles = max((n + kBodyPairThreads - 1) / kBodyPairThreads, 1u);
    for (;;) {
        const uint32_t tile = takeTile(counter, &s_tile);
        if (tile >= ntiles) return;
        const uint32_t a = tile * kBodyPairThreads + threadIdx.x;
        uint32_t part[kBodyPartners];
        uint32_t cnt = 0;
        uint32_t cmp = 0;
        if (a < n) {
            const float4 amn = in.mn[a], amx = in.mx[a];
            auto add = [&](uint32_t b) {
                if (cnt < kBodyPartners) part[cnt] = b;
                ++cnt;
            };
            // The body's cell range is read with its box (unused off the grid).
            const int4 fa = firstCell[a];
            if (inGrid[a]) {
                const int cx = fa.w & 0xFF, cy = (fa.w >> 8) & 0xFF, cz = (fa.w >> 16) & 0xFF;
                const int cells = cx * cy * cz;
                unsigned long long faKey;
                cellKey21(fa.x, fa.y, fa.z, faKey);
                // The list heads of four cells are requested together; then each
                // list node's key, body and link in one round trip, and a
                // candidate's box and cell range in one more.  Partners are
                // sorted afterwards, so the visit order does not matter.  A
                // list holds at most ecap nodes.
                int x = 0, y = 0, z = 0;  // next cell, z fastest
                for (int c0 = 0; c0 < cells; c0 += 4) {
                    unsigned long long key[4];
                    uint32_t head[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        key[j] = 0;
                        head[j] = kNoEntry;
                        if (c0 + j < cells) {
                            cellKey21(fa.x + x, fa.y + y, fa.z + z, key[j]);
                            head[j] = bucketHead[bucketOf(key[j], logB)];
                            if (++z == cz) {
                                z = 0;
                                if (++y == cy) {
                                    y = 0;
                                    ++x;
                                }
                            }
                        }
                    }
                    // the four lists are walked side by side: one round trip
                    // (one 16-byte record per list) per hop for all of them
                    uint32_t e[4] = {head[0], head[1], head[2], head[3]};
                    for (uint32_t hops = 0; hops < ecap; ++hops) {
                        unsigned long long k2[4];
                        uint32_t bv[4];
                        bool live = false;
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            k2[j] = 0;
                            bv[j] = 0;
                            if (e[j] < ecap) {
                                const uint4 r = entryRec[e[j]];
                                k2[j] = ((unsigned long long)r.y << 32) | r.x;
                                bv[j] = r.z;
                                e[j] = r.w;
                                live = true;
                            } else {
                                k2[j] = ~key[j];  // no match
                            }
                        }
                        if (!live) break;
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const uint32_t b = bv[j];
                            if (k2[j] != key[j] || b <= a || b >= n) continue;
                            ++cmp;
                            // the candidate's box and first cell: one sector
                            const float4 c0 = cand[2 * b], c1 = cand[2 * b + 1];
                            if (!overlaps(amn, amx, c0, c1)) continue;
                            const unsigned long long fbKey =
                                ((unsigned long long)__float_as_uint(c1.w) << 32) | __float_as_uint(c0.w);
                            // the lowest cell both boxes cover: per-axis maxima
                            // of the biased 21-bit coordinate fields
                            const unsigned long long fx = max(faKey >> 42, fbKey >> 42);
                            const unsigned long long fy = max((faKey >> 21) & 0x1FFFFFull, (fbKey >> 21) & 0x1FFFFFull);
                            const unsigned long long fz = max(faKey & 0x1FFFFFull, fbKey & 0x1FFFFFull);
                            if (((fx << 42) | (fy << 21) | fz) == key[j]) add(b);
                        }
                    }
                }
                for (uint32_t k = 0; k < F; ++k) {
                    const uint32_t o = overflow[k];
                    if (o > a && overlaps(amn, amx, in.mn[o], in.mx[o])) add(o);
                }
            } else {
                for (uint32_t b = a + 1; b < n; ++b)
                    if (overlaps(amn, amx, in.mn[b], in.mx[b])) add(b);
            }
            if (cnt > kBodyPartners) atomicOr(&st->err, kErrBodyPairs);
            const uint32_t m = min(cnt, kBodyPartners);
            for (uint32_t i = 1; i < m; ++i) {
                const uint32_t v = part[i];
                uint32_t j = i;
                while (j > 0 && part[j - 1] > v) {
                    part[j] = part[j - 1];
                    --j;
                }
                part[j] = v;
            }
        }
        const uint32_t m = min(cnt, kBodyPartners);
        const uint32_t sa = a < n ? (inSlot ? inSlot[a] : a) : 0u;
        // partners to collider slots, same-body pairs dropped (once; part[]
        // then holds the kept slots)
        uint32_t kept = 0;
        if (m) {
            const uint32_t ba = cbody ? cbody[sa] : 0u, ga = cbody ? cbgen[sa] : 0u;
            for (uint32_t j = 0; j < m; ++j) {
                const uint32_t sb = inSlot ? inSlot[part[j]] : part[j];
                if (cbody && ba == cbody[sb] && ga == cbgen[sb]) continue;
                part[kept++] = sb;
            }
        }
        {
            // one atomic per warp and counter
            const uint32_t wc = __reduce_add_sync(0xffffffffu, cnt);
            const uint32_t wm = __reduce_add_sync(0xffffffffu, cmp);
            if ((threadIdx.x & 31) == 0) {
                if (wc) {
                    atomicAdd(&st->rawPairs, wc);  // no duplicates: raw = unique
                    atomicAdd(&st->uniquePairs, wc);
                }
                if (wm) atomicAdd(&st->gridComparisons, (unsigned long long)wm);
            }
        }
        uint32_t total;
        const uint32_t local = blockExclusiveScan(kept, total, s_scan);
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
        uint32_t o = s_prefix + local;
        for (uint32_t j = 0; j < kept; ++j, ++o) {
            if (o < cap) {
                pairA[o] = sa;
                pairB[o] = part[j];
            }
        }
        if (threadIdx.x == 0 && tile + 1 == ntiles) st->pairs = s_prefix + total;
        __syncthreads();
    }
}

void launchGridBodyPairs(const BroadInput &in, const BroadBuffers &bb, PairBuffers &pb, const uint32_t *inSlot,
                         const uint32_t *cbody, const uint32_t *cbgen, DevStats *st, Scratch &ws, cudaStream_t s,
                         bool stateCleared) {
    uint32_t tiles = (in.maxN + kBodyPairThreads - 1) / kBodyPairThreads;
    if (tiles == 0) tiles = 1;
    if (!stateCleared) PE_CHECK(cudaMemsetAsync(ws.scanState, 0, sizeof(unsigned long long) * (tiles + 1), s));
    const uint32_t maxGrid = 8u * (uint32_t)smCount();
    const uint32_t grid = tiles < maxGrid ? tiles : maxGrid;
    if (bb.hashed) {
        k_hgrid_pairs<<<grid, kBodyPairThreads, 0, s>>>(in, bb.firstCell, bb.inGrid, bb.overflow, bb.bucketHead,
                                                         bb.logBuckets, bb.entryCap, bb.entryRec, bb.cand, inSlot,
                                                         cbody, cbgen, pb.a, pb.b, pb.cap, st, ws.scanState,
                                                         (uint32_t *)(ws.scanState + tiles));
        PE_LAUNCHED();
        return;
    }
    k_grid_body_pairs<<<grid, kBodyPairThreads, 0, s>>>(in, bb.firstCell, bb.inGrid, bb.overflow,
                                                         &st->gridEntryCount, bb.entryCap, bb.entryKeys,
                                                         bb.entryVals, inSlot, cbody, cbgen, pb.a, pb.b, pb.cap, st,
                                                         ws.scanState, (uint32_t *)(ws.scanState + tiles));
    PE_LAUNCHED();
}

// ------------------------------------------------------------ finalize -----
__global__ void k_pairs_flags(const uint32_t *d_raw, uint32_t cap, uint32_t bits, const unsigned long long *keys,
                              const uint32_t *inSlot, const uint32_t *cbody, const uint32_t *cbgen, uint32_t *flags,
                              DevStats *st) {
    const uint32_t n = min(*d_raw, cap);
    const unsigned long long mask = (1ull << bits) - 1ull;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        unsigned long long key = keys[k];
        bool keep = !(k > 0 && keys[k - 1] == key);
        if (keep) {
            aggregatedAppend(&st->uniquePairs);
            uint32_t a = (uint32_t)(key >> bits), b = (uint32_t)(key & mask);
            if (inSlot) {
                a = inSlot[a];
                b = inSlot[b];
            }
            if (cbody && cbody[a] == cbody[b] && cbgen[a] == cbgen[b]) keep = false;
        }
        flags[k] = keep ? 1u : 0u;
    }
}

__global__ void k_pairs_scatter(const uint32_t *d_raw, uint32_t cap, uint32_t bits, const unsigned long long *keys,
                                const uint32_t *inSlot, const uint32_t *flags, const uint32_t *pos, uint32_t *pairA,
                                uint32_t *pairB) {
    const uint32_t n = min(*d_raw, cap);
    const unsigned long long mask = (1ull << bits) - 1ull;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        if (!flags[k]) continue;
        unsigned long long key = keys[k];
        uint32_t a = (uint32_t)(key >> bits), b = (uint32_t)(key & mask);
        if (inSlot) {
            a = inSlot[a];
            b = inSlot[b];
        }
        pairA[pos[k]] = a;
        pairB[pos[k]] = b;
    }
}

static inline int gridFor(uint32_t n, int threads = 256, int maxBlocks = 0) {
    if (maxBlocks <= 0) maxBlocks = 8 * smCount();
    uint32_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b < (uint32_t)maxBlocks ? b : (uint32_t)maxBlocks);
}

void launchStepInit(DevStats *st, uint32_t inputCount, cudaStream_t s) {
    k_step_init<<<1, 32, 0, s>>>(st, inputCount);
    PE_LAUNCHED();
}

__global__ void k_set_manifolds(DevStats *st, uint32_t count) { st->manifolds = count; }
void launchSetManifoldCount(DevStats *st, uint32_t count, cudaStream_t s) {
    k_set_manifolds<<<1, 1, 0, s>>>(st, count);
    PE_LAUNCHED();
}

__global__ void k_sap_keys(BroadInput in, uint32_t *keys, uint32_t *vals) {
    const uint32_t n = *in.d_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = orderedFloatKey(in.mn[i].x);
        vals[i] = i;
    }
}

void launchSapKeys(const BroadInput &in, uint32_t *keys, uint32_t *vals, cudaStream_t s) {
    k_sap_keys<<<gridFor(in.maxN), 256, 0, s>>>(in, keys, vals);
    PE_LAUNCHED();
}

bool sapFinalizesPairs(const BroadInput &in, const PairBuffers &pb) {
    return in.maxN <= kSapBlockMax && pb.blockPath && 2 * pb.bits <= 32;
}

bool launchSap(const BroadInput &in, uint32_t *sapKeys, uint32_t *sapVals, BroadBuffers &bb, PairBuffers &pb,
               DevStats *st, Scratch &ws, cudaStream_t s, const SapCoherence *coh, const PairMapping *finalize) {
    uint32_t *err = &st->err;
    if (in.maxN <= kSapBlockMax) {
        static bool configured = false;
        if (!configured) {
            PE_CHECK(cudaFuncSetAttribute(k_sap_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kSapBlockSmem));
            configured = true;
        }
        const bool fin = finalize && sapFinalizesPairs(in, pb);
        k_sap_block<<<1, kSapBlockThreads, kSapBlockSmem, s>>>(
            in, sapKeys, sapVals, coh ? coh->unsorted : nullptr, pb.keys, pb.cap, pb.bits, st, fin ? 1 : 0,
            fin ? finalize->inSlot : nullptr, fin ? finalize->cbody : nullptr, fin ? finalize->cbgen : nullptr, pb.a,
            pb.b);
        PE_LAUNCHED();
        return fin;
    }
    const uint32_t *sortN = in.d_n;
    if (coh) {
        k_sap_presort<<<gridFor(in.maxN), 256, 0, s>>>(in.d_n, coh->keyOf, sapKeys, sapVals, coh->unsorted);
        PE_LAUNCHED();
        k_sap_order<<<gridFor(in.maxN), 256, 0, s>>>(in.d_n, coh->keyOf, sapKeys, sapVals, coh->unsorted,
                                                     coh->sortCount);
        PE_LAUNCHED();
        sortN = coh->sortCount;
    }
    launchRadixSort<uint32_t>(sapKeys, bb.keyTmp32, sapVals, bb.valTmp, sortN, in.maxN, 0, 32, ws, err, s);
    k_sap_gather<<<gridFor(in.maxN), 256, 0, s>>>(in, sapVals, bb.sMinX, bb.sMaxX, bb.sYZ, bb.sIdx,
                                                  coh ? coh->unsorted : nullptr);
    PE_LAUNCHED();
    k_sap_window<<<gridFor(in.maxN), 256, 0, s>>>(in.d_n, bb.sMinX, bb.sMaxX, bb.len, st);
    PE_LAUNCHED();
    launchScanExclusive(bb.len, bb.off, in.d_n, in.maxN, &st->windowWork, ws, err, s);
    k_sap_emit<<<8 * smCount(), 256, 0, s>>>(in.d_n, bb.off, bb.len, bb.sYZ, bb.sIdx, pb.keys, pb.cap, pb.bits, st);
    PE_LAUNCHED();
    return false;
}

void launchGrid(const BroadInput &in, double fixedCell, BroadBuffers &bb, PairBuffers &pb, DevStats *st, Scratch &ws,
                cudaStream_t s) {
    uint32_t *err = &st->err;
    if (bb.hashed) {
        // fixed cell size: bucket lists of the covered cells (pairs: launchGridBodyPairs)
        const uint32_t B = 1u << bb.logBuckets;
        if (!bb.headsCleared) PE_CHECK(cudaMemsetAsync(bb.bucketHead, 0xFF, B * sizeof(uint32_t), s));
        k_hgrid_insert<<<gridFor(in.maxN), 256, 0, s>>>(in, st, bb.firstCell, bb.inGrid, bb.overflow, fixedCell,
                                                        (float)(1.0 / fixedCell), bb.bucketHead, bb.logBuckets,
                                                        bb.entryRec, bb.cand, bb.entryCap, bb.zeroState,
                                                        bb.nZeroState);
        PE_LAUNCHED();
        return;
    }
    // counters[0] counts the non-zero widths of this call.
    PE_CHECK(cudaMemsetAsync(bb.counters, 0, 4 * sizeof(uint32_t), s));
    if (fixedCell <= 0.0) {
        k_grid_widths<<<gridFor(in.maxN), 256, 0, s>>>(in, bb.widthKeys, &bb.counters[0]);
        PE_LAUNCHED();
        launchRadixSort<unsigned long long>(bb.widthKeys, bb.widthTmp, nullptr, nullptr, in.d_n, in.maxN, 0, 64, ws,
                                            err, s);
    }
    if (fixedCell <= 0.0) {
        k_grid_cellsize<<<1, 1, 0, s>>>(bb.widthKeys, &bb.counters[0], fixedCell, st);
        PE_LAUNCHED();
    }
    k_grid_range<<<gridFor(in.maxN), 256, 0, s>>>(in, st, bb.firstCell, bb.cellCount, bb.inGrid, bb.overflow,
                                                  fixedCell);
    PE_LAUNCHED();
    launchScanExclusive(bb.cellCount, bb.entryOff, in.d_n, in.maxN, &st->gridEntryCount, ws, err, s);
    k_grid_entries<<<gridFor(in.maxN), 256, 0, s>>>(in, bb.firstCell, bb.inGrid, bb.entryOff, bb.entryKeys,
                                                    bb.entryVals, bb.entryCap, bb.keyBits, st);
    PE_LAUNCHED();
    launchRadixSort<unsigned long long>(bb.entryKeys, bb.entryKeysTmp, bb.entryVals, bb.entryValsTmp,
                                        &st->gridEntryCount, bb.entryCap, 0, (int)bb.keyBits, ws, err, s);
    if (pb.bodyPath) return;  // pairs come from launchGridBodyPairs
    k_grid_cell_pairs<<<gridFor(bb.entryCap), 256, 0, s>>>(&st->gridEntryCount, bb.entryCap, bb.entryKeys,
                                                           bb.entryVals, bb.firstCell, in, pb.keys, pb.cap, pb.bits,
                                                           st);
    PE_LAUNCHED();
    k_grid_overflow_pairs<<<4 * smCount(), 256, 0, s>>>(in, bb.overflow, bb.inGrid, pb.keys, pb.cap, pb.bits, st);
    PE_LAUNCHED();
}

// The n raw pair keys, sorted in registers (blockRegisterSort), into s_buf[0, n);
// s_buf holds 2 kBlockMaxPairs keys (the sort's two buffers).
template <int E>
__device__ __forceinline__ void pairsSortKeys(const unsigned long long *keys, uint32_t n, unsigned long long *s_buf) {
    static_assert(kRegSortThreads * E <= kBlockMaxPairs, "sort buffers hold the keys");
    unsigned long long v[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const uint32_t i = threadIdx.x * E + r;
        v[r] = i < n ? keys[i] : ~0ull;
    }
    blockRegisterSort<unsigned long long, E>(v, s_buf, s_buf + kBlockMaxPairs);
    __syncthreads();  // the last shared-memory stage's reads are done
#pragma unroll
    for (int r = 0; r < E; ++r) {
        const uint32_t i = threadIdx.x * E + r;
        if (i < n) s_buf[i] = v[r];
    }
    __syncthreads();
}

// Single-block finalize for up to kBlockMaxPairs raw pairs: sort, dedup, slot
// mapping, same-body filter and order-preserving compaction in shared memory.
__global__ void __launch_bounds__(1024)
k_pairs_block(const unsigned long long *keys, uint32_t bits, const uint32_t *inSlot, const uint32_t *cbody,
              const uint32_t *cbgen, uint32_t *pairA, uint32_t *pairB, DevStats *st) {
    extern __shared__ unsigned long long s_buf[];  // 2 x kBlockMaxPairs keys, then kBlockMaxPairs flags
    uint32_t *s_flag = reinterpret_cast<uint32_t *>(s_buf + 2 * kBlockMaxPairs);
    __shared__ uint32_t s_scan[40];
    const uint32_t n = st->rawPairs;
    if (n > kBlockMaxPairs) {
        if (threadIdx.x == 0) atomicOr(&st->err, kErrSmallPath);
        return;
    }
    // up to 4096 keys sorted in registers; more (eight 64-bit keys a thread
    // would not stay in registers) by the shared-memory merge sort
    const unsigned long long *s_keys = s_buf;
    if (n <= kRegSortThreads) pairsSortKeys<1>(keys, n, s_buf);
    else if (n <= 2 * kRegSortThreads) pairsSortKeys<2>(keys, n, s_buf);
    else if (n <= 4 * kRegSortThreads) pairsSortKeys<4>(keys, n, s_buf);
    else {
        const uint32_t n2 = nextPow2(n);
        for (uint32_t i = threadIdx.x; i < n2; i += blockDim.x) s_buf[i] = i < n ? keys[i] : ~0ull;
        __syncthreads();
        s_keys = blockMergeSort<unsigned long long>(s_buf, s_buf + kBlockMaxPairs, n2);
    }
    const unsigned long long mask = (1ull << bits) - 1ull;
    uint32_t unique = 0;
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const unsigned long long key = s_keys[k];
        bool keep = !(k > 0 && s_keys[k - 1] == key);
        if (keep) {
            ++unique;
            uint32_t a = (uint32_t)(key >> bits), b = (uint32_t)(key & mask);
            if (inSlot) {
                a = inSlot[a];
                b = inSlot[b];
            }
            if (cbody && cbody[a] == cbody[b] && cbgen[a] == cbgen[b]) keep = false;
        }
        s_flag[k] = keep ? 1u : 0u;
    }
    if (unique) atomicAdd(&st->uniquePairs, unique);
    __syncthreads();
    const uint32_t total = blockExclusiveScanArray(s_flag, n, s_scan);
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const uint32_t next = k + 1 < n ? s_flag[k + 1] : total;
        if (next == s_flag[k]) continue;
        const unsigned long long key = s_keys[k];
        uint32_t a = (uint32_t)(key >> bits), b = (uint32_t)(key & mask);
        if (inSlot) {
            a = inSlot[a];
            b = inSlot[b];
        }
        pairA[s_flag[k]] = a;
        pairB[s_flag[k]] = b;
    }
    if (threadIdx.x == 0) st->pairs = total;
}

void launchPairsFinalize(const uint32_t *inSlot, const uint32_t *cbody, const uint32_t *cbgen, PairBuffers &pb,
                         DevStats *st, Scratch &ws, cudaStream_t s) {
    uint32_t *err = &st->err;
    if (pb.blockPath) {
        static bool configured = false;
        const size_t smem = kBlockMaxPairs * (2 * sizeof(unsigned long long) + sizeof(uint32_t));
        if (!configured) {
            PE_CHECK(cudaFuncSetAttribute(k_pairs_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            configured = true;
        }
        k_pairs_block<<<1, 1024, smem, s>>>(pb.keys, pb.bits, inSlot, cbody, cbgen, pb.a, pb.b, st);
        PE_LAUNCHED();
        return;
    }
    launchRadixSort<unsigned long long>(pb.keys, pb.keysTmp, nullptr, nullptr, &st->rawPairs, pb.cap, 0,
                                        2 * (int)pb.bits, ws, err, s);
    k_pairs_flags<<<gridFor(pb.cap), 256, 0, s>>>(&st->rawPairs, pb.cap, pb.bits, pb.keys, inSlot, cbody, cbgen,
                                                  pb.flags, st);
    PE_LAUNCHED();
    launchScanExclusive(pb.flags, pb.pos, &st->rawPairs, pb.cap, &st->pairs, ws, err, s);
    k_pairs_scatter<<<gridFor(pb.cap), 256, 0, s>>>(&st->rawPairs, pb.cap, pb.bits, pb.keys, inSlot, pb.flags,
                                                    pb.pos, pb.a, pb.b);
    PE_LAUNCHED();
}

void setSpinLimitBroad(uint32_t limit) { setSpinLimitOfUnit(limit); }

} // namespace pe
