// Block-level primitives for work that fits one thread block (shared-memory
// bitonic and merge sorts, a bitonic sort in registers, block-wide exclusive
// scan over many items).
#pragma once
#include <cstdint>

namespace pe {

// Sorts s[0, n) ascending in shared memory; n is a power of two (pad the tail
// with the key type's maximum).  All threads of the block call it.
template <class K> __device__ __forceinline__ void blockBitonicSort(K *s, uint32_t n) {
    for (uint32_t k = 2; k <= n; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const K a = s[i], b = s[ixj];
                    const bool ascending = (i & k) == 0;
                    if ((a > b) == ascending) {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Sorts a[0, n) ascending (n a power of two, tail padded with the maximum key)
// by merging: each thread sorts its own C = max(1, n / blockDim.x) consecutive
// keys in registers, then runs of C, 2C, ... are merged pairwise between a and
// b, every thread producing C outputs after a merge-path binary search (ties
// taken from the left run).  Returns the buffer (a or b) that holds the result.
// C is at most kMergeSortPer; all threads of the block call it.
constexpr uint32_t kMergeSortPer = 16;
template <class K> __device__ __forceinline__ K *blockMergeSort(K *a, K *b, uint32_t n) {
    const uint32_t T = blockDim.x, t = threadIdx.x;
    const uint32_t C = n > T ? n / T : 1u;
    if (t * C < n) {
        K r[kMergeSortPer];
#pragma unroll
        for (uint32_t c = 0; c < kMergeSortPer; ++c)
            if (c < C) r[c] = a[t * C + c];
        // insertion sort of the thread's run
        for (uint32_t c = 1; c < C; ++c) {
            const K v = r[c];
            uint32_t d = c;
            while (d > 0 && r[d - 1] > v) {
                r[d] = r[d - 1];
                --d;
            }
            r[d] = v;
        }
#pragma unroll
        for (uint32_t c = 0; c < kMergeSortPer; ++c)
            if (c < C) a[t * C + c] = r[c];
    }
    __syncthreads();
    K *src = a, *dst = b;
    for (uint32_t R = C; R < n; R <<= 1) {
        const uint32_t o = t * C;
        if (o < n) {
            const uint32_t base = (o / (2 * R)) * (2 * R), k = o - base;
            const K *A = src + base, *B = src + base + R;
            uint32_t lo = k > R ? k - R : 0u, hi = k < R ? k : R;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (A[mid] <= B[k - mid - 1]) lo = mid + 1;
                else hi = mid;
            }
            uint32_t i = lo, j = k - lo;
            for (uint32_t c = 0; c < C; ++c) {
                if (j >= R || (i < R && A[i] <= B[j])) dst[o + c] = A[i++];
                else dst[o + c] = B[j++];
            }
        }
        __syncthreads();
        K *tmp = src;
        src = dst;
        dst = tmp;
    }
    return src;
}

// Bitonic sort of N = kRegSortThreads * E keys held in registers, ascending;
// thread t holds positions [t E, t E + E) before and after.  Compare-exchange
// stages whose partner is in the same thread run in registers, those whose
// partner is in the same warp through shuffles, and only the stages with
// partners in other warps (j >= 32 E) through shared memory: bufA and bufB
// (N keys each) are used in turn, so one barrier per such stage suffices.
// All kRegSortThreads threads of the block call it (blockDim.x must be that).
constexpr uint32_t kRegSortThreads = 1024;
template <class K, int E> __device__ __forceinline__ void blockRegisterSort(K (&v)[E], K *bufA, K *bufB) {
    constexpr uint32_t N = kRegSortThreads * E;
    const uint32_t t = threadIdx.x;
    bool useA = true;
#pragma unroll
    for (uint32_t k = 2; k <= N; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32u * E) {
                K *buf = useA ? bufA : bufB;
                useA = !useA;
#pragma unroll
                for (int r = 0; r < E; ++r) buf[t * E + r] = v[r];
                __syncthreads();
#pragma unroll
                for (int r = 0; r < E; ++r) {
                    const uint32_t i = t * E + r;
                    const K p = buf[i ^ j];
                    const bool keepMin = ((i & j) == 0) == ((i & k) == 0);
                    v[r] = keepMin ? (p < v[r] ? p : v[r]) : (p > v[r] ? p : v[r]);
                }
            } else if (j >= (uint32_t)E) {
#pragma unroll
                for (int r = 0; r < E; ++r) {
                    const uint32_t i = t * E + r;
                    const K p = __shfl_xor_sync(0xffffffffu, v[r], j / E);
                    const bool keepMin = ((i & j) == 0) == ((i & k) == 0);
                    v[r] = keepMin ? (p < v[r] ? p : v[r]) : (p > v[r] ? p : v[r]);
                }
            } else {
#pragma unroll
                for (int r = 0; r < E; ++r) {
                    if ((r & j) != 0) continue;
                    const uint32_t i = t * E + r;
                    const K x = v[r], y = v[r ^ j];
                    if ((x > y) == ((i & k) == 0)) {
                        v[r] = y;
                        v[r ^ j] = x;
                    }
                }
            }
        }
    }
}

__device__ __forceinline__ uint32_t nextPow2(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

// In-place exclusive scan of s[0, n) (u32) by one block; returns the total.
// scratch needs blockDim.x / 32 + 1 entries.  All threads call it.
__device__ __forceinline__ uint32_t blockExclusiveScanArray(uint32_t *s, uint32_t n, uint32_t *scratch) {
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t b = threadIdx.x * per, e = min(n, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += s[i];
    // warp-level inclusive scan of the per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = (blockDim.x + 31) >> 5;
    uint32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) scratch[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int w = 0; w < warps; ++w) {
            uint32_t t = scratch[w];
            scratch[w] = acc;
            acc += t;
        }
        scratch[warps] = acc;
    }
    __syncthreads();
    uint32_t run = scratch[warp] + incl - sum;
    for (uint32_t i = b; i < e; ++i) {
        uint32_t t = s[i];
        s[i] = run;
        run += t;
    }
    const uint32_t total = scratch[warps];
    __syncthreads();
    return total;
}

} // namespace pe
