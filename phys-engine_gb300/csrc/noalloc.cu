// Allocation-free sweep-and-prune broadphase: the entry point behind
// pe_broadphase_find_pairs_noalloc (include/phys_gb300.h).
//
// Some callers cannot let a library allocate device memory: a host engine that
// hands this library a slice of its own pre-reserved arena and forbids any other
// allocation, a frame loop with a hard time budget in which cudaMalloc's
// implicit device synchronisation is not acceptable, or a process that already
// holds nearly all of the GPU's memory.  For them this file keeps every byte of
// scratch the kernel needs in one file-scope device array, sized at compile
// time.  The module loader places it in device memory when the library's code
// is first loaded on a GPU, and every GPU that loads the library keeps it until
// the process exits.  The caller passes only its own inputs and outputs.
//
// Results equal those of pe_broadphase_find_pairs with PE_BROADPHASE_SAP on the
// same boxes (same keys, same sweep test, same lexicographic pair order), up to
// PE_NOALLOC_MAX_BOXES boxes and PE_NOALLOC_MAX_PAIRS pairs.
#include <mutex>
#include <stdexcept>
#include <string>

#include "pe_block.cuh"
#include "pe_engine.h"
#include "pe_math.cuh"
#include "phys_gb300.h"

namespace pe {
namespace {

constexpr uint32_t kMaxBoxes = PE_NOALLOC_MAX_BOXES;
constexpr uint32_t kMaxPairs = PE_NOALLOC_MAX_PAIRS;
constexpr uint32_t kThreads = 1024;
constexpr int kMaxDevices = 64;

// Scratch layout (byte offsets, each a multiple of 256).
constexpr size_t kOrderOff = 0;                                     // u64 (min.x key << 32 | box) x kMaxBoxes
constexpr size_t kPairOff = kOrderOff + 8ull * kMaxBoxes;           // u64 (first << 32 | second) x kMaxPairs
constexpr size_t kMinXOff = kPairOff + 8ull * kMaxPairs;            // f32 sorted min.x x kMaxBoxes
constexpr size_t kMaxXOff = kMinXOff + 4ull * kMaxBoxes;            // f32 sorted max.x x kMaxBoxes
constexpr size_t kYZOff = kMaxXOff + 4ull * kMaxBoxes;              // float4 (min.y, max.y, min.z, max.z)
constexpr size_t kIdxOff = kYZOff + 16ull * kMaxBoxes;              // u32 box index of sorted entry
constexpr size_t kScratchBytes = kIdxOff + 4ull * kMaxBoxes;        // 557,056 bytes
static_assert(kScratchBytes % 256 == 0, "scratch sections stay 256-byte aligned");

// The only scratch the allocation-free path uses.  In host code this name is a
// stand-in for the device symbol, not a device address: the address is taken
// with cudaGetSymbolAddress on each device.
static __device__ __align__(256) unsigned char g_sapScratch[kScratchBytes];

__device__ __forceinline__ bool overlapYZ(const float4 &f, const float4 &s) {
    // f, s = (min.y, max.y, min.z, max.z): the y/z test of the sweep,
    // src/collision/broadphase.cpp:233-236
    return f.x <= s.y && f.y >= s.x && f.z <= s.w && f.w >= s.z;
}

// One block does the whole query: sort by min.x, sweep, sort the pairs.
// Nothing in the scratch is assumed to start at any value: every word read is
// written earlier in the same launch (sort padding included), and the pair
// counter lives in shared memory.
__global__ void __launch_bounds__(kThreads) k_sap_noalloc(const float *mins, const float *maxs, uint32_t n,
                                                          unsigned char *scratch, uint32_t *pairsOut,
                                                          uint32_t capacity, uint32_t *result) {
    unsigned long long *order = reinterpret_cast<unsigned long long *>(scratch + kOrderOff);
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(scratch + kPairOff);
    float *sMinX = reinterpret_cast<float *>(scratch + kMinXOff);
    float *sMaxX = reinterpret_cast<float *>(scratch + kMaxXOff);
    float4 *sYZ = reinterpret_cast<float4 *>(scratch + kYZOff);
    uint32_t *sIdx = reinterpret_cast<uint32_t *>(scratch + kIdxOff);
    __shared__ uint32_t s_count;

    // Sort entries by (min.x, index), the sweep's comparator
    // (src/collision/broadphase.cpp:212-216); -0 and +0 share a key.
    const uint32_t np = nextPow2(n > 0 ? n : 1);
    for (uint32_t i = threadIdx.x; i < np; i += blockDim.x)
        order[i] = i < n ? ((unsigned long long)orderedFloatKey(mins[3 * i]) << 32) | i : ~0ull;
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    blockBitonicSort(order, np);
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t b = (uint32_t)order[i];
        sMinX[i] = mins[3 * b];
        sMaxX[i] = maxs[3 * b];
        sYZ[i] = make_float4(mins[3 * b + 1], maxs[3 * b + 1], mins[3 * b + 2], maxs[3 * b + 2]);
        sIdx[i] = b;
    }
    __syncthreads();

    // Sweep: entry i meets every later entry whose min.x <= max.x(i)
    // (src/collision/broadphase.cpp:226-241); the window end is found by the
    // same binary search as the device-wide path.
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float x = sMaxX[i];
        uint32_t lo = i + 1, hi = n;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (sMinX[mid] > x) hi = mid;
            else lo = mid + 1;
        }
        const float4 f = sYZ[i];
        const uint32_t fi = sIdx[i];
        for (uint32_t j = i + 1; j < lo; ++j) {
            if (!overlapYZ(f, sYZ[j])) continue;
            const uint32_t sj = sIdx[j];
            const uint32_t slot = atomicAdd(&s_count, 1u);
            if (slot < kMaxPairs)
                keys[slot] = ((unsigned long long)min(fi, sj) << 32) | max(fi, sj);
        }
    }
    __syncthreads();

    const uint32_t total = s_count;
    if (total > kMaxPairs) {
        if (threadIdx.x == 0) {
            result[0] = total;
            result[1] = 2;
        }
        return;
    }
    // Lexicographic pair order (src/collision/broadphase.cpp:18-60).
    const uint32_t pp = nextPow2(total > 0 ? total : 1);
    for (uint32_t i = total + threadIdx.x; i < pp; i += blockDim.x) keys[i] = ~0ull;
    __syncthreads();
    blockBitonicSort(keys, pp);
    const uint32_t written = total < capacity ? total : capacity;
    for (uint32_t k = threadIdx.x; k < written; k += blockDim.x) {
        const unsigned long long key = keys[k];
        pairsOut[2 * k] = (uint32_t)(key >> 32);
        pairsOut[2 * k + 1] = (uint32_t)key;
    }
    if (threadIdx.x == 0) {
        result[0] = total;
        result[1] = total > capacity ? 1 : 0;
    }
}

std::mutex g_setupMutex;
unsigned char *g_scratchPtr[kMaxDevices] = {};

// Device address of g_sapScratch on `device`, looked up on the first call for
// that device with the device current.  The lookup makes the runtime load this
// library's device code on that GPU if it has not yet done so.  The address is
// kept for the life of the process: it stays valid as long as the device's
// primary context does, so the entry point must not be used on a device after
// cudaDeviceReset (the module would be reloaded and the array could move).
unsigned char *scratchOn(int device) {
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_scratchPtr[device]) {
        void *p = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&p, g_sapScratch);
        if (rc != cudaSuccess)
            throw CudaError(std::string("cudaGetSymbolAddress(broadphase scratch): ") + cudaGetErrorString(rc));
        g_scratchPtr[device] = static_cast<unsigned char *>(p);
    }
    return g_scratchPtr[device];
}

} // namespace

void findPairsNoAlloc(int device, const float *mins, const float *maxs, uint32_t n, uint32_t *pairs,
                      uint32_t capacity, uint32_t *result, cudaStream_t s) {
    if (device < 0 || device >= kMaxDevices) throw std::invalid_argument("device ordinal out of range");
    if (n > kMaxBoxes)
        throw std::invalid_argument("pe_broadphase_find_pairs_noalloc: " + std::to_string(n) +
                                    " boxes exceed its limit of " + std::to_string(kMaxBoxes) +
                                    " (PE_NOALLOC_MAX_BOXES); use pe_broadphase_find_pairs");
    // The caller's current device is put back on every return, the error
    // paths included: a host engine that drives several GPUs from one thread
    // keeps its own notion of the current device.
    int previous = 0;
    PE_CHECK(cudaGetDevice(&previous));
    struct RestoreDevice {
        int device;
        ~RestoreDevice() { cudaSetDevice(device); }
    } restore{previous};
    PE_CHECK(cudaSetDevice(device));
    unsigned char *scratch = scratchOn(device);
    k_sap_noalloc<<<1, kThreads, 0, s>>>(mins, maxs, n, scratch, pairs, capacity, result);
    PE_LAUNCHED();
}

} // namespace pe
