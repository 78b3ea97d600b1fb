// Scan and radix-sort kernels (see pe_prims.cuh) and their stream launchers.
//
// Both run as persistent grids: a fixed number of blocks (independent of the
// buffer capacity) loop over tiles taken from an atomic counter, so a launch
// sized for a large buffer costs nothing when the live count is small.  Tile
// ids are taken in launch order by running blocks, so the decoupled look-back
// of a tile only ever waits on tiles that are being processed.
#include <algorithm>
#include <atomic>

#include "pe_engine.h"
#include "pe_prims.cuh"

namespace pe {

unsigned long long g_kernelLaunches = 0;

void setSpinLimitPrims(uint32_t limit) { setSpinLimitOfUnit(limit); }

void setSpinLimit(uint32_t limit) {
    if (limit == 0) limit = kSpinLimitDefault;
    setSpinLimitPrims(limit);
    setSpinLimitBroad(limit);
    setSpinLimitNarrow(limit);
    setSpinLimitSleep(limit);
    setSpinLimitSolve(limit);
    setSpinLimitIslands(limit);
}

int smCount() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cached[kMaxDevices] = {};
    int dev = 0;
    PE_CHECK(cudaGetDevice(&dev));
    const bool cacheable = dev >= 0 && dev < kMaxDevices;
    int n = cacheable ? cached[dev].load(std::memory_order_relaxed) : 0;
    if (n == 0) {
        PE_CHECK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
        if (n < 1) n = 1;
        if (cacheable) cached[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

void *deviceAddress(const void *p, size_t align, int device) {
    if (!p || reinterpret_cast<uintptr_t>(p) % align) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // not a CUDA allocation: no sticky error
        return nullptr;
    }
    if (at.type == cudaMemoryTypeHost) return at.devicePointer;
    if ((at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == device)
        return at.devicePointer;
    return nullptr;
}

namespace {
inline uint32_t persistentGrid(uint32_t tiles) {
    return std::max<uint32_t>(1, std::min<uint32_t>(tiles, 4u * (uint32_t)smCount()));
}
__device__ __forceinline__ uint32_t liveCount(const uint32_t *d_n, uint32_t cap) {
    if (!d_n) return cap;
    const uint32_t n = *d_n;
    return n < cap ? n : cap;
}
} // namespace

// ---------------------------------------------------------------------------
// Exclusive scan (u32), one pass with decoupled look-back.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kScanThreads)
k_scan_exclusive(const uint32_t *in, uint32_t *out, const uint32_t *d_n, uint32_t cap, unsigned long long *state,
                 uint32_t *counter, uint32_t *total, uint32_t *err) {
    __shared__ uint32_t s_tile, s_scan[9], s_prefix, s_abort;
    const uint32_t n = liveCount(d_n, cap);
    const uint32_t ntiles = max((n + kScanTile - 1) / kScanTile, 1u);
    for (;;) {
        const uint32_t tile = takeTile(counter, &s_tile);
        if (tile >= ntiles) return;
        const uint32_t i0 = tile * kScanTile + threadIdx.x * kScanItems;
        uint32_t v[kScanItems];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = (i0 + k < n) ? in[i0 + k] : 0u;
            sum += v[k];
        }
        uint32_t agg;
        const uint32_t excl = blockExclusiveScan(sum, agg, s_scan);
        if (threadIdx.x < 32) {
            bool timedOut;
            const uint32_t pre = lookbackExclusiveWarp(state, tile, agg, err, &timedOut);
            if (threadIdx.x == 0) {
                s_prefix = pre;
                s_abort = timedOut ? 1u : 0u;
            }
        }
        __syncthreads();
        if (s_abort) return;  // a bounded wait ran out: nothing of this tile is written
        uint32_t run = s_prefix + excl;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (i0 + k < n) out[i0 + k] = run;
            run += v[k];
        }
        if (threadIdx.x == 0 && tile + 1 == ntiles && total) *total = s_prefix + agg;
        __syncthreads();
    }
}

void launchScanExclusive(const uint32_t *in, uint32_t *out, const uint32_t *d_n, uint32_t max_n, uint32_t *d_total,
                         Scratch &ws, uint32_t *d_err, cudaStream_t s) {
    const uint32_t tiles = std::max<uint32_t>((max_n + kScanTile - 1) / kScanTile, 1);
    PE_CHECK(cudaMemsetAsync(ws.scanState, 0, sizeof(unsigned long long) * (tiles + 1), s));
    k_scan_exclusive<<<persistentGrid(tiles), kScanThreads, 0, s>>>(in, out, d_n, max_n, ws.scanState,
                                                                    (uint32_t *)(ws.scanState + tiles), d_total,
                                                                    d_err);
    PE_LAUNCHED();
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits, keys u32/u64 with optional u32 values.
// ---------------------------------------------------------------------------
// Histograms of every pass in one read of the keys; also clears the look-back
// state and tile counters of all passes for the live tile count.
template <class K>
__global__ void k_radix_hist(const K *keys, const uint32_t *d_n, uint32_t cap, int bit_begin, int passes,
                             uint32_t *hist, uint32_t *state, size_t passStride, uint32_t *counters) {
    __shared__ uint32_t sh[8 * 256];
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) sh[i] = 0;
    const uint32_t n = liveCount(d_n, cap);
    const uint32_t ntiles = (n + kSortTile - 1) / kSortTile;
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    for (int p = 0; p < passes; ++p)
        for (uint32_t i = gtid; i < ntiles * 256; i += gstride) state[p * passStride + i] = 0;
    if (gtid < (uint32_t)passes) counters[gtid] = 0;
    __syncthreads();
    for (uint32_t i = gtid; i < n; i += gstride) {
        const K k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p * 256 + (uint32_t)((k >> (bit_begin + 8 * p)) & 0xFF)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// One 8-bit pass.  The pass reads from buffer sel[pass] and writes the other;
// a pass whose digit is the same for every key is skipped on the device
// (sel[pass + 1] = sel[pass]), so key widths need not be exact on the host.
template <class K, bool VALS>
__global__ void __launch_bounds__(kSortThreads)
k_radix_pass(K *buf0, K *buf1, uint32_t *vbuf0, uint32_t *vbuf1, const uint32_t *d_n, uint32_t cap, int shift,
             const uint32_t *__restrict__ hist, uint32_t *state, uint32_t *counter, uint32_t *sel, int pass,
             uint32_t *err) {
    __shared__ uint32_t s_tile, s_trivial, s_abort;
    __shared__ uint32_t s_warp[kSortWarps][256];
    __shared__ uint32_t s_tileStart[256];
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_bucket[256];
    __shared__ uint32_t s_scan[9];
    __shared__ K s_keys[kSortTile];
    __shared__ uint32_t s_vals[VALS ? kSortTile : 1];

    const uint32_t n = liveCount(d_n, cap);
    const uint32_t from = sel[pass];
    if (threadIdx.x == 0) s_trivial = 0;
    __syncthreads();
    if (hist[threadIdx.x] == n) s_trivial = 1;
    __syncthreads();
    if (s_trivial) {
        if (blockIdx.x == 0 && threadIdx.x == 0) sel[pass + 1] = from;
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sel[pass + 1] = 1u - from;
    const K *kin = from ? buf1 : buf0;
    K *kout = from ? buf0 : buf1;
    const uint32_t *vin = from ? vbuf1 : vbuf0;
    uint32_t *vout = from ? vbuf0 : vbuf1;
    {
        uint32_t tot;
        s_bucket[threadIdx.x] = blockExclusiveScan(hist[threadIdx.x], tot, s_scan);
    }
    const uint32_t ntiles = (n + kSortTile - 1) / kSortTile;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    for (;;) {
        const uint32_t tile = takeTile(counter, &s_tile);
        if (tile >= ntiles) return;
        const uint32_t base = tile * kSortTile;
        for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads) (&s_warp[0][0])[i] = 0;
        if (threadIdx.x == 0) s_abort = 0;
        __syncthreads();

        K key[kSortRounds];
        uint32_t val[kSortRounds], dig[kSortRounds], rank[kSortRounds];
#pragma unroll
        for (int r = 0; r < kSortRounds; ++r) {
            const uint32_t idx = base + warp * (32 * kSortRounds) + r * 32 + lane;
            const bool valid = idx < n;
            key[r] = valid ? kin[idx] : (K)0;
            if (VALS) val[r] = valid ? vin[idx] : 0u;
            dig[r] = valid ? (uint32_t)((key[r] >> shift) & 0xFF) : 0xFFu;
            const uint32_t peers = __match_any_sync(0xffffffffu, dig[r]);
            const uint32_t lower = __popc(peers & lanemask_lt);
            const uint32_t old = s_warp[warp][dig[r]];
            __syncwarp();
            if (lower == 0) s_warp[warp][dig[r]] = old + __popc(peers);
            __syncwarp();
            rank[r] = old + lower;
        }
        __syncthreads();
        const uint32_t d = threadIdx.x;
        uint32_t cnt = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = s_warp[w][d];
            s_warp[w][d] = cnt;
            cnt += c;
        }
        uint32_t tot;
        const uint32_t tileStart = blockExclusiveScan(cnt, tot, s_scan);
        s_tileStart[d] = tileStart;
        // Look-back for this digit (flag in bits 30-31, count in bits 0-29).
        uint32_t prefix = 0;
        if (tile == 0) {
            atomicExch(&state[d], (2u << 30) | cnt);
        } else {
            atomicExch(&state[tile * 256 + d], (1u << 30) | cnt);
            int64_t t = (int64_t)tile - 1;
            uint32_t spins = 0;
            bool timedOut = false;
            while (t >= 0) {
                const uint32_t v = ldvol(&state[t * 256 + d]);
                const uint32_t f = v >> 30;
                if (f == 0) {
                    if (++spins > spinLimit()) {
                        atomicOr(err, kErrTimeout);
                        s_abort = 1;
                        timedOut = true;
                        break;
                    }
                    continue;
                }
                prefix += v & 0x3FFFFFFFu;
                if (f == 2) break;
                --t;
            }
            // a digit whose wait ran out publishes nothing
            if (!timedOut) atomicExch(&state[tile * 256 + d], (2u << 30) | (prefix + cnt));
        }
        s_base[d] = s_bucket[d] + prefix - tileStart;
        __syncthreads();
        if (s_abort) return;  // a bounded wait ran out: nothing of this tile is written
#pragma unroll
        for (int r = 0; r < kSortRounds; ++r) {
            const uint32_t idx = base + warp * (32 * kSortRounds) + r * 32 + lane;
            if (idx < n) {
                const uint32_t pos = s_tileStart[dig[r]] + s_warp[warp][dig[r]] + rank[r];
                s_keys[pos] = key[r];
                if (VALS) s_vals[pos] = val[r];
            }
        }
        __syncthreads();
        const uint32_t live = min((uint32_t)kSortTile, n - base);
        for (uint32_t j = threadIdx.x; j < live; j += kSortThreads) {
            const K k = s_keys[j];
            const uint32_t dst = s_base[(uint32_t)((k >> shift) & 0xFF)] + j;
            kout[dst] = k;
            if (VALS) vout[dst] = s_vals[j];
        }
        __syncthreads();
    }
}

// Moves the result back into buffer 0 when an odd number of passes ran.
template <class K>
__global__ void k_radix_fixup(K *buf0, const K *buf1, uint32_t *v0, const uint32_t *v1, const uint32_t *d_n,
                              uint32_t cap, const uint32_t *sel) {
    if (*sel == 0) return;
    const uint32_t n = liveCount(d_n, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        buf0[i] = buf1[i];
        if (v0) v0[i] = v1[i];
    }
}

// Sorts keys (and values) in place over bits [bit_begin, bit_end); keys_tmp /
// vals_tmp are scratch of the same size.  Stable.  The live count is
// min(*d_n, max_n) (max_n alone when d_n is null).
template <class K>
void launchRadixSort(K *keys, K *keys_tmp, uint32_t *vals, uint32_t *vals_tmp, const uint32_t *d_n, uint32_t max_n,
                     int bit_begin, int bit_end, Scratch &ws, uint32_t *d_err, cudaStream_t s) {
    if (max_n == 0 || bit_end <= bit_begin) return;
    const int passes = std::min((bit_end - bit_begin + 7) / 8, 8);
    const uint32_t tiles = (max_n + kSortTile - 1) / kSortTile;
    const size_t passStride = 256 * (size_t)tiles;
    uint32_t *sel = ws.sortHist + 256 * 8;
    uint32_t *counters = ws.sortHist + 256 * 8 + 16;
    PE_CHECK(cudaMemsetAsync(ws.sortHist, 0, sizeof(uint32_t) * (256 * 8 + 16), s));
    const uint32_t hb = std::max<uint32_t>(1, std::min<uint32_t>((max_n + 255) / 256, 4u * (uint32_t)smCount()));
    k_radix_hist<K><<<hb, 256, 0, s>>>(keys, d_n, max_n, bit_begin, passes, ws.sortHist, ws.sortState, passStride,
                                       counters);
    PE_LAUNCHED();
    const uint32_t grid = persistentGrid(tiles);
    for (int p = 0; p < passes; ++p) {
        uint32_t *state = ws.sortState + p * passStride;
        if (vals)
            k_radix_pass<K, true><<<grid, kSortThreads, 0, s>>>(keys, keys_tmp, vals, vals_tmp, d_n, max_n,
                                                                bit_begin + 8 * p, ws.sortHist + 256 * p, state,
                                                                counters + p, sel, p, d_err);
        else
            k_radix_pass<K, false><<<grid, kSortThreads, 0, s>>>(keys, keys_tmp, nullptr, nullptr, d_n, max_n,
                                                                 bit_begin + 8 * p, ws.sortHist + 256 * p, state,
                                                                 counters + p, sel, p, d_err);
        PE_LAUNCHED();
    }
    k_radix_fixup<K><<<hb, 256, 0, s>>>(keys, keys_tmp, vals, vals_tmp, d_n, max_n, sel + passes);
    PE_LAUNCHED();
}

template void launchRadixSort<uint32_t>(uint32_t *, uint32_t *, uint32_t *, uint32_t *, const uint32_t *, uint32_t,
                                        int, int, Scratch &, uint32_t *, cudaStream_t);
template void launchRadixSort<unsigned long long>(unsigned long long *, unsigned long long *, uint32_t *, uint32_t *,
                                                  const uint32_t *, uint32_t, int, int, Scratch &, uint32_t *,
                                                  cudaStream_t);

__global__ void k_clamp_u32(const uint32_t *src, uint32_t cap, uint32_t *dst) {
    uint32_t v = *src;
    *dst = v < cap ? v : cap;
}
void launchClamp(const uint32_t *src, uint32_t cap, uint32_t *dst, cudaStream_t s) {
    k_clamp_u32<<<1, 1, 0, s>>>(src, cap, dst);
    PE_LAUNCHED();
}

size_t scratchBytesScan(uint32_t max_n) {
    uint32_t tiles = (max_n + kScanTile - 1) / kScanTile + 1;
    return sizeof(unsigned long long) * tiles + 16;
}
// Look-back state of all (up to 8) passes of one sort.
size_t scratchBytesSort(uint32_t max_n) {
    uint32_t tiles = (max_n + kSortTile - 1) / kSortTile + 1;
    return sizeof(uint32_t) * (8 * 256 * (size_t)tiles + 16);
}

} // namespace pe
