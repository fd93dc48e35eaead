// radix_sort.cu - stage 3: stable LSD key-value radix sort, onesweep style.
//
// Replaces RadixSort (NexusBVH/src/Cuda/Setup.cu:62-112), which calls CUB
// 3.0.1 cub::DeviceRadixSort::SortPairs on bits [2,32) of 32-bit keys or
// [1,64) of 64-bit keys, carrying the full keys.  Written from the published
// onesweep algorithm (Adinets & Merrill 2022): the digit histograms of all
// passes come from one up-front read (fused into the Morton kernel), then
// one kernel per 8-bit digit:
//   * tiles are claimed in order through an atomic counter, so a tile only
//     ever waits on tiles that are already running;
//   * each warp ranks its keys stably with ballots over the digit bits;
//   * the tile's digit counts are published and the exclusive prefix is
//     found by decoupled look-back over predecessor tiles (bounded polls:
//     on expiry the error word is set and the kernel finishes);
//   * keys are reordered in shared memory so that the global scatter writes
//     runs of consecutive addresses.
#include <algorithm>
#include <mutex>

#include "pipeline.h"

namespace nxb {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;

template <typename K>
struct Tile;
template <>
struct Tile<uint32_t> {
    static constexpr int kKeysPerThread = 16;
};
template <>
struct Tile<uint64_t> {
    static constexpr int kKeysPerThread = 12;
};

template <typename K>
__host__ __device__ constexpr int tile_keys() {
    return kThreads * Tile<K>::kKeysPerThread;
}

// Dynamic shared memory of a tile: its keys and values, then one digit
// histogram per warp (RB-bit digits).
template <typename K, int RB>
__host__ __device__ constexpr size_t dyn_smem_bytes() {
    return (size_t)tile_keys<K>() * (sizeof(K) + sizeof(uint32_t)) + (size_t)kWarps * (1u << RB) * sizeof(uint32_t);
}

// Exclusive scan of one value per thread over a 256-thread CTA.
__device__ __forceinline__ uint32_t cta_exclusive_scan(uint32_t v, uint32_t* s_tmp) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) s_tmp[warp] = incl;
    __syncthreads();
    uint32_t pre = 0;
    for (uint32_t w = 0; w < warp; ++w) pre += s_tmp[w];
    __syncthreads();
    return pre + incl - v;
}

template <bool L2, typename T>
__device__ __forceinline__ T ld_data(const T* p) {
    if constexpr (L2)
        return __ldcg(p);
    else
        return *p;
}

// One onesweep tile: `bits`-bit digits at `shift` (bits <= RB), RB-bit
// digit tables.  The caller has zeroed the per-warp histograms in the
// dynamic shared memory and synchronised.  With RB = 9 each thread owns two
// adjacent digits in the tile-wide steps (publish, look-back, scans).  L2:
// every load of data written by other CTAs bypasses L1 (the persistent
// fallback kernel reads buffers that other CTAs of the same launch wrote).
template <typename K, bool HAS_VALS, int RB, bool L2>
__device__ __forceinline__ void sort_tile(uint32_t tile, const K* __restrict__ kin, K* __restrict__ kout,
                                          const uint32_t* __restrict__ vin, uint32_t* __restrict__ vout, uint32_t n,
                                          uint32_t shift, uint32_t bits, const uint32_t* __restrict__ hist,
                                          uint32_t* lookback, uint32_t* err, unsigned char* smem, uint32_t* s_delta,
                                          uint16_t* s_local, uint32_t* s_tmp) {
    constexpr int KPT = Tile<K>::kKeysPerThread;
    constexpr int TILE = tile_keys<K>();
    constexpr int BINS = 1 << RB;
    constexpr int DPT = BINS / kThreads;  // digits per thread: 1 or 2
    static_assert(DPT == 1 || DPT == 2, "8- or 9-bit digit tables");
    K* s_keys = reinterpret_cast<K*>(smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
    uint32_t* s_whist = s_vals + TILE;

    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const uint32_t mask = (1u << bits) - 1u;
    const uint32_t tile_base = tile * (uint32_t)TILE;
    if (tile_base >= n) return;  // only reachable when a launch claims more tiles than exist
    const uint32_t d0 = tid * DPT;  // first digit this thread owns in the tile-wide steps
    // the global start of each digit (exclusive scan of this pass's
    // histogram): only tile 0 needs it, the others inherit it through the
    // look-back
    uint32_t excl[DPT];
#pragma unroll
    for (int k = 0; k < DPT; ++k) excl[k] = 0;
    if (tile == 0) {
        uint32_t h[DPT], hs = 0;
#pragma unroll
        for (int k = 0; k < DPT; ++k) {
            h[k] = d0 + k <= mask ? ld_data<L2>(hist + d0 + k) : 0u;
            hs += h[k];
        }
        uint32_t e = cta_exclusive_scan(hs, s_tmp);
#pragma unroll
        for (int k = 0; k < DPT; ++k) {
            excl[k] = e;
            e += h[k];
        }
    }

    // ---- load (warp-striped: warp w owns a contiguous run of 32*KPT keys)
    K key[KPT];
    uint32_t val[KPT];
    uint32_t rank[KPT];
    const uint32_t wbase = tile_base + warp * 32u * KPT + lane;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const uint32_t idx = wbase + 32u * j;
        const bool valid = idx < n;
        key[j] = valid ? ld_data<L2>(kin + idx) : (K)0;
        if (HAS_VALS)
            val[j] = valid ? ld_data<L2>(vin + idx) : 0u;
        else
            val[j] = idx;
    }

    // ---- stable rank within the warp, one digit group at a time
    uint32_t* wh = s_whist + warp * BINS;
    const uint32_t lt_mask = lanemask_lt();
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const bool valid = wbase + 32u * j < n;
        const uint32_t d = (uint32_t)(key[j] >> shift) & mask;
        uint32_t peers = __ballot_sync(kFullMask, valid);
#pragma unroll
        for (int b = 0; b < RB; ++b) {
            if (b < (int)bits) {
                const bool bit = (d >> b) & 1u;
                const uint32_t bb = __ballot_sync(kFullMask, bit);
                peers &= bit ? bb : ~bb;
            }
        }
        const uint32_t below = __popc(peers & lt_mask);
        const uint32_t leader = (uint32_t)(__ffs(peers) - 1) & 31u;
        uint32_t base = 0;
        if (valid && below == 0) {
            base = wh[d];
            wh[d] = base + __popc(peers);
        }
        base = __shfl_sync(kFullMask, base, leader);
        rank[j] = base + below;
        __syncwarp();
    }
    __syncthreads();

    // ---- per-digit tile count and per-warp exclusive offsets (thread = digits d0 .. d0+DPT-1)
    uint32_t cnt[DPT];
#pragma unroll
    for (int k = 0; k < DPT; ++k) {
        uint32_t c = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t x = s_whist[w * BINS + d0 + k];
            s_whist[w * BINS + d0 + k] = c;
            c += x;
        }
        cnt[k] = c;
    }

    // ---- publish, then decoupled look-back for these digits
    uint32_t* lb = lookback + (size_t)tile * BINS + d0;
    const bool mine = d0 <= mask;  // digits beyond this pass's width are empty
    if (tile == 0) {
        if (mine) {
            if constexpr (DPT == 1)
                atomicExch(lb, kFlagInc | (excl[0] + cnt[0]));
            else
                st_relaxed_u64(reinterpret_cast<uint64_t*>(lb),
                               (uint64_t)(kFlagInc | (excl[0] + cnt[0])) |
                                   ((uint64_t)(kFlagInc | (excl[1] + cnt[1])) << 32));
        }
    } else if (mine) {
        if constexpr (DPT == 1) {
            atomicExch(lb, kFlagAgg | cnt[0]);
            int32_t pred = (int32_t)tile - 1;
            uint32_t polls = 0;
            while (pred >= 0) {
                const uint32_t v = ld_relaxed_u32(lookback + (size_t)pred * BINS + d0);
                const uint32_t flag = v & ~kCountMask;
                if (flag == 0) {
                    if (++polls > kSpinLimit) {
                        set_error(err, NXB_DEVERR_SORT_LOOKBACK_TIMEOUT);
                        break;
                    }
                    if (polls > 64) __nanosleep(64);
                    continue;
                }
                excl[0] += v & kCountMask;
                if (flag == kFlagInc) break;
                --pred;
            }
            atomicExch(lb, kFlagInc | (excl[0] + cnt[0]));
        } else {
            // both digits' words in one 64-bit access; a digit stops adding
            // once it has met an inclusive word
            st_relaxed_u64(reinterpret_cast<uint64_t*>(lb),
                           (uint64_t)(kFlagAgg | cnt[0]) | ((uint64_t)(kFlagAgg | cnt[1]) << 32));
            int32_t pred = (int32_t)tile - 1;
            uint32_t polls = 0;
            bool done0 = false, done1 = false;
            while (pred >= 0) {
                const uint64_t v2 =
                    ld_relaxed_u64(reinterpret_cast<const uint64_t*>(lookback + (size_t)pred * BINS + d0));
                const uint32_t v0 = (uint32_t)v2, v1 = (uint32_t)(v2 >> 32);
                const uint32_t f0 = v0 & ~kCountMask, f1 = v1 & ~kCountMask;
                if ((!done0 && f0 == 0) || (!done1 && f1 == 0)) {
                    if (++polls > kSpinLimit) {
                        set_error(err, NXB_DEVERR_SORT_LOOKBACK_TIMEOUT);
                        break;
                    }
                    if (polls > 64) __nanosleep(64);
                    continue;
                }
                if (!done0) {
                    excl[0] += v0 & kCountMask;
                    done0 = f0 == kFlagInc;
                }
                if (!done1) {
                    excl[1] += v1 & kCountMask;
                    done1 = f1 == kFlagInc;
                }
                if (done0 && done1) break;
                --pred;
            }
            st_relaxed_u64(reinterpret_cast<uint64_t*>(lb), (uint64_t)(kFlagInc | (excl[0] + cnt[0])) |
                                                                 ((uint64_t)(kFlagInc | (excl[1] + cnt[1])) << 32));
        }
    }
    // local start of each digit in the tile (s_local), and the offset that
    // maps a tile position to its global position (s_delta)
    {
        uint32_t cs = 0;
#pragma unroll
        for (int k = 0; k < DPT; ++k) cs += d0 + k <= mask ? cnt[k] : 0u;
        uint32_t e = cta_exclusive_scan(cs, s_tmp);
#pragma unroll
        for (int k = 0; k < DPT; ++k) {
            s_local[d0 + k] = (uint16_t)e;
            s_delta[d0 + k] = excl[k] - e;
            e += cnt[k];
        }
    }
    __syncthreads();

    // ---- reorder the tile by digit in shared memory
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        if (wbase + 32u * j < n) {
            const uint32_t d = (uint32_t)(key[j] >> shift) & mask;
            const uint32_t pos = s_local[d] + wh[d] + rank[j];
            s_keys[pos] = key[j];
            s_vals[pos] = val[j];
        }
    }
    __syncthreads();

    // ---- scatter runs of equal digits to consecutive global addresses
    const uint32_t tile_n = min((uint32_t)TILE, n - tile_base);
    for (uint32_t i = tid; i < tile_n; i += kThreads) {
        const K k = s_keys[i];
        const uint32_t d = (uint32_t)(k >> shift) & mask;
        const uint32_t g = s_delta[d] + i;
        if (g < n) {  // always true unless a look-back wait expired
            kout[g] = k;
            vout[g] = s_vals[i];
        }
    }
}

template <typename K, bool HAS_VALS, int RB>
__global__ __launch_bounds__(kThreads, 4) void onesweep_kernel(const K* __restrict__ kin, K* __restrict__ kout,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ vout, uint32_t n, uint32_t shift,
                                                            uint32_t bits, const uint32_t* __restrict__ hist,
                                                            uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_delta[1 << RB];
    __shared__ uint16_t s_local[1 << RB];
    __shared__ uint32_t s_tmp[kWarps];
    __shared__ uint32_t s_tile;
    uint32_t* s_whist = reinterpret_cast<uint32_t*>(smem + (size_t)tile_keys<K>() * (sizeof(K) + sizeof(uint32_t)));
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int i = threadIdx.x; i < kWarps * (1 << RB); i += kThreads) s_whist[i] = 0;
    __syncthreads();
    sort_tile<K, HAS_VALS, RB, false>(s_tile, kin, kout, vin, vout, n, shift, bits, hist, lookback, err, smem, s_delta,
                                      s_local, s_tmp);
}

// The same pass for 32-bit keys (8-bit digits, one digit per thread) as a
// kernel of its own: sort_tile compiled for 32-bit keys executes 24 % more
// warp instructions (28.4 M against 22.8 M for a 4.19M-key pass) and takes
// 11 % longer (0.478 against 0.428 ms for the four passes of 12.58M 30-bit
// keys); for 64-bit keys sort_tile is not slower.
template <bool HAS_VALS>
__global__ __launch_bounds__(kThreads, 4) void onesweep32_kernel(const uint32_t* __restrict__ kin, uint32_t* __restrict__ kout,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ vout, uint32_t n, uint32_t shift,
                                                            uint32_t bits, const uint32_t* __restrict__ hist,
                                                            uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err) {
    using K = uint32_t;
    constexpr int KPT = Tile<K>::kKeysPerThread;
    constexpr int TILE = tile_keys<K>();
    extern __shared__ __align__(16) unsigned char smem[];
    K* s_keys = reinterpret_cast<K*>(smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
    uint32_t* s_whist = s_vals + TILE;
    __shared__ uint32_t s_local_start[kRadixBins];
    __shared__ uint32_t s_global_start[kRadixBins];
    __shared__ uint32_t s_tmp[kWarps];
    __shared__ uint32_t s_tile;

    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const uint32_t mask = (1u << bits) - 1u;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int i = tid; i < kWarps * kRadixBins; i += kThreads) s_whist[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t tile_base = tile * (uint32_t)TILE;
    if (tile_base >= n) return;  // only reachable when a launch claims more tiles than exist
    // global start of each digit (exclusive scan of this pass's histogram):
    // only tile 0 needs it, the others inherit it through the look-back
    uint32_t digit_base = 0;
    if (tile == 0) digit_base = cta_exclusive_scan(tid <= mask ? hist[tid] : 0u, s_tmp);

    // ---- load (warp-striped: warp w owns a contiguous run of 32*KPT keys)
    K key[KPT];
    uint32_t val[KPT];
    uint32_t rank[KPT];
    const uint32_t wbase = tile_base + warp * 32u * KPT + lane;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const uint32_t idx = wbase + 32u * j;
        const bool valid = idx < n;
        key[j] = valid ? kin[idx] : (K)0;
        if (HAS_VALS)
            val[j] = valid ? vin[idx] : 0u;
        else
            val[j] = idx;
    }

    // ---- stable rank within the warp, one digit group at a time
    uint32_t* wh = s_whist + warp * kRadixBins;
    const uint32_t lt_mask = lanemask_lt();
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        const bool valid = wbase + 32u * j < n;
        const uint32_t d = (uint32_t)(key[j] >> shift) & mask;
        uint32_t peers = __ballot_sync(kFullMask, valid);
#pragma unroll
        for (int b = 0; b < kRadixBits; ++b) {
            if (b < (int)bits) {
                const bool bit = (d >> b) & 1u;
                const uint32_t bb = __ballot_sync(kFullMask, bit);
                peers &= bit ? bb : ~bb;
            }
        }
        const uint32_t below = __popc(peers & lt_mask);
        const uint32_t leader = (uint32_t)(__ffs(peers) - 1) & 31u;
        uint32_t base = 0;
        if (valid && below == 0) {
            base = wh[d];
            wh[d] = base + __popc(peers);
        }
        base = __shfl_sync(kFullMask, base, leader);
        rank[j] = base + below;
        __syncwarp();
    }
    __syncthreads();

    // ---- per-digit tile count and per-warp exclusive offsets (thread = digit)
    uint32_t tile_cnt = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const uint32_t c = s_whist[w * kRadixBins + tid];
        s_whist[w * kRadixBins + tid] = tile_cnt;
        tile_cnt += c;
    }

    // ---- publish, then decoupled look-back for this digit
    uint32_t* lb = lookback + (size_t)tile * kRadixBins;
    uint32_t excl = 0;
    if (tid <= mask) {
        if (tile == 0) {
            excl = digit_base;
            atomicExch(lb + tid, kFlagInc | (excl + tile_cnt));
        } else {
            atomicExch(lb + tid, kFlagAgg | tile_cnt);
            int32_t pred = (int32_t)tile - 1;
            uint32_t polls = 0;
            while (pred >= 0) {
                const uint32_t v = ld_relaxed_u32(lookback + (size_t)pred * kRadixBins + tid);
                const uint32_t flag = v & ~kCountMask;
                if (flag == 0) {
                    if (++polls > kSpinLimit) {
                        set_error(err, NXB_DEVERR_SORT_LOOKBACK_TIMEOUT);
                        break;
                    }
                    if (polls > 64) __nanosleep(64);
                    continue;
                }
                excl += v & kCountMask;
                if (flag == kFlagInc) break;
                --pred;
            }
            atomicExch(lb + tid, kFlagInc | (excl + tile_cnt));
        }
    }
    s_global_start[tid] = excl;
    s_local_start[tid] = cta_exclusive_scan(tid <= mask ? tile_cnt : 0u, s_tmp);
    __syncthreads();

    // ---- reorder the tile by digit in shared memory
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        if (wbase + 32u * j < n) {
            const uint32_t d = (uint32_t)(key[j] >> shift) & mask;
            const uint32_t pos = s_local_start[d] + wh[d] + rank[j];
            s_keys[pos] = key[j];
            s_vals[pos] = val[j];
        }
    }
    __syncthreads();

    // ---- scatter runs of equal digits to consecutive global addresses
    const uint32_t tile_n = min((uint32_t)TILE, n - tile_base);
    for (uint32_t i = tid; i < tile_n; i += kThreads) {
        const K k = s_keys[i];
        const uint32_t d = (uint32_t)(k >> shift) & mask;
        const uint32_t g = s_global_start[d] + (i - s_local_start[d]);
        if (g < n) {  // always true unless a look-back wait expired
            kout[g] = k;
            vout[g] = s_vals[i];
        }
    }
}

// Dynamic shared memory above the 48 KB default (the 9-bit tables) and the
// carveout for four tiles per SM: shared memory, not L1.
template <typename Kern>
cudaError_t set_smem_attributes(Kern* kernel, size_t bytes) {
    cudaError_t r = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (!r) r = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    return r;
}

template <typename K, int RB>
cudaError_t configure_onesweep() {
    return once_per_device([] {
        constexpr size_t smem = dyn_smem_bytes<K, RB>();
        cudaError_t r;
        if constexpr (sizeof(K) == 4) {
            r = set_smem_attributes(onesweep32_kernel<true>, smem);
            if (!r) r = set_smem_attributes(onesweep32_kernel<false>, smem);
        } else {
            r = set_smem_attributes(onesweep_kernel<K, true, RB>, smem);
            if (!r) r = set_smem_attributes(onesweep_kernel<K, false, RB>, smem);
        }
        return r;
    });
}

template <typename K, int RB>
cudaError_t launch_pass_t(const K* kin, K* kout, const uint32_t* vin, uint32_t* vout, uint32_t n, uint32_t shift,
                          uint32_t bits, const uint32_t* hist, uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err,
                          cudaStream_t s) {
    constexpr size_t smem = dyn_smem_bytes<K, RB>();
    cudaError_t e = configure_onesweep<K, RB>();
    if (e != cudaSuccess) return e;
    const uint32_t tiles = (n + tile_keys<K>() - 1) / tile_keys<K>();
    if constexpr (sizeof(K) == 4) {
        static_assert(RB == kRadixBits, "32-bit keys take 8-bit digits");
        if (vin)
            onesweep32_kernel<true><<<tiles, kThreads, smem, s>>>(kin, kout, vin, vout, n, shift, bits, hist, lookback,
                                                                  tile_ctr, err);
        else
            onesweep32_kernel<false><<<tiles, kThreads, smem, s>>>(kin, kout, vin, vout, n, shift, bits, hist,
                                                                   lookback, tile_ctr, err);
    } else {
        if (vin)
            onesweep_kernel<K, true, RB><<<tiles, kThreads, smem, s>>>(kin, kout, vin, vout, n, shift, bits, hist,
                                                                      lookback, tile_ctr, err);
        else
            onesweep_kernel<K, false, RB><<<tiles, kThreads, smem, s>>>(kin, kout, vin, vout, n, shift, bits, hist,
                                                                       lookback, tile_ctr, err);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- bucket sort
// The pipeline sorts 63-bit Morton keys on bits [1,64) (Setup.cu:74-78) in
// two steps.  Four 9-bit onesweep passes sort them stably on bits [28,64);
// that groups the keys into buckets of equal key >> 28 (a cell of the Morton
// order 12 levels deep), which on meshes hold a handful of keys each.  Then
// bucket_sort_kernel sorts every bucket in place, stably, on bits [1,28)
// inside shared memory.  Keys equal on bits [1,64) keep their input order
// through both steps, so the result is exactly the stable sort of the whole
// range.  A bucket larger than kBucketCap is not sorted here: the kernel
// raises the overflow word and sort_fallback_kernel then sorts the whole
// array again with the plain eight 8-bit passes (a stable sort of an array
// in which equal keys are still in input order gives the same permutation).
constexpr uint32_t kBucketWindow = 2048;  // buckets owned by one CTA start in its window
constexpr uint32_t kBucketCap = 1024;     // largest bucket sorted in shared memory
constexpr uint32_t kBucketHalo = 32;      // positions past the window read with it
constexpr uint32_t kBucketSlots = kBucketWindow + kBucketCap;
constexpr uint32_t kBucketWords = kBucketSlots / 32;  // bucket-start bitmask
constexpr int kBucketThreads = 256;
static_assert(kBucketWindow % kBucketThreads == 0 && kBucketSlots % 32 == 0, "whole rows and words");
constexpr size_t kBucketSmem = (size_t)kBucketSlots * (8 + 4) + 4 * kBucketWords;

// One CTA per window of kBucketWindow positions: it owns the buckets that
// start in its window (the last one may run on past the window, into at
// most kBucketCap more positions), ranks each key in its bucket and writes
// the keys that move.  Bucket starts are one bit per position, from warp
// ballots: a warp's lanes hold 32 consecutive positions.  Other CTAs only
// read the top bits of keys outside their own buckets, which a permutation
// inside a bucket does not change, so the sort runs in place.
__global__ __launch_bounds__(kBucketThreads, 6) void bucket_sort_kernel(uint64_t* keys, uint32_t* vals, uint32_t n,
                                                                        uint32_t top_shift, uint32_t begin_bit,
                                                                        uint32_t* overflow) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t* s_key = reinterpret_cast<uint64_t*>(smem);
    uint32_t* s_val = reinterpret_cast<uint32_t*>(s_key + kBucketSlots);
    uint32_t* s_start = s_val + kBucketSlots;
    __shared__ uint32_t s_first, s_len, s_open;

    const uint32_t tid = threadIdx.x, lane = lane_id();
    const uint32_t w0 = blockIdx.x * kBucketWindow;
    const uint32_t rest = n - w0;
    const uint32_t wn = min(kBucketWindow, rest);
    const uint32_t avail = min(rest, kBucketWindow + kBucketHalo);  // positions read in the first sweep
    const uint32_t cmp_mask = (uint32_t)((1ull << (top_shift - begin_bit)) - 1ull);
    if (tid == 0) {
        s_first = kInvalid;
        s_open = 0;
    }
    for (uint32_t w = tid; w < kBucketWords; w += kBucketThreads) s_start[w] = 0;
    __syncthreads();
    // ---- keys and values of positions [0, avail), every load issued
    // before any is used, then the bucket-start bits
    constexpr int kRows = (kBucketWindow + kBucketHalo + kBucketThreads - 1) / kBucketThreads;
    {
        uint64_t k[kRows];
        uint32_t v[kRows];
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
            const uint32_t j = r * kBucketThreads + tid;
            if (j < avail) {
                k[r] = __ldcg(keys + w0 + j);
                v[r] = __ldcg(vals + w0 + j);
            }
        }
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
            const uint32_t j = r * kBucketThreads + tid;
            if (j < avail) {
                s_key[j] = k[r];
                s_val[j] = v[r];
            }
        }
    }
    const uint64_t before = tid == 0 && w0 > 0 ? __ldcg(keys + w0 - 1) >> top_shift : 0;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
        const uint32_t j = r * kBucketThreads + tid;
        bool start = false;
        if (j < avail) {
            const uint64_t top = s_key[j] >> top_shift;
            start = j == 0 ? w0 == 0 || before != top : (s_key[j - 1] >> top_shift) != top;
        }
        const uint32_t bits = __ballot_sync(kFullMask, start);
        if (lane == 0) s_start[j >> 5] = bits;
    }
    __syncthreads();
    // ---- the first bucket start of the window
    if (tid < kBucketWindow / 32) {
        const uint32_t b = s_start[tid];
        if (b) atomicMin(&s_first, tid * 32 + __ffs(b) - 1);
    }
    // ---- the end of the window's last bucket: the first start past the
    // window, searched further than the first sweep when it is not there
    if (tid < 32) {
        uint32_t len = rest;  // no start after the window: the last bucket ends with the keys
        if (wn == kBucketWindow && rest > kBucketWindow) {
            uint32_t found = kInvalid;
            for (uint32_t w = kBucketWindow / 32 + lane; w * 32 < avail; w += 32) {
                const uint32_t b = s_start[w];
                if (b) found = min(found, w * 32 + __ffs(b) - 1);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) found = min(found, __shfl_xor_sync(kFullMask, found, o));
            if (found != kInvalid) {
                len = found;
            } else if (avail < rest) {
                // the last bucket runs past the first sweep: read on, 32 keys
                // at a time, until its end, the end of the keys or the slots
                const uint64_t last = s_key[avail - 1] >> top_shift;
                uint32_t at = avail;
                for (;;) {
                    const uint32_t j = at + lane;
                    const bool in = j < rest && j < kBucketSlots;
                    uint64_t k = 0;
                    if (in) k = __ldcg(keys + w0 + j);
                    const uint32_t stop = __ballot_sync(kFullMask, !in || (k >> top_shift) != last);
                    const uint32_t take = stop ? (uint32_t)(__ffs(stop) - 1) : 32u;
                    if (lane < take) {
                        s_key[j] = k;
                        s_val[j] = __ldcg(vals + w0 + j);
                    }
                    at += take;
                    if (stop) break;
                }
                len = at;
                if (at >= kBucketSlots && at < rest && lane == 0 && (__ldcg(keys + w0 + at) >> top_shift) == last)
                    s_open = 1;
            } else {
                len = avail;
            }
        }
        if (lane == 0) s_len = len;
    }
    __syncthreads();
    const uint32_t s0 = s_first, len = s_len;
    if (s0 == kInvalid) return;  // the window lies inside a bucket that started earlier
    if (s_open) {                // its last bucket is larger than the slots: the fallback sorts everything
        if (tid == 0) atomicOr(overflow, 1u);
        return;
    }
    // ---- rank of each key in its bucket: keys below it, and equal keys before it
    const uint32_t* s_lo = reinterpret_cast<const uint32_t*>(s_key);  // low words of the keys
    const uint32_t last_word = (len - 1) >> 5;
    bool over = false;
    for (uint32_t j = s0 + tid; j < len; j += kBucketThreads) {
        uint32_t w = j >> 5;
        const uint32_t word = s_start[w];
        // a bucket of one key (a start followed by a start): nothing moves
        if ((word >> (j & 31)) & 1u) {
            const uint32_t nxt = j + 1;
            if (nxt >= len || ((nxt & 31) ? (word >> (nxt & 31)) & 1u : s_start[w + 1] & 1u)) continue;
        }
        // bucket bounds from the start bits: bs = the last start <= j,
        // be = the first start > j (or len)
        const uint32_t upto = 0xFFFFFFFFu >> (31 - (j & 31));  // bits <= j within the word
        uint32_t m = word & upto;
        while (m == 0) m = s_start[--w];  // s0 <= j is a start: the walk ends
        const uint32_t bs = w * 32 + 31 - __clz(m);
        w = j >> 5;
        m = s_start[w] & ~upto;
        while (m == 0 && w < last_word) m = s_start[++w];
        const uint32_t be = m ? min(w * 32 + __ffs(m) - 1, len) : len;
        if (be - bs > kBucketCap) {
            over = true;
            continue;
        }
        if (be - bs == 1) continue;
        const uint32_t c = (s_lo[2 * j] >> begin_bit) & cmp_mask;
        uint32_t r = 0;
        for (uint32_t i = bs; i < be; ++i) {
            const uint32_t ci = (s_lo[2 * i] >> begin_bit) & cmp_mask;
            r += (ci < c || (ci == c && i < j)) ? 1u : 0u;
        }
        const uint32_t dst = bs + r;
        if (dst != j) {
            keys[w0 + dst] = s_key[j];
            vals[w0 + dst] = s_val[j];
        }
    }
    if (over) atomicOr(overflow, 1u);
}

// ---------------------------------------------------------------- fallback
// The whole-array re-sort of the bucket overflow case as ONE persistent
// launch that does nothing when the overflow word is clear.  Its work is a
// sequence of tickets claimed in order from one counter: clearing the
// look-back words and histograms, counting the digits of every pass, then
// the tiles of pass 0, 1, ...  A ticket whose stage needs the previous
// stage complete waits (bounded) on that stage's done counter; every
// ticket it waits on was claimed earlier by a running CTA, which only
// waits on tickets claimed before its own, so the waits always end.
constexpr uint32_t kFbZeroWords = 1u << 16;  // look-back words cleared per ticket
constexpr uint32_t kFbHistKeys = 1u << 14;   // keys counted per ticket

template <typename K>
__global__ __launch_bounds__(kThreads, 4) void sort_fallback_kernel(K* ka, K* kb, uint32_t* va, uint32_t* vb,
                                                                   uint32_t n, const uint32_t* overflow,
                                                                   SortFallback f, uint32_t* err) {
    if (ld_relaxed_u32(overflow) == 0) return;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_delta[kRadixBins];
    __shared__ uint16_t s_local[kRadixBins];
    __shared__ uint32_t s_tmp[kWarps];
    __shared__ uint32_t s_ticket, s_ok;
    uint32_t* s_whist = reinterpret_cast<uint32_t*>(smem + (size_t)tile_keys<K>() * (sizeof(K) + sizeof(uint32_t)));
    const uint32_t passes = (uint32_t)f.plan.passes;
    const uint32_t total = f.zero_tickets + f.hist_tickets + passes * f.tiles;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_ticket = atomicAdd(f.ticket, 1u);
        for (int i = threadIdx.x; i < kWarps * kRadixBins; i += kThreads) s_whist[i] = 0;
        __syncthreads();
        const uint32_t t = s_ticket;
        if (t >= total) return;
        uint32_t stage, local, wait_stage = 0, wait_for = 0;
        if (t < f.zero_tickets) {
            stage = 0;
            local = t;
        } else if (t < f.zero_tickets + f.hist_tickets) {
            stage = 1;
            local = t - f.zero_tickets;
            wait_stage = 0;
            wait_for = f.zero_tickets;
        } else {
            const uint32_t q = t - f.zero_tickets - f.hist_tickets;
            const uint32_t p = q / f.tiles;
            stage = 2 + p;
            local = q - p * f.tiles;
            wait_stage = stage - 1;
            wait_for = p == 0 ? f.hist_tickets : f.tiles;
        }
        if (threadIdx.x == 0) {
            uint32_t ok = 1, polls = 0;
            if (stage > 0) {
                while (ld_acquire_u32(f.done + wait_stage) < wait_for) {
                    if (++polls > kSpinLimit) {
                        set_error(err, NXB_DEVERR_SORT_LOOKBACK_TIMEOUT);
                        ok = 0;
                        break;
                    }
                    __nanosleep(polls > 64 ? 256 : 32);
                }
            }
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) return;
        if (stage == 0) {
            const size_t words = f.lookback_per_pass * passes;
            const size_t b = (size_t)local * kFbZeroWords, e = min(words, b + kFbZeroWords);
            for (size_t w = b + threadIdx.x; w < e; w += kThreads) f.lookback[w] = 0;
            if (local == 0)
                for (uint32_t i = threadIdx.x; i < passes * kRadixBins; i += kThreads) f.hist[i] = 0;
        } else if (stage == 1) {
            const uint32_t b = local * kFbHistKeys, e = min(n, b + kFbHistKeys);
            for (uint32_t i = b + threadIdx.x; i < e; i += kThreads) {
                const K k = __ldcg(ka + i);
                for (uint32_t p = 0; p < passes; ++p)
                    atomicAdd(&s_whist[p * kRadixBins + ((uint32_t)(k >> f.plan.shift[p]) & ((1u << f.plan.bits[p]) - 1u))],
                              1u);
            }
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < passes * kRadixBins; i += kThreads)
                if (s_whist[i]) atomicAdd(f.hist + i, s_whist[i]);
        } else {
            const uint32_t p = stage - 2;
            const bool even = (p & 1u) == 0;
            sort_tile<K, true, kRadixBits, true>(local, even ? ka : kb, even ? kb : ka, even ? va : vb, even ? vb : va,
                                                 n, f.plan.shift[p], f.plan.bits[p], f.hist + p * kRadixBins,
                                                 f.lookback + (size_t)p * f.lookback_per_pass, err, smem, s_delta,
                                                 s_local, s_tmp);
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd(f.done + stage, 1u);
    }
}

}  // namespace

// Bounded-wait check: one CTA claims tile 1 of a two-tile sort while tile 0
// is never processed, so its look-back poll expires.  Returns the error word.
cudaError_t run_sort_stall_probe(uint32_t* err_out) {
    const uint32_t n = 2u * tile_keys<uint32_t>();
    const size_t tiles_words = 2u * kRadixBins;
    unsigned char* buf = nullptr;
    const size_t bytes = 4ull * (3ull * n + kRadixBins + tiles_words + 2);
    cudaError_t e = cudaMalloc(&buf, bytes);
    if (e) return e;
    uint32_t* keys = (uint32_t*)buf;
    uint32_t* kout = keys + n;
    uint32_t* vout = kout + n;
    uint32_t* hist = vout + n;
    uint32_t* lookback = hist + kRadixBins;
    uint32_t* ctr = lookback + tiles_words;
    uint32_t* err = ctr + 1;
    e = cudaMemset(buf, 0, bytes);
    const uint32_t one = 1;
    if (!e) e = cudaMemcpy(ctr, &one, 4, cudaMemcpyHostToDevice);
    constexpr size_t smem = dyn_smem_bytes<uint32_t, kRadixBits>();
    if (!e) e = configure_onesweep<uint32_t, kRadixBits>();
    if (!e) {
        onesweep32_kernel<false><<<1, kThreads, smem>>>(keys, kout, nullptr, vout, n, 0, 8, hist, lookback, ctr, err);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(err_out, err, 4, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    return e;
}

SortPlan make_sort_plan(uint32_t begin_bit, uint32_t end_bit, uint32_t digit_bits) {
    SortPlan p{};
    digit_bits = std::max(1u, std::min<uint32_t>(digit_bits, kMaxRadixBits));
    for (uint32_t b = begin_bit; b < end_bit && p.passes < kMaxSortPasses; b += digit_bits) {
        p.shift[p.passes] = b;
        p.bits[p.passes] = std::min<uint32_t>(digit_bits, end_bit - b);
        p.passes++;
    }
    return p;
}

SortPlan hybrid63_top_plan() { return make_sort_plan(kHybridTopShift, 64, kMaxRadixBits); }

size_t sort_lookback_words(uint32_t n, uint32_t key_bytes, int passes, uint32_t bins) {
    uint32_t tk = key_bytes == 4 ? tile_keys<uint32_t>() : tile_keys<uint64_t>();
    size_t tiles = (n + tk - 1) / tk;
    return tiles * bins * (size_t)passes;
}

cudaError_t launch_sort_pass(uint32_t key_bytes, const void* keys_in, void* keys_out, const uint32_t* vals_in,
                             uint32_t* vals_out, uint32_t n, uint32_t shift, uint32_t bits, const uint32_t* hist,
                             uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err, cudaStream_t s) {
    if (key_bytes == 4) {
        if (bits > kRadixBits) return cudaErrorInvalidValue;
        return launch_pass_t<uint32_t, kRadixBits>((const uint32_t*)keys_in, (uint32_t*)keys_out, vals_in, vals_out, n,
                                                   shift, bits, hist, lookback, tile_ctr, err, s);
    }
    if (bits > kRadixBits)
        return launch_pass_t<uint64_t, kMaxRadixBits>((const uint64_t*)keys_in, (uint64_t*)keys_out, vals_in, vals_out,
                                                      n, shift, bits, hist, lookback, tile_ctr, err, s);
    return launch_pass_t<uint64_t, kRadixBits>((const uint64_t*)keys_in, (uint64_t*)keys_out, vals_in, vals_out, n,
                                               shift, bits, hist, lookback, tile_ctr, err, s);
}

cudaError_t launch_sort63_hybrid(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_a, uint64_t* keys_b,
                                 uint32_t* vals_a, uint32_t* vals_b, uint32_t n, const uint32_t* top_hist,
                                 uint32_t* lookback, uint32_t* tile_ctr, uint32_t* overflow, uint32_t* fb_hist,
                                 uint32_t* fb_ticket, uint32_t* fb_done, uint32_t* err, cudaStream_t s) {
    const SortPlan top = hybrid63_top_plan();
    constexpr uint32_t kTopBins = 1u << kMaxRadixBits;
    const size_t top_words = sort_lookback_words(n, 8, 1, kTopBins);
    // even pass count: the keys end in A
    for (int p = 0; p < top.passes; ++p) {
        const bool even = (p % 2) == 0;
        const uint64_t* kin = p == 0 && keys_in ? keys_in : (even ? keys_a : keys_b);
        const uint32_t* vin = p == 0 ? vals_in : (even ? vals_a : vals_b);
        cudaError_t e = launch_sort_pass(8, kin, even ? keys_b : keys_a, vin, even ? vals_b : vals_a, n,
                                         top.shift[p], top.bits[p], top_hist + p * kTopBins, lookback + p * top_words,
                                         tile_ctr + p, err, s);
        if (e != cudaSuccess) return e;
    }
    {
        cudaError_t attr = once_per_device([] { return set_smem_attributes(bucket_sort_kernel, kBucketSmem); });
        if (attr != cudaSuccess) return attr;
        const uint32_t windows = (n + kBucketWindow - 1) / kBucketWindow;
        bucket_sort_kernel<<<windows, kBucketThreads, kBucketSmem, s>>>(keys_a, vals_a, n, kHybridTopShift, 1,
                                                                         overflow);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    SortFallback f{};
    f.plan = make_sort_plan(1, 64);
    f.tiles = (n + tile_keys<uint64_t>() - 1) / tile_keys<uint64_t>();
    f.lookback_per_pass = sort_lookback_words(n, 8, 1, kRadixBins);
    f.zero_tickets = (uint32_t)((f.lookback_per_pass * f.plan.passes + kFbZeroWords - 1) / kFbZeroWords);
    f.hist_tickets = (n + kFbHistKeys - 1) / kFbHistKeys;
    f.lookback = lookback;
    f.hist = fb_hist;
    f.ticket = fb_ticket;
    f.done = fb_done;
    constexpr size_t smem = dyn_smem_bytes<uint64_t, kRadixBits>();
    cudaError_t e = once_per_device([] { return set_smem_attributes(sort_fallback_kernel<uint64_t>, smem); });
    if (e != cudaSuccess) return e;
    const uint32_t total = f.zero_tickets + f.hist_tickets + (uint32_t)f.plan.passes * f.tiles;
    const uint32_t grid = std::max(1u, std::min(total, (uint32_t)device_info().sms * 4u));
    sort_fallback_kernel<uint64_t><<<grid, kThreads, smem, s>>>(keys_a, keys_b, vals_a, vals_b, n, overflow, f, err);
    return cudaGetLastError();
}

}  // namespace nxb

// ---------------------------------------------------------------------------
// Radix sort with library-owned scratch (nxb_stage_radix_sort_noalloc).
//
// Some callers cannot hand this library a scratch buffer or let it allocate
// one: a renderer that rebuilds BVHs inside its frame loop on a real-time
// thread (cudaMalloc and cudaFree synchronise the whole device, which
// stalls every other stream of the frame), an engine whose device memory is
// owned by its own sub-allocator or budget, or a plugin that runs in a host
// process it does not control.  For them the sort's scratch lives in a
// fixed device array of this file, which every GPU that loads the library
// keeps until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocAlign = 256;
constexpr size_t align_na(size_t x) { return (x + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }
// 8-bit digits: at most 8 passes over a 64-bit key
constexpr int kNoAllocPasses = 8;
constexpr size_t kNoAllocHist = align_na(sizeof(uint32_t) * kNoAllocPasses * nxb::kRadixBins);
constexpr size_t kNoAllocCtr = align_na(sizeof(uint32_t) * kNoAllocPasses);
// one look-back word per (tile, digit, pass); the 64-bit tile is the smaller one
constexpr size_t kNoAllocTiles =
    (NXB_NOALLOC_SORT_MAX_COUNT + nxb::tile_keys<uint64_t>() - 1) / nxb::tile_keys<uint64_t>();
constexpr size_t kNoAllocLookback = align_na(4ull * kNoAllocTiles * nxb::kRadixBins * kNoAllocPasses);
constexpr size_t kNoAllocKeys = align_na(8ull * NXB_NOALLOC_SORT_MAX_COUNT);
constexpr size_t kNoAllocVals = align_na(4ull * NXB_NOALLOC_SORT_MAX_COUNT);
constexpr size_t kNoAllocZeroed = kNoAllocHist + kNoAllocCtr + kNoAllocLookback;
constexpr size_t kNoAllocBytes = kNoAllocZeroed + kNoAllocKeys + kNoAllocVals;

// The scratch itself (about 3.7 MB).  Host code must not pass this name to a
// kernel: on the host it is only a stand-in for the symbol, not a device
// address.  noalloc_scratch() looks up the real address per device.
static __device__ __align__(256) unsigned char g_noalloc_sort_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (with that device current) on its first call and kept for the
// life of the process (a cudaDeviceReset would invalidate it; the header
// tells callers not to reset a device they used this entry point on).
cudaError_t noalloc_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" nxb_status nxb_stage_radix_sort_noalloc(uint32_t key_bytes, const void* d_keys_in, void* d_keys_out,
                                                   const uint32_t* d_vals_in, uint32_t* d_vals_out, uint32_t count,
                                                   uint32_t begin_bit, uint32_t end_bit, uint32_t* d_error_word,
                                                   struct CUstream_st* stream) {
    using namespace nxb;
    if (key_bytes != 4 && key_bytes != 8) return NXB_ERR_UNSUPPORTED;
    if (begin_bit >= end_bit || end_bit > key_bytes * 8) return NXB_ERR_INVALID_ARGUMENT;
    if (!d_keys_in || !d_keys_out || !d_vals_out || count == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (count > NXB_NOALLOC_SORT_MAX_COUNT) return NXB_ERR_UNSUPPORTED;  // larger sorts: nxb_stage_radix_sort
    unsigned char* base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    if (e != cudaSuccess) return record_cuda_error(e);
    const SortPlan plan = make_sort_plan(begin_bit, end_bit);
    uint32_t* hist = reinterpret_cast<uint32_t*>(base);
    uint32_t* ctr = reinterpret_cast<uint32_t*>(base + kNoAllocHist);
    uint32_t* lookback = reinterpret_cast<uint32_t*>(base + kNoAllocHist + kNoAllocCtr);
    void* keys_tmp = base + kNoAllocZeroed;
    uint32_t* vals_tmp = reinterpret_cast<uint32_t*>(base + kNoAllocZeroed + kNoAllocKeys);
    // the histograms, tile counters and look-back flags of the previous call
    // are still there: clear them
    e = cudaMemsetAsync(base, 0, kNoAllocZeroed, stream);
    if (e == cudaSuccess) e = launch_sort_histogram(key_bytes, d_keys_in, count, plan, hist, stream);
    const size_t per_pass = sort_lookback_words(count, key_bytes, 1);
    const void* kin = d_keys_in;
    const uint32_t* vin = d_vals_in;
    for (int p = 0; p < plan.passes && e == cudaSuccess; ++p) {
        const bool last_is_out = ((plan.passes - 1 - p) % 2) == 0;
        void* kout = last_is_out ? d_keys_out : keys_tmp;
        uint32_t* vout = last_is_out ? d_vals_out : vals_tmp;
        e = launch_sort_pass(key_bytes, kin, kout, vin, vout, count, plan.shift[p], plan.bits[p],
                             hist + p * kRadixBins, lookback + p * per_pass, ctr + p, d_error_word, stream);
        kin = kout;
        vin = vout;
    }
    return e == cudaSuccess ? NXB_OK : record_cuda_error(e);
}
