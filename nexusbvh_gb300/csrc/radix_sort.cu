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

template <typename K>
__host__ __device__ constexpr size_t dyn_smem_bytes() {
    return (size_t)tile_keys<K>() * (sizeof(K) + sizeof(uint32_t)) + (size_t)kWarps * kRadixBins * sizeof(uint32_t);
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

template <typename K, bool HAS_VALS>
__global__ __launch_bounds__(kThreads) void onesweep_kernel(const K* __restrict__ kin, K* __restrict__ kout,
                                                            const uint32_t* __restrict__ vin,
                                                            uint32_t* __restrict__ vout, uint32_t n, uint32_t shift,
                                                            uint32_t bits, const uint32_t* __restrict__ hist,
                                                            uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err) {
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
    // global start of each digit: exclusive scan of this pass's histogram
    const uint32_t digit_base = cta_exclusive_scan(tid <= mask ? hist[tid] : 0u, s_tmp);
    const uint32_t tile = s_tile;
    const uint32_t tile_base = tile * (uint32_t)TILE;
    if (tile_base >= n) return;  // only reachable when a launch claims more tiles than exist

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

template <typename K>
cudaError_t launch_pass_t(const K* kin, K* kout, const uint32_t* vin, uint32_t* vout, uint32_t n, uint32_t shift,
                          uint32_t bits, const uint32_t* hist, uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err,
                          cudaStream_t s) {
    constexpr size_t smem = dyn_smem_bytes<K>();
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(onesweep_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(onesweep_kernel<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    const uint32_t tiles = (n + tile_keys<K>() - 1) / tile_keys<K>();
    if (vin)
        onesweep_kernel<K, true><<<tiles, kThreads, smem, s>>>(kin, kout, vin, vout, n, shift, bits, hist, lookback,
                                                              tile_ctr, err);
    else
        onesweep_kernel<K, false><<<tiles, kThreads, smem, s>>>(kin, kout, vin, vout, n, shift, bits, hist, lookback,
                                                               tile_ctr, err);
    return cudaGetLastError();
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
    constexpr size_t smem = dyn_smem_bytes<uint32_t>();
    if (!e) e = cudaFuncSetAttribute(onesweep_kernel<uint32_t, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
    if (!e) {
        onesweep_kernel<uint32_t, false><<<1, kThreads, smem>>>(keys, kout, nullptr, vout, n, 0, 8, hist, lookback,
                                                                 ctr, err);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(err_out, err, 4, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    return e;
}

SortPlan make_sort_plan(uint32_t begin_bit, uint32_t end_bit) {
    SortPlan p{};
    for (uint32_t b = begin_bit; b < end_bit && p.passes < kMaxSortPasses; b += kRadixBits) {
        p.shift[p.passes] = b;
        p.bits[p.passes] = std::min<uint32_t>(kRadixBits, end_bit - b);
        p.passes++;
    }
    return p;
}

size_t sort_lookback_words(uint32_t n, uint32_t key_bytes, int passes) {
    uint32_t tk = key_bytes == 4 ? tile_keys<uint32_t>() : tile_keys<uint64_t>();
    size_t tiles = (n + tk - 1) / tk;
    return tiles * kRadixBins * (size_t)passes;
}

cudaError_t launch_sort_pass(uint32_t key_bytes, const void* keys_in, void* keys_out, const uint32_t* vals_in,
                             uint32_t* vals_out, uint32_t n, uint32_t shift, uint32_t bits, const uint32_t* hist,
                             uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err, cudaStream_t s) {
    if (key_bytes == 4)
        return launch_pass_t<uint32_t>((const uint32_t*)keys_in, (uint32_t*)keys_out, vals_in, vals_out, n, shift,
                                       bits, hist, lookback, tile_ctr, err, s);
    return launch_pass_t<uint64_t>((const uint64_t*)keys_in, (uint64_t*)keys_out, vals_in, vals_out, n, shift, bits,
                                   hist, lookback, tile_ctr, err, s);
}

}  // namespace nxb
