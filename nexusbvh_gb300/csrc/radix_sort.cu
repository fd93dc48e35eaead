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
__global__ __launch_bounds__(kThreads, 4) void onesweep_kernel(const K* __restrict__ kin, K* __restrict__ kout,
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

template <typename K>
cudaError_t launch_pass_t(const K* kin, K* kout, const uint32_t* vin, uint32_t* vout, uint32_t n, uint32_t shift,
                          uint32_t bits, const uint32_t* hist, uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err,
                          cudaStream_t s) {
    constexpr size_t smem = dyn_smem_bytes<K>();
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(onesweep_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(onesweep_kernel<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        // four tiles per SM: shared memory, not L1, gets the carveout
        cudaFuncSetAttribute(onesweep_kernel<K, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaFuncSetAttribute(onesweep_kernel<K, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
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

SortPlan make_sort_plan(uint32_t begin_bit, uint32_t end_bit, uint32_t digit_bits) {
    SortPlan p{};
    digit_bits = std::max(1u, std::min<uint32_t>(digit_bits, kRadixBits));
    for (uint32_t b = begin_bit; b < end_bit && p.passes < kMaxSortPasses; b += digit_bits) {
        p.shift[p.passes] = b;
        p.bits[p.passes] = std::min<uint32_t>(digit_bits, end_bit - b);
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
constexpr size_t kNoAllocHist = align_na(sizeof(uint32_t) * nxb::kMaxSortPasses * nxb::kRadixBins);
constexpr size_t kNoAllocCtr = align_na(sizeof(uint32_t) * nxb::kMaxSortPasses);
// one look-back word per (tile, digit, pass); the 64-bit tile is the smaller one
constexpr size_t kNoAllocTiles =
    (NXB_NOALLOC_SORT_MAX_COUNT + nxb::tile_keys<uint64_t>() - 1) / nxb::tile_keys<uint64_t>();
constexpr size_t kNoAllocLookback = align_na(4ull * kNoAllocTiles * nxb::kRadixBins * nxb::kMaxSortPasses);
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
// device (with that device current) on its first call.
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
