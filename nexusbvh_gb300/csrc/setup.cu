// setup.cu - stage 1 (scene bounds + leaf write) and stage 2 (Morton codes).
//
// Stage 1 replaces ComputeSceneBoundsKernel (NexusBVH/src/Cuda/Setup.cu:12-39).
// The reference reads one 36-byte triangle per thread (strided, 9 scalar
// loads) and folds the scene box with 6 float CAS loops per warp.  Here a
// 256-thread CTA stages a tile of 256 primitives through shared memory with
// coalesced 16-byte loads, writes the 32-byte leaves, and reduces the scene
// box to one set of 6 integer atomicMax per CTA (floats mapped to a
// monotone uint32 order), with the grid sized to the SM count.
//
// Stage 2 replaces ComputeMortonCodesKernel (Setup.cu:42-59) and fuses the
// work the host builder does around it: the digit histograms of every radix
// sort pass (onesweep's up-front histogram), the parentIdx = INVALID memset
// (BVHBuilder.cpp:23), clearing the sort look-back flags and seeding the
// H-PLOC and BVH8 counters (BVHBuilder.cpp:24,193-202).
#include <algorithm>

#include "pipeline.h"

namespace nxb {
namespace {

constexpr int kThreads = 256;

template <int FLOATS>
__global__ __launch_bounds__(kThreads) void scene_bounds_kernel(const float* __restrict__ prims, uint32_t n,
                                                                Node2* __restrict__ nodes, uint32_t* scene_ord,
                                                                bool aligned16) {
    __shared__ __align__(16) float tile[kThreads * FLOATS];
    __shared__ float red[kThreads / 32][6];
    Box acc;
    acc.mn = make_float3(3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f);
    acc.mx = make_float3(-3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f);
    const uint32_t tiles = (n + kThreads - 1) / kThreads;
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint32_t first = t * kThreads;
        const uint32_t cnt = min((uint32_t)kThreads, n - first);
        const float* src = prims + (size_t)first * FLOATS;
        __syncthreads();
        if (cnt == kThreads && aligned16) {
            constexpr int V = kThreads * FLOATS / 4;
            const float4* s4 = reinterpret_cast<const float4*>(src);
            float4* d4 = reinterpret_cast<float4*>(tile);
#pragma unroll
            for (int v = threadIdx.x; v < V; v += kThreads) d4[v] = __ldcs(s4 + v);
        } else {
            for (uint32_t v = threadIdx.x; v < cnt * FLOATS; v += kThreads) tile[v] = __ldcs(src + v);
        }
        __syncthreads();
        if (threadIdx.x < cnt) {
            const float* f = tile + threadIdx.x * FLOATS;
            Box b;
            if (FLOATS == 9) {
                // AABB(v0, v1, v2): min(v0, min(v1, v2)) (NXB AABB.h:16-20)
                float3 v0 = make_float3(f[0], f[1], f[2]);
                float3 v1 = make_float3(f[3], f[4], f[5]);
                float3 v2 = make_float3(f[6], f[7], f[8]);
                b.mn = fmin3(v0, fmin3(v1, v2));
                b.mx = fmax3(v0, fmax3(v1, v2));
            } else {
                b.mn = make_float3(f[0], f[1], f[2]);
                b.mx = make_float3(f[3], f[4], f[5]);
            }
            store_node(nodes, first + threadIdx.x, b, kInvalid, first + threadIdx.x);
            grow(acc, b);
        }
    }
    // CTA reduction: warp shuffles, then one warp over the partials.
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Box other;
        other.mn.x = __shfl_down_sync(kFullMask, acc.mn.x, o);
        other.mn.y = __shfl_down_sync(kFullMask, acc.mn.y, o);
        other.mn.z = __shfl_down_sync(kFullMask, acc.mn.z, o);
        other.mx.x = __shfl_down_sync(kFullMask, acc.mx.x, o);
        other.mx.y = __shfl_down_sync(kFullMask, acc.mx.y, o);
        other.mx.z = __shfl_down_sync(kFullMask, acc.mx.z, o);
        grow(acc, other);
    }
    const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
    if (lane == 0) {
        red[warp][0] = acc.mn.x;
        red[warp][1] = acc.mn.y;
        red[warp][2] = acc.mn.z;
        red[warp][3] = acc.mx.x;
        red[warp][4] = acc.mx.y;
        red[warp][5] = acc.mx.z;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int a = threadIdx.x;
        float v = red[0][a];
        for (int w = 1; w < kThreads / 32; ++w) v = a < 3 ? fminf(v, red[w][a]) : fmaxf(v, red[w][a]);
        atomicMax(&scene_ord[a], a < 3 ? ~f2ord(v) : f2ord(v));
    }
}

struct PassDigits {
    int passes;
    uint32_t shift[kMaxSortPasses];
    uint32_t mask[kMaxSortPasses];
};

// Warp-aggregated shared-memory histogram update: keys of a warp usually
// share their high digits, so a uniform digit is added once.
__device__ __forceinline__ void hist_add(uint32_t* h, uint32_t d, bool valid) {
    const uint32_t vmask = __ballot_sync(kFullMask, valid);
    const uint32_t d0 = __shfl_sync(kFullMask, d, 0);
    if (__all_sync(kFullMask, !valid || d == d0)) {
        if (lane_id() == 0 && vmask) atomicAdd(&h[d0], (uint32_t)__popc(vmask));
    } else if (valid) {
        atomicAdd(&h[d], 1u);
    }
}

template <typename K>
__device__ __forceinline__ K morton_key(const Box& b, float3 smin, float3 smax) {
    // centroid = (bMin + bMax) * 0.5f (AABB.h:40-43); normalised by the
    // scene box (Setup.cu:52-54); quantised by truncation (BuilderUtils.h:234-253).
    float cx = (b.mn.x + b.mx.x) * 0.5f;
    float cy = (b.mn.y + b.mx.y) * 0.5f;
    float cz = (b.mn.z + b.mx.z) * 0.5f;
    float tx = (cx - smin.x) / (smax.x - smin.x);
    float ty = (cy - smin.y) / (smax.y - smin.y);
    float tz = (cz - smin.z) / (smax.z - smin.z);
    if constexpr (sizeof(K) == 4) {
        uint32_t x = tx * 0x3ff;
        uint32_t y = ty * 0x3ff;
        uint32_t z = tz * 0x3ff;
        return spread3_10(x) | spread3_10(y) << 1 | spread3_10(z) << 2;
    } else {
        uint32_t x = tx * 0x1fffff;
        uint32_t y = ty * 0x1fffff;
        uint32_t z = tz * 0x1fffff;
        return spread3_21(x) | spread3_21(y) << 1 | spread3_21(z) << 2;
    }
}

struct MortonArgs {
    PassDigits pd;
    uint32_t* cluster_idx;
    uint32_t* parent;
    uint4* zero_ptr;
    size_t zero_vec4;
    uint4* ones_ptr;
    size_t ones_vec4;
    nxb_aabb* scene_out;
    int seed;
};

// PASSES > 0: the pass count of the plan, known at compile time (4 for
// 30-bit keys, 4 for the 9-bit top passes of 63-bit keys), so the histogram
// loop unrolls.  BINS: digits per pass (256, or 512 for 9-bit digits); the
// histograms are laid out pass after pass, BINS words each.
template <typename K, bool HIST, int PASSES = 0, int BINS = kRadixBins>
__global__ __launch_bounds__(kThreads) void morton_kernel(const Node2* __restrict__ nodes, uint32_t n, Control* ctrl,
                                                          K* __restrict__ keys, MortonArgs a) {
    static_assert(PASSES * BINS <= kMaxSortPasses * kRadixBins, "histograms fit the control block");
    __shared__ float s_scene[6];
    __shared__ uint32_t s_hist[HIST ? kMaxSortPasses * kRadixBins : 1];
    if (threadIdx.x < 6) {
        uint32_t o = ctrl->scene_ord[threadIdx.x];
        s_scene[threadIdx.x] = ord2f(threadIdx.x < 3 ? ~o : o);
    }
    if (HIST)
        for (int i = threadIdx.x; i < a.pd.passes * BINS; i += kThreads) s_hist[i] = 0;
    __syncthreads();
    const float3 smin = make_float3(s_scene[0], s_scene[1], s_scene[2]);
    const float3 smax = make_float3(s_scene[3], s_scene[4], s_scene[5]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.seed) {
            ctrl->cluster_count = n;
            ctrl->parent_of_last = kInvalid;
        }
        if (a.scene_out) {
            a.scene_out->bmin[0] = smin.x;
            a.scene_out->bmin[1] = smin.y;
            a.scene_out->bmin[2] = smin.z;
            a.scene_out->bmax[0] = smax.x;
            a.scene_out->bmax[1] = smax.y;
            a.scene_out->bmax[2] = smax.z;
        }
    }
    const uint32_t lane = lane_id();
    const uint32_t stride = gridDim.x * kThreads;
    for (uint32_t base = blockIdx.x * kThreads + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t i = base + lane;
        const bool valid = i < n;
        K key = 0;
        if (valid) {
            const float4* p = reinterpret_cast<const float4*>(nodes + i);
            float4 lo = __ldcs(p);
            float2 hi = __ldcs(reinterpret_cast<const float2*>(p + 1));
            Box b;
            b.mn = make_float3(lo.x, lo.y, lo.z);
            b.mx = make_float3(lo.w, hi.x, hi.y);
            key = morton_key<K>(b, smin, smax);
            keys[i] = key;
            if (a.cluster_idx) a.cluster_idx[i] = i;
            if (a.parent) a.parent[i] = kInvalid;
        }
        if (HIST) {
            if constexpr (PASSES > 0) {
#pragma unroll
                for (int p = 0; p < PASSES; ++p) {
                    const uint32_t d = (uint32_t)(key >> a.pd.shift[p]) & a.pd.mask[p];
                    if (p < PASSES / 2) {
                        // low digits: neighbouring keys rarely share them,
                        // so the warp-uniform test seldom pays for itself
                        if (valid) atomicAdd(&s_hist[p * BINS + d], 1u);
                    } else {
                        hist_add(s_hist + p * BINS, d, valid);
                    }
                }
            } else {
#pragma unroll 1
                for (int p = 0; p < a.pd.passes; ++p) {
                    uint32_t d = (uint32_t)(key >> a.pd.shift[p]) & a.pd.mask[p];
                    hist_add(s_hist + p * BINS, d, valid);
                }
            }
        }
    }
    for (size_t w = (size_t)blockIdx.x * kThreads + threadIdx.x; w < a.zero_vec4; w += stride)
        a.zero_ptr[w] = make_uint4(0, 0, 0, 0);
    for (size_t w = (size_t)blockIdx.x * kThreads + threadIdx.x; w < a.ones_vec4; w += stride)
        a.ones_ptr[w] = make_uint4(kInvalid, kInvalid, kInvalid, kInvalid);
    if (HIST) {
        __syncthreads();
        for (int i = threadIdx.x; i < a.pd.passes * BINS; i += kThreads)
            if (s_hist[i]) atomicAdd(&ctrl->hist[0][0] + i, s_hist[i]);
    }
}

template <typename K>
__global__ __launch_bounds__(kThreads) void morton_scene_kernel(const Node2* __restrict__ nodes, uint32_t n,
                                                                const nxb_aabb* scene, K* __restrict__ keys,
                                                                uint32_t* cluster_idx) {
    const float3 smin = make_float3(scene->bmin[0], scene->bmin[1], scene->bmin[2]);
    const float3 smax = make_float3(scene->bmax[0], scene->bmax[1], scene->bmax[2]);
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
        keys[i] = morton_key<K>(load_box(nodes, i), smin, smax);
        if (cluster_idx) cluster_idx[i] = i;
    }
}

// bins: histogram words per pass (1 << the plan's widest digit).
template <typename K>
__global__ __launch_bounds__(kThreads) void sort_histogram_kernel(const K* __restrict__ keys, uint32_t n,
                                                                  PassDigits pd, uint32_t bins, uint32_t* hist) {
    __shared__ uint32_t s_hist[kMaxSortPasses * kRadixBins];
    for (int i = threadIdx.x; i < pd.passes * bins; i += kThreads) s_hist[i] = 0;
    __syncthreads();
    const uint32_t lane = lane_id();
    for (uint32_t base = blockIdx.x * kThreads + (threadIdx.x & ~31u); base < n; base += gridDim.x * kThreads) {
        const uint32_t i = base + lane;
        const bool valid = i < n;
        K key = valid ? keys[i] : 0;
#pragma unroll 1
        for (int p = 0; p < pd.passes; ++p) hist_add(s_hist + p * bins, (uint32_t)(key >> pd.shift[p]) & pd.mask[p], valid);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < pd.passes * bins; i += kThreads)
        if (s_hist[i]) atomicAdd(hist + i, s_hist[i]);
}

// ---------------------------------------------------------------- batches
// The meshes of a tile's first and last element, found once per tile by
// thread 0 (a mesh usually covers many tiles, so both are the same).
__device__ __forceinline__ uint2 tile_meshes(const MeshBatch& b, uint32_t first, uint32_t last) {
    const uint32_t lo = owner_of(b.off, 0, b.meshes - 1, first);
    return make_uint2(lo, owner_of(b.off, lo, b.meshes - 1, last));
}

// The mesh range of every T-primitive tile, one thread per tile, so that the
// tile kernels read it with one load instead of searching in one thread
// while the others wait at a barrier.
__global__ void batch_tile_ranges_kernel(MeshBatch batch, uint32_t total, uint32_t T, uint2* rng) {
    const uint32_t tiles = (total + T - 1) / T;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < tiles; t += gridDim.x * blockDim.x) {
        const uint32_t first = t * T;
        rng[t] = tile_meshes(batch, first, min(first + T, total) - 1);
    }
}

__device__ __forceinline__ void ord_max(uint32_t* o, const Box& b) {
    atomicMax(o + 0, ~f2ord(b.mn.x));
    atomicMax(o + 1, ~f2ord(b.mn.y));
    atomicMax(o + 2, ~f2ord(b.mn.z));
    atomicMax(o + 3, f2ord(b.mx.x));
    atomicMax(o + 4, f2ord(b.mx.y));
    atomicMax(o + 5, f2ord(b.mx.z));
}

__device__ __forceinline__ void warp_reduce_box(Box& b) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Box other;
        other.mn.x = __shfl_down_sync(kFullMask, b.mn.x, o);
        other.mn.y = __shfl_down_sync(kFullMask, b.mn.y, o);
        other.mn.z = __shfl_down_sync(kFullMask, b.mn.z, o);
        other.mx.x = __shfl_down_sync(kFullMask, b.mx.x, o);
        other.mx.y = __shfl_down_sync(kFullMask, b.mx.y, o);
        other.mx.z = __shfl_down_sync(kFullMask, b.mx.z, o);
        grow(b, other);
    }
}

// Stage 1 over a batch: the same tile staging; mesh m's leaves go to BVH2
// nodes [2*off[m], 2*off[m] + count) with mesh-local primitive indices.  A
// tile inside one mesh reduces its box over the CTA into one set of 6
// atomics on scene_ord[6m .. 6m+5]; a tile that spans meshes (about one per
// mesh boundary) reduces per warp, or per lane where a warp spans meshes.
template <int FLOATS, int T>
__global__ __launch_bounds__(T) void batch_bounds_kernel(const float* __restrict__ prims, MeshBatch batch,
                                                                uint32_t total, Node2* __restrict__ nodes,
                                                                uint32_t* scene_ord, bool aligned16,
                                                                const uint2* __restrict__ tile_rng) {
    __shared__ __align__(16) float tile[T * FLOATS];
    __shared__ float s_red[T / 32][6];
    const uint32_t tiles = (total + T - 1) / T;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint32_t first = t * T;
        const uint32_t cnt = min((uint32_t)T, total - first);
        const float* src = prims + (size_t)first * FLOATS;
        __syncthreads();
        const uint2 rng = __ldg(tile_rng + t);  // the tile's first and last mesh
        if (cnt == T && aligned16) {
            constexpr int V = T * FLOATS / 4;
            const float4* s4 = reinterpret_cast<const float4*>(src);
            float4* d4 = reinterpret_cast<float4*>(tile);
#pragma unroll
            for (int v = threadIdx.x; v < V; v += T) d4[v] = __ldcs(s4 + v);
        } else {
            for (uint32_t v = threadIdx.x; v < cnt * FLOATS; v += T) tile[v] = __ldcs(src + v);
        }
        __syncthreads();
        const uint32_t lo = rng.x, hi = rng.y;
        const bool valid = threadIdx.x < cnt;
        const uint32_t g = first + min(threadIdx.x, cnt - 1);
        const MeshSpan me = batch.span(lo == hi ? lo : owner_of(batch.off, lo, hi, g));
        Box b;
        b.mn = make_float3(3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f);
        b.mx = make_float3(-3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f);
        if (valid) {
            const float* f = tile + threadIdx.x * FLOATS;
            if (FLOATS == 9) {
                float3 v0 = make_float3(f[0], f[1], f[2]);
                float3 v1 = make_float3(f[3], f[4], f[5]);
                float3 v2 = make_float3(f[6], f[7], f[8]);
                b.mn = fmin3(v0, fmin3(v1, v2));
                b.mx = fmax3(v0, fmax3(v1, v2));
            } else {
                b.mn = make_float3(f[0], f[1], f[2]);
                b.mx = make_float3(f[3], f[4], f[5]);
            }
            const uint32_t local = g - me.start;
            store_node(nodes, 2 * me.start + local, b, kInvalid, local);
        }
        if (lo == hi) {  // CTA-uniform
            warp_reduce_box(b);
            if (lane == 0) {
                s_red[warp][0] = b.mn.x;
                s_red[warp][1] = b.mn.y;
                s_red[warp][2] = b.mn.z;
                s_red[warp][3] = b.mx.x;
                s_red[warp][4] = b.mx.y;
                s_red[warp][5] = b.mx.z;
            }
            __syncthreads();
            if (threadIdx.x < 6) {
                const int a = threadIdx.x;
                float v = s_red[0][a];
                for (int w = 1; w < T / 32; ++w) v = a < 3 ? fminf(v, s_red[w][a]) : fmaxf(v, s_red[w][a]);
                atomicMax(scene_ord + 6ull * lo + a, a < 3 ? ~f2ord(v) : f2ord(v));
            }
        } else {
            const uint32_t m0 = __shfl_sync(kFullMask, me.m, 0);
            if (__all_sync(kFullMask, !valid || me.m == m0)) {
                warp_reduce_box(b);
                if (lane == 0 && first + (threadIdx.x & ~31u) < first + cnt) ord_max(scene_ord + 6ull * m0, b);
            } else if (valid) {
                ord_max(scene_ord + 6ull * me.m, b);
            }
        }
    }
}

// Stage 2 over a batch: 30-bit codes from each mesh's own box, written as
// one sort key mesh << 32 | code, the value being the mesh-local primitive
// index; digit histograms of every pass of that key fused as in the plain
// kernel, and the same fill work (parent slots, look-back flags).  Tiles of
// 256 elements: a tile inside one mesh reads the mesh's span and scene box
// once, into shared memory.
template <bool HIST, int T, int PASSES = 0>
__global__ __launch_bounds__(T) void batch_morton_kernel(const Node2* __restrict__ nodes, MeshBatch batch,
                                                                uint32_t total, const uint32_t* scene_ord,
                                                                uint64_t* __restrict__ keys, uint32_t* vals,
                                                                uint32_t* hist, MortonArgs a,
                                                                const uint2* __restrict__ tile_rng) {
    __shared__ uint32_t s_hist[HIST ? kMaxSortPasses * kRadixBins : 1];
    if (HIST)
        for (int i = threadIdx.x; i < a.pd.passes * kRadixBins; i += T) s_hist[i] = 0;
    __syncthreads();
    const uint32_t tiles = (total + T - 1) / T;
    const uint32_t stride = gridDim.x * T;
    for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint32_t first = t * T;
        const uint32_t cnt = min((uint32_t)T, total - first);
        const uint2 rng = __ldg(tile_rng + t);  // the tile's first and last mesh
        const uint32_t lo = rng.x, hi = rng.y;
        const uint32_t i = first + threadIdx.x;
        const bool valid = threadIdx.x < cnt;
        uint64_t key = 0;
        if (valid) {
            const MeshSpan me = batch.span(lo == hi ? lo : owner_of(batch.off, lo, hi, i));
            // the mesh's scene box (one L1 line that the whole tile reads)
            const uint32_t* o = scene_ord + 6ull * me.m;
            const float3 smin = make_float3(ord2f(~__ldg(o + 0)), ord2f(~__ldg(o + 1)), ord2f(~__ldg(o + 2)));
            const float3 smax = make_float3(ord2f(__ldg(o + 3)), ord2f(__ldg(o + 4)), ord2f(__ldg(o + 5)));
            const uint32_t local = i - me.start;
            const float4* p = reinterpret_cast<const float4*>(nodes + 2ull * me.start + local);
            float4 lo4 = __ldcs(p);
            float2 hi2 = __ldcs(reinterpret_cast<const float2*>(p + 1));
            Box b;
            b.mn = make_float3(lo4.x, lo4.y, lo4.z);
            b.mx = make_float3(lo4.w, hi2.x, hi2.y);
            key = ((uint64_t)me.m << 32) | morton_key<uint32_t>(b, smin, smax);
            keys[i] = key;
            vals[i] = local;
        }
        if (HIST) {
            if constexpr (PASSES > 0) {
#pragma unroll
                for (int p = 0; p < PASSES; ++p) {
                    const uint32_t d = (uint32_t)(key >> a.pd.shift[p]) & a.pd.mask[p];
                    if (p < PASSES / 2) {
                        if (valid) atomicAdd(&s_hist[p * kRadixBins + d], 1u);
                    } else {
                        hist_add(s_hist + p * kRadixBins, d, valid);
                    }
                }
            } else {
#pragma unroll 1
                for (int p = 0; p < a.pd.passes; ++p) {
                    uint32_t d = (uint32_t)(key >> a.pd.shift[p]) & a.pd.mask[p];
                    hist_add(s_hist + p * kRadixBins, d, valid);
                }
            }
        }
    }
    for (size_t w = (size_t)blockIdx.x * T + threadIdx.x; w < a.zero_vec4; w += stride)
        a.zero_ptr[w] = make_uint4(0, 0, 0, 0);
    for (size_t w = (size_t)blockIdx.x * T + threadIdx.x; w < a.ones_vec4; w += stride)
        a.ones_ptr[w] = make_uint4(kInvalid, kInvalid, kInvalid, kInvalid);
    if (HIST) {
        __syncthreads();
        for (int i = threadIdx.x; i < a.pd.passes * kRadixBins; i += T)
            if (s_hist[i]) atomicAdd(hist + i, s_hist[i]);
    }
}

// Per-mesh results of a batch: scene box, BVH8 range and counts.
__global__ void batch_finalize_kernel(MeshBatch batch, const uint32_t* scene_ord, const uint32_t* mesh_nodes,
                                      const uint32_t* mesh_leaves, nxb_batch_mesh* out) {
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < batch.meshes; m += gridDim.x * blockDim.x) {
        const MeshSpan me = batch.span(m);
        nxb_batch_mesh r{};
        if (me.count) {
            const uint32_t* o = scene_ord + 6ull * m;
            for (int k = 0; k < 3; ++k) {
                r.scene_bounds.bmin[k] = ord2f(~o[k]);
                r.scene_bounds.bmax[k] = ord2f(o[3 + k]);
            }
        }
        r.prim_offset = me.start;
        r.prim_count = me.count;
        r.bvh2_offset = 2 * me.start;
        r.bvh2_node_count = me.count ? 2 * me.count - 1 : 0;
        r.bvh8_offset = __ldg(batch.off8 + m);
        r.bvh8_node_count = mesh_nodes[m];
        r.bvh8_leaf_count = mesh_leaves[m];
        out[m] = r;
    }
}

PassDigits to_digits(const SortPlan& plan) {
    PassDigits pd{};
    pd.passes = plan.passes;
    for (int p = 0; p < plan.passes; ++p) {
        pd.shift[p] = plan.shift[p];
        pd.mask[p] = (1u << plan.bits[p]) - 1u;
    }
    return pd;
}

uint32_t grid_for(uint32_t n, int blocks_per_sm) {
    uint32_t want = (n + kThreads - 1) / kThreads;
    uint32_t cap = (uint32_t)(device_info().sms * blocks_per_sm);
    return std::max(1u, std::min(want, cap));
}

}  // namespace

cudaError_t launch_scene_bounds(const void* prims, int prim_type, uint32_t n, Node2* nodes, uint32_t* scene_ord,
                                cudaStream_t s) {
    bool aligned = (reinterpret_cast<uintptr_t>(prims) & 15u) == 0;
    uint32_t grid = grid_for(n, 8);
    if (prim_type == NXB_PRIM_TRIANGLE)
        scene_bounds_kernel<9><<<grid, kThreads, 0, s>>>((const float*)prims, n, nodes, scene_ord, aligned);
    else
        scene_bounds_kernel<6><<<grid, kThreads, 0, s>>>((const float*)prims, n, nodes, scene_ord, aligned);
    return cudaGetLastError();
}

cudaError_t launch_morton(const Node2* nodes, uint32_t n, Control* ctrl, int key_bits, void* keys,
                          const MortonFused& f, cudaStream_t s) {
    MortonArgs a{};
    if (f.plan) a.pd = to_digits(*f.plan);
    a.cluster_idx = f.cluster_idx;
    a.parent = f.parent;
    a.zero_ptr = reinterpret_cast<uint4*>(f.zero_ptr);
    a.zero_vec4 = f.zero_words / 4;
    a.ones_ptr = reinterpret_cast<uint4*>(f.ones_ptr);
    a.ones_vec4 = f.ones_words / 4;
    a.scene_out = f.scene_out;
    a.seed = f.seed_counters ? 1 : 0;
    uint32_t grid = grid_for(n, 8);
    if (key_bits == 30) {
        if (f.plan && a.pd.passes == 4)
            morton_kernel<uint32_t, true, 4><<<grid, kThreads, 0, s>>>(nodes, n, ctrl, (uint32_t*)keys, a);
        else if (f.plan)
            morton_kernel<uint32_t, true><<<grid, kThreads, 0, s>>>(nodes, n, ctrl, (uint32_t*)keys, a);
        else
            morton_kernel<uint32_t, false><<<grid, kThreads, 0, s>>>(nodes, n, ctrl, (uint32_t*)keys, a);
    } else {
        if (f.plan && a.pd.passes == 4 && a.pd.mask[0] == (1u << kMaxRadixBits) - 1u)
            morton_kernel<uint64_t, true, 4, 1 << kMaxRadixBits><<<grid, kThreads, 0, s>>>(nodes, n, ctrl,
                                                                                           (uint64_t*)keys, a);
        else if (f.plan && a.pd.passes == 8)
            morton_kernel<uint64_t, true, 8><<<grid, kThreads, 0, s>>>(nodes, n, ctrl, (uint64_t*)keys, a);
        else if (f.plan)
            morton_kernel<uint64_t, true><<<grid, kThreads, 0, s>>>(nodes, n, ctrl, (uint64_t*)keys, a);
        else
            morton_kernel<uint64_t, false><<<grid, kThreads, 0, s>>>(nodes, n, ctrl, (uint64_t*)keys, a);
    }
    return cudaGetLastError();
}

cudaError_t launch_morton_scene(const Node2* nodes, uint32_t n, const nxb_aabb* scene, int key_bits, void* keys,
                                uint32_t* cluster_idx, cudaStream_t s) {
    uint32_t grid = grid_for(n, 8);
    if (key_bits == 30)
        morton_scene_kernel<uint32_t><<<grid, kThreads, 0, s>>>(nodes, n, scene, (uint32_t*)keys, cluster_idx);
    else
        morton_scene_kernel<uint64_t><<<grid, kThreads, 0, s>>>(nodes, n, scene, (uint64_t*)keys, cluster_idx);
    return cudaGetLastError();
}

cudaError_t launch_sort_histogram(uint32_t key_bytes, const void* keys, uint32_t n, const SortPlan& plan,
                                  uint32_t* hist, cudaStream_t s) {
    PassDigits pd = to_digits(plan);
    uint32_t widest = 1;
    for (int p = 0; p < plan.passes; ++p) widest = std::max(widest, plan.bits[p]);
    const uint32_t bins = 1u << std::max<uint32_t>(widest, kRadixBits);
    if ((size_t)plan.passes * bins > (size_t)kMaxSortPasses * kRadixBins) return cudaErrorInvalidValue;
    uint32_t grid = grid_for(n, 4);
    if (key_bytes == 4)
        sort_histogram_kernel<uint32_t><<<grid, kThreads, 0, s>>>((const uint32_t*)keys, n, pd, bins, hist);
    else
        sort_histogram_kernel<uint64_t><<<grid, kThreads, 0, s>>>((const uint64_t*)keys, n, pd, bins, hist);
    return cudaGetLastError();
}

template <int T>
uint32_t batch_grid(uint32_t total) {
    const uint32_t want = (total + T - 1) / T;
    const uint32_t cap = (uint32_t)device_info().sms * (2048 / T);
    return std::max(1u, std::min(want, cap));
}

template <int T>
void bounds_t(const void* prims, int prim_type, const MeshBatch& batch, uint32_t total, Node2* nodes,
              uint32_t* scene_ord, bool aligned, const uint2* tile_rng, cudaStream_t s) {
    if (prim_type == NXB_PRIM_TRIANGLE)
        batch_bounds_kernel<9, T><<<batch_grid<T>(total), T, 0, s>>>((const float*)prims, batch, total, nodes,
                                                                     scene_ord, aligned, tile_rng);
    else
        batch_bounds_kernel<6, T><<<batch_grid<T>(total), T, 0, s>>>((const float*)prims, batch, total, nodes,
                                                                     scene_ord, aligned, tile_rng);
}

cudaError_t launch_batch_tile_ranges(const MeshBatch& batch, uint32_t total, uint32_t block, uint2* tile_rng,
                                     cudaStream_t s) {
    const uint32_t tiles = (total + block - 1) / block;
    const uint32_t grid = std::max(1u, std::min<uint32_t>((tiles + 255) / 256, (uint32_t)device_info().sms * 4));
    batch_tile_ranges_kernel<<<grid, 256, 0, s>>>(batch, total, block, tile_rng);
    return cudaGetLastError();
}

cudaError_t launch_batch_bounds(const void* prims, int prim_type, const MeshBatch& batch, uint32_t total,
                                Node2* nodes, uint32_t* scene_ord, uint32_t block, const uint2* tile_rng,
                                cudaStream_t s) {
    const bool aligned = (reinterpret_cast<uintptr_t>(prims) & 15u) == 0;
    if (block == 128)
        bounds_t<128>(prims, prim_type, batch, total, nodes, scene_ord, aligned, tile_rng, s);
    else if (block == 512)
        bounds_t<512>(prims, prim_type, batch, total, nodes, scene_ord, aligned, tile_rng, s);
    else
        bounds_t<256>(prims, prim_type, batch, total, nodes, scene_ord, aligned, tile_rng, s);
    return cudaGetLastError();
}

cudaError_t launch_batch_morton(const Node2* nodes, const MeshBatch& batch, uint32_t total, const uint32_t* scene_ord,
                                uint64_t* keys, uint32_t* vals, const SortPlan& plan, uint32_t* hist,
                                const MortonFused& f, uint32_t block, const uint2* tile_rng, cudaStream_t s) {
    MortonArgs a{};
    a.pd = to_digits(plan);
    a.zero_ptr = reinterpret_cast<uint4*>(f.zero_ptr);
    a.zero_vec4 = f.zero_words / 4;
    a.ones_ptr = reinterpret_cast<uint4*>(f.ones_ptr);
    a.ones_vec4 = f.ones_words / 4;
    const bool five = a.pd.passes == 5;  // 8-bit digits over 40 bits: 1024 meshes
    if (block == 128) {
        if (five)
            batch_morton_kernel<true, 128, 5><<<batch_grid<128>(total), 128, 0, s>>>(nodes, batch, total, scene_ord,
                                                                                    keys, vals, hist, a, tile_rng);
        else
            batch_morton_kernel<true, 128><<<batch_grid<128>(total), 128, 0, s>>>(nodes, batch, total, scene_ord, keys,
                                                                                  vals, hist, a, tile_rng);
    } else if (block == 512) {
        if (five)
            batch_morton_kernel<true, 512, 5><<<batch_grid<512>(total), 512, 0, s>>>(nodes, batch, total, scene_ord,
                                                                                    keys, vals, hist, a, tile_rng);
        else
            batch_morton_kernel<true, 512><<<batch_grid<512>(total), 512, 0, s>>>(nodes, batch, total, scene_ord, keys,
                                                                                  vals, hist, a, tile_rng);
    } else {
        if (five)
            batch_morton_kernel<true, 256, 5><<<batch_grid<256>(total), 256, 0, s>>>(nodes, batch, total, scene_ord,
                                                                                    keys, vals, hist, a, tile_rng);
        else
            batch_morton_kernel<true, 256><<<batch_grid<256>(total), 256, 0, s>>>(nodes, batch, total, scene_ord, keys,
                                                                                  vals, hist, a, tile_rng);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_finalize(const MeshBatch& batch, const uint32_t* scene_ord, const uint32_t* mesh_nodes,
                                  const uint32_t* mesh_leaves, nxb_batch_mesh* out, cudaStream_t s) {
    const uint32_t grid = std::max(1u, std::min<uint32_t>((batch.meshes + 255) / 256, 1024u));
    batch_finalize_kernel<<<grid, 256, 0, s>>>(batch, scene_ord, mesh_nodes, mesh_leaves, out);
    return cudaGetLastError();
}

}  // namespace nxb
