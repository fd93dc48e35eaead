// pipeline.h - host-side launchers of the build stages and the workspace
// control block shared by the kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nxb_gb300.h"
#include "common.cuh"

namespace nxb {

constexpr int kMaxSortPasses = 8;

// BVH8 work-queue counters, each on its own 128-byte line (they are polled
// and bumped by every warp): next slot to claim, BVH8 nodes, leaves, work
// slots allocated, work items allocated but not finished.
constexpr int kBvh8Claim = 0, kBvh8Nodes = 32, kBvh8Leaves = 64, kBvh8Alloc = 96, kBvh8Pending = 128;
constexpr int kBvh8CtrWords = 160;
constexpr int kRadixBits = 8;
constexpr int kRadixBins = 1 << kRadixBits;

// Small per-build state, cleared by one memset at the start of a build.
struct Control {
    uint32_t scene_ord[6];  // [0..2]: ~ordered(min) (atomicMax), [3..5]: ordered(max)
    uint32_t cluster_count; // H-PLOC node allocator
    uint32_t error_word;
    uint32_t pad0[16];
    alignas(128) uint32_t bvh8_ctr[160];  // BVH8 counters, one per 128-byte line (kBvh8* below)
    uint32_t parent_of_last; // H-PLOC: the node whose child is node 2n-2 (seeded INVALID)
    uint32_t hploc_leaf_ctr; // H-PLOC: next unclaimed leaf
    uint32_t pad[2];
    uint32_t tile_ctr[kMaxSortPasses];
    uint32_t hist[kMaxSortPasses][kRadixBins];
};

// Sort pass plan for the reference's bit ranges: [2,32) for 30-bit codes in
// uint32 keys, [1,64) for 63-bit codes in uint64 keys (Setup.cu:74-78).
struct SortPlan {
    int passes;
    uint32_t shift[kMaxSortPasses];
    uint32_t bits[kMaxSortPasses];
};
SortPlan make_sort_plan(uint32_t begin_bit, uint32_t end_bit);

struct DeviceInfo {
    int sms;
    int max_smem_optin;
};
const DeviceInfo& device_info();

// Records e as this thread's last CUDA error and maps it to a status.
nxb_status record_cuda_error(cudaError_t e);

// ---------------------------------------------------------------- stage 1
// Leaves + scene bounds; scene_ord (6 words, the Control::scene_ord
// encoding) must be zero on entry.
cudaError_t launch_scene_bounds(const void* prims, int prim_type, uint32_t n, Node2* nodes, uint32_t* scene_ord,
                                cudaStream_t s);
// Converts the 6 ordered words in place into an nxb_aabb.
cudaError_t launch_ord_to_aabb(uint32_t* scene_ord, cudaStream_t s);
// ---------------------------------------------------------------- stage 2
// Morton keys from the leaves and ctrl->scene_ord.  Optional fused work:
// histograms of every sort pass into ctrl->hist (plan != nullptr),
// cluster_idx[i] = i, parent[i] = INVALID, clearing `zero_words` words at
// `zero_ptr`, seeding ctrl counters, writing the float scene box to
// `scene_out`.
struct MortonFused {
    const SortPlan* plan;
    uint32_t* cluster_idx;
    uint32_t* parent;
    uint32_t* zero_ptr;
    size_t zero_words;
    uint32_t* ones_ptr;   // filled with all-ones words (ones_words, multiple of 4)
    size_t ones_words;
    nxb_aabb* scene_out;
    bool seed_counters;
};
cudaError_t launch_morton(const Node2* nodes, uint32_t n, Control* ctrl, int key_bits, void* keys,
                          const MortonFused& fused, cudaStream_t s);
// Morton keys from an explicit scene box (stage entry point).
cudaError_t launch_morton_scene(const Node2* nodes, uint32_t n, const nxb_aabb* scene, int key_bits, void* keys,
                                uint32_t* cluster_idx, cudaStream_t s);
// ---------------------------------------------------------------- stage 3
size_t sort_lookback_words(uint32_t n, uint32_t key_bytes, int passes);
// Digit histograms of all passes (standalone sort only; the pipeline fuses
// this into the Morton kernel).  hist must be zero on entry.
cudaError_t launch_sort_histogram(uint32_t key_bytes, const void* keys, uint32_t n, const SortPlan& plan,
                                  uint32_t* hist, cudaStream_t s);
// One onesweep pass.  vals_in == nullptr means values = input position.
cudaError_t launch_sort_pass(uint32_t key_bytes, const void* keys_in, void* keys_out, const uint32_t* vals_in,
                             uint32_t* vals_out, uint32_t n, uint32_t shift, uint32_t bits, const uint32_t* hist,
                             uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err, cudaStream_t s);
// ---------------------------------------------------------------- stage 4
// tokens: n words of scratch (no initialisation needed); parent_of_last:
// one word that must hold INVALID on entry; leaf_ctr: one word that must
// be zero on entry.
cudaError_t launch_hploc(uint32_t key_bytes, const void* keys, uint32_t* cluster_idx, uint32_t* parent, Node2* nodes,
                         uint32_t n, uint32_t radius, uint32_t* tokens, uint32_t* parent_of_last, uint32_t* leaf_ctr,
                         uint32_t* err, cudaStream_t s);
// ---------------------------------------------------------------- stage 5
// pairs: n uint64 slots; ctr: kBvh8CtrWords words (128-byte aligned).
// Both are initialised by launch_bvh8_init.
cudaError_t launch_bvh8_init(uint64_t* pairs, uint32_t n, uint32_t* ctr, cudaStream_t s);
cudaError_t launch_bvh8(const Node2* bvh2, uint32_t n, Node8* out, uint32_t cap, uint32_t* prim_idx, uint64_t* pairs,
                        uint32_t* ctr, uint32_t* err, cudaStream_t s);
// ---------------------------------------------------------------- eval
cudaError_t launch_bvh2_cost(const Node2* nodes, uint32_t count, const nxb_aabb* root, float* cost, cudaStream_t s);
cudaError_t launch_bvh8_cost(const Node8* nodes, uint32_t count, const nxb_aabb* root, float* cost, cudaStream_t s);
// Same, with the node count read on the device from *count_ptr (<= cap).
cudaError_t launch_bvh8_cost_dev(const Node8* nodes, const uint32_t* count_ptr, uint32_t cap, const nxb_aabb* root,
                                 float* cost, cudaStream_t s);
cudaError_t launch_fill_u32(uint32_t* p, uint32_t value, size_t count, cudaStream_t s);
// Numerics probes (see eval.cu); report has 40 entries.
cudaError_t run_selftest(uint32_t* report);
// Bounded-wait probes: each returns the error word its expired wait set.
cudaError_t run_sort_stall_probe(uint32_t* err_out);
cudaError_t run_bvh8_stall_probe(uint32_t* err_out);
// Copies counters / error word / scene box into a device nxb_build_result.
cudaError_t launch_finalize(const Control* ctrl, nxb_build_result* result, uint32_t n, cudaStream_t s);

}  // namespace nxb
