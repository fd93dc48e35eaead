// pipeline.h - host-side launchers of the build stages and the workspace
// control block shared by the kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <mutex>

#include "../../include/nxb_gb300.h"
#include "common.cuh"

namespace nxb {

// Most passes of a sort plan: 10 for the batched 4-bit plan over 40-bit
// keys (30-bit codes and a 10-bit mesh index).
constexpr int kMaxSortPasses = 10;

// BVH8 work-queue counters (they are polled and bumped by every warp):
// next slot to claim; one 64-bit word of work slots allocated (low half)
// and leaves (high half), bumped with one atomic, where one mesh's BVH8
// nodes are its slots (every internal node is one work item, root
// included); work items allocated but not finished.  Each counter has its
// own 128-byte line.
constexpr int kBvh8Claim = 0, kBvh8Alloc = 32, kBvh8Nodes = kBvh8Alloc, kBvh8Leaves = kBvh8Alloc + 1,
              kBvh8Pending = 64;
constexpr int kBvh8CtrWords = 160;

// The BVH8 work queue of an n-primitive build before the collapse: slot 0
// holds the root item (BVH2 root 2n-2 into BVH8 node 0), every other slot
// is empty; one BVH8 node and one work item exist.
__device__ __forceinline__ uint64_t bvh8_queue_slot(uint32_t i, uint32_t n) {
    return i == 0 ? ((uint64_t)(2 * n - 2) << 32) : ~0ull;
}
__device__ __forceinline__ void bvh8_queue_counters(uint32_t* ctr) {
    ctr[kBvh8Claim] = 0;
    ctr[kBvh8Alloc] = 1;  // = kBvh8Nodes: the root
    ctr[kBvh8Leaves] = 0;
    ctr[kBvh8Pending] = 1;
}
constexpr int kRadixBits = 8;
constexpr int kRadixBins = 1 << kRadixBits;
// Widest digit of a onesweep pass (the pipeline's 63-bit sort uses 9-bit
// digits for its top passes; see launch_sort63_hybrid).
constexpr int kMaxRadixBits = 9;
// The 63-bit sort's top passes cover bits [kHybridTopShift, 64).
constexpr uint32_t kHybridTopShift = 28;

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
    // histograms: kMaxSortPasses x 256 words, or 4 passes x 512 words of the
    // 63-bit sort's top passes (the same storage)
    uint32_t hist[kMaxSortPasses][kRadixBins];
    uint32_t sort_overflow;                // 63-bit sort: a bucket too large for shared memory
    uint32_t fb_ticket;                    // 63-bit sort fallback: next ticket
    uint32_t fb_done[kMaxSortPasses + 2];  // 63-bit sort fallback: finished tickets per stage
};

// Sort pass plan for the reference's bit ranges: [2,32) for 30-bit codes in
// uint32 keys, [1,64) for 63-bit codes in uint64 keys (Setup.cu:74-78).
struct SortPlan {
    int passes;
    uint32_t shift[kMaxSortPasses];
    uint32_t bits[kMaxSortPasses];
};
// Passes of at most digit_bits (1..9) bits each, lowest digit first.
SortPlan make_sort_plan(uint32_t begin_bit, uint32_t end_bit, uint32_t digit_bits = kRadixBits);
// The top passes of the 63-bit sort: bits [kHybridTopShift, 64) in 9-bit digits.
SortPlan hybrid63_top_plan();

// The whole-array re-sort of the 63-bit sort (launch_sort63_hybrid): its
// pass plan, look-back and histogram storage and ticket counters.
struct SortFallback {
    SortPlan plan;
    uint32_t tiles;              // tiles per pass
    uint32_t zero_tickets;       // tickets that clear the look-back words
    uint32_t hist_tickets;       // tickets that count digits
    size_t lookback_per_pass;    // words
    uint32_t* lookback;
    uint32_t* hist;              // plan.passes x 256 words
    uint32_t* ticket;            // zero on entry
    uint32_t* done;              // plan.passes + 2 words, zero on entry
};

// Runs `set` (kernel attribute calls) once per device, with that device
// current, from any number of host threads; later calls return its result.
// Each call site passes its own lambda type and so has its own flags.
template <typename F>
cudaError_t once_per_device(F set) {
    constexpr int kMaxDev = 64;
    static std::once_flag once[kMaxDev];
    static cudaError_t result[kMaxDev];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    std::call_once(once[dev], [&] { result[dev] = set(); });
    return result[dev];
}

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
// Look-back words of `passes` passes with `bins` digits.
size_t sort_lookback_words(uint32_t n, uint32_t key_bytes, int passes, uint32_t bins = kRadixBins);
// Digit histograms of all passes (standalone sort only; the pipeline fuses
// this into the Morton kernel), pass after pass, 1 << (widest digit of the
// plan) words each.  hist must be zero on entry.
cudaError_t launch_sort_histogram(uint32_t key_bytes, const void* keys, uint32_t n, const SortPlan& plan,
                                  uint32_t* hist, cudaStream_t s);
// One onesweep pass of `bits` <= 9 bits (9 only for 64-bit keys).
// vals_in == nullptr means values = input position.
cudaError_t launch_sort_pass(uint32_t key_bytes, const void* keys_in, void* keys_out, const uint32_t* vals_in,
                             uint32_t* vals_out, uint32_t n, uint32_t shift, uint32_t bits, const uint32_t* hist,
                             uint32_t* lookback, uint32_t* tile_ctr, uint32_t* err, cudaStream_t s);
// The sort of 64-bit keys on bits [1,64) (the pipeline's 63-bit Morton
// keys): four 9-bit passes over bits [28,64) (in -> B -> A -> B -> A;
// top_hist = their 4 x 512 digit counts, lookback = their zeroed look-back
// words, tile_ctr = 4 zeroed counters), the in-place sort of every bucket of
// equal key >> 28, and the whole-array fallback, which runs only if a bucket
// was too large (overflow, fb_ticket, fb_done zero on entry; it clears
// fb_hist and lookback itself).  The first pass reads keys_in (keys_a if
// null) and vals_in (the input positions if null); the sorted keys and the
// permutation end in keys_a / vals_a.
cudaError_t launch_sort63_hybrid(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_a, uint64_t* keys_b,
                                 uint32_t* vals_a, uint32_t* vals_b, uint32_t n, const uint32_t* top_hist,
                                 uint32_t* lookback, uint32_t* tile_ctr, uint32_t* overflow, uint32_t* fb_hist,
                                 uint32_t* fb_ticket, uint32_t* fb_done, uint32_t* err, cudaStream_t s);
// ---------------------------------------------------------------- stage 4
// tokens: n words of scratch (no initialisation needed); parent_of_last:
// one word that must hold INVALID on entry; leaf_ctr: one word that must
// be zero on entry.
// records: n records of 32 bytes (no initialisation needed), where merges
// store each window's clusters as {box, id, token}.
// bvh8_pairs / bvh8_ctr (both or neither): the BVH8 work queue of stage 5,
// which the climb initialises as launch_bvh8_init would (each lane writes
// the slot of the leaf it takes), so that the collapse can follow without
// an initialisation launch of its own.
// child_pairs (optional): n-1 records of 64 bytes, 64-byte aligned; record
// X - n receives the children of internal node X (boxes and indices), for
// launch_bvh8 to read instead of the BVH2 nodes.
cudaError_t launch_hploc(uint32_t key_bytes, const void* keys, uint32_t* cluster_idx, uint32_t* parent, Node2* nodes,
                         uint32_t n, uint32_t radius, uint32_t* tokens, uint32_t* parent_of_last, uint32_t* leaf_ctr,
                         uint32_t* err, cudaStream_t s, Node2* records, uint64_t* bvh8_pairs = nullptr,
                         uint32_t* bvh8_ctr = nullptr, ChildPair* child_pairs = nullptr);
// ---------------------------------------------------------------- stage 5
// pairs: n uint64 slots; ctr: kBvh8CtrWords words (128-byte aligned).
// Both are initialised by launch_bvh8_init.
cudaError_t launch_bvh8_init(uint64_t* pairs, uint32_t n, uint32_t* ctr, cudaStream_t s);
// auction: the reference's USE_AUCTION slot assignment instead of the greedy one.
// child_pairs (optional): the records launch_hploc wrote for this BVH2; the
// collapse then opens nodes through them and reads no BVH2 node.
cudaError_t launch_bvh8(const Node2* bvh2, uint32_t n, Node8* out, uint32_t cap, uint32_t* prim_idx, uint64_t* pairs,
                        uint32_t* ctr, uint32_t* err, bool auction, cudaStream_t s,
                        const ChildPair* child_pairs = nullptr);
// ---------------------------------------------------------------- batches
// The same stages over independent meshes laid end to end (MeshBatch in
// common.cuh): one launch per stage for the whole batch.
// scene_ord: 6 words per mesh, zero on entry.
// block: CTA size of the two tile kernels (128, 256 or 512).
// tile_rng: the first and last mesh of every `block`-primitive tile
// (launch_batch_tile_ranges with the same block).
cudaError_t launch_batch_tile_ranges(const MeshBatch& batch, uint32_t total, uint32_t block, uint2* tile_rng,
                                     cudaStream_t s);
cudaError_t launch_batch_bounds(const void* prims, int prim_type, const MeshBatch& batch, uint32_t total,
                                Node2* nodes, uint32_t* scene_ord, uint32_t block, const uint2* tile_rng,
                                cudaStream_t s);
// keys: mesh << 32 | 30-bit code; vals: mesh-local primitive index; hist:
// kMaxSortPasses x kRadixBins words, zero on entry.
cudaError_t launch_batch_morton(const Node2* nodes, const MeshBatch& batch, uint32_t total, const uint32_t* scene_ord,
                                uint64_t* keys, uint32_t* vals, const SortPlan& plan, uint32_t* hist,
                                const MortonFused& fill, uint32_t block, const uint2* tile_rng, cudaStream_t s);
// H-PLOC over the sorted positions [begin, end), which must cover whole
// meshes; leaf_ctr: a zeroed word of its own.  parent_of_last: one word per
// mesh holding INVALID on entry; ctas_per_sm caps the persistent grid (0: as
// many CTAs as fit).  child_pairs (optional): one 64-byte record per
// primitive of the batch; mesh m's internal node X gets record off[m] + X - n_m.
cudaError_t launch_hploc_batch(const uint64_t* keys, uint32_t* cluster_idx, uint32_t* parent, Node2* nodes,
                               const MeshBatch& batch, uint32_t begin, uint32_t end, uint32_t radius,
                               uint32_t* tokens, uint32_t* parent_of_last, uint32_t* leaf_ctr, uint32_t* err,
                               uint32_t ctas_per_sm, cudaStream_t s, ChildPair* child_pairs = nullptr);
// Meshes cut into consecutive groups whose BVH8 collapses are separate
// launches: group g holds meshes [mesh[g], mesh[g+1]), primitives
// [prim[g], prim[g+1]) and BVH8 slots [slot[g], slot[g+1]).
constexpr uint32_t kMaxMeshGroups = 8;
struct MeshGroups {
    uint32_t count;
    uint32_t mesh[kMaxMeshGroups + 1];
    uint32_t prim[kMaxMeshGroups + 1];
    uint32_t slot[kMaxMeshGroups + 1];
};
// pairs: `slots` = off8[meshes] uint64 slots; ctr: kBvh8CtrWords words per
// group.  Seeds every group's queue with the root items of its meshes.
cudaError_t launch_bvh8_batch_init(uint64_t* pairs, uint32_t slots, const MeshBatch& batch, uint32_t* ctr,
                                   uint32_t* mesh_nodes, uint32_t* mesh_leaves, const MeshGroups& groups,
                                   cudaStream_t s);
// The collapse of the meshes of `batch` (a whole batch, or one group's view:
// off, off8, mesh_nodes and mesh_leaves advanced to the group's first mesh,
// pairs to its first slot, ctr to its counters).  child_pairs: as for
// launch_bvh8, the records launch_hploc_batch wrote (mesh m's at off[m]).
cudaError_t launch_bvh8_batch(const Node2* bvh2, const MeshBatch& batch, uint32_t total, Node8* out, uint32_t slots,
                              uint32_t* prim_idx, uint64_t* pairs, uint32_t* ctr, uint32_t* mesh_nodes,
                              uint32_t* mesh_leaves, uint32_t* err, bool auction, cudaStream_t s,
                              const ChildPair* child_pairs = nullptr);
cudaError_t launch_batch_finalize(const MeshBatch& batch, const uint32_t* scene_ord, const uint32_t* mesh_nodes,
                                  const uint32_t* mesh_leaves, nxb_batch_mesh* out, cudaStream_t s);
// One batched build's device memory (a single allocation carved into
// 256-byte aligned segments; batch.cu).  off/off8 hold the mesh offsets and
// the BVH8 offsets; results receives one nxb_batch_mesh per mesh.
struct BatchCtrl {
    uint32_t error_word;
    uint32_t pad[31];
    uint32_t leaf_ctr[kMaxMeshGroups];  // one H-PLOC leaf counter per mesh group
    uint32_t pad2[32 - kMaxMeshGroups];
    uint32_t tile_ctr[kMaxSortPasses];
    uint32_t hist[kMaxSortPasses][kRadixBins];
};
struct BatchArena {
    uint32_t meshes = 0, total = 0, slots = 0, mesh_bits = 0;
    size_t bytes = 0;
    uint32_t* off = nullptr;
    uint32_t* off8 = nullptr;
    unsigned char* zero_begin = nullptr;
    size_t zero_bytes = 0;
    BatchCtrl* ctrl = nullptr;
    uint32_t* scene_ord = nullptr;
    uint32_t* parent = nullptr;  // then parent_of_last, one word per mesh
    uint32_t* pol = nullptr;
    size_t ones_words = 0;
    uint32_t* lookback = nullptr;
    size_t lookback_words_per_pass = 0;
    uint32_t* ctr8 = nullptr;
    uint32_t* mesh_nodes = nullptr;
    uint32_t* mesh_leaves = nullptr;
    uint2* tile_rng = nullptr;  // mesh range of each bounds/Morton tile (up to total / 128 tiles)
    uint64_t* keys_a = nullptr;
    uint64_t* keys_b = nullptr;
    uint32_t* vals_a = nullptr;
    uint32_t* vals_b = nullptr;
    uint64_t* pairs = nullptr;
    ChildPair* kids = nullptr;  // child-pair records (one per primitive, 64-byte aligned)
    Node2* bvh2 = nullptr;
    Node8* bvh8 = nullptr;
    uint32_t* prim_idx = nullptr;
    nxb_batch_mesh* results = nullptr;
};
struct BatchTuning {
    uint32_t digit_bits = 8, radius = 8, hploc_ctas_per_sm = 0;
    bool auction = false;
    uint32_t groups = 1;   // BVH2/BVH8 fusion point: mesh groups (needs a BatchFork when > 1)
    uint32_t block = 256;  // CTA size of the bounds and Morton tile kernels
};
// A second stream and two events per mesh group: the BVH8 collapse of group
// g runs on `side` after H-PLOC of group g (event hploc[g]) while H-PLOC of
// group g+1 runs on the main stream; `join` brings the side stream back.
struct BatchFork {
    cudaStream_t side;
    cudaEvent_t hploc[kMaxMeshGroups];
    cudaEvent_t join;
};
// BVH8 node capacity of one mesh (the reference's ceil((4n-1)/7); 1 for an
// empty mesh, so that BVH8 offsets are strictly increasing).
uint32_t batch_bvh8_capacity(uint32_t n);
// Sizes the arena for meshes with host offsets h_off[0..meshes] and fills
// h_off8[0..meshes]; returns false if the batch is too large.  The device
// pointers stay null until batch_bind.
bool batch_layout(const uint32_t* h_off, uint32_t meshes, uint32_t* h_off8, BatchArena* a);
void batch_bind(unsigned char* base, BatchArena* a);
bool batch_digit_ok(uint32_t mesh_bits, uint32_t digit_bits);
// Cuts meshes [0, meshes) with host offsets h_off / h_off8 into at most
// `want` groups of about equal primitive counts (never an empty group).
void batch_groups(const uint32_t* h_off, const uint32_t* h_off8, uint32_t meshes, uint32_t want, MeshGroups* g);
// The batched pipeline on stream s; off/off8 must already be on the device.
// If h_err is not null, the error word is copied there at the end.  With
// groups (count > 1) and a fork, H-PLOC runs group by group on s and the
// collapse of each group follows on fork->side, overlapping H-PLOC of the
// next group; without, the whole batch is one group.
nxb_status batch_enqueue(const BatchArena& a, const void* prims, nxb_prim_type type, const BatchTuning& t,
                         uint32_t* h_err, cudaStream_t s, const MeshGroups* groups = nullptr,
                         const BatchFork* fork = nullptr);
// ---------------------------------------------------------------- eval
cudaError_t launch_bvh2_cost(const Node2* nodes, uint32_t count, const nxb_aabb* root, float* cost, cudaStream_t s);
cudaError_t launch_bvh8_cost(const Node8* nodes, uint32_t count, const nxb_aabb* root, float* cost, cudaStream_t s);
// Device-side validity checks (validate.cu); scratch sizes in bytes.
size_t validate_bvh2_scratch(uint32_t n);
size_t validate_bvh8_scratch(uint32_t node_count, uint32_t n);
cudaError_t launch_validate_bvh2(const Node2* nodes, uint32_t n, uint32_t root, uint64_t* report, void* scratch,
                                 cudaStream_t s);
cudaError_t launch_validate_bvh8(const Node8* nodes, uint32_t node_count, const uint32_t* prim_idx, uint32_t n,
                                 const void* prims, int prim_type, uint64_t* report, void* scratch, cudaStream_t s);
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
