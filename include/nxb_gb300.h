/*
 * nxb_gb300.h - C ABI of the GB300 (sm_103a) BVH build pipeline.
 *
 * The pipeline is: scene bounds + leaf write -> 30/63-bit Morton codes ->
 * stable key-value radix sort -> H-PLOC binary BVH (BVH2) -> compressed
 * 8-wide BVH (BVH8, 80-byte nodes with 8-bit quantised child boxes).
 *
 * Every entry point takes plain pointers and sizes, returns an nxb_status and
 * never terminates the process.  Device pointers are CUDA global-memory
 * pointers on the current device; every launch goes to the stream given
 * (NULL = legacy default stream, which is what NexusBVH uses).
 *
 * Reference interfaces replaced (paths inside the NexusBVH project):
 *   NXB::BuildBVH2<PrimT>   NexusBVH/include/NXB/BVHBuilder.h:18-31,
 *                           NexusBVH/src/BVHBuilder.cpp:114-171
 *   NXB::BuildBVH8<PrimT>   NexusBVH/include/NXB/BVHBuilder.h:32-43,
 *                           NexusBVH/src/BVHBuilder.cpp:173-267
 *   NXB::ToHost / FreeHostBVH / FreeDeviceBVH
 *                           NexusBVH/include/NXB/BVHBuilder.h:45-55,
 *                           NexusBVH/src/BVHBuilder.cpp:269-294
 * The per-stage entry points (nxb_stage_*) replace the kernels the host
 * builder launches one by one:
 *   ComputeSceneBoundsKernel  NexusBVH/src/Cuda/Setup.cu:12-39
 *   ComputeMortonCodesKernel  NexusBVH/src/Cuda/Setup.cu:42-59
 *   RadixSort                 NexusBVH/src/Cuda/Setup.cu:62-112
 *   BuildBVH2Kernel           NexusBVH/src/Cuda/BinaryBuilder.cu:200-273
 *   BuildBVH8Kernel           NexusBVH/src/Cuda/WideConverter.cu:225-414
 *   ComputeBVH2CostKernel / ComputeBVH8CostKernel
 *                             NexusBVH/src/Cuda/Eval.cu:12-80
 *
 * The struct layouts below are byte-identical to the reference's
 * NXB::AABB (24 B), NXB::Triangle (36 B), NXB::BVH2::Node (32 B),
 * NXB::BVH8::Node (80 B), NXB::BVH2 (40 B), NXB::BVH8 (56 B) and
 * NXB::BVHBuildMetrics (36 B) (NexusBVH/include/NXB/AABB.h:8-53,
 * Triangle.h:10-47, BVH.h:8-96, BVHBuildMetrics.h:7-50), so arrays built
 * here can be handed to code written against the reference unchanged.
 */
#ifndef NXB_GB300_H
#define NXB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct CUstream_st; /* cudaStream_t is `struct CUstream_st*` */

#define NXB_INVALID_IDX 0xFFFFFFFFu

/* ------------------------------------------------------------------ status */
typedef enum nxb_status {
    NXB_OK = 0,
    NXB_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad prim type, n == 0, ... */
    NXB_ERR_UNSUPPORTED = 2,      /* a size or option this build does not support */
    NXB_ERR_OUT_OF_MEMORY = 3,    /* a device allocation was refused */
    NXB_ERR_CUDA = 4,             /* a CUDA runtime call failed (see nxb_last_cuda_error) */
    NXB_ERR_WORKSPACE_TOO_SMALL = 5,
    NXB_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait gave up (error word set) */
    NXB_ERR_DEVICE_INVARIANT = 7, /* a kernel found an impossible state (error word set), or
                                     NXB_BUILD_VALIDATE found an invalid tree */
    NXB_ERR_ADMISSION = 8,        /* server: the request does not fit the memory budget */
    NXB_ERR_IO = 9                /* a BVH file could not be opened, read or written, or is not
                                     a BVH file of this format */
} nxb_status;

/* Returns a static, human-readable name for a status code. */
const char* nxb_status_string(nxb_status status);
/* Last CUDA error code seen by this thread inside the library (0 if none). */
int nxb_last_cuda_error(void);

/* ------------------------------------------------------------------- types */
/* Values match NXB::PrimType (NexusBVH/include/NXB/BVH.h:12-16). */
typedef enum nxb_prim_type { NXB_PRIM_AABB = 0, NXB_PRIM_TRIANGLE = 1 } nxb_prim_type;

typedef struct nxb_aabb {      /* NXB::AABB, 24 B */
    float bmin[3];
    float bmax[3];
} nxb_aabb;

typedef struct nxb_triangle {  /* NXB::Triangle, 36 B */
    float v0[3], v1[3], v2[3];
} nxb_triangle;

typedef struct nxb_bvh2_node { /* NXB::BVH2::Node, 32 B */
    nxb_aabb bounds;
    uint32_t left;  /* NXB_INVALID_IDX for a leaf */
    uint32_t right; /* primitive index for a leaf */
} nxb_bvh2_node;

typedef struct nxb_bvh8_node { /* NXB::BVH8::Node / NodeExplicit, 80 B */
    float p[3];            /* origin of the child grid */
    uint8_t e[3];          /* biased exponents of the grid scale */
    uint8_t imask;         /* bit i: child slot i is an inner node */
    uint32_t child_base;   /* index of the first inner child node */
    uint32_t prim_base;    /* index of the first leaf in prim_idx[] */
    uint8_t meta[8];       /* 0 = empty; 0x20|(24+i) inner; 0x20|rank leaf */
    uint8_t qlo[3][8];     /* qlox, qloy, qloz */
    uint8_t qhi[3][8];     /* qhix, qhiy, qhiz */
} nxb_bvh8_node;

typedef struct nxb_bvh2 {      /* NXB::BVH2, 40 B */
    nxb_bvh2_node* nodes;  /* 2n-1 nodes: leaves [0,n), internal [n,2n-1), root 2n-2 */
    uint32_t node_count;
    uint32_t prim_count;
    nxb_aabb bounds;       /* root (= scene) bounds, host copy */
} nxb_bvh2;

typedef struct nxb_bvh8 {      /* NXB::BVH8, 56 B */
    nxb_bvh8_node* nodes;  /* root is node 0 */
    uint32_t node_count;
    uint32_t* prim_idx;    /* n entries, one primitive per leaf */
    uint32_t prim_count;
    nxb_aabb bounds;
} nxb_bvh8;

/* NXB::BVHBuildMetrics (NexusBVH/include/NXB/BVHBuildMetrics.h:7-50), 36 B.
 * Times are CUDA-event milliseconds per stage; total_time is the sum of the
 * stage times, exactly as the reference defines it
 * (NexusBVH/src/BVHBuilder.cpp:75-76,223). Costs are only filled when
 * metrics are requested. */
typedef struct nxb_build_metrics {
    float scene_bounds_time;
    float morton_codes_time;
    float radix_sort_time;
    float bvh2_build_time;
    float bvh8_conversion_time;
    float total_time;
    float bvh2_cost;
    float bvh8_cost;
    float average_child_per_node;
} nxb_build_metrics;

/* NXB::BuildConfig (NexusBVH/include/NXB/BuildConfig.h:6-12) plus the knobs
 * the reference fixes at compile time (SEARCH_RADIUS, BinaryBuilder.cu:9).
 * Zero-initialise and set what you need: zero means "reference default". */
typedef struct nxb_build_config {
    uint32_t prioritize_speed; /* nonzero: 30-bit Morton in 32-bit keys; else 63-bit in 64-bit keys */
    uint32_t search_radius;    /* H-PLOC nearest-neighbour radius: 0 (= 8), 4, 8 or 16 */
    uint32_t flags;            /* NXB_BUILD_* bits; 0 = the reference's default build */
    uint32_t reserved;
} nxb_build_config;

/* BVH8 child-slot assignment by the auction algorithm, the reference's
 * compile-time alternative to the greedy assignment (USE_AUCTION,
 * NexusBVH/src/Cuda/WideConverter.cu:5,50-102,337-358; off in the reference's
 * build).  Same tree and boxes, different child order inside BVH8 nodes. */
#define NXB_BUILD_AUCTION 0x1u
/* Plain calls (nxb_build_bvh2 / nxb_build_bvh8) only: after the build, check
 * the trees on the device (nxb_validate_bvh2, and nxb_validate_bvh8 for a
 * BVH8 build, whose intermediate BVH2 is checked too) and return
 * NXB_ERR_DEVICE_INVARIANT, with no tree, when one is invalid.  The other
 * entry points answer NXB_ERR_UNSUPPORTED; their callers run the
 * validators themselves. */
#define NXB_BUILD_VALIDATE 0x2u

/* -------------------------------------------- reference-shaped entry points */
/* Builds a BVH2 from n device primitives (nxb_triangle or nxb_aabb).  The
 * input is not modified.  out->nodes is allocated here (stream-ordered) and
 * owned by the caller (nxb_free_device_bvh2).  Synchronises the stream before
 * returning, like the reference.  metrics may be NULL; when given, stage
 * times are measured with CUDA events and the SAH cost is computed. */
nxb_status nxb_build_bvh2(const void* d_prims, nxb_prim_type prim_type, uint32_t prim_count,
                          const nxb_build_config* config, struct CUstream_st* stream,
                          nxb_bvh2* out_bvh, nxb_build_metrics* metrics);

/* Builds a compressed BVH8 (through a BVH2 that is freed before returning).
 * out->nodes and out->prim_idx are owned by the caller (nxb_free_device_bvh8). */
nxb_status nxb_build_bvh8(const void* d_prims, nxb_prim_type prim_type, uint32_t prim_count,
                          const nxb_build_config* config, struct CUstream_st* stream,
                          nxb_bvh8* out_bvh, nxb_build_metrics* metrics);

/* Synchronous device -> host copy of a BVH2 into malloc'd memory. */
nxb_status nxb_bvh2_to_host(const nxb_bvh2* device_bvh, nxb_bvh2* host_bvh);
nxb_status nxb_free_host_bvh2(nxb_bvh2* host_bvh);
/* The same for a BVH8 (nodes and prim_idx).  The reference has no BVH8
 * host export; this is the BVH2 ToHost contract applied to the BVH8. */
nxb_status nxb_bvh8_to_host(const nxb_bvh8* device_bvh, nxb_bvh8* host_bvh);
nxb_status nxb_free_host_bvh8(nxb_bvh8* host_bvh);
nxb_status nxb_free_device_bvh2(nxb_bvh2* device_bvh);
nxb_status nxb_free_device_bvh8(nxb_bvh8* device_bvh);

/* On-disk form of a host BVH (the node layouts of NexusBVH/include/NXB/BVH.h:20-86, which the
 * reference keeps in memory only).  A file is a 64-byte header -- magic "NXBVH2\0\0" or
 * "NXBVH8\0\0", format version 1, node count, primitive count, node size in bytes (32 or 80),
 * root bounds -- then the nodes in their in-memory layout and, for a BVH8, prim_idx; all
 * little-endian.  Writing takes a host BVH (nxb_bvh*_to_host, or a file read back); reading
 * fills malloc'd arrays that nxb_free_host_bvh* frees, and checks the magic, the version, the
 * node size, the counts and the file length, returning NXB_ERR_IO when any is wrong. */
nxb_status nxb_write_bvh2(const char* path, const nxb_bvh2* host_bvh);
nxb_status nxb_read_bvh2(const char* path, nxb_bvh2* host_bvh);
nxb_status nxb_write_bvh8(const char* path, const nxb_bvh8* host_bvh);
nxb_status nxb_read_bvh8(const char* path, nxb_bvh8* host_bvh);

/* ------------------------------------- allocation-free (workspace) builds */
/* Sizes, in bytes, of what a build of prim_count primitives needs.  All
 * device buffers must be 256-byte aligned (cudaMalloc alignment). */
typedef struct nxb_build_sizes {
    size_t workspace_bytes;  /* scratch: keys, values, sort state, counters, H-PLOC cluster records and
                              * the child-pair records a BVH8 build reads (64 bytes per primitive; a
                              * build without a BVH8 may pass a workspace that much smaller) */
    size_t bvh2_node_count;  /* 2n-1 */
    size_t bvh8_node_capacity; /* ceil((4n-1)/7), the reference's worst case */
} nxb_build_sizes;

nxb_status nxb_query_build_sizes(uint32_t prim_count, const nxb_build_config* config,
                                 nxb_build_sizes* out_sizes);

/* Device-side results of an asynchronous build (written by the kernels). */
typedef struct nxb_build_result {
    nxb_aabb scene_bounds;
    uint32_t bvh8_node_count;
    uint32_t bvh8_leaf_count;
    uint32_t error_word;   /* 0 = fine; else an NXB_DEVERR_* bit set */
    uint32_t bvh2_root;    /* 2n-2 */
} nxb_build_result;

#define NXB_DEVERR_SORT_LOOKBACK_TIMEOUT 0x1u
#define NXB_DEVERR_BVH8_QUEUE_TIMEOUT    0x2u
#define NXB_DEVERR_HPLOC_INVALID_CLUSTER 0x4u
#define NXB_DEVERR_BVH8_OVERFLOW         0x8u

/* Enqueues the whole BVH2 (+ optional BVH8) build on `stream` with no
 * allocation, no host synchronisation and no host<->device copy, so it can
 * be captured in a CUDA graph.  d_bvh8_nodes / d_prim_idx may be NULL to
 * stop after the BVH2.  d_result receives the counters and the error word. */
nxb_status nxb_build_async(const void* d_prims, nxb_prim_type prim_type, uint32_t prim_count,
                           const nxb_build_config* config, void* d_workspace,
                           size_t workspace_bytes, nxb_bvh2_node* d_bvh2_nodes,
                           nxb_bvh8_node* d_bvh8_nodes, uint32_t* d_prim_idx,
                           nxb_build_result* d_result, struct CUstream_st* stream);

/* nxb_build_async that also records six caller-created CUDA events
 * (cudaEvent_t handles) on `stream` at the stage boundaries: before scene
 * bounds, after bounds, after Morton, after the sort, after H-PLOC, after
 * the BVH8 collapse.  Used to time each stage on the launching stream. */
nxb_status nxb_build_async_timed(const void* d_prims, nxb_prim_type prim_type, uint32_t prim_count,
                                 const nxb_build_config* config, void* d_workspace,
                                 size_t workspace_bytes, nxb_bvh2_node* d_bvh2_nodes,
                                 nxb_bvh8_node* d_bvh8_nodes, uint32_t* d_prim_idx,
                                 nxb_build_result* d_result, struct CUstream_st* stream,
                                 void* const* stage_events);

/* ------------------------------------------------------ per-stage entries */
/* Stage 1 (ComputeSceneBoundsKernel): leaf i of d_nodes = {bounds(prim i),
 * INVALID, i}; *d_scene = union of all leaf bounds. */
nxb_status nxb_stage_scene_bounds(const void* d_prims, nxb_prim_type prim_type,
                                  uint32_t prim_count, nxb_bvh2_node* d_nodes,
                                  nxb_aabb* d_scene, struct CUstream_st* stream);

/* Stage 2 (ComputeMortonCodesKernel): key i = Morton code of leaf i's
 * centroid normalised by *d_scene (key_bits 30 -> uint32 keys, 63 -> uint64);
 * d_cluster_idx[i] = i (may be NULL). */
nxb_status nxb_stage_morton(const nxb_bvh2_node* d_nodes, uint32_t prim_count,
                            const nxb_aabb* d_scene, uint32_t key_bits, void* d_keys,
                            uint32_t* d_cluster_idx, struct CUstream_st* stream);

/* Stage 3 (RadixSort): stable sort of (key, value) pairs by key bits
 * [begin_bit, end_bit); full keys are carried.  Sorted output lands in
 * d_keys_out / d_vals_out; the inputs are left unmodified.  d_vals_in NULL
 * means values 0..n-1.  Scratch: nxb_sort_scratch_bytes(). */
size_t nxb_sort_scratch_bytes(uint32_t count, uint32_t key_bytes, uint32_t begin_bit,
                              uint32_t end_bit);
nxb_status nxb_stage_radix_sort(uint32_t key_bytes, const void* d_keys_in, void* d_keys_out,
                                const uint32_t* d_vals_in, uint32_t* d_vals_out,
                                uint32_t count, uint32_t begin_bit, uint32_t end_bit,
                                void* d_scratch, size_t scratch_bytes, uint32_t* d_error_word,
                                struct CUstream_st* stream);

/* Stage 3 without caller scratch: this entry point has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory or
 * pass this library a scratch buffer: for example a renderer rebuilding
 * BVHs in its frame loop (cudaMalloc and cudaFree synchronise the whole
 * device and stall the frame), or an engine whose device memory belongs to
 * its own sub-allocator.  Same arguments and results as
 * nxb_stage_radix_sort, minus the scratch: the scratch is a fixed array of
 * about 3.7 MB inside the library, which every GPU that loads the library
 * holds until the process exits.  It allocates nothing (no cudaMalloc,
 * cudaFree or allocating library call).
 *   - count may be at most NXB_NOALLOC_SORT_MAX_COUNT; larger counts return
 *     NXB_ERR_UNSUPPORTED (use nxb_stage_radix_sort for those).
 *   - The first call on a device is not yet allocation-free: with CUDA's
 *     lazy module loading (the default) it loads the library's kernels on
 *     that device, which creates the array and may synchronise, and it looks
 *     up the array's device address with that device current.  Make that
 *     first call once at start-up, outside the frame loop and before any
 *     stream capture; later calls on that device allocate nothing.
 *   - The address is kept per device for the life of the process: after
 *     cudaDeviceReset the array may move, so do not use this entry point in
 *     a process that resets a device it has already used.
 *   - Every call, from any thread or stream, shares the one array: calls
 *     whose work overlaps on the GPU race and corrupt each other's results.
 *     Order them on one stream (or wait on the previous call's work). */
#define NXB_NOALLOC_SORT_MAX_COUNT 262144u
nxb_status nxb_stage_radix_sort_noalloc(uint32_t key_bytes, const void* d_keys_in, void* d_keys_out,
                                        const uint32_t* d_vals_in, uint32_t* d_vals_out, uint32_t count,
                                        uint32_t begin_bit, uint32_t end_bit, uint32_t* d_error_word,
                                        struct CUstream_st* stream);

/* Stage 4 (BuildBVH2Kernel): H-PLOC over sorted keys; d_cluster_idx is the
 * sorted permutation (treat its contents as undefined afterwards); d_nodes
 * leaves [0,n) must hold the stage-1 output; internal nodes are written to
 * [n, 2n-1).  Scratch: nxb_hploc_scratch_bytes() (about 40 bytes per
 * primitive: hand-over slots, tokens and 32-byte cluster records). */
size_t nxb_hploc_scratch_bytes(uint32_t prim_count);
nxb_status nxb_stage_hploc(uint32_t key_bytes, const void* d_sorted_keys,
                           uint32_t* d_cluster_idx, nxb_bvh2_node* d_nodes,
                           uint32_t prim_count, uint32_t search_radius, void* d_scratch,
                           size_t scratch_bytes, uint32_t* d_error_word,
                           struct CUstream_st* stream);

/* Stage 5 (BuildBVH8Kernel): collapse the BVH2 rooted at node 2n-2 into a
 * BVH8 rooted at node 0.  d_counts receives {node_count, leaf_count}.
 * Scratch: nxb_bvh8_scratch_bytes(). */
size_t nxb_bvh8_scratch_bytes(uint32_t prim_count);
nxb_status nxb_stage_bvh8(const nxb_bvh2_node* d_bvh2_nodes, uint32_t prim_count,
                          nxb_bvh8_node* d_bvh8_nodes, uint32_t* d_prim_idx,
                          uint32_t* d_counts, void* d_scratch, size_t scratch_bytes,
                          uint32_t* d_error_word, struct CUstream_st* stream);
/* The same with NXB_BUILD_* flags (NXB_BUILD_AUCTION selects the auction
 * slot assignment). */
nxb_status nxb_stage_bvh8_ex(const nxb_bvh2_node* d_bvh2_nodes, uint32_t prim_count,
                             nxb_bvh8_node* d_bvh8_nodes, uint32_t* d_prim_idx,
                             uint32_t* d_counts, void* d_scratch, size_t scratch_bytes,
                             uint32_t build_flags, uint32_t* d_error_word,
                             struct CUstream_st* stream);

/* Cost evaluation (Eval.cu): SAH of a BVH2 (all 2n-1 nodes) and the cost of
 * a BVH8 (children only), relative to the root area; *d_cost is overwritten. */
nxb_status nxb_eval_bvh2_cost(const nxb_bvh2_node* d_nodes, uint32_t node_count,
                              const nxb_aabb* d_root_bounds, float* d_cost,
                              struct CUstream_st* stream);
nxb_status nxb_eval_bvh8_cost(const nxb_bvh8_node* d_nodes, uint32_t node_count,
                              const nxb_aabb* d_root_bounds, float* d_cost,
                              struct CUstream_st* stream);

/* Device-side validity checks: the checks of an exhaustive tree validator,
 * run data-parallel on the GPU so that a full-size tree is checked without
 * copying it to the host (the reference has no validator; the trees are the
 * ones BuildBVH2Kernel / BuildBVH8Kernel write, BinaryBuilder.cu:200-273,
 * WideConverter.cu:225-330).  Enqueued on `stream` with no host
 * synchronisation and no allocation; d_report (device) is overwritten when
 * the work runs.  Scratch: nxb_validate_bvh2/8_scratch_bytes().  "Reached"
 * means the node's chain of parent references ends at the root.
 *
 * BVH2: prim_count leaves, 2*prim_count-1 nodes, root `root`.  d_report gets
 * NXB_BVH2_CHECK_FIELDS words: [0] nodes reached (root included), [1] leaves
 * among them, [2] extra copies of primitives held by several reached leaves,
 * [3] primitives held by no reached leaf, [4] reached internal nodes whose
 * box is not bit for bit the union of their children's, [5] children of
 * reached nodes not contained in their parent's box, [6] reached nodes with a
 * child or primitive index out of range, [7] maximum depth (root 0), [8]
 * extra parent references (beyond one per node, all of them for the root),
 * [9] errors = [2]+[3]+[4]+[5]+[6]+[8] + ([0] != 2n-1) + ([1] != n).
 * A tree is valid when [9] is 0. */
#define NXB_BVH2_CHECK_FIELDS 10
size_t nxb_validate_bvh2_scratch_bytes(uint32_t prim_count);
nxb_status nxb_validate_bvh2(const nxb_bvh2_node* d_nodes, uint32_t prim_count, uint32_t root,
                             uint64_t* d_report, void* d_scratch, size_t scratch_bytes,
                             struct CUstream_st* stream);
/* BVH8: node_count nodes rooted at node 0, d_prim_idx[prim_count]; the
 * primitives (d_prims, prim_type) give the exact leaf boxes.  d_report gets
 * NXB_BVH8_CHECK_FIELDS words: [0] nodes reached, [1] leaf slots among them,
 * [2] extra copies of primitives, [3] primitives in no leaf slot, [4] bad
 * indices (inner child out of range, extra references of a node or any of
 * the root, leaf slot or primitive index out of range), [5] / [6] decoded
 * lower / upper child bounds p + 2^(e-127)*q (evaluated in double) that lie
 * inside the exact box of the child's primitives, per axis, [7] slots used,
 * [8] maximum depth, [9] meta errors (an inner bit on an empty slot, or a
 * meta byte other than 0x20|(24+slot) for an inner child and 0x20|rank for a
 * leaf), [10] errors = [2]+[3]+[4]+[9] + ([0] != node_count) +
 * ([1] != prim_count).  Conservativeness ([5], [6]) is reported and not
 * counted in [10]. */
#define NXB_BVH8_CHECK_FIELDS 11
size_t nxb_validate_bvh8_scratch_bytes(uint32_t node_count, uint32_t prim_count);
nxb_status nxb_validate_bvh8(const nxb_bvh8_node* d_nodes, uint32_t node_count,
                             const uint32_t* d_prim_idx, uint32_t prim_count, const void* d_prims,
                             nxb_prim_type prim_type, uint64_t* d_report, void* d_scratch,
                             size_t scratch_bytes, struct CUstream_st* stream);

/* ------------------------------------------------------------ batched builds */
/* No counterpart in the reference's API, which builds one mesh per call
 * (NXB::BuildBVH8, NexusBVH/include/NXB/BVHBuilder.h:18-31).  A batch builds
 * many independent meshes, concatenated in one device array, with one
 * launch per stage over all of them, replayed from a CUDA graph.  Each mesh
 * is built exactly as a plain build of that mesh alone would build it (own
 * scene box, same Morton codes, same sort order, same H-PLOC decisions, same
 * BVH8 collapse): only BVH8 node numbering differs, as it does between two
 * plain builds.  Batches use 30-bit Morton codes (config->prioritize_speed
 * must be nonzero).  Results live in batch-owned device memory, valid until
 * the next build of the batch or nxb_batch_destroy. */
typedef struct nxb_batch nxb_batch; /* opaque */

typedef struct nxb_batch_mesh {        /* per-mesh result, 52 B */
    nxb_aabb scene_bounds;             /* this mesh's own scene box */
    uint32_t prim_offset, prim_count;  /* its primitives in the input; its prim_idx slice */
    uint32_t bvh2_offset;              /* its BVH2 nodes start here (leaves first, root at +2n-2) */
    uint32_t bvh2_node_count;          /* 2n-1 (0 for an empty mesh) */
    uint32_t bvh8_offset;              /* its BVH8 nodes start here, root first */
    uint32_t bvh8_node_count, bvh8_leaf_count;
} nxb_batch_mesh;

/* Indices are mesh-local, so each mesh's trees are standalone: nxb_validate_bvh2
 * on bvh2_nodes + bvh2_offset (prim_count leaves, root 2n-2) and nxb_validate_bvh8
 * on bvh8_nodes + bvh8_offset, prim_idx + prim_offset and the mesh's primitives
 * check one mesh in place. */
typedef struct nxb_batch_arrays {      /* device views owned by the batch */
    const nxb_bvh2_node* bvh2_nodes;   /* child indices are mesh-local */
    const nxb_bvh8_node* bvh8_nodes;   /* child_base / prim_base are mesh-local */
    const uint32_t* prim_idx;          /* mesh-local primitive indices */
    const nxb_batch_mesh* meshes;      /* [mesh_count], written by every build */
    uint32_t mesh_count;
    uint32_t prim_count;
    size_t bvh2_node_capacity, bvh8_node_capacity;
} nxb_batch_arrays;

typedef struct nxb_batch_tuning {
    uint32_t sort_digit_bits;   /* 4..8: bits per radix sort pass (at most 10 passes) */
    uint32_t search_radius;     /* H-PLOC radius in use */
    uint32_t hploc_ctas_per_sm; /* cap on the H-PLOC persistent grid (0 = occupancy) */
    uint32_t fusion_groups;     /* BVH2/BVH8 fusion point: 0 or 1 = collapse after H-PLOC has built
                                   every mesh; 2..8 = meshes cut into that many groups of about equal
                                   triangle count, the BVH8 collapse of each group running while
                                   H-PLOC builds the next */
    uint32_t block_size;        /* threads per CTA of the bounds and Morton kernels: 128, 256 or 512 */
    uint32_t candidates_tried;
    float build_ms;             /* median time of one build with these settings */
} nxb_batch_tuning;

/* Tuning flags for nxb_batch_autotune. */
#define NXB_TUNE_RADIUS 0x1u /* also try radius 4, 8 and 16: this changes the trees */

/* Creates a batch for mesh_count meshes whose primitive counts are given as
 * a host prefix array h_prim_offsets[0..mesh_count] (h_prim_offsets[0] = 0,
 * non-decreasing; empty meshes allowed).  Allocates all device memory the
 * batch needs on the current device (one allocation). */
nxb_status nxb_batch_create(nxb_prim_type prim_type, const uint32_t* h_prim_offsets, uint32_t mesh_count,
                            const nxb_build_config* config, nxb_batch** out_batch);
nxb_status nxb_batch_destroy(nxb_batch* batch);
/* Enqueues one build of the batch from d_prims (all meshes' primitives end
 * to end) on `stream`: a graph launch, nothing else (the graph is captured
 * on the first call and again when d_prims or the tuning changes).  No host
 * synchronisation; nxb_batch_wait reports the outcome. */
nxb_status nxb_batch_build_async(nxb_batch* batch, const void* d_prims, struct CUstream_st* stream);
/* Waits for `stream`, checks the device error word and, if h_meshes is not
 * NULL, copies the mesh_count per-mesh results into it. */
nxb_status nxb_batch_wait(nxb_batch* batch, struct CUstream_st* stream, nxb_batch_mesh* h_meshes);
/* nxb_batch_build_async + nxb_batch_wait. */
nxb_status nxb_batch_build(nxb_batch* batch, const void* d_prims, struct CUstream_st* stream,
                           nxb_batch_mesh* h_meshes);
nxb_status nxb_batch_get_arrays(const nxb_batch* batch, nxb_batch_arrays* out_arrays);
/* Times candidate settings on this batch and input (each: one warm-up build,
 * then the median of `repeats` builds) and keeps the fastest.  Without
 * NXB_TUNE_RADIUS only settings that leave the results unchanged are tried
 * (sort digit width, H-PLOC grid size, BVH2/BVH8 fusion point). */
nxb_status nxb_batch_autotune(nxb_batch* batch, const void* d_prims, uint32_t tune_flags, uint32_t repeats,
                              struct CUstream_st* stream, nxb_batch_tuning* out_choice);
nxb_status nxb_batch_set_tuning(nxb_batch* batch, const nxb_batch_tuning* tuning);
nxb_status nxb_batch_get_tuning(const nxb_batch* batch, nxb_batch_tuning* out_tuning);
/* Host copy of one mesh's BVH8 (like nxb_bvh8_to_host; free with
 * nxb_free_host_bvh8) after a successful build. */
nxb_status nxb_batch_mesh_bvh8_to_host(const nxb_batch* batch, uint32_t mesh, nxb_bvh8* host_bvh);

/* ------------------------------------------------------------- build server */
/* No counterpart in the reference's API.  A build server for a stream of
 * independent requests (one mesh each): requests are admitted against a
 * device-memory budget, started as soon as a stream slot and memory are free
 * (continuous batching: small requests of the same prim type that wait at
 * the same time are built together by the batched pipeline, one launch per
 * stage; large or 63-bit requests run the plain pipeline), and their BVH8s
 * kept in server memory until released.  A request's result is the one a
 * plain build of that mesh alone gives (same tree, boxes and quantisation;
 * only BVH8 node numbering may differ, as between two plain builds).
 * One worker thread per server drives the GPU; every call is thread-safe. */
typedef struct nxb_server nxb_server; /* opaque */

typedef struct nxb_server_config {
    size_t memory_budget_bytes; /* device memory held at once: inputs, scratch, results (0 = 32 GiB) */
    uint32_t streams;           /* builds in flight at once (0 = 4) */
    uint32_t batch_max_prims;   /* requests up to this size may share a batched build (0 = 65536; 1 = never) */
    uint32_t batch_max_meshes;  /* meshes per batched build (0 = 256) */
    uint32_t flags;             /* NXB_SERVER_* bits */
} nxb_server_config;

/* Reserve the whole budget in the server's memory pool at creation, so that
 * no request waits for the pool to grow (creation then takes longer). */
#define NXB_SERVER_RESERVE 0x1u

typedef struct nxb_server_result {
    nxb_bvh8 bvh8;          /* device arrays owned by the server until nxb_server_release */
    int32_t status;         /* nxb_status of the build */
    uint32_t batched_with;  /* meshes in the build that produced it (1 = built alone) */
    double queue_ms;        /* submit -> launch (host clock) */
    double latency_ms;      /* submit -> completion seen by the server (host clock) */
    /* The build's work on the GPU, in milliseconds since the server was
     * created, from events recorded on its stream before its first operation
     * (the input copy or the build) and after its last (the result copies):
     * requests whose intervals intersect had work on the GPU at the same
     * time.  Requests built together share one interval. */
    double device_start_ms;
    double device_end_ms;
} nxb_server_result;

typedef struct nxb_server_stats {
    /* builds: GPU builds started; batched_builds: those that built more than
     * one request; batched_requests: the requests those built */
    uint64_t submitted, completed, rejected, builds, batched_builds, batched_requests;
    size_t bytes_in_use, peak_bytes_in_use;
} nxb_server_stats;

/* Creates a server on the current device.  Before returning it runs one tiny build through
 * each pipeline it serves at the default radius (plain 30- and 63-bit, batched; triangles and
 * boxes), so that the CUDA runtime has loaded those kernels before the first request arrives. */
nxb_status nxb_server_create(const nxb_server_config* config, nxb_server** out_server);
/* Waits for the builds in flight, then frees everything (unreleased results too). */
nxb_status nxb_server_destroy(nxb_server* server);
/* Queues one build.  prims is a device pointer if prims_on_device is nonzero,
 * else host memory (pinned for best latency); either way it must stay valid
 * until the request completes.  config as for nxb_build_bvh8 (may be NULL).
 * Returns NXB_ERR_ADMISSION if the request alone needs more than the budget. */
nxb_status nxb_server_submit(nxb_server* server, const void* prims, int prims_on_device,
                             nxb_prim_type prim_type, uint32_t prim_count,
                             const nxb_build_config* config, uint64_t* out_ticket);
/* Blocks until the request completes; fills *out (its status is also returned). */
nxb_status nxb_server_wait(nxb_server* server, uint64_t ticket, nxb_server_result* out);
/* Non-blocking: *done = 1 and *out filled if the request has completed. */
nxb_status nxb_server_poll(nxb_server* server, uint64_t ticket, nxb_server_result* out, int* done);
/* Frees a completed request's result memory and forgets the ticket. */
nxb_status nxb_server_release(nxb_server* server, uint64_t ticket);
nxb_status nxb_server_get_stats(nxb_server* server, nxb_server_stats* out);

/* Library version and the compile flags that define its numerics. */
const char* nxb_version(void);

/* Diagnostics: evaluates, on the current device, the plain source
 * expressions whose rounding the reference's results depend on (box area
 * FMA contraction, float -> uint8 quantisation, signed-zero min/max,
 * fast-math division) next to the forms this library pins, and fills
 * report[0..39] (layout in nexusbvh_gb300/csrc/eval.cu).  Allocates a few
 * MB of device memory and synchronises the device. */
nxb_status nxb_selftest_numerics(uint32_t* report, uint32_t report_len);

/* Diagnostics: runs the two kernels that wait on other CTAs (the sort's
 * look-back and the BVH8 work queue) on inputs where the awaited flag is
 * never set, and returns in words[0..1] the error words their bounded
 * waits set (NXB_DEVERR_SORT_LOOKBACK_TIMEOUT, NXB_DEVERR_BVH8_QUEUE_TIMEOUT).
 * The context stays usable.  Takes about a second. */
nxb_status nxb_selftest_bounded_waits(uint32_t* words);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* NXB_GB300_H */
