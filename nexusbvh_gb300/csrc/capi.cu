// capi.cu - the C ABI: host orchestration of the five build stages.
//
// Replaces the reference's host builder (NexusBVH/src/BVHBuilder.cpp:13-300).
// Differences in how, not in what:
//   * one explicit stream, no device-wide synchronisation inside a build;
//   * every temporary lives in one workspace carved into 256-byte aligned
//     segments (keys, values, sort look-back, parent slots, BVH8 work
//     slots, a small control block), so the build itself allocates nothing
//     and can be captured in a CUDA graph (nxb_build_async);
//   * the plain entry points allocate the workspace and outputs
//     stream-ordered (cudaMallocAsync from a pool that keeps its memory);
//   * errors are returned as status codes: nothing calls cudaDeviceReset or
//     exit (the reference's CUDA_CHECK does, NexusBVH/src/Cuda/CudaUtils.h:6-16).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "pipeline.h"

namespace nxb {

namespace {
thread_local int g_last_cuda_error = 0;

nxb_status cuda_fail(cudaError_t e) {
    g_last_cuda_error = (int)e;
    if (e == cudaErrorMemoryAllocation) return NXB_ERR_OUT_OF_MEMORY;
    return NXB_ERR_CUDA;
}

#define NXB_TRY(expr)                                   \
    do {                                                \
        cudaError_t e_ = (expr);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_);    \
    } while (0)

constexpr size_t kAlign = 256;
// Largest primitive count the validators take (2n-1 nodes fit in uint32).
constexpr uint32_t kMaxValidatePrims = 0x7FFFFFFFu;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

uint32_t key_bits_of(const nxb_build_config* c) { return c && c->prioritize_speed ? 30u : 63u; }
uint32_t radius_of(const nxb_build_config* c) {
    uint32_t r = c ? c->search_radius : 0u;
    return r == 0 ? 8u : r;
}

// Largest primitive count: node indices 2n-1 and the BVH8 worst case
// 4n-1 stay below 2^32, and sort look-back counts fit in 30 bits.
constexpr uint32_t kMaxPrims = (1u << 30) - 1;

struct Layout {
    uint32_t n = 0, key_bytes = 0;
    SortPlan plan{};
    size_t tiles_words = 0;  // look-back words for all passes
    size_t ctrl = 0, result = 0, cost = 0, keys_a = 0, keys_b = 0, vals_a = 0, vals_b = 0, lookback = 0, parent = 0,
           pairs = 0, records = 0, kids = 0, total = 0;
    size_t total_bvh2 = 0;  // a build that stops at the BVH2 needs no child-pair records (the last segment)
};

Layout make_layout(uint32_t n, uint32_t key_bits) {
    Layout L;
    L.n = n;
    L.key_bytes = key_bits == 30 ? 4 : 8;
    // 30-bit keys: four 8-bit passes over [2,32); 63-bit keys: the hybrid
    // sort (launch_sort63_hybrid), whose Morton-fused histograms are those of
    // its four 9-bit top passes and whose look-back storage also serves its
    // eight-pass fallback (the same number of words)
    L.plan = key_bits == 30 ? make_sort_plan(2, 32) : hybrid63_top_plan();
    L.tiles_words = key_bits == 30 ? sort_lookback_words(n, L.key_bytes, L.plan.passes)
                                   : sort_lookback_words(n, L.key_bytes, kMaxSortPasses);
    size_t off = 0;
    auto seg = [&](size_t bytes) {
        size_t o = off;
        off += align_up(bytes);
        return o;
    };
    L.ctrl = seg(sizeof(Control));
    L.result = seg(sizeof(nxb_build_result));
    L.cost = seg(2 * sizeof(float));
    L.keys_a = seg((size_t)L.key_bytes * n);
    L.keys_b = seg((size_t)L.key_bytes * n);
    L.vals_a = seg(4ull * n);
    L.vals_b = seg(4ull * n);
    L.lookback = seg(4ull * L.tiles_words);
    L.parent = seg(4ull * n);
    L.pairs = seg(8ull * n);
    L.records = seg(32ull * n);
    L.total_bvh2 = off;
    L.kids = seg(64ull * n);
    L.total = off;
    return L;
}

size_t bvh8_capacity(uint32_t n) { return ((size_t)4 * n - 1 + 6) / 7; }

// allowed: the NXB_BUILD_* flags the calling entry point takes.
nxb_status check_config(const nxb_build_config* c, uint32_t allowed = NXB_BUILD_AUCTION) {
    if (!c) return NXB_OK;
    uint32_t r = c->search_radius;
    if (r != 0 && r != 4 && r != 8 && r != 16) return NXB_ERR_UNSUPPORTED;
    if (c->flags & ~allowed) return NXB_ERR_UNSUPPORTED;
    return NXB_OK;
}

bool validate_of(const nxb_build_config* c) { return c && (c->flags & NXB_BUILD_VALIDATE); }

// NXB_BUILD_VALIDATE: checks the BVH2 (root 2n-2) and, when bvh8 is given,
// the BVH8 of a finished build on stream s; NXB_ERR_DEVICE_INVARIANT when
// either is invalid.
nxb_status validate_built(const void* prims, nxb_prim_type type, uint32_t n, const Node2* bvh2, const Node8* bvh8,
                          const uint32_t* prim_idx, uint32_t bvh8_nodes, cudaStream_t s) {
    size_t bytes = validate_bvh2_scratch(n);
    if (bvh8) bytes = std::max(bytes, validate_bvh8_scratch(bvh8_nodes, n));
    void* scratch = nullptr;
    uint64_t* rep = nullptr;
    uint64_t h2[NXB_BVH2_CHECK_FIELDS] = {}, h8[NXB_BVH8_CHECK_FIELDS] = {};
    cudaError_t e = cudaMallocAsync(&scratch, bytes, s);
    if (!e) e = cudaMallocAsync((void**)&rep, sizeof(h2) + sizeof(h8), s);
    // one scratch for both checks: they run one after the other on s
    if (!e) e = launch_validate_bvh2(bvh2, n, 2 * n - 2, rep, scratch, s);
    if (!e && bvh8)
        e = launch_validate_bvh8(bvh8, bvh8_nodes, prim_idx, n, prims, (int)type, rep + NXB_BVH2_CHECK_FIELDS, scratch,
                                 s);
    if (!e) e = cudaMemcpyAsync(h2, rep, sizeof(h2), cudaMemcpyDeviceToHost, s);
    if (!e && bvh8) e = cudaMemcpyAsync(h8, rep + NXB_BVH2_CHECK_FIELDS, sizeof(h8), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (scratch) cudaFreeAsync(scratch, s);
    if (rep) cudaFreeAsync(rep, s);
    if (e) return cuda_fail(e);
    if (h2[NXB_BVH2_CHECK_FIELDS - 1] || h8[NXB_BVH8_CHECK_FIELDS - 1]) return NXB_ERR_DEVICE_INVARIANT;
    return NXB_OK;
}

bool auction_of(const nxb_build_config* c) { return c && (c->flags & NXB_BUILD_AUCTION); }

nxb_status check_prims(const void* prims, nxb_prim_type t, uint32_t n) {
    if (!prims) return NXB_ERR_INVALID_ARGUMENT;
    if (t != NXB_PRIM_AABB && t != NXB_PRIM_TRIANGLE) return NXB_ERR_INVALID_ARGUMENT;
    if (n == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (n > kMaxPrims) return NXB_ERR_UNSUPPORTED;
    if ((reinterpret_cast<uintptr_t>(prims) & 3u) != 0) return NXB_ERR_INVALID_ARGUMENT;
    return NXB_OK;
}

struct StageEvents {
    cudaEvent_t ev[6];
};

// Enqueues the whole pipeline.  bvh8 == nullptr stops after the BVH2.
nxb_status enqueue_build(const void* prims, nxb_prim_type type, uint32_t n, const nxb_build_config* cfg,
                         unsigned char* ws, size_t ws_bytes, Node2* bvh2, Node8* bvh8, uint32_t* prim_idx,
                         nxb_build_result* result, cudaStream_t s, StageEvents* evs) {
    const uint32_t key_bits = key_bits_of(cfg);
    const Layout L = make_layout(n, key_bits);
    if (ws_bytes < (bvh8 ? L.total : L.total_bvh2)) return NXB_ERR_WORKSPACE_TOO_SMALL;
    Control* ctrl = reinterpret_cast<Control*>(ws + L.ctrl);
    void* keys_a = ws + L.keys_a;
    void* keys_b = ws + L.keys_b;
    uint32_t* vals_a = reinterpret_cast<uint32_t*>(ws + L.vals_a);
    uint32_t* vals_b = reinterpret_cast<uint32_t*>(ws + L.vals_b);
    uint32_t* lookback = reinterpret_cast<uint32_t*>(ws + L.lookback);
    uint32_t* parent = reinterpret_cast<uint32_t*>(ws + L.parent);
    uint64_t* pairs = reinterpret_cast<uint64_t*>(ws + L.pairs);
    auto mark = [&](int i) -> cudaError_t { return evs ? cudaEventRecord(evs->ev[i], s) : cudaSuccess; };

    NXB_TRY(cudaMemsetAsync(ctrl, 0, sizeof(Control), s));
    NXB_TRY(mark(0));
    NXB_TRY(launch_scene_bounds(prims, type, n, bvh2, ctrl->scene_ord, s));
    NXB_TRY(mark(1));
    MortonFused f{};
    f.plan = &L.plan;
    f.cluster_idx = nullptr;  // the first sort pass generates the values
    f.parent = parent;
    f.zero_ptr = lookback;
    f.zero_words = align_up(4ull * L.tiles_words) / 4;  // both plans: the top passes' words, all of them
    f.scene_out = nullptr;
    f.seed_counters = true;
    NXB_TRY(launch_morton(bvh2, n, ctrl, (int)key_bits, keys_a, f, s));
    NXB_TRY(mark(2));
    if (key_bits == 30) {
        const size_t tiles_per_pass = L.tiles_words / L.plan.passes;
        for (int p = 0; p < L.plan.passes; ++p) {
            const bool even = (p % 2) == 0;
            NXB_TRY(launch_sort_pass(L.key_bytes, even ? keys_a : keys_b, even ? keys_b : keys_a,
                                     p == 0 ? nullptr : (even ? vals_a : vals_b), even ? vals_b : vals_a, n,
                                     L.plan.shift[p], L.plan.bits[p], ctrl->hist[p], lookback + p * tiles_per_pass,
                                     ctrl->tile_ctr + p, &ctrl->error_word, s));
        }
    } else {
        NXB_TRY(launch_sort63_hybrid(nullptr, nullptr, reinterpret_cast<uint64_t*>(keys_a),
                                     reinterpret_cast<uint64_t*>(keys_b), vals_a, vals_b, n, &ctrl->hist[0][0], lookback,
                                     ctrl->tile_ctr, &ctrl->sort_overflow, &ctrl->hist[0][0], &ctrl->fb_ticket,
                                     ctrl->fb_done, &ctrl->error_word, s));
    }
    // an even number of passes leaves the sorted keys / permutation in A
    NXB_TRY(mark(3));
    // the sort's second value buffer holds the H-PLOC cluster tokens
    // with a BVH8 to build, the climb also writes each internal node's
    // children side by side, which the collapse reads instead of the BVH2
    ChildPair* kids = bvh8 ? reinterpret_cast<ChildPair*>(ws + L.kids) : nullptr;
    NXB_TRY(launch_hploc(L.key_bytes, keys_a, vals_a, parent, bvh2, n, radius_of(cfg), vals_b,
                         &ctrl->parent_of_last, &ctrl->hploc_leaf_ctr, &ctrl->error_word, s,
                         reinterpret_cast<Node2*>(ws + L.records), bvh8 ? pairs : nullptr,
                         bvh8 ? ctrl->bvh8_ctr : nullptr, kids));
    NXB_TRY(mark(4));
    if (bvh8) {
        // the climb initialised the collapse's work queue
        NXB_TRY(launch_bvh8(bvh2, n, bvh8, (uint32_t)bvh8_capacity(n), prim_idx, pairs, ctrl->bvh8_ctr,
                            &ctrl->error_word, auction_of(cfg), s, kids));
    }
    NXB_TRY(mark(5));
    if (result) NXB_TRY(launch_finalize(ctrl, result, n, s));
    return NXB_OK;
}

nxb_status status_from_error_word(uint32_t w) {
    if (w == 0) return NXB_OK;
    if (w & (NXB_DEVERR_SORT_LOOKBACK_TIMEOUT | NXB_DEVERR_BVH8_QUEUE_TIMEOUT))
        return NXB_ERR_DEVICE_TIMEOUT;
    return NXB_ERR_DEVICE_INVARIANT;
}

std::once_flag g_pool_once;
void configure_pool() {
    std::call_once(g_pool_once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    });
}

// Shared body of nxb_build_bvh2 / nxb_build_bvh8.
nxb_status build_plain(const void* prims, nxb_prim_type type, uint32_t n, const nxb_build_config* cfg,
                       cudaStream_t s, bool wide, nxb_bvh2* out2, nxb_bvh8* out8, nxb_build_metrics* metrics) {
    nxb_status st = check_prims(prims, type, n);
    if (st != NXB_OK) return st;
    if ((st = check_config(cfg, NXB_BUILD_AUCTION | NXB_BUILD_VALIDATE)) != NXB_OK) return st;
    configure_pool();
    const Layout L = make_layout(n, key_bits_of(cfg));
    unsigned char* ws = nullptr;
    Node2* bvh2 = nullptr;
    Node8* bvh8 = nullptr;
    uint32_t* prim_idx = nullptr;
    StageEvents evs{};
    bool have_events = false;
    nxb_status status = NXB_OK;
    nxb_build_result res{};
    const size_t ws_bytes = wide ? L.total : L.total_bvh2;
    cudaError_t e = cudaMallocAsync((void**)&ws, ws_bytes, s);
    if (!e) e = cudaMallocAsync((void**)&bvh2, sizeof(Node2) * (2ull * n - 1), s);
    if (!e && wide) e = cudaMallocAsync((void**)&bvh8, sizeof(Node8) * bvh8_capacity(n), s);
    if (!e && wide) e = cudaMallocAsync((void**)&prim_idx, 4ull * n, s);
    if (!e && metrics) {
        have_events = true;
        for (int i = 0; i < 6 && !e; ++i) e = cudaEventCreate(&evs.ev[i]);
    }
    if (e) {
        status = cuda_fail(e);
    } else {
        nxb_build_result* d_res = reinterpret_cast<nxb_build_result*>(ws + L.result);
        float* d_cost = reinterpret_cast<float*>(ws + L.cost);
        status = enqueue_build(prims, type, n, cfg, ws, ws_bytes, bvh2, bvh8, prim_idx, d_res, s,
                               have_events ? &evs : nullptr);
        if (status == NXB_OK && metrics) {
            e = launch_bvh2_cost(bvh2, 2 * n - 1, &d_res->scene_bounds, d_cost, s);
            if (!e && wide)
                e = launch_bvh8_cost_dev(bvh8, &d_res->bvh8_node_count, (uint32_t)bvh8_capacity(n),
                                         &d_res->scene_bounds, d_cost + 1, s);
            if (e) status = cuda_fail(e);
        }
        if (status == NXB_OK) {
            e = cudaMemcpyAsync(&res, d_res, sizeof(res), cudaMemcpyDeviceToHost, s);
            float costs[2] = {0.f, 0.f};
            if (!e && metrics) e = cudaMemcpyAsync(costs, d_cost, sizeof(costs), cudaMemcpyDeviceToHost, s);
            if (!e) e = cudaStreamSynchronize(s);
            if (e) status = cuda_fail(e);
            if (status == NXB_OK) status = status_from_error_word(res.error_word);
            if (status == NXB_OK && validate_of(cfg))
                status = validate_built(prims, type, n, bvh2, wide ? bvh8 : nullptr, prim_idx, res.bvh8_node_count, s);
            if (status == NXB_OK && metrics) {
                float t[5] = {0, 0, 0, 0, 0};
                for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&t[i], evs.ev[i], evs.ev[i + 1]);
                metrics->scene_bounds_time = t[0];
                metrics->morton_codes_time = t[1];
                metrics->radix_sort_time = t[2];
                metrics->bvh2_build_time = t[3];
                metrics->bvh8_conversion_time = wide ? t[4] : 0.f;
                metrics->total_time = t[0] + t[1] + t[2] + t[3] + (wide ? t[4] : 0.f);
                metrics->bvh2_cost = costs[0];
                metrics->bvh8_cost = wide ? costs[1] : 0.f;
                metrics->average_child_per_node =
                    wide && res.bvh8_node_count ? (float)(n + res.bvh8_node_count - 1) / res.bvh8_node_count : 0.f;
            }
        }
    }
    if (have_events)
        for (int i = 0; i < 6; ++i)
            if (evs.ev[i]) cudaEventDestroy(evs.ev[i]);
    if (ws) cudaFreeAsync(ws, s);
    if (status != NXB_OK || wide) {
        if (bvh2) cudaFreeAsync(bvh2, s);
        bvh2 = nullptr;
    }
    if (status != NXB_OK) {
        if (bvh8) cudaFreeAsync(bvh8, s);
        if (prim_idx) cudaFreeAsync(prim_idx, s);
        return status;
    }
    if (wide) {
        out8->nodes = reinterpret_cast<nxb_bvh8_node*>(bvh8);
        out8->node_count = res.bvh8_node_count;
        out8->prim_idx = prim_idx;
        out8->prim_count = n;
        out8->bounds = res.scene_bounds;
    } else {
        out2->nodes = reinterpret_cast<nxb_bvh2_node*>(bvh2);
        out2->node_count = 2 * n - 1;
        out2->prim_count = n;
        out2->bounds = res.scene_bounds;
    }
    // like the reference, the call returns with the stream drained
    e = cudaStreamSynchronize(s);
    return e ? cuda_fail(e) : NXB_OK;
}

// ---- BVH files: a 64-byte header, the nodes, then (BVH8) prim_idx
struct BvhFileHeader {
    char magic[8];  // "NXBVH2\0\0" or "NXBVH8\0\0"
    uint32_t version;
    uint32_t node_count;
    uint32_t prim_count;
    uint32_t node_bytes;
    nxb_aabb bounds;
    uint8_t reserved[16];
};
static_assert(sizeof(BvhFileHeader) == 64, "BVH file header is 64 bytes");
constexpr uint32_t kBvhFileVersion = 1;

// Largest node count a BVH of prim_count primitives can have (BVH2: 2n-1;
// BVH8: the reference's allocation, ceil((4n-1)/7), at least 1).
uint64_t max_nodes(bool wide, uint32_t prim_count) {
    if (prim_count == 0) return 0;
    return wide ? std::max<uint64_t>(1, (4ull * prim_count - 1 + 6) / 7) : 2ull * prim_count - 1;
}

nxb_status write_bvh_file(const char* path, bool wide, const void* nodes, uint32_t node_count,
                          const uint32_t* prim_idx, uint32_t prim_count, const nxb_aabb& bounds) {
    if (!path || !nodes || node_count == 0 || prim_count == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (wide && !prim_idx) return NXB_ERR_INVALID_ARGUMENT;
    if (node_count > max_nodes(wide, prim_count)) return NXB_ERR_INVALID_ARGUMENT;
    BvhFileHeader h{};
    std::memcpy(h.magic, wide ? "NXBVH8\0\0" : "NXBVH2\0\0", 8);
    h.version = kBvhFileVersion;
    h.node_count = node_count;
    h.prim_count = prim_count;
    h.node_bytes = wide ? sizeof(nxb_bvh8_node) : sizeof(nxb_bvh2_node);
    h.bounds = bounds;
    FILE* f = std::fopen(path, "wb");
    if (!f) return NXB_ERR_IO;
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 &&
              std::fwrite(nodes, h.node_bytes, node_count, f) == node_count &&
              (!wide || std::fwrite(prim_idx, sizeof(uint32_t), prim_count, f) == prim_count);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? NXB_OK : NXB_ERR_IO;
}

// Reads and checks a BVH file; on success *nodes and (BVH8) *prim_idx are
// malloc'd and owned by the caller.
nxb_status read_bvh_file(const char* path, bool wide, void** nodes, uint32_t* node_count, uint32_t** prim_idx,
                         uint32_t* prim_count, nxb_aabb* bounds) {
    if (!path) return NXB_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return NXB_ERR_IO;
    BvhFileHeader h{};
    const size_t node_bytes = wide ? sizeof(nxb_bvh8_node) : sizeof(nxb_bvh2_node);
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 &&
              std::memcmp(h.magic, wide ? "NXBVH8\0\0" : "NXBVH2\0\0", 8) == 0 && h.version == kBvhFileVersion &&
              h.node_bytes == node_bytes && h.prim_count > 0 && h.node_count > 0 &&
              h.node_count <= max_nodes(wide, h.prim_count);
    long size = -1;
    if (ok && std::fseek(f, 0, SEEK_END) == 0) size = std::ftell(f);
    const uint64_t want = sizeof h + (uint64_t)h.node_count * node_bytes + (wide ? 4ull * h.prim_count : 0ull);
    ok = ok && size >= 0 && (uint64_t)size == want && std::fseek(f, (long)sizeof h, SEEK_SET) == 0;
    void* n = nullptr;
    uint32_t* p = nullptr;
    if (ok) {
        n = std::malloc(node_bytes * h.node_count);
        p = wide ? (uint32_t*)std::malloc(4ull * h.prim_count) : nullptr;
        if (!n || (wide && !p)) {
            std::free(n);
            std::free(p);
            std::fclose(f);
            return NXB_ERR_OUT_OF_MEMORY;
        }
        ok = std::fread(n, node_bytes, h.node_count, f) == h.node_count &&
             (!wide || std::fread(p, sizeof(uint32_t), h.prim_count, f) == h.prim_count);
    }
    std::fclose(f);
    if (!ok) {
        std::free(n);
        std::free(p);
        return NXB_ERR_IO;
    }
    *nodes = n;
    *node_count = h.node_count;
    if (wide) *prim_idx = p;
    *prim_count = h.prim_count;
    *bounds = h.bounds;
    return NXB_OK;
}

}  // namespace

nxb_status record_cuda_error(cudaError_t e) { return cuda_fail(e); }

const DeviceInfo& device_info() {
    static DeviceInfo infos[64];
    static bool ready[64] = {false};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (!ready[dev]) {
        DeviceInfo d{};
        cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&d.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (d.sms <= 0) d.sms = 1;
        infos[dev] = d;
        ready[dev] = true;
    }
    return infos[dev];
}

}  // namespace nxb

using namespace nxb;

extern "C" {

const char* nxb_status_string(nxb_status s) {
    switch (s) {
        case NXB_OK: return "NXB_OK";
        case NXB_ERR_INVALID_ARGUMENT: return "NXB_ERR_INVALID_ARGUMENT";
        case NXB_ERR_UNSUPPORTED: return "NXB_ERR_UNSUPPORTED";
        case NXB_ERR_OUT_OF_MEMORY: return "NXB_ERR_OUT_OF_MEMORY";
        case NXB_ERR_CUDA: return "NXB_ERR_CUDA";
        case NXB_ERR_WORKSPACE_TOO_SMALL: return "NXB_ERR_WORKSPACE_TOO_SMALL";
        case NXB_ERR_DEVICE_TIMEOUT: return "NXB_ERR_DEVICE_TIMEOUT";
        case NXB_ERR_DEVICE_INVARIANT: return "NXB_ERR_DEVICE_INVARIANT";
        case NXB_ERR_ADMISSION: return "NXB_ERR_ADMISSION";
        case NXB_ERR_IO: return "NXB_ERR_IO";
    }
    return "NXB_ERR_UNKNOWN";
}

int nxb_last_cuda_error(void) { return g_last_cuda_error; }

const char* nxb_version(void) { return "nxb-gb300 0.1 (sm_103a, --use_fast_math)"; }

nxb_status nxb_build_bvh2(const void* d_prims, nxb_prim_type prim_type, uint32_t prim_count,
                          const nxb_build_config* config, struct CUstream_st* stream, nxb_bvh2* out_bvh,
                          nxb_build_metrics* metrics) {
    if (!out_bvh) return NXB_ERR_INVALID_ARGUMENT;
    return build_plain(d_prims, prim_type, prim_count, config, stream, false, out_bvh, nullptr, metrics);
}

nxb_status nxb_build_bvh8(const void* d_prims, nxb_prim_type prim_type, uint32_t prim_count,
                          const nxb_build_config* config, struct CUstream_st* stream, nxb_bvh8* out_bvh,
                          nxb_build_metrics* metrics) {
    if (!out_bvh) return NXB_ERR_INVALID_ARGUMENT;
    return build_plain(d_prims, prim_type, prim_count, config, stream, true, nullptr, out_bvh, metrics);
}

nxb_status nxb_bvh2_to_host(const nxb_bvh2* d, nxb_bvh2* h) {
    if (!d || !h || !d->nodes || d->node_count == 0) return NXB_ERR_INVALID_ARGUMENT;
    nxb_bvh2 out = *d;
    out.nodes = (nxb_bvh2_node*)std::malloc(sizeof(nxb_bvh2_node) * d->node_count);
    if (!out.nodes) return NXB_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaMemcpy(out.nodes, d->nodes, sizeof(nxb_bvh2_node) * d->node_count, cudaMemcpyDeviceToHost);
    if (e) {
        std::free(out.nodes);
        return cuda_fail(e);
    }
    *h = out;
    return NXB_OK;
}

nxb_status nxb_free_host_bvh2(nxb_bvh2* h) {
    if (!h) return NXB_ERR_INVALID_ARGUMENT;
    std::free(h->nodes);
    h->nodes = nullptr;
    return NXB_OK;
}

nxb_status nxb_bvh8_to_host(const nxb_bvh8* d, nxb_bvh8* h) {
    if (!d || !h || !d->nodes || !d->prim_idx || d->node_count == 0) return NXB_ERR_INVALID_ARGUMENT;
    nxb_bvh8 out = *d;
    out.nodes = (nxb_bvh8_node*)std::malloc(sizeof(nxb_bvh8_node) * d->node_count);
    out.prim_idx = (uint32_t*)std::malloc(sizeof(uint32_t) * d->prim_count);
    if (!out.nodes || !out.prim_idx) {
        std::free(out.nodes);
        std::free(out.prim_idx);
        return NXB_ERR_OUT_OF_MEMORY;
    }
    cudaError_t e = cudaMemcpy(out.nodes, d->nodes, sizeof(nxb_bvh8_node) * d->node_count, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(out.prim_idx, d->prim_idx, sizeof(uint32_t) * d->prim_count, cudaMemcpyDeviceToHost);
    if (e) {
        std::free(out.nodes);
        std::free(out.prim_idx);
        return cuda_fail(e);
    }
    *h = out;
    return NXB_OK;
}

nxb_status nxb_free_host_bvh8(nxb_bvh8* h) {
    if (!h) return NXB_ERR_INVALID_ARGUMENT;
    std::free(h->nodes);
    std::free(h->prim_idx);
    h->nodes = nullptr;
    h->prim_idx = nullptr;
    return NXB_OK;
}

nxb_status nxb_free_device_bvh2(nxb_bvh2* d) {
    if (!d) return NXB_ERR_INVALID_ARGUMENT;
    cudaError_t e = d->nodes ? cudaFree(d->nodes) : cudaSuccess;
    d->nodes = nullptr;
    return e ? cuda_fail(e) : NXB_OK;
}

nxb_status nxb_free_device_bvh8(nxb_bvh8* d) {
    if (!d) return NXB_ERR_INVALID_ARGUMENT;
    cudaError_t e = d->nodes ? cudaFree(d->nodes) : cudaSuccess;
    cudaError_t e2 = d->prim_idx ? cudaFree(d->prim_idx) : cudaSuccess;
    d->nodes = nullptr;
    d->prim_idx = nullptr;
    if (e) return cuda_fail(e);
    return e2 ? cuda_fail(e2) : NXB_OK;
}

nxb_status nxb_write_bvh2(const char* path, const nxb_bvh2* h) {
    if (!h) return NXB_ERR_INVALID_ARGUMENT;
    return write_bvh_file(path, false, h->nodes, h->node_count, nullptr, h->prim_count, h->bounds);
}

nxb_status nxb_read_bvh2(const char* path, nxb_bvh2* h) {
    if (!h) return NXB_ERR_INVALID_ARGUMENT;
    nxb_bvh2 out{};
    void* nodes = nullptr;
    const nxb_status st = read_bvh_file(path, false, &nodes, &out.node_count, nullptr, &out.prim_count, &out.bounds);
    if (st != NXB_OK) return st;
    out.nodes = (nxb_bvh2_node*)nodes;
    *h = out;
    return NXB_OK;
}

nxb_status nxb_write_bvh8(const char* path, const nxb_bvh8* h) {
    if (!h) return NXB_ERR_INVALID_ARGUMENT;
    return write_bvh_file(path, true, h->nodes, h->node_count, h->prim_idx, h->prim_count, h->bounds);
}

nxb_status nxb_read_bvh8(const char* path, nxb_bvh8* h) {
    if (!h) return NXB_ERR_INVALID_ARGUMENT;
    nxb_bvh8 out{};
    void* nodes = nullptr;
    const nxb_status st =
        read_bvh_file(path, true, &nodes, &out.node_count, &out.prim_idx, &out.prim_count, &out.bounds);
    if (st != NXB_OK) return st;
    out.nodes = (nxb_bvh8_node*)nodes;
    *h = out;
    return NXB_OK;
}

nxb_status nxb_query_build_sizes(uint32_t n, const nxb_build_config* config, nxb_build_sizes* out) {
    if (!out || n == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (n > kMaxPrims) return NXB_ERR_UNSUPPORTED;
    nxb_status st = check_config(config);
    if (st != NXB_OK) return st;
    const Layout L = make_layout(n, key_bits_of(config));
    out->workspace_bytes = L.total;
    out->bvh2_node_count = 2ull * n - 1;
    out->bvh8_node_capacity = bvh8_capacity(n);
    return NXB_OK;
}

nxb_status nxb_build_async(const void* d_prims, nxb_prim_type prim_type, uint32_t n, const nxb_build_config* config,
                           void* d_workspace, size_t workspace_bytes, nxb_bvh2_node* d_bvh2_nodes,
                           nxb_bvh8_node* d_bvh8_nodes, uint32_t* d_prim_idx, nxb_build_result* d_result,
                           struct CUstream_st* stream) {
    nxb_status st = check_prims(d_prims, prim_type, n);
    if (st != NXB_OK) return st;
    if ((st = check_config(config)) != NXB_OK) return st;
    if (!d_workspace || !d_bvh2_nodes || !d_result) return NXB_ERR_INVALID_ARGUMENT;
    if ((d_bvh8_nodes == nullptr) != (d_prim_idx == nullptr)) return NXB_ERR_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(d_workspace) & (kAlign - 1)) != 0) return NXB_ERR_INVALID_ARGUMENT;
    return enqueue_build(d_prims, prim_type, n, config, (unsigned char*)d_workspace, workspace_bytes,
                         reinterpret_cast<Node2*>(d_bvh2_nodes), reinterpret_cast<Node8*>(d_bvh8_nodes), d_prim_idx,
                         d_result, stream, nullptr);
}

nxb_status nxb_build_async_timed(const void* d_prims, nxb_prim_type prim_type, uint32_t n,
                                 const nxb_build_config* config, void* d_workspace, size_t workspace_bytes,
                                 nxb_bvh2_node* d_bvh2_nodes, nxb_bvh8_node* d_bvh8_nodes, uint32_t* d_prim_idx,
                                 nxb_build_result* d_result, struct CUstream_st* stream, void* const* stage_events) {
    if (!stage_events) return NXB_ERR_INVALID_ARGUMENT;
    nxb_status st = check_prims(d_prims, prim_type, n);
    if (st != NXB_OK) return st;
    if ((st = check_config(config)) != NXB_OK) return st;
    if (!d_workspace || !d_bvh2_nodes || !d_result) return NXB_ERR_INVALID_ARGUMENT;
    if ((d_bvh8_nodes == nullptr) != (d_prim_idx == nullptr)) return NXB_ERR_INVALID_ARGUMENT;
    StageEvents evs;
    for (int i = 0; i < 6; ++i) {
        if (!stage_events[i]) return NXB_ERR_INVALID_ARGUMENT;
        evs.ev[i] = (cudaEvent_t)stage_events[i];
    }
    return enqueue_build(d_prims, prim_type, n, config, (unsigned char*)d_workspace, workspace_bytes,
                         reinterpret_cast<Node2*>(d_bvh2_nodes), reinterpret_cast<Node8*>(d_bvh8_nodes), d_prim_idx,
                         d_result, stream, &evs);
}

nxb_status nxb_stage_scene_bounds(const void* d_prims, nxb_prim_type prim_type, uint32_t n, nxb_bvh2_node* d_nodes,
                                  nxb_aabb* d_scene, struct CUstream_st* stream) {
    nxb_status st = check_prims(d_prims, prim_type, n);
    if (st != NXB_OK) return st;
    if (!d_nodes || !d_scene) return NXB_ERR_INVALID_ARGUMENT;
    uint32_t* ord = reinterpret_cast<uint32_t*>(d_scene);
    NXB_TRY(cudaMemsetAsync(ord, 0, sizeof(nxb_aabb), stream));
    NXB_TRY(launch_scene_bounds(d_prims, prim_type, n, reinterpret_cast<Node2*>(d_nodes), ord, stream));
    NXB_TRY(launch_ord_to_aabb(ord, stream));
    return NXB_OK;
}

nxb_status nxb_stage_morton(const nxb_bvh2_node* d_nodes, uint32_t n, const nxb_aabb* d_scene, uint32_t key_bits,
                            void* d_keys, uint32_t* d_cluster_idx, struct CUstream_st* stream) {
    if (!d_nodes || !d_scene || !d_keys || n == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (key_bits != 30 && key_bits != 63) return NXB_ERR_UNSUPPORTED;
    NXB_TRY(launch_morton_scene(reinterpret_cast<const Node2*>(d_nodes), n, d_scene, (int)key_bits, d_keys,
                                d_cluster_idx, stream));
    return NXB_OK;
}

namespace {
// 64-bit keys on the reference's 63-bit range [1,64) take the hybrid sort
// (launch_sort63_hybrid); every other range the plain 8-bit passes.
bool sort_is_hybrid(uint32_t key_bytes, uint32_t begin_bit, uint32_t end_bit) {
    return key_bytes == 8 && begin_bit == 1 && end_bit == 64;
}
SortPlan sort_plan_of(uint32_t key_bytes, uint32_t begin_bit, uint32_t end_bit) {
    return sort_is_hybrid(key_bytes, begin_bit, end_bit) ? hybrid63_top_plan() : make_sort_plan(begin_bit, end_bit);
}

struct SortScratch {
    size_t hist, ctr, hybrid, lookback, keys_tmp, vals_tmp, total;
};
// hist | tile counters | hybrid words | look-back | keys | values; the
// segments before keys_tmp are cleared by every call
SortScratch sort_scratch(uint32_t n, uint32_t key_bytes, uint32_t begin_bit, uint32_t end_bit) {
    const SortPlan plan = sort_plan_of(key_bytes, begin_bit, end_bit);
    SortScratch S{};
    size_t off = 0;
    auto seg = [&](size_t b) {
        size_t o = off;
        off += align_up(b);
        return o;
    };
    S.hist = seg(sizeof(uint32_t) * kMaxSortPasses * kRadixBins);
    S.ctr = seg(sizeof(uint32_t) * kMaxSortPasses);
    S.hybrid = seg(sizeof(uint32_t) * (kMaxSortPasses + 4));  // overflow, ticket, done[passes + 2]
    // the hybrid's look-back serves its top passes and its 8-pass fallback
    S.lookback = seg(4ull * (sort_is_hybrid(key_bytes, begin_bit, end_bit)
                                 ? sort_lookback_words(n, key_bytes, kMaxSortPasses)
                                 : sort_lookback_words(n, key_bytes, plan.passes)));
    S.keys_tmp = seg((size_t)key_bytes * n);
    S.vals_tmp = seg(4ull * n);
    S.total = off;
    return S;
}
}  // namespace

size_t nxb_sort_scratch_bytes(uint32_t count, uint32_t key_bytes, uint32_t begin_bit, uint32_t end_bit) {
    if ((key_bytes != 4 && key_bytes != 8) || begin_bit >= end_bit || end_bit > key_bytes * 8) return 0;
    return sort_scratch(count, key_bytes, begin_bit, end_bit).total;
}

nxb_status nxb_stage_radix_sort(uint32_t key_bytes, const void* d_keys_in, void* d_keys_out,
                                const uint32_t* d_vals_in, uint32_t* d_vals_out, uint32_t n, uint32_t begin_bit,
                                uint32_t end_bit, void* d_scratch, size_t scratch_bytes, uint32_t* d_error_word,
                                struct CUstream_st* stream) {
    if (key_bytes != 4 && key_bytes != 8) return NXB_ERR_UNSUPPORTED;
    if (begin_bit >= end_bit || end_bit > key_bytes * 8) return NXB_ERR_INVALID_ARGUMENT;
    if (!d_keys_in || !d_keys_out || !d_vals_out || !d_scratch || n == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (n > kMaxPrims) return NXB_ERR_UNSUPPORTED;
    const SortPlan plan = sort_plan_of(key_bytes, begin_bit, end_bit);
    const SortScratch S = sort_scratch(n, key_bytes, begin_bit, end_bit);
    if (scratch_bytes < S.total) return NXB_ERR_WORKSPACE_TOO_SMALL;
    unsigned char* base = (unsigned char*)d_scratch;
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + S.hist);
    uint32_t* ctr = reinterpret_cast<uint32_t*>(base + S.ctr);
    uint32_t* lookback = reinterpret_cast<uint32_t*>(base + S.lookback);
    NXB_TRY(cudaMemsetAsync(base, 0, S.keys_tmp, stream));
    NXB_TRY(launch_sort_histogram(key_bytes, d_keys_in, n, plan, hist, stream));
    if (sort_is_hybrid(key_bytes, begin_bit, end_bit)) {
        uint32_t* hy = reinterpret_cast<uint32_t*>(base + S.hybrid);
        NXB_TRY(launch_sort63_hybrid(static_cast<const uint64_t*>(d_keys_in), d_vals_in,
                                     static_cast<uint64_t*>(d_keys_out), reinterpret_cast<uint64_t*>(base + S.keys_tmp),
                                     d_vals_out, reinterpret_cast<uint32_t*>(base + S.vals_tmp), n, hist, lookback, ctr,
                                     hy, hist, hy + 1, hy + 2, d_error_word, stream));
        return NXB_OK;
    }
    const size_t per_pass = sort_lookback_words(n, key_bytes, 1);
    const void* kin = d_keys_in;
    const uint32_t* vin = d_vals_in;
    for (int p = 0; p < plan.passes; ++p) {
        const bool last_is_out = ((plan.passes - 1 - p) % 2) == 0;
        void* kout = last_is_out ? d_keys_out : (void*)(base + S.keys_tmp);
        uint32_t* vout = last_is_out ? d_vals_out : reinterpret_cast<uint32_t*>(base + S.vals_tmp);
        NXB_TRY(launch_sort_pass(key_bytes, kin, kout, vin, vout, n, plan.shift[p], plan.bits[p],
                                 hist + p * kRadixBins, lookback + p * per_pass, ctr + p, d_error_word, stream));
        kin = kout;
        vin = vout;
    }
    return NXB_OK;
}

// parent slots (4n) | cluster tokens (4n) | 2 counters | cluster records (32n)
size_t nxb_hploc_scratch_bytes(uint32_t n) { return 2 * align_up(4ull * n) + kAlign + align_up(32ull * n); }

nxb_status nxb_stage_hploc(uint32_t key_bytes, const void* d_sorted_keys, uint32_t* d_cluster_idx,
                           nxb_bvh2_node* d_nodes, uint32_t n, uint32_t search_radius, void* d_scratch,
                           size_t scratch_bytes, uint32_t* d_error_word, struct CUstream_st* stream) {
    if (key_bytes != 4 && key_bytes != 8) return NXB_ERR_UNSUPPORTED;
    if (search_radius == 0) search_radius = 8;
    if (search_radius != 4 && search_radius != 8 && search_radius != 16) return NXB_ERR_UNSUPPORTED;
    if (!d_sorted_keys || !d_cluster_idx || !d_nodes || !d_scratch || n == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (n > kMaxPrims) return NXB_ERR_UNSUPPORTED;
    if (scratch_bytes < nxb_hploc_scratch_bytes(n)) return NXB_ERR_WORKSPACE_TOO_SMALL;
    unsigned char* base = (unsigned char*)d_scratch;
    uint32_t* parent = (uint32_t*)base;
    uint32_t* tokens = reinterpret_cast<uint32_t*>(base + align_up(4ull * n));
    uint32_t* words = reinterpret_cast<uint32_t*>(base + 2 * align_up(4ull * n));
    NXB_TRY(launch_fill_u32(parent, kInvalid, n, stream));
    NXB_TRY(launch_fill_u32(words, kInvalid, 1, stream));  // parent_of_last
    NXB_TRY(launch_fill_u32(words + 1, 0, 1, stream));      // leaf counter
    Node2* records = reinterpret_cast<Node2*>(base + 2 * align_up(4ull * n) + kAlign);
    NXB_TRY(launch_hploc(key_bytes, d_sorted_keys, d_cluster_idx, parent, reinterpret_cast<Node2*>(d_nodes), n,
                         search_radius, tokens, words, words + 1, d_error_word, stream, records));
    return NXB_OK;
}

size_t nxb_bvh8_scratch_bytes(uint32_t n) { return align_up(8ull * n) + align_up(4 * kBvh8CtrWords); }

nxb_status nxb_stage_bvh8_ex(const nxb_bvh2_node* d_bvh2_nodes, uint32_t n, nxb_bvh8_node* d_bvh8_nodes,
                             uint32_t* d_prim_idx, uint32_t* d_counts, void* d_scratch, size_t scratch_bytes,
                             uint32_t build_flags, uint32_t* d_error_word, struct CUstream_st* stream) {
    if (!d_bvh2_nodes || !d_bvh8_nodes || !d_prim_idx || !d_counts || !d_scratch || n == 0)
        return NXB_ERR_INVALID_ARGUMENT;
    if (n > kMaxPrims) return NXB_ERR_UNSUPPORTED;
    if (build_flags & ~NXB_BUILD_AUCTION) return NXB_ERR_UNSUPPORTED;
    if (scratch_bytes < nxb_bvh8_scratch_bytes(n)) return NXB_ERR_WORKSPACE_TOO_SMALL;
    uint64_t* pairs = (uint64_t*)d_scratch;
    uint32_t* ctr = reinterpret_cast<uint32_t*>((unsigned char*)d_scratch + align_up(8ull * n));
    NXB_TRY(launch_bvh8_init(pairs, n, ctr, stream));
    NXB_TRY(launch_bvh8(reinterpret_cast<const Node2*>(d_bvh2_nodes), n, reinterpret_cast<Node8*>(d_bvh8_nodes),
                        (uint32_t)bvh8_capacity(n), d_prim_idx, pairs, ctr, d_error_word,
                        (build_flags & NXB_BUILD_AUCTION) != 0, stream));
    NXB_TRY(cudaMemcpyAsync(d_counts, ctr + kBvh8Nodes, sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
    NXB_TRY(cudaMemcpyAsync(d_counts + 1, ctr + kBvh8Leaves, sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
    return NXB_OK;
}

nxb_status nxb_stage_bvh8(const nxb_bvh2_node* d_bvh2_nodes, uint32_t n, nxb_bvh8_node* d_bvh8_nodes,
                          uint32_t* d_prim_idx, uint32_t* d_counts, void* d_scratch, size_t scratch_bytes,
                          uint32_t* d_error_word, struct CUstream_st* stream) {
    return nxb_stage_bvh8_ex(d_bvh2_nodes, n, d_bvh8_nodes, d_prim_idx, d_counts, d_scratch, scratch_bytes, 0u,
                             d_error_word, stream);
}

nxb_status nxb_eval_bvh2_cost(const nxb_bvh2_node* d_nodes, uint32_t count, const nxb_aabb* d_root, float* d_cost,
                              struct CUstream_st* stream) {
    if (!d_nodes || !d_root || !d_cost || count == 0) return NXB_ERR_INVALID_ARGUMENT;
    NXB_TRY(launch_bvh2_cost(reinterpret_cast<const Node2*>(d_nodes), count, d_root, d_cost, stream));
    return NXB_OK;
}

nxb_status nxb_eval_bvh8_cost(const nxb_bvh8_node* d_nodes, uint32_t count, const nxb_aabb* d_root, float* d_cost,
                              struct CUstream_st* stream) {
    if (!d_nodes || !d_root || !d_cost || count == 0) return NXB_ERR_INVALID_ARGUMENT;
    NXB_TRY(launch_bvh8_cost(reinterpret_cast<const Node8*>(d_nodes), count, d_root, d_cost, stream));
    return NXB_OK;
}

size_t nxb_validate_bvh2_scratch_bytes(uint32_t n) {
    if (n == 0 || n > kMaxValidatePrims) return 0;
    return validate_bvh2_scratch(n);
}

nxb_status nxb_validate_bvh2(const nxb_bvh2_node* d_nodes, uint32_t n, uint32_t root, uint64_t* d_report,
                             void* d_scratch, size_t scratch_bytes, struct CUstream_st* stream) {
    if (!d_nodes || !d_report || !d_scratch || n == 0 || n > kMaxValidatePrims || root >= 2 * n - 1)
        return NXB_ERR_INVALID_ARGUMENT;
    if (scratch_bytes < validate_bvh2_scratch(n)) return NXB_ERR_INVALID_ARGUMENT;
    NXB_TRY(launch_validate_bvh2(reinterpret_cast<const Node2*>(d_nodes), n, root, d_report, d_scratch, stream));
    return NXB_OK;
}

size_t nxb_validate_bvh8_scratch_bytes(uint32_t node_count, uint32_t n) {
    if (node_count == 0 || n == 0 || n > kMaxValidatePrims) return 0;
    return validate_bvh8_scratch(node_count, n);
}

nxb_status nxb_validate_bvh8(const nxb_bvh8_node* d_nodes, uint32_t node_count, const uint32_t* d_prim_idx,
                             uint32_t n, const void* d_prims, nxb_prim_type prim_type, uint64_t* d_report,
                             void* d_scratch, size_t scratch_bytes, struct CUstream_st* stream) {
    if (!d_nodes || !d_prim_idx || !d_prims || !d_report || !d_scratch || node_count == 0 || n == 0 ||
        n > kMaxValidatePrims || (prim_type != NXB_PRIM_AABB && prim_type != NXB_PRIM_TRIANGLE))
        return NXB_ERR_INVALID_ARGUMENT;
    if (scratch_bytes < validate_bvh8_scratch(node_count, n)) return NXB_ERR_INVALID_ARGUMENT;
    NXB_TRY(launch_validate_bvh8(reinterpret_cast<const Node8*>(d_nodes), node_count, d_prim_idx, n, d_prims,
                                 (int)prim_type, d_report, d_scratch, stream));
    return NXB_OK;
}

nxb_status nxb_selftest_bounded_waits(uint32_t* words) {
    if (!words) return NXB_ERR_INVALID_ARGUMENT;
    words[0] = words[1] = 0;
    NXB_TRY(run_sort_stall_probe(&words[0]));
    NXB_TRY(run_bvh8_stall_probe(&words[1]));
    NXB_TRY(cudaDeviceSynchronize());
    return NXB_OK;
}

nxb_status nxb_selftest_numerics(uint32_t* report, uint32_t report_len) {
    if (!report || report_len < 40) return NXB_ERR_INVALID_ARGUMENT;
    NXB_TRY(run_selftest(report));
    return NXB_OK;
}

}  // extern "C"
