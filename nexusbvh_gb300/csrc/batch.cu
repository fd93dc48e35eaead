// batch.cu - batched builds: many independent meshes, one launch per stage.
//
// The reference builds one mesh per call (NXB::BuildBVH8,
// NexusBVH/src/BVHBuilder.cpp:173-267): about ten launches, a few
// allocations and two device synchronisations per mesh, which is what a
// small mesh's build time consists of.  A batch lays the meshes end to end
// and runs each stage once over all of them:
//   * scene bounds per mesh (warp-reduced into 6 ordered words per mesh);
//   * 30-bit Morton codes from each mesh's own box, sorted as one 64-bit
//     key mesh << 32 | code over bits [2, 32 + mesh bits): per mesh this is
//     exactly the plain sort by code >> 2 (stable), and the meshes stay in
//     order;
//   * H-PLOC and the BVH8 collapse with mesh-local indices (MeshBatch in
//     common.cuh), so every mesh's BVH2 is the plain build's array;
//   * nxb_batch_* capture the whole sequence once in a CUDA graph and
//     replay it; the build server (server.cu) runs it eagerly on arenas it
//     sizes per group of requests.
// Everything lives in one device allocation; a build allocates nothing.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pipeline.h"

namespace nxb {

namespace {
constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr uint32_t kMaxTotal = (1u << 30) - 1;
uint32_t mesh_bits_of(uint32_t meshes) { return meshes > 1 ? 32u - (uint32_t)__builtin_clz(meshes - 1) : 0u; }

#define NXB_TRY(expr)                                          \
    do {                                                       \
        cudaError_t e_ = (expr);                               \
        if (e_ != cudaSuccess) return record_cuda_error(e_);   \
    } while (0)

// Segment offsets of an arena, in allocation order.
struct Segments {
    size_t off, off8, ctrl, scene, zero_end, parent, look, ctr8, mnodes, mleaves, trng, ka, kb, va, vb, pairs, kids,
        bvh2, bvh8, prim, res, total;
};

Segments segments_of(const BatchArena& a) {
    Segments g{};
    size_t at = 0;
    auto seg = [&](size_t bytes) {
        const size_t o = at;
        at += align_up(bytes);
        return o;
    };
    const size_t n = a.total, M = a.meshes;
    g.off = seg(4 * (M + 1));
    g.off8 = seg(4 * (M + 1));
    g.ctrl = seg(sizeof(BatchCtrl));
    g.scene = seg(24 * M);
    g.zero_end = at;
    g.parent = seg(4 * (n + M));
    g.look = seg(4 * a.lookback_words_per_pass * kMaxSortPasses);
    g.ctr8 = seg(4 * kBvh8CtrWords * kMaxMeshGroups);
    g.mnodes = seg(4 * M);
    g.mleaves = seg(4 * M);
    g.trng = seg(8 * ((n + 127) / 128));
    g.ka = seg(8 * n);
    g.kb = seg(8 * n);
    g.va = seg(4 * n);
    g.vb = seg(4 * n);
    g.pairs = seg(8ull * a.slots);
    g.kids = seg(sizeof(ChildPair) * n);
    g.bvh2 = seg(sizeof(Node2) * 2 * n);
    g.bvh8 = seg(sizeof(Node8) * (size_t)a.slots);
    g.prim = seg(4 * n);
    g.res = seg(sizeof(nxb_batch_mesh) * M);
    g.total = at;
    return g;
}
}  // namespace

uint32_t batch_bvh8_capacity(uint32_t n) { return n == 0 ? 1u : (uint32_t)(((size_t)4 * n - 1 + 6) / 7); }

bool batch_digit_ok(uint32_t mesh_bits, uint32_t d) {
    if (d < 4 || d > 8) return false;
    return (30 + mesh_bits + d - 1) / d <= (uint32_t)kMaxSortPasses;
}

bool batch_layout(const uint32_t* h_off, uint32_t meshes, uint32_t* h_off8, BatchArena* a) {
    *a = BatchArena{};
    a->meshes = meshes;
    a->total = h_off[meshes];
    if (a->total > kMaxTotal) return false;
    a->mesh_bits = mesh_bits_of(meshes);
    uint64_t acc = 0;
    for (uint32_t m = 0; m < meshes; ++m) {
        h_off8[m] = (uint32_t)acc;
        acc += batch_bvh8_capacity(h_off[m + 1] - h_off[m]);
        if (acc > 0xFFFFFFF0ull) return false;
    }
    h_off8[meshes] = (uint32_t)acc;
    a->slots = (uint32_t)acc;
    a->lookback_words_per_pass = sort_lookback_words(a->total ? a->total : 1, 8, 1);
    a->bytes = segments_of(*a).total;
    return true;
}

void batch_bind(unsigned char* p, BatchArena* a) {
    const Segments g = segments_of(*a);
    a->off = reinterpret_cast<uint32_t*>(p + g.off);
    a->off8 = reinterpret_cast<uint32_t*>(p + g.off8);
    a->zero_begin = p + g.ctrl;
    a->zero_bytes = g.zero_end - g.ctrl;
    a->ctrl = reinterpret_cast<BatchCtrl*>(p + g.ctrl);
    a->scene_ord = reinterpret_cast<uint32_t*>(p + g.scene);
    a->parent = reinterpret_cast<uint32_t*>(p + g.parent);
    a->pol = a->parent + a->total;
    a->ones_words = align_up(4ull * (a->total + a->meshes)) / 4;
    a->lookback = reinterpret_cast<uint32_t*>(p + g.look);
    a->ctr8 = reinterpret_cast<uint32_t*>(p + g.ctr8);
    a->mesh_nodes = reinterpret_cast<uint32_t*>(p + g.mnodes);
    a->mesh_leaves = reinterpret_cast<uint32_t*>(p + g.mleaves);
    a->tile_rng = reinterpret_cast<uint2*>(p + g.trng);
    a->keys_a = reinterpret_cast<uint64_t*>(p + g.ka);
    a->keys_b = reinterpret_cast<uint64_t*>(p + g.kb);
    a->vals_a = reinterpret_cast<uint32_t*>(p + g.va);
    a->vals_b = reinterpret_cast<uint32_t*>(p + g.vb);
    a->pairs = reinterpret_cast<uint64_t*>(p + g.pairs);
    a->kids = reinterpret_cast<ChildPair*>(p + g.kids);
    a->bvh2 = reinterpret_cast<Node2*>(p + g.bvh2);
    a->bvh8 = reinterpret_cast<Node8*>(p + g.bvh8);
    a->prim_idx = reinterpret_cast<uint32_t*>(p + g.prim);
    a->results = reinterpret_cast<nxb_batch_mesh*>(p + g.res);
}

void batch_groups(const uint32_t* h_off, const uint32_t* h_off8, uint32_t meshes, uint32_t want, MeshGroups* g) {
    want = std::max(1u, std::min(want, kMaxMeshGroups));
    const uint64_t total = h_off[meshes];
    g->count = 0;
    g->mesh[0] = 0;
    for (uint32_t k = 1; k < want; ++k) {
        // the first mesh starting at or after k/want of the primitives
        const uint32_t target = (uint32_t)(total * k / want);
        const uint32_t m = (uint32_t)(std::lower_bound(h_off, h_off + meshes, target) - h_off);
        if (m > g->mesh[g->count] && m < meshes) g->mesh[++g->count] = m;
    }
    g->mesh[++g->count] = meshes;
    for (uint32_t k = 0; k <= g->count; ++k) {
        g->prim[k] = h_off[g->mesh[k]];
        g->slot[k] = h_off8[g->mesh[k]];
    }
}

nxb_status batch_enqueue(const BatchArena& a, const void* prims, nxb_prim_type type, const BatchTuning& t,
                         uint32_t* h_err, cudaStream_t s, const MeshGroups* groups, const BatchFork* fork) {
    MeshGroups one{};
    one.count = 1;
    one.mesh[1] = a.meshes;
    one.prim[1] = a.total;
    one.slot[1] = a.slots;
    const MeshGroups& g = (groups && fork && groups->count > 1) ? *groups : one;
    const MeshBatch mb{a.off, a.off8, a.meshes};
    const SortPlan plan = make_sort_plan(2, 32 + a.mesh_bits, t.digit_bits);
    NXB_TRY(cudaMemsetAsync(a.zero_begin, 0, a.zero_bytes, s));
    if (a.total > 0) {
        NXB_TRY(launch_batch_tile_ranges(mb, a.total, t.block, a.tile_rng, s));
        NXB_TRY(launch_batch_bounds(prims, type, mb, a.total, a.bvh2, a.scene_ord, t.block, a.tile_rng, s));
        MortonFused f{};
        f.zero_ptr = a.lookback;
        f.zero_words = align_up(4 * a.lookback_words_per_pass * plan.passes) / 4;
        f.ones_ptr = a.parent;
        f.ones_words = a.ones_words;
        NXB_TRY(launch_batch_morton(a.bvh2, mb, a.total, a.scene_ord, a.keys_a, a.vals_a, plan, &a.ctrl->hist[0][0],
                                    f, t.block, a.tile_rng, s));
        for (int p = 0; p < plan.passes; ++p) {
            const bool even = (p % 2) == 0;
            NXB_TRY(launch_sort_pass(8, even ? a.keys_a : a.keys_b, even ? a.keys_b : a.keys_a,
                                     even ? a.vals_a : a.vals_b, even ? a.vals_b : a.vals_a, a.total, plan.shift[p],
                                     plan.bits[p], a.ctrl->hist[p], a.lookback + p * a.lookback_words_per_pass,
                                     a.ctrl->tile_ctr + p, &a.ctrl->error_word, s));
        }
    }
    NXB_TRY(launch_bvh8_batch_init(a.pairs, a.slots, mb, a.ctr8, a.mesh_nodes, a.mesh_leaves, g, s));
    if (a.total > 0) {
        const bool in_a = (plan.passes % 2) == 0;
        uint64_t* keys = in_a ? a.keys_a : a.keys_b;
        uint32_t* perm = in_a ? a.vals_a : a.vals_b;
        uint32_t* tokens = in_a ? a.vals_b : a.vals_a;
        // H-PLOC group by group on s; the collapse of group k follows it on
        // the side stream (ordered by an event, no wait inside any kernel),
        // overlapping H-PLOC of group k+1
        for (uint32_t k = 0; k < g.count; ++k) {
            NXB_TRY(launch_hploc_batch(keys, perm, a.parent, a.bvh2, mb, g.prim[k], g.prim[k + 1], t.radius, tokens,
                                       a.pol, a.ctrl->leaf_ctr + k, &a.ctrl->error_word, t.hploc_ctas_per_sm, s,
                                       a.kids));
            const uint32_t m0 = g.mesh[k];
            const MeshBatch view{a.off + m0, a.off8 + m0, g.mesh[k + 1] - m0};
            cudaStream_t bs = s;
            if (g.count > 1) {
                NXB_TRY(cudaEventRecord(fork->hploc[k], s));
                NXB_TRY(cudaStreamWaitEvent(fork->side, fork->hploc[k], 0));
                bs = fork->side;
            }
            NXB_TRY(launch_bvh8_batch(a.bvh2, view, g.prim[k + 1] - g.prim[k], a.bvh8, g.slot[k + 1] - g.slot[k],
                                      a.prim_idx, a.pairs + g.slot[k], a.ctr8 + k * kBvh8CtrWords,
                                      a.mesh_nodes + m0, a.mesh_leaves + m0, &a.ctrl->error_word, t.auction, bs,
                                      a.kids));
        }
        if (g.count > 1) {
            NXB_TRY(cudaEventRecord(fork->join, fork->side));
            NXB_TRY(cudaStreamWaitEvent(s, fork->join, 0));
        }
    }
    NXB_TRY(launch_batch_finalize(mb, a.scene_ord, a.mesh_nodes, a.mesh_leaves, a.results, s));
    if (h_err)
        NXB_TRY(cudaMemcpyAsync(h_err, &a.ctrl->error_word, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    return NXB_OK;
}

}  // namespace nxb

using namespace nxb;

struct nxb_batch {
    nxb_prim_type type = NXB_PRIM_TRIANGLE;
    bool auction = false;
    BatchArena arena;
    nxb_batch_tuning tuning{};
    unsigned char* mem = nullptr;
    uint32_t* h_err = nullptr;  // pinned; the graph copies the error word here
    cudaStream_t cap_stream = nullptr;
    BatchFork fork{};               // side stream and events of a grouped capture
    std::vector<uint32_t> h_off;    // host copies of the offsets (mesh groups)
    std::vector<uint32_t> h_off8;
    MeshGroups groups{};            // of the current tuning
    cudaGraphExec_t exec = nullptr;
    const void* graph_prims = nullptr;
    bool graph_valid = false;
};

namespace {

nxb_status status_of_word(uint32_t w) {
    if (w == 0) return NXB_OK;
    if (w & (NXB_DEVERR_SORT_LOOKBACK_TIMEOUT | NXB_DEVERR_BVH8_QUEUE_TIMEOUT)) return NXB_ERR_DEVICE_TIMEOUT;
    return NXB_ERR_DEVICE_INVARIANT;
}

BatchTuning tuning_of(const nxb_batch_tuning& t, bool auction) {
    BatchTuning r;
    r.auction = auction;
    r.digit_bits = t.sort_digit_bits;
    r.radius = t.search_radius;
    r.hploc_ctas_per_sm = t.hploc_ctas_per_sm;
    r.groups = t.fusion_groups ? t.fusion_groups : 1u;
    r.block = t.block_size ? t.block_size : 256u;
    return r;
}

nxb_status capture(nxb_batch* b, const void* prims) {
    cudaGraph_t g = nullptr;
    NXB_TRY(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeRelaxed));
    const nxb_status st = batch_enqueue(b->arena, prims, b->type, tuning_of(b->tuning, b->auction), b->h_err,
                                        b->cap_stream, &b->groups, &b->fork);
    const cudaError_t ec = cudaStreamEndCapture(b->cap_stream, &g);
    if (st != NXB_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (ec) return record_cuda_error(ec);
    cudaError_t e = cudaSuccess;
    if (b->exec) {
        cudaGraphExecUpdateResultInfo info{};
        if (cudaGraphExecUpdate(b->exec, g, &info) != cudaSuccess) {
            cudaGetLastError();  // the update is refused when the topology changed: instantiate anew
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
    }
    if (!b->exec) e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e) return record_cuda_error(e);
    b->graph_prims = prims;
    b->graph_valid = true;
    return NXB_OK;
}

void release(nxb_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->fork.side) cudaStreamDestroy(b->fork.side);
    for (cudaEvent_t ev : b->fork.hploc)
        if (ev) cudaEventDestroy(ev);
    if (b->fork.join) cudaEventDestroy(b->fork.join);
    if (b->h_err) cudaFreeHost(b->h_err);
    if (b->mem) cudaFree(b->mem);
    delete b;
}

}  // namespace

extern "C" {

nxb_status nxb_batch_create(nxb_prim_type type, const uint32_t* h_off, uint32_t meshes,
                            const nxb_build_config* cfg, nxb_batch** out) {
    if (!h_off || !out || meshes == 0) return NXB_ERR_INVALID_ARGUMENT;
    if (type != NXB_PRIM_AABB && type != NXB_PRIM_TRIANGLE) return NXB_ERR_INVALID_ARGUMENT;
    if (!cfg || !cfg->prioritize_speed) return NXB_ERR_UNSUPPORTED;  // batches sort 30-bit codes
    const uint32_t radius = cfg->search_radius ? cfg->search_radius : 8u;
    if (radius != 4 && radius != 8 && radius != 16) return NXB_ERR_UNSUPPORTED;
    if (cfg->flags & ~NXB_BUILD_AUCTION) return NXB_ERR_UNSUPPORTED;
    if (h_off[0] != 0) return NXB_ERR_INVALID_ARGUMENT;
    for (uint32_t m = 0; m < meshes; ++m)
        if (h_off[m + 1] < h_off[m]) return NXB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::vector<uint32_t> off8(meshes + 1);
    nxb_batch* b = new nxb_batch();
    if (!batch_layout(h_off, meshes, off8.data(), &b->arena)) {
        delete b;
        return NXB_ERR_UNSUPPORTED;
    }
    b->type = type;
    b->auction = (cfg->flags & NXB_BUILD_AUCTION) != 0;
    b->tuning.sort_digit_bits = 8;
    b->tuning.search_radius = radius;
    b->tuning.hploc_ctas_per_sm = 0;
    b->tuning.fusion_groups = 1;
    b->tuning.block_size = 256;
    b->h_off.assign(h_off, h_off + meshes + 1);
    b->h_off8 = off8;
    batch_groups(h_off, off8.data(), meshes, 1, &b->groups);
    cudaError_t e = cudaMalloc(&b->mem, b->arena.bytes);
    if (!e) e = cudaMallocHost(&b->h_err, sizeof(uint32_t));
    if (!e) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
    if (!e) e = cudaStreamCreateWithFlags(&b->fork.side, cudaStreamNonBlocking);
    for (uint32_t k = 0; k < kMaxMeshGroups && !e; ++k)
        e = cudaEventCreateWithFlags(&b->fork.hploc[k], cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&b->fork.join, cudaEventDisableTiming);
    if (!e) {
        batch_bind(b->mem, &b->arena);
        e = cudaMemcpy(b->arena.off, h_off, 4ull * (meshes + 1), cudaMemcpyHostToDevice);
    }
    if (!e) e = cudaMemcpy(b->arena.off8, off8.data(), 4ull * (meshes + 1), cudaMemcpyHostToDevice);
    if (e) {
        const nxb_status st = record_cuda_error(e);
        release(b);
        return st;
    }
    *out = b;
    return NXB_OK;
}

nxb_status nxb_batch_destroy(nxb_batch* b) {
    if (!b) return NXB_ERR_INVALID_ARGUMENT;
    release(b);
    return NXB_OK;
}

nxb_status nxb_batch_build_async(nxb_batch* b, const void* prims, cudaStream_t s) {
    if (!b || (!prims && b->arena.total)) return NXB_ERR_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(prims) & 3u) != 0) return NXB_ERR_INVALID_ARGUMENT;
    if (!b->graph_valid || b->graph_prims != prims) {
        const nxb_status st = capture(b, prims);
        if (st != NXB_OK) return st;
    }
    NXB_TRY(cudaGraphLaunch(b->exec, s));
    return NXB_OK;
}

nxb_status nxb_batch_wait(nxb_batch* b, cudaStream_t s, nxb_batch_mesh* h_meshes) {
    if (!b) return NXB_ERR_INVALID_ARGUMENT;
    NXB_TRY(cudaStreamSynchronize(s));
    const nxb_status st = status_of_word(*b->h_err);
    if (st != NXB_OK) return st;
    if (h_meshes)
        NXB_TRY(cudaMemcpy(h_meshes, b->arena.results, sizeof(nxb_batch_mesh) * b->arena.meshes,
                           cudaMemcpyDeviceToHost));
    return NXB_OK;
}

nxb_status nxb_batch_build(nxb_batch* b, const void* prims, cudaStream_t s, nxb_batch_mesh* h_meshes) {
    const nxb_status st = nxb_batch_build_async(b, prims, s);
    if (st != NXB_OK) return st;
    return nxb_batch_wait(b, s, h_meshes);
}

nxb_status nxb_batch_get_arrays(const nxb_batch* b, nxb_batch_arrays* out) {
    if (!b || !out) return NXB_ERR_INVALID_ARGUMENT;
    const BatchArena& a = b->arena;
    out->bvh2_nodes = reinterpret_cast<const nxb_bvh2_node*>(a.bvh2);
    out->bvh8_nodes = reinterpret_cast<const nxb_bvh8_node*>(a.bvh8);
    out->prim_idx = a.prim_idx;
    out->meshes = a.results;
    out->mesh_count = a.meshes;
    out->prim_count = a.total;
    out->bvh2_node_capacity = 2ull * a.total;
    out->bvh8_node_capacity = a.slots;
    return NXB_OK;
}

nxb_status nxb_batch_set_tuning(nxb_batch* b, const nxb_batch_tuning* t) {
    if (!b || !t) return NXB_ERR_INVALID_ARGUMENT;
    if (!batch_digit_ok(b->arena.mesh_bits, t->sort_digit_bits)) return NXB_ERR_UNSUPPORTED;
    if (t->search_radius != 4 && t->search_radius != 8 && t->search_radius != 16) return NXB_ERR_UNSUPPORTED;
    if (t->block_size != 0 && t->block_size != 128 && t->block_size != 256 && t->block_size != 512)
        return NXB_ERR_UNSUPPORTED;
    if (t->fusion_groups > kMaxMeshGroups) return NXB_ERR_UNSUPPORTED;
    b->tuning.sort_digit_bits = t->sort_digit_bits;
    b->tuning.search_radius = t->search_radius;
    b->tuning.hploc_ctas_per_sm = t->hploc_ctas_per_sm;
    b->tuning.fusion_groups = t->fusion_groups ? t->fusion_groups : 1u;
    b->tuning.block_size = t->block_size ? t->block_size : 256u;
    batch_groups(b->h_off.data(), b->h_off8.data(), b->arena.meshes, b->tuning.fusion_groups, &b->groups);
    b->graph_valid = false;
    return NXB_OK;
}

nxb_status nxb_batch_get_tuning(const nxb_batch* b, nxb_batch_tuning* t) {
    if (!b || !t) return NXB_ERR_INVALID_ARGUMENT;
    *t = b->tuning;
    return NXB_OK;
}

nxb_status nxb_batch_autotune(nxb_batch* b, const void* prims, uint32_t flags, uint32_t repeats, cudaStream_t s,
                              nxb_batch_tuning* out) {
    if (!b) return NXB_ERR_INVALID_ARGUMENT;
    if (flags & ~NXB_TUNE_RADIUS) return NXB_ERR_UNSUPPORTED;
    if (repeats == 0) repeats = 3;
    std::vector<uint32_t> radii;
    if (flags & NXB_TUNE_RADIUS)
        radii = {4, 8, 16};
    else
        radii = {b->tuning.search_radius};
    // candidates: every combination of the knobs that keep each tree as it
    // is (and the radius, when asked for)
    const nxb_batch_tuning start = b->tuning;
    std::vector<nxb_batch_tuning> cand;
    for (uint32_t r : radii)
        for (uint32_t d : {8u, 7u, 6u, 5u, 4u}) {
            if (!batch_digit_ok(b->arena.mesh_bits, d)) continue;
            for (uint32_t c : {0u, 4u})
                for (uint32_t g : {1u, 2u, 4u})
                    for (uint32_t bs : {256u, 128u, 512u}) {
                        nxb_batch_tuning t = start;
                        t.search_radius = r;
                        t.sort_digit_bits = d;
                        t.hploc_ctas_per_sm = c;
                        t.fusion_groups = g;
                        t.block_size = bs;
                        cand.push_back(t);
                    }
        }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    NXB_TRY(cudaEventCreate(&e0));
    const cudaError_t ce = cudaEventCreate(&e1);
    if (ce) {
        cudaEventDestroy(e0);
        return record_cuda_error(ce);
    }
    nxb_batch_tuning best = start;
    best.build_ms = 3.4e38f;
    uint32_t tried = 0;
    nxb_status st = NXB_OK;
    for (nxb_batch_tuning t : cand) {
        if ((st = nxb_batch_set_tuning(b, &t)) != NXB_OK) break;
        if ((st = nxb_batch_build(b, prims, s, nullptr)) != NXB_OK) break;  // capture + warm-up
        std::vector<float> ms;
        for (uint32_t k = 0; k < repeats && st == NXB_OK; ++k) {
            cudaEventRecord(e0, s);
            st = nxb_batch_build_async(b, prims, s);
            cudaEventRecord(e1, s);
            if (st == NXB_OK) st = nxb_batch_wait(b, s, nullptr);
            float t_ms = 0.f;
            cudaEventElapsedTime(&t_ms, e0, e1);
            ms.push_back(t_ms);
        }
        if (st != NXB_OK) break;
        std::sort(ms.begin(), ms.end());
        t.build_ms = ms[ms.size() / 2];
        ++tried;
        if (t.build_ms < best.build_ms) best = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != NXB_OK) {
        nxb_batch_set_tuning(b, &start);
        return st;
    }
    nxb_batch_set_tuning(b, &best);
    b->tuning.build_ms = best.build_ms;
    b->tuning.candidates_tried = tried;
    if (out) *out = b->tuning;
    return NXB_OK;
}

nxb_status nxb_batch_mesh_bvh8_to_host(const nxb_batch* b, uint32_t mesh, nxb_bvh8* h) {
    if (!b || !h || mesh >= b->arena.meshes) return NXB_ERR_INVALID_ARGUMENT;
    nxb_batch_mesh r{};
    NXB_TRY(cudaMemcpy(&r, b->arena.results + mesh, sizeof(r), cudaMemcpyDeviceToHost));
    if (r.prim_count == 0 || r.bvh8_node_count == 0) return NXB_ERR_INVALID_ARGUMENT;
    nxb_bvh8 d{};
    d.nodes = reinterpret_cast<nxb_bvh8_node*>(b->arena.bvh8 + r.bvh8_offset);
    d.node_count = r.bvh8_node_count;
    d.prim_idx = b->arena.prim_idx + r.prim_offset;
    d.prim_count = r.prim_count;
    d.bounds = r.scene_bounds;
    return nxb_bvh8_to_host(&d, h);
}

}  // extern "C"
