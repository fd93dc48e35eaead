// hploc.cu - stage 4: H-PLOC binary BVH (Benthin et al. 2024).
//
// Replaces BuildBVH2Kernel (NexusBVH/src/Cuda/BinaryBuilder.cu:200-273).
// The decisions are the reference's, so the topology and every box are
// identical; how they are computed on the GPU differs:
//   * the bottom-up LBVH climb (Apetrei 2014; FindParentId/Delta,
//     BinaryBuilder.cu:14-40) runs on a persistent grid whose lanes take a
//     new leaf as soon as their climb stops (see hploc_kernel); ranges are
//     handed over with relaxed exchanges, a pass that merges is bracketed by
//     acquire/release fences, and all cross-CTA data is read through L2
//     (the reference reads cluster ids and node boxes with plain,
//     L1-cacheable loads, which can return stale lines written by another
//     SM);
//   * LoadIndices (:42-57) loads the left and right windows of 16 cluster
//     ids in one round trip (lanes 0-15 and 16-31) and packs them with one
//     shuffle, instead of two dependent loads;
//   * FindNearestNeighbor (:126-163) is evaluated as what it computes: for
//     lane i, the first minimum of the union area (compared as uint32 bit
//     patterns) over candidates i+1, i-1, i+2, i-2, ..., i+R, i-R.  Each
//     pair's area is computed once and sent back to the partner with one
//     shuffle (7 shuffles per radius step instead of 10); at radius 8 a lane
//     fetches only 4 neighbour boxes, at the offsets of a difference cover
//     of the distances 1..8, and every pair is computed by one lane and
//     shuffled to both of its lanes (36 shuffles per round instead of 56;
//     at radius 16, 8 fetches and 72 shuffles instead of 16 and 112; at
//     radius 4, 3 fetches and 23 shuffles instead of 4 and 28);
//   * the merge and the order-preserving compaction follow
//     MergeClustersCreateBVH2Node (:71-124); internal nodes are numbered
//     from the tokens of the clusters they absorb instead of from a global
//     atomic counter (see merge_step), and the root still lands at 2n-2.
// A window whose valid ids are not a prefix (impossible for a correct
// climb) sets NXB_DEVERR_HPLOC_INVALID_CLUSTER instead of reading out of
// bounds.
#include <algorithm>

#include "pipeline.h"

namespace nxb {
namespace {

constexpr int kThreads = 128;
constexpr uint32_t kMergeThreshold = 16;  // MERGING_THRESHOLD, BinaryBuilder.cu:10

// Delta (BinaryBuilder.cu:16-28) of sorted positions a and b of the mesh
// whose first position is s; the index tie-break uses mesh-local positions.
__device__ __forceinline__ uint64_t delta(const uint32_t* k, uint32_t a, uint32_t b, uint32_t s) {
    return (((uint64_t)__ldg(k + a) << 32) | (a - s)) ^ (((uint64_t)__ldg(k + b) << 32) | (b - s));
}
__device__ __forceinline__ uint64_t delta(const uint64_t* k, uint32_t a, uint32_t b, uint32_t s) {
    const uint64_t d = __ldg(k + a) ^ __ldg(k + b);
    return d ? d : (uint64_t)((a - s) ^ (b - s));
}
// Batched 30-bit keys: mesh << 32 | code, sorted as one key; the delta is
// the 32-bit one of the code.
__device__ __forceinline__ uint64_t delta(const MeshKey* k, uint32_t a, uint32_t b, uint32_t s) {
    const uint32_t ka = (uint32_t)__ldg(&k[a].v), kb = (uint32_t)__ldg(&k[b].v);
    return (((uint64_t)ka << 32) | (a - s)) ^ (((uint64_t)kb << 32) | (b - s));
}

// The warp's row of shared memory: cluster k of the window at row[k]
// (min xyz, max x) and row[32 + k] (max yz, id, token).
__device__ __forceinline__ void put_row(uint4* row, uint32_t k, const Box& b, uint32_t cid, uint32_t ctok) {
    row[k] = make_uint4(__float_as_uint(b.mn.x), __float_as_uint(b.mn.y), __float_as_uint(b.mn.z),
                        __float_as_uint(b.mx.x));
    row[32 + k] = make_uint4(__float_as_uint(b.mx.y), __float_as_uint(b.mx.z), cid, ctok);
}
__device__ __forceinline__ Box row_box(const uint4* row, uint32_t k) {
    const uint4 a = row[k];
    const uint2 b = *reinterpret_cast<const uint2*>(row + 32 + k);
    Box r;
    r.mn = make_float3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
    r.mx = make_float3(__uint_as_float(a.w), __uint_as_float(b.x), __uint_as_float(b.y));
    return r;
}

// COVER selects the difference-cover search (single-mesh builds, where it
// measured faster at every radius; the batched kernel keeps the plain one).
// ROW: the neighbour boxes are read from the warp's row of shared memory
// instead of shuffled (see merge_step).
template <int R, bool COVER, bool ROW = false>
__device__ __forceinline__ uint32_t nearest_neighbour(uint32_t num, const Box& cb, const uint4* row = nullptr) {
    const uint32_t lane = lane_id();
    auto fetch = [&](uint32_t k) -> Box {
        if constexpr (ROW)
            return row_box(row, (lane + k) & 31u);
        else
            return shfl_box(cb, (lane + k) & 31u);
    };
    uint32_t best = kInvalid, best_idx = kInvalid;
    if constexpr (R == 4 && COVER) {
        // marks {0, 1, 2, 4}: 1 = 1-0, 2 = 2-0, 3 = 4-1, 4 = 4-0
        auto pair = [&](const Box& lo_box, const Box& hi_box, uint32_t a, uint32_t d) -> uint32_t {
            if (((lane + a) & 31u) + d >= num) return kInvalid;
            Box u = hi_box;
            grow(u, lo_box);
            return __float_as_uint(half_area(u));
        };
        auto pick = [&](uint32_t f, uint32_t a, uint32_t d) {
            const uint32_t fwd = a ? __shfl_sync(kFullMask, f, (lane - a) & 31u) : f;
            const uint32_t back = __shfl_sync(kFullMask, f, (lane - d - a) & 31u);
            if (fwd < best) {
                best = fwd;
                best_idx = lane + d;
            }
            if (back < best) {
                best = back;
                best_idx = lane - d;
            }
        };
        const Box b1 = fetch(1);
        pick(pair(cb, b1, 0, 1), 0, 1);
        {
            const Box b2 = fetch(2);
            pick(pair(cb, b2, 0, 2), 0, 2);
        }
        const Box b4 = fetch(4);
        const uint32_t f3 = pair(b1, b4, 1, 3), f4 = pair(cb, b4, 0, 4);
        pick(f3, 1, 3);
        pick(f4, 0, 4);
    } else if constexpr ((R == 8 || R == 16) && COVER) {
        // The marks {0, 1, 2, 5, 8} have every distance 1..8 as a difference
        // (1 = 1-0, 2 = 2-0, 3 = 5-2, 4 = 5-1, 5 = 5-0, 6 = 8-2, 7 = 8-1,
        // 8 = 8-0).  Each lane fetches the boxes of lanes +1, +2, +5 and +8
        // (4 boxes instead of 8) and computes, for each distance d, the area
        // of the pair (lane + a_d, lane + a_d + d), lanes taken modulo 32; a
        // pair that wraps or reaches past the last cluster is invalid.  Every
        // pair of the window is thereby computed by exactly one lane, and its
        // area is shuffled to the two lanes it belongs to: 36 shuffles per
        // round instead of 56.  The union is grown in the same operand order
        // as below (upper box grown by the lower one), so every area has the
        // same bits, and the candidates are compared in the same order.
        auto pair = [&](const Box& lo_box, const Box& hi_box, uint32_t a, uint32_t d) -> uint32_t {
            if (((lane + a) & 31u) + d >= num) return kInvalid;
            Box u = hi_box;
            grow(u, lo_box);
            return __float_as_uint(half_area(u));
        };
        // two pairs' areas at once (half_area2)
        auto pair2 = [&](const Box& lo0, const Box& hi0, uint32_t a0, uint32_t d0, const Box& lo1, const Box& hi1,
                         uint32_t a1, uint32_t d1, uint32_t& f0, uint32_t& f1) {
            Box u0 = hi0, u1 = hi1;
            grow(u0, lo0);
            grow(u1, lo1);
            float r0, r1;
            half_area2(u0, u1, r0, r1);
            f0 = ((lane + a0) & 31u) + d0 >= num ? kInvalid : __float_as_uint(r0);
            f1 = ((lane + a1) & 31u) + d1 >= num ? kInvalid : __float_as_uint(r1);
        };
        auto pick = [&](uint32_t f, uint32_t a, uint32_t d) {
            const uint32_t fwd = a ? __shfl_sync(kFullMask, f, (lane - a) & 31u) : f;
            const uint32_t back = __shfl_sync(kFullMask, f, (lane - d - a) & 31u);
            if (fwd < best) {
                best = fwd;
                best_idx = lane + d;
            }
            if (back < best) {
                best = back;
                best_idx = lane - d;
            }
        };
        const Box b1 = fetch(1);
        const Box b2 = fetch(2);
        {
            uint32_t f1, f2;
            pair2(cb, b1, 0, 1, cb, b2, 0, 2, f1, f2);
            pick(f1, 0, 1);
            pick(f2, 0, 2);
        }
        {
            const Box b5 = fetch(5);
            uint32_t f3, f4;
            pair2(b2, b5, 2, 3, b1, b5, 1, 4, f3, f4);
            pick(f3, 2, 3);
            pick(f4, 1, 4);
            pick(pair(cb, b5, 0, 5), 0, 5);
        }
        {
            const Box b8 = fetch(8);
            uint32_t f6, f7;
            pair2(b2, b8, 2, 6, b1, b8, 1, 7, f6, f7);
            pick(f6, 2, 6);
            pick(f7, 1, 7);
            pick(pair(cb, b8, 0, 8), 0, 8);
        }
        if constexpr (R == 16) {
            // distances 9..16 are 8 + (1..8): the same low boxes 0, 1, 2
            // against the boxes of lanes +9, +10, +13 and +16
            {
                const Box b9 = fetch(9);
                const Box b10 = fetch(10);
                uint32_t f9, f10;
                pair2(cb, b9, 0, 9, cb, b10, 0, 10, f9, f10);
                pick(f9, 0, 9);
                pick(f10, 0, 10);
            }
            {
                const Box b13 = fetch(13);
                uint32_t f11, f12;
                pair2(b2, b13, 2, 11, b1, b13, 1, 12, f11, f12);
                pick(f11, 2, 11);
                pick(f12, 1, 12);
                pick(pair(cb, b13, 0, 13), 0, 13);
            }
            const Box b16 = fetch(16);
            uint32_t f14, f15;
            pair2(b2, b16, 2, 14, b1, b16, 1, 15, f14, f15);
            pick(f14, 2, 14);
            pick(f15, 1, 15);
            pick(pair(cb, b16, 0, 16), 0, 16);
        }
    } else {
#pragma unroll
        for (uint32_t r = 1; r <= (uint32_t)R; ++r) {
            Box nb = shfl_box(cb, (lane + r) & 31u);
            uint32_t a = kInvalid;
            if (lane + r < num) {
                grow(nb, cb);
                a = __float_as_uint(half_area(nb));
            }
            const uint32_t back = __shfl_sync(kFullMask, a, (lane - r) & 31u);
            if (a < best) {
                best = a;
                best_idx = lane + r;
            }
            if (back < best) {
                best = back;
                best_idx = lane - r;
            }
        }
    }
    return best_idx;
}

struct MergeCtx {
    Node2* nodes;
    uint32_t* tok;             // first-leaf token of each stored cluster
    Node2* rec;                // if not null: stored clusters as {box, id, token} records
    ChildPair* kids;           // if not null: each internal node's two children, at node - n
    uint32_t* parent_of_last;  // node whose child is node 2n-2 (root fix-up)
    uint32_t n;
    uint32_t node_limit;       // 2n-1
    uint32_t* err;
};

// One round of PLOC merging (MergeClustersCreateBVH2Node,
// BinaryBuilder.cu:71-124).  Node numbering: every cluster carries the
// sorted position of its first leaf (its token); merging lanes i < j keeps
// token i, and token j is never seen again.  The n-1 merges therefore
// absorb the tokens 1..n-1 exactly once, and node n-1+token(j) is a
// collision-free index in [n, 2n-1) that needs no global counter (the
// reference takes one atomicAdd on a single counter per merge round).
// ROW: the window's clusters also live in the warp's row of shared memory,
// which holds them at the start of every round: the merge reads its
// partner there, and the order-preserving compaction goes through it (each
// kept cluster written at its rank, every lane reading its own slot)
// instead of a find-n-th-set-bit and eight shuffles.
template <bool ROW>
__device__ __forceinline__ uint32_t merge_step(const MergeCtx& m, uint32_t num, uint32_t nn, uint32_t& cid,
                                               uint32_t& ctok, Box& cb, uint4* row) {
    const uint32_t lane = lane_id();
    const uint32_t nn_of_nn = __shfl_sync(kFullMask, nn, nn & 31u);
    const bool mutual = lane < num && lane == nn_of_nn;
    const bool merge = mutual && lane < nn;
    const uint32_t mmask = __ballot_sync(kFullMask, merge);
    const uint32_t mcount = __popc(mmask);
    uint32_t ncid, ntok;
    Box nb;
    if constexpr (ROW) {
        if (merge) {
            nb = row_box(row, nn & 31u);
            const uint2 it = *reinterpret_cast<const uint2*>(&row[32 + (nn & 31u)].z);
            ncid = it.x;
            ntok = it.y;
        }
    } else {
        ncid = __shfl_sync(kFullMask, cid, nn & 31u);
        ntok = __shfl_sync(kFullMask, ctok, nn & 31u);
        nb = shfl_box(cb, nn & 31u);
    }
    if (merge) {
        const uint32_t idx = m.n - 1 + ntok;
        const bool ok = idx < m.node_limit && ntok != 0;
        if (ok && m.kids) store_child_pair(m.kids + (idx - m.n), cb, nb, cid, ncid);
        grow(cb, nb);
        if (ok) {
            store_node(m.nodes, idx, cb, cid, ncid);
            if (cid == m.node_limit - 1 || ncid == m.node_limit - 1) atomicExch(m.parent_of_last, idx);
        } else {
            set_error(m.err, NXB_DEVERR_HPLOC_INVALID_CLUSTER);
        }
        cid = idx;
    }
    const uint32_t vmask = __ballot_sync(kFullMask, merge || !mutual);
    if constexpr (ROW) {
        const uint32_t rank = __popc(vmask & lanemask_lt());
        __syncwarp();  // the previous round's reads of the row are done
        if ((vmask >> lane) & 1u) put_row(row, rank, cb, cid, ctok);
        __syncwarp();
        if (lane < (uint32_t)__popc(vmask)) {
            const uint4 a = row[lane], b = row[32 + lane];
            cb.mn = make_float3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
            cb.mx = make_float3(__uint_as_float(a.w), __uint_as_float(b.x), __uint_as_float(b.y));
            cid = b.z;
            ctok = b.w;
        } else {
            cid = kInvalid;
        }
    } else {
        const int sh = __fns(vmask, 0, lane + 1);
        cid = __shfl_sync(kFullMask, cid, (uint32_t)sh & 31u);
        ctok = __shfl_sync(kFullMask, ctok, (uint32_t)sh & 31u);
        cb = shfl_box(cb, (uint32_t)sh & 31u);
        if (sh < 0) cid = kInvalid;
    }
    return num - mcount;
}

// The last merge of the build (the root, two clusters left in lanes 0 and
// 1).  The root must sit at node 2n-2, like the reference's; if the token
// numbering put another node there, that node moves to the root's own
// slot n-1+token(lane 1) and its parent's child index is patched.
__device__ __forceinline__ void merge_root(const MergeCtx& m, uint32_t& cid, uint32_t& ctok, Box& cb) {
    const uint32_t lane = lane_id();
    const uint32_t b_cid = __shfl_sync(kFullMask, cid, 1);
    const uint32_t b_tok = __shfl_sync(kFullMask, ctok, 1);
    const Box b_box = shfl_box(cb, 1);
    __syncwarp();
    if (lane == 0) {
        const uint32_t root = m.node_limit - 1;
        const uint32_t natural = m.n - 1 + b_tok;
        uint32_t a = cid, b = b_cid;
        if (natural != root) {
            if (natural >= m.node_limit) {
                set_error(m.err, NXB_DEVERR_HPLOC_INVALID_CLUSTER);
            } else {
                const uint4* src = reinterpret_cast<const uint4*>(m.nodes + root);
                uint4* dst = reinterpret_cast<uint4*>(m.nodes + natural);
                const uint4 lo = __ldcg(src), hi = __ldcg(src + 1);
                __stcg(dst, lo);
                __stcg(dst + 1, hi);
                if (m.kids) {  // the moved node's child pair moves with it
                    const uint4* ks = reinterpret_cast<const uint4*>(m.kids + (root - m.n));
                    uint4* kd = reinterpret_cast<uint4*>(m.kids + (natural - m.n));
                    const uint4 k0 = __ldcg(ks), k1 = __ldcg(ks + 1), k2 = __ldcg(ks + 2), k3 = __ldcg(ks + 3);
                    __stcg(kd, k0);
                    __stcg(kd + 1, k1);
                    __stcg(kd + 2, k2);
                    __stcg(kd + 3, k3);
                }
                if (a == root) {
                    a = natural;
                } else if (b == root) {
                    b = natural;
                } else {
                    const uint32_t p = __ldcg(m.parent_of_last);
                    if (p < m.node_limit && p >= m.n) {
                        uint32_t* pl = reinterpret_cast<uint32_t*>(m.nodes + p) + 6;
                        const uint32_t side = __ldcg(pl) == root ? 0u : 1u;
                        __stcg(pl + side, natural);
                        if (m.kids) __stcg(&m.kids[p - m.n].li + side, natural);
                    } else {
                        set_error(m.err, NXB_DEVERR_HPLOC_INVALID_CLUSTER);
                    }
                }
            }
        }
        if (m.kids) store_child_pair(m.kids + (root - m.n), cb, b_box, a, b);
        grow(cb, b_box);
        store_node(m.nodes, root, cb, a, b);
        cid = root;
    }
    if (lane == 1) cid = kInvalid;
}

// The mesh of the owner lane: `all` holds the bases of the concatenated
// arrays; the context returned addresses this mesh's nodes and counter.
template <typename Seg>
__device__ __forceinline__ MergeCtx mesh_ctx(const MergeCtx& all, const Seg& seg, MeshSpan me, uint32_t owner,
                                             uint32_t& start) {
    if constexpr (Seg::kBatch) {
        const uint32_t mesh = __shfl_sync(kFullMask, me.m, owner);
        start = __shfl_sync(kFullMask, me.start, owner);
        const uint32_t count = __shfl_sync(kFullMask, me.count, owner);
        return MergeCtx{all.nodes + 2ull * start, all.tok, all.rec, all.kids ? all.kids + start : nullptr,
                        all.parent_of_last + mesh, count, 2 * count - 1, all.err};
    } else {
        start = 0;
        return all;
    }
}

// PlocMerge (BinaryBuilder.cu:200-273, the merge part) for the range of
// lane `owner`; `start` is the first sorted position of its mesh and m
// addresses that mesh's nodes.
template <int R, bool COVER, bool REC>
__device__ __forceinline__ void merge_windows(uint32_t owner, uint32_t left, uint32_t right, uint32_t split,
                                              bool final, uint32_t start, uint32_t* cluster, const MergeCtx& m,
                                              uint4* row) {
    const uint32_t lane = lane_id();
    const uint32_t l_start = __shfl_sync(kFullMask, left, owner);
    const uint32_t r_end = __shfl_sync(kFullMask, right, owner) + 1;
    const uint32_t mid = __shfl_sync(kFullMask, split, owner);
    const bool fin = __shfl_sync(kFullMask, final ? 1u : 0u, owner) != 0;

    // LoadIndices (BinaryBuilder.cu:42-57) for both children at once: lanes
    // 0-15 read the left window, lanes 16-31 the right one.  A child of at
    // most 16 primitives was never merged, so its ids and tokens are the
    // original ones (token = mesh-local position); a larger child was stored
    // compacted.
    const uint32_t l_len = mid - l_start, r_len = r_end - mid;
    const uint32_t l_size = min(l_len, kMergeThreshold);
    const uint32_t r_size = min(r_len, kMergeThreshold);
    uint32_t v = kInvalid, t = kInvalid;
    Box wb;  // REC: the window's box at its position, before compaction
    wb.mn = make_float3(0.f, 0.f, 0.f);
    wb.mx = wb.mn;
    {
        const bool lo = lane < 16;
        const uint32_t k = lo ? lane : lane - 16;
        if (k < (lo ? l_size : r_size)) {
            const uint32_t pos = (lo ? l_start : mid) + k;
            const bool stored = (lo ? l_len : r_len) > kMergeThreshold;
            if constexpr (REC) {
                if (stored) {
                    // a stored window: id, token and box in one record, 16
                    // consecutive records per window
                    const uint4* p = reinterpret_cast<const uint4*>(m.rec + pos);
                    const uint4 a = __ldcg(p), b = __ldcg(p + 1);
                    wb.mn = make_float3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
                    wb.mx = make_float3(__uint_as_float(a.w), __uint_as_float(b.x), __uint_as_float(b.y));
                    v = b.z;
                    t = b.w;
                } else {
                    v = __ldcg(cluster + pos);
                    t = pos - start;
                    if (v < m.node_limit) wb = load_box_cg(m.nodes, v);
                }
            } else {
                v = __ldcg(cluster + pos);
                t = stored ? __ldcg(m.tok + pos) : pos - start;
            }
        }
    }
    const uint32_t vb = __ballot_sync(kFullMask, v != kInvalid);
    const uint32_t num_left = __popc(vb & 0xFFFFu), num_right = __popc(vb >> 16);
    if ((vb & 0xFFFFu) != ((1u << num_left) - 1u) || (vb >> 16) != ((1u << num_right) - 1u)) {
        if (lane == 0) set_error(m.err, NXB_DEVERR_HPLOC_INVALID_CLUSTER);
        return;
    }
    uint32_t num = num_left + num_right;
    const uint32_t src = (lane < num_left ? lane : 16u + lane - num_left) & 31u;
    uint32_t cid = __shfl_sync(kFullMask, v, src);
    uint32_t ctok = __shfl_sync(kFullMask, t, src);
    if (lane >= num) cid = kInvalid;
    if (__ballot_sync(kFullMask, lane < num && (cid >= m.node_limit || ctok >= m.n))) {
        if (lane == 0) set_error(m.err, NXB_DEVERR_HPLOC_INVALID_CLUSTER);
        return;
    }
    Box cb;
    if constexpr (REC) {
        cb = shfl_box(wb, src);
        if (lane >= num) {
            cb.mn = make_float3(0.f, 0.f, 0.f);
            cb.mx = cb.mn;
        }
    } else {
        if (lane < num) {
            cb = load_box_cg(m.nodes, cid);
        } else {
            cb.mn = make_float3(0.f, 0.f, 0.f);
            cb.mx = cb.mn;
        }
    }
    if constexpr (REC) {
        put_row(row, lane, cb, cid, ctok);
        __syncwarp();
    }
    const uint32_t threshold = fin ? 1u : kMergeThreshold;
    while (num > threshold) {
        if (fin && num == 2) {
            merge_root(m, cid, ctok, cb);
            num = 1;
            break;
        }
        const uint32_t nn = nearest_neighbour<R, COVER, REC>(num, cb, row);
        num = merge_step<REC>(m, num, nn, cid, ctok, cb, row);
    }
    // StoreIndices (BinaryBuilder.cu:59-69)
    if (lane < num_left + num_right) {
        if constexpr (REC) {
            uint4* p = reinterpret_cast<uint4*>(m.rec + l_start + lane);
            __stcg(p, make_uint4(__float_as_uint(cb.mn.x), __float_as_uint(cb.mn.y), __float_as_uint(cb.mn.z),
                                 __float_as_uint(cb.mx.x)));
            __stcg(p + 1, make_uint4(__float_as_uint(cb.mx.y), __float_as_uint(cb.mx.z), cid, ctok));
        } else {
            __stcg(cluster + l_start + lane, cid);
            __stcg(m.tok + l_start + lane, ctok);
        }
    }
}

// Inlined into the climb loop (measured on GB300: batch1024 9.74 -> 9.35 ms,
// clustered12m H-PLOC 2.52 -> 2.49 ms against an out-of-line call; with the
// launch bounds above neither kernel spills).
template <int R, typename Seg>
__device__ __forceinline__ void ploc_merge(uint32_t owner, uint32_t left, uint32_t right, uint32_t split, bool final,
                                        MeshSpan me, uint32_t* cluster, const MergeCtx& all, const Seg& seg,
                                        uint4* row) {
    if constexpr (Seg::kBatch) {
        uint32_t start;
        const MergeCtx m = mesh_ctx<Seg>(all, seg, me, owner, start);
        merge_windows<R, false, false>(owner, left, right, split, final, start, cluster, m, row);
    } else {
        merge_windows<R, true, true>(owner, left, right, split, final, 0u, cluster, all, row);
    }
}

// The climb with lane refill.  Each lane climbs from a leaf as in the
// reference (FindParentId, exchange on the parent's hand-over slot, merge
// and continue when second to arrive), but a lane that stops takes the next
// unclaimed leaf from its warp's chunk (chunks of `chunk` leaves are
// claimed with one atomicAdd), instead of idling until every lane of its
// warp has finished: the reference runs one thread per leaf, and a warp
// stays resident for as long as any of its lanes still climbs (most stop
// after a step or two).  Nothing waits on another warp.
// Memory order: the hand-over exchanges are relaxed; a pass that merges
// fences (acquire) after its exchanges, before reading the siblings'
// clusters, and (release) after its merges, before the next exchanges.
// Chunk size, measured on GB300 (12.58M clustered triangles, 6,080 resident
// warps): 64 -> 2.91 ms, 256 -> 2.68 ms, 1024 -> 2.90 ms, 4096 -> 5.33 ms.
// Larger chunks keep more of each subtree's climb inside one warp and
// touch the shared counter less; too large leaves warps without work.  So
// the chunk is about two per resident warp, rounded to a multiple of 32
// between 32 and a cap (384 for one mesh, 256 for a batch: the best
// measured caps).  65,536 triangles: 32 (H-PLOC 0.162 -> 0.125 ms against a
// fixed 256); 4.19M: 384 (0.655 -> 0.614 ms); 12.58M: 384 (2.52 ms, as 256).
uint32_t leaf_chunk(uint32_t leaves, uint32_t warps, bool batch) {
    const uint32_t cap = batch ? 256u : 384u;
    const uint32_t c = (leaves / (2u * std::max(warps, 1u)) + 16u) / 32u * 32u;
    return std::max(32u, std::min(c, cap));
}

// Resident CTAs per SM, measured on GB300: a single-mesh build keeps the
// neighbour boxes of its difference-cover search in registers (radius 8:
// 56 registers, 9 CTAs; radius 16: 64 registers, 8 CTAs; with fewer
// registers they spill and lose the gain); the batched kernel and radius 4
// (3 boxes) run at 40 registers.
template <int R, typename Seg>
constexpr int hploc_ctas_per_sm() {
    if constexpr (Seg::kBatch) return 12;
    return R == 8 ? 9 : (R == 16 ? 8 : 12);
}

template <typename K, int R, typename Seg>
__global__ __launch_bounds__(kThreads, hploc_ctas_per_sm<R, Seg>()) void hploc_kernel(const K* __restrict__ keys, uint32_t* cluster,
                                                         uint32_t* parent, Node2* nodes, Seg seg, uint32_t begin,
                                                         uint32_t* tok, uint32_t* parent_of_last, uint32_t* leaf_ctr,
                                                         uint32_t* err, uint32_t end, uint32_t chunk, Node2* rec,
                                                         uint64_t* bvh8_pairs, uint32_t* bvh8_ctr, ChildPair* kids) {
    const uint32_t lane = lane_id();
    if (!Seg::kBatch && bvh8_ctr && blockIdx.x == 0 && threadIdx.x == 0) bvh8_queue_counters(bvh8_ctr);
    const MergeCtx all{nodes, tok, rec, kids, parent_of_last, end, 2 * end - 1, err};
    // each warp's row for the merge compaction (single-mesh builds)
    __shared__ uint4 s_rows[Seg::kBatch ? 1 : kThreads / 32][64];
    uint4* row = s_rows[Seg::kBatch ? 0 : threadIdx.x >> 5];
    uint32_t left = 0, right = 0, split = 0;
    // the lane's mesh; a plain build has one, known at compile time
    MeshSpan me = Seg::kBatch ? MeshSpan{0, 0, 0} : seg.of_prim(0);
    bool active = false;
    uint32_t chunk_next = 0, chunk_end = 0;  // warp-uniform
    bool exhausted = false;                  // warp-uniform
    bool release_due = false;                // warp-uniform: a pass merged, its release fence is pending
    for (;;) {
        // refill stopped lanes with fresh leaves
        uint32_t need = __ballot_sync(kFullMask, !active);
        while (need && !exhausted) {
            if (chunk_next == chunk_end) {
                uint32_t b = 0;
                if (lane == 0) b = begin + atomicAdd(leaf_ctr, chunk);
                b = __shfl_sync(kFullMask, b, 0);
                if (b >= end) {
                    exhausted = true;
                    break;
                }
                chunk_next = b;
                chunk_end = min(b + chunk, end);
            }
            const uint32_t avail = chunk_end - chunk_next;
            const uint32_t rank = __popc(need & lanemask_lt());
            if (!active && ((need >> lane) & 1u) && rank < avail) {
                left = right = chunk_next + rank;
                active = true;
                if constexpr (Seg::kBatch) {
                    me = seg.of_prim(left);
                } else if (bvh8_pairs) {
                    bvh8_pairs[left] = bvh8_queue_slot(left, end);
                }
            }
            const uint32_t took = min((uint32_t)__popc(need), avail);
            chunk_next += took;
            need = __ballot_sync(kFullMask, !active);
        }
        if (!__any_sync(kFullMask, active)) {
            if (release_due) fence_acq_rel_gpu();
            return;
        }
        bool second = false;
        bool go_right = false;
        if (active)
            go_right = left == me.start ||
                       (right != me.start + me.count - 1 &&
                        delta(keys, right, right + 1, me.start) < delta(keys, left - 1, left, me.start));
        if (release_due) {
            // release: the previous pass's clusters and nodes before this
            // pass's hand-overs (the store drain overlaps the refill and the
            // key loads above)
            fence_acq_rel_gpu();
            release_due = false;
        }
        if (active) {
            uint32_t prev;
            if (go_right) {
                prev = atomicExch(parent + right, left);
                if (prev != kInvalid) {
                    split = right + 1;
                    right = prev;
                }
            } else {
                prev = atomicExch(parent + left - 1, right);
                if (prev != kInvalid) {
                    split = left;
                    left = prev;
                }
            }
            second = prev != kInvalid;
            active = second;
        }
        const uint32_t size = right - left + 1;
        const bool final = second && size == me.count;
        uint32_t todo = __ballot_sync(kFullMask, second && (size > kMergeThreshold || final));
        if (todo) {
            fence_acq_rel_gpu();  // acquire: the siblings' clusters
            while (todo) {
                const uint32_t owner = __ffs(todo) - 1;
                ploc_merge<R, Seg>(owner, left, right, split, final, me, cluster, all, seg, row);
                todo &= todo - 1;
            }
            __syncwarp();  // every lane's stores before the owners' next hand-overs
            release_due = true;
        }
    }
}

template <typename K, int R, typename Seg>
cudaError_t launch_r(const K* keys, uint32_t* cluster, uint32_t* parent, Node2* nodes, Seg seg, uint32_t begin,
                     uint32_t end, uint32_t* tok, uint32_t* pol, uint32_t* leaf_ctr, uint32_t* err,
                     uint32_t max_per_sm, cudaStream_t s, Node2* rec, uint64_t* pairs, uint32_t* ctr,
                     ChildPair* kids) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hploc_kernel<K, R, Seg>, kThreads, 0);
    if (max_per_sm && (uint32_t)per_sm > max_per_sm) per_sm = (int)max_per_sm;
    if (per_sm < 1) per_sm = 1;
    const uint32_t want = (end - begin + kThreads - 1) / kThreads;
    const uint32_t grid = std::max(1u, std::min(want, (uint32_t)(device_info().sms * per_sm)));
    const uint32_t chunk = leaf_chunk(end - begin, grid * (kThreads / 32), Seg::kBatch);
    hploc_kernel<K, R, Seg><<<grid, kThreads, 0, s>>>(keys, cluster, parent, nodes, seg, begin, tok, pol, leaf_ctr,
                                                      err, end, chunk, rec, pairs, ctr, kids);
    return cudaGetLastError();
}

template <typename K, typename Seg>
cudaError_t launch_t(const K* keys, uint32_t* cluster, uint32_t* parent, Node2* nodes, Seg seg, uint32_t begin,
                     uint32_t end, uint32_t radius, uint32_t* tok, uint32_t* pol, uint32_t* leaf_ctr, uint32_t* err,
                     uint32_t max_per_sm, cudaStream_t s, Node2* rec = nullptr, uint64_t* pairs = nullptr,
                     uint32_t* ctr = nullptr, ChildPair* kids = nullptr) {
    switch (radius) {
        case 4:
            return launch_r<K, 4>(keys, cluster, parent, nodes, seg, begin, end, tok, pol, leaf_ctr, err, max_per_sm,
                                  s, rec, pairs, ctr, kids);
        case 16:
            return launch_r<K, 16>(keys, cluster, parent, nodes, seg, begin, end, tok, pol, leaf_ctr, err,
                                   max_per_sm, s, rec, pairs, ctr, kids);
        default:
            return launch_r<K, 8>(keys, cluster, parent, nodes, seg, begin, end, tok, pol, leaf_ctr, err, max_per_sm,
                                  s, rec, pairs, ctr, kids);
    }
}

}  // namespace

cudaError_t launch_hploc(uint32_t key_bytes, const void* keys, uint32_t* cluster_idx, uint32_t* parent, Node2* nodes,
                         uint32_t n, uint32_t radius, uint32_t* tokens, uint32_t* parent_of_last, uint32_t* leaf_ctr,
                         uint32_t* err, cudaStream_t s, Node2* records, uint64_t* bvh8_pairs, uint32_t* bvh8_ctr,
                         ChildPair* child_pairs) {
    const SingleMesh seg{n};
    if (!bvh8_pairs != !bvh8_ctr) return cudaErrorInvalidValue;
    if (key_bytes == 4)
        return launch_t((const uint32_t*)keys, cluster_idx, parent, nodes, seg, 0u, n, radius, tokens,
                        parent_of_last, leaf_ctr, err, 0u, s, records, bvh8_pairs, bvh8_ctr, child_pairs);
    return launch_t((const uint64_t*)keys, cluster_idx, parent, nodes, seg, 0u, n, radius, tokens, parent_of_last,
                    leaf_ctr, err, 0u, s, records, bvh8_pairs, bvh8_ctr, child_pairs);
}

cudaError_t launch_hploc_batch(const uint64_t* keys, uint32_t* cluster_idx, uint32_t* parent, Node2* nodes,
                               const MeshBatch& batch, uint32_t begin, uint32_t end, uint32_t radius,
                               uint32_t* tokens, uint32_t* parent_of_last, uint32_t* leaf_ctr, uint32_t* err,
                               uint32_t ctas_per_sm, cudaStream_t s, ChildPair* child_pairs) {
    return launch_t(reinterpret_cast<const MeshKey*>(keys), cluster_idx, parent, nodes, batch, begin, end, radius,
                    tokens, parent_of_last, leaf_ctr, err, ctas_per_sm, s, nullptr, nullptr, nullptr, child_pairs);
}

}  // namespace nxb
