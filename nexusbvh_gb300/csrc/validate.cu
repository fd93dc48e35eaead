// validate.cu - device-side validity checks of a BVH2 and a BVH8.
//
// The checks are the structural and geometric ones of an exhaustive tree
// validator (every primitive in exactly one leaf, every box the union of its
// children's, quantised BVH8 child boxes conservative), computed on the GPU
// so that a full-size build can be checked without copying it to the host.
// The reference has no validator; its trees are the ones built by
// BuildBVH2Kernel / BuildBVH8Kernel (NexusBVH/src/Cuda/BinaryBuilder.cu:200-273,
// WideConverter.cu:225-330) with the node layouts of NexusBVH/include/NXB/BVH.h:8-96.
//
// A host validator walks the tree from the root.  Here every node is checked
// by its own thread instead, and "reached from the root" is decided by
// pointer jumping over parent links: each node holds (ancestor, distance)
// packed in one 64-bit word, and every round replaces it by its ancestor's,
// so after ceil(log2(nodes)) rounds each node's ancestor is the root (then
// the distance is its depth), a node without a parent, or a node of a
// cycle.  The exact box of every BVH8 subtree, needed for the
// conservativeness check, is built bottom-up: a node whose children are all
// leaves starts a climb, and at each parent the last child to arrive (an
// atomic countdown of its inner children) computes the parent's box and
// climbs on; no thread waits for another.
#include <algorithm>

#include "pipeline.h"

namespace nxb {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint64_t pack_link(uint32_t ancestor, uint32_t dist) {
    return ((uint64_t)dist << 32) | ancestor;
}
__device__ __forceinline__ uint32_t link_node(uint64_t l) { return (uint32_t)l; }
__device__ __forceinline__ uint32_t link_dist(uint64_t l) { return (uint32_t)(l >> 32); }

__device__ __forceinline__ uint32_t below(uint32_t mask, uint32_t i) { return __popc(mask & ((1u << i) - 1u)); }

__device__ __forceinline__ Box empty_box() {
    Box b;
    b.mn = make_float3(3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f);
    b.mx = make_float3(-3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f);
    return b;
}

// Box of primitive p, the stage-1 leaf box (triangle: min(v0, min(v1, v2))).
__device__ __forceinline__ Box prim_box(const float* prims, int prim_type, uint32_t p) {
    Box b;
    if (prim_type == NXB_PRIM_TRIANGLE) {
        const float* f = prims + (size_t)p * 9;
        const float3 v0 = make_float3(f[0], f[1], f[2]);
        const float3 v1 = make_float3(f[3], f[4], f[5]);
        const float3 v2 = make_float3(f[6], f[7], f[8]);
        b.mn = fmin3(v0, fmin3(v1, v2));
        b.mx = fmax3(v0, fmax3(v1, v2));
    } else {
        const float* f = prims + (size_t)p * 6;
        b.mn = make_float3(f[0], f[1], f[2]);
        b.mx = make_float3(f[3], f[4], f[5]);
    }
    return b;
}

__device__ __forceinline__ bool same_bits(const Box& a, const Box& b) {
    return __float_as_uint(a.mn.x) == __float_as_uint(b.mn.x) && __float_as_uint(a.mn.y) == __float_as_uint(b.mn.y) &&
           __float_as_uint(a.mn.z) == __float_as_uint(b.mn.z) && __float_as_uint(a.mx.x) == __float_as_uint(b.mx.x) &&
           __float_as_uint(a.mx.y) == __float_as_uint(b.mx.y) && __float_as_uint(a.mx.z) == __float_as_uint(b.mx.z);
}

__device__ __forceinline__ bool contained(const Box& c, const Box& p) {
    return c.mn.x >= p.mn.x && c.mx.x <= p.mx.x && c.mn.y >= p.mn.y && c.mx.y <= p.mx.y && c.mn.z >= p.mn.z &&
           c.mx.z <= p.mx.z;
}

// Sub-box storage of the BVH8 climb: 6 floats per node, read through L2.
__device__ __forceinline__ void store_sub(float* sub, uint32_t i, const Box& b) {
    float* s = sub + (size_t)6 * i;
    s[0] = b.mn.x, s[1] = b.mn.y, s[2] = b.mn.z, s[3] = b.mx.x, s[4] = b.mx.y, s[5] = b.mx.z;
}
__device__ __forceinline__ Box load_sub_cg(const float* sub, uint32_t i) {
    const float* s = sub + (size_t)6 * i;
    Box b;
    b.mn = make_float3(__ldcg(s), __ldcg(s + 1), __ldcg(s + 2));
    b.mx = make_float3(__ldcg(s + 3), __ldcg(s + 4), __ldcg(s + 5));
    return b;
}

// Adds a per-thread count to a report word, one atomic per warp.  Every lane
// of the warp must call it.
__device__ __forceinline__ void report_add(uint64_t* w, uint32_t v) {
    v = __reduce_add_sync(kFullMask, v);
    if (lane_id() == 0 && v) atomicAdd(reinterpret_cast<unsigned long long*>(w), (unsigned long long)v);
}
__device__ __forceinline__ void report_max(uint64_t* w, uint32_t v) {
    v = __reduce_max_sync(kFullMask, v);
    if (lane_id() == 0 && v) atomicMax(reinterpret_cast<unsigned long long*>(w), (unsigned long long)v);
}

// ------------------------------------------------------------ pointer jumping
// One round: link[i] = link[link[i].ancestor] composed with link[i].  The
// root and unlinked nodes are terminal.  Words are read and written in
// place: a word read in the same round is at least as far along as the
// round-start value, so the rounds only converge faster.  A round that
// changes no word leaves a fixed point, so every later round would change
// none either: round r sets moved[r] when it changed a word, and round r+1
// returns at once when moved[r] is clear (the rounds of a tree of depth D
// stop after about log2(D) of them instead of log2(nodes)).
__global__ __launch_bounds__(kThreads) void jump_kernel(uint64_t* link, uint32_t count, uint32_t root,
                                                        const uint32_t* prev_moved, uint32_t* moved) {
    if (prev_moved && *prev_moved == 0) return;
    bool changed = false;
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < count; i += gridDim.x * kThreads) {
        if (i == root) continue;
        const uint64_t x = ld_relaxed_u64(link + i);
        const uint32_t a = link_node(x);
        if (a == root || a >= count) continue;
        const uint64_t y = ld_relaxed_u64(link + a);
        const uint64_t d = min((uint64_t)link_dist(x) + link_dist(y), (uint64_t)0xFFFFFFFEu);
        const uint64_t next = pack_link(link_node(y), (uint32_t)d);
        if (next != x) {
            st_relaxed_u64(link + i, next);
            changed = true;
        }
    }
    if (__syncthreads_or(changed) && threadIdx.x == 0) *moved = 1;
}

// Parent references: [i] = extra references of node i (all of them for the
// root).
__device__ __forceinline__ uint32_t extra_parents(const uint32_t* pcount, uint32_t i, uint32_t root) {
    const uint32_t c = pcount[i];
    return i == root ? c : (c > 1 ? c - 1 : 0);
}

// Duplicate and missing primitives from the per-primitive leaf counts.
__global__ __launch_bounds__(kThreads) void prim_count_kernel(const uint32_t* seen, uint32_t n, uint64_t* dup,
                                                              uint64_t* missing) {
    uint32_t nd = 0, nm = 0;
    for (uint32_t p = blockIdx.x * kThreads + threadIdx.x; p < n; p += gridDim.x * kThreads) {
        const uint32_t s = seen[p];
        nd += s > 1 ? s - 1 : 0;
        nm += s == 0;
    }
    report_add(dup, nd);
    report_add(missing, nm);
}

// ------------------------------------------------------------ BVH2
// report: reached, leaves, dup, missing, bad_union, not_contained,
// bad_index, max_depth, extra_parents, errors.
__global__ __launch_bounds__(kThreads) void bvh2_link_kernel(const Node2* nodes, uint32_t total, uint64_t* link,
                                                             uint32_t* pcount) {
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < total; i += gridDim.x * kThreads) {
        const uint32_t l = nodes[i].left, r = nodes[i].right;
        if (l == kInvalid || l >= total || r >= total) continue;
        atomicAdd(pcount + l, 1u);
        atomicAdd(pcount + r, 1u);
        link[l] = pack_link(i, 1);
        link[r] = pack_link(i, 1);
    }
}

__global__ __launch_bounds__(kThreads) void bvh2_check_kernel(const Node2* nodes, uint32_t n, uint32_t root,
                                                              const uint64_t* link, const uint32_t* pcount,
                                                              uint32_t* seen, uint64_t* report) {
    const uint32_t total = 2 * n - 1;
    uint32_t reached = 0, leaves = 0, bad_union = 0, not_contained = 0, bad_index = 0, depth = 0, extra = 0;
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < total; i += gridDim.x * kThreads) {
        extra += extra_parents(pcount, i, root);
        const uint64_t x = link[i];
        if (i != root && link_node(x) != root) continue;
        ++reached;
        depth = max(depth, i == root ? 0u : link_dist(x));
        const Node2 nd = nodes[i];
        if (nd.left == kInvalid) {
            ++leaves;
            if (nd.right >= n)
                ++bad_index;
            else
                atomicAdd(seen + nd.right, 1u);
            continue;
        }
        if (nd.left >= total || nd.right >= total) {
            ++bad_index;
            continue;
        }
        const Box lb = load_box(nodes, nd.left), rb = load_box(nodes, nd.right);
        Box u = lb;
        grow(u, rb);
        bad_union += !same_bits(u, nd.b);
        not_contained += !contained(lb, nd.b);
        not_contained += !contained(rb, nd.b);
    }
    report_add(report + 0, reached);
    report_add(report + 1, leaves);
    report_add(report + 4, bad_union);
    report_add(report + 5, not_contained);
    report_add(report + 6, bad_index);
    report_max(report + 7, depth);
    report_add(report + 8, extra);
}

__global__ void bvh2_errors_kernel(uint64_t* r, uint32_t n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    r[9] = r[2] + r[3] + r[4] + r[5] + r[6] + r[8] + (r[0] != 2ull * n - 1) + (r[1] != n);
}

// ------------------------------------------------------------ BVH8
// report: reached, leaf slots, dup, missing, bad_index, lo_not_conservative,
// hi_not_conservative, slots_used, max_depth, meta_errors, errors.
struct Bvh8Scratch {
    uint64_t* link;
    uint32_t* par;
    uint32_t* pcount;
    uint32_t* pending;
    float* sub;
    uint32_t* seen;
};

__device__ __forceinline__ bool is_inner(const Node8& nd, uint32_t s) {
    return nd.meta[s] != 0 && ((nd.imask >> s) & 1u);
}

__global__ __launch_bounds__(kThreads) void bvh8_link_kernel(const Node8* nodes, uint32_t m, Bvh8Scratch w) {
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < m; i += gridDim.x * kThreads) {
        const Node8 nd = nodes[i];
        uint32_t inner = 0;
        for (uint32_t s = 0; s < 8; ++s) {
            if (!is_inner(nd, s)) continue;
            const uint32_t c = nd.child_base + below(nd.imask, s);
            if (c >= m) continue;
            atomicAdd(w.pcount + c, 1u);
            w.link[c] = pack_link(i, 1);
            w.par[c] = i;
            ++inner;
        }
        w.pending[i] = inner;
        store_sub(w.sub, i, empty_box());
    }
}

// Exact box of node i: the union of its leaf primitives' boxes and of its
// inner children's subtree boxes (children finished before this call).
__device__ __forceinline__ Box bvh8_node_box(const Node8& nd, uint32_t m, const uint32_t* prim_idx, uint32_t n,
                                             const float* prims, int prim_type, const float* sub) {
    Box acc = empty_box();
    for (uint32_t s = 0; s < 8; ++s) {
        if (!nd.meta[s]) continue;
        if ((nd.imask >> s) & 1u) {
            const uint32_t c = nd.child_base + below(nd.imask, s);
            if (c < m) grow(acc, load_sub_cg(sub, c));
        } else {
            const uint32_t li = nd.prim_base + (nd.meta[s] & 0x1Fu);
            if (li >= n) continue;
            const uint32_t p = prim_idx[li];
            if (p < n) grow(acc, prim_box(prims, prim_type, p));
        }
    }
    return acc;
}

__global__ __launch_bounds__(kThreads) void bvh8_box_kernel(const Node8* nodes, uint32_t m, const uint32_t* prim_idx,
                                                            uint32_t n, const float* prims, int prim_type,
                                                            Bvh8Scratch w) {
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < m; i += gridDim.x * kThreads) {
        Node8 nd = nodes[i];
        bool starter = true;
        for (uint32_t s = 0; s < 8; ++s)
            if (is_inner(nd, s) && nd.child_base + below(nd.imask, s) < m) starter = false;
        if (!starter) continue;
        store_sub(w.sub, i, bvh8_node_box(nd, m, prim_idx, n, prims, prim_type, w.sub));
        // Climb while this thread is the last child to finish; at most one
        // step per node.
        uint32_t c = i;
        for (uint32_t step = 0; step < m && c != 0; ++step) {
            const uint32_t p = w.par[c];
            if (p >= m) break;
            __threadfence();
            if (atomicSub(w.pending + p, 1u) != 1u) break;
            __threadfence();
            nd = nodes[p];
            store_sub(w.sub, p, bvh8_node_box(nd, m, prim_idx, n, prims, prim_type, w.sub));
            c = p;
        }
    }
}

// 2^(e-127) as a double (e is a biased float exponent byte; every value is
// a normal double).
__device__ __forceinline__ double pow2_biased(uint32_t e) {
    return __longlong_as_double((long long)((uint64_t)(e + 896u) << 52));
}

__global__ __launch_bounds__(kThreads) void bvh8_check_kernel(const Node8* nodes, uint32_t m, const uint32_t* prim_idx,
                                                              uint32_t n, const float* prims, int prim_type,
                                                              Bvh8Scratch w, uint64_t* report) {
    uint32_t reached = 0, leaves = 0, bad_index = 0, lo_bad = 0, hi_bad = 0, slots = 0, depth = 0, meta_err = 0;
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < m; i += gridDim.x * kThreads) {
        bad_index += extra_parents(w.pcount, i, 0);
        const uint64_t x = w.link[i];
        if (i != 0 && link_node(x) != 0) continue;
        ++reached;
        depth = max(depth, i == 0 ? 0u : link_dist(x));
        const Node8 nd = nodes[i];
        uint32_t leafmask = 0;
        for (uint32_t s = 0; s < 8; ++s)
            if (nd.meta[s] && !((nd.imask >> s) & 1u)) leafmask |= 1u << s;
        double sc[3];
        for (int a = 0; a < 3; ++a) sc[a] = pow2_biased(nd.e[a]);
        for (uint32_t s = 0; s < 8; ++s) {
            if (!nd.meta[s]) {
                meta_err += (nd.imask >> s) & 1u;
                continue;
            }
            ++slots;
            Box cb;
            if ((nd.imask >> s) & 1u) {
                meta_err += nd.meta[s] != (uint8_t)(0x20u | (24u + s));
                const uint32_t c = nd.child_base + below(nd.imask, s);
                if (c >= m) {
                    ++bad_index;
                    continue;
                }
                cb = load_sub_cg(w.sub, c);
            } else {
                meta_err += nd.meta[s] != (uint8_t)(0x20u | below(leafmask, s));
                ++leaves;
                const uint32_t li = nd.prim_base + (nd.meta[s] & 0x1Fu);
                const uint32_t p = li < n ? prim_idx[li] : kInvalid;
                if (p >= n) {
                    ++bad_index;
                    continue;
                }
                atomicAdd(w.seen + p, 1u);
                cb = prim_box(prims, prim_type, p);
            }
            const float cmn[3] = {cb.mn.x, cb.mn.y, cb.mn.z}, cmx[3] = {cb.mx.x, cb.mx.y, cb.mx.z};
            for (int a = 0; a < 3; ++a) {
                // p + 2^(e-127) * q: the product is exact, the sum rounds once
                const double lo = __dadd_rn((double)nd.p[a], __dmul_rn(sc[a], (double)nd.qlo[a][s]));
                const double hi = __dadd_rn((double)nd.p[a], __dmul_rn(sc[a], (double)nd.qhi[a][s]));
                lo_bad += lo > (double)cmn[a];
                hi_bad += hi < (double)cmx[a];
            }
        }
    }
    report_add(report + 0, reached);
    report_add(report + 1, leaves);
    report_add(report + 4, bad_index);
    report_add(report + 5, lo_bad);
    report_add(report + 6, hi_bad);
    report_add(report + 7, slots);
    report_max(report + 8, depth);
    report_add(report + 9, meta_err);
}

__global__ void bvh8_errors_kernel(uint64_t* r, uint32_t m, uint32_t n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    r[10] = r[2] + r[3] + r[4] + r[9] + (r[0] != m) + (r[1] != n);
}

uint32_t grid_for(size_t count) {
    const size_t want = (count + kThreads - 1) / kThreads;
    return (uint32_t)std::max<size_t>(1, std::min<size_t>(want, (size_t)device_info().sms * 8));
}

uint32_t jump_rounds(uint32_t count) {
    uint32_t r = 0;
    while (r < 32 && (1ull << r) < count) ++r;
    return r;
}

// The rounds of pointer jumping, each skipped once a round before it moved
// no link; moved holds one word per round.
void jump(uint64_t* link, uint32_t count, uint32_t root, uint32_t* moved, uint32_t grid, cudaStream_t s) {
    for (uint32_t r = 0, rounds = jump_rounds(count); r < rounds; ++r)
        jump_kernel<<<grid, kThreads, 0, s>>>(link, count, root, r ? moved + r - 1 : nullptr, moved + r);
}

constexpr size_t kMovedBytes = 4 * 32;

size_t seg(size_t bytes) { return (bytes + 255) / 256 * 256; }

}  // namespace

size_t validate_bvh2_scratch(uint32_t n) {
    const size_t total = 2ull * n - 1;
    return seg(8 * total) + seg(4 * total) + seg(4ull * n) + seg(kMovedBytes);
}

size_t validate_bvh8_scratch(uint32_t m, uint32_t n) {
    return seg(8ull * m) + 3 * seg(4ull * m) + seg(24ull * m) + seg(4ull * n) + seg(kMovedBytes);
}

cudaError_t launch_validate_bvh2(const Node2* nodes, uint32_t n, uint32_t root, uint64_t* report, void* scratch,
                                 cudaStream_t s) {
    const uint32_t total = 2 * n - 1;
    char* p = static_cast<char*>(scratch);
    uint64_t* link = reinterpret_cast<uint64_t*>(p);
    p += seg(8ull * total);
    uint32_t* pcount = reinterpret_cast<uint32_t*>(p);
    p += seg(4ull * total);
    uint32_t* seen = reinterpret_cast<uint32_t*>(p);
    p += seg(4ull * n);
    uint32_t* moved = reinterpret_cast<uint32_t*>(p);
    cudaError_t e = cudaMemsetAsync(report, 0, NXB_BVH2_CHECK_FIELDS * sizeof(uint64_t), s);
    if (!e) e = cudaMemsetAsync(link, 0xFF, 8ull * total, s);
    if (!e) e = cudaMemsetAsync(pcount, 0, 4ull * total, s);
    if (!e) e = cudaMemsetAsync(seen, 0, 4ull * n, s);
    if (!e) e = cudaMemsetAsync(moved, 0, kMovedBytes, s);
    if (e) return e;
    const uint32_t g = grid_for(total);
    bvh2_link_kernel<<<g, kThreads, 0, s>>>(nodes, total, link, pcount);
    jump(link, total, root, moved, g, s);
    bvh2_check_kernel<<<g, kThreads, 0, s>>>(nodes, n, root, link, pcount, seen, report);
    prim_count_kernel<<<grid_for(n), kThreads, 0, s>>>(seen, n, report + 2, report + 3);
    bvh2_errors_kernel<<<1, 32, 0, s>>>(report, n);
    return cudaGetLastError();
}

cudaError_t launch_validate_bvh8(const Node8* nodes, uint32_t m, const uint32_t* prim_idx, uint32_t n,
                                 const void* prims, int prim_type, uint64_t* report, void* scratch, cudaStream_t s) {
    char* p = static_cast<char*>(scratch);
    Bvh8Scratch w;
    w.link = reinterpret_cast<uint64_t*>(p);
    p += seg(8ull * m);
    w.par = reinterpret_cast<uint32_t*>(p);
    p += seg(4ull * m);
    w.pcount = reinterpret_cast<uint32_t*>(p);
    p += seg(4ull * m);
    w.pending = reinterpret_cast<uint32_t*>(p);
    p += seg(4ull * m);
    w.sub = reinterpret_cast<float*>(p);
    p += seg(24ull * m);
    w.seen = reinterpret_cast<uint32_t*>(p);
    p += seg(4ull * n);
    uint32_t* moved = reinterpret_cast<uint32_t*>(p);
    cudaError_t e = cudaMemsetAsync(report, 0, NXB_BVH8_CHECK_FIELDS * sizeof(uint64_t), s);
    if (!e) e = cudaMemsetAsync(w.link, 0xFF, 8ull * m, s);
    if (!e) e = cudaMemsetAsync(w.par, 0xFF, 4ull * m, s);
    if (!e) e = cudaMemsetAsync(w.pcount, 0, 4ull * m, s);
    if (!e) e = cudaMemsetAsync(w.seen, 0, 4ull * n, s);
    if (!e) e = cudaMemsetAsync(moved, 0, kMovedBytes, s);
    if (e) return e;
    const float* f = static_cast<const float*>(prims);
    const uint32_t g = grid_for(m);
    bvh8_link_kernel<<<g, kThreads, 0, s>>>(nodes, m, w);
    bvh8_box_kernel<<<g, kThreads, 0, s>>>(nodes, m, prim_idx, n, f, prim_type, w);
    jump(w.link, m, 0, moved, g, s);
    bvh8_check_kernel<<<g, kThreads, 0, s>>>(nodes, m, prim_idx, n, f, prim_type, w, report);
    prim_count_kernel<<<grid_for(n), kThreads, 0, s>>>(w.seen, n, report + 2, report + 3);
    bvh8_errors_kernel<<<1, 32, 0, s>>>(report, m, n);
    return cudaGetLastError();
}

}  // namespace nxb
