// wide.cu - stage 5: BVH2 -> compressed 8-wide BVH (Ylitie et al. 2017).
//
// Replaces BuildBVH8Kernel (NexusBVH/src/Cuda/WideConverter.cu:225-414).
// The reference launches one thread per work slot (n threads, one work
// item per BVH8 node and one per primitive) and keeps every CTA spinning in
// lock-step on __syncthreads_count until its slots are filled.  Here:
//   * only internal BVH8 nodes are work items; a parent writes its leaf
//     children's primitives into primIdx directly;
//   * a persistent grid (occupancy x SM count) whose lanes each hold one
//     work slot, claimed in increasing order, and poll it with bounded
//     relaxed loads, so no resident lane ever waits on a lane that has not
//     started;
//   * the allocation counters are bumped once per warp iteration with a
//     warp scan instead of once per node;
//   * each thread keeps the children it expands in a slot table in shared
//     memory (BVH2 index, children, box), so popping a child, the slot
//     assignment and the quantisation never reload a node (the reference
//     reloads each child box up to three times);
//   * in a whole-pipeline build the H-PLOC merges also write each internal
//     node's two children side by side (ChildPair, 64 bytes): the collapse
//     then opens a node with one aligned load of its record and reads no
//     BVH2 node at all (a leaf child's box is in its parent's record).
//     Measured on GB300 at 12.58M clustered triangles: BVH8 0.833 ->
//     0.553 ms, H-PLOC 2.16 -> 2.34 ms (the records' stores), build 3.91 ->
//     3.81 ms; the BVH8 kernel's time hardly depends on its occupancy (3 / 6
//     CTAs per SM: 0.898 / 0.833 ms), it follows the random node traffic.
// The decisions are the reference's:
//   * expansion always re-opens the highest-indexed inner child, the child
//     with the smaller area going to the re-opened position (:284-330);
//   * greedy slot assignment in child order, first strictly best slot
//     (GreedyAssignment, :104-153);
//   * node encoding with 8-bit quantised child boxes (CreateBVH8Node,
//     :156-206; CeilLog2/InvPow2, BuilderUtils.h:335-347);
//   * the one-primitive tree special case (CreateBVH8SingleLeaf, :209-222).
#include <algorithm>

#include "pipeline.h"

namespace nxb {
namespace {

constexpr int kThreads = 128;
constexpr float kQuantStep = 1.0f / 255.0f;  // 1/((1<<NQ)-1), NQ = 8
constexpr uint32_t kQueueSpinLimit = 1u << 20;
constexpr uint32_t kFallback = 0xFFFFFFFEu;  // auction_assign: use the greedy assignment
// Opening a BVH2 node needs its children; the opens of one item form a chain
// of dependent loads.  With prefetching on, loading a child that is itself
// internal also asks L2 for that child's two children (or, with child-pair
// records, for the child's record), so that the next open (or the child's
// own work item) finds them there.
constexpr bool kPrefetch = true;
constexpr int kSlotWords = 9;  // BVH2 index, left, right, box (6 floats)
constexpr size_t kSlotSmem = (size_t)kThreads * 8 * kSlotWords * sizeof(uint32_t);

__device__ __forceinline__ uint32_t nib(uint32_t x, uint32_t i) { return (x >> (4 * i)) & 0xFu; }
__device__ __forceinline__ uint32_t popc_below(uint32_t m, uint32_t i) { return __popc(m & ((1u << i) - 1u)); }

__device__ __forceinline__ uint32_t ceil_log2_biased(float x) {
    const uint32_t ix = __float_as_uint(x);
    const uint32_t ex = (ix >> 23) & 0xFFu;
    return ex + ((ix & 0x7FFFFFu) != 0 ? 1u : 0u);
}
__device__ __forceinline__ float inv_pow2(uint8_t e) { return __uint_as_float((uint32_t)(254 - (int)e) << 23); }

// A BVH2 node, through the read-only path (the BVH2 was finished by an
// earlier kernel).
__device__ __forceinline__ Node2 load_node(const Node2* b2, uint32_t i) {
    const uint4* p = reinterpret_cast<const uint4*>(b2 + i);
    const uint4 a = __ldg(p), b = __ldg(p + 1);
    Node2 r;
    r.b.mn = make_float3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
    r.b.mx = make_float3(__uint_as_float(a.w), __uint_as_float(b.x), __uint_as_float(b.y));
    r.left = b.z;
    r.right = b.w;
    return r;
}

// Per-thread table of the (up to 8) children being collected, in shared
// memory, word-interleaved across the CTA's threads (bank-conflict free).
struct SlotTable {
    uint32_t* base;
    __device__ uint32_t* at(uint32_t slot, uint32_t field) const {
        return base + (slot * kSlotWords + field) * kThreads + threadIdx.x;
    }
    __device__ void put(uint32_t slot, uint32_t idx, const Node2& nd) const {
        *at(slot, 0) = idx;
        *at(slot, 1) = nd.left;
        *at(slot, 2) = nd.right;
        *at(slot, 3) = __float_as_uint(nd.b.mn.x);
        *at(slot, 4) = __float_as_uint(nd.b.mn.y);
        *at(slot, 5) = __float_as_uint(nd.b.mn.z);
        *at(slot, 6) = __float_as_uint(nd.b.mx.x);
        *at(slot, 7) = __float_as_uint(nd.b.mx.y);
        *at(slot, 8) = __float_as_uint(nd.b.mx.z);
    }
    // child-pair builds: the index and the box (the children come from the
    // node's own record when it is opened)
    __device__ void put(uint32_t slot, uint32_t idx, const Box& b) const {
        *at(slot, 0) = idx;
        *at(slot, 3) = __float_as_uint(b.mn.x);
        *at(slot, 4) = __float_as_uint(b.mn.y);
        *at(slot, 5) = __float_as_uint(b.mn.z);
        *at(slot, 6) = __float_as_uint(b.mx.x);
        *at(slot, 7) = __float_as_uint(b.mx.y);
        *at(slot, 8) = __float_as_uint(b.mx.z);
    }
    __device__ uint32_t idx(uint32_t slot) const { return *at(slot, 0); }
    __device__ uint32_t left(uint32_t slot) const { return *at(slot, 1); }
    __device__ uint32_t right(uint32_t slot) const { return *at(slot, 2); }
    __device__ Box box(uint32_t slot) const {
        Box b;
        b.mn = make_float3(__uint_as_float(*at(slot, 3)), __uint_as_float(*at(slot, 4)), __uint_as_float(*at(slot, 5)));
        b.mx = make_float3(__uint_as_float(*at(slot, 6)), __uint_as_float(*at(slot, 7)), __uint_as_float(*at(slot, 8)));
        return b;
    }
};

// GetCost (WideConverter.cu:25-30): sign pattern of slot s applied to the
// parent-to-child centroid offset.
__device__ __forceinline__ float slot_cost(uint32_t s, float3 o) {
    return ((s >> 2) & 1 ? -1.0f : 1.0f) * o.x + ((s >> 1) & 1 ? -1.0f : 1.0f) * o.y + (s & 1 ? -1.0f : 1.0f) * o.z;
}

template <typename Boxes>
__device__ __forceinline__ uint32_t greedy_assign(float3 pc, const Boxes& boxes, uint32_t count) {
    uint32_t asg = kInvalid;
    for (uint32_t c = 0; c < count; ++c) {
        const Box cb = boxes.box(c);
        const float3 off = make_float3(pc.x - (cb.mx.x + cb.mn.x), pc.y - (cb.mx.y + cb.mn.y),
                                       pc.z - (cb.mx.z + cb.mn.z));
        float best = -3.402823466e+38f;
        uint32_t slot = 0xFu;
#pragma unroll
        for (uint32_t s = 0; s < 8; ++s) {
            if (nib(asg, s) != 0xFu) continue;
            const float cost = slot_cost(s, off);
            if (cost > best) {
                best = cost;
                slot = s;
            }
        }
        if (slot < 8) {
            asg &= ~(0xFu << (4 * slot));
            asg |= c << (4 * slot);
        }
    }
    return asg;
}

// AuctionAssignment (WideConverter.cu:50-102) over the cost table of the
// reference's USE_AUCTION branch (:337-358): child offsets from the parent
// centroid scaled so that the parent's largest extent maps to
// MAX_COST / 2 = 5, prices start at 0, epsilon runs from max(maxCost, 1/n)
// down to 1/n in steps of 1/THETA = 1/8, bidders are taken last-in first-out
// from a nibble stack.  The reference's loop has no bound and indexes
// prices[] with an invalid slot when no reward is finite; here bids are
// capped and both cases fall back to the greedy assignment.
constexpr uint32_t kAuctionBidLimit = 4096;

template <typename Boxes>
__device__ uint32_t auction_assign(const Box& pb, const Boxes& boxes, uint32_t count) {
    const float max_dim = fmaxf(pb.mx.x - pb.mn.x, fmaxf(pb.mx.y - pb.mn.y, pb.mx.z - pb.mn.z));
    float cost_scale = max_dim == 0.0f ? 0.0f : 10.0f / max_dim;
    cost_scale *= 0.5f;
    const float3 pc = make_float3(pb.mn.x + pb.mx.x, pb.mn.y + pb.mx.y, pb.mn.z + pb.mx.z);
    float3 off[8];
    float max_cost = -3.402823466e+38f;
    for (uint32_t c = 0; c < count; ++c) {
        const Box cb = boxes.box(c);
        off[c] = make_float3((pc.x - (cb.mn.x + cb.mx.x)) * cost_scale, (pc.y - (cb.mn.y + cb.mx.y)) * cost_scale,
                             (pc.z - (cb.mn.z + cb.mx.z)) * cost_scale);
        const float cost = fabsf(off[c].x) + fabsf(off[c].y) + fabsf(off[c].z);
        if (cost > max_cost) max_cost = cost;
    }
    float prices[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) prices[i] = 0.0f;
    const float threshold = 1.0f / (float)count;
    float epsilon = fmaxf(max_cost, threshold);
    uint32_t asg = kInvalid, bids = 0;
    while (epsilon >= threshold) {
        asg = kInvalid;
        uint32_t bidders = 0x76543210u, waiting = count;
        while (waiting > 0) {
            const uint32_t c = nib(bidders, --waiting);
            float win = -3.402823466e+38f, second = -3.402823466e+38f;
            uint32_t slot = 0xFu;
#pragma unroll
            for (uint32_t s = 0; s < 8; ++s) {
                const float reward = slot_cost(s, off[c]) - prices[s];
                if (reward > win) {
                    second = win;
                    win = reward;
                    slot = s;
                } else if (reward > second) {
                    second = reward;
                }
            }
            if (slot > 7 || ++bids > kAuctionBidLimit) return kFallback;
            float bump = (win - second) + epsilon;
#pragma unroll
            for (uint32_t s = 0; s < 8; ++s)
                if (s == slot) prices[s] += bump;
            const uint32_t prev = nib(asg, slot);
            asg = (asg & ~(0xFu << (4 * slot))) | (c << (4 * slot));
            if (prev != 0xFu) {
                bidders = (bidders & ~(0xFu << (4 * waiting))) | (prev << (4 * waiting));
                ++waiting;
            }
        }
        epsilon *= 0.125f;
    }
    return asg;
}

template <typename Boxes>
__device__ __forceinline__ void write_node8(Node8* dst, const Box& bounds, const Boxes& boxes, uint32_t child_base,
                                            uint32_t prim_base, uint32_t asg, uint32_t inner, uint32_t leaf) {
    uint32_t w[20];
#pragma unroll
    for (int i = 0; i < 20; ++i) w[i] = 0;
    const float3 diag = make_float3(bounds.mx.x - bounds.mn.x, bounds.mx.y - bounds.mn.y, bounds.mx.z - bounds.mn.z);
    const uint8_t ex = (uint8_t)ceil_log2_biased(diag.x * kQuantStep);
    const uint8_t ey = (uint8_t)ceil_log2_biased(diag.y * kQuantStep);
    const uint8_t ez = (uint8_t)ceil_log2_biased(diag.z * kQuantStep);
    const float3 inv = make_float3(inv_pow2(ex), inv_pow2(ey), inv_pow2(ez));
    w[0] = __float_as_uint(bounds.mn.x);
    w[1] = __float_as_uint(bounds.mn.y);
    w[2] = __float_as_uint(bounds.mn.z);
    uint32_t imask = 0;
    w[4] = child_base;
    w[5] = prim_base;
#pragma unroll
    for (uint32_t i = 0; i < 8; ++i) {
        const uint32_t a = nib(asg, i);
        uint32_t meta;
        if (inner & (1u << i)) {
            imask |= 1u << i;
            meta = 0x20u | (24u + i);
        } else if (a != 0xFu) {
            meta = 0x20u | popc_below(leaf, i);
        } else {
            continue;
        }
        const uint32_t sh = 8u * (i & 3u);
        w[6 + (i >> 2)] |= meta << sh;
        const Box cb = boxes.box(a);
        const uint32_t qlx = (uint8_t)floorf((cb.mn.x - bounds.mn.x) * inv.x);
        const uint32_t qly = (uint8_t)floorf((cb.mn.y - bounds.mn.y) * inv.y);
        const uint32_t qlz = (uint8_t)floorf((cb.mn.z - bounds.mn.z) * inv.z);
        const uint32_t qhx = (uint8_t)ceilf((cb.mx.x - bounds.mn.x) * inv.x);
        const uint32_t qhy = (uint8_t)ceilf((cb.mx.y - bounds.mn.y) * inv.y);
        const uint32_t qhz = (uint8_t)ceilf((cb.mx.z - bounds.mn.z) * inv.z);
        w[8 + (i >> 2)] |= qlx << sh;
        w[10 + (i >> 2)] |= qly << sh;
        w[12 + (i >> 2)] |= qlz << sh;
        w[14 + (i >> 2)] |= qhx << sh;
        w[16 + (i >> 2)] |= qhy << sh;
        w[18 + (i >> 2)] |= qhz << sh;
    }
    w[3] = (uint32_t)ex | ((uint32_t)ey << 8) | ((uint32_t)ez << 16) | (imask << 24);
    uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
    for (int k = 0; k < 5; ++k) d[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
}

struct LeafZero {
    const Node2* b2;
    __device__ Box box(uint32_t) const { return load_box(b2, 0); }
};

__global__ void bvh8_init_kernel(uint64_t* pairs, uint32_t n, uint32_t* ctr) {
    const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t i = i0; i < n; i += gridDim.x * blockDim.x) pairs[i] = bvh8_queue_slot(i, n);
    if (i0 == 0) bvh8_queue_counters(ctr);
}

// Batched form: slot m holds the root item of mesh m (empty meshes too,
// they finish without output); per-mesh node and leaf counters.
__global__ void bvh8_batch_init_kernel(uint64_t* pairs, uint32_t slots, MeshBatch batch, uint32_t* ctr,
                                       uint32_t* mesh_nodes, uint32_t* mesh_leaves, MeshGroups groups) {
    const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t i = i0; i < slots; i += gridDim.x * blockDim.x) {
        // group g's queue is slots [slot[g], slot[g+1]); its first entries
        // are the root items of the group's meshes
        uint32_t g = 0;
        while (g + 1 < groups.count && i >= groups.slot[g + 1]) ++g;
        const uint32_t local = i - groups.slot[g];
        uint64_t v = ~0ull;
        if (local < groups.mesh[g + 1] - groups.mesh[g]) {
            const uint32_t m = groups.mesh[g] + local;
            const MeshSpan me = batch.span(m);
            const uint32_t root = me.count ? 2 * me.count - 2 : 0u;
            v = ((uint64_t)root << 32) | __ldg(batch.off8 + m);
        }
        if (i < batch.meshes) {
            const MeshSpan me = batch.span(i);
            mesh_nodes[i] = me.count ? 1u : 0u;
            mesh_leaves[i] = 0;
        }
        pairs[i] = v;
    }
    if (i0 < groups.count) {
        uint32_t* c = ctr + i0 * kBvh8CtrWords;
        const uint32_t meshes = groups.mesh[i0 + 1] - groups.mesh[i0];
        c[kBvh8Claim] = 0;
        c[kBvh8Alloc] = meshes;  // a batch counts nodes and leaves per mesh
        c[kBvh8Leaves] = 0;
        c[kBvh8Pending] = meshes;
    }
}

// Work items are the internal BVH8 nodes only: a parent writes the
// primitive of each leaf child straight into primIdx (it holds the leaf's
// node in its slot table), instead of queueing a work item per leaf as the
// reference does (one per primitive, each re-reading the leaf node).  Every
// inner child gets a fresh slot (breadth-first), so a slot is always written
// by an item in a lower slot.  Each lane holds one slot at a time and claims
// the next one (warp-aggregated: one atomic on the claim counter) once its
// item is done, whether or not a parent has allocated it yet, and polls it
// until its item arrives; a slot is only ever waited on by its own lane, so
// lanes that wait hold no other lane up.  The kernel ends when the count of
// allocated-but-unfinished items drops to zero (the slots still held then
// are never allocated).  Claiming without first reading the allocation
// counter keeps two loads per warp pass off the counters' cache lines,
// which every warp of the grid hits (measured on GB300: BVH8 0.858 ->
// 0.836 ms at 12.58M clustered triangles, 0.340 -> 0.320 ms at 4.19M).
// An item is (mesh-local BVH2 index << 32 | BVH8 index in `out`).  In the
// batched form (Seg = MeshBatch) the items of all meshes share the queue,
// the BVH8 index names the mesh, and nodes and leaves are counted per mesh
// in mesh_nodes / mesh_leaves.
template <typename Seg, bool AUCTION, bool KIDS>
__global__ __launch_bounds__(kThreads) void bvh8_kernel(const Node2* __restrict__ b2, Seg seg, Node8* out,
                                                        uint32_t cap, uint32_t slots, uint32_t* prim_idx,
                                                        uint64_t* pairs, uint32_t* ctr, uint32_t* mesh_nodes,
                                                        uint32_t* mesh_leaves, uint32_t* err,
                                                        const ChildPair* __restrict__ kids) {
    extern __shared__ uint32_t s_slots[];
    const SlotTable tab{s_slots};
    const uint32_t lane = lane_id();
    if constexpr (!Seg::kBatch) {
        if (seg.n == 1) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                write_node8(out, load_box(b2, 0), LeafZero{b2}, 0, 0, 0xFFFFFFF0u, 0u, 1u);
                prim_idx[0] = 0;
                ctr[kBvh8Leaves] = 1;
                ctr[kBvh8Pending] = 0;
            }
            return;
        }
    }
    uint32_t slot = kInvalid;
    bool retired = false;
    uint32_t idle = 0;
    for (;;) {
        // lanes without a slot claim the next ones, in increasing order; a
        // slot past the queue's end is never allocated and retires the lane
        const bool want = !retired && slot == kInvalid;
        const uint32_t wmask = __ballot_sync(kFullMask, want);
        if (wmask) {
            const uint32_t leader = __ffs(wmask) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(ctr + kBvh8Claim, (uint32_t)__popc(wmask));
            base = __shfl_sync(kFullMask, base, leader);
            if (want) {
                const uint32_t claimed = base + __popc(wmask & lanemask_lt());
                if (claimed < slots && claimed >= base)
                    slot = claimed;
                else
                    retired = true;
            }
        }
        if (__all_sync(kFullMask, retired)) return;
        uint64_t pr = 0;
        bool ready = false;
        if (slot != kInvalid) {
            pr = ld_relaxed_u64(pairs + slot);
            ready = (uint32_t)(pr >> 32) != kInvalid;
        }
        if (!__any_sync(kFullMask, ready)) {
            // nothing ready: finished when no allocated item is outstanding
            if (ld_relaxed_u32(ctr + kBvh8Pending) == 0) return;
            if (++idle > kQueueSpinLimit) {
                if (lane == 0) set_error(err, NXB_DEVERR_BVH8_QUEUE_TIMEOUT);
                return;
            }
            __nanosleep(min(32u << min(idle, 5u), 1024u));  // back off: idle warps poll the counters
            continue;
        }
        idle = 0;
        const uint32_t b2i = (uint32_t)(pr >> 32), b8i = (uint32_t)pr;
        // the item's mesh: its BVH2 nodes, BVH8 range and primitive range
        MeshSpan me{0, 0, 0};
        const Node2* mb2 = b2;
        uint32_t base8 = 0, cap8 = cap;
        bool internal = false;
        Node2 nd;
        ChildPair kp;  // KIDS: the item node's children
        if (ready) {
            if constexpr (Seg::kBatch) {
                me = seg.span(owner_of(seg.off8, 0, seg.meshes - 1, b8i));
                mb2 = b2 + 2ull * me.start;
                base8 = __ldg(seg.off8 + me.m);
                cap8 = __ldg(seg.off8 + me.m + 1) - base8;
            } else {
                me.count = seg.n;
            }
            const uint32_t node_limit = 2 * me.count - 1;
            if (Seg::kBatch && me.count <= 1) {
                // an empty mesh has no tree; a one-primitive mesh gets the
                // single-leaf node (CreateBVH8SingleLeaf, WideConverter.cu:209-222)
                if (me.count == 1) {
                    write_node8(out + b8i, load_box(mb2, 0), LeafZero{mb2}, 0, 0, 0xFFFFFFF0u, 0u, 1u);
                    prim_idx[me.start] = 0;
                    mesh_leaves[me.m] = 1;
                }
            } else if (b2i >= node_limit || b8i - base8 >= cap8) {
                set_error(err, NXB_DEVERR_BVH8_OVERFLOW);
            } else if constexpr (KIDS) {
                // an item is an internal node; its box is the union of its children's
                if (b2i < me.count) {
                    set_error(err, NXB_DEVERR_BVH8_OVERFLOW);
                } else {
                    kp = load_child_pair(kids + me.start + (b2i - me.count));
                    if (kp.li >= node_limit || kp.ri >= node_limit) {
                        set_error(err, NXB_DEVERR_BVH8_OVERFLOW);
                    } else {
                        nd.b = kp.l;
                        grow(nd.b, kp.r);
                        internal = true;
                    }
                }
            } else {
                nd = load_node(mb2, b2i);
                if (nd.left >= node_limit || nd.right >= node_limit)
                    set_error(err, NXB_DEVERR_BVH8_OVERFLOW);
                else
                    internal = true;
            }
            if (!internal) slot = kInvalid;  // done (or reported); the item counts as finished
        }
        const uint32_t node_limit = 2 * me.count - 1;
        uint32_t inner = 0, count = 0, asg = kInvalid, leaf = 0;
        if (internal) {
            // open BVH2 nodes top-down until 8 children or no inner child
            uint32_t l0, l1;
            if constexpr (KIDS) {
                l0 = kp.li;
                l1 = kp.ri;
            } else {
                l0 = nd.left;
                l1 = nd.right;
            }
            uint32_t msb = 0;
            while (true) {
                bool in0, in1, first;
                if constexpr (KIDS) {
                    // the children of the opened node and their boxes are in
                    // its record; an internal child's own record is the next
                    // load of its chain
                    in0 = l0 >= me.count;
                    in1 = l1 >= me.count;
                    if (kPrefetch) {
                        if (in0) prefetch_l2(kids + me.start + (l0 - me.count));
                        if (in1) prefetch_l2(kids + me.start + (l1 - me.count));
                    }
                    first = !(half_area(kp.l) < half_area(kp.r));
                    tab.put(msb, first ? l1 : l0, first ? kp.r : kp.l);
                    tab.put(count + 1, first ? l0 : l1, first ? kp.l : kp.r);
                } else {
                    const Node2 c0 = load_node(mb2, l0), c1 = load_node(mb2, l1);
                    if (kPrefetch) {
                        if (c0.left < node_limit && c0.right < node_limit) {
                            prefetch_l2(mb2 + c0.left);
                            prefetch_l2(mb2 + c0.right);
                        }
                        if (c1.left < node_limit && c1.right < node_limit) {
                            prefetch_l2(mb2 + c1.left);
                            prefetch_l2(mb2 + c1.right);
                        }
                    }
                    first = !(half_area(c0.b) < half_area(c1.b));
                    // the smaller-area child takes the re-opened position
                    tab.put(msb, first ? l1 : l0, first ? c1 : c0);
                    tab.put(count + 1, first ? l0 : l1, first ? c0 : c1);
                    in0 = c0.left != kInvalid;
                    in1 = c1.left != kInvalid;
                }
                if (first ? in1 : in0) inner |= 1u << msb;
                if (first ? in0 : in1) inner |= 1u << (count + 1);
                count += 2;
                if (inner == 0 || count == 8) break;
                msb = 31 - __clz(inner);
                inner &= ~(1u << msb);
                count--;
                if constexpr (KIDS) {
                    kp = load_child_pair(kids + me.start + (tab.idx(msb) - me.count));
                    l0 = kp.li;
                    l1 = kp.ri;
                } else {
                    l0 = tab.left(msb);
                    l1 = tab.right(msb);
                }
                if (l0 >= node_limit || l1 >= node_limit) {  // corrupt BVH2: report, stop expanding
                    set_error(err, NXB_DEVERR_BVH8_OVERFLOW);
                    inner |= 1u << msb;
                    count++;
                    break;
                }
            }
            const float3 pc = make_float3(nd.b.mn.x + nd.b.mx.x, nd.b.mn.y + nd.b.mx.y, nd.b.mn.z + nd.b.mx.z);
            if constexpr (AUCTION) {
                asg = auction_assign(nd.b, tab, count);
                if (asg == kFallback) asg = greedy_assign(pc, tab, count);
            } else {
                asg = greedy_assign(pc, tab, count);
            }
            uint32_t ninner = 0;
#pragma unroll
            for (uint32_t i = 0; i < 8; ++i) {
                const uint32_t a = nib(asg, i);
                if (a == 0xFu) continue;
                const uint32_t bit = (inner >> a) & 1u;
                ninner |= bit << i;
                leaf |= (bit ^ 1u) << i;
            }
            inner = ninner;
        }
        // warp-aggregated allocation of work slots (and, for one mesh, of
        // BVH8 nodes and leaves; a batch counts those per mesh)
        const uint32_t ic = internal ? (uint32_t)__popc(inner) : 0u;
        const uint32_t lc = internal ? count - ic : 0u;
        const uint32_t wc = ic;  // every inner child becomes a work item of its own
        const uint32_t packed = Seg::kBatch ? (wc << 20) : (ic | (lc << 10) | (wc << 20));
        uint32_t incl = packed;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t done = __popc(__ballot_sync(kFullMask, ready));
        // one 64-bit atomic: work slots (one mesh: = BVH8 nodes) low, leaves high
        uint64_t bases = 0;
        if (lane == 31) {
            const uint64_t tl = (incl >> 10) & 0x3FFu, tw = incl >> 20;
            if (tl | tw)
                bases = atomicAdd(reinterpret_cast<unsigned long long*>(ctr + kBvh8Alloc),
                                  (unsigned long long)((tl << 32) | tw));
        }
        bases = __shfl_sync(kFullMask, bases, 31);
        const uint32_t wb = (uint32_t)bases, nb = wb, lb = (uint32_t)(bases >> 32);
        if (internal) {
            const uint32_t excl = incl - packed;
            uint32_t child_base, prim_base;
            if constexpr (Seg::kBatch) {
                child_base = ic ? atomicAdd(mesh_nodes + me.m, ic) : 0u;
                prim_base = lc ? atomicAdd(mesh_leaves + me.m, lc) : 0u;
            } else {
                child_base = nb + (excl & 0x3FFu);
                prim_base = lc ? lb + ((excl >> 10) & 0x3FFu) : 0u;
            }
            const uint32_t work_base = wb + (excl >> 20);
            if (child_base + ic > cap8 || work_base + wc > slots || prim_base + lc > me.count) {
                set_error(err, NXB_DEVERR_BVH8_OVERFLOW);
            } else {
#pragma unroll
                for (uint32_t i = 0; i < 8; ++i) {
                    const uint32_t a = nib(asg, i);
                    if ((inner >> i) & 1u) {
                        const uint32_t k = popc_below(inner, i);
                        const uint64_t pair = ((uint64_t)tab.idx(a) << 32) | (base8 + child_base + k);
                        st_relaxed_u64(pairs + work_base + k, pair);
                    } else if ((leaf >> i) & 1u) {
                        // leaf i of the BVH2 is primitive i (its node's right field)
                        prim_idx[me.start + prim_base + popc_below(leaf, i)] = KIDS ? tab.idx(a) : tab.right(a);
                    }
                }
                write_node8(out + b8i, nd.b, tab, child_base, prim_base, asg, inner, leaf);
            }
            slot = kInvalid;
        }
        // pending += items allocated - items finished (one atomic, so it can
        // only reach zero when no item is in flight)
        __syncwarp();
        const uint32_t new_items = __shfl_sync(kFullMask, incl >> 20, 31);
        if (lane == 0 && new_items != done) atomicAdd(ctr + kBvh8Pending, new_items - done);
    }
}

template <typename Seg, bool AUCTION, bool KIDS>
cudaError_t configure_smem() {
    return once_per_device([] {
        return cudaFuncSetAttribute(bvh8_kernel<Seg, AUCTION, KIDS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSlotSmem);
    });
}

template <typename Seg, bool AUCTION, bool KIDS>
uint32_t persistent_grid(uint32_t items) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bvh8_kernel<Seg, AUCTION, KIDS>, kThreads, kSlotSmem);
    if (per_sm < 1) per_sm = 1;
    const uint32_t want = (items + kThreads - 1) / kThreads;
    return std::max(1u, std::min(want, (uint32_t)(device_info().sms * per_sm)));
}

template <typename Seg, bool AUCTION, bool KIDS = false>
cudaError_t launch_wide(const Node2* bvh2, Seg seg, uint32_t items, Node8* out, uint32_t cap, uint32_t slots,
                        uint32_t* prim_idx, uint64_t* pairs, uint32_t* ctr, uint32_t* mesh_nodes,
                        uint32_t* mesh_leaves, uint32_t* err, cudaStream_t s, const ChildPair* kids = nullptr) {
    cudaError_t e = configure_smem<Seg, AUCTION, KIDS>();
    if (e) return e;
    bvh8_kernel<Seg, AUCTION, KIDS><<<persistent_grid<Seg, AUCTION, KIDS>(items), kThreads, kSlotSmem, s>>>(
        bvh2, seg, out, cap, slots, prim_idx, pairs, ctr, mesh_nodes, mesh_leaves, err, kids);
    return cudaGetLastError();
}

}  // namespace

// Bounded-wait check: a two-primitive BVH2 whose work queue is never seeded,
// so every slot poll expires.  Returns the error word.
cudaError_t run_bvh8_stall_probe(uint32_t* err_out) {
    const uint32_t n = 2;
    unsigned char* buf = nullptr;
    const size_t bytes = 4 * (kBvh8CtrWords + 32) + 3 * sizeof(Node2) + 2 * sizeof(Node8) + 8 * n + 4 * n;
    cudaError_t e = configure_smem<SingleMesh, false, false>();
    if (!e) e = cudaMalloc(&buf, bytes);
    if (e) return e;
    uint32_t* ctr = (uint32_t*)buf;  // 256-byte aligned
    uint32_t* err = ctr + kBvh8CtrWords;
    Node2* b2 = (Node2*)(buf + 4 * (kBvh8CtrWords + 32));
    Node8* out = (Node8*)(b2 + 3);
    uint64_t* pairs = (uint64_t*)(out + 2);
    uint32_t* prim = (uint32_t*)(pairs + n);
    e = cudaMemset(buf, 0, bytes);
    if (!e) e = cudaMemset(pairs, 0xFF, 8 * n);
    uint32_t c[kBvh8CtrWords] = {};
    c[kBvh8Alloc] = 1;    // slot 0 is allocated ...
    c[kBvh8Pending] = 1;  // ... but its pair is never written
    if (!e) e = cudaMemcpy(ctr, c, sizeof(c), cudaMemcpyHostToDevice);
    if (!e) {
        bvh8_kernel<SingleMesh, false, false><<<1, kThreads, kSlotSmem>>>(b2, SingleMesh{n}, out, 2, n, prim, pairs,
                                                                          ctr, nullptr, nullptr, err, nullptr);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(err_out, err, 4, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    return e;
}

cudaError_t launch_bvh8_init(uint64_t* pairs, uint32_t n, uint32_t* ctr, cudaStream_t s) {
    uint32_t grid = std::min<uint32_t>((n + 255) / 256, (uint32_t)device_info().sms * 8);
    bvh8_init_kernel<<<grid, 256, 0, s>>>(pairs, n, ctr);
    return cudaGetLastError();
}

cudaError_t launch_bvh8(const Node2* bvh2, uint32_t n, Node8* out, uint32_t cap, uint32_t* prim_idx, uint64_t* pairs,
                        uint32_t* ctr, uint32_t* err, bool auction, cudaStream_t s, const ChildPair* child_pairs) {
    const SingleMesh seg{n};
    if (child_pairs) {
        if (auction)
            return launch_wide<SingleMesh, true, true>(bvh2, seg, n, out, cap, n, prim_idx, pairs, ctr, nullptr,
                                                       nullptr, err, s, child_pairs);
        return launch_wide<SingleMesh, false, true>(bvh2, seg, n, out, cap, n, prim_idx, pairs, ctr, nullptr,
                                                    nullptr, err, s, child_pairs);
    }
    if (auction)
        return launch_wide<SingleMesh, true>(bvh2, seg, n, out, cap, n, prim_idx, pairs, ctr, nullptr, nullptr, err,
                                             s);
    return launch_wide<SingleMesh, false>(bvh2, seg, n, out, cap, n, prim_idx, pairs, ctr, nullptr, nullptr, err, s);
}

cudaError_t launch_bvh8_batch_init(uint64_t* pairs, uint32_t slots, const MeshBatch& batch, uint32_t* ctr,
                                   uint32_t* mesh_nodes, uint32_t* mesh_leaves, const MeshGroups& groups,
                                   cudaStream_t s) {
    uint32_t grid = std::max(1u, std::min<uint32_t>((slots + 255) / 256, (uint32_t)device_info().sms * 8));
    bvh8_batch_init_kernel<<<grid, 256, 0, s>>>(pairs, slots, batch, ctr, mesh_nodes, mesh_leaves, groups);
    return cudaGetLastError();
}

cudaError_t launch_bvh8_batch(const Node2* bvh2, const MeshBatch& batch, uint32_t total, Node8* out, uint32_t slots,
                              uint32_t* prim_idx, uint64_t* pairs, uint32_t* ctr, uint32_t* mesh_nodes,
                              uint32_t* mesh_leaves, uint32_t* err, bool auction, cudaStream_t s,
                              const ChildPair* child_pairs) {
    if (child_pairs) {
        if (auction)
            return launch_wide<MeshBatch, true, true>(bvh2, batch, total, out, 0u, slots, prim_idx, pairs, ctr,
                                                      mesh_nodes, mesh_leaves, err, s, child_pairs);
        return launch_wide<MeshBatch, false, true>(bvh2, batch, total, out, 0u, slots, prim_idx, pairs, ctr,
                                                   mesh_nodes, mesh_leaves, err, s, child_pairs);
    }
    if (auction)
        return launch_wide<MeshBatch, true>(bvh2, batch, total, out, 0u, slots, prim_idx, pairs, ctr, mesh_nodes,
                                            mesh_leaves, err, s);
    return launch_wide<MeshBatch, false>(bvh2, batch, total, out, 0u, slots, prim_idx, pairs, ctr, mesh_nodes,
                                         mesh_leaves, err, s);
}

}  // namespace nxb
