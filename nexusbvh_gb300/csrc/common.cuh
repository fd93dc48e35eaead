// common.cuh - shared device-side definitions of the GB300 BVH builder.
//
// Numerics: the whole library is compiled with --use_fast_math, the flag
// the reference builds with (NexusBVH/CMakeLists.txt:46-59), so float
// add/sub/mul/min/max flush subnormals and `/` is the fast-math divide.
// Expressions whose rounding decides topology are written with explicit
// intrinsics so that they do not depend on the compiler's contraction
// choices; the self-test (nxb_selftest_numerics) checks them against the
// plain source expressions the reference uses.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nxb_gb300.h"

namespace nxb {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr uint32_t kFullMask = 0xFFFFFFFFu;

// Upper bound on polls of a cross-CTA flag before a kernel gives up, sets
// its error word and returns (polls back off with __nanosleep, so this is
// well under a second of waiting on GB300).
constexpr uint32_t kSpinLimit = 1u << 20;

struct Box {
    float3 mn;
    float3 mx;
};

struct __align__(16) Node2 {
    Box b;
    uint32_t left;
    uint32_t right;
};
static_assert(sizeof(Node2) == 32, "BVH2 node layout");

struct __align__(16) Node8 {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t prim_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(Node8) == 80, "BVH8 node layout");

// ------------------------------------------------------------ float helpers
__device__ __forceinline__ float3 fmin3(float3 a, float3 b) {
    return make_float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z));
}
__device__ __forceinline__ float3 fmax3(float3 a, float3 b) {
    return make_float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z));
}
__device__ __forceinline__ void grow(Box& self, const Box& other) {
    self.mn = fmin3(self.mn, other.mn);
    self.mx = fmax3(self.mx, other.mx);
}

// Surface area / 2 of a box: dx*dy + dy*dz + dz*dx with the reference's
// rounding, fma(dz, dx, fma(dx, dy, dy*dz)) (pinned by the self-test).
__device__ __forceinline__ float half_area(const Box& b) {
    float dx = b.mx.x - b.mn.x;
    float dy = b.mx.y - b.mn.y;
    float dz = b.mx.z - b.mn.z;
    return __fmaf_rn(dz, dx, __fmaf_rn(dx, dy, dy * dz));
}

// half_area of two boxes at once, with Blackwell's paired f32x2 arithmetic:
// the same operations in the same order, each rounded to nearest with
// subnormals flushed (the library is built with --use_fast_math), so both
// results have half_area's bits (checked by the numerics self-test).
__device__ __forceinline__ void half_area2(const Box& a, const Box& b, float& ra, float& rb) {
    auto pack = [](float lo, float hi) {
        uint64_t r;
        asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
        return r;
    };
    uint64_t dx, dy, dz, t;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(dx) : "l"(pack(a.mx.x, b.mx.x)), "l"(pack(a.mn.x, b.mn.x)));
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(dy) : "l"(pack(a.mx.y, b.mx.y)), "l"(pack(a.mn.y, b.mn.y)));
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(dz) : "l"(pack(a.mx.z, b.mx.z)), "l"(pack(a.mn.z, b.mn.z)));
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(t) : "l"(dy), "l"(dz));
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(t) : "l"(dx), "l"(dy), "l"(t));
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(t) : "l"(dz), "l"(dx), "l"(t));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(ra), "=f"(rb) : "l"(t));
}

// Float <-> monotone uint32 (for atomicMin/Max on floats without CAS
// loops); -0 orders below +0.
__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// ------------------------------------------------------------ Morton
// Spread the low 10 / 21 bits of x three bits apart (magic-number form).
__device__ __forceinline__ uint32_t spread3_10(uint32_t x) {
    x &= 0x3FFu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}
__device__ __forceinline__ uint64_t spread3_21(uint64_t x) {
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x001F00000000FFFFull;
    x = (x | (x << 16)) & 0x001F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// ------------------------------------------------------------ memory ops
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ uint32_t atom_exch_acq_rel(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Box of a BVH2 node read through L2 (data written by other CTAs).
__device__ __forceinline__ Box load_box_cg(const Node2* nodes, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    float4 a = __ldcg(p);
    float2 b = __ldcg(reinterpret_cast<const float2*>(p + 1));
    Box r;
    r.mn = make_float3(a.x, a.y, a.z);
    r.mx = make_float3(a.w, b.x, b.y);
    return r;
}
__device__ __forceinline__ Box load_box(const Node2* nodes, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    float4 a = __ldg(p);
    float2 b = __ldg(reinterpret_cast<const float2*>(p + 1));
    Box r;
    r.mn = make_float3(a.x, a.y, a.z);
    r.mx = make_float3(a.w, b.x, b.y);
    return r;
}
__device__ __forceinline__ void store_node(Node2* nodes, uint32_t i, const Box& b, uint32_t l, uint32_t r) {
    float4* p = reinterpret_cast<float4*>(nodes + i);
    p[0] = make_float4(b.mn.x, b.mn.y, b.mn.z, b.mx.x);
    p[1] = make_float4(b.mx.y, b.mx.z, __uint_as_float(l), __uint_as_float(r));
}

// The two children of an internal BVH2 node X side by side: both boxes and
// both indices in one 64-byte record (at X - n), written by the merge that
// creates X.  The BVH8 collapse opens X with this one aligned load instead
// of reading X's node and then both child nodes; X's own box is the union
// of the two, exactly (every internal box is computed as that union).
struct __align__(64) ChildPair {
    Box l, r;
    uint32_t li, ri;
    uint32_t pad[2];
};
static_assert(sizeof(ChildPair) == 64, "child pair record");

__device__ __forceinline__ void store_child_pair(ChildPair* p, const Box& l, const Box& r, uint32_t li,
                                                 uint32_t ri) {
    uint4* q = reinterpret_cast<uint4*>(p);
    __stcg(q, make_uint4(__float_as_uint(l.mn.x), __float_as_uint(l.mn.y), __float_as_uint(l.mn.z),
                         __float_as_uint(l.mx.x)));
    __stcg(q + 1, make_uint4(__float_as_uint(l.mx.y), __float_as_uint(l.mx.z), __float_as_uint(r.mn.x),
                             __float_as_uint(r.mn.y)));
    __stcg(q + 2, make_uint4(__float_as_uint(r.mn.z), __float_as_uint(r.mx.x), __float_as_uint(r.mx.y),
                             __float_as_uint(r.mx.z)));
    __stcg(q + 3, make_uint4(li, ri, 0u, 0u));
}
// Through the read-only path: the records are finished by an earlier kernel.
__device__ __forceinline__ ChildPair load_child_pair(const ChildPair* p) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    const uint4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
    ChildPair r;
    r.l.mn = make_float3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
    r.l.mx = make_float3(__uint_as_float(a.w), __uint_as_float(b.x), __uint_as_float(b.y));
    r.r.mn = make_float3(__uint_as_float(b.z), __uint_as_float(b.w), __uint_as_float(c.x));
    r.r.mx = make_float3(__uint_as_float(c.y), __uint_as_float(c.z), __uint_as_float(c.w));
    r.li = d.x;
    r.ri = d.y;
    return r;
}

__device__ __forceinline__ Box shfl_box(const Box& b, uint32_t src) {
    Box r;
    r.mn.x = __shfl_sync(kFullMask, b.mn.x, src);
    r.mn.y = __shfl_sync(kFullMask, b.mn.y, src);
    r.mn.z = __shfl_sync(kFullMask, b.mn.z, src);
    r.mx.x = __shfl_sync(kFullMask, b.mx.x, src);
    r.mx.y = __shfl_sync(kFullMask, b.mx.y, src);
    r.mx.z = __shfl_sync(kFullMask, b.mx.z, src);
    return r;
}

// Asks L2 for the line holding p without waiting for it.
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t bit) {
    if (err) atomicOr(err, bit);
}

// ------------------------------------------------------------ mesh batches
// The largest m in [lo, hi] with off[m] <= x.  With off a prefix array of
// element counts, this is the mesh that owns element x (empty meshes repeat
// an offset and are skipped).
__device__ __forceinline__ uint32_t owner_of(const uint32_t* off, uint32_t lo, uint32_t hi, uint32_t x) {
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= x)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Sort key of a batched 30-bit build: mesh index << 32 | Morton code.
struct MeshKey {
    uint64_t v;
};

// One mesh of a build: its index, its first element in the concatenated
// arrays and its primitive count.
struct MeshSpan {
    uint32_t m, start, count;
};

// A plain build: one mesh, everything at offset 0.
struct SingleMesh {
    static constexpr bool kBatch = false;
    uint32_t n;
    __device__ __forceinline__ MeshSpan of_prim(uint32_t) const { return {0u, 0u, n}; }
};

// Independent meshes laid end to end.  Mesh m owns primitives (and sorted
// positions, parent slots, cluster slots) [off[m], off[m+1]), BVH2 nodes
// [2*off[m], 2*off[m] + 2*count - 1) and BVH8 nodes [off8[m], off8[m+1]).
struct MeshBatch {
    static constexpr bool kBatch = true;
    const uint32_t* off;   // meshes + 1 entries
    const uint32_t* off8;  // meshes + 1 entries, strictly increasing
    uint32_t meshes;
    __device__ __forceinline__ MeshSpan span(uint32_t m) const {
        const uint32_t s = __ldg(off + m);
        return {m, s, __ldg(off + m + 1) - s};
    }
    __device__ __forceinline__ MeshSpan of_prim(uint32_t g) const { return span(owner_of(off, 0, meshes - 1, g)); }
};

}  // namespace nxb
