// eval.cu - cost evaluation, small utility kernels and the numerics
// self-test.
//
// Cost kernels replace ComputeBVH2CostKernel / ComputeBVH8CostKernel
// (NexusBVH/src/Cuda/Eval.cu:12-80), keeping the reference's weights:
// BVH2 internal nodes C_T = 3, leaves C_I = 2, every node including the
// root; BVH8 children only, internal children 2, leaf children 3, boxes
// decoded as p + 2^(e-127) * q.  Sums are reduced per CTA and added with
// one float atomic per CTA, so the last bits depend on CTA order (the
// reference has the same property); parity is judged within 0.1%.
#include <cstring>
#include <vector>

#include <algorithm>

#include "pipeline.h"

namespace nxb {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float cta_sum(float v) {
    __shared__ float s[kThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFullMask, v, o);
    if (lane_id() == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = 0.f;
    if (threadIdx.x < 32) {
        t = threadIdx.x < kThreads / 32 ? s[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(kFullMask, t, o);
    }
    return t;
}

__device__ __forceinline__ Box to_box(const nxb_aabb* a) {
    Box b;
    b.mn = make_float3(a->bmin[0], a->bmin[1], a->bmin[2]);
    b.mx = make_float3(a->bmax[0], a->bmax[1], a->bmax[2]);
    return b;
}

__global__ __launch_bounds__(kThreads) void bvh2_cost_kernel(const Node2* nodes, uint32_t count,
                                                             const nxb_aabb* root, float* cost) {
    const float ra = half_area(to_box(root));
    float acc = 0.f;
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < count; i += gridDim.x * kThreads) {
        const Node2 nd = nodes[i];
        const float m = half_area(nd.b) / ra;
        acc += (nd.left != kInvalid ? 3.0f : 2.0f) * m;
    }
    acc = cta_sum(acc);
    if (threadIdx.x == 0) atomicAdd(cost, acc);
}

__global__ __launch_bounds__(kThreads) void bvh8_cost_kernel(const Node8* nodes, const uint32_t* count_ptr,
                                                             uint32_t count, const nxb_aabb* root, float* cost) {
    if (count_ptr) count = min(*count_ptr, count);
    const float ra = half_area(to_box(root));
    float acc = 0.f;
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < count; i += gridDim.x * kThreads) {
        const Node8 nd = nodes[i];
        float sc[3];
        for (int a = 0; a < 3; ++a) sc[a] = __uint_as_float((uint32_t)nd.e[a] << 23);
        for (int c = 0; c < 8; ++c) {
            if (!nd.meta[c]) continue;
            const bool internal = (nd.meta[c] & 0x1Fu) >= 24u;
            Box b;
            b.mn = make_float3(__fmaf_rn(sc[0], (float)nd.qlo[0][c], nd.p[0]),
                               __fmaf_rn(sc[1], (float)nd.qlo[1][c], nd.p[1]),
                               __fmaf_rn(sc[2], (float)nd.qlo[2][c], nd.p[2]));
            b.mx = make_float3(__fmaf_rn(sc[0], (float)nd.qhi[0][c], nd.p[0]),
                               __fmaf_rn(sc[1], (float)nd.qhi[1][c], nd.p[1]),
                               __fmaf_rn(sc[2], (float)nd.qhi[2][c], nd.p[2]));
            acc += (internal ? 2.0f : 3.0f) * (half_area(b) / ra);
        }
    }
    acc = cta_sum(acc);
    if (threadIdx.x == 0) atomicAdd(cost, acc);
}

__global__ void finalize_kernel(const Control* ctrl, nxb_build_result* r, uint32_t n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int a = 0; a < 3; ++a) {
        r->scene_bounds.bmin[a] = ord2f(~ctrl->scene_ord[a]);
        r->scene_bounds.bmax[a] = ord2f(ctrl->scene_ord[3 + a]);
    }
    r->bvh8_node_count = ctrl->bvh8_ctr[kBvh8Nodes];
    r->bvh8_leaf_count = ctrl->bvh8_ctr[kBvh8Leaves];
    r->error_word = ctrl->error_word;
    r->bvh2_root = 2 * n - 2;
}

__global__ void ord_to_aabb_kernel(uint32_t* ord) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t o[6];
    for (int a = 0; a < 6; ++a) o[a] = ord[a];
    float* f = reinterpret_cast<float*>(ord);
    for (int a = 0; a < 3; ++a) {
        f[a] = ord2f(~o[a]);
        f[3 + a] = ord2f(o[3 + a]);
    }
}

__global__ void fill_u32_kernel(uint32_t* p, uint32_t value, size_t count) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        p[i] = value;
}

// ---- numerics self-test probes: the reference's plain source expressions
// compiled with the same flags, next to the library's pinned forms.
__global__ void probe_area_kernel(const float* boxes, uint32_t count, uint32_t* out, uint32_t* paired_diff) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float* f = boxes + 6 * i;
    Box b;
    b.mn = make_float3(f[0], f[1], f[2]);
    b.mx = make_float3(f[3], f[4], f[5]);
    {
        // the paired form against the single one, with box i^1 as partner
        const float* g = boxes + 6 * (i ^ 1u);
        Box c;
        c.mn = make_float3(g[0], g[1], g[2]);
        c.mx = make_float3(g[3], g[4], g[5]);
        float rb, rc;
        half_area2(b, c, rb, rc);
        if (__float_as_uint(rb) != __float_as_uint(half_area(b)) || __float_as_uint(rc) != __float_as_uint(half_area(c)))
            atomicAdd(paired_diff, 1u);
    }
    const float dx = b.mx.x - b.mn.x, dy = b.mx.y - b.mn.y, dz = b.mx.z - b.mn.z;
    const float plain = dx * dy + dy * dz + dz * dx;  // AABB::Area, NXB AABB.h:46-50
    const float f0 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
    const float f1 = __fmaf_rn(dz, dx, __fmaf_rn(dy, dz, __fmul_rn(dx, dy)));
    out[4 * i + 0] = __float_as_uint(plain);
    out[4 * i + 1] = __float_as_uint(f0);
    out[4 * i + 2] = __float_as_uint(f1);
    out[4 * i + 3] = __float_as_uint(half_area(b));
}

// (uint8_t)floorf((a-b)*c) and (uint8_t)ceilf((a-b)*c) as in CreateBVH8Node
// (WideConverter.cu:195-201); fminf/fmaxf of signed zeros; fast-math
// division against IEEE division.
__global__ void probe_misc_kernel(const float* v, uint32_t count, uint32_t* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float a = v[3 * i], b = v[3 * i + 1], c = v[3 * i + 2];
    const uint8_t lo = (uint8_t)floorf((a - b) * c);
    const uint8_t hi = (uint8_t)ceilf((a - b) * c);
    out[6 * i + 0] = lo;
    out[6 * i + 1] = hi;
    out[6 * i + 2] = __float_as_uint(fminf(a, b));
    out[6 * i + 3] = __float_as_uint(fmaxf(a, b));
    out[6 * i + 4] = __float_as_uint(a / c);
    out[6 * i + 5] = __float_as_uint(__fdiv_rn(a, c));
}

}  // namespace

cudaError_t launch_bvh2_cost(const Node2* nodes, uint32_t count, const nxb_aabb* root, float* cost, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(cost, 0, sizeof(float), s);
    if (e != cudaSuccess) return e;
    uint32_t grid = std::min<uint32_t>((count + kThreads - 1) / kThreads, (uint32_t)device_info().sms * 8);
    bvh2_cost_kernel<<<std::max(1u, grid), kThreads, 0, s>>>(nodes, count, root, cost);
    return cudaGetLastError();
}

cudaError_t launch_bvh8_cost_dev(const Node8* nodes, const uint32_t* count_ptr, uint32_t cap, const nxb_aabb* root,
                                 float* cost, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(cost, 0, sizeof(float), s);
    if (e != cudaSuccess) return e;
    uint32_t grid = std::min<uint32_t>((cap + kThreads - 1) / kThreads, (uint32_t)device_info().sms * 8);
    bvh8_cost_kernel<<<std::max(1u, grid), kThreads, 0, s>>>(nodes, count_ptr, cap, root, cost);
    return cudaGetLastError();
}

cudaError_t launch_bvh8_cost(const Node8* nodes, uint32_t count, const nxb_aabb* root, float* cost, cudaStream_t s) {
    return launch_bvh8_cost_dev(nodes, nullptr, count, root, cost, s);
}

cudaError_t launch_finalize(const Control* ctrl, nxb_build_result* result, uint32_t n, cudaStream_t s) {
    finalize_kernel<<<1, 32, 0, s>>>(ctrl, result, n);
    return cudaGetLastError();
}

cudaError_t launch_ord_to_aabb(uint32_t* ord, cudaStream_t s) {
    ord_to_aabb_kernel<<<1, 32, 0, s>>>(ord);
    return cudaGetLastError();
}

cudaError_t launch_fill_u32(uint32_t* p, uint32_t value, size_t count, cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    size_t want = (count + 255) / 256;
    uint32_t grid = (uint32_t)std::min<size_t>(want, (size_t)device_info().sms * 8);
    fill_u32_kernel<<<grid, 256, 0, s>>>(p, value, count);
    return cudaGetLastError();
}

// Runs the numerics probes on deterministic inputs.  report (length >= 40):
//  [0] boxes probed; [1..3] boxes where the plain Area expression differs
//  from: no contraction / fma(dz,dx,fma(dy,dz,dx*dy)) / the pinned form;
//  [4..11] (uint8_t)floorf and [12..19] (uint8_t)ceilf of
//  {254.5, 255, 255.25, 256, 256.5, 300, 511.75, -1.5};
//  [20..23] bits of fminf(+0,-0), fminf(-0,+0), fmaxf(+0,-0), fmaxf(-0,+0);
//  [24] divisions probed, [25] fast-math quotients != IEEE quotients,
//  [26] of those, differences larger than 1 ulp;
//  [27] boxes whose paired area (half_area2) differs from half_area.
cudaError_t run_selftest(uint32_t* report) {
    const uint32_t nb = 1u << 16;
    std::vector<float> boxes(6 * nb);
    uint64_t st = 0x9E3779B97F4A7C15ull;
    auto rnd = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return (float)((st >> 40) & 0xFFFFFFu) / 16777216.0f;
    };
    for (uint32_t i = 0; i < nb; ++i) {
        float c[3], h[3];
        // the last 4,096 boxes near the smallest normal floats, where
        // flushing subnormal differences and products matters
        const bool tiny = i >= nb - 4096;
        for (int a = 0; a < 3; ++a) {
            c[a] = (rnd() - 0.5f) * (tiny ? 4e-38f : 20.0f);
            h[a] = rnd() * rnd() * (tiny ? 2e-38f : 2.0f);
        }
        for (int a = 0; a < 3; ++a) {
            boxes[6 * i + a] = c[a] - h[a];
            boxes[6 * i + 3 + a] = c[a] + h[a];
        }
    }
    const float lv[8] = {254.5f, 255.0f, 255.25f, 256.0f, 256.5f, 300.0f, 511.75f, -1.5f};
    const uint32_t nm = 8 + 2 + (1u << 14);
    std::vector<float> misc(3 * nm);
    for (int k = 0; k < 8; ++k) {
        misc[3 * k] = lv[k];
        misc[3 * k + 1] = 0.0f;
        misc[3 * k + 2] = 1.0f;
    }
    misc[24] = 0.0f, misc[25] = -0.0f, misc[26] = 1.0f;
    misc[27] = -0.0f, misc[28] = 0.0f, misc[29] = 1.0f;
    for (uint32_t k = 10; k < nm; ++k) {
        misc[3 * k] = rnd() * 3.0f;
        misc[3 * k + 1] = 0.0f;
        misc[3 * k + 2] = 0.25f + rnd() * 4.0f;
    }
    float *d_boxes = nullptr, *d_misc = nullptr;
    uint32_t *d_out = nullptr, *d_out2 = nullptr, *d_paired = nullptr;
    cudaError_t e = cudaMalloc(&d_boxes, boxes.size() * 4);
    if (!e) e = cudaMalloc(&d_paired, 4);
    if (!e) e = cudaMemset(d_paired, 0, 4);
    if (!e) e = cudaMalloc(&d_misc, misc.size() * 4);
    if (!e) e = cudaMalloc(&d_out, (size_t)nb * 16);
    if (!e) e = cudaMalloc(&d_out2, (size_t)nm * 24);
    if (!e) e = cudaMemcpy(d_boxes, boxes.data(), boxes.size() * 4, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d_misc, misc.data(), misc.size() * 4, cudaMemcpyHostToDevice);
    if (!e) {
        probe_area_kernel<<<(nb + 255) / 256, 256>>>(d_boxes, nb, d_out, d_paired);
        probe_misc_kernel<<<(nm + 255) / 256, 256>>>(d_misc, nm, d_out2);
        e = cudaGetLastError();
    }
    std::vector<uint32_t> o1((size_t)nb * 4), o2((size_t)nm * 6);
    if (!e) e = cudaMemcpy(o1.data(), d_out, o1.size() * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(o2.data(), d_out2, o2.size() * 4, cudaMemcpyDeviceToHost);
    uint32_t paired = 0;
    if (!e) e = cudaMemcpy(&paired, d_paired, 4, cudaMemcpyDeviceToHost);
    cudaFree(d_paired);
    cudaFree(d_boxes);
    cudaFree(d_misc);
    cudaFree(d_out);
    cudaFree(d_out2);
    if (e) return e;
    std::memset(report, 0, 40 * sizeof(uint32_t));
    report[0] = nb;
    for (uint32_t i = 0; i < nb; ++i)
        for (int f = 0; f < 3; ++f) report[1 + f] += o1[4 * i] != o1[4 * i + 1 + f];
    for (int k = 0; k < 8; ++k) {
        report[4 + k] = o2[6 * k];
        report[12 + k] = o2[6 * k + 1];
    }
    report[20] = o2[6 * 8 + 2];
    report[21] = o2[6 * 9 + 2];
    report[22] = o2[6 * 8 + 3];
    report[23] = o2[6 * 9 + 3];
    for (uint32_t k = 10; k < nm; ++k) {
        report[24]++;
        uint32_t q = o2[6 * k + 4], r = o2[6 * k + 5];
        if (q != r) {
            report[25]++;
            if ((q > r ? q - r : r - q) > 1) report[26]++;
        }
    }
    report[27] = paired;
    return cudaSuccess;
}

}  // namespace nxb
