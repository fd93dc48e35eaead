// ref_harness.cpp - drives the reference's own CUDA build (NexusBVH) for
// parity fixtures and for the timed reference arm.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.py against the
// reference's headers (never copied into this repository) and linked with
// the reference's own translation units into oracle/_ref/libnxbref_r*.so.
//
// Public path: NXB::BuildBVH2 / NXB::BuildBVH8 (NexusBVH/include/NXB/BVHBuilder.h).
// Stage path: the private kernels launched exactly as BuildBVH2 launches
// them (NexusBVH/src/BVHBuilder.cpp:13-56,114-155), to read back the Morton
// codes and the sorted permutation, which the public API does not expose.
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "Cuda/BuildState.h"
#include "Cuda/CudaUtils.h"
#include "Cuda/Setup.h"
#include "NXB/BVHBuilder.h"

using namespace NXB;

namespace {

void metrics_out(const BVHBuildMetrics& m, float* out9) {
    if (!out9) return;
    const float v[9] = {m.computeSceneBoundsTime, m.computeMortonCodesTime, m.radixSortTime,
                        m.bvhBuildTime,           m.bvh8ConversionTime,     m.totalTime,
                        m.bvh2Cost,               m.bvh8Cost,               m.averageChildPerNode};
    std::memcpy(out9, v, sizeof(v));
}

void bounds_out(const AABB& b, float* out6) {
    if (!out6) return;
    const float v[6] = {b.bMin.x, b.bMin.y, b.bMin.z, b.bMax.x, b.bMax.y, b.bMax.z};
    std::memcpy(out6, v, sizeof(v));
}

template <typename PrimT>
int build8(const void* d_prims, uint32_t n, int ps, void* d_nodes_out, uint32_t* d_prim_out, uint32_t* node_count,
           float* bounds6, float* metrics9) {
    BuildConfig cfg;
    cfg.prioritizeSpeed = ps != 0;
    BVHBuildMetrics m;
    BVH8 b = BuildBVH8<PrimT>((PrimT*)d_prims, n, cfg, metrics9 ? &m : nullptr);
    if (d_nodes_out) cudaMemcpy(d_nodes_out, b.nodes, sizeof(BVH8::Node) * b.nodeCount, cudaMemcpyDeviceToDevice);
    if (d_prim_out) cudaMemcpy(d_prim_out, b.primIdx, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice);
    *node_count = b.nodeCount;
    bounds_out(b.bounds, bounds6);
    metrics_out(m, metrics9);
    FreeDeviceBVH(b);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

template <typename PrimT>
int build2(const void* d_prims, uint32_t n, int ps, void* d_nodes_out, float* bounds6, float* metrics9) {
    BuildConfig cfg;
    cfg.prioritizeSpeed = ps != 0;
    BVHBuildMetrics m;
    BVH2 b = BuildBVH2<PrimT>((PrimT*)d_prims, n, cfg, metrics9 ? &m : nullptr);
    if (d_nodes_out) cudaMemcpy(d_nodes_out, b.nodes, sizeof(BVH2::Node) * b.nodeCount, cudaMemcpyDeviceToDevice);
    bounds_out(b.bounds, bounds6);
    metrics_out(m, metrics9);
    FreeDeviceBVH(b);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

template <typename PrimT, typename McT>
int stages(const void* d_prims, uint32_t n, void* d_nodes, float* scene6, void* d_keys, void* d_sorted,
           uint32_t* d_perm) {
    BVH2BuildState st;
    st.primCount = n;
    st.nodes = (BVH2::Node*)d_nodes;
    cudaMalloc((void**)&st.sceneBounds, sizeof(AABB));
    AABB clr;
    clr.Clear();
    cudaMemcpy(st.sceneBounds, &clr, sizeof(AABB), cudaMemcpyHostToDevice);
    uint32_t bs = 64;
    PrimT* prims = (PrimT*)d_prims;
    void* a1[2] = {&st, &prims};
    uint32_t grid = CudaUtils::GetGridSizeFullOccupancy((void*)ComputeSceneBoundsKernel<PrimT>, bs);
    cudaLaunchKernel((void*)ComputeSceneBoundsKernel<PrimT>, grid, bs, a1, 0, 0);
    // stream-ordered like CudaMemory::AllocAsync, because RadixSort frees
    // the buffers that end up not current with cudaFreeAsync
    cudaMallocAsync((void**)&st.clusterIdx, sizeof(uint32_t) * n, 0);
    McT* mc = nullptr;
    cudaMallocAsync((void**)&mc, sizeof(McT) * n, 0);
    void* a2[2] = {&st, &mc};
    grid = CudaUtils::GetGridSizeFullOccupancy((void*)ComputeMortonCodesKernel<McT>, bs);
    cudaLaunchKernel((void*)ComputeMortonCodesKernel<McT>, grid, bs, a2, 0, 0);
    cudaMemcpy(d_keys, mc, sizeof(McT) * n, cudaMemcpyDeviceToDevice);
    RadixSort<McT>(st, mc, nullptr);
    cudaMemcpy(d_sorted, mc, sizeof(McT) * n, cudaMemcpyDeviceToDevice);
    cudaMemcpy(d_perm, st.clusterIdx, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice);
    AABB scene;
    cudaMemcpy(&scene, st.sceneBounds, sizeof(AABB), cudaMemcpyDeviceToHost);
    bounds_out(scene, scene6);
    cudaDeviceSynchronize();
    // RadixSort freed the buffers that are not current; free the current ones
    cudaFreeAsync(mc, 0);
    cudaFreeAsync(st.clusterIdx, 0);
    cudaFree(st.sceneBounds);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

}  // namespace

extern "C" {

// prim_type: 1 = Triangle, 0 = AABB.  Device buffers are the caller's.
int ref_build_bvh8(const void* d_prims, int prim_type, uint32_t n, int prioritize_speed, void* d_nodes_out,
                   uint32_t* d_prim_out, uint32_t* node_count, float* bounds6, float* metrics9) {
    return prim_type == 1 ? build8<Triangle>(d_prims, n, prioritize_speed, d_nodes_out, d_prim_out, node_count,
                                             bounds6, metrics9)
                          : build8<AABB>(d_prims, n, prioritize_speed, d_nodes_out, d_prim_out, node_count, bounds6,
                                         metrics9);
}

int ref_build_bvh2(const void* d_prims, int prim_type, uint32_t n, int prioritize_speed, void* d_nodes_out,
                   float* bounds6, float* metrics9) {
    return prim_type == 1 ? build2<Triangle>(d_prims, n, prioritize_speed, d_nodes_out, bounds6, metrics9)
                          : build2<AABB>(d_prims, n, prioritize_speed, d_nodes_out, bounds6, metrics9);
}

// Stage outputs: leaves in d_nodes[0, n), scene box, unsorted and sorted
// Morton keys, sorted permutation.
int ref_stages(const void* d_prims, int prim_type, uint32_t n, int prioritize_speed, void* d_nodes, float* scene6,
               void* d_keys, void* d_sorted, uint32_t* d_perm) {
    if (prim_type == 1)
        return prioritize_speed ? stages<Triangle, uint32_t>(d_prims, n, d_nodes, scene6, d_keys, d_sorted, d_perm)
                                : stages<Triangle, uint64_t>(d_prims, n, d_nodes, scene6, d_keys, d_sorted, d_perm);
    return prioritize_speed ? stages<AABB, uint32_t>(d_prims, n, d_nodes, scene6, d_keys, d_sorted, d_perm)
                            : stages<AABB, uint64_t>(d_prims, n, d_nodes, scene6, d_keys, d_sorted, d_perm);
}

// The reference arm of the benchmark: host triangles in, one BuildBVH8 call,
// BVH8 freed.  Host->device copy inside, like a caller with host data.
int ref_e2e_bvh8(const void* h_prims, size_t prim_bytes, void* d_prims, int prim_type, uint32_t n,
                 int prioritize_speed, uint32_t* node_count) {
    cudaMemcpy(d_prims, h_prims, prim_bytes, cudaMemcpyHostToDevice);
    return ref_build_bvh8(d_prims, prim_type, n, prioritize_speed, nullptr, nullptr, node_count, nullptr, nullptr);
}

}  // extern "C"
