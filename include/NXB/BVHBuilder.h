// NXB/BVHBuilder.h - drop-in for NexusBVH/include/NXB/BVHBuilder.h.
//
// Header-only facade over the C ABI (nxb_gb300.h): the same templates, names
// and argument meaning as the reference (BVHBuilder.h:18-55).  Builds run
// on the legacy default stream and return with it drained, like the
// reference.  On any error the reference prints and exits with status 99
// (NexusBVH/src/Cuda/CudaUtils.h:6-16); so does this facade, unless
// NXB_FACADE_THROW is defined, in which case it throws std::runtime_error.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../nxb_gb300.h"
#include "AABB.h"
#include "BVH.h"
#include "BVHBuildMetrics.h"
#include "BuildConfig.h"
#include "Triangle.h"

namespace NXB {

namespace detail {
inline void on_error(nxb_status s, const char* what) {
    if (s == NXB_OK) return;
#ifdef NXB_FACADE_THROW
    throw std::runtime_error(std::string(what) + ": " + nxb_status_string(s));
#else
    std::fprintf(stderr, "NXB error %s in %s (cuda error %d)\n", nxb_status_string(s), what, nxb_last_cuda_error());
    std::exit(99);
#endif
}
template <typename PrimT>
constexpr nxb_prim_type prim_type() {
    static_assert(std::is_same_v<PrimT, Triangle> || std::is_same_v<PrimT, AABB>, "PrimT is Triangle or AABB");
    return std::is_same_v<PrimT, Triangle> ? NXB_PRIM_TRIANGLE : NXB_PRIM_AABB;
}
inline nxb_build_config to_c(const BuildConfig& c) {
    nxb_build_config r{};
    r.prioritize_speed = c.prioritizeSpeed ? 1u : 0u;
    r.search_radius = c.searchRadius;
    r.flags = (c.useAuction ? NXB_BUILD_AUCTION : 0u) | (c.validate ? NXB_BUILD_VALIDATE : 0u);
    return r;
}
inline void from_c(const nxb_build_metrics& m, BVHBuildMetrics* out) {
    if (!out) return;
    out->computeSceneBoundsTime = m.scene_bounds_time;
    out->computeMortonCodesTime = m.morton_codes_time;
    out->radixSortTime = m.radix_sort_time;
    out->bvhBuildTime = m.bvh2_build_time;
    out->bvh8ConversionTime = m.bvh8_conversion_time;
    out->totalTime = m.total_time;
    out->bvh2Cost = m.bvh2_cost;
    out->bvh8Cost = m.bvh8_cost;
    out->averageChildPerNode = m.average_child_per_node;
}
}  // namespace detail

template <typename PrimT>
BVH2 BuildBVH2(PrimT* primitives, uint32_t primCount, BuildConfig buildConfig = BuildConfig(),
               BVHBuildMetrics* buildMetrics = nullptr) {
    nxb_build_config c = detail::to_c(buildConfig);
    nxb_build_metrics m{};
    nxb_bvh2 out{};
    detail::on_error(nxb_build_bvh2(primitives, detail::prim_type<PrimT>(), primCount, &c, nullptr, &out,
                                    buildMetrics ? &m : nullptr),
                     "BuildBVH2");
    detail::from_c(m, buildMetrics);
    BVH2 r;
    r.nodes = reinterpret_cast<BVH2::Node*>(out.nodes);
    r.nodeCount = out.node_count;
    r.primCount = out.prim_count;
    r.bounds.bMin = float3{out.bounds.bmin[0], out.bounds.bmin[1], out.bounds.bmin[2]};
    r.bounds.bMax = float3{out.bounds.bmax[0], out.bounds.bmax[1], out.bounds.bmax[2]};
    return r;
}

template <typename PrimT>
BVH8 BuildBVH8(PrimT* primitives, uint32_t primCount, BuildConfig buildConfig = BuildConfig(),
               BVHBuildMetrics* buildMetrics = nullptr) {
    nxb_build_config c = detail::to_c(buildConfig);
    nxb_build_metrics m{};
    nxb_bvh8 out{};
    detail::on_error(nxb_build_bvh8(primitives, detail::prim_type<PrimT>(), primCount, &c, nullptr, &out,
                                    buildMetrics ? &m : nullptr),
                     "BuildBVH8");
    detail::from_c(m, buildMetrics);
    BVH8 r;
    r.nodes = reinterpret_cast<BVH8::Node*>(out.nodes);
    r.nodeCount = out.node_count;
    r.primIdx = out.prim_idx;
    r.primCount = out.prim_count;
    r.bounds.bMin = float3{out.bounds.bmin[0], out.bounds.bmin[1], out.bounds.bmin[2]};
    r.bounds.bMax = float3{out.bounds.bmax[0], out.bounds.bmax[1], out.bounds.bmax[2]};
    return r;
}

inline nxb_bvh2 to_c(const BVH2& b) {
    nxb_bvh2 r{};
    r.nodes = reinterpret_cast<nxb_bvh2_node*>(b.nodes);
    r.node_count = b.nodeCount;
    r.prim_count = b.primCount;
    return r;
}

inline BVH2 ToHost(BVH2 deviceBvh) {
    nxb_bvh2 d = to_c(deviceBvh), h{};
    detail::on_error(nxb_bvh2_to_host(&d, &h), "ToHost");
    BVH2 r = deviceBvh;
    r.nodes = reinterpret_cast<BVH2::Node*>(h.nodes);
    return r;
}

inline void FreeHostBVH(BVH2 hostBvh) {
    nxb_bvh2 h = to_c(hostBvh);
    detail::on_error(nxb_free_host_bvh2(&h), "FreeHostBVH");
}

inline void FreeDeviceBVH(BVH2 deviceBvh) {
    nxb_bvh2 d = to_c(deviceBvh);
    detail::on_error(nxb_free_device_bvh2(&d), "FreeDeviceBVH");
}

inline void FreeDeviceBVH(BVH8 deviceBvh) {
    nxb_bvh8 d{};
    d.nodes = reinterpret_cast<nxb_bvh8_node*>(deviceBvh.nodes);
    d.node_count = deviceBvh.nodeCount;
    d.prim_idx = deviceBvh.primIdx;
    d.prim_count = deviceBvh.primCount;
    detail::on_error(nxb_free_device_bvh8(&d), "FreeDeviceBVH");
}

}  // namespace NXB
