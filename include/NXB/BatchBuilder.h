// NXB/BatchBuilder.h - C++ wrappers of the batched and served builds.
//
// No counterpart in the reference, whose API builds one mesh per call
// (NexusBVH/include/NXB/BVHBuilder.h:18-43).  These classes own the C-ABI
// handles (nxb_batch / nxb_server in nxb_gb300.h) and report errors the way
// the rest of the facade does (print and exit(99), or throw with
// NXB_FACADE_THROW).
#pragma once

#include <cstdint>
#include <vector>

#include "BVHBuilder.h"

namespace NXB {

// Many independent meshes built together: one launch per stage for all of
// them, replayed from a CUDA graph.  Every mesh equals its BuildBVH8 result
// (30-bit Morton codes: buildConfig.prioritizeSpeed must be true).
template <typename PrimT>
class BatchBuilder {
public:
    // primCounts[m] = primitive count of mesh m; the meshes' primitives are
    // passed end to end to Build().
    BatchBuilder(const std::vector<uint32_t>& primCounts, BuildConfig buildConfig) {
        offsets_.assign(primCounts.size() + 1, 0);
        for (size_t m = 0; m < primCounts.size(); ++m) offsets_[m + 1] = offsets_[m] + primCounts[m];
        nxb_build_config c = detail::to_c(buildConfig);
        detail::on_error(nxb_batch_create(detail::prim_type<PrimT>(), offsets_.data(),
                                          (uint32_t)primCounts.size(), &c, &batch_),
                         "BatchBuilder");
        meshes_.resize(primCounts.size());
    }
    BatchBuilder(const BatchBuilder&) = delete;
    BatchBuilder& operator=(const BatchBuilder&) = delete;
    ~BatchBuilder() {
        if (batch_) nxb_batch_destroy(batch_);
    }

    // Builds every mesh from device primitives and waits for the stream.
    void Build(const PrimT* primitives, struct CUstream_st* stream = nullptr) {
        detail::on_error(nxb_batch_build(batch_, primitives, stream, meshes_.data()), "BatchBuilder::Build");
    }
    // Picks the fastest settings on this batch and input (see nxb_batch_autotune).
    nxb_batch_tuning Autotune(const PrimT* primitives, bool tuneRadius = false, struct CUstream_st* stream = nullptr) {
        nxb_batch_tuning t{};
        detail::on_error(nxb_batch_autotune(batch_, primitives, tuneRadius ? NXB_TUNE_RADIUS : 0u, 3, stream, &t),
                         "BatchBuilder::Autotune");
        return t;
    }
    // Per-mesh results of the last Build().
    const std::vector<nxb_batch_mesh>& Meshes() const { return meshes_; }
    // Device view of mesh m's BVH8 (valid until the next Build()); its
    // child_base / prim_base / primIdx are mesh-local, as in BuildBVH8.
    BVH8 MeshBVH8(uint32_t m) const {
        nxb_batch_arrays a{};
        detail::on_error(nxb_batch_get_arrays(batch_, &a), "BatchBuilder::MeshBVH8");
        const nxb_batch_mesh& r = meshes_.at(m);
        BVH8 b;
        b.nodes = reinterpret_cast<BVH8::Node*>(const_cast<nxb_bvh8_node*>(a.bvh8_nodes + r.bvh8_offset));
        b.nodeCount = r.bvh8_node_count;
        b.primIdx = const_cast<uint32_t*>(a.prim_idx + r.prim_offset);
        b.primCount = r.prim_count;
        b.bounds.bMin = float3{r.scene_bounds.bmin[0], r.scene_bounds.bmin[1], r.scene_bounds.bmin[2]};
        b.bounds.bMax = float3{r.scene_bounds.bmax[0], r.scene_bounds.bmax[1], r.scene_bounds.bmax[2]};
        return b;
    }

private:
    std::vector<uint32_t> offsets_;
    std::vector<nxb_batch_mesh> meshes_;
    nxb_batch* batch_ = nullptr;
};

// A build service: Submit() meshes (host or device memory) and Wait() for
// their BVH8s; requests that wait together are built as one batch, under a
// device-memory budget.  A result's device arrays stay valid until Release().
class BuildServer {
public:
    explicit BuildServer(size_t memoryBudgetBytes = 0, uint32_t streams = 0) {
        nxb_server_config c{};
        c.memory_budget_bytes = memoryBudgetBytes;
        c.streams = streams;
        detail::on_error(nxb_server_create(&c, &server_), "BuildServer");
    }
    BuildServer(const BuildServer&) = delete;
    BuildServer& operator=(const BuildServer&) = delete;
    ~BuildServer() {
        if (server_) nxb_server_destroy(server_);
    }

    template <typename PrimT>
    uint64_t Submit(const PrimT* primitives, uint32_t primCount, bool onDevice, BuildConfig buildConfig = BuildConfig()) {
        nxb_build_config c = detail::to_c(buildConfig);
        uint64_t ticket = 0;
        detail::on_error(nxb_server_submit(server_, primitives, onDevice ? 1 : 0, detail::prim_type<PrimT>(),
                                           primCount, &c, &ticket),
                         "BuildServer::Submit");
        return ticket;
    }
    // Blocks until the request completes; latency and batching in `info`.
    BVH8 Wait(uint64_t ticket, nxb_server_result* info = nullptr) {
        nxb_server_result r{};
        detail::on_error(nxb_server_wait(server_, ticket, &r), "BuildServer::Wait");
        if (info) *info = r;
        BVH8 b;
        b.nodes = reinterpret_cast<BVH8::Node*>(r.bvh8.nodes);
        b.nodeCount = r.bvh8.node_count;
        b.primIdx = r.bvh8.prim_idx;
        b.primCount = r.bvh8.prim_count;
        b.bounds.bMin = float3{r.bvh8.bounds.bmin[0], r.bvh8.bounds.bmin[1], r.bvh8.bounds.bmin[2]};
        b.bounds.bMax = float3{r.bvh8.bounds.bmax[0], r.bvh8.bounds.bmax[1], r.bvh8.bounds.bmax[2]};
        return b;
    }
    void Release(uint64_t ticket) { detail::on_error(nxb_server_release(server_, ticket), "BuildServer::Release"); }

private:
    nxb_server* server_ = nullptr;
};

}  // namespace NXB
