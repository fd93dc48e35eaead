// NXB/BVHBuildMetrics.h - drop-in for NexusBVH/include/NXB/BVHBuildMetrics.h:
// per-stage CUDA-event times (totalTime = their sum), SAH costs, and the
// BenchmarkBuild helper (warm-up runs, then averaged measured runs).
#pragma once

#include <cstdint>
#include <iostream>
#include <type_traits>
#include <utility>

#include "BVH.h"

namespace NXB {

struct BVHBuildMetrics {
    BVHBuildMetrics& operator+=(const BVHBuildMetrics& o) {
        computeSceneBoundsTime += o.computeSceneBoundsTime;
        computeMortonCodesTime += o.computeMortonCodesTime;
        radixSortTime += o.radixSortTime;
        bvhBuildTime += o.bvhBuildTime;
        bvh8ConversionTime += o.bvh8ConversionTime;
        totalTime += o.totalTime;
        bvh2Cost += o.bvh2Cost;
        bvh8Cost += o.bvh8Cost;
        averageChildPerNode += o.averageChildPerNode;
        return *this;
    }
    BVHBuildMetrics operator/(float d) const {
        BVHBuildMetrics r = *this;
        r.computeSceneBoundsTime /= d;
        r.computeMortonCodesTime /= d;
        r.radixSortTime /= d;
        r.bvhBuildTime /= d;
        r.bvh8ConversionTime /= d;
        r.totalTime /= d;
        r.bvh2Cost /= d;
        r.bvh8Cost /= d;
        r.averageChildPerNode /= d;
        return r;
    }

    float computeSceneBoundsTime = 0.0f;
    float computeMortonCodesTime = 0.0f;
    float radixSortTime = 0.0f;
    float bvhBuildTime = 0.0f;
    float bvh8ConversionTime = 0.0f;
    float totalTime = 0.0f;
    float bvh2Cost = 0.0f;
    float bvh8Cost = 0.0f;
    float averageChildPerNode = 0.0f;
};
static_assert(sizeof(BVHBuildMetrics) == 36, "metrics layout");

void FreeDeviceBVH(BVH2 bvh);
void FreeDeviceBVH(BVH8 bvh);

// Calls func(args..., &metrics) warmup + measured times, frees every result
// and returns the averaged metrics (printed like the reference does).
template <typename Func, typename... Args>
BVHBuildMetrics BenchmarkBuild(Func&& func, uint32_t warmupIterations, uint32_t measuredIterations, Args&&... args) {
    using ReturnT = decltype(func(std::forward<Args>(args)..., nullptr));
    BVHBuildMetrics sum = {};
    for (uint32_t i = 0; i < warmupIterations; ++i) {
        BVHBuildMetrics scratch;
        FreeDeviceBVH(func(std::forward<Args>(args)..., &scratch));
    }
    for (uint32_t i = 0; i < measuredIterations; ++i) {
        BVHBuildMetrics m = {};
        FreeDeviceBVH(func(std::forward<Args>(args)..., &m));
        sum += m;
    }
    BVHBuildMetrics avg = measuredIterations ? sum / static_cast<float>(measuredIterations) : sum;
    std::cout << "Scene bounds: " << avg.computeSceneBoundsTime << " ms\n"
              << "Morton codes: " << avg.computeMortonCodesTime << " ms\n"
              << "Radix sort: " << avg.radixSortTime << " ms\n"
              << "BVH2 build time: " << avg.bvhBuildTime << " ms\n";
    if constexpr (std::is_same_v<ReturnT, BVH8>)
        std::cout << "BVH8 conversion time: " << avg.bvh8ConversionTime << " ms\n";
    std::cout << "Total BVH build time: " << avg.totalTime << " ms\n"
              << "BVH2 cost: " << avg.bvh2Cost << "\n";
    if constexpr (std::is_same_v<ReturnT, BVH8>)
        std::cout << "BVH8 cost: " << avg.bvh8Cost << "\nAverage children per node: " << avg.averageChildPerNode
                  << "\n";
    return avg;
}

}  // namespace NXB
