// NXB/AABB.h - drop-in for NexusBVH/include/NXB/AABB.h (same layout, 24 B).
#pragma once

#include <cfloat>
#include <vector_types.h>

#if defined(__CUDACC__)
#define NXB_HD __host__ __device__
#else
#define NXB_HD
#endif

namespace NXB {

namespace detail {
NXB_HD inline float fmin1(float a, float b) { return a < b ? a : b; }
NXB_HD inline float fmax1(float a, float b) { return a > b ? a : b; }
NXB_HD inline float3 min3(float3 a, float3 b) { return float3{fmin1(a.x, b.x), fmin1(a.y, b.y), fmin1(a.z, b.z)}; }
NXB_HD inline float3 max3(float3 a, float3 b) { return float3{fmax1(a.x, b.x), fmax1(a.y, b.y), fmax1(a.z, b.z)}; }
}  // namespace detail

struct AABB {
    AABB() = default;
    NXB_HD AABB(float3 a, float3 b) : bMin(detail::min3(a, b)), bMax(detail::max3(a, b)) {}
    NXB_HD AABB(float3 a, float3 b, float3 c)
        : bMin(detail::min3(a, detail::min3(b, c))), bMax(detail::max3(a, detail::max3(b, c))) {}

    NXB_HD void Grow(float3 v) {
        bMin = detail::min3(bMin, v);
        bMax = detail::max3(bMax, v);
    }
    NXB_HD void Grow(const AABB& o) {
        bMin = detail::min3(bMin, o.bMin);
        bMax = detail::max3(bMax, o.bMax);
    }
    NXB_HD void Clear() {
        bMin = float3{FLT_MAX, FLT_MAX, FLT_MAX};
        bMax = float3{-FLT_MAX, -FLT_MAX, -FLT_MAX};
    }
    NXB_HD float3 Centroid() const {
        return float3{(bMin.x + bMax.x) * 0.5f, (bMin.y + bMax.y) * 0.5f, (bMin.z + bMax.z) * 0.5f};
    }
    // half the surface area, as the reference defines it
    NXB_HD float Area() const {
        float dx = bMax.x - bMin.x, dy = bMax.y - bMin.y, dz = bMax.z - bMin.z;
        return dx * dy + dy * dz + dz * dx;
    }

    float3 bMin;
    float3 bMax;
};
static_assert(sizeof(AABB) == 24, "NXB::AABB layout");

}  // namespace NXB
