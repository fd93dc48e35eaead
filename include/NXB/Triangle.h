// NXB/Triangle.h - drop-in for NexusBVH/include/NXB/Triangle.h (36 B).
#pragma once

#include "AABB.h"

namespace NXB {

struct Triangle {
    Triangle() = default;
    NXB_HD Triangle(float3 a, float3 b, float3 c) : v0(a), v1(b), v2(c) {}
    NXB_HD AABB Bounds() const { return AABB(v0, v1, v2); }
    float3 v0, v1, v2;
};
static_assert(sizeof(Triangle) == 36, "NXB::Triangle layout");

}  // namespace NXB
