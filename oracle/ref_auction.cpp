// ref_auction.cpp - test infrastructure: the reference's own auction slot
// assignment compiled as host code, to pin the oracle's restatement.
//
// The reference's BVH8 kernel, built with USE_AUCTION, assigns child slots
// with AuctionAssignment (NexusBVH/src/Cuda/WideConverter.cu:50-102) over
// the cost table that its kernel fills (:337-361).  Both are plain float
// arithmetic.  oracle/build_ref.py copies those lines verbatim out of the
// reference's source into oracle/_ref/ (git-ignored; nothing of the
// reference is committed) and compiles them with this file, which supplies
// host stand-ins for the CUDA vector type and qualifiers they use.  The
// helpers GetNibble/SetNibble (BuilderUtils.h:368-377) are copied the same
// way.  Divisions are IEEE here (the GPU build uses the fast-math divide),
// as in the oracle, so the two must agree exactly.
#include <cfloat>
#include <cmath>
#include <cstdint>

#define __device__
#define __forceinline__ inline
#define INVALID_IDX (uint32_t)(-1)

struct float3 {
    float x, y, z;
};
inline float3 operator+(float3 a, float3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator-(float3 a, float3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator*(float3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
// the largest component (the float3 overload the cost table calls)
inline float fmaxf(float3 v) { return std::fmax(std::fmax(v.x, v.y), v.z); }
using std::fabs;
using std::fmaxf;

namespace NXB {
#include "_ref/auction_nibbles.inc"
#include "_ref/auction_functions.inc"
}  // namespace NXB

namespace {
struct AABB {
    float3 bMin, bMax;
};
struct Node {
    AABB bounds;
};
}  // namespace

// parent6: the parent's box (min xyz, max xyz); child6: childCount boxes.
// Returns the nibble-packed slot assignment (slot s -> child).
extern "C" uint32_t ref_auction(const float* parent6, const float* child6, uint32_t childCount) {
    using namespace NXB;
    Node bvh2Node{{{parent6[0], parent6[1], parent6[2]}, {parent6[3], parent6[4], parent6[5]}}};
    Node bvh2Nodes[8];
    uint32_t childNodes[8];
    for (uint32_t c = 0; c < childCount && c < 8; ++c) {
        const float* b = child6 + 6 * c;
        bvh2Nodes[c] = Node{{{b[0], b[1], b[2]}, {b[3], b[4], b[5]}}};
        childNodes[c] = c;
    }
    // from `float3 parentCentroid = ...` (WideConverter.cu:332) through the
    // USE_AUCTION branch's call of AuctionAssignment (:361)
#include "_ref/auction_cost_table.inc"
    return assignments;
}
