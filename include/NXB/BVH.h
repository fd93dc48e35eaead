// NXB/BVH.h - drop-in for NexusBVH/include/NXB/BVH.h: the BVH2 (32-byte
// nodes) and compressed BVH8 (80-byte nodes) layouts.
#pragma once

#include <cstdint>

#include "AABB.h"

#ifndef INVALID_IDX
#define INVALID_IDX (uint32_t)(-1)
#endif

namespace NXB {

enum struct PrimType : unsigned char { AABB, TRIANGLE };

struct BVH2 {
    struct Node {
        AABB bounds;
        uint32_t leftChild;   // INVALID_IDX for a leaf
        uint32_t rightChild;  // primitive index for a leaf
    };
    Node* nodes;
    uint32_t nodeCount;
    uint32_t primCount;
    AABB bounds;
};

struct BVH8 {
    // the 80-byte node spelled out field by field
    struct NodeExplicit {
        float3 p;
        uint8_t e[3];
        uint8_t imask = 0;
        uint32_t childBaseIdx = 0;
        uint32_t primBaseIdx = 0;
        uint8_t meta[8];
        uint8_t qlox[8], qloy[8], qloz[8];
        uint8_t qhix[8], qhiy[8], qhiz[8];
    };
    // the same 80 bytes as five 16-byte vectors
    struct Node {
        float4 p_e_imask;
        float4 childidx_tridx_meta;
        float4 qlox_qloy;
        float4 qloz_qhix;
        float4 qhiy_qhiz;
    };
    Node* nodes;
    uint32_t nodeCount;
    uint32_t* primIdx;
    uint32_t primCount;
    AABB bounds;
};

static_assert(sizeof(BVH2::Node) == 32 && sizeof(BVH8::Node) == 80 && sizeof(BVH8::NodeExplicit) == 80,
              "node layouts");
static_assert(sizeof(BVH2) == 40 && sizeof(BVH8) == 56, "BVH layouts");

}  // namespace NXB
