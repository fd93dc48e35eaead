// NXB/BuildConfig.h - drop-in for NexusBVH/include/NXB/BuildConfig.h.
#pragma once

#include <cstdint>

#include "BVHBuildMetrics.h"

namespace NXB {

struct BuildConfig {
    // true: 30-bit Morton codes in 32-bit keys (faster sort, lower quality);
    // false: 63-bit codes in 64-bit keys
    bool prioritizeSpeed = false;
    // H-PLOC search radius (4, 8 or 16); the reference fixes it at 8
    uint32_t searchRadius = 8;
    // BVH8 child slots by the auction algorithm (the reference's compile-time
    // USE_AUCTION) instead of the greedy assignment
    bool useAuction = false;
    // check the trees on the device before returning (BuildBVH2 / BuildBVH8
    // fail as on any other error when a tree is invalid)
    bool validate = false;
};

}  // namespace NXB
