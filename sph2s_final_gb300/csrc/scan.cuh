// scan.cuh -- device-wide exclusive prefix sum of uint32 flags/counts, the
// building block of the two-scale step's stream compaction (it replaces the
// reference's atomicAdd re-listing, SPH2S_FINAL_TWO_SCALE/Solver.cu:566,
// 1287-1288, whose output order is not deterministic).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sph {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;  // 1024 elements per block

// Scratch (uint32 count) for scanning up to max_n elements.
inline size_t scan_scratch_words(uint32_t max_n) {
    return (size_t)(max_n + kScanTile - 1) / kScanTile + 1;
}

// out[i] = sum_{k<i} in[i]; out may alias in.  `total` (device, nullable)
// receives the sum of all n elements.  Up to kScanTile^2 (1M) * kScanTile
// elements.
void scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                    uint32_t* total, cudaStream_t st);

}  // namespace sph
