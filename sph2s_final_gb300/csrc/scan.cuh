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

// Scratch (uint32 count) of one scanned array of up to max_n elements.
inline size_t scan_scratch_words(uint32_t max_n) {
    return (size_t)(max_n + kScanTile - 1) / kScanTile + 1;
}

// Up to kScanMaxSegs independent exclusive scans in three launches: segment k
// computes seg[k].out[i] = sum_{j<i} seg[k].in[j] over its n elements (out may
// alias in) and writes the sum of all of them to *seg[k].total (device).
// Scratch: the sum of scan_scratch_words(seg[k].n) over the segments.
constexpr int kScanMaxSegs = 4;
struct ScanSeg {
    const uint32_t* in;
    uint32_t* out;
    uint32_t n;
    uint32_t* total;
};
void scan_exclusive_batch(const ScanSeg* segs, int count, uint32_t* scratch, cudaStream_t st);

}  // namespace sph
