// scan.cu -- reduce-then-scan exclusive prefix sums, several arrays per launch (see scan.cuh).
#include "scan.cuh"

namespace sph {

namespace {

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// Exclusive scan of one value per thread across the block; *block_total gets the sum.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_warp,
                                                    uint32_t* block_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = warp_incl_scan(v);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
        uint32_t wi = warp_incl_scan(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    uint32_t r = s_warp[warp] + incl - v;
    *block_total = s_warp[32];
    __syncthreads();
    return r;
}

// ---- batched form: segment k owns tiles [tile0[k], tile0[k + 1]) and tile
// sums scratch[sums0[k] ...] (tiles + 1 words) ----
struct ScanBatch {
    ScanSeg seg[kScanMaxSegs];
    uint32_t tile0[kScanMaxSegs + 1];
    uint32_t sums0[kScanMaxSegs];
    int count;
};

__device__ __forceinline__ int batch_segment(const ScanBatch& b, uint32_t tile) {
    int k = 0;
    while (k + 1 < b.count && tile >= b.tile0[k + 1]) ++k;
    return k;
}

__global__ void __launch_bounds__(kScanThreads) tile_sums_batch_kernel(ScanBatch b,
                                                                       uint32_t* __restrict__ scratch) {
    __shared__ uint32_t s_warp[33];
    const int k = batch_segment(b, blockIdx.x);
    const uint32_t tile = blockIdx.x - b.tile0[k];
    const uint32_t* __restrict__ in = b.seg[k].in;
    const uint32_t n = b.seg[k].n;
    const uint32_t base = tile * kScanTile + threadIdx.x * kScanItems;
    uint32_t t = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q)
        if (base + q < n) t += in[base + q];
    uint32_t tot;
    block_excl_scan(t, s_warp, &tot);
    if (threadIdx.x == 0) scratch[b.sums0[k] + tile] = tot;
}

// One block per segment: its tile sums, scanned in place, and its total.
__global__ void __launch_bounds__(kScanThreads) scan_sums_batch_kernel(ScanBatch b,
                                                                       uint32_t* scratch) {
    __shared__ uint32_t s_warp[33];
    const int k = blockIdx.x;
    uint32_t* sums = scratch + b.sums0[k];
    const uint32_t count = b.tile0[k + 1] - b.tile0[k];
    uint32_t carry = 0;
    for (uint32_t q = 0; q < count; q += kScanThreads) {
        const uint32_t i = q + threadIdx.x;
        const uint32_t v = i < count ? sums[i] : 0u;
        uint32_t tot;
        const uint32_t e = block_excl_scan(v, s_warp, &tot);
        if (i < count) sums[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        sums[count] = carry;
        *b.seg[k].total = carry;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles_batch_kernel(
    ScanBatch b, const uint32_t* __restrict__ scratch) {
    __shared__ uint32_t s_warp[33];
    const int k = batch_segment(b, blockIdx.x);
    const uint32_t tile = blockIdx.x - b.tile0[k];
    const uint32_t* in = b.seg[k].in;
    uint32_t* out = b.seg[k].out;
    const uint32_t n = b.seg[k].n;
    const uint32_t base = tile * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t t = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        v[q] = base + q < n ? in[base + q] : 0u;
        t += v[q];
    }
    uint32_t tot;
    uint32_t run = scratch[b.sums0[k] + tile] + block_excl_scan(t, s_warp, &tot);
#pragma unroll
    for (int q = 0; q < kScanItems; ++q)
        if (base + q < n) {
            out[base + q] = run;
            run += v[q];
        }
}

}  // namespace

void scan_exclusive_batch(const ScanSeg* segs, int count, uint32_t* scratch, cudaStream_t st) {
    if (count <= 0) return;
    ScanBatch b;
    b.count = count < kScanMaxSegs ? count : kScanMaxSegs;
    uint32_t tiles = 0, words = 0;
    for (int k = 0; k < b.count; ++k) {
        b.seg[k] = segs[k];
        b.tile0[k] = tiles;
        b.sums0[k] = words;
        const uint32_t t = (segs[k].n + kScanTile - 1) / kScanTile;
        tiles += t;
        words += t + 1;
    }
    b.tile0[b.count] = tiles;
    if (tiles) tile_sums_batch_kernel<<<tiles, kScanThreads, 0, st>>>(b, scratch);
    scan_sums_batch_kernel<<<b.count, kScanThreads, 0, st>>>(b, scratch);
    if (tiles) scan_tiles_batch_kernel<<<tiles, kScanThreads, 0, st>>>(b, scratch);
}

}  // namespace sph
