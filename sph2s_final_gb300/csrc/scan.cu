// scan.cu -- reduce-then-scan exclusive prefix sum (see scan.cuh).
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

__global__ void __launch_bounds__(kScanThreads) tile_sums_kernel(const uint32_t* __restrict__ in,
                                                                 uint32_t n,
                                                                 uint32_t* __restrict__ sums) {
    __shared__ uint32_t s_warp[33];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) t += in[base + k];
    uint32_t tot;
    block_excl_scan(t, s_warp, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Exclusive scan of the tile sums in place (one block, any count up to
// kScanThreads * 64), total written to sums[count] and *total.
__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(uint32_t* sums, uint32_t count,
                                                                 uint32_t* total) {
    __shared__ uint32_t s_warp[33];
    uint32_t carry = 0;
    for (uint32_t b = 0; b < count; b += kScanThreads) {
        const uint32_t i = b + threadIdx.x;
        const uint32_t v = i < count ? sums[i] : 0u;
        uint32_t tot;
        const uint32_t e = block_excl_scan(v, s_warp, &tot);
        if (i < count) sums[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        sums[count] = carry;
        if (total) *total = carry;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(const uint32_t* in,
                                                                  uint32_t* out, uint32_t n,
                                                                  const uint32_t* __restrict__ sums) {
    __shared__ uint32_t s_warp[33];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? in[base + k] : 0u;
        t += v[k];
    }
    uint32_t tot;
    uint32_t run = sums[blockIdx.x] + block_excl_scan(t, s_warp, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) {
            out[base + k] = run;
            run += v[k];
        }
}

}  // namespace

void scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                    uint32_t* total, cudaStream_t st) {
    if (n == 0) {
        if (total) cudaMemsetAsync(total, 0, 4, st);
        return;
    }
    const uint32_t tiles = (n + kScanTile - 1) / kScanTile;
    tile_sums_kernel<<<tiles, kScanThreads, 0, st>>>(in, n, scratch);
    scan_sums_kernel<<<1, kScanThreads, 0, st>>>(scratch, tiles, total);
    scan_tiles_kernel<<<tiles, kScanThreads, 0, st>>>(in, out, n, scratch);
}

}  // namespace sph
