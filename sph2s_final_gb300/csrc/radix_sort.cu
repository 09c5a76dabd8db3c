// radix_sort.cu -- onesweep LSD radix sort (see radix_sort.cuh).
#include "radix_sort.cuh"
#include "errors.h"

namespace sph {

namespace {

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPfx = 2u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1u;
constexpr int kWarps = kSortThreads / 32;
// Bounded look-back: about 0.1 s of polling with nanosleep back-off before a
// tile gives up (a predecessor that is resident never needs that long).
constexpr int kSpinLimit = 1 << 20;
constexpr int kSpinLimitForced = 64;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wpre = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w)
        if (w < warp) wpre += s_warp[w];
    __syncthreads();
    return wpre + x - v;
}

__global__ void __launch_bounds__(256) histogram_kernel(const uint32_t* __restrict__ keys,
                                                        uint32_t n, int passes,
                                                        uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    for (int i = threadIdx.x; i < kSortMaxPasses * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        sort_hist_add(sh, keys[i], passes);
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

__global__ void __launch_bounds__(256) scan_kernel(uint32_t* hist, int passes) {
    __shared__ uint32_t s_warp[kWarps];
    for (int p = 0; p < passes; ++p) {
        uint32_t v = hist[p * 256 + threadIdx.x];
        uint32_t e = block_exclusive_scan(v, s_warp);
        hist[p * 256 + threadIdx.x] = e;
    }
}

__global__ void __launch_bounds__(kSortThreads) onesweep_kernel(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n,
    const uint32_t* __restrict__ n_dev, uint32_t small_max, int shift,
    const uint32_t* __restrict__ digit_offsets, uint32_t* status, uint32_t* tile_ctr,
    uint32_t* err, int force_timeout) {
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    __shared__ uint32_t s_whist[kWarps][257];  // column 256 collects out-of-range items
    __shared__ uint32_t s_local_start[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_warp[kWarps];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int ni = kSortItems;  // keys per thread
    if (n_dev) {  // key count known on the device only: the grid covers n keys
        n = min(*n_dev, n);
        if (n == 0) return;
        if (n <= small_max) ni = kSortItemsSmall;  // few keys: more, smaller tiles
    }
    const uint32_t tile_keys = (uint32_t)ni * kSortThreads;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int i = tid; i < kWarps * 257; i += kSortThreads) (&s_whist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * tile_keys;
    if (base >= n) return;  // tiles are handed out in order: no later tile waits on this one
    const uint32_t seg = base + (uint32_t)warp * ((uint32_t)ni * 32);

    uint32_t k[kSortItems], v[kSortItems], rank[kSortItems];
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = seg + i * 32 + lane;
        bool ok = i < ni && idx < n;
        k[i] = ok ? keys_in[idx] : 0xFFFFFFFFu;
        v[i] = ok ? (vals_in ? vals_in[idx] : idx) : 0u;
    }

    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        if (i >= ni) break;
        uint32_t idx = seg + i * 32 + lane;
        uint32_t d = idx < n ? ((k[i] >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        int leader = 31 - __clz(peers);
        uint32_t b = s_whist[warp][d];
        rank[i] = b + __popc(peers & lt);
        __syncwarp();
        if (lane == leader) s_whist[warp][d] = b + __popc(peers);
        __syncwarp();
    }
    __syncthreads();

    // Thread t owns digit t: exclusive offsets across warps and the tile total.
    uint32_t total = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        uint32_t c = s_whist[w][tid];
        s_whist[w][tid] = total;
        total += c;
    }
    uint32_t* my_status = status + (size_t)tile * 256 + tid;
    st_relaxed(my_status, (tile == 0 ? kFlagPfx : kFlagAgg) | total);

    uint32_t local_start = block_exclusive_scan(total, s_warp);
    s_local_start[tid] = local_start;

    uint32_t prefix = 0;
    if (tile > 0) {
        int pred = (int)tile - 1;
        int spins = 0;
        const int limit = force_timeout ? kSpinLimitForced : kSpinLimit;
        while (pred >= 0) {
            uint32_t sv = force_timeout ? 0u : ld_relaxed(status + (size_t)pred * 256 + tid);
            uint32_t flag = sv & ~kValMask;
            if (flag == 0u) {
                if (++spins > limit) {
                    atomicOr(err, 1u);
                    break;
                }
                __nanosleep(64);
                continue;
            }
            prefix += sv & kValMask;
            if (flag == kFlagPfx) break;
            --pred;
        }
        st_relaxed(my_status, kFlagPfx | ((prefix + total) & kValMask));
    }
    s_gbase[tid] = digit_offsets[tid] + prefix - local_start;
    __syncthreads();

#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = seg + i * 32 + lane;
        if (i < ni && idx < n) {
            uint32_t d = (k[i] >> shift) & 255u;
            uint32_t pos = s_local_start[d] + s_whist[warp][d] + rank[i];
            s_keys[pos] = k[i];
            s_vals[pos] = v[i];
        }
    }
    __syncthreads();

    const uint32_t tile_n = (n - base) < tile_keys ? (n - base) : tile_keys;
    for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
        uint32_t key = s_keys[i];
        uint32_t g = s_gbase[(key >> shift) & 255u] + i;
        keys_out[g] = key;
        vals_out[g] = s_vals[i];
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

SortScratch sort_scratch_from(void* base, uint32_t max_n) {
    SortScratch s;
    uint32_t tiles = (max_n + kSortTile - 1) / kSortTile;
    if (tiles == 0) tiles = 1;
    char* p = (char*)base;
    s.hist = (uint32_t*)p;
    p += align256(kSortMaxPasses * 256 * 4);
    s.tile_ctr = (uint32_t*)p;
    p += align256(kSortMaxPasses * 4);
    s.status = (uint32_t*)p;
    p += align256((size_t)kSortMaxPasses * tiles * 256 * 4);
    s.max_tiles = tiles;
    s.zero_bytes = (size_t)(p - (char*)base);
    return s;
}

void sort_reset(const SortScratch& s, cudaStream_t st) {
    cudaMemsetAsync(s.hist, 0, s.zero_bytes, st);
}

void sort_histogram(const uint32_t* keys, uint32_t n, int passes, const SortScratch& s,
                    cudaStream_t st) {
    if (n == 0) return;
    uint32_t blocks = (n + 255) / 256;
    if (blocks > 152 * 4) blocks = 152 * 4;
    histogram_kernel<<<blocks, 256, 0, st>>>(keys, n, passes, s.hist);
}

void sort_scan(int passes, const SortScratch& s, cudaStream_t st) {
    scan_kernel<<<1, 256, 0, st>>>(s.hist, passes);
}

void sort_pass(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
               uint32_t* vals_out, uint32_t n, int p, const SortScratch& s, uint32_t* err,
               int force_timeout, cudaStream_t st) {
    if (n == 0) return;
    uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    onesweep_kernel<<<tiles, kSortThreads, 0, st>>>(
        keys_in, vals_in, keys_out, vals_out, n, nullptr, 0u, 8 * p, s.hist + p * 256,
        s.status + (size_t)p * s.max_tiles * 256, s.tile_ctr + p, err, force_timeout);
}

int sort_passes_run_dev(uint32_t* keys[2], uint32_t* vals[2], const uint32_t* first_vals,
                        uint32_t n, const uint32_t* n_dev, uint32_t small_max, int passes,
                        const SortScratch& s, uint32_t* err, int force_timeout, cudaStream_t st) {
    if (n == 0) return 0;
    uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    if (n_dev) {
        const uint32_t few = n < small_max ? n : small_max;
        const uint32_t small_tiles = (few + kSortTileSmall - 1) / kSortTileSmall;
        if (small_tiles > tiles) tiles = small_tiles;
    }
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        const uint32_t* vin = (p == 0) ? first_vals : vals[cur];
        onesweep_kernel<<<tiles, kSortThreads, 0, st>>>(
            keys[cur], vin, keys[cur ^ 1], vals[cur ^ 1], n, n_dev, small_max, 8 * p, s.hist + p * 256,
            s.status + (size_t)p * s.max_tiles * 256, s.tile_ctr + p, err, force_timeout);
        cur ^= 1;
    }
    return cur;
}

int sort_passes_run(uint32_t* keys[2], uint32_t* vals[2], const uint32_t* first_vals, uint32_t n,
                    int passes, const SortScratch& s, uint32_t* err, int force_timeout,
                    cudaStream_t st) {
    return sort_passes_run_dev(keys, vals, first_vals, n, nullptr, 0u, passes, s, err,
                               force_timeout, st);
}

int sort_pairs(uint32_t* keys[2], uint32_t* vals[2], uint32_t n, int key_bits,
               const SortScratch& s, uint32_t* err, int force_timeout, cudaStream_t st) {
    int passes = sort_passes(key_bits);
    sort_reset(s, st);
    sort_histogram(keys[0], n, passes, s, st);
    sort_scan(passes, s, st);
    return sort_passes_run(keys, vals, vals[0], n, passes, s, err, force_timeout, st);
}

}  // namespace sph
