// coherent_sort.cu -- stable (key, index) sort from the previous order (see
// coherent_sort.cuh).
#include "coherent_sort.cuh"

namespace sph {

namespace {

constexpr int kCoWarps = kCoThreads / 32;
constexpr uint32_t kMoverBlocks = 4 * 152;  // grid-stride blocks placing the movers
constexpr uint32_t kMoverSmallMax = 32768;   // up to this many movers: small sort tiles

inline uint32_t mover_plan_keys(uint32_t n) {  // sort plan size for both tile sizes
    const uint32_t few = n < kMoverSmallMax ? n : kMoverSmallMax;
    return n > 8 * few ? n : 8 * few;
}

// Mover flags of one tile of 2048 indices (bit = lane of a 32-index word) and
// the tile's mover count.  FROM_POS: the keys are the cell keys of pos[i],
// written to keys[i]; otherwise they are read from keys[i].
template <bool FROM_POS>
__global__ void __launch_bounds__(kCoThreads) coherent_flag_kernel(
    const float4* __restrict__ pos, GridParams g, uint32_t* __restrict__ keys, uint32_t n,
    const uint32_t* __restrict__ kprev, uint32_t* __restrict__ flags,
    uint32_t* __restrict__ toff) {
    __shared__ uint32_t s_cnt[kCoWarps];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t base = blockIdx.x * kCoTile;
    uint32_t cnt = 0;
#pragma unroll
    for (int it = 0; it < kCoItems; ++it) {
        const uint32_t i = base + it * kCoThreads + tid;
        bool mover = false;
        if (i < n) {
            uint32_t k;
            if (FROM_POS) {
                const float4 p = pos[i];
                k = cell_key(g, p.x, p.y, p.z);
                keys[i] = k;
            } else {
                k = keys[i];
            }
            mover = k != kprev[i];
        }
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, mover);
        const uint32_t w0 = base + it * kCoThreads + warp * 32;
        if (lane == 0 && w0 < n) flags[w0 >> 5] = b;
        cnt += __popc(b);
    }
    if (lane == 0) s_cnt[warp] = cnt;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kCoWarps; ++w) t += s_cnt[w];
        toff[blockIdx.x] = t;
    }
}

// Exclusive scan of the per-tile mover counts in place (one block);
// toff[tiles] = the number of movers.
__global__ void __launch_bounds__(1024) coherent_scan_kernel(uint32_t* __restrict__ toff,
                                                            uint32_t tiles) {
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_carry;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t b = 0; b < tiles; b += 1024) {
        const uint32_t i = b + tid;
        const uint32_t v = i < tiles ? toff[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_w[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t y = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t z = __shfl_up_sync(0xFFFFFFFFu, y, o);
                if (lane >= (uint32_t)o) y += z;
            }
            s_w[lane] = y;
        }
        __syncthreads();
        const uint32_t excl = s_carry + (warp ? s_w[warp - 1] : 0u) + x - v;
        if (i < tiles) toff[i] = excl;
        __syncthreads();
        if (tid == 1023) s_carry = excl + v;
        __syncthreads();
    }
    if (tid == 0) toff[tiles] = s_carry;
}

// Movers of one tile, in index order, to mk/mv at the tile's offset; movers
// before each flag word (wpre); digit histograms of the movers' keys.
__global__ void __launch_bounds__(kCoThreads) coherent_compact_kernel(
    const uint32_t* __restrict__ keys, uint32_t n, const uint32_t* __restrict__ flags,
    const uint32_t* __restrict__ toff, uint32_t* __restrict__ wpre, uint32_t* __restrict__ mk,
    uint32_t* __restrict__ mv, int passes, uint32_t* __restrict__ hist) {
    constexpr int kWords = kCoTile / 32;  // 64
    __shared__ uint32_t sh[kSortMaxPasses][256];
    __shared__ uint32_t s_flag[kWords], s_incl[kWords], s_ex[kWords];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < kSortMaxPasses * 256; i += kCoThreads) (&sh[0][0])[i] = 0;
    const uint32_t nwords = (n + 31) >> 5;
    const uint32_t w0 = blockIdx.x * kWords;
    if (tid < kWords) {
        const uint32_t w = w0 + tid;
        const uint32_t f = w < nwords ? flags[w] : 0u;
        s_flag[tid] = f;
        uint32_t x = __popc(f);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        s_incl[tid] = x;
    }
    __syncthreads();
    if (tid < kWords) {
        const uint32_t f = s_flag[tid];
        const uint32_t ex = toff[blockIdx.x] + (tid >= 32 ? s_incl[31] : 0u) + s_incl[tid] -
                            __popc(f);
        s_ex[tid] = ex;
        const uint32_t w = w0 + tid;
        if (w < nwords) wpre[w] = ex;
    }
    __syncthreads();
    const uint32_t base = blockIdx.x * kCoTile;
#pragma unroll
    for (int it = 0; it < kCoItems; ++it) {
        const uint32_t wl = it * kCoWarps + warp;
        const uint32_t f = s_flag[wl];
        if ((f >> lane) & 1u) {  // bits are set only below n
            const uint32_t i = base + it * kCoThreads + tid;
            const uint32_t p = s_ex[wl] + __popc(f & ((1u << lane) - 1u));
            const uint32_t k = keys[i];
            mk[p] = k;
            mv[p] = i;
            sort_hist_add(sh, k, passes);
        }
    }
    __syncthreads();
    for (int i = tid; i < passes * 256; i += kCoThreads) {
        const uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Movers with index below q (q <= n).
__device__ __forceinline__ uint32_t movers_below_index(const uint32_t* __restrict__ flags,
                                                       const uint32_t* __restrict__ wpre,
                                                       uint32_t q, uint32_t n, uint32_t m) {
    if (q >= n) return m;
    const uint32_t w = q >> 5;
    return wpre[w] + __popc(flags[w] & ((1u << (q & 31)) - 1u));
}

// Movers of the sorted mover list below (key, i), searched in [lo, hi).
__device__ __forceinline__ uint32_t movers_below_key(const uint32_t* __restrict__ smk,
                                                     const uint32_t* __restrict__ smv, uint32_t lo,
                                                     uint32_t hi, uint32_t key, uint32_t i) {
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t k = smk[mid];
        if (k < key || (k == key && smv[mid] < i))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Places every particle: blocks [0, kMoverBlocks) the sorted movers
// (grid-stride; first, so that their searches of kprev overlap the rest), the
// others one index per thread, which places it if it is a stayer.  Each writes
// its key and input index at the destination and, with out_a / out_b, its two
// float4 records (the step's positions and velocities in sorted order).  Every
// destination is range-checked (a sort that gave up on a bounded wait leaves
// garbage behind; the error word then already holds that failure).
__global__ void __launch_bounds__(256) coherent_merge_kernel(
    const uint32_t* __restrict__ kprev, uint32_t n, const uint32_t* __restrict__ flags,
    const uint32_t* __restrict__ wpre, const uint32_t* __restrict__ m_dev,
    const uint32_t* __restrict__ smk, const uint32_t* __restrict__ smv,
    const uint2* __restrict__ cells_prev, GridParams g, uint32_t* __restrict__ keys_out,
    uint32_t* __restrict__ perm_out, const float4* __restrict__ rec_a,
    const float4* __restrict__ rec_b, float4* __restrict__ out_a, float4* __restrict__ out_b,
    uint32_t* __restrict__ err) {
    const uint32_t m = min(*m_dev, n);
    if (blockIdx.x < kMoverBlocks) {
        const uint32_t stride = kMoverBlocks * 256;
        for (uint32_t r = blockIdx.x * 256 + threadIdx.x; r < m; r += stride) {
            const uint32_t k = smk[r], v = smv[r];
            // first index q with (kprev[q], q) >= (k, v).  The cell table of
            // the sort that wrote kprev usually holds the run of key k; any
            // table is accepted only where kprev confirms it (a run [s, e) of
            // key k with smaller keys before and larger after), else search.
            uint32_t lo = 0, hi = n;
            if (cells_prev) {
                const uint32_t c = morton_to_linear_checked(g, k);
                if (c != kEmptyCell) {
                    const uint2 se = cells_prev[c];
                    if (se.x < se.y && se.y <= n) {  // four independent loads
                        const uint32_t first = kprev[se.x], last = kprev[se.y - 1];
                        const uint32_t before = kprev[se.x ? se.x - 1 : 0];
                        const uint32_t after = kprev[se.y < n ? se.y : n - 1];
                        const bool run = first == k && last == k && (se.x == 0 || before < k) &&
                                         (se.y == n || after > k);
                        if (run) lo = hi = min(max(v, se.x), se.y);
                    }
                }
            }
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                const uint32_t kp = kprev[mid];
                if (kp < k || (kp == k && mid < v))
                    lo = mid + 1;
                else
                    hi = mid;
            }
            const uint32_t d = r + lo - movers_below_index(flags, wpre, lo, n, m);
            if (d >= n || v >= n) {
                atomicOr(err, 2u);
                continue;
            }
            keys_out[d] = k;
            perm_out[d] = v;
            if (out_a) {
                out_a[d] = rec_a[v];
                out_b[d] = rec_b[v];
            }
        }
        return;
    }
    const uint32_t i = (blockIdx.x - kMoverBlocks) * 256 + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    const bool valid = i < n;
    const uint32_t act = __ballot_sync(0xFFFFFFFFu, valid);
    if (act == 0u) return;
    const uint32_t key = valid ? kprev[i] : 0u;
    // The warp's (key, index) pairs increase with the lane.  lo = movers
    // below lane 0's pair, by a 32-way search (each lane tests one pivot);
    // usually no mover lies below the last lane's pair either, and every
    // lane's count is lo.
    const int last = 31 - __clz(act);
    const uint32_t k0 = __shfl_sync(0xFFFFFFFFu, key, 0);
    const uint32_t i0 = __shfl_sync(0xFFFFFFFFu, i, 0);
    uint32_t lo = 0, hi = m;  // answer in [lo, hi]
    while (hi - lo > 32) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t q = lo + lane * step;  // pivot of this lane (below hi for lane 0)
        bool below = false;
        if (q < hi) {
            const uint32_t kq = smk[q];
            below = kq < k0 || (kq == k0 && smv[q] < i0);
        }
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, below);  // a prefix of the lanes
        const uint32_t nb = __popc(b);
        if (nb == 0) {
            hi = lo;
        } else {
            const uint32_t nlo = lo + (nb - 1) * step + 1;
            hi = min(hi, lo + nb * step);
            lo = nlo;
        }
    }
    {  // the last <= 32 candidates: one per lane
        const uint32_t q = lo + lane;
        bool below = false;
        if (q < hi) {
            const uint32_t kq = smk[q];
            below = kq < k0 || (kq == k0 && smv[q] < i0);
        }
        lo += __popc(__ballot_sync(0xFFFFFFFFu, below));
    }
    const uint32_t kl = __shfl_sync(0xFFFFFFFFu, key, last);
    const uint32_t il = __shfl_sync(0xFFFFFFFFu, i, last);
    bool inside = false;  // a mover between lane 0's and the last lane's pairs
    if (lo < m) {
        const uint32_t kq = smk[lo];
        inside = kq < kl || (kq == kl && smv[lo] < il);
    }
    if (!valid) return;
    const uint32_t f = flags[i >> 5];
    if ((f >> lane) & 1u) return;  // a mover, placed above
    const uint32_t below = inside ? movers_below_key(smk, smv, lo, m, key, i) : lo;
    const uint32_t d = i - (wpre[i >> 5] + __popc(f & ((1u << lane) - 1u))) + below;
    if (d >= n) {
        atomicOr(err, 2u);
        return;
    }
    keys_out[d] = key;
    perm_out[d] = i;
    if (out_a) {
        out_a[d] = rec_a[i];
        out_b[d] = rec_b[i];
    }
}

// Cell ranges of the sorted keys (as gather_cells_kernel) and the keys
// themselves as the next sort's kprev.
constexpr uint32_t kCellsThreads = 256;

__global__ void __launch_bounds__(kCellsThreads) coherent_cells_kernel(
    const uint32_t* __restrict__ keys, uint32_t n, GridParams g, uint2* __restrict__ cells,
    uint32_t* __restrict__ kprev, uint32_t* __restrict__ err, NearList near) {
    // After a look-back timeout earlier in this sort (err bit 1, set only by
    // previous kernels, so every block sees the same value) the keys are not
    // sorted; 0xFFFFFFFF everywhere keeps kprev non-decreasing and makes every
    // particle a mover in the next step, which then sorts from scratch.  One
    // thread per block reads the word: a read per thread put ~65,000 requests
    // for one address on one L2 slice at 2M particles.
    __shared__ uint32_t s_failed, s_base, s_warp[kCellsThreads / 32];
    if (threadIdx.x == 0) s_failed = *(volatile const uint32_t*)err & 1u;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const uint32_t key = valid ? keys[i] : 0u;
    if (valid) kprev[i] = s_failed ? 0xFFFFFFFFu : key;
    uint32_t* cw = reinterpret_cast<uint32_t*>(cells);
    const uint32_t c = valid ? morton_to_linear_checked(g, key) : kEmptyCell;
    if (near.list) {  // near_append with one atomic per block instead of per warp
        const bool want = c != kEmptyCell && near.bnear[c] != 0;
        if (near.flag && valid) near.flag[i] = want ? 1 : 0;
        const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, want);
        if (lane == 0) s_warp[warp] = __popc(b);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (uint32_t w = 0; w < kCellsThreads / 32; ++w) {
                const uint32_t cnt = s_warp[w];
                s_warp[w] = t;
                t += cnt;
            }
            s_base = t ? atomicAdd(near.count, t) : 0u;
        }
        __syncthreads();
        if (want) near.list[s_base + s_warp[warp] + __popc(b & ((1u << lane) - 1u))] = i;
    }
    if (!valid) return;
    if (c == kEmptyCell) {
        atomicOr(err, 2u);
        return;
    }
    const uint32_t prev = i > 0 ? keys[i - 1] : 0u;
    if (i == 0 || prev != key) {
        cw[2 * c] = i;
        if (i > 0) {
            const uint32_t cp = morton_to_linear_checked(g, prev);
            if (cp != kEmptyCell) cw[2 * cp + 1] = i;
        }
    }
    if (i == n - 1) cw[2 * c + 1] = n;
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

void coherent_run(const CoherentSort& c, const float4* pos, const GridParams* g,
                  const uint2* cells_prev, uint32_t* keys, int key_bits, uint32_t* keys_out,
                  uint32_t* perm_out, const float4* rec_a, const float4* rec_b, float4* out_a,
                  float4* out_b, uint32_t* err, int force_timeout, cudaStream_t st) {
    const SortScratch& s = c.sort;
    const uint32_t n = c.n;
    if (n == 0) return;
    const uint32_t tiles = coherent_tiles(n);
    const int passes = sort_passes(key_bits);
    sort_reset(s, st);
    if (pos)
        coherent_flag_kernel<true><<<tiles, kCoThreads, 0, st>>>(pos, *g, keys, n, c.kprev,
                                                                 c.flags, c.toff);
    else
        coherent_flag_kernel<false><<<tiles, kCoThreads, 0, st>>>(nullptr, GridParams{}, keys, n,
                                                                  c.kprev, c.flags, c.toff);
    coherent_scan_kernel<<<1, 1024, 0, st>>>(c.toff, tiles);
    coherent_compact_kernel<<<tiles, kCoThreads, 0, st>>>(keys, n, c.flags, c.toff, c.wpre,
                                                          c.mk[0], c.mv[0], passes, s.hist);
    sort_scan(passes, s, st);
    uint32_t* mk[2] = {c.mk[0], c.mk[1]};
    uint32_t* mv[2] = {c.mv[0], c.mv[1]};
    const int o = sort_passes_run_dev(mk, mv, c.mv[0], n, c.toff + tiles, kMoverSmallMax, passes,
                                      s, err, force_timeout, st);
    const uint32_t stay_blocks = (n + 255) / 256;
    coherent_merge_kernel<<<kMoverBlocks + stay_blocks, 256, 0, st>>>(
        c.kprev, n, c.flags, c.wpre, c.toff + tiles, mk[o], mv[o], cells_prev,
        g ? *g : GridParams{}, keys_out, perm_out, rec_a, rec_b, out_a, out_b, err);
}

}  // namespace

size_t coherent_bytes(uint32_t n) {
    const size_t words = (n + 31) / 32 + 1, tiles = coherent_tiles(n) + 1, nn = n ? n : 1;
    return align256(4 * nn) + 2 * align256(4 * words) + align256(4 * tiles) +
           4 * align256(4 * nn) + align256(sort_scratch_bytes(mover_plan_keys(n)));
}

CoherentSort coherent_from(void* base, uint32_t n) {
    const size_t words = (n + 31) / 32 + 1, tiles = coherent_tiles(n) + 1, nn = n ? n : 1;
    char* p = (char*)base;
    CoherentSort c;
    c.n = n;
    c.kprev = (uint32_t*)p;
    p += align256(4 * nn);
    c.flags = (uint32_t*)p;
    p += align256(4 * words);
    c.wpre = (uint32_t*)p;
    p += align256(4 * words);
    c.toff = (uint32_t*)p;
    p += align256(4 * tiles);
    for (int b = 0; b < 2; ++b) {
        c.mk[b] = (uint32_t*)p;
        p += align256(4 * nn);
        c.mv[b] = (uint32_t*)p;
        p += align256(4 * nn);
    }
    c.sort = sort_scratch_from(p, mover_plan_keys(n));
    return c;
}

void coherent_reset(const CoherentSort& c, cudaStream_t st) {
    if (c.n) cudaMemsetAsync(c.kprev, 0xFF, 4 * (size_t)c.n, st);
}

void coherent_sort_cells(const CoherentSort& c, const float4* pos, const float4* vel,
                         const GridParams& g, uint2* cells, int key_bits, uint32_t* keys,
                         uint32_t* keys_out, uint32_t* perm_out, float4* pos_out, float4* vel_out,
                         uint32_t* err, int force_timeout, cudaStream_t st, NearList near) {
    coherent_run(c, pos, &g, cells, keys, key_bits, keys_out, perm_out, pos, vel, pos_out, vel_out,
                 err, force_timeout, st);
    if (c.n == 0) return;
    cudaMemsetAsync(cells, 0xFF, sizeof(uint2) * (size_t)g.dx * g.dy * g.dz, st);
    coherent_cells_kernel<<<(c.n + kCellsThreads - 1) / kCellsThreads, kCellsThreads, 0, st>>>(
        keys_out, c.n, g, cells, c.kprev, err, near);
}

void coherent_sort_keys(const CoherentSort& c, const uint32_t* keys, int key_bits,
                        uint32_t* keys_out, uint32_t* perm_out, uint32_t* err, int force_timeout,
                        cudaStream_t st) {
    coherent_run(c, nullptr, nullptr, nullptr, const_cast<uint32_t*>(keys), key_bits, keys_out,
                 perm_out, nullptr, nullptr, nullptr, nullptr, err, force_timeout, st);
}

}  // namespace sph
