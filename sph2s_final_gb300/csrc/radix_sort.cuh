// radix_sort.cuh -- hand-written onesweep LSD radix sort of (uint32 key,
// uint32 value) pairs, replacing thrust::sort_by_key on the step path
// (SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1110-1115, boundary once at 1022-1027).
//
// Algorithm (Adinets & Merrill, "Onesweep", 2022): one upfront pass computes
// the digit histograms of every 8-bit digit pass; then each digit pass is a
// single kernel in which every CTA ranks one tile of keys, publishes its
// per-digit counts, and obtains its global offsets by decoupled look-back over
// the preceding tiles.  Tiles are handed out by an atomic counter, so a tile
// only ever waits on tiles that were handed out earlier and are therefore
// resident or finished; every wait is additionally bounded and records
// SPH_E_TIMEOUT in an error word instead of spinning forever.
//
// The sort is stable: within a tile, items are ranked in input order (warp-
// striped loads, match_any ranking by lane), tiles are ordered by index.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sph {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys
// Device-counted sorts of at most small_max keys use tiles of 512 keys: twice
// the tiles run in parallel per 1,024 keys and each tile's chain is 8x shorter.
constexpr int kSortItemsSmall = 2;
constexpr int kSortTileSmall = kSortThreads * kSortItemsSmall;
constexpr int kSortMaxPasses = 4;

// Device scratch of one sort plan.  Everything that must start at zero lives
// in one contiguous block so a single memset resets it.
struct SortScratch {
    uint32_t* hist;      // [kSortMaxPasses][256] histograms, then exclusive offsets
    uint32_t* tile_ctr;  // [kSortMaxPasses]
    uint32_t* status;    // [kSortMaxPasses][max_tiles][256] look-back words
    uint32_t max_tiles;
    size_t zero_bytes;   // bytes from hist through status
};

constexpr size_t sort_align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of scratch a plan for up to max_n keys needs (a constant expression, so
// fixed-size scratch regions can be checked at build time).
constexpr size_t sort_scratch_bytes(uint32_t max_n) {
    return sort_align256(kSortMaxPasses * 256 * 4) + sort_align256(kSortMaxPasses * 4) +
           sort_align256((size_t)kSortMaxPasses *
                         (max_n == 0 ? 1u : (max_n + kSortTile - 1) / kSortTile) * 256 * 4);
}
// Carves a SortScratch out of a caller-provided device block of
// sort_scratch_bytes(max_n) bytes (256-byte aligned).
SortScratch sort_scratch_from(void* base, uint32_t max_n);

// Number of 8-bit digit passes for keys of `key_bits` significant bits.
inline int sort_passes(int key_bits) {
    int p = (key_bits + 7) / 8;
    return p < 1 ? 1 : p;
}

// Enqueues the histogram-independent part of a sort: clears the scratch.
void sort_reset(const SortScratch& s, cudaStream_t st);

// Histograms of all passes for keys already in memory (the step fuses this
// into the hash kernel instead).
void sort_histogram(const uint32_t* keys, uint32_t n, int passes, const SortScratch& s,
                    cudaStream_t st);

// Turns the histograms into exclusive digit offsets (in place).
void sort_scan(int passes, const SortScratch& s, cudaStream_t st);

// Runs the digit passes.  keys[0] holds the input keys and first_vals the
// input values (NULL: the values are the input indices 0..n-1, generated in
// the first pass); keys[1]/vals[1] and vals[0] are ping-pong buffers.  Returns
// the index (0 or 1) of the buffers that hold the sorted output.  `err` is a
// device word that receives kErrLookbackTimeout on a look-back timeout;
// `force_timeout` makes every look-back give up (test hook).
int sort_passes_run(uint32_t* keys[2], uint32_t* vals[2], const uint32_t* first_vals, uint32_t n,
                    int passes, const SortScratch& s, uint32_t* err, int force_timeout,
                    cudaStream_t st);

// sort_passes_run for a key count that only the device knows: each pass sorts
// m = min(*n_dev, n) keys, in tiles of kSortTileSmall keys when m <= small_max
// and of kSortTile keys otherwise; the grid covers both cases and tiles
// beyond m exit at once.  The plan's status area must hold
// max(tiles of n, small tiles of min(n, small_max)) tiles per pass
// (sort_scratch_bytes(max(n, 8 * min(n, small_max)))).
int sort_passes_run_dev(uint32_t* keys[2], uint32_t* vals[2], const uint32_t* first_vals,
                        uint32_t n, const uint32_t* n_dev, uint32_t small_max, int passes,
                        const SortScratch& s, uint32_t* err, int force_timeout, cudaStream_t st);

// One digit pass p (bits 8p..8p+7) from explicit input to output buffers
// (vals_in NULL: values are the input indices).  Needs the histograms of
// sort_histogram + sort_scan in `s`.
void sort_pass(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
               uint32_t* vals_out, uint32_t n, int p, const SortScratch& s, uint32_t* err,
               int force_timeout, cudaStream_t st);

// Convenience: reset + histogram + scan + passes.
int sort_pairs(uint32_t* keys[2], uint32_t* vals[2], uint32_t n, int key_bits,
               const SortScratch& s, uint32_t* err, int force_timeout, cudaStream_t st);

// Device helper for fused producers: adds `key` to the shared histograms
// sh[pass][digit] of `passes` passes.
__device__ __forceinline__ void sort_hist_add(uint32_t (*sh)[256], uint32_t key, int passes) {
    for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(key >> (8 * p)) & 255u], 1u);
}

}  // namespace sph
