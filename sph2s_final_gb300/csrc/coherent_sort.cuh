// coherent_sort.cuh -- the step's stable sort of (cell key, index) pairs,
// computed from the order the particles are already in.
//
// The reference sorts every step from scratch (thrust::sort_by_key of the
// hashes and indices, SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1110-1115).  Between
// two steps a particle moves a small fraction of a cell, so almost every
// particle keeps its cell and the array is still sorted apart from the few
// that crossed a cell face.  With a non-decreasing array `kprev` of the same
// length (the previous step's sorted keys; any non-decreasing array is valid,
// 0xFFFFFFFF everywhere at creation):
//
//   stayers  i with key[i] == kprev[i]: their keys are non-decreasing in i,
//            so they are already in (key, index) order;
//   movers   all others: compacted in index order and sorted by the onesweep
//            radix sort (stable: ties stay in index order; tiles of 512 keys
//            while they are few);
//   merge    each stayer lands at (stayers before it) + (movers below it),
//            each mover at (its rank among movers) + (stayers below it), both
//            counted by binary search in (key, index) order.
//
// The output is the stable sort of (key, index) -- identical to a full sort
// for every input, however many particles moved; only the cost depends on
// how many did (all of them at the first step after creation).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "common.cuh"
#include "radix_sort.cuh"

namespace sph {

constexpr int kCoThreads = 256;
constexpr int kCoItems = 8;
constexpr uint32_t kCoTile = kCoThreads * kCoItems;  // 2048 indices = 64 mover-flag words

struct CoherentSort {
    uint32_t n = 0;
    uint32_t* kprev = nullptr;  // [n] non-decreasing: the last step's sorted keys
    uint32_t* flags = nullptr;  // [n/32] mover bit per index
    uint32_t* wpre = nullptr;   // [n/32] movers before each flag word
    uint32_t* toff = nullptr;   // [tiles + 1] movers per tile -> exclusive offsets; [tiles] = total
    uint32_t* mk[2] = {nullptr, nullptr};  // mover keys, radix-sort ping-pong
    uint32_t* mv[2] = {nullptr, nullptr};  // mover indices
    SortScratch sort;                       // the movers' radix-sort plan
};

inline uint32_t coherent_tiles(uint32_t n) { return (n + kCoTile - 1) / kCoTile; }

// Device bytes of the scratch for n keys, and the carving of a block of that
// size (256-byte aligned).
size_t coherent_bytes(uint32_t n);
CoherentSort coherent_from(void* base, uint32_t n);

// Sets kprev to 0xFFFFFFFF (no particle is a stayer at the next sort).
void coherent_reset(const CoherentSort& c, cudaStream_t st);

// Enqueues the step's neighbourhood build from the cell keys of pos[0..n):
// writes the keys in the current order to `keys`, the sorted keys and the
// permutation (sorted position -> index) to keys_out / perm_out, pos and vel
// in sorted order to pos_out / vel_out, the cell table of g (start, end per
// linear cell) to `cells`, and the sorted keys to kprev for the next call.
// `cells` is read first: if it is the table of the last call (the one built
// with kprev), placing the particles that changed cell is a lookup; every
// entry is checked against kprev before use, so a stale or garbage table is
// safe.  With near.list, the sorted indices of the particles whose cell is
// flagged in near.bnear are appended to it (near.count zeroed beforehand).
void coherent_sort_cells(const CoherentSort& c, const float4* pos, const float4* vel,
                         const GridParams& g, uint2* cells, int key_bits, uint32_t* keys,
                         uint32_t* keys_out, uint32_t* perm_out, float4* pos_out, float4* vel_out,
                         uint32_t* err, int force_timeout, cudaStream_t st,
                         NearList near = NearList{});

// The same for keys already in memory (n = c.n keys); kprev is read, not
// written.
void coherent_sort_keys(const CoherentSort& c, const uint32_t* keys, int key_bits,
                        uint32_t* keys_out, uint32_t* perm_out, uint32_t* err, int force_timeout,
                        cudaStream_t st);

}  // namespace sph
