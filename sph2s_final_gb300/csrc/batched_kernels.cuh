// batched_kernels.cuh -- kernels that step many independent single-scale
// scenes at once.
//
// All scenes live in one packed particle array (scene s owns
// [p_off, p_off + p_n)) and one packed cell table (scene s's cells start at
// c_off).  Sort keys put the scene index above the Morton bits, so a single
// global sort keeps every scene contiguous and orders each scene exactly as
// the single-scale solver would.  Every kernel is persistent: a grid of
// (multiple of the SM count) blocks walks a list of tiles, each tile a run of
// consecutive particles of ONE scene, so a block's per-scene constants are
// uniform and the per-particle code is the single-scale device code
// (density_one, force_one) with that scene's parameters.
#pragma once
#include "common.cuh"
#include "density_kernel.cuh"
#include "force_kernel.cuh"
#include "radix_sort.cuh"

namespace sph {

struct SceneRec {
    SimParams P;
    uint32_t p_off, p_n;  // fluid particles
    uint32_t c_off;       // first cell of the scene's tables
    uint32_t b_off, b_n;  // boundary particles (sorted once)
};

// tiles[t] = (scene, first particle); a tile covers up to BS particles of its scene.
template <int BS>
__global__ void __launch_bounds__(BS) b_hash_hist_kernel(const uint2* __restrict__ tiles,
                                                         uint32_t num_tiles,
                                                         const SceneRec* __restrict__ recs,
                                                         const float4* __restrict__ pos,
                                                         int shift, int passes,
                                                         uint32_t* __restrict__ keys,
                                                         uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    for (int i = threadIdx.x; i < kSortMaxPasses * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t end = R.p_off + R.p_n;
        const uint32_t i = tile.y + threadIdx.x;
        if (i < end) {
            const float4 p = pos[i];
            const uint32_t k = (tile.x << shift) | cell_key(R.P.g, p.x, p.y, p.z);
            keys[i] = k;
            sort_hist_add(sh, k, passes);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Boundary presort keys of a batch: (scene, cell) above qb bits of depth
// class (depth_class, quantum = h/16 of the scene); w becomes the class's
// lower bound, as in the single-scene presort.
template <int BS>
__global__ void __launch_bounds__(BS) b_boundary_hash_hist_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    float4* __restrict__ b, int shift, int qb, int passes, uint32_t* __restrict__ keys,
    uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    for (int i = threadIdx.x; i < kSortMaxPasses * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t i = tile.y + threadIdx.x;
        if (i < R.b_off + R.b_n) {
            float4 p = b[i];
            const DepthClass dc = depth_class(R.P.g, p.x, p.y, p.z, R.P.h / 16.0f, qb);
            const uint32_t k = (((tile.x << shift) | cell_key(R.P.g, p.x, p.y, p.z)) << qb) | dc.cls;
            p.w = dc.lb;
            b[i] = p;
            keys[i] = k;
            sort_hist_add(sh, k, passes);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Reorder + per-scene cell ranges; indices stored in the tables are global.
// Keys are shifted right by key_shift first (the boundary presort's depth bits).
// With bflag, also bflag[i] = bnear of particle i's cell (1 if boundary
// particles lie within its stencil reach), for the boundary and force passes.
template <int BS, bool WITH_VEL>
__global__ void __launch_bounds__(BS) b_gather_cells_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const uint32_t* __restrict__ keys_sorted, const uint32_t* __restrict__ perm, uint32_t n,
    int shift, bool boundary, const float4* __restrict__ pos_in, const float4* __restrict__ vel_in,
    float4* __restrict__ pos_out, float4* __restrict__ vel_out, uint2* __restrict__ cells,
    uint32_t* __restrict__ err, int key_shift = 0, uint32_t* __restrict__ kprev_out = nullptr,
    const uint8_t* __restrict__ bnear = nullptr, uint8_t* __restrict__ bflag = nullptr) {
    const uint32_t lmask = (1u << shift) - 1u;
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t beg = boundary ? R.b_off : R.p_off;
        const uint32_t end = beg + (boundary ? R.b_n : R.p_n);
        const uint32_t i = tile.y + threadIdx.x;
        if (i >= end) continue;
        if (kprev_out) kprev_out[i] = keys_sorted[i];  // the next coherent sort starts here
        uint32_t q = perm[i];
        if (q < beg || q >= end) {  // a sort that gave up: stay in bounds, report
            atomicOr(err, 2u);
            q = i;
        }
        pos_out[i] = pos_in[q];
        if (WITH_VEL) vel_out[i] = vel_in[q];
        const uint32_t key = keys_sorted[i] >> key_shift;
        uint32_t* cw = reinterpret_cast<uint32_t*>(cells + R.c_off);
        const uint32_t c = (key >> shift) == tile.x ? morton_to_linear_checked(R.P.g, key & lmask)
                                                    : kEmptyCell;
        if (bflag) bflag[i] = (c != kEmptyCell && __ldg(&bnear[R.c_off + c]) != 0) ? 1 : 0;
        if (c == kEmptyCell) {
            atomicOr(err, 2u);
            continue;
        }
        const uint32_t prev = i > beg ? keys_sorted[i - 1] >> key_shift : 0u;
        if (i == beg || prev != key) {
            cw[2 * c] = i;
            if (i > beg) {
                const uint32_t cp = morton_to_linear_checked(R.P.g, prev & lmask);
                if (cp != kEmptyCell) cw[2 * cp + 1] = i;
            }
        }
        if (i == end - 1) cw[2 * c + 1] = end;
    }
}

template <int BS>
__global__ void __launch_bounds__(BS) b_density_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const float4* __restrict__ pos, const uint2* __restrict__ cells, uint32_t n,
    float* __restrict__ rho, float2* __restrict__ aux, uint4* __restrict__ nbr4,
    uint32_t* __restrict__ nbr_count, float4* __restrict__ xa, float4* __restrict__ svel) {
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t i = tile.y + threadIdx.x;
        if (i >= R.p_off + R.p_n) continue;
        const SimParams P = R.P;
        density_one<false>(i, pos, cells + R.c_off, n, P, rho, aux, nbr4, nbr_count, nullptr, xa,
                           svel);
    }
}

// Boundary force sums of the scenes' near-boundary particles (bnear of the
// scene's cell, or bflag[i] where given), from the scenes' static candidate
// tables (boundary_force_one), for b_force_kernel to load.
template <int BS>
__global__ void __launch_bounds__(BS) b_boundary_force_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const float4* __restrict__ pos, const float4* __restrict__ bpos,
    const uint2* __restrict__ bcells, const uint8_t* __restrict__ bnear,
    const uint32_t* __restrict__ bstart,
    const uint32_t* __restrict__ bcand, uint32_t nb, float4* __restrict__ bacc,
    const uint8_t* __restrict__ bflag = nullptr) {
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t i = tile.y + threadIdx.x;
        if (i >= R.p_off + R.p_n) continue;
        if (bflag && !__ldg(&bflag[i])) continue;
        const float4 xi = pos[i];
        const GridParams& g = R.P.g;
        const int hx = cell_coord(xi.x, g.ox, g.spacing, g.dx);
        const int hy = cell_coord(xi.y, g.oy, g.spacing, g.dy);
        const int hz = cell_coord(xi.z, g.oz, g.spacing, g.dz);
        const uint32_t home = linear_cell(g, hx, hy, hz);
        if (!__ldg(&bnear[R.c_off + home])) continue;
        const SimParams P = R.P;
        boundary_force_one(i, xi, hx, hy, hz, home, bpos, bcells + R.c_off, bstart + R.c_off,
                           bcand, nb, P, bacc);
    }
}

template <int BS>
__global__ void __launch_bounds__(BS) b_force_kernel(
    const uint2* __restrict__ tiles, uint32_t num_tiles, const SceneRec* __restrict__ recs,
    const float4* __restrict__ pos, const float4* __restrict__ xa, const float4* __restrict__ va,
    const uint2* __restrict__ cells, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const float4* __restrict__ bpos,
    const uint2* __restrict__ bcells, const uint8_t* __restrict__ bnear, uint32_t n, uint32_t nb,
    float dt, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
    const float4* __restrict__ bacc, const uint8_t* __restrict__ bflag = nullptr) {
    for (uint32_t t = blockIdx.x; t < num_tiles; t += gridDim.x) {
        const uint2 tile = tiles[t];
        const SceneRec& R = recs[tile.x];
        const uint32_t i = tile.y + threadIdx.x;
        if (i >= R.p_off + R.p_n) continue;
        const SimParams P = R.P;
        force_one<0, true>(i, pos, xa, va, cells + R.c_off, nbr4, nbr_count, bpos,
                           bcells + R.c_off, bnear + R.c_off, n, nb, P, dt, pos_out, vel_out,
                           nullptr, nullptr, bacc, bflag);
    }
}

}  // namespace sph
