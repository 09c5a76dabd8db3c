// single_scale_kernels.cuh -- device kernels of the single-scale SPH2S step.
//
//   hash + histogram   computeHashs                 SPH2S_FINAL_SINGLE_SCALE/Solver.cu:401-424
//   gather + ranges    reorderAndComputeCellStartEndD        Solver.cu:478-534
//   density            computeDensitiesPressuresD           Solver.cu:536-599 (+198-229)
//   force + integrate  computeAccelerationsD + integrateD   Solver.cu:601-755 (+231-344)
//
// Layout in HBM (all in the sorted order of the current step):
//   pos  float4 (x, y, z, w = persistent id bits)
//   vel  float4 (vx, vy, vz, 0)
//   rho  float,  aux float2 (p / rho^2, 1 / rho)
//   cells uint2 per linear cell (start, end), 0xFFFFFFFF when empty
#pragma once
#include "common.cuh"
#include "radix_sort.cuh"

namespace sph {

// Morton key per particle, fused with the digit histograms of every sort pass.
static __global__ void __launch_bounds__(256) hash_hist_kernel(const float4* __restrict__ pos, uint32_t n,
                                                        GridParams g, int passes,
                                                        uint32_t* __restrict__ keys,
                                                        uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    for (int i = threadIdx.x; i < kSortMaxPasses * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = pos[i];
        uint32_t k = cell_key(g, p.x, p.y, p.z);
        keys[i] = k;
        sort_hist_add(sh, k, passes);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Boundary presort keys: the cell's Morton key above qb bits of depth class
// (depth_class), so that the stable sort stores each cell's boundary
// particles by non-decreasing w; w becomes the class's lower bound.
static __global__ void __launch_bounds__(256) boundary_hash_hist_kernel(
    float4* __restrict__ b, uint32_t n, GridParams g, int qb, float quantum, int passes,
    uint32_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    for (int i = threadIdx.x; i < kSortMaxPasses * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = b[i];
        const DepthClass dc = depth_class(g, p.x, p.y, p.z, quantum, qb);
        const uint32_t k = (cell_key(g, p.x, p.y, p.z) << qb) | dc.cls;
        p.w = dc.lb;
        b[i] = p;
        keys[i] = k;
        sort_hist_add(sh, k, passes);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Reorders the state by the sorted permutation and records cell ranges (keys
// shifted right by key_shift first: the boundary presort's depth bits); with
// kprev_out, also stores the sorted keys for the next coherent sort.
// Every index read from the sort output is range-checked: if a bounded wait in
// the sort gave up, its output is garbage, and this kernel then records an
// error and stays in bounds instead of faulting.
template <bool WITH_VEL>
__global__ void __launch_bounds__(256) gather_cells_kernel(
    const uint32_t* __restrict__ keys_sorted, const uint32_t* __restrict__ perm, uint32_t n,
    GridParams g, const float4* __restrict__ pos_in, const float4* __restrict__ vel_in,
    float4* __restrict__ pos_out, float4* __restrict__ vel_out, uint2* __restrict__ cells,
    uint32_t* __restrict__ err, int key_shift = 0, uint32_t* __restrict__ kprev_out = nullptr,
    NearList near = NearList{}) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (kprev_out) kprev_out[i] = keys_sorted[i];  // the next step's coherent sort starts here
    uint32_t q = perm[i];
    if (q >= n) {
        atomicOr(err, 2u);
        q = i;
    }
    pos_out[i] = pos_in[q];
    if (WITH_VEL) vel_out[i] = vel_in[q];
    uint32_t key = keys_sorted[i] >> key_shift;
    uint32_t* cw = reinterpret_cast<uint32_t*>(cells);
    uint32_t c = morton_to_linear_checked(g, key);
    near_append(near, c, i);
    if (c == kEmptyCell) {
        atomicOr(err, 2u);
        return;
    }
    const uint32_t prev = i > 0 ? keys_sorted[i - 1] >> key_shift : 0u;
    if (i == 0 || prev != key) {
        cw[2 * c] = i;
        if (i > 0) {
            uint32_t cp = morton_to_linear_checked(g, prev);
            if (cp != kEmptyCell) cw[2 * cp + 1] = i;
        }
    }
    if (i == n - 1) cw[2 * c + 1] = n;
}

// Packs xyz of a float4 array into AoS floats, in sorted order or scattered
// to the persistent ids held in ids[k].w.
static __global__ void __launch_bounds__(256) pack_xyz_kernel(const float4* __restrict__ src,
                                                       const float4* __restrict__ ids, uint32_t n,
                                                       int by_id, float* __restrict__ dst) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float4 v = src[k];
    uint32_t d = k;
    if (by_id) {
        d = __float_as_uint(ids[k].w);
        if (d >= n) return;
    }
    dst[3 * (size_t)d + 0] = v.x;
    dst[3 * (size_t)d + 1] = v.y;
    dst[3 * (size_t)d + 2] = v.z;
}

// Caller xyz (3 floats per particle) -> float4; w = the input index as bits
// (a persistent id) or 0.
static __global__ void __launch_bounds__(256) unpack_xyz_kernel(const float* __restrict__ xyz,
                                                         uint32_t n, int with_id,
                                                         float4* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const size_t b = 3 * (size_t)k;
    out[k] = make_float4(xyz[b], xyz[b + 1], xyz[b + 2], with_id ? __uint_as_float(k) : 0.0f);
}

// Scalar field (one float per particle) into a caller's array, in sorted order
// or scattered by the persistent ids in ids[k].w.
static __global__ void __launch_bounds__(256) pack_scalar_kernel(const float* __restrict__ src,
                                                         const float4* __restrict__ ids, uint32_t n,
                                                         int by_id, float* __restrict__ dst) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t d = k;
    if (by_id) {
        d = __float_as_uint(ids[k].w);
        if (d >= n) return;
    }
    dst[d] = src[k];
}

// Per-cell flag: does any boundary particle lie within `reach` cells of this
// cell?  A particle's stencil [cell(x-h), cell(x+h)] never leaves
// cell(x) +- (ceil(h/spacing) + 1), so particles in cells without the flag
// skip the boundary stencil without changing any result.
static __global__ void __launch_bounds__(256) boundary_near_kernel(const uint2* __restrict__ bcells,
                                                            GridParams g, int reach,
                                                            uint8_t* __restrict__ near) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nc = (uint32_t)g.dx * g.dy * g.dz;
    if (c >= nc) return;
    int cx = (int)(c % (uint32_t)g.dx);
    int cy = (int)((c / (uint32_t)g.dx) % (uint32_t)g.dy);
    int cz = (int)(c / ((uint32_t)g.dx * g.dy));
    uint8_t f = 0;
    for (int z = max(cz - reach, 0); z <= min(cz + reach, g.dz - 1) && !f; ++z)
        for (int y = max(cy - reach, 0); y <= min(cy + reach, g.dy - 1) && !f; ++y)
            for (int x = max(cx - reach, 0); x <= min(cx + reach, g.dx - 1); ++x) {
                uint2 r = bcells[linear_cell(g, x, y, z)];
                if (r.x != kEmptyCell && r.x < r.y) {
                    f = 1;
                    break;
                }
            }
    near[c] = f;
}

// Static boundary candidates of each cell flagged in `near`: the boundary
// particles of the cells c +-1 (clamped), in stencil order (z, y, x, then the
// cell's presorted order), whose distance to the cell's box is at most lim.
// FILL = false counts them into cnt[c]; FILL = true writes their indices
// from start[c] on.
template <bool FILL>
static __global__ void __launch_bounds__(256) boundary_cand_kernel(
    const uint2* __restrict__ bcells, const float4* __restrict__ bpos,
    const uint8_t* __restrict__ near, GridParams g, uint32_t nb, float lim,
    uint32_t* __restrict__ cnt_or_start, uint32_t* __restrict__ cand) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nc = (uint32_t)g.dx * g.dy * g.dz;
    if (c >= nc) return;
    if (!near[c]) {
        if (!FILL) cnt_or_start[c] = 0;
        return;
    }
    const int cx = (int)(c % (uint32_t)g.dx);
    const int cy = (int)((c / (uint32_t)g.dx) % (uint32_t)g.dy);
    const int cz = (int)(c / ((uint32_t)g.dx * g.dy));
    const float lx = g.ox + cx * g.spacing, hx = g.ox + (cx + 1) * g.spacing;
    const float ly = g.oy + cy * g.spacing, hy = g.oy + (cy + 1) * g.spacing;
    const float lz = g.oz + cz * g.spacing, hz = g.oz + (cz + 1) * g.spacing;
    const float lim2 = lim * lim;
    uint32_t k = FILL ? cnt_or_start[c] : 0u;
    for (int z = max(cz - 1, 0); z <= min(cz + 1, g.dz - 1); ++z)
        for (int y = max(cy - 1, 0); y <= min(cy + 1, g.dy - 1); ++y)
            for (int x = max(cx - 1, 0); x <= min(cx + 1, g.dx - 1); ++x) {
                const uint2 r = bcells[linear_cell(g, x, y, z)];
                const uint32_t e = min(r.y, nb);
                for (uint32_t j = r.x; j < e; ++j) {
                    const float4 b = bpos[j];
                    const float dx = fmaxf(fmaxf(lx - b.x, b.x - hx), 0.0f);
                    const float dy = fmaxf(fmaxf(ly - b.y, b.y - hy), 0.0f);
                    const float dz = fmaxf(fmaxf(lz - b.z, b.z - hz), 0.0f);
                    if (dx * dx + dy * dy + dz * dz <= lim2) {
                        if (FILL) cand[k] = j;
                        ++k;
                    }
                }
            }
    if (!FILL) cnt_or_start[c] = k;
}

}  // namespace sph

#include "density_kernel.cuh"
#include "xsph_kernel.cuh"
#include "force_kernel.cuh"
