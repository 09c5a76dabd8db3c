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
__global__ void __launch_bounds__(256) hash_hist_kernel(const float4* __restrict__ pos, uint32_t n,
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

// Reorders the state by the sorted permutation and records cell ranges.
// Every index read from the sort output is range-checked: if a bounded wait in
// the sort gave up, its output is garbage, and this kernel then records an
// error and stays in bounds instead of faulting.
template <bool WITH_VEL>
__global__ void __launch_bounds__(256) gather_cells_kernel(
    const uint32_t* __restrict__ keys_sorted, const uint32_t* __restrict__ perm, uint32_t n,
    GridParams g, const float4* __restrict__ pos_in, const float4* __restrict__ vel_in,
    float4* __restrict__ pos_out, float4* __restrict__ vel_out, uint2* __restrict__ cells,
    uint32_t* __restrict__ err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t q = perm[i];
    if (q >= n) {
        atomicOr(err, 2u);
        q = i;
    }
    pos_out[i] = pos_in[q];
    if (WITH_VEL) vel_out[i] = vel_in[q];
    uint32_t key = keys_sorted[i];
    uint32_t* cw = reinterpret_cast<uint32_t*>(cells);
    uint32_t c = morton_to_linear_checked(g, key);
    if (c == kEmptyCell) {
        atomicOr(err, 2u);
        return;
    }
    if (i == 0 || keys_sorted[i - 1] != key) {
        cw[2 * c] = i;
        if (i > 0) {
            uint32_t cp = morton_to_linear_checked(g, keys_sorted[i - 1]);
            if (cp != kEmptyCell) cw[2 * cp + 1] = i;
        }
    }
    if (i == n - 1) cw[2 * c + 1] = n;
}

// Packs xyz of a float4 array into AoS floats, in sorted order or scattered
// to the persistent ids held in ids[k].w.
__global__ void __launch_bounds__(256) pack_xyz_kernel(const float4* __restrict__ src,
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

// Poly6 density (self included), linear EOS, and the per-particle factors the
// force pass needs from every neighbour.
template <bool DEBUG>
__global__ void __launch_bounds__(256) density_kernel(const float4* __restrict__ pos,
                                                      const uint2* __restrict__ cells, uint32_t n,
                                                      SimParams P, float* __restrict__ rho,
                                                      float2* __restrict__ aux,
                                                      uint32_t* __restrict__ nbr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = pos[i];
    const Stencil s = stencil(P.g, xi.x, xi.y, xi.z, P.h);
    float sum = 0.0f;
    uint32_t cnt = 0;
    for (int cz = s.z0; cz <= s.z1; ++cz)
        for (int cy = s.y0; cy <= s.y1; ++cy) {
            const uint32_t row = linear_cell(P.g, 0, cy, cz);
            for (int cx = s.x0; cx <= s.x1; ++cx) {
                const uint2 r = __ldg(&cells[row + cx]);
                const uint32_t e = min(r.y, n);
                for (uint32_t j = r.x; j < e; ++j) {
                    const float4 xj = __ldg(&pos[j]);
                    float dx, dy, dz;
                    float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    if (r2 < P.T) {
                        float a = P.h2 - r2;
                        sum = fmaf(a * a, a, sum);
                        if (DEBUG) ++cnt;
                    }
                }
            }
        }
    const float rh = P.dens_coef * sum;
    const float p = P.bulk * (rh - P.rho0);
    const float inv = 1.0f / rh;
    rho[i] = rh;
    aux[i] = make_float2(p * inv * inv, inv);
    if (DEBUG) nbr[i] = cnt;
}

// Pressure (spiky gradient), viscosity (Laplacian), tension (Poly6), boundary
// force and gravity; MODE 0 integrates (symplectic Euler) into pos_out/vel_out,
// MODE 1 writes the acceleration and the boundary neighbour count instead.
template <int MODE>
__global__ void __launch_bounds__(256) force_kernel(
    const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ aux,
    const uint2* __restrict__ cells, const float4* __restrict__ bpos,
    const uint2* __restrict__ bcells, uint32_t n, uint32_t nb, SimParams P, float dt,
    float4* __restrict__ pos_out, float4* __restrict__ vel_out, float* __restrict__ acc_out,
    uint32_t* __restrict__ nbr_b) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = pos[i];
    const float4 vi = vel[i];
    const float2 ai = aux[i];
    const float tcoef = P.tens_coef * ai.y;
    const Stencil s = stencil(P.g, xi.x, xi.y, xi.z, P.h);
    float fx = 0.f, fy = 0.f, fz = 0.f;  // sum of s_ij * x_ij
    float wx = 0.f, wy = 0.f, wz = 0.f;  // sum of (h - r)/rho_j (v_j - v_i)
    for (int cz = s.z0; cz <= s.z1; ++cz)
        for (int cy = s.y0; cy <= s.y1; ++cy) {
            const uint32_t row = linear_cell(P.g, 0, cy, cz);
            for (int cx = s.x0; cx <= s.x1; ++cx) {
                const uint2 r = __ldg(&cells[row + cx]);
                const uint32_t e = min(r.y, n);
                for (uint32_t j = r.x; j < e; ++j) {
                    const float4 xj = __ldg(&pos[j]);
                    float dx, dy, dz;
                    float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    if (r2 < P.T && r2 != 0.0f) {
                        const float2 aj = __ldg(&aux[j]);
                        const float4 vj = __ldg(&vel[j]);
                        float rs = rsqrtf(r2);
                        float hr = P.h - r2 * rs;
                        float a = P.h2 - r2;
                        float sc = P.pres_coef * (ai.x + aj.x) * hr * hr * rs - tcoef * a * a * a;
                        fx = fmaf(sc, dx, fx);
                        fy = fmaf(sc, dy, fy);
                        fz = fmaf(sc, dz, fz);
                        float vc = aj.y * hr;
                        wx = fmaf(vc, vj.x - vi.x, wx);
                        wy = fmaf(vc, vj.y - vi.y, wy);
                        wz = fmaf(vc, vj.z - vi.z, wz);
                    }
                }
            }
        }
    float bx = 0.f, by = 0.f, bz = 0.f;
    uint32_t bcnt = 0;
    for (int cz = s.z0; cz <= s.z1; ++cz)
        for (int cy = s.y0; cy <= s.y1; ++cy) {
            const uint32_t row = linear_cell(P.g, 0, cy, cz);
            for (int cx = s.x0; cx <= s.x1; ++cx) {
                const uint2 r = __ldg(&bcells[row + cx]);
                const uint32_t e = min(r.y, nb);
                for (uint32_t j = r.x; j < e; ++j) {
                    const float4 xj = __ldg(&bpos[j]);
                    float dx, dy, dz;
                    float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    if (r2 < P.T) {
                        float rs = rsqrtf(r2);
                        float q = r2 * rs * P.two_over_h;
                        float w = P.bnd_coef * boundary_shape(q) * rs * rs;
                        bx = fmaf(w, dx, bx);
                        by = fmaf(w, dy, by);
                        bz = fmaf(w, dz, bz);
                        if (MODE == 1) ++bcnt;
                    }
                }
            }
        }
    const float vf = P.visc_coef * ai.y;
    const float axx = fmaf(vf, wx, fx) + bx;
    const float ayy = fmaf(vf, wy, fy) + P.gravity + by;
    const float azz = fmaf(vf, wz, fz) + bz;
    if (MODE == 0) {
        float nvx = fmaf(dt, axx, vi.x), nvy = fmaf(dt, ayy, vi.y), nvz = fmaf(dt, azz, vi.z);
        pos_out[i] = make_float4(fmaf(dt, nvx, xi.x), fmaf(dt, nvy, xi.y), fmaf(dt, nvz, xi.z), xi.w);
        vel_out[i] = make_float4(nvx, nvy, nvz, 0.0f);
    } else {
        acc_out[3 * i + 0] = axx;
        acc_out[3 * i + 1] = ayy;
        acc_out[3 * i + 2] = azz;
        nbr_b[i] = bcnt;
    }
}

}  // namespace sph
