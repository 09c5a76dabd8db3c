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

// Per-cell flag: does any boundary particle lie within `reach` cells of this
// cell?  A particle's stencil [cell(x-h), cell(x+h)] never leaves
// cell(x) +- (ceil(h/spacing) + 1), so particles in cells without the flag
// skip the boundary stencil without changing any result.
__global__ void __launch_bounds__(256) boundary_near_kernel(const uint2* __restrict__ bcells,
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

// Poly6 density (self included), linear EOS, the per-particle factors the
// force pass needs from every neighbour, and the neighbour list of the force
// pass: every j with 0 < r2 < T, in stencil order.  The lists are stored
// transposed in groups of four, group g of particle i at nbr4[g * n + i], so
// that the force pass reads 512 contiguous bytes per warp instruction; here a
// lane stores a group as soon as it holds four indices.  nbr_count[i] may
// exceed kMaxNbr, in which case the force pass rescans the stencil for that
// particle.
constexpr int kDensityThreads = 256;

template <bool DEBUG>
__global__ void __launch_bounds__(kDensityThreads) density_kernel(
    const float4* __restrict__ pos, const uint2* __restrict__ cells, uint32_t n, SimParams P,
    float* __restrict__ rho, float2* __restrict__ aux, uint4* __restrict__ nbr4,
    uint32_t* __restrict__ nbr_count, uint32_t* __restrict__ dbg_count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t k = 0, zero = 0;
    uint4 buf = make_uint4(0u, 0u, 0u, 0u);
    float sum = 0.0f;
    const float4 xi = pos[i];
    const Stencil s = stencil(P.g, xi.x, xi.y, xi.z, P.h);
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
                        if (r2 != 0.0f) {
                            const uint32_t q = k & 3u;
                            buf.x = q == 0u ? j : buf.x;
                            buf.y = q == 1u ? j : buf.y;
                            buf.z = q == 2u ? j : buf.z;
                            buf.w = q == 3u ? j : buf.w;
                            if (q == 3u && k < (uint32_t)kMaxNbr) nbr4[(size_t)(k >> 2) * n + i] = buf;
                            ++k;
                        } else {
                            ++zero;
                        }
                    }
                }
            }
        }
    if ((k & 3u) != 0u && k < (uint32_t)kMaxNbr) nbr4[(size_t)(k >> 2) * n + i] = buf;
    const float rh = P.dens_coef * sum;
    const float p = P.bulk * (rh - P.rho0);
    const float inv = 1.0f / rh;
    rho[i] = rh;
    aux[i] = make_float2(p * inv * inv, inv);
    nbr_count[i] = k;
    if (DEBUG) dbg_count[i] = k + zero;
}

// Pair term of the force pass for one fluid neighbour j (0 < r2 < T).
struct ForceAcc {
    float fx, fy, fz;  // sum of s_ij * x_ij
    float wx, wy, wz;  // sum of (h - r) / rho_j * (v_j - v_i)
};

__device__ __forceinline__ void force_pair(ForceAcc& A, const SimParams& P, float ai_x, float tcoef,
                                           const float4& vi, float dx, float dy, float dz,
                                           float r2, const float2& aj, const float4& vj) {
    float rs = rsqrtf(r2);
    float hr = P.h - r2 * rs;
    float a = P.h2 - r2;
    float sc = P.pres_coef * (ai_x + aj.x) * hr * hr * rs - tcoef * a * a * a;
    A.fx = fmaf(sc, dx, A.fx);
    A.fy = fmaf(sc, dy, A.fy);
    A.fz = fmaf(sc, dz, A.fz);
    float vc = aj.y * hr;
    A.wx = fmaf(vc, vj.x - vi.x, A.wx);
    A.wy = fmaf(vc, vj.y - vi.y, A.wy);
    A.wz = fmaf(vc, vj.z - vi.z, A.wz);
}

// Pressure (spiky gradient), viscosity (Laplacian), tension (Poly6), boundary
// force and gravity; MODE 0 integrates (symplectic Euler) into pos_out/vel_out,
// MODE 1 writes the acceleration and the boundary neighbour count instead.
template <int MODE>
__global__ void __launch_bounds__(256) force_kernel(
    const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ aux,
    const uint2* __restrict__ cells, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const float4* __restrict__ bpos,
    const uint2* __restrict__ bcells, const uint8_t* __restrict__ bnear, uint32_t n, uint32_t nb,
    SimParams P, float dt, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
    float* __restrict__ acc_out, uint32_t* __restrict__ nbr_b) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = pos[i];
    const float4 vi = vel[i];
    const float2 ai = aux[i];
    const float tcoef = P.tens_coef * ai.y;
    ForceAcc A = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const uint32_t kc = nbr_count[i];
    if (kc <= (uint32_t)kMaxNbr) {
        for (uint32_t t = 0; t < kc; t += 4) {
            const uint4 g = __ldg(&nbr4[(size_t)(t >> 2) * n + i]);
            const uint32_t js[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (t + u < kc) {
                    const uint32_t j = min(js[u], n - 1);
                    const float4 xj = __ldg(&pos[j]);
                    float dx, dy, dz;
                    float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    force_pair(A, P, ai.x, tcoef, vi, dx, dy, dz, r2, __ldg(&aux[j]),
                               __ldg(&vel[j]));
                }
            }
        }
    } else {
        const Stencil s = stencil(P.g, xi.x, xi.y, xi.z, P.h);
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
                        if (r2 < P.T && r2 != 0.0f)
                            force_pair(A, P, ai.x, tcoef, vi, dx, dy, dz, r2, __ldg(&aux[j]),
                                       __ldg(&vel[j]));
                    }
                }
            }
    }
    float bx = 0.f, by = 0.f, bz = 0.f;
    uint32_t bcnt = 0;
    const uint32_t home = linear_cell(P.g, cell_coord(xi.x, P.g.ox, P.g.spacing, P.g.dx),
                                      cell_coord(xi.y, P.g.oy, P.g.spacing, P.g.dy),
                                      cell_coord(xi.z, P.g.oz, P.g.spacing, P.g.dz));
    if (__ldg(&bnear[home])) {
        const Stencil s = stencil(P.g, xi.x, xi.y, xi.z, P.h);
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
    }
    const float vf = P.visc_coef * ai.y;
    const float axx = fmaf(vf, A.wx, A.fx) + bx;
    const float ayy = fmaf(vf, A.wy, A.fy) + P.gravity + by;
    const float azz = fmaf(vf, A.wz, A.fz) + bz;
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
