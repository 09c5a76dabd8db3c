// adjoint_kernels.cuh -- reverse-mode derivatives of the single-scale step.
//
// Forward step (sorted order of the step, P = the sort permutation):
//   xh = P x, vh = P v;  rho = D(xh);  a = F(xh, vh, rho; mu)
//   v' = vh + dt a;      x' = xh + dt v'
// with, for 0 < r_ij < h (x_ij = x_i - x_j),
//   a_i = sum_j [ S_ij x_ij + psi_ij (v_j - v_i) ] + b_i(x_i) + g
//   S_ij = m Cs (A_i + A_j) (h-r)^2/r - sigma m C6 (h^2-r^2)^3 / rho_i,
//   A_k = K (rho_k - rho0) / rho_k^2,  psi_ij = mu m Cs (h-r) / (rho_i rho_j)
//   rho_i = m C6 sum_j (h^2 - r_ij^2)^3   (self included)
// (SPH2S_FINAL_SINGLE_SCALE/Solver.cu:103-344, 536-755).
//
// Given the adjoints gx', gv' of the step's outputs, with
// lam_i = dt (gv'_i + dt gx'_i):
//   gxh_i = gx'_i + sum_j [ phi_i lam_i - phi_j lam_j
//                           + (((phi'_i lam_i - phi'_j lam_j) . x_ij) / r) x_ij
//                           + psi' ((lam_i - lam_j) . (v_j - v_i)) / r x_ij ]
//           + sum_k [ beta lam_i + beta' (lam_i . x_ik) / r x_ik ]       (boundary)
//           - 6 m C6 sum_j (h^2 - r^2)^2 (grho_i + grho_j) x_ij       (density)
//   gvh_i = gv'_i + dt gx'_i + sum_j psi_ij (lam_j - lam_i)
//   grho_i = sum_j [ m Cs A'_i f (lam_i - lam_j) . x_ij
//                    + sigma m C6 w / rho_i^2 lam_i . x_ij
//                    - psi_ij / rho_i (lam_i - lam_j) . (v_j - v_i) ]
//   gmu += sum_i lam_i . sum_j (psi_ij / mu) (v_j - v_i)
// where phi_k = m Cs (A_i + A_j) f - sigma m C6 w / rho_k, f = (h-r)^2/r,
// w = (h^2-r^2)^3, A'(rho) = K (2 rho0 - rho) / rho^3.  Every particle sums
// its own pair terms in both roles, so no atomics are needed; the neighbour
// set is the forward step's list (indices held constant).
#pragma once
#include "common.cuh"
#include "force_kernel.cuh"

namespace sph {

// Calls f(j, xj, dx, dy, dz, r2) for every fluid neighbour 0 < r2 < T of
// particle i, from the list or, on overflow, by rescanning the stencil.
template <class F>
__device__ __forceinline__ void visit_force_neighbors(uint32_t i, const float4& xi,
                                                      const float4* __restrict__ pos,
                                                      const uint4* __restrict__ nbr4,
                                                      const uint32_t* __restrict__ nbr_count,
                                                      const uint2* __restrict__ cells, uint32_t n,
                                                      const SimParams& P, F& f) {
    const uint32_t kc = nbr_count[i];
    if (kc <= (uint32_t)kMaxNbr) {
        for (uint32_t t = 0; t < kc; t += 4) {
            const uint4 g = __ldg(&nbr4[(size_t)(t >> 2) * n + i]);
            const uint32_t js[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (t + u < kc) {
                    const uint32_t j = min(js[u], n - 1);
                    const float4 xj = __ldg(&pos[j]);
                    float dx, dy, dz;
                    const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    f(j, dx, dy, dz, r2);
                }
        }
        return;
    }
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
                    const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    if (r2 < P.T && r2 != 0.0f) f(j, dx, dy, dz, r2);
                }
            }
        }
}

// lam = dt (gv' + dt gx')
static __global__ void __launch_bounds__(256) adj_lambda_kernel(const float4* __restrict__ gx,
                                                                const float4* __restrict__ gv,
                                                                uint32_t n, float dt,
                                                                float4* __restrict__ lam) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = gx[i], b = gv[i];
    lam[i] = make_float4(dt * fmaf(dt, a.x, b.x), dt * fmaf(dt, a.y, b.y), dt * fmaf(dt, a.z, b.z), 0.f);
}

struct AdjForcePair {
    const float4* vel;
    const float2* aux;
    const float4* lam;
    float h, h2, mu, mCs, sC6;  // mCs = m * 45/(pi h^6) (spiky and viscosity), sC6 = sigma m C6
    float4 vi, li;
    float Ai, dAi, inv_i;
    float gx, gy, gz, gvx, gvy, gvz, grho, gmu;
    __device__ __forceinline__ void operator()(uint32_t j, float dx, float dy, float dz, float r2) {
        const float rs = rsqrtf(r2);
        const float r = r2 * rs;
        const float hr = h - r;
        const float f = hr * hr * rs;
        const float fp = -hr * (h + r) * rs * rs;
        const float a2 = h2 - r2;
        const float w = a2 * a2 * a2;
        const float wp = -6.0f * r * a2 * a2;
        const float2 aj = __ldg(&aux[j]);
        const float inv_j = aj.y;
        const float4 vj = __ldg(&vel[j]);
        const float4 lj = __ldg(&lam[j]);
        const float Asum = Ai + aj.x;
        const float phi_i = mCs * Asum * f - sC6 * w * inv_i;
        const float phi_j = mCs * Asum * f - sC6 * w * inv_j;
        const float php_i = mCs * Asum * fp - sC6 * wp * inv_i;
        const float php_j = mCs * Asum * fp - sC6 * wp * inv_j;
        const float psi_over_mu = mCs * hr * inv_i * inv_j;  // m Cv (h-r) / (rho_i rho_j)
        const float psi = mu * psi_over_mu;
        const float psip = -mu * mCs * inv_i * inv_j;      // d psi / dr
        const float dvx = vj.x - vi.x, dvy = vj.y - vi.y, dvz = vj.z - vi.z;
        const float lx = li.x - lj.x, ly = li.y - lj.y, lz = li.z - lj.z;
        const float pdx = php_i * li.x - php_j * lj.x, pdy = php_i * li.y - php_j * lj.y,
                    pdz = php_i * li.z - php_j * lj.z;
        const float radial = (pdx * dx + pdy * dy + pdz * dz) * rs +
                             psip * (lx * dvx + ly * dvy + lz * dvz) * rs;
        gx += phi_i * li.x - phi_j * lj.x + radial * dx;
        gy += phi_i * li.y - phi_j * lj.y + radial * dy;
        gz += phi_i * li.z - phi_j * lj.z + radial * dz;
        gvx += psi * (lj.x - li.x);
        gvy += psi * (lj.y - li.y);
        gvz += psi * (lj.z - li.z);
        grho += mCs * dAi * f * (lx * dx + ly * dy + lz * dz) +
                sC6 * w * inv_i * inv_i * (li.x * dx + li.y * dy + li.z * dz) -
                psi * inv_i * (lx * dvx + ly * dvy + lz * dvz);
        gmu += psi_over_mu * (li.x * dvx + li.y * dvy + li.z * dvz);
    }
};

// Adjoint of force + integrate for particle i of the step's sorted order;
// returns particle i's share of d L / d mu.  cells/bcells/bnear are the
// particle's own grid tables (the batched rollout passes per-scene tables, P
// and mu).
__device__ __forceinline__ float adj_force_one(
    uint32_t i, const float4* __restrict__ pos, const float4* __restrict__ vel,
    const float* __restrict__ rho, const float2* __restrict__ aux, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const uint2* __restrict__ cells,
    const float4* __restrict__ bpos, const uint2* __restrict__ bcells,
    const uint8_t* __restrict__ bnear, const uint32_t* __restrict__ bstart,
    const uint32_t* __restrict__ bcand, uint32_t n, uint32_t nb, const SimParams& P, float mu,
    float dt, const float4* __restrict__ lam, const float4* __restrict__ gx_in,
    const float4* __restrict__ gv_in, float4* __restrict__ gx_out, float4* __restrict__ gv_out,
    float* __restrict__ grho) {
    {
        const float4 xi = pos[i];
        AdjForcePair A;
        A.vel = vel;
        A.aux = aux;
        A.lam = lam;
        A.h = P.h;
        A.h2 = P.h2;
        A.mu = mu;
        A.mCs = P.pres_coef;
        A.sC6 = P.tens_coef;
        A.vi = vel[i];
        A.li = lam[i];
        const float2 ai = aux[i];
        A.Ai = ai.x;
        A.inv_i = ai.y;
        A.dAi = P.bulk * (2.0f * P.rho0 - rho[i]) * ai.y * ai.y * ai.y;  // dA/drho
        A.gx = A.gy = A.gz = A.gvx = A.gvy = A.gvz = A.grho = A.gmu = 0.0f;
        visit_force_neighbors(i, xi, pos, nbr4, nbr_count, cells, n, P, A);
        // boundary: b_i = sum_k beta(r) x_ik, beta = Bc shape(2r/h) / r^2
        float bx = 0.f, by = 0.f, bz = 0.f;
        const int hx = cell_coord(xi.x, P.g.ox, P.g.spacing, P.g.dx);
        const int hy = cell_coord(xi.y, P.g.oy, P.g.spacing, P.g.dy);
        const int hz = cell_coord(xi.z, P.g.oz, P.g.spacing, P.g.dz);
        const uint32_t home = linear_cell(P.g, hx, hy, hz);
        if (__ldg(&bnear[home])) {
            visit_boundary(xi, hx, hy, hz, home, bpos, bcells, bstart, bcand, nb, P,
                           [&](const float4& xk) {
                float dx, dy, dz;
                const float r2 = dist2(xi.x, xi.y, xi.z, xk.x, xk.y, xk.z, dx, dy, dz);
                if (r2 < P.T) {
                    const float rs = rsqrtf(r2);
                    const float rr = r2 * rs;
                    const float q = rr * P.two_over_h;
                    float sh, shp;
                    if (q < 2.0f / 3.0f) {
                        sh = 2.0f / 3.0f;
                        shp = 0.0f;
                    } else if (q < 1.0f) {
                        sh = q * (2.0f - 1.5f * q);
                        shp = 2.0f - 3.0f * q;
                    } else {
                        const float t2 = 2.0f - q;
                        sh = 0.5f * t2 * t2;
                        shp = -t2;
                    }
                    const float beta = P.bnd_coef * sh * rs * rs;
                    const float betap = P.bnd_coef * (shp * P.two_over_h * rs * rs -
                                                      2.0f * sh * rs * rs * rs);
                    const float rad = betap * rs * (A.li.x * dx + A.li.y * dy + A.li.z * dz);
                    bx += beta * A.li.x + rad * dx;
                    by += beta * A.li.y + rad * dy;
                    bz += beta * A.li.z + rad * dz;
                }
            });
        }
        const float4 gxi = gx_in[i], gvi = gv_in[i];
        gx_out[i] = make_float4(gxi.x + A.gx + bx, gxi.y + A.gy + by, gxi.z + A.gz + bz, 0.f);
        gv_out[i] = make_float4(fmaf(dt, gxi.x, gvi.x) + A.gvx, fmaf(dt, gxi.y, gvi.y) + A.gvy,
                                fmaf(dt, gxi.z, gvi.z) + A.gvz, 0.f);
        grho[i] = A.grho;
        return A.gmu;
    }
}

// Block sum of one value per thread in a fixed order (warp shuffles, then the
// warps in index order); the result is valid in thread 0.  Every thread of
// the block must call it.
__device__ __forceinline__ float block_sum_fixed(float v) {
    __shared__ float s_red[32];
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = 0.0f;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
    return t;
}

static __global__ void __launch_bounds__(256) adj_force_kernel(
    const float4* __restrict__ pos, const float4* __restrict__ vel, const float* __restrict__ rho,
    const float2* __restrict__ aux, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const uint2* __restrict__ cells,
    const float4* __restrict__ bpos, const uint2* __restrict__ bcells,
    const uint8_t* __restrict__ bnear, const uint32_t* __restrict__ bstart,
    const uint32_t* __restrict__ bcand, uint32_t n, uint32_t nb, SimParams P, float mu, float dt,
    const float4* __restrict__ lam, const float4* __restrict__ gx_in,
    const float4* __restrict__ gv_in, float4* __restrict__ gx_out, float4* __restrict__ gv_out,
    float* __restrict__ grho, float* __restrict__ gmu_block) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float gmu_i = 0.0f;
    if (i < n)
        gmu_i = adj_force_one(i, pos, vel, rho, aux, nbr4, nbr_count, cells, bpos, bcells, bnear,
                              bstart, bcand, n,
                              nb, P, mu, dt, lam, gx_in, gv_in, gx_out, gv_out, grho);
    // per-block sum of d L / d mu (reduced in a fixed order afterwards)
    const float t = block_sum_fixed(gmu_i);
    if (threadIdx.x == 0) gmu_block[blockIdx.x] = t;
}

struct AdjDensityPair {
    const float* grho;
    float gi, h2, coef;  // coef = -6 m C6
    float gx, gy, gz;
    __device__ __forceinline__ void operator()(uint32_t j, float dx, float dy, float dz, float r2) {
        const float a = h2 - r2;
        const float c = coef * a * a * (gi + __ldg(&grho[j]));
        gx = fmaf(c, dx, gx);
        gy = fmaf(c, dy, gy);
        gz = fmaf(c, dz, gz);
    }
};

// Density adjoint: gx_i += -6 m C6 sum_j (h^2 - r^2)^2 (grho_i + grho_j) x_ij.
__device__ __forceinline__ void adj_density_one(uint32_t i, const float4* __restrict__ pos,
                                                const uint4* __restrict__ nbr4,
                                                const uint32_t* __restrict__ nbr_count,
                                                const uint2* __restrict__ cells, uint32_t n,
                                                const SimParams& P, const float* __restrict__ grho,
                                                float4* __restrict__ gx) {
    const float4 xi = pos[i];
    AdjDensityPair A;
    A.grho = grho;
    A.gi = grho[i];
    A.h2 = P.h2;
    A.coef = -6.0f * P.dens_coef;
    A.gx = A.gy = A.gz = 0.0f;
    visit_force_neighbors(i, xi, pos, nbr4, nbr_count, cells, n, P, A);
    float4 g = gx[i];
    g.x += A.gx;
    g.y += A.gy;
    g.z += A.gz;
    gx[i] = g;
}

static __global__ void __launch_bounds__(256) adj_density_kernel(
    const float4* __restrict__ pos, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const uint2* __restrict__ cells, uint32_t n,
    SimParams P, const float* __restrict__ grho, float4* __restrict__ gx) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    adj_density_one(i, pos, nbr4, nbr_count, cells, n, P, grho, gx);
}

// Scatter from the step's sorted order back to the order before the sort:
// out[perm[i]] = in[i].
static __global__ void __launch_bounds__(256) adj_unpermute_kernel(const uint32_t* __restrict__ perm,
                                                                   uint32_t n,
                                                                   const float4* __restrict__ a,
                                                                   const float4* __restrict__ b,
                                                                   float4* __restrict__ ao,
                                                                   float4* __restrict__ bo) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t q = min(perm[i], n - 1);
    ao[q] = a[i];
    bo[q] = b[i];
}

// Deterministic sum of the per-block mu partials into acc (double).
static __global__ void adj_sum_kernel(const float* __restrict__ part, uint32_t count,
                                      double* __restrict__ acc) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (uint32_t k = 0; k < count; ++k) s += (double)part[k];
    *acc += s;
}

// Poly6 splat of the particles on the cell centres of a node grid:
// G_n = m C6 sum_i (h^2 - r^2)^3 over r < h (the same stencil rule as the
// density pass, on the particles' grid).
__device__ __forceinline__ float splat_node(uint32_t c, const float4* __restrict__ pos,
                                            const uint2* __restrict__ cells, uint32_t n,
                                            const SimParams& P, const GridParams& ng) {
    const int ix = (int)(c % (uint32_t)ng.dx), iy = (int)((c / (uint32_t)ng.dx) % (uint32_t)ng.dy),
              iz = (int)(c / ((uint32_t)ng.dx * ng.dy));
    const float y0 = ng.ox + ((float)ix + 0.5f) * ng.spacing;
    const float y1 = ng.oy + ((float)iy + 0.5f) * ng.spacing;
    const float y2 = ng.oz + ((float)iz + 0.5f) * ng.spacing;
    const Stencil s = stencil(P.g, y0, y1, y2, P.h);
    float sum = 0.0f;
    for (int cz = s.z0; cz <= s.z1; ++cz)
        for (int cy = s.y0; cy <= s.y1; ++cy) {
            const uint32_t row = linear_cell(P.g, 0, cy, cz);
            for (int cx = s.x0; cx <= s.x1; ++cx) {
                const uint2 r = __ldg(&cells[row + cx]);
                const uint32_t e = min(r.y, n);
                for (uint32_t j = r.x; j < e; ++j) {
                    const float4 xj = __ldg(&pos[j]);
                    float dx, dy, dz;
                    const float r2 = dist2(y0, y1, y2, xj.x, xj.y, xj.z, dx, dy, dz);
                    if (r2 < P.T) {
                        const float a = P.h2 - r2;
                        sum = fmaf(a * a, a, sum);
                    }
                }
            }
        }
    return P.dens_coef * sum;
}

static __global__ void __launch_bounds__(256) splat_kernel(const float4* __restrict__ pos,
                                                           const uint2* __restrict__ cells,
                                                           uint32_t n, SimParams P, GridParams ng,
                                                           float* __restrict__ field) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nn = (uint32_t)ng.dx * ng.dy * ng.dz;
    if (c >= nn) return;
    field[c] = splat_node(c, pos, cells, n, P, ng);
}

// dL/dx_i of L = mean_n (G_n - target_n)^2, for the sorted particles:
// sum over nodes n with |x_i - y_n| < h of (2/N_n) e_n m C6 3 (h^2-r^2)^2 (-2)(x_i - y_n).
__device__ __forceinline__ float4 splat_grad_one(uint32_t i, const float4* __restrict__ pos,
                                                 const SimParams& P, const GridParams& ng,
                                                 const float* __restrict__ err_n, float scale) {
    const float4 xi = pos[i];
    const float inv = 1.0f / ng.spacing;
    const int x0 = max(0, (int)ceilf((xi.x - P.h - ng.ox) * inv - 0.5f) - 1);
    const int x1 = min(ng.dx - 1, (int)floorf((xi.x + P.h - ng.ox) * inv - 0.5f) + 1);
    const int y0 = max(0, (int)ceilf((xi.y - P.h - ng.oy) * inv - 0.5f) - 1);
    const int y1 = min(ng.dy - 1, (int)floorf((xi.y + P.h - ng.oy) * inv - 0.5f) + 1);
    const int z0 = max(0, (int)ceilf((xi.z - P.h - ng.oz) * inv - 0.5f) - 1);
    const int z1 = min(ng.dz - 1, (int)floorf((xi.z + P.h - ng.oz) * inv - 0.5f) + 1);
    float gxx = 0.f, gyy = 0.f, gzz = 0.f;
    for (int iz = z0; iz <= z1; ++iz)
        for (int iy = y0; iy <= y1; ++iy)
            for (int ix = x0; ix <= x1; ++ix) {
                const float yx = ng.ox + ((float)ix + 0.5f) * ng.spacing;
                const float yy = ng.oy + ((float)iy + 0.5f) * ng.spacing;
                const float yz = ng.oz + ((float)iz + 0.5f) * ng.spacing;
                float dx, dy, dz;
                const float r2 = dist2(yx, yy, yz, xi.x, xi.y, xi.z, dx, dy, dz);
                if (r2 < P.T) {
                    // node-particle stencil rule: the node's stencil must contain the particle's cell
                    const Stencil s = stencil(P.g, yx, yy, yz, P.h);
                    const int cx = cell_coord(xi.x, P.g.ox, P.g.spacing, P.g.dx);
                    const int cy = cell_coord(xi.y, P.g.oy, P.g.spacing, P.g.dy);
                    const int cz = cell_coord(xi.z, P.g.oz, P.g.spacing, P.g.dz);
                    if (cx < s.x0 || cx > s.x1 || cy < s.y0 || cy > s.y1 || cz < s.z0 || cz > s.z1)
                        continue;
                    const float a = P.h2 - r2;
                    const float c = scale * err_n[ix + ng.dx * (iy + ng.dy * iz)] * a * a;
                    // d/dx_i of (h^2 - |y - x_i|^2)^3 = 6 (h^2 - r^2)^2 (y - x_i); here d = y - x_i
                    gxx = fmaf(c, dx, gxx);
                    gyy = fmaf(c, dy, gyy);
                    gzz = fmaf(c, dz, gzz);
                }
            }
    return make_float4(gxx, gyy, gzz, 0.f);
}

static __global__ void __launch_bounds__(256) splat_grad_kernel(const float4* __restrict__ pos,
                                                                uint32_t n, SimParams P,
                                                                GridParams ng,
                                                                const float* __restrict__ err_n,
                                                                float scale,
                                                                float4* __restrict__ gx) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    gx[i] = splat_grad_one(i, pos, P, ng, err_n, scale);
}

}  // namespace sph
