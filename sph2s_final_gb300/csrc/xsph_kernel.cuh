// xsph_kernel.cuh -- the XSPH integrator variant of the single-scale step.
//
// integrateXSPHD + computeVelXSPHCell (SPH2S_FINAL_SINGLE_SCALE/Solver.cu:
// 345-395, 757-853; its launch is commented out in Solver::Advance,
// Solver.cu:1185-1196):
//   v'_i  = v_i + dt a_i
//   dv_i  = sum_{j: r_ij < h} (v'_j - v'_i) m / rho_j W_poly6(r_ij)
//   v''_i = v'_i + eps dv_i        (per component; the reference adds dv.x to
//                                   all three components, fixed here)
//   x'_i  = x_i + dt v''_i
// v'' is stored as the new velocity.  The self term vanishes (v'_i - v'_i is
// exactly 0); neighbours come from the density pass's list (0 < r < h), the
// force pass having written a_i; partners at distance 0 other than i itself
// (flagged by the density pass's full count) are picked up from the home
// cell, and particles whose list overflowed rescan the stencil.
#pragma once
#include "common.cuh"

namespace sph {

struct XsphAcc {
    float x = 0.f, y = 0.f, z = 0.f;
};

__device__ __forceinline__ void xsph_pair(XsphAcc& S, const SimParams& P, float r2, float inv_rho_j,
                                          float vix, float viy, float viz, const float4& vj,
                                          const float* __restrict__ acc, uint32_t j, float dt) {
    const float a = P.h2 - r2;
    const float w = a * a * a * inv_rho_j;
    S.x = fmaf(fmaf(dt, acc[3 * j + 0], vj.x) - vix, w, S.x);
    S.y = fmaf(fmaf(dt, acc[3 * j + 1], vj.y) - viy, w, S.y);
    S.z = fmaf(fmaf(dt, acc[3 * j + 2], vj.z) - viz, w, S.z);
}

static __global__ void __launch_bounds__(256) xsph_integrate_kernel(
    const float4* __restrict__ pos, const float4* __restrict__ vel, const float* __restrict__ acc,
    const float2* __restrict__ aux, const uint2* __restrict__ cells, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const uint32_t* __restrict__ nbr_all, uint32_t n,
    SimParams P, float dt, float eps, float4* __restrict__ pos_out, float4* __restrict__ vel_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xi = pos[i];
    const float4 vi = vel[i];
    const float vix = fmaf(dt, acc[3 * i + 0], vi.x);
    const float viy = fmaf(dt, acc[3 * i + 1], vi.y);
    const float viz = fmaf(dt, acc[3 * i + 2], vi.z);
    XsphAcc S;
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
                    const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    xsph_pair(S, P, r2, __ldg(&aux[j]).y, vix, viy, viz, __ldg(&vel[j]), acc, j, dt);
                }
            }
        }
        if (nbr_all[i] > kc + 1u) {  // coincident partners: same position, same cell
            const uint32_t home = linear_cell(P.g, cell_coord(xi.x, P.g.ox, P.g.spacing, P.g.dx),
                                              cell_coord(xi.y, P.g.oy, P.g.spacing, P.g.dy),
                                              cell_coord(xi.z, P.g.oz, P.g.spacing, P.g.dz));
            const uint2 r = __ldg(&cells[home]);
            const uint32_t e = min(r.y, n);
            for (uint32_t j = r.x; j < e; ++j) {
                const float4 xj = __ldg(&pos[j]);
                float dx, dy, dz;
                const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                if (j != i && r2 == 0.0f)
                    xsph_pair(S, P, r2, __ldg(&aux[j]).y, vix, viy, viz, __ldg(&vel[j]), acc, j, dt);
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
                        const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                        if (r2 < P.T && j != i)
                            xsph_pair(S, P, r2, __ldg(&aux[j]).y, vix, viy, viz, __ldg(&vel[j]),
                                      acc, j, dt);
                    }
                }
            }
    }
    const float c = eps * P.dens_coef;  // dens_coef = m * 315 / (64 pi h^9)
    const float nvx = fmaf(c, S.x, vix), nvy = fmaf(c, S.y, viy), nvz = fmaf(c, S.z, viz);
    pos_out[i] = make_float4(fmaf(dt, nvx, xi.x), fmaf(dt, nvy, xi.y), fmaf(dt, nvz, xi.z), xi.w);
    vel_out[i] = make_float4(nvx, nvy, nvz, 0.0f);
}

}  // namespace sph
