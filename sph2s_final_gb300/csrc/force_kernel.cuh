// force_kernel.cuh -- the force + integrate pass of the single-scale step.
//
// computeAccelerationsD + integrateD (SPH2S_FINAL_SINGLE_SCALE/Solver.cu:601-755,
// with the pair terms of computeAccelerationCell / computeBoundaryForceCell,
// Solver.cu:231-344).  Fluid neighbours come from the density pass's list; each
// neighbour costs two 16-byte gathers, xa[j] = (x, p/rho^2) and
// va[j] = (v, 1/rho) (the step's velocity array with 1/rho in w), and the next
// group of four indices is fetched while the current group is processed.
//
// The boundary force needs only the step's sorted positions, so the step
// computes it in boundary_force_kernel, on a second graph branch that runs
// beside the density pass, for the particles whose cell has boundary particles
// within stencil reach; the force pass then loads those sums (BSEP).  Inside
// the force pass the boundary stencil scan of a few near-wall lanes held their
// whole warps: ~21 % of the pass at 2M particles on GB300.  The sums are the
// same bit for bit (same loop, same positions).
#pragma once
#include "common.cuh"

namespace sph {

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

// One boundary particle's term: true (and accumulated) if it lies within h.
__device__ __forceinline__ bool boundary_pair(const float4& xi, const float4& xj,
                                              const SimParams& P, float& bx, float& by,
                                              float& bz) {
    float dx, dy, dz;
    const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
    if (!(r2 < P.T)) return false;
    const float rs = rsqrtf(r2);
    const float q = r2 * rs * P.two_over_h;
    const float w = P.bnd_coef * boundary_shape(q) * rs * rs;
    bx = fmaf(w, dx, bx);
    by = fmaf(w, dy, by);
    bz = fmaf(w, dz, bz);
    return true;
}

// Boundary force on a fluid particle at xi (computeBoundaryForceCell,
// Solver.cu:300-344, scaled by m_b / (m + m_b)): every boundary particle of
// the stencil within h, each cell's scan cut at the depth boundary_reach
// allows; COUNT also counts them.
template <bool COUNT>
__device__ __forceinline__ void boundary_sum(const float4& xi, const float4* __restrict__ bpos,
                                             const uint2* __restrict__ bcells, uint32_t nb,
                                             const SimParams& P, float& bx, float& by, float& bz,
                                             uint32_t& bcnt) {
    const Stencil s = stencil(P.g, xi.x, xi.y, xi.z, P.h);
    const float reach = boundary_reach(P.g, P.h, P.bmargin, xi.x, xi.y, xi.z);
    for (int cz = s.z0; cz <= s.z1; ++cz)
        for (int cy = s.y0; cy <= s.y1; ++cy) {
            const uint32_t row = linear_cell(P.g, 0, cy, cz);
            for (int cx = s.x0; cx <= s.x1; ++cx) {
                const uint2 r = __ldg(&bcells[row + cx]);
                const uint32_t e = min(r.y, nb);
                for (uint32_t j = r.x; j < e; ++j) {
                    const float4 xj = __ldg(&bpos[j]);
                    if (xj.w >= reach) break;  // the rest of the cell lies deeper
                    if (boundary_pair(xi, xj, P, bx, by, bz) && COUNT) ++bcnt;
                }
            }
        }
}

// Calls f(xk) for the boundary particles a particle at xi (home cell
// (hx, hy, hz), linear `home`) must test, in the full scan's order: from the
// home cell's static candidate list where it applies (inside the grid's box,
// stencil = home +-1 clamped; see boundary_force_kernel), else from the
// stencil scan cut by depth (boundary_reach).  A superset of the boundary
// particles within h in both cases; f applies the r < h test itself.
template <class F>
__device__ __forceinline__ void visit_boundary(const float4& xi, int hx, int hy, int hz,
                                               uint32_t home, const float4* __restrict__ bpos,
                                               const uint2* __restrict__ bcells,
                                               const uint32_t* __restrict__ bstart,
                                               const uint32_t* __restrict__ bcand, uint32_t nb,
                                               const SimParams& P, F&& f) {
    const Stencil S = stencil(P.g, xi.x, xi.y, xi.z, P.h);
    const bool inside = xi.x >= P.g.ox && xi.x < P.g.ex && xi.y >= P.g.oy && xi.y < P.g.ey &&
                        xi.z >= P.g.oz && xi.z < P.g.ez;
    if (bstart && inside && S.x0 == max(hx - 1, 0) && S.x1 == min(hx + 1, P.g.dx - 1) &&
        S.y0 == max(hy - 1, 0) && S.y1 == min(hy + 1, P.g.dy - 1) &&
        S.z0 == max(hz - 1, 0) && S.z1 == min(hz + 1, P.g.dz - 1)) {
        const uint32_t e = __ldg(&bstart[home + 1]);
        for (uint32_t k = __ldg(&bstart[home]); k < e; ++k)
            f(__ldg(&bpos[min(__ldg(&bcand[k]), nb - 1)]));
        return;
    }
    const float reach = boundary_reach(P.g, P.h, P.bmargin, xi.x, xi.y, xi.z);
    for (int cz = S.z0; cz <= S.z1; ++cz)
        for (int cy = S.y0; cy <= S.y1; ++cy) {
            const uint32_t row = linear_cell(P.g, 0, cy, cz);
            for (int cx = S.x0; cx <= S.x1; ++cx) {
                const uint2 r = __ldg(&bcells[row + cx]);
                const uint32_t e = min(r.y, nb);
                for (uint32_t j = r.x; j < e; ++j) {
                    const float4 xk = __ldg(&bpos[j]);
                    if (xk.w >= reach) break;  // the rest of the cell lies deeper
                    f(xk);
                }
            }
        }
}

// The particle's home cell in the linear cell table.
__device__ __forceinline__ uint32_t home_cell(const GridParams& g, const float4& xi) {
    return linear_cell(g, cell_coord(xi.x, g.ox, g.spacing, g.dx),
                       cell_coord(xi.y, g.oy, g.spacing, g.dy),
                       cell_coord(xi.z, g.oz, g.spacing, g.dz));
}

// Boundary sums of the particles listed by the cell-range kernel (those whose
// cell has boundary particles within stencil reach, bnear), for the force
// pass to load: bacc[i] = (b, 0).  Grid-stride over the list, or, without a
// list, over all n particles, skipping those whose cell is not flagged in
// near_all (P.g is the grid of the boundary tables).  A particle
// inside the grid's box whose stencil is its home cell +-1 (clamped) walks
// the home cell's static candidate list (bcand[bstart[c] .. bstart[c+1]):
// the boundary particles of those cells, in stencil order, that lie within
// h plus a margin of the cell's box, a superset of every such particle's
// boundary neighbours in the order of the full scan), whose loads do not
// depend on one another; any other particle scans the stencil (visit_boundary).
// Both give the full scan's sum bit for bit.  boundary_force_one is the per-particle part
// (the batched step calls it per scene with that scene's tables).
__device__ __forceinline__ void boundary_force_one(
    uint32_t i, const float4& xi, int hx, int hy, int hz, uint32_t home,
    const float4* __restrict__ bpos, const uint2* __restrict__ bcells,
    const uint32_t* __restrict__ bstart, const uint32_t* __restrict__ bcand, uint32_t nb,
    const SimParams& P, float4* __restrict__ bacc) {
    float bx = 0.f, by = 0.f, bz = 0.f;
    visit_boundary(xi, hx, hy, hz, home, bpos, bcells, bstart, bcand, nb, P,
                   [&](const float4& xk) { boundary_pair(xi, xk, P, bx, by, bz); });
    bacc[i] = make_float4(bx, by, bz, 0.0f);
}

static __global__ void __launch_bounds__(256) boundary_force_kernel(
    const float4* __restrict__ pos, const float4* __restrict__ bpos,
    const uint2* __restrict__ bcells, const uint32_t* __restrict__ bstart,
    const uint32_t* __restrict__ bcand, const uint32_t* __restrict__ list, const uint32_t* __restrict__ count, uint32_t n,
    uint32_t nb, SimParams P, float4* __restrict__ bacc,
    const uint8_t* __restrict__ near_all = nullptr) {
    const uint32_t cnt = list ? min(*count, n) : n;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
        const uint32_t i = list ? min(list[t], n - 1) : t;
        const float4 xi = pos[i];
        const int hx = cell_coord(xi.x, P.g.ox, P.g.spacing, P.g.dx);
        const int hy = cell_coord(xi.y, P.g.oy, P.g.spacing, P.g.dy);
        const int hz = cell_coord(xi.z, P.g.oz, P.g.spacing, P.g.dz);
        const uint32_t home = linear_cell(P.g, hx, hy, hz);
        if (!list && !__ldg(&near_all[home])) continue;
        boundary_force_one(i, xi, hx, hy, hz, home, bpos, bcells, bstart, bcand, nb, P, bacc);
    }
}

// Pressure (spiky gradient), viscosity (Laplacian), tension (Poly6), boundary
// force and gravity; MODE 0 integrates (symplectic Euler) into pos_out/vel_out,
// MODE 1 writes the acceleration and the boundary neighbour count instead.
// Particle i of the sorted array; cells/bcells/bnear are the particle's own
// grid tables (the batched solver passes per-scene tables and P).  BSEP: the
// boundary sums were computed by boundary_force_kernel into bacc.  nflag: the
// per-particle near-boundary flags written with the boundary pass's list
// (NearList::flag); without it the particle's cell is recomputed and looked
// up in bnear (the same answer: both test bnear of the particle's cell).
template <int MODE, bool BSEP = false>
__device__ __forceinline__ void force_one(
    uint32_t i, const float4* __restrict__ pos, const float4* __restrict__ xa,
    const float4* __restrict__ va, const uint2* __restrict__ cells, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const float4* __restrict__ bpos,
    const uint2* __restrict__ bcells, const uint8_t* __restrict__ bnear, uint32_t n, uint32_t nb,
    const SimParams& P, float dt, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
    float* __restrict__ acc_out, uint32_t* __restrict__ nbr_b,
    const float4* __restrict__ bacc = nullptr, const uint8_t* __restrict__ nflag = nullptr) {
    const float4 xi = xa[i];  // (x, y, z, p/rho^2)
    const float4 vi = va[i];  // (v, 1/rho)
    const bool listed = nflag && __ldg(&nflag[i]) != 0;
    const float tcoef = P.tens_coef * vi.w;
    ForceAcc A = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const uint32_t kc = nbr_count[i];
    if (kc <= (uint32_t)kMaxNbr) {
        // list groups are read once: streaming loads (evict-first)
        uint4 g = kc ? __ldcs(&nbr4[i]) : make_uint4(0u, 0u, 0u, 0u);
        for (uint32_t t = 0; t < kc; t += 4) {
            const uint4 gn = (t + 4 < kc) ? __ldcs(&nbr4[(size_t)((t >> 2) + 1) * n + i]) : g;
            const uint32_t js[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (t + u < kc) {
                    const uint32_t j = min(js[u], n - 1);
                    const float4 xj = __ldg(&xa[j]);
                    const float4 vj = __ldg(&va[j]);
                    float dx, dy, dz;
                    float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                    force_pair(A, P, xi.w, tcoef, vi, dx, dy, dz, r2, make_float2(xj.w, vj.w), vj);
                }
            }
            g = gn;
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
                        const float4 xj = __ldg(&xa[j]);
                        float dx, dy, dz;
                        float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                        if (r2 < P.T && r2 != 0.0f) {
                            const float4 vj = __ldg(&va[j]);
                            force_pair(A, P, xi.w, tcoef, vi, dx, dy, dz, r2,
                                       make_float2(xj.w, vj.w), vj);
                        }
                    }
                }
            }
    }
    float bx = 0.f, by = 0.f, bz = 0.f;
    uint32_t bcnt = 0;
    if (nflag ? listed : __ldg(&bnear[home_cell(P.g, xi)]) != 0) {
        if (BSEP) {
            const float4 b = bacc[i];
            bx = b.x;
            by = b.y;
            bz = b.z;
        } else {
            boundary_sum<MODE == 1>(xi, bpos, bcells, nb, P, bx, by, bz, bcnt);
        }
    }
    const float vf = P.visc_coef * vi.w;
    const float axx = fmaf(vf, A.wx, A.fx) + bx;
    const float ayy = fmaf(vf, A.wy, A.fy) + P.gravity + by;
    const float azz = fmaf(vf, A.wz, A.fz) + bz;
    if (MODE == 0) {
        float nvx = fmaf(dt, axx, vi.x), nvy = fmaf(dt, ayy, vi.y), nvz = fmaf(dt, azz, vi.z);
        pos_out[i] = make_float4(fmaf(dt, nvx, xi.x), fmaf(dt, nvy, xi.y), fmaf(dt, nvz, xi.z),
                                 pos[i].w);
        vel_out[i] = make_float4(nvx, nvy, nvz, 0.0f);
    } else {
        acc_out[3 * i + 0] = axx;
        acc_out[3 * i + 1] = ayy;
        acc_out[3 * i + 2] = azz;
        nbr_b[i] = bcnt;
    }
}

template <int MODE, bool BSEP = false>
__global__ void __launch_bounds__(256, 6) force_kernel(
    const float4* __restrict__ pos, const float4* __restrict__ xa, const float4* __restrict__ va,
    const uint2* __restrict__ cells, const uint4* __restrict__ nbr4,
    const uint32_t* __restrict__ nbr_count, const float4* __restrict__ bpos,
    const uint2* __restrict__ bcells, const uint8_t* __restrict__ bnear, uint32_t n, uint32_t nb,
    SimParams P, float dt, float4* __restrict__ pos_out, float4* __restrict__ vel_out,
    float* __restrict__ acc_out, uint32_t* __restrict__ nbr_b,
    const float4* __restrict__ bacc = nullptr, const uint8_t* __restrict__ nflag = nullptr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    force_one<MODE, BSEP>(i, pos, xa, va, cells, nbr4, nbr_count, bpos, bcells, bnear, n, nb, P,
                          dt, pos_out, vel_out, acc_out, nbr_b, bacc, nflag);
}

}  // namespace sph
