// density_kernel.cuh -- the density pass of the single-scale step.
//
// computeDensitiesPressuresD + computeDensityCell (SPH2S_FINAL_SINGLE_SCALE/
// Solver.cu:536-599, 198-229): rho_i = m sum_j W_poly6(r_ij) over the stencil
// [cell(x - h), cell(x + h)] with r < h (self included), p_i = K (rho_i - rho0).
//
// Besides rho and the factors the force pass needs from every neighbour
// (p/rho^2, 1/rho, in aux), it writes the force pass's per-neighbour records:
// xa[i] = (x, y, z, p/rho^2) and the w slot of the step's velocity,
// svel[i].w = 1/rho, so the force pass gathers two 16-byte records per
// neighbour instead of three loads.  It also emits the neighbour list: every j with
// 0 < r2 < T, in stencil order.  Lists are stored transposed in groups of
// four, group g of particle i at nbr4[g * n + i], so the force pass reads 512
// contiguous bytes per warp instruction; the density pass stores each index
// as it is found (one 4-byte store into its slot, cheaper per hit than
// assembling groups in registers: 0.68 -> 0.58 ms at 2M particles on GB300).
// The list traffic (~136 bytes per particle, read once by the force pass) is
// stored and loaded with streaming (evict-first) cache hints, so it displaces
// less of the force records the force pass gathers from L2 (2M step
// 0.837 -> 0.830 ms).
// nbr_count[i] may exceed kMaxNbr; the force pass then
// rescans the stencil for that particle.
//
// One thread per particle, particles in Morton order (a warp's particles
// share most of their stencil cells, so candidate loads hit in L1).  Measured
// alternatives that were slower on GB300 at 2M particles: a warp-cooperative
// scan of the warp's union stencil through shared memory (Morton order puts
// about a quarter of all warps across octant jumps, whose union boxes hold
// hundreds of cells), Morton-contiguous multi-cell runs (parity-dependent
// control flow diverges inside a warp), and branch-free hit masks with
// deferred list appends.
#pragma once
#include "common.cuh"

namespace sph {

constexpr int kDensityThreads = 256;

// Density of particle i of the sorted array (n particles, indices in `cells`
// refer to that array); the batched solver calls this with per-scene P and
// cell table.
template <bool DEBUG>
__device__ __forceinline__ void density_one(uint32_t i, const float4* __restrict__ pos,
                                            const uint2* __restrict__ cells, uint32_t n,
                                            const SimParams& P, float* __restrict__ rho,
                                            float2* __restrict__ aux, uint4* __restrict__ nbr4,
                                            uint32_t* __restrict__ nbr_count,
                                            uint32_t* __restrict__ dbg_count,
                                            float4* __restrict__ xa, float4* __restrict__ svel) {
    uint32_t k = 0, zero = 0;
    float sum = 0.0f;
    const float4 xi = pos[i];
    // next list slot: element k & 3 of group k >> 2, i.e. u32 offset 4 (g n + i) + (k & 3)
    uint32_t* out = reinterpret_cast<uint32_t*>(nbr4) + 4 * (size_t)i;
    const uint32_t next_group = 4u * n - 3u;  // fits 32 bits: n <= 2^30
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
                    if (r2 < P.T) {
                        const float a = P.h2 - r2;
                        sum = fmaf(a * a, a, sum);
                        if (r2 != 0.0f) {
                            if (k < (uint32_t)kMaxNbr) __stcs(out, j);  // evict-first
                            out += (k & 3u) == 3u ? next_group : 1u;
                            ++k;
                        } else {
                            ++zero;
                        }
                    }
                }
            }
        }
    const float rh = P.dens_coef * sum;
    const float p = P.bulk * (rh - P.rho0);
    const float inv = 1.0f / rh;
    rho[i] = rh;
    aux[i] = make_float2(p * inv * inv, inv);
    xa[i] = make_float4(xi.x, xi.y, xi.z, p * inv * inv);
    reinterpret_cast<float*>(svel + i)[3] = inv;
    nbr_count[i] = k;
    if (DEBUG) dbg_count[i] = k + zero;
}

template <bool DEBUG>
__global__ void __launch_bounds__(kDensityThreads) density_kernel(
    const float4* __restrict__ pos, const uint2* __restrict__ cells, uint32_t n, SimParams P,
    float* __restrict__ rho, float2* __restrict__ aux, uint4* __restrict__ nbr4,
    uint32_t* __restrict__ nbr_count, uint32_t* __restrict__ dbg_count, float4* __restrict__ xa,
    float4* __restrict__ svel) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    density_one<DEBUG>(i, pos, cells, n, P, rho, aux, nbr4, nbr_count, dbg_count, xa, svel);
}

}  // namespace sph
