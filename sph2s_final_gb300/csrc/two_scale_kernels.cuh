// two_scale_kernels.cuh -- device kernels of the two-scale SPH2S step.
//
// Two populations: LOW (r = 0, support h, mass m) and HIGH (r = 1, support
// h/2, mass m/8), each sorted on its own grid, each particle carrying a blend
// coefficient lambda and a state (bits &3: 0 normal, 1 fading out, 2 fading
// in, 3 marked for split; bit 4: HIGH population), as in
// SPH2S_FINAL_TWO_SCALE/Solver.cu:14-20, 1163-1289.
//
// Layout per population (sorted order of the step):
//   spos float4 (x, y, z, lambda)   svel float4 (vx, vy, vz, persistent id bits)
//   sstt int32 state                sgrp uint32 group (children of one split)
// State arrays between steps: pos (x, y, z, id bits), vel (v, lambda), stt, grp.
#pragma once
#include "common.cuh"

namespace sph {

constexpr uint32_t kNoGroup = 0xFFFFFFFFu;
// Complementary-neighbour list capacity per particle: a LOW particle inside a
// refined region has ~8x34 fine neighbours within its support, a HIGH
// particle at most ~40 coarse ones.  Particles beyond it rescan the stencil.
template <int R>
struct ComplCap {
    static constexpr uint32_t value = R == 0 ? 320u : 64u;
};

struct TSParams {
    GridParams g[2];
    float h[2], h2[2], T[2];  // support, its square, neighbour threshold on r2
    float mass[2];
    float rho0, bulk, mu, sigma;
    float poly6[2];           // 315 / (64 pi h^9)
    float spiky[2];           // 45 / (pi h^6) (spiky gradient and viscosity Laplacian)
    float bnd_coef;           // 0.02 c^2 m_b / (m_LOW + m_b)
    float two_over_h0;
    float gravity;
    float blend_inc;
    int axis;                 // refinement slab axis, -1 = no slab split/merge
    float lo, hi;
    long long lo43, hi43;     // slab bounds in the group-centroid fixed point (x 2^43)
    int coupled;              // fixed populations: unit weights, no clamp, no state changes
    int surface;              // surface trigger: split / merge by rho < surf_rho
    float surf_rho;
    float bmargin;            // rounding allowance of the boundary depth cut (boundary_reach)
};

// Mexican hat wavelet of the colour output (evaluateMexicanHat3D,
// SPH2S_FINAL_TWO_SCALE/Solver.cu:206-213): c (q2 - 3) exp(-q2 / 2), q2 = |x/h|^2.
constexpr float kMexicanHatC = 0.8673250705840776f;  // 2 / (sqrt(3) pi^(1/4))

// Per-step control words on the device (written by ts_totals_kernel).
enum TSCtl {
    kCtlSurvH = 0,   // HIGH survivors
    kCtlSurvL,       // LOW survivors
    kCtlSplits,
    kCtlMerges,
    kCtlNextH,       // HIGH count after the step
    kCtlNextL,
    kCtlGroupBase,   // group ids used before the step
    kCtlPidH,        // next persistent ids
    kCtlPidL,
    kCtlFadedL,      // fade-in completions (atomic counters, cleared per step)
    kCtlFadedH,
    kCtlOverflow,    // capacity exceeded (HIGH, LOW or groups)
    kCtlErr,         // the step's device error word, read back with the counts
    kCtlWords
};

__device__ __forceinline__ long long fixed40(float x) {
    return __double2ll_rn((double)x * 1099511627776.0);
}

// Cell keys of both populations for one stable sort: LOW keys on the LOW
// grid, HIGH keys on the HIGH grid with bit `pop_bit` set, so the sorted
// array is [LOW, HIGH], each part in the order a sort of its own would give
// (SPH2S_FINAL_TWO_SCALE/Solver.cu:594-617, 1616-1661 sorts them one by one).
// Input index i < n_l is LOW particle i, otherwise HIGH particle i - n_l.
static __global__ void __launch_bounds__(256) ts_hash_hist_kernel(
    const float4* __restrict__ pos_l, uint32_t n_l, GridParams g_l,
    const float4* __restrict__ pos_h, uint32_t n_h, GridParams g_h, int pop_bit, int passes,
    uint32_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kSortMaxPasses][256];
    for (int i = threadIdx.x; i < kSortMaxPasses * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    const uint32_t n = n_l + n_h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k;
        if (i < n_l) {
            const float4 p = pos_l[i];
            k = cell_key(g_l, p.x, p.y, p.z);
        } else {
            const float4 p = pos_h[i - n_l];
            k = cell_key(g_h, p.x, p.y, p.z) | (1u << pop_bit);
        }
        keys[i] = k;
        sort_hist_add(sh, k, passes);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// Reorder + cell ranges for one population's part of the sorted array (keys
// masked by key_mask, sorted values minus val_base are its indices); for HIGH
// also accumulates the group centroid (slab axis, fixed point) and the number
// of members in state 4.
template <bool HIGH_POP>
__global__ void __launch_bounds__(256) ts_gather_kernel(
    const uint32_t* __restrict__ keys_sorted, const uint32_t* __restrict__ perm, uint32_t n,
    uint32_t key_mask, uint32_t val_base,
    GridParams g, const float4* __restrict__ pos, const float4* __restrict__ vel,
    const int32_t* __restrict__ stt, const uint32_t* __restrict__ grp, float4* __restrict__ spos,
    float4* __restrict__ svel, int32_t* __restrict__ sstt, uint32_t* __restrict__ sgrp,
    uint2* __restrict__ cells, uint32_t* __restrict__ err, int axis, int surface,
    uint32_t group_base, unsigned long long* __restrict__ gsum, uint32_t* __restrict__ gready) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t q = perm[i] - val_base;
    if (q >= n) {
        atomicOr(err, 2u);
        q = i;
    }
    const float4 p = pos[q], v = vel[q];
    spos[i] = make_float4(p.x, p.y, p.z, v.w);  // lambda in w
    svel[i] = make_float4(v.x, v.y, v.z, p.w);  // persistent id in w
    const int32_t s = stt[q];
    const uint32_t gid = grp[q];
    sstt[i] = s;
    sgrp[i] = gid;
    if (HIGH_POP && (axis >= 0 || surface) && gid != kNoGroup && gid < group_base) {
        if (axis >= 0) {
            const float xa = axis == 0 ? p.x : (axis == 1 ? p.y : p.z);
            atomicAdd(&gsum[gid], (unsigned long long)fixed40(xa));
        }
        if (s == 4) atomicAdd(&gready[gid], 1u);
    }
    const uint32_t key = keys_sorted[i] & key_mask;
    uint32_t* cw = reinterpret_cast<uint32_t*>(cells);
    const uint32_t c = morton_to_linear_checked(g, key);
    if (c == kEmptyCell) {
        atomicOr(err, 2u);
        return;
    }
    const uint32_t prev = i > 0 ? keys_sorted[i - 1] & key_mask : 0u;
    if (i == 0 || prev != key) {
        cw[2 * c] = i;
        if (i > 0) {
            const uint32_t cp = morton_to_linear_checked(g, prev);
            if (cp != kEmptyCell) cw[2 * cp + 1] = i;
        }
    }
    if (i == n - 1) cw[2 * c + 1] = n;
}

// merge[g] = all 8 members fully blended in and, for the slab trigger, the
// centroid outside the slab; for the surface trigger, no member below the
// surface density (gsum then counts those members).
static __global__ void __launch_bounds__(256) ts_group_decide_kernel(
    const unsigned long long* __restrict__ gsum, const uint32_t* __restrict__ gready,
    uint32_t group_base, long long lo43, long long hi43, int surface,
    uint32_t* __restrict__ gmerge) {
    uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= group_base) return;
    const long long s = (long long)gsum[gi];
    const bool away = surface ? s == 0 : !(lo43 < s && s < hi43);
    gmerge[gi] = (gready[gi] == 8u && away) ? 1u : 0u;
}

// Density of population r: same population weighted by lambda_j, plus the
// complementary population on its own grid with the LOW radius and the
// averaged kernel 0.5 (W_h0 + W_h1) (SPH2S_FINAL_TWO_SCALE/Solver.cu:732-845).
template <int R, bool DEBUG>
__global__ void __launch_bounds__(256) ts_density_kernel(
    const float4* __restrict__ spos_r, const uint2* __restrict__ cells_r, uint32_t n_r,
    const float4* __restrict__ spos_c, const uint2* __restrict__ cells_c, uint32_t n_c,
    TSParams P, float* __restrict__ rho, float2* __restrict__ aux, uint32_t* __restrict__ nbr_same,
    uint32_t* __restrict__ nbr_compl, const uint32_t* __restrict__ sgrp_r, uint32_t group_base,
    unsigned long long* __restrict__ gsurf, uint4* __restrict__ list4,
    uint32_t* __restrict__ list_count, uint4* __restrict__ clist4,
    uint32_t* __restrict__ clist_count) {
    constexpr int C = 1 - R;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_r) return;
    const float4 xi = spos_r[i];
    float s = 0.0f, sc = 0.0f;
    uint32_t ns = 0, nc = 0;
    // same-population force neighbours (0 < r2 < T_r) in stencil order, grouped
    // layout: element k & 3 of group k >> 2 at u32 offset 4 (g n + i) + (k & 3)
    uint32_t k = 0;
    uint32_t* out = reinterpret_cast<uint32_t*>(list4) + 4 * (size_t)i;
    const uint32_t next_group = 4u * n_r - 3u;
    {
        const Stencil st = stencil(P.g[R], xi.x, xi.y, xi.z, P.h[R]);
        for (int cz = st.z0; cz <= st.z1; ++cz)
            for (int cy = st.y0; cy <= st.y1; ++cy) {
                const uint32_t row = linear_cell(P.g[R], 0, cy, cz);
                for (int cx = st.x0; cx <= st.x1; ++cx) {
                    const uint2 r = __ldg(&cells_r[row + cx]);
                    const uint32_t e = min(r.y, n_r);
                    for (uint32_t j = r.x; j < e; ++j) {
                        const float4 xj = __ldg(&spos_r[j]);
                        float dx, dy, dz;
                        const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                        if (r2 < P.T[R]) {
                            const float a = P.h2[R] - r2;
                            s = fmaf(P.coupled ? 1.0f : xj.w, a * a * a, s);
                            if (DEBUG) ++ns;
                            if (r2 != 0.0f) {
                                if (k < (uint32_t)kMaxNbr) __stcs(out, j);  // lists: evict-first
                                out += (k & 3u) == 3u ? next_group : 1u;
                                ++k;
                            }
                        }
                    }
                }
            }
    }
    // complementary force neighbours (0 < r2 < T_0) in stencil order, same layout
    uint32_t kcl = 0;
    uint32_t* cout = reinterpret_cast<uint32_t*>(clist4) + 4 * (size_t)i;
    if (n_c > 0) {
        const Stencil st = stencil(P.g[C], xi.x, xi.y, xi.z, P.h[0]);
        for (int cz = st.z0; cz <= st.z1; ++cz)
            for (int cy = st.y0; cy <= st.y1; ++cy) {
                const uint32_t row = linear_cell(P.g[C], 0, cy, cz);
                for (int cx = st.x0; cx <= st.x1; ++cx) {
                    const uint2 r = __ldg(&cells_c[row + cx]);
                    const uint32_t e = min(r.y, n_c);
                    for (uint32_t j = r.x; j < e; ++j) {
                        const float4 xj = __ldg(&spos_c[j]);
                        float dx, dy, dz;
                        const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                        if (r2 < P.T[0]) {
                            const float a0 = P.h2[0] - r2, a1 = P.h2[1] - r2;
                            float w = P.poly6[0] * a0 * a0 * a0;
                            if (r2 < P.T[1]) w += P.poly6[1] * a1 * a1 * a1;
                            sc = fmaf(P.coupled ? 1.0f : xj.w, 0.5f * w, sc);
                            if (DEBUG) ++nc;
                            if (r2 != 0.0f) {
                                if (kcl < ComplCap<R>::value) __stcs(cout, j);
                                cout += (kcl & 3u) == 3u ? next_group : 1u;
                                ++kcl;
                            }
                        }
                    }
                }
            }
    }
    clist_count[i] = kcl;
    const float rh = P.mass[R] * P.poly6[R] * s + P.mass[C] * sc;
    const float p = P.bulk * (rh - P.rho0);
    const float inv = 1.0f / rh;
    rho[i] = rh;
    aux[i] = make_float2(p * inv * inv, inv);
    list_count[i] = k;
    if (DEBUG) {
        nbr_same[i] = ns;
        nbr_compl[i] = nc;
    }
    if (R == 1 && P.surface && rh < P.surf_rho) {  // members of a group at the surface
        const uint32_t gid = sgrp_r[i];
        if (gid != kNoGroup && gid < group_base) atomicAdd(&gsurf[gid], 1ull);
    }
}

struct TSOut {
    float4* ipos;     // (x', y', z', id bits)
    float4* ivel;     // (v', lambda')
    int32_t* istt;
    uint32_t* igrp;
    uint32_t* keep;   // survives into the next step
    uint32_t* split;  // LOW only: emits 8 children
    float* acc;       // DEBUG: accelerations (3 per particle)
    uint32_t* nbr_bnd;
    float* colour;    // colour / energy output per particle of the step's sorted order, or null
};

// Accelerations (SPH2S_FINAL_TWO_SCALE/Solver.cu:847-1048) and integration
// with the blend/state machine (Solver.cu:1163-1289) of population r.
template <int R, bool DEBUG>
__global__ void __launch_bounds__(256) ts_force_kernel(
    const float4* __restrict__ spos_r, const float4* __restrict__ svel_r,
    const int32_t* __restrict__ sstt_r, const uint32_t* __restrict__ sgrp_r,
    const float2* __restrict__ aux_r, const uint2* __restrict__ cells_r, uint32_t n_r,
    const float4* __restrict__ spos_c, const float4* __restrict__ svel_c,
    const float2* __restrict__ aux_c, const uint2* __restrict__ cells_c, uint32_t n_c,
    const float4* __restrict__ bpos, const uint2* __restrict__ bcells,
    const uint8_t* __restrict__ bnear, uint32_t nb, TSParams P,
    float dt, const uint32_t* __restrict__ gmerge, uint32_t n_groups,
    unsigned long long* __restrict__ gacc, uint32_t* __restrict__ ctl,
    const float* __restrict__ rho_r, const uint4* __restrict__ list4,
    const uint32_t* __restrict__ list_count, const uint4* __restrict__ clist4,
    const uint32_t* __restrict__ clist_count, TSOut out, const float4* __restrict__ bacc) {
    constexpr int C = 1 - R;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_r) return;
    const float4 xi = spos_r[i];
    const float4 vi = svel_r[i];
    const float2 ai = aux_r[i];
    float fx = 0.f, fy = 0.f, fz = 0.f, wx = 0.f, wy = 0.f, wz = 0.f;
    // colour output (Solver.cu:897-907, 378-387, 1050-1070): Mexican-hat velocity
    // wavelet and mass centre over the same population, self included
    const bool colour = out.colour != nullptr;
    const float psi0 = -3.0f * kMexicanHatC;
    float psum = psi0, cwx = vi.x * psi0, cwy = vi.y * psi0, cwz = vi.z * psi0;
    float csx = xi.x, csy = xi.y, csz = xi.z, ccnt = 1.0f;
    const float inv_h2 = 1.0f / P.h2[R];
    {
        const float tco = P.sigma * P.mass[R] * P.poly6[R] * ai.y;
        const float pco = P.mass[R] * P.spiky[R];
        // one same-population neighbour j (0 < r2 < T_r)
        auto pair = [&](uint32_t j, const float4& xj, float dx, float dy, float dz, float r2) {
            const float2 aj = __ldg(&aux_r[j]);
            const float4 vj = __ldg(&svel_r[j]);
            const float rs = rsqrtf(r2);
            const float hr = P.h[R] - r2 * rs;
            const float a = P.h2[R] - r2;
            const float lj = P.coupled ? 1.0f : xj.w;
            const float sc = lj * (pco * (ai.x + aj.x) * hr * hr * rs - tco * a * a * a);
            fx = fmaf(sc, dx, fx);
            fy = fmaf(sc, dy, fy);
            fz = fmaf(sc, dz, fz);
            const float vc = lj * aj.y * hr * P.spiky[R] * P.mass[R];
            wx = fmaf(vc, vj.x - vi.x, wx);
            wy = fmaf(vc, vj.y - vi.y, wy);
            wz = fmaf(vc, vj.z - vi.z, wz);
            if (colour) {
                const float q2 = r2 * inv_h2;
                const float psi = kMexicanHatC * (q2 - 3.0f) * expf(-0.5f * q2);
                psum += psi;
                cwx = fmaf(vj.x, psi, cwx);
                cwy = fmaf(vj.y, psi, cwy);
                cwz = fmaf(vj.z, psi, cwz);
                csx += xj.x;
                csy += xj.y;
                csz += xj.z;
                ccnt += 1.0f;
            }
        };
        const uint32_t kc = list_count[i];
        if (kc <= (uint32_t)kMaxNbr) {  // the density pass's list, in stencil order
            uint4 g = kc ? __ldcs(&list4[i]) : make_uint4(0u, 0u, 0u, 0u);
            for (uint32_t t = 0; t < kc; t += 4) {
                const uint4 gn = (t + 4 < kc) ? __ldcs(&list4[(size_t)((t >> 2) + 1) * n_r + i]) : g;
                const uint32_t js[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (t + u < kc) {
                        const uint32_t j = min(js[u], n_r - 1);
                        const float4 xj = __ldg(&spos_r[j]);
                        float dx, dy, dz;
                        const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                        pair(j, xj, dx, dy, dz, r2);
                    }
                }
                g = gn;
            }
        } else {
            const Stencil st = stencil(P.g[R], xi.x, xi.y, xi.z, P.h[R]);
            for (int cz = st.z0; cz <= st.z1; ++cz)
                for (int cy = st.y0; cy <= st.y1; ++cy) {
                    const uint32_t row = linear_cell(P.g[R], 0, cy, cz);
                    for (int cx = st.x0; cx <= st.x1; ++cx) {
                        const uint2 r = __ldg(&cells_r[row + cx]);
                        const uint32_t e = min(r.y, n_r);
                        for (uint32_t j = r.x; j < e; ++j) {
                            const float4 xj = __ldg(&spos_r[j]);
                            float dx, dy, dz;
                            const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                            if (r2 < P.T[R] && r2 != 0.0f) pair(j, xj, dx, dy, dz, r2);
                        }
                    }
                }
        }
    }
    if (n_c > 0) {
        // one complementary neighbour j (0 < r2 < T_0)
        auto cpair = [&](uint32_t j, const float4& xj, float dx, float dy, float dz, float r2) {
            const float2 aj = __ldg(&aux_c[j]);
            const float4 vj = __ldg(&svel_c[j]);
            const float rs = rsqrtf(r2);
            const float rr = r2 * rs;
            const bool in1 = r2 < P.T[1];
            const float h0r = P.h[0] - rr, h1r = P.h[1] - rr;
            const float a0 = P.h2[0] - r2, a1 = P.h2[1] - r2;
            float g = P.spiky[0] * h0r * h0r;
            float l = P.spiky[0] * h0r;
            float w = P.poly6[0] * a0 * a0 * a0;
            if (in1) {
                g += P.spiky[1] * h1r * h1r;
                l += P.spiky[1] * h1r;
                w += P.poly6[1] * a1 * a1 * a1;
            }
            // coupled: the neighbour support's Poly6 for tension
            // (SPH2S_FINAL_TWO_SCALE_COUPLED/Solver.cu:448-460)
            const float wt = !P.coupled ? 0.5f * w
                                        : (C == 0 ? P.poly6[0] * a0 * a0 * a0
                                                  : (in1 ? P.poly6[1] * a1 * a1 * a1 : 0.0f));
            const float lj = P.coupled ? 1.0f : xj.w;
            const float sc = lj * (P.mass[C] * (ai.x + aj.x) * 0.5f * g * rs -
                                   P.sigma * P.mass[C] * wt * ai.y);
            fx = fmaf(sc, dx, fx);
            fy = fmaf(sc, dy, fy);
            fz = fmaf(sc, dz, fz);
            const float vc = lj * P.mass[C] * aj.y * 0.5f * l;
            wx = fmaf(vc, vj.x - vi.x, wx);
            wy = fmaf(vc, vj.y - vi.y, wy);
            wz = fmaf(vc, vj.z - vi.z, wz);
        };
        const uint32_t kc = clist_count[i];
        if (kc <= ComplCap<R>::value) {  // the density pass's list, in stencil order
            uint4 gc = kc ? __ldcs(&clist4[i]) : make_uint4(0u, 0u, 0u, 0u);
            for (uint32_t t = 0; t < kc; t += 4) {
                const uint4 g = gc;  // this group; the next one is fetched meanwhile
                gc = (t + 4 < kc) ? __ldcs(&clist4[(size_t)((t >> 2) + 1) * n_r + i]) : g;
                const uint32_t js[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (t + u < kc) {
                        const uint32_t j = min(js[u], n_c - 1);
                        const float4 xj = __ldg(&spos_c[j]);
                        float dx, dy, dz;
                        const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                        cpair(j, xj, dx, dy, dz, r2);
                    }
                }
            }
        } else {
            const Stencil st = stencil(P.g[C], xi.x, xi.y, xi.z, P.h[0]);
            for (int cz = st.z0; cz <= st.z1; ++cz)
                for (int cy = st.y0; cy <= st.y1; ++cy) {
                    const uint32_t row = linear_cell(P.g[C], 0, cy, cz);
                    for (int cx = st.x0; cx <= st.x1; ++cx) {
                        const uint2 r = __ldg(&cells_c[row + cx]);
                        const uint32_t e = min(r.y, n_c);
                        for (uint32_t j = r.x; j < e; ++j) {
                            const float4 xj = __ldg(&spos_c[j]);
                            float dx, dy, dz;
                            const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                            if (r2 < P.T[0] && r2 != 0.0f) cpair(j, xj, dx, dy, dz, r2);
                        }
                    }
                }
        }
    }
    float bx = 0.f, by = 0.f, bz = 0.f;
    uint32_t bcnt = 0;
    // the boundary stencil lives on the LOW grid; particles of LOW cells with no
    // boundary particle within stencil reach skip it (bnear, set once at creation).
    // With bacc the step computed the sums beside the density passes
    // (boundary_force_kernel, the same bits).
    const uint32_t bhome = linear_cell(P.g[0], cell_coord(xi.x, P.g[0].ox, P.g[0].spacing, P.g[0].dx),
                                       cell_coord(xi.y, P.g[0].oy, P.g[0].spacing, P.g[0].dy),
                                       cell_coord(xi.z, P.g[0].oz, P.g[0].spacing, P.g[0].dz));
    if (!DEBUG && bacc != nullptr) {
        if (__ldg(&bnear[bhome])) {
            const float4 b = bacc[i];
            bx = b.x;
            by = b.y;
            bz = b.z;
        }
    } else if (__ldg(&bnear[bhome])) {
        const Stencil st = stencil(P.g[0], xi.x, xi.y, xi.z, P.h[0]);
        const float reach = boundary_reach(P.g[0], P.h[0], P.bmargin, xi.x, xi.y, xi.z);
        for (int cz = st.z0; cz <= st.z1; ++cz)
            for (int cy = st.y0; cy <= st.y1; ++cy) {
                const uint32_t row = linear_cell(P.g[0], 0, cy, cz);
                for (int cx = st.x0; cx <= st.x1; ++cx) {
                    const uint2 r = __ldg(&bcells[row + cx]);
                    const uint32_t e = min(r.y, nb);
                    for (uint32_t j = r.x; j < e; ++j) {
                        const float4 xj = __ldg(&bpos[j]);
                        if (xj.w >= reach) break;  // the rest of the cell lies deeper
                        float dx, dy, dz;
                        const float r2 = dist2(xi.x, xi.y, xi.z, xj.x, xj.y, xj.z, dx, dy, dz);
                        if (r2 < P.T[0]) {
                            const float rs = rsqrtf(r2);
                            const float w = P.bnd_coef * boundary_shape(r2 * rs * P.two_over_h0) * rs * rs;
                            bx = fmaf(w, dx, bx);
                            by = fmaf(w, dy, by);
                            bz = fmaf(w, dz, bz);
                            if (DEBUG) ++bcnt;
                        }
                    }
                }
            }
    }
    // f / rho_i: the pressure terms carry rho_i * (1/rho_i) = 1 already and the
    // tension terms folded 1/rho_i in; the viscosity sum still needs mu / rho_i.
    const float vf = P.mu * ai.y;
    const float axx = fmaf(vf, wx, fx) + bx;
    const float ayy = fmaf(vf, wy, fy) + P.gravity + by;
    const float azz = fmaf(vf, wz, fz) + bz;
    if (DEBUG) {
        out.acc[3 * i + 0] = axx;
        out.acc[3 * i + 1] = ayy;
        out.acc[3 * i + 2] = azz;
        out.nbr_bnd[i] = bcnt;
    }
    if (colour) {  // Solver.cu:1050-1070
        const float inv_c = 1.0f / ccnt;
        const float ex = xi.x - csx * inv_c, ey = xi.y - csy * inv_c, ez = xi.z - csz * inv_c;
        const float dist_cm = sqrtf(ex * ex + ey * ey + ez * ez);
        float ene = (cwx * cwx + cwy * cwy + cwz * cwz) / (psum * psum * P.h[R]);
        ene = fminf(ene, 300.0f);
        out.colour[i] = dist_cm < 0.0025f ? 0.3f : ene / 300.0f;
    }
    // integrate with the velocity clamp |v| <= 0.8 h_r / dt (Solver.cu:1207-1227);
    // the coupled solver integrates without it (SPH2S_FINAL_TWO_SCALE_COUPLED/Solver.cu:930-970)
    float nvx = fmaf(dt, axx, vi.x), nvy = fmaf(dt, ayy, vi.y), nvz = fmaf(dt, azz, vi.z);
    const float norm = sqrtf(nvx * nvx + nvy * nvy + nvz * nvz);
    const float vmax = 0.8f * P.h[R] / dt;
    if (!P.coupled && norm > vmax) {
        const float sc = vmax / norm;
        nvx *= sc;
        nvy *= sc;
        nvz *= sc;
    }
    const float px = fmaf(dt, nvx, xi.x), py = fmaf(dt, nvy, xi.y), pz = fmaf(dt, nvz, xi.z);
    // blend coefficient and state machine (Solver.cu:1242-1288)
    int32_t state = sstt_r[i];
    uint32_t group = sgrp_r[i];
    if (R == 0 && P.axis >= 0 && (state & 3) == 0) {
        const float xa = P.axis == 0 ? xi.x : (P.axis == 1 ? xi.y : xi.z);
        if (P.lo < xa && xa < P.hi) state = (state & 4) | 3;
    }
    if (R == 0 && P.surface && (state & 3) == 0 && rho_r[i] < P.surf_rho) state = (state & 4) | 3;
    const int sb = P.coupled ? 0 : (state & 3);
    const float cb = sb == 1 ? -1.0f : (sb == 2 ? 1.0f : 0.0f);
    float lam = __fadd_rn(xi.w, __fmul_rn(cb, P.blend_inc));
    uint32_t keep = 1u, split = 0u;
    if (lam <= 0.0f && sb == 1) keep = 0u;
    if (keep && lam >= 1.0f && sb == 2) {
        state &= 4;
        lam = 1.0f;
        atomicAdd(&ctl[R == 0 ? kCtlFadedL : kCtlFadedH], 1u);
    }
    if (keep && R == 0 && !P.coupled && (state & 3) == 3) {
        split = 1u;
        state = 1;
    }
    if (keep && R == 1 && group < n_groups && gmerge != nullptr && gmerge[group]) {
        unsigned long long* gsl = gacc + 6 * (size_t)group;
        atomicAdd(&gsl[0], (unsigned long long)fixed40(px));
        atomicAdd(&gsl[1], (unsigned long long)fixed40(py));
        atomicAdd(&gsl[2], (unsigned long long)fixed40(pz));
        atomicAdd(&gsl[3], (unsigned long long)fixed40(nvx));
        atomicAdd(&gsl[4], (unsigned long long)fixed40(nvy));
        atomicAdd(&gsl[5], (unsigned long long)fixed40(nvz));
        state = 5;
        group = kNoGroup;
    }
    out.ipos[i] = make_float4(px, py, pz, vi.w);
    out.ivel[i] = make_float4(nvx, nvy, nvz, lam);
    out.istt[i] = state;
    out.igrp[i] = group;
    out.keep[i] = keep;
    if (R == 0) out.split[i] = split;
}

// Counts of the step from the scans; checks capacities.  One thread.
static __global__ void ts_totals_kernel(const uint32_t* __restrict__ tot, uint32_t n_high, uint32_t n_low,
                                 uint32_t cap_high, uint32_t cap_low, uint32_t cap_groups,
                                 uint32_t* __restrict__ ctl, uint32_t* __restrict__ err) {
    // tot[0] = HIGH survivors, tot[1] = LOW survivors, tot[2] = splits, tot[3] = merges
    const uint32_t sH = n_high ? tot[0] : 0u, sL = n_low ? tot[1] : 0u;
    const uint32_t ns = n_low ? tot[2] : 0u, nm = tot[3];
    ctl[kCtlSurvH] = sH;
    ctl[kCtlSurvL] = sL;
    ctl[kCtlSplits] = ns;
    ctl[kCtlMerges] = nm;
    uint64_t nh = (uint64_t)sH + 8ull * ns, nl = (uint64_t)sL + nm;
    const uint32_t gb = ctl[kCtlGroupBase];
    uint32_t ov = 0;
    if (nh > cap_high || nl > cap_low || (uint64_t)gb + ns > cap_groups) ov = 1;
    ctl[kCtlOverflow] = ov;
    if (ov) atomicOr(err, 4u);
    ctl[kCtlNextH] = (uint32_t)(nh > cap_high ? cap_high : nh);
    ctl[kCtlNextL] = (uint32_t)(nl > cap_low ? cap_low : nl);
}

// Survivors -> state arrays at their compacted positions.
__device__ __forceinline__ void ts_compact_one(uint32_t i, const TSOut& o,
                                               const uint32_t* __restrict__ off, uint32_t cap,
                                               float4* __restrict__ pos, float4* __restrict__ vel,
                                               int32_t* __restrict__ stt,
                                               uint32_t* __restrict__ grp) {
    if (!o.keep[i]) return;
    const uint32_t d = off[i];
    if (d >= cap) return;
    pos[d] = o.ipos[i];
    vel[d] = o.ivel[i];
    stt[d] = o.istt[i];
    grp[d] = o.igrp[i];
}

// Eight HIGH children per split LOW particle, after the HIGH survivors, in the
// sorted order of their parents (insertHighResParticles,
// SPH2S_FINAL_TWO_SCALE/Solver.cu:541-586: radius 0.5 (3 m / (4 pi rho))^(1/3),
// directions (+-1, +-1, +-1)/sqrt(3), parent velocity, lambda 0, state 6).
__device__ __forceinline__ void ts_children_one(uint32_t i, const TSOut& o,
                                                const uint32_t* __restrict__ split_off,
                                                const float* __restrict__ rho_low, float mass_low,
                                                const uint32_t* __restrict__ ctl, uint32_t cap_high,
                                                float4* __restrict__ pos_h, float4* __restrict__ vel_h,
                                                int32_t* __restrict__ stt_h,
                                                uint32_t* __restrict__ grp_h) {
    if (!o.split[i]) return;
    const uint32_t q = split_off[i];
    const uint32_t base = ctl[kCtlSurvH] + 8u * q;
    const float4 x = o.ipos[i], v = o.ivel[i];
    const float rs = 0.5f * cbrtf(3.0f / (4.0f * 3.14159265358979f) * mass_low / rho_low[i]);
    const float d = 0.57735026919f * rs;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t dst = base + (uint32_t)k;
        if (dst >= cap_high) return;
        const float sx = (k & 4) ? -d : d, sy = (k & 2) ? -d : d, sz = (k & 1) ? -d : d;
        const uint32_t pid = ctl[kCtlPidH] + 8u * q + (uint32_t)k;
        pos_h[dst] = make_float4(x.x + sx, x.y + sy, x.z + sz, __uint_as_float(pid));
        vel_h[dst] = make_float4(v.x, v.y, v.z, 0.0f);
        stt_h[dst] = 6;
        grp_h[dst] = ctl[kCtlGroupBase] + q;
    }
}

// One LOW particle per merged group, after the LOW survivors, by group id.
__device__ __forceinline__ void ts_merge_spawn_one(
    uint32_t gi, const uint32_t* __restrict__ gmerge, const uint32_t* __restrict__ merge_off,
    const unsigned long long* __restrict__ gacc, const uint32_t* __restrict__ ctl,
    uint32_t cap_low, float4* __restrict__ pos_l, float4* __restrict__ vel_l,
    int32_t* __restrict__ stt_l, uint32_t* __restrict__ grp_l) {
    if (!gmerge[gi]) return;
    const uint32_t m = merge_off[gi];
    const uint32_t dst = ctl[kCtlSurvL] + m;
    if (dst >= cap_low) return;
    const unsigned long long* s = gacc + 6 * (size_t)gi;
    const double inv = 1.0 / (8.0 * 1099511627776.0);
    float f[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) f[k] = (float)((double)(long long)s[k] * inv);
    pos_l[dst] = make_float4(f[0], f[1], f[2], __uint_as_float(ctl[kCtlPidL] + m));
    vel_l[dst] = make_float4(f[3], f[4], f[5], 0.0f);
    stt_l[dst] = 2;
    grp_l[dst] = kNoGroup;
}

// The next step's state arrays of one population.
struct TSState {
    float4* pos;
    float4* vel;
    int32_t* stt;
    uint32_t* grp;
    uint32_t cap;
};

// Everything that builds the next state after the prefix sums, in one launch
// over [HIGH particles | LOW particles | groups]: survivors to their compacted
// slots, the split children after the HIGH survivors, merged particles after
// the LOW survivors.
static __global__ void __launch_bounds__(256) ts_finish_kernel(
    const TSOut oh, const uint32_t* __restrict__ off_h, uint32_t n_h, const TSOut ol,
    const uint32_t* __restrict__ off_l, const uint32_t* __restrict__ split_off,
    const float* __restrict__ rho_l, uint32_t n_l, float mass_low,
    const uint32_t* __restrict__ gmerge, const uint32_t* __restrict__ merge_off,
    const unsigned long long* __restrict__ gacc, uint32_t n_groups,
    const uint32_t* __restrict__ ctl, TSState H, TSState L) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_h) {
        ts_compact_one(i, oh, off_h, H.cap, H.pos, H.vel, H.stt, H.grp);
        return;
    }
    i -= n_h;
    if (i < n_l) {
        ts_compact_one(i, ol, off_l, L.cap, L.pos, L.vel, L.stt, L.grp);
        ts_children_one(i, ol, split_off, rho_l, mass_low, ctl, H.cap, H.pos, H.vel, H.stt, H.grp);
        return;
    }
    i -= n_l;
    if (i < n_groups)
        ts_merge_spawn_one(i, gmerge, merge_off, gacc, ctl, L.cap, L.pos, L.vel, L.stt, L.grp);
}

// Advances the persistent counters after the step; the group count saturates
// at the group capacity (the overflow was already reported).  One thread.
static __global__ void ts_advance_counters_kernel(uint32_t* ctl, uint32_t cap_groups,
                                                  const uint32_t* err) {
    ctl[kCtlErr] = *(volatile const uint32_t*)err;  // the last kernel of the step
    ctl[kCtlPidH] += 8u * ctl[kCtlSplits];
    ctl[kCtlPidL] += ctl[kCtlMerges];
    const uint64_t gb = (uint64_t)ctl[kCtlGroupBase] + ctl[kCtlSplits];
    ctl[kCtlGroupBase] = (uint32_t)(gb > cap_groups ? cap_groups : gb);
}

}  // namespace sph
