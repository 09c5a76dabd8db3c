// ============================================================================
// sph_oracle.cpp -- FP64 CPU restatement of the SPH2S single-scale particle
// step.  TEST INFRASTRUCTURE ONLY: the test suite, the smoke check and the CPU
// baseline leg of bench.py load this library as the checker.  The product
// (libsph2s.so) never links, loads or calls it.
//
// What it restates (file:line within segfault11/SPH2S_FINAL):
//   * cell coordinates, clamping, stencil       SPH2S_FINAL_SINGLE_SCALE/Solver.cu:20-83
//   * Poly6 / spiky / viscosity / boundary       SPH2S_FINAL_SINGLE_SCALE/Solver.cu:103-196
//   * density + linear EOS                       SPH2S_FINAL_SINGLE_SCALE/Solver.cu:198-229, 536-599
//   * pressure/viscosity/tension + boundary      SPH2S_FINAL_SINGLE_SCALE/Solver.cu:231-344, 601-711
//   * symplectic Euler, output in sorted order   SPH2S_FINAL_SINGLE_SCALE/Solver.cu:713-755
//   * step order hash -> sort -> reorder -> rho -> a -> integrate
//                                                SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1082-1198
//   * boundary sorted once on the fluid grid     SPH2S_FINAL_SINGLE_SCALE/Solver.cu:989-1061
//   * grid / configuration                       SPH2S_FINAL_SINGLE_SCALE/Grid.h:11-46, Solver.h:15-48
//
// Precision contract.  Physics sums, kernels and the integrator run in double.
// The structural predicates -- cell coordinates, the stencil bounds, and the
// "r < h" neighbour test -- run in FP32 with single-rounded operations in a
// fixed order, exactly as the GPU kernels evaluate them, so that cell keys,
// sorted order and neighbour counts can be compared bit for bit:
//   cell(x, off) = clamp((int)(((x + off) - o) / s), 0, D-1)   (FP32, trunc)
//   r2           = fmaf(dz, dz, fmaf(dy, dy, dx*dx)),  d = xi - xj (FP32)
//   neighbour    <=>  r2 < T,  T = min{ t : sqrtf(t) >= h }
// The last line is equivalent to the reference's sqrtf(r2) < h because sqrtf
// is correctly rounded and monotone.  This file must be compiled with
// -ffp-contract=off so the compiler does not fuse any other operation.
//
// Sort order.  The reference sorts uniform-grid hashes cx + Dx(cy + Dy cz)
// with thrust::sort_by_key (Solver.cu:1110-1115).  The GB300 build sorts by
// the Morton code of the same (cx, cy, cz) and defines ties by the previous
// array position (a stable sort); this oracle does the same.  Cell tables are
// indexed by the reference's linear hash.
//
// Parity pins: the reference ships no tests, fixtures or golden vectors and
// cannot run as a program here (CUDA 5.0 / Windows / OpenGL, no CPU path), but
// its single-scale device code compiles unmodified for sm_103a
// (oracle/ref_build.py) and runs on the GPU under oracle/ref_harness.cu, which
// replays its host sequence.  tests/golden/ref_*.npz hold those outputs and
// tests/test_oracle_vs_reference.py checks this restatement against them
// (hashes and sorted order bit-exact, fields to ~3e-7); tests/test_oracle.py
// adds known-answer cases derived by hand from the reference formulas.  The
// sort is a third-party dependency of the reference (Thrust, bundled with
// CUDA 5.0, not vendored); its only contract used here is "ascending by key",
// with ties in input order.
// ============================================================================
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <algorithm>
#include <numeric>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.h"

namespace {

using namespace oracle;

// ---- single-scale fields for an arbitrary float state -----------------------

struct Boundary {
    std::vector<float> xf;      // sorted float positions (3 per particle)
    std::vector<double> xd;     // sorted double positions
    SortedSet set;
};

void make_boundary(const OGrid& g, const float* bxyz, size_t nb, Boundary& B) {
    sort_set(g, bxyz, nb, B.set);
    B.xf.resize(3 * nb);
    B.xd.resize(3 * nb);
    for (size_t k = 0; k < nb; ++k)
        for (int a = 0; a < 3; ++a) {
            B.xf[3 * k + a] = bxyz[3 * B.set.perm[k] + a];
            B.xd[3 * k + a] = (double)B.xf[3 * k + a];
        }
}

// Density, pressure and acceleration for fluid particles given in SORTED order
// (xf/xd/v index k, cells built on the same order).  Outputs in sorted order.
void fields_sorted(const OConfig& C, const std::vector<float>& xf, const std::vector<double>& xd,
                   const std::vector<double>& v, const CellList& cl, const Boundary& B,
                   std::vector<double>& rho, std::vector<double>& acc,
                   std::vector<uint32_t>* nbr_f, std::vector<uint32_t>* nbr_b) {
    const OGrid& g = C.grid;
    const size_t n = xf.size() / 3;
    const float h = C.effective_radius;
    const float T = thresh_sq(h);
    const Kern K((double)h);
    const double m = C.fluid_particle_mass, mb = C.boundary_particle_mass;
    const double rho0 = C.rest_density, bulk = C.bulk_modulus;
    const double mu = C.viscosity, sigma = C.tension_coefficient, c = C.speed_sound;
    rho.assign(n, 0.0);
    acc.assign(3 * n, 0.0);
    std::vector<double> p(n);
    if (nbr_f) nbr_f->assign(n, 0);
    if (nbr_b) nbr_b->assign(n, 0);

    // density + pressure: Solver.cu:536-599 (self included, r < h)
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        const float* xi = &xf[3 * i];
        double s = 0.0;
        uint32_t cnt = 0;
        for_stencil(g, cl, xi, h, [&](uint32_t j) {
            if (r2_f32(xi, &xf[3 * j]) < T) {
                double dx = xd[3 * i] - xd[3 * j], dy = xd[3 * i + 1] - xd[3 * j + 1],
                       dz = xd[3 * i + 2] - xd[3 * j + 2];
                s += K.W(std::sqrt(dx * dx + dy * dy + dz * dz));
                ++cnt;
            }
        });
        rho[i] = m * s;
        p[i] = bulk * (rho[i] - rho0);
        if (nbr_f) (*nbr_f)[i] = cnt;
    }

    // accelerations: Solver.cu:601-711 (fluid: r != 0 && r < h; boundary: r < h)
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        const float* xi = &xf[3 * i];
        const double ri = rho[i], pi = p[i];
        double f[3] = {0, 0, 0}, b[3] = {0, 0, 0};
        for_stencil(g, cl, xi, h, [&](uint32_t j) {
            float r2 = r2_f32(xi, &xf[3 * j]);
            if (r2 != 0.0f && r2 < T) {
                double d[3] = {xd[3 * i] - xd[3 * j], xd[3 * i + 1] - xd[3 * j + 1],
                               xd[3 * i + 2] - xd[3 * j + 2]};
                double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                double coeffP = -ri * m * (pi / (ri * ri) + p[j] / (rho[j] * rho[j]));
                double gw = K.gradW_factor(r);
                double coeffV = mu * m / rho[j] * K.lapl(r);
                double coeffT = -K.W(r) * m * sigma;
                for (int a = 0; a < 3; ++a)
                    f[a] += coeffP * gw * d[a] + coeffV * (v[3 * j + a] - v[3 * i + a]) +
                            coeffT * d[a];
            }
        });
        uint32_t bc = 0;
        for_stencil(g, B.set.cells, xi, h, [&](uint32_t j) {
            if (r2_f32(xi, &B.xf[3 * j]) < T) {
                double d[3] = {xd[3 * i] - B.xd[3 * j], xd[3 * i + 1] - B.xd[3 * j + 1],
                               xd[3 * i + 2] - B.xd[3 * j + 2]};
                double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                double w = boundary_weight(r, (double)h, c) * mb / (m + mb);
                for (int a = 0; a < 3; ++a) b[a] += w * d[a] / r;
                ++bc;
            }
        });
        acc[3 * i + 0] = f[0] / ri + b[0];
        acc[3 * i + 1] = f[1] / ri - 9.81 + b[1];
        acc[3 * i + 2] = f[2] / ri + b[2];
        if (nbr_b) (*nbr_b)[i] = bc;
    }
}

// ---- rollout state --------------------------------------------------------

struct SSState {
    OConfig C;
    Boundary B;
    std::vector<double> x, v, rho;
    std::vector<uint32_t> ids;
};

void ss_step(SSState& S, double dt) {
    const size_t n = S.ids.size();
    std::vector<float> xf(3 * n);
    for (size_t i = 0; i < 3 * n; ++i) xf[i] = (float)S.x[i];
    SortedSet set;
    sort_set(S.C.grid, xf.data(), n, set);
    std::vector<float> xs(3 * n);
    std::vector<double> xd(3 * n), vd(3 * n);
    std::vector<uint32_t> ids(n);
    for (size_t k = 0; k < n; ++k) {
        uint32_t q = set.perm[k];
        for (int a = 0; a < 3; ++a) {
            xs[3 * k + a] = xf[3 * q + a];
            xd[3 * k + a] = S.x[3 * q + a];
            vd[3 * k + a] = S.v[3 * q + a];
        }
        ids[k] = S.ids[q];
    }
    std::vector<double> rho, acc;
    fields_sorted(S.C, xs, xd, vd, set.cells, S.B, rho, acc, nullptr, nullptr);
    // Solver.cu:713-755: v += dt a; x += dt v (new v); written in sorted order.
    for (size_t k = 0; k < n; ++k)
        for (int a = 0; a < 3; ++a) {
            vd[3 * k + a] += dt * acc[3 * k + a];
            xd[3 * k + a] += dt * vd[3 * k + a];
        }
    S.x.swap(xd);
    S.v.swap(vd);
    S.ids.swap(ids);
    S.rho.swap(rho);
}

}  // namespace

// ============================================================================
// extern "C" surface used by oracle/oracle.py
// ============================================================================
extern "C" {

float or_thresh_sq(float h) { return thresh_sq(h); }

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_num_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

int or_morton_bits(const OGrid* g) { return morton_bits(*g); }

// Per particle: Morton key and linear cell index of its cell (Solver.cu:40-83).
void or_cell_keys(const OGrid* g, const float* xyz, uint32_t n, uint32_t* keys, uint32_t* lin) {
    for (uint32_t i = 0; i < n; ++i) {
        int cx = cell_coord(xyz[3 * i + 0], g->origin[0], g->spacing, g->dims[0]);
        int cy = cell_coord(xyz[3 * i + 1], g->origin[1], g->spacing, g->dims[1]);
        int cz = cell_coord(xyz[3 * i + 2], g->origin[2], g->spacing, g->dims[2]);
        if (keys) keys[i] = morton(cx, cy, cz);
        if (lin) lin[i] = linear_cell(*g, cx, cy, cz);
    }
}

// Stencil bounds [cs, ce] per axis for a radius h (Solver.cu:559-570).
void or_stencil(const OGrid* g, const float* xyz, uint32_t n, float h, int32_t* cs, int32_t* ce) {
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            cs[3 * i + a] = cell_coord_off(xyz[3 * i + a], -h, g->origin[a], g->spacing, g->dims[a]);
            ce[3 * i + a] = cell_coord_off(xyz[3 * i + a], h, g->origin[a], g->spacing, g->dims[a]);
        }
}

// Neighbourhood structure of a float position set in its given order:
// stable Morton sort (perm, sorted keys) and the per-cell [start, end) table.
void or_neighborhood(const OGrid* g, const float* xyz, uint32_t n, uint32_t* perm,
                     uint32_t* keys_sorted, uint32_t* cell_start, uint32_t* cell_end) {
    SortedSet s;
    sort_set(*g, xyz, n, s);
    if (perm) std::memcpy(perm, s.perm.data(), n * 4);
    if (keys_sorted) std::memcpy(keys_sorted, s.keys.data(), n * 4);
    size_t nc = (size_t)g->dims[0] * g->dims[1] * g->dims[2];
    if (cell_start) std::memcpy(cell_start, s.cells.start.data(), nc * 4);
    if (cell_end) std::memcpy(cell_end, s.cells.end.data(), nc * 4);
}

// Single-scale density, acceleration and neighbour counts for one float state
// (positions/velocities in any order; outputs in that same input order).
void or_ss_fields(const OConfig* C, const float* fxyz, const float* fvel, uint32_t n,
                  const float* bxyz, uint32_t nb, double* rho_out, double* acc_out,
                  uint32_t* nbr_f_out, uint32_t* nbr_b_out) {
    Boundary B;
    make_boundary(C->grid, bxyz, nb, B);
    SortedSet s;
    sort_set(C->grid, fxyz, n, s);
    std::vector<float> xs(3 * (size_t)n);
    std::vector<double> xd(3 * (size_t)n), vd(3 * (size_t)n);
    for (uint32_t k = 0; k < n; ++k)
        for (int a = 0; a < 3; ++a) {
            xs[3 * k + a] = fxyz[3 * s.perm[k] + a];
            xd[3 * k + a] = (double)xs[3 * k + a];
            vd[3 * k + a] = fvel ? (double)fvel[3 * s.perm[k] + a] : 0.0;
        }
    std::vector<double> rho, acc;
    std::vector<uint32_t> nf, nbb;
    fields_sorted(*C, xs, xd, vd, s.cells, B, rho, acc, &nf, &nbb);
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t q = s.perm[k];
        if (rho_out) rho_out[q] = rho[k];
        for (int a = 0; a < 3; ++a)
            if (acc_out) acc_out[3 * q + a] = acc[3 * k + a];
        if (nbr_f_out) nbr_f_out[q] = nf[k];
        if (nbr_b_out) nbr_b_out[q] = nbb[k];
    }
}

// One step with the XSPH integrator from a float state (any order; outputs in
// that order): integrateXSPHD + computeVelXSPHCell, SPH2S_FINAL_SINGLE_SCALE/
// Solver.cu:345-395, 757-853, with the velocity correction applied per
// component (the reference adds its x component to all three):
//   v' = v + dt a,  v'' = v' + eps sum_{r<h} (v'_j - v'_i) m/rho_j W(r),  x' = x + dt v''.
void or_ss_xsph_step(const OConfig* C, const float* fxyz, const float* fvel, uint32_t n,
                     const float* bxyz, uint32_t nb, double dt, double eps, double* x_out,
                     double* v_out) {
    Boundary B;
    make_boundary(C->grid, bxyz, nb, B);
    SortedSet s;
    sort_set(C->grid, fxyz, n, s);
    std::vector<float> xs(3 * (size_t)n);
    std::vector<double> xd(3 * (size_t)n), vd(3 * (size_t)n);
    for (uint32_t k = 0; k < n; ++k)
        for (int a = 0; a < 3; ++a) {
            xs[3 * k + a] = fxyz[3 * s.perm[k] + a];
            xd[3 * k + a] = (double)xs[3 * k + a];
            vd[3 * k + a] = fvel ? (double)fvel[3 * s.perm[k] + a] : 0.0;
        }
    std::vector<double> rho, acc;
    fields_sorted(*C, xs, xd, vd, s.cells, B, rho, acc, nullptr, nullptr);
    std::vector<double> vp(3 * (size_t)n);
    for (size_t k = 0; k < 3 * (size_t)n; ++k) vp[k] = vd[k] + dt * acc[k];
    const float h = C->effective_radius;
    const float T = thresh_sq(h);
    const Kern K((double)h);
    const double m = C->fluid_particle_mass;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        const float* xi = &xs[3 * i];
        double sum[3] = {0, 0, 0};
        for_stencil(C->grid, s.cells, xi, h, [&](uint32_t j) {
            if (r2_f32(xi, &xs[3 * j]) < T) {
                double dx = xd[3 * i] - xd[3 * j], dy = xd[3 * i + 1] - xd[3 * j + 1],
                       dz = xd[3 * i + 2] - xd[3 * j + 2];
                const double w = K.W(std::sqrt(dx * dx + dy * dy + dz * dz)) * m / rho[j];
                for (int a = 0; a < 3; ++a) sum[a] += (vp[3 * j + a] - vp[3 * i + a]) * w;
            }
        });
        const uint32_t q = s.perm[i];
        for (int a = 0; a < 3; ++a) {
            const double v2 = vp[3 * i + a] + eps * sum[a];
            v_out[3 * q + a] = v2;
            x_out[3 * q + a] = xd[3 * i + a] + dt * v2;
        }
    }
}

// ---- rollout handle (state in double, sorted order after every step) --------

void* or_ss_create(const OConfig* C, const float* fxyz, uint32_t n, const float* bxyz,
                   uint32_t nb, const float* fvel) {
    SSState* S = new SSState();
    S->C = *C;
    make_boundary(C->grid, bxyz, nb, S->B);
    S->x.resize(3 * (size_t)n);
    S->v.assign(3 * (size_t)n, 0.0);
    S->rho.assign(n, 0.0);
    S->ids.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        S->ids[i] = i;
        for (int a = 0; a < 3; ++a) {
            S->x[3 * i + a] = fxyz[3 * i + a];
            if (fvel) S->v[3 * i + a] = fvel[3 * i + a];
        }
    }
    return S;
}

void or_ss_advance(void* h, double dt, int steps) {
    SSState* S = (SSState*)h;
    for (int s = 0; s < steps; ++s) ss_step(*S, dt);
}

// Copies the state in its current (sorted) order.  Any pointer may be NULL.
void or_ss_get(void* h, double* x, double* v, double* rho, uint32_t* ids) {
    SSState* S = (SSState*)h;
    size_t n = S->ids.size();
    if (x) std::memcpy(x, S->x.data(), 3 * n * sizeof(double));
    if (v) std::memcpy(v, S->v.data(), 3 * n * sizeof(double));
    if (rho) std::memcpy(rho, S->rho.data(), n * sizeof(double));
    if (ids) std::memcpy(ids, S->ids.data(), n * 4);
}

void or_ss_destroy(void* h) { delete (SSState*)h; }

}  // extern "C"
