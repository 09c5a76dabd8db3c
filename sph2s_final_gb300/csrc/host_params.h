// host_params.h -- derives the per-solver kernel constants from a sph_config.
// Kernel normalisations follow SPH2S_FINAL_SINGLE_SCALE/Solver.cu:103-196
// (Poly6 315/(64 pi h^9), spiky gradient -45/(pi h^6), viscosity Laplacian
// 45/(pi h^6), boundary 0.02 c^2 / r); they are evaluated in double and
// rounded once to float.
#pragma once
#include <algorithm>
#include <cmath>
#include <string>
#include "common.cuh"
#include "errors.h"

namespace sph {

constexpr uint32_t kMaxParticles = 1u << 30;  // 30-bit look-back counts

// Smallest float t with sqrtf(t) >= h: "sqrtf(r2) < h" <=> "r2 < t".
inline float neighbor_threshold(float h) {
    float t = h * h;
    while (!(std::sqrt(t) >= h)) t = std::nextafter(t, INFINITY);
    while (t > 0.0f && std::sqrt(std::nextafter(t, 0.0f)) >= h) t = std::nextafter(t, 0.0f);
    return t;
}

inline int morton_bits_for(const sph_grid& g) {
    int dmax = g.dims[0];
    if (g.dims[1] > dmax) dmax = g.dims[1];
    if (g.dims[2] > dmax) dmax = g.dims[2];
    int b = 1;
    while ((1 << b) < dmax) ++b;
    return b;
}

inline int validate_grid(const sph_grid& g, const char* who) {
    for (int a = 0; a < 3; ++a)
        if (g.dims[a] < 1 || g.dims[a] > 1024)
            return fail(SPH_E_INVALID, std::string(who) + ": grid dims must be in 1..1024");
    if (!(g.spacing > 0.0f) || !std::isfinite(g.spacing))
        return fail(SPH_E_INVALID, std::string(who) + ": grid spacing must be positive");
    return SPH_OK;
}

inline GridParams make_grid_params(const sph_grid& g) {
    GridParams p;
    p.ox = g.origin[0];
    p.oy = g.origin[1];
    p.oz = g.origin[2];
    p.dx = g.dims[0];
    p.dy = g.dims[1];
    p.dz = g.dims[2];
    p.spacing = g.spacing;
    p.mbits = morton_bits_for(g);
    p.ex = (float)((double)g.origin[0] + (double)g.dims[0] * (double)g.spacing);
    p.ey = (float)((double)g.origin[1] + (double)g.dims[1] * (double)g.spacing);
    p.ez = (float)((double)g.origin[2] + (double)g.dims[2] * (double)g.spacing);
    return p;
}

// Rounding allowance of the boundary depth cut (boundary_reach): 1e-3 h plus
// a few ulps of the box's coordinates.
inline float boundary_margin(const GridParams& p, float h) {
    double m = 0.0;
    for (float v : {p.ox, p.oy, p.oz, p.ex, p.ey, p.ez}) m = std::max(m, std::fabs((double)v));
    return (float)(1e-3 * (double)h + 32.0 * std::ldexp(1.0, -24) * (m + (double)h));
}

// Depth classes of the boundary presort (depth_class): quantum h/16, and as
// many key bits as the cell key leaves free, at most 8; 0 (no cut) when the
// quantum is not far above the coordinates' rounding.
inline float boundary_quantum(float h) { return h / 16.0f; }
inline int boundary_depth_bits(const GridParams& p, float h, int key_bits) {
    double m = 0.0;
    for (float v : {p.ox, p.oy, p.oz, p.ex, p.ey, p.ez}) m = std::max(m, std::fabs((double)v));
    if ((double)boundary_quantum(h) < std::ldexp(m + (double)h, -16)) return 0;
    return std::max(0, std::min(8, 32 - key_bits));
}

inline int make_sim_params(const sph_config& c, SimParams* out) {
    int rc = validate_grid(c.grid, "sph_config");
    if (rc != SPH_OK) return rc;
    const float h = c.effective_radius;
    if (!(h > 0.0f) || !std::isfinite(h))
        return fail(SPH_E_INVALID, "sph_config: effective_radius must be positive");
    if (!(c.fluid_particle_mass > 0.0f) || !(c.boundary_particle_mass >= 0.0f))
        return fail(SPH_E_INVALID, "sph_config: particle masses must be positive");
    const double pi = 3.14159265358979323846;
    const double hd = h, h3 = hd * hd * hd;
    const double poly6 = 315.0 / (64.0 * pi * h3 * h3 * h3);
    const double spiky = 45.0 / (pi * h3 * h3);
    const double m = c.fluid_particle_mass, mb = c.boundary_particle_mass;
    SimParams P;
    P.g = make_grid_params(c.grid);
    P.h = h;
    P.h2 = h * h;
    P.T = neighbor_threshold(h);
    P.mass = c.fluid_particle_mass;
    P.rho0 = c.rest_density;
    P.bulk = c.bulk_modulus;
    P.dens_coef = (float)(m * poly6);
    P.pres_coef = (float)(m * spiky);
    P.tens_coef = (float)((double)c.tension_coefficient * m * poly6);
    P.visc_coef = (float)((double)c.viscosity * m * spiky);
    P.bnd_coef = (float)(0.02 * (double)c.speed_sound * c.speed_sound * mb / (m + mb));
    P.two_over_h = (float)(2.0 / hd);
    P.gravity = -9.81f;
    P.bmargin = boundary_margin(P.g, h);
    *out = P;
    return SPH_OK;
}

}  // namespace sph
