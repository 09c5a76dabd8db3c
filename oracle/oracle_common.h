// oracle_common.h -- helpers shared by the single- and two-scale oracles.
// TEST INFRASTRUCTURE ONLY (see sph_oracle.cpp).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <numeric>

namespace oracle {


// Same field order as sph_grid / sph_config in include/sph2s.h.  The oracle
// declares its own copy so that it does not depend on the product's headers.
struct OGrid {
    float origin[3];
    int dims[3];
    float spacing;
};

struct OConfig {
    float effective_radius;       // h
    float fluid_particle_mass;    // m
    float boundary_particle_mass; // m_b
    float rest_density;           // rho0
    float bulk_modulus;           // K
    float viscosity;              // mu
    float speed_sound;            // c
    float tension_coefficient;    // sigma
    float xsph_coeff;             // epsilon (XSPH, unused on the step path)
    OGrid grid;
};

constexpr double kPi = 3.14159265358979323846;

// ---- FP32 structural helpers ------------------------------------------------

// Solver.cu:20-38 (computeCoordinatesOff) with the float->int conversion made
// well defined for out-of-range and NaN inputs: t is clamped to [-1, D] first,
// which does not change the clamped result for any finite input.
inline int cell_coord_off(float x, float off, float o, float s, int D) {
    float t = ((x + off) - o) / s;
    t = std::fmin(std::fmax(t, -1.0f), (float)D);
    int c = (int)t;
    return c < 0 ? 0 : (c > D - 1 ? D - 1 : c);
}

// Solver.cu:40-57 (computeCoordinates).
inline int cell_coord(float x, float o, float s, int D) {
    float t = (x - o) / s;
    t = std::fmin(std::fmax(t, -1.0f), (float)D);
    int c = (int)t;
    return c < 0 ? 0 : (c > D - 1 ? D - 1 : c);
}

inline uint32_t spread3(uint32_t v) {
    uint32_t r = 0;
    for (int b = 0; b < 10; ++b) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}

inline int morton_bits(const OGrid& g) {
    int dmax = std::max(g.dims[0], std::max(g.dims[1], g.dims[2]));
    int b = 1;
    while ((1 << b) < dmax) ++b;
    return b;
}

inline uint32_t morton(int cx, int cy, int cz) {
    return spread3((uint32_t)cx) | (spread3((uint32_t)cy) << 1) |
           (spread3((uint32_t)cz) << 2);
}

// Solver.cu:59-69 (computeHash): the reference's linear cell index.
inline uint32_t linear_cell(const OGrid& g, int cx, int cy, int cz) {
    return (uint32_t)(cx + g.dims[0] * (cy + g.dims[1] * cz));
}

inline float r2_f32(const float* a, const float* b) {
    float dx = a[0] - b[0];
    float dy = a[1] - b[1];
    float dz = a[2] - b[2];
    return std::fmaf(dz, dz, std::fmaf(dy, dy, dx * dx));
}

inline float thresh_sq(float h) {
    float t = h * h;
    while (!(std::sqrt(t) >= h)) t = std::nextafter(t, INFINITY);
    while (t > 0.0f && std::sqrt(std::nextafter(t, 0.0f)) >= h)
        t = std::nextafter(t, 0.0f);
    return t;
}

// ---- cell lists -----------------------------------------------------------

struct CellList {
    std::vector<uint32_t> start, end;  // per linear cell; 0xFFFFFFFF = empty
};

// Stable sort of keys; perm[k] = input index of the k-th smallest key with
// ties in input order (what an LSD radix sort over (key, index) yields).
inline void stable_argsort(const std::vector<uint32_t>& keys, std::vector<uint32_t>& perm) {
    perm.resize(keys.size());
    std::iota(perm.begin(), perm.end(), 0u);
    std::stable_sort(perm.begin(), perm.end(),
                     [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
}

// Solver.cu:478-534 (cell start/end from sorted hashes), with tables indexed
// by the linear cell index of each sorted particle.
inline void build_cells(const OGrid& g, const std::vector<uint32_t>& lin_sorted, CellList& cl) {
    size_t nc = (size_t)g.dims[0] * g.dims[1] * g.dims[2];
    cl.start.assign(nc, 0xFFFFFFFFu);
    cl.end.assign(nc, 0xFFFFFFFFu);
    size_t n = lin_sorted.size();
    for (size_t i = 0; i < n; ++i) {
        uint32_t c = lin_sorted[i];
        if (i == 0 || c != lin_sorted[i - 1]) {
            cl.start[c] = (uint32_t)i;
            if (i > 0) cl.end[lin_sorted[i - 1]] = (uint32_t)i;
        }
        if (i == n - 1) cl.end[c] = (uint32_t)(i + 1);
    }
}

// Sorts a float position set by Morton key (stable) and builds its cell list.
struct SortedSet {
    std::vector<uint32_t> perm;     // sorted k -> input index
    std::vector<uint32_t> keys;     // Morton keys in sorted order
    std::vector<uint32_t> lin;      // linear cells in sorted order
    CellList cells;
};

inline void sort_set(const OGrid& g, const float* xyz, size_t n, SortedSet& s) {
    std::vector<uint32_t> keys(n), lin(n);
    for (size_t i = 0; i < n; ++i) {
        int cx = cell_coord(xyz[3 * i + 0], g.origin[0], g.spacing, g.dims[0]);
        int cy = cell_coord(xyz[3 * i + 1], g.origin[1], g.spacing, g.dims[1]);
        int cz = cell_coord(xyz[3 * i + 2], g.origin[2], g.spacing, g.dims[2]);
        keys[i] = morton(cx, cy, cz);
        lin[i] = linear_cell(g, cx, cy, cz);
    }
    stable_argsort(keys, s.perm);
    s.keys.resize(n);
    s.lin.resize(n);
    for (size_t k = 0; k < n; ++k) {
        s.keys[k] = keys[s.perm[k]];
        s.lin[k] = lin[s.perm[k]];
    }
    build_cells(g, s.lin, s.cells);
}

// Visits every candidate j (sorted index) of the reference's stencil around
// xf (float position) with radius h on grid g: Solver.cu:559-593.
template <class F>
inline void for_stencil(const OGrid& g, const CellList& cl, const float* xf, float h, F&& f) {
    int cs[3], ce[3];
    for (int a = 0; a < 3; ++a) {
        cs[a] = cell_coord_off(xf[a], -h, g.origin[a], g.spacing, g.dims[a]);
        ce[a] = cell_coord_off(xf[a], h, g.origin[a], g.spacing, g.dims[a]);
    }
    for (int cz = cs[2]; cz <= ce[2]; ++cz)
        for (int cy = cs[1]; cy <= ce[1]; ++cy)
            for (int cx = cs[0]; cx <= ce[0]; ++cx) {
                uint32_t c = linear_cell(g, cx, cy, cz);
                uint32_t b = cl.start[c], e = cl.end[c];
                for (uint32_t j = b; j < e; ++j) f(j);
            }
}

// ---- kernel functions in double (Solver.cu:103-196) -------------------------

struct Kern {
    double h, h2, poly6, spiky, visc;
    explicit Kern(double hh) : h(hh), h2(hh * hh) {
        double h3 = hh * hh * hh;
        poly6 = 315.0 / (64.0 * kPi * h3 * h3 * h3);
        spiky = 45.0 / (kPi * h3 * h3);
        visc = 45.0 / (kPi * h3 * h3);
    }
    double W(double r) const {
        double a = h2 - r * r;
        return poly6 * a * a * a;
    }
    // magnitude factor g such that grad W = g * x_ij  (for 0 < r)
    double gradW_factor(double r) const { return -spiky * (h - r) * (h - r) / r; }
    double lapl(double r) const { return visc * (h - r); }
};

// Solver.cu:169-196 (evaluateBoundaryWeight).
inline double boundary_weight(double r, double h, double c) {
    double q = 2.0 * r / h;
    double coeff = 0.02 * c * c / r;
    if (q < 2.0 / 3.0) return coeff * 2.0 / 3.0;
    if (q < 1.0) return coeff * (2.0 * q - 1.5 * q * q);
    if (q < 2.0) return coeff * 0.5 * (2.0 - q) * (2.0 - q);
    return 0.0;
}


}  // namespace oracle
