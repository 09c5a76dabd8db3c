// common.cuh -- device-side building blocks shared by every SPH2S kernel.
//
// Structural predicates (cell coordinates, stencil bounds, the r < h test) are
// evaluated with explicitly rounded FP32 intrinsics so that nvcc cannot
// contract them into FMAs; the CPU oracle evaluates the identical sequence,
// which is what makes cell keys, sorted order and neighbour counts comparable
// bit for bit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sph {

constexpr uint32_t kEmptyCell = 0xFFFFFFFFu;  // EMPTY_CELL_ID, SPH2S_FINAL_SINGLE_SCALE/Solver.cu:862
// Neighbour-list slots per particle (about twice the ~34 neighbours at h = 2s);
// particles with more neighbours fall back to a stencil rescan.
constexpr int kMaxNbr = 64;

struct GridParams {
    float ox, oy, oz;   // Grid::Origin
    int dx, dy, dz;     // Grid::Dimensions
    float spacing;      // Grid::Spacing
    int mbits;          // Morton bits per axis: ceil(log2(max dim))
    float ex, ey, ez;   // far corner of the grid's box, origin + dims * spacing
};

// Per-solver constants, passed by value to every kernel (the reference keeps
// one SolverConfiguration in __constant__ memory, Solver.cu:12).
struct SimParams {
    GridParams g;
    float h;          // effective radius
    float h2;         // h*h (FP32)
    float T;          // neighbour threshold on r2: r < h  <=>  r2 < T
    float mass;       // fluid particle mass
    float rho0;       // rest density
    float bulk;       // K
    float dens_coef;  // m * 315 / (64 pi h^9)
    float pres_coef;  // m * 45 / (pi h^6)        (spiky gradient)
    float tens_coef;  // sigma * m * 315 / (64 pi h^9)
    float visc_coef;  // mu * m * 45 / (pi h^6)   (viscosity Laplacian)
    float bnd_coef;   // 0.02 c^2 * m_b / (m + m_b)
    float two_over_h; // 2 / h
    float gravity;    // -9.81 along y
    float bmargin;    // rounding allowance of the boundary scan's depth cut (boundary_reach)
};

// computeCoordinates(Off), SPH2S_FINAL_SINGLE_SCALE/Solver.cu:20-57.  The
// clamp of t to [-1, D] before the conversion keeps NaN / huge inputs well
// defined and leaves every finite result unchanged.
__device__ __forceinline__ int cell_coord_off(float x, float off, float o, float s, int D) {
    float t = __fdiv_rn(__fsub_rn(__fadd_rn(x, off), o), s);
    t = fminf(fmaxf(t, -1.0f), (float)D);
    int c = __float2int_rz(t);
    return min(max(c, 0), D - 1);
}

__device__ __forceinline__ int cell_coord(float x, float o, float s, int D) {
    float t = __fdiv_rn(__fsub_rn(x, o), s);
    t = fminf(fmaxf(t, -1.0f), (float)D);
    int c = __float2int_rz(t);
    return min(max(c, 0), D - 1);
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t compact3(uint32_t v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030C30C3u;
    v = (v | (v >> 4)) & 0x0300F00Fu;
    v = (v | (v >> 8)) & 0x030000FFu;
    v = (v | (v >> 16)) & 0x000003FFu;
    return v;
}

__device__ __forceinline__ uint32_t morton3(int cx, int cy, int cz) {
    return spread3((uint32_t)cx) | (spread3((uint32_t)cy) << 1) | (spread3((uint32_t)cz) << 2);
}

// Linear cell index of the reference's hash (Solver.cu:59-69).
__device__ __forceinline__ uint32_t linear_cell(const GridParams& g, int cx, int cy, int cz) {
    return (uint32_t)(cx + g.dx * (cy + g.dy * cz));
}

__device__ __forceinline__ uint32_t morton_to_linear(const GridParams& g, uint32_t key) {
    int cx = (int)compact3(key), cy = (int)compact3(key >> 1), cz = (int)compact3(key >> 2);
    return linear_cell(g, cx, cy, cz);
}

// Linear cell of a Morton key, or kEmptyCell if the key lies outside the grid.
__device__ __forceinline__ uint32_t morton_to_linear_checked(const GridParams& g, uint32_t key) {
    int cx = (int)compact3(key), cy = (int)compact3(key >> 1), cz = (int)compact3(key >> 2);
    if (cx >= g.dx || cy >= g.dy || cz >= g.dz || (key >> (3 * g.mbits)) != 0u) return kEmptyCell;
    return linear_cell(g, cx, cy, cz);
}

__device__ __forceinline__ uint32_t cell_key(const GridParams& g, float x, float y, float z) {
    int cx = cell_coord(x, g.ox, g.spacing, g.dx);
    int cy = cell_coord(y, g.oy, g.spacing, g.dy);
    int cz = cell_coord(z, g.oz, g.spacing, g.dz);
    return morton3(cx, cy, cz);
}

// r2 = fma(dz,dz, fma(dy,dy, dx*dx)) with d = a - b, all single-rounded.
__device__ __forceinline__ float dist2(float ax, float ay, float az, float bx, float by, float bz,
                                       float& dx, float& dy, float& dz) {
    dx = __fsub_rn(ax, bx);
    dy = __fsub_rn(ay, by);
    dz = __fsub_rn(az, bz);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

struct Stencil {
    int x0, x1, y0, y1, z0, z1;
};

// Stencil bounds clamp(trunc((x -/+ h - o)/s)), Solver.cu:559-570.
__device__ __forceinline__ Stencil stencil(const GridParams& g, float x, float y, float z, float h) {
    Stencil s;
    s.x0 = cell_coord_off(x, -h, g.ox, g.spacing, g.dx);
    s.x1 = cell_coord_off(x, h, g.ox, g.spacing, g.dx);
    s.y0 = cell_coord_off(y, -h, g.oy, g.spacing, g.dy);
    s.y1 = cell_coord_off(y, h, g.oy, g.spacing, g.dy);
    s.z0 = cell_coord_off(z, -h, g.oz, g.spacing, g.dz);
    s.z1 = cell_coord_off(z, h, g.oz, g.spacing, g.dz);
    return s;
}

// Boundary particles are stored, within each cell, by non-decreasing w, a
// lower bound on their depth outside the grid's box (depth_class: the
// Euclidean distance to the box, quantised down).  The clamped cell
// assignment (Solver.cu:35-37) puts every layer of the reference's boundary
// shell that lies outside the grid into the edge cells, up to five layers on
// each clamped axis.  A boundary particle j within h of a particle at x
// satisfies depth_j <= |x_j - x| + dist(x, box) < h + dist(x, box), so a cell
// scan may stop at the first particle deeper than the returned reach: the
// neighbour set is that of the full scan.  dist(x, box) is bounded above by
// the sum of the per-axis distances outside; bmargin covers the rounding.
__device__ __forceinline__ float boundary_reach(const GridParams& g, float h, float bmargin,
                                                float x, float y, float z) {
    const float ox = fmaxf(fmaxf(__fsub_rn(g.ox, x), __fsub_rn(x, g.ex)), 0.0f);
    const float oy = fmaxf(fmaxf(__fsub_rn(g.oy, y), __fsub_rn(y, g.ey)), 0.0f);
    const float oz = fmaxf(fmaxf(__fsub_rn(g.oz, z), __fsub_rn(z, g.ez)), 0.0f);
    return h + ox + oy + oz + bmargin;
}

// Depth class of a boundary particle for its presort key (qb low bits below
// the cell key; qb = 0 disables the cut) and the class's lower bound, which
// becomes the particle's w.  The class is one below floor(depth / quantum) so
// that the bound stays below the exact depth whatever the rounding of the
// computed one (quantum is far above the coordinates' ulp).
struct DepthClass {
    uint32_t cls;
    float lb;
};
__device__ __forceinline__ DepthClass depth_class(const GridParams& g, float x, float y, float z,
                                                  float quantum, int qb) {
    if (qb <= 0) return {0u, 0.0f};
    const float ax = fmaxf(fmaxf(__fsub_rn(g.ox, x), __fsub_rn(x, g.ex)), 0.0f);
    const float ay = fmaxf(fmaxf(__fsub_rn(g.oy, y), __fsub_rn(y, g.ey)), 0.0f);
    const float az = fmaxf(fmaxf(__fsub_rn(g.oz, z), __fsub_rn(z, g.ez)), 0.0f);
    const float d = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)),
                                         __fmul_rn(az, az)));  // distance to the box
    float c = floorf(__fdiv_rn(d, quantum)) - 1.0f;
    c = fminf(fmaxf(c, 0.0f), (float)((1u << qb) - 1u));
    return {(uint32_t)c, __fmul_rn(c, quantum)};
}

// Particles whose cell has boundary particles within stencil reach, listed
// by the kernel that builds the step's cell ranges (sorted index, in no
// particular order) for the step's boundary force pass; with `flag`, the same
// fact per sorted particle (1 = listed), which the force pass reads in place
// of recomputing the particle's cell and looking up bnear.
struct NearList {
    const uint8_t* bnear = nullptr;  // per cell (static); nullptr: no list
    uint32_t* list = nullptr;        // capacity n
    uint32_t* count = nullptr;       // zeroed before the kernel
    uint8_t* flag = nullptr;         // per sorted particle, or nullptr
};

// Appends sorted index i if its cell c is near the boundary: one atomic per
// warp, each lane's slot from its rank among the appending lanes.  c may be
// kEmptyCell (a key outside the grid after a failed sort): not listed.
__device__ __forceinline__ void near_append(const NearList& L, uint32_t c, uint32_t i) {
    if (!L.list) return;
    const bool want = c != kEmptyCell && L.bnear[c] != 0;
    if (L.flag) L.flag[i] = want ? 1 : 0;
    const uint32_t am = __activemask();
    const uint32_t b = __ballot_sync(am, want);
    if (!b) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = (uint32_t)__ffs(b) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(L.count, (uint32_t)__popc(b));
    base = __shfl_sync(am, base, (int)leader);
    if (want) L.list[base + (uint32_t)__popc(b & ((1u << lane) - 1u))] = i;
}

// Boundary weight shape of evaluateBoundaryWeight (Solver.cu:169-196)
// without the 0.02 c^2 / r factor: q = 2r/h.
__device__ __forceinline__ float boundary_shape(float q) {
    if (q < 2.0f / 3.0f) return 2.0f / 3.0f;
    if (q < 1.0f) return q * (2.0f - 1.5f * q);
    if (q < 2.0f) {
        float a = 2.0f - q;
        return 0.5f * a * a;
    }
    return 0.0f;
}

}  // namespace sph
