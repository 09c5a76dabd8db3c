// boundary_tables.cuh -- the static tables of the boundary force pass
// (boundary_force_kernel), built once per handle from the presorted boundary:
// per near-boundary cell the boundary particles of its cells +-1 within h plus
// a margin of the cell's box, in the full scan's order (start, cand).
#pragma once
#include "scan.cuh"
#include "single_scale_kernels.cuh"

namespace sph {

struct BoundaryTables {
    uint32_t* start = nullptr;  // per cell, plus the total at [ncells]
    uint32_t* cand = nullptr;   // boundary particle indices
};

// Builds the tables of grid g (ncells cells, boundary presorted into bpos /
// bcells, near-boundary flags bnear) on stream st and waits for them.  Returns
// the first CUDA error; what was allocated is in t either way (the caller
// frees it).
inline cudaError_t build_boundary_tables(const uint2* bcells, const float4* bpos,
                                         const uint8_t* bnear, const GridParams& g,
                                         uint32_t ncells, uint32_t nb, float h, float bmargin,
                                         cudaStream_t st, BoundaryTables& t) {
    const uint32_t blocks = (ncells + 255) / 256;
    cudaError_t e = cudaMalloc(&t.start, 4 * ((size_t)ncells + 1));
    if (e != cudaSuccess) return e;
    const uint32_t words = (uint32_t)scan_scratch_words(ncells + 1);
    uint32_t* scratch = nullptr;
    e = cudaMalloc(&scratch, 4 * ((size_t)words + 1));
    if (e != cudaSuccess) return e;
    uint32_t* total_d = scratch + words;
    const float lim = h * 1.01f + 4.0f * bmargin;  // any superset of the neighbours will do
    if (ncells) {
        boundary_cand_kernel<false><<<blocks, 256, 0, st>>>(bcells, bpos, bnear, g, nb, lim,
                                                            t.start, nullptr);
    }
    e = cudaMemsetAsync(t.start + ncells, 0, 4, st);
    const ScanSeg seg = {t.start, t.start, ncells + 1, total_d};
    if (e == cudaSuccess) {
        scan_exclusive_batch(&seg, 1, scratch, st);
        e = cudaGetLastError();
    }
    uint32_t total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, total_d, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(scratch);
    if (e == cudaSuccess) e = cudaMalloc(&t.cand, 4 * (size_t)(total ? total : 1));
    if (e != cudaSuccess) return e;
    if (ncells)
        boundary_cand_kernel<true><<<blocks, 256, 0, st>>>(bcells, bpos, bnear, g, nb, lim, t.start,
                                                           t.cand);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

}  // namespace sph
