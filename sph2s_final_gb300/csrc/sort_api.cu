// sort_api.cu -- the onesweep radix sort as a C-ABI entry point.
//
// Replaces thrust::sort_by_key(hashes, hashes + n, ids) at
// SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1110-1115 (and 1022-1027 for the
// boundary): ascending by key, stable (equal keys keep their input order).
#include <cstring>
#include "errors.h"
#include "coherent_sort.cuh"
#include "radix_sort.cuh"

using namespace sph;

extern "C" int sph_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                              uint32_t* vals_out, uint32_t n, int32_t key_bits, void* stream) {
    if (n == 0) return SPH_OK;
    if (!keys_in || !keys_out || !vals_out)
        return fail(SPH_E_INVALID, "sph_sort_pairs: NULL key or output pointer");
    if (key_bits < 1 || key_bits > 32)
        return fail(SPH_E_INVALID, "sph_sort_pairs: key_bits must be in 1..32");
    if (n > (1u << 30)) return fail(SPH_E_CAPACITY, "sph_sort_pairs: more than 2^30 keys");
    cudaStream_t st = (cudaStream_t)stream;
    const int passes = sort_passes(key_bits);
    uint32_t* tmp = nullptr;
    void* scratch_mem = nullptr;
    uint32_t* err = nullptr;
    cudaError_t e = cudaMalloc(&tmp, 8 * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&scratch_mem, sort_scratch_bytes(n));
    if (e == cudaSuccess) e = cudaMalloc(&err, 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, 4, st);
    uint32_t herr = 0;
    if (e == cudaSuccess) {
        SortScratch s = sort_scratch_from(scratch_mem, n);
        // Ping-pong so that the last pass writes keys_out/vals_out:
        // an odd pass count starts into the outputs, an even one into tmp.
        uint32_t* ka = (passes & 1) ? keys_out : tmp;
        uint32_t* va = (passes & 1) ? vals_out : tmp + n;
        uint32_t* kb = (passes & 1) ? tmp : keys_out;
        uint32_t* vb = (passes & 1) ? tmp + n : vals_out;
        sort_reset(s, st);
        sort_histogram(keys_in, n, passes, s, st);
        sort_scan(passes, s, st);
        const uint32_t* kin = keys_in;
        const uint32_t* vin = vals_in;
        for (int p = 0; p < passes; ++p) {
            uint32_t* ko = (p & 1) ? kb : ka;
            uint32_t* vo = (p & 1) ? vb : va;
            sort_pass(kin, vin, ko, vo, n, p, s, err, 0, st);
            kin = ko;
            vin = vo;
        }
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(tmp);
    cudaFree(scratch_mem);
    cudaFree(err);
    SPH_CUDA(e);
    if (herr) return fail(SPH_E_TIMEOUT, "sph_sort_pairs: look-back timed out; output invalid");
    return SPH_OK;
}

namespace {

__global__ void nondecreasing_check_kernel(const uint32_t* __restrict__ a, uint32_t n,
                                           uint32_t* __restrict__ bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 < n && a[i] > a[i + 1]) *bad = 1u;
}

}  // namespace

extern "C" int sph_sort_keys_coherent(const uint32_t* keys_in, const uint32_t* hint,
                                      uint32_t* keys_out, uint32_t* perm_out, uint32_t n,
                                      int32_t key_bits, void* stream) {
    if (n == 0) return SPH_OK;
    if (!keys_in || !hint || !keys_out || !perm_out)
        return fail(SPH_E_INVALID, "sph_sort_keys_coherent: NULL pointer");
    if (key_bits < 1 || key_bits > 32)
        return fail(SPH_E_INVALID, "sph_sort_keys_coherent: key_bits must be in 1..32");
    if (n > (1u << 30)) return fail(SPH_E_CAPACITY, "sph_sort_keys_coherent: more than 2^30 keys");
    cudaStream_t st = (cudaStream_t)stream;
    void* co_mem = nullptr;
    uint32_t* err = nullptr;  // [0] sort errors, [1] hint out of order
    cudaError_t e = cudaMalloc(&co_mem, coherent_bytes(n));
    if (e == cudaSuccess) e = cudaMalloc(&err, 8);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, 8, st);
    uint32_t herr[2] = {0, 0};
    if (e == cudaSuccess) {
        nondecreasing_check_kernel<<<(n + 255) / 256, 256, 0, st>>>(hint, n, err + 1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(herr, err, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e == cudaSuccess && !herr[1]) {
        CoherentSort c = coherent_from(co_mem, n);
        c.kprev = const_cast<uint32_t*>(hint);  // read only: the step's gather writes it
        coherent_sort_keys(c, keys_in, key_bits, keys_out, perm_out, err, 0, st);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(herr, err, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(co_mem);
    cudaFree(err);
    SPH_CUDA(e);
    if (herr[1]) return fail(SPH_E_INVALID, "sph_sort_keys_coherent: hint is not non-decreasing");
    if (herr[0] & 1u) return fail(SPH_E_TIMEOUT, "sph_sort_keys_coherent: look-back timed out; output invalid");
    if (herr[0]) return fail(SPH_E_CAPACITY, "sph_sort_keys_coherent: placement out of range");
    return SPH_OK;
}
