// ref_harness.cu -- runs the reference's own single-scale kernels on a GPU.
//
// TEST INFRASTRUCTURE ONLY.  Loads oracle/_ref/ss_solver.cubin (the
// reference's SPH2S_FINAL_SINGLE_SCALE/Solver.cu compiled unmodified by
// oracle/ref_build.py) with the CUDA driver API and replays the host side of
// the reference's Solver around its kernels:
//   constructor boundary presort       Solver.cu:989-1061
//   Advance = computeNeighborhoods, computeDensities, computeAccelerations,
//             integrate                 Solver.cu:1082-1198
// with the reference's launch shape (256 threads, ceil(n/256) blocks,
// (256+1)*4 bytes of shared memory for the cell-range kernels) and its sort,
// thrust::sort_by_key on (hash, id).  The harness itself adds only two
// things the reference does not have: initial velocities (the reference
// starts from rest) and a persistent id per particle, gathered through the
// sort's permutation, so results can be matched particle by particle.
//
// usage: ref_harness <cubin> <input.bin> <output.bin> [--time W]
//   --time W: run W untimed steps first, then time the input's steps with
//             CUDA events around each whole step (the reference's own
//             CUDA::Timer around Advance, Solver.cu:1084-1095) and print
//             "ref_harness_ms_per_step <ms>"; the output file is still written,
//             but the timed steps do not track persistent ids (W >= 1).
//   input : "SPHREF01" | config (64 bytes, SolverConfiguration layout) |
//           u32 n, u32 nb, u32 steps, f32 dt | f32 x[3n] | f32 v[3n] | f32 b[3nb]
//   output: "SPHOUT01" | u32 n, u32 ncells |
//           after the first step's neighbourhood and force passes, in that
//           step's sorted order: u32 ids[n], u32 hash[n], u32 cell_start[nc],
//           u32 cell_end[nc], f32 rho[n], f32 p[n], f32 acc[3n] |
//           after all steps, sorted order of the last step:
//           f32 x[3n], f32 v[3n], u32 ids[n]
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/gather.h>
#include <thrust/sort.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

void die(const char* what, int code) {
    std::fprintf(stderr, "ref_harness: %s failed (%d)\n", what, code);
    std::exit(2);
}

#define CU(x)                                    \
    do {                                         \
        CUresult _r = (x);                       \
        if (_r != CUDA_SUCCESS) die(#x, (int)_r); \
    } while (0)
#define RT(x)                                      \
    do {                                           \
        cudaError_t _r = (x);                      \
        if (_r != cudaSuccess) die(#x, (int)_r);   \
    } while (0)

struct Grid {
    float origin[3];
    int32_t dims[3];
    float spacing;
};

struct Config {  // SolverConfiguration, SPH2S_FINAL_SINGLE_SCALE/Solver.h:50-60
    float h, m, mb, rho0, K, mu, c, sigma, eps;
    Grid grid;
};

// Itanium-mangled names of the reference kernels (Solver.cu:401-755).
const char* kHash = "_Z12computeHashsPjS_PKfj";
const char* kReorderB = "_Z35reorderComputeCellStartEndBoundaryDPjS_PfPKfPKjS4_j";
const char* kReorder = "_Z30reorderAndComputeCellStartEndDPjS_PfS0_S_PKfS2_PKjj";
const char* kDensity = "_Z26computeDensitiesPressuresDPfS_PKfPKjS3_j";
const char* kAccel = "_Z21computeAccelerationsDPfPKfS1_S1_S1_PKjS3_S1_S3_S3_j";
const char* kIntegrate = "_Z10integrateDPfS_PKfS1_S1_fj";

CUfunction fn(CUmodule m, const char* name) {
    CUfunction f;
    CU(cuModuleGetFunction(&f, m, name));
    return f;
}

void launch(CUfunction f, uint32_t n, void** args, unsigned smem = 0) {
    const unsigned blocks = n % 256 == 0 ? n / 256 : n / 256 + 1;  // computeGridDimensions
    if (blocks == 0) return;
    CU(cuLaunchKernel(f, blocks, 1, 1, 256, 1, 1, smem, 0, args, nullptr));
}

template <class T>
T* dalloc(size_t count) {
    T* p = nullptr;
    RT(cudaMalloc(&p, sizeof(T) * (count ? count : 1)));
    return p;
}

template <class T>
void rd(FILE* f, T* dst, size_t count) {
    if (count && std::fread(dst, sizeof(T), count, f) != count) die("read input", 0);
}

template <class T>
void wr(FILE* f, const T* src, size_t count) {
    if (count) std::fwrite(src, sizeof(T), count, f);
}

template <class T>
std::vector<T> down(const T* d, size_t count) {
    std::vector<T> h(count);
    if (count) RT(cudaMemcpy(h.data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost));
    return h;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 4 && !(argc == 6 && std::strcmp(argv[4], "--time") == 0)) {
        std::fprintf(stderr, "usage: ref_harness <cubin> <input.bin> <output.bin> [--time W]\n");
        return 1;
    }
    const int warm = argc == 6 ? std::atoi(argv[5]) : -1;
    if (argc == 6 && warm < 1) {
        std::fprintf(stderr, "ref_harness: --time needs at least one warm-up step\n");
        return 1;
    }
    FILE* in = std::fopen(argv[2], "rb");
    if (!in) die("open input", 0);
    char magic[8];
    rd(in, magic, 8);
    if (std::memcmp(magic, "SPHREF01", 8) != 0) die("input magic", 0);
    Config cfg;
    rd(in, &cfg, 1);
    uint32_t n, nb, steps;
    float dt;
    rd(in, &n, 1);
    rd(in, &nb, 1);
    rd(in, &steps, 1);
    rd(in, &dt, 1);
    std::vector<float> hx(3 * (size_t)n), hv(3 * (size_t)n), hb(3 * (size_t)nb);
    rd(in, hx.data(), hx.size());
    rd(in, hv.data(), hv.size());
    rd(in, hb.data(), hb.size());
    std::fclose(in);
    const uint32_t nc = (uint32_t)cfg.grid.dims[0] * cfg.grid.dims[1] * cfg.grid.dims[2];

    RT(cudaFree(nullptr));  // primary context shared by the runtime (thrust) and the driver API
    CUmodule mod;
    CU(cuModuleLoad(&mod, argv[1]));
    CUdeviceptr gconf;
    size_t gsize = 0;
    CU(cuModuleGetGlobal(&gconf, &gsize, mod, "gConfiguration"));
    if (gsize != sizeof(Config)) die("gConfiguration size", (int)gsize);
    CU(cuMemcpyHtoD(gconf, &cfg, sizeof(Config)));  // Solver::Bind, Solver.cu:1068-1080
    CUfunction fHash = fn(mod, kHash), fReorderB = fn(mod, kReorderB), fReorder = fn(mod, kReorder),
               fDensity = fn(mod, kDensity), fAccel = fn(mod, kAccel), fInt = fn(mod, kIntegrate);

    // SPHParticleData / BoundaryParticleData buffers (Solver.cu:898-981)
    float* pos = dalloc<float>(3 * (size_t)n);
    float* vel = dalloc<float>(3 * (size_t)n);
    float* dens = dalloc<float>(n);
    float* pres = dalloc<float>(n);
    float* acc = dalloc<float>(3 * (size_t)n);
    float* tpos = dalloc<float>(3 * (size_t)n);
    float* tvel = dalloc<float>(3 * (size_t)n);
    unsigned* ids = dalloc<unsigned>(n);
    unsigned* hashs = dalloc<unsigned>(n);
    unsigned* cs = dalloc<unsigned>(nc);
    unsigned* ce = dalloc<unsigned>(nc);
    float* bpos = dalloc<float>(3 * (size_t)nb);
    float* btmp = dalloc<float>(3 * (size_t)nb);
    unsigned* bids = dalloc<unsigned>(nb);
    unsigned* bhashs = dalloc<unsigned>(nb);
    unsigned* bcs = dalloc<unsigned>(nc);
    unsigned* bce = dalloc<unsigned>(nc);
    unsigned* pid = dalloc<unsigned>(n);   // harness-side persistent ids
    unsigned* pid2 = dalloc<unsigned>(n);
    RT(cudaMemcpy(pos, hx.data(), 4 * hx.size(), cudaMemcpyHostToDevice));
    RT(cudaMemcpy(vel, hv.data(), 4 * hv.size(), cudaMemcpyHostToDevice));
    RT(cudaMemcpy(bpos, hb.data(), 4 * hb.size(), cudaMemcpyHostToDevice));
    {
        std::vector<unsigned> iota(n);
        for (uint32_t i = 0; i < n; ++i) iota[i] = i;
        if (n) RT(cudaMemcpy(pid, iota.data(), 4 * (size_t)n, cudaMemcpyHostToDevice));
    }
    const unsigned smem = sizeof(int) * (256 + 1);

    // boundary presort on the fluid grid (Solver.cu:1013-1055)
    {
        void* a[] = {&bhashs, &bids, &bpos, &nb};
        launch(fHash, nb, a);
        if (nb)
            thrust::sort_by_key(thrust::device_ptr<unsigned>(bhashs),
                                thrust::device_ptr<unsigned>(bhashs + nb),
                                thrust::device_ptr<unsigned>(bids));
        RT(cudaMemset(bcs, 0xFF, 4 * (size_t)nc));
        RT(cudaMemset(bce, 0xFF, 4 * (size_t)nc));
        void* r[] = {&bcs, &bce, &btmp, &bpos, &bids, &bhashs, &nb};
        launch(fReorderB, nb, r, smem);
        RT(cudaMemcpy(bpos, btmp, 4 * 3 * (size_t)nb, cudaMemcpyDeviceToDevice));
    }

    FILE* out = std::fopen(argv[3], "wb");
    if (!out) die("open output", 0);
    wr(out, "SPHOUT01", 8);
    wr(out, &n, 1);
    wr(out, &nc, 1);
    cudaEvent_t ev0, ev1;
    RT(cudaEventCreate(&ev0));
    RT(cudaEventCreate(&ev1));
    const uint32_t total = steps + (uint32_t)(warm > 0 ? warm : 0);
    for (uint32_t s = 0; s < total; ++s) {
        if (warm >= 0 && s == (uint32_t)warm) {
            RT(cudaDeviceSynchronize());
            RT(cudaEventRecord(ev0));
        }
        // computeNeighborhoods (Solver.cu:1098-1140)
        void* h[] = {&hashs, &ids, &pos, &n};
        launch(fHash, n, h);
        if (n)
            thrust::sort_by_key(thrust::device_ptr<unsigned>(hashs),
                                thrust::device_ptr<unsigned>(hashs + n),
                                thrust::device_ptr<unsigned>(ids));
        // Timed steps skip the harness-only id tracking (final ids then stale).
        if (n && (warm < 0 || s < (uint32_t)warm)) {
            thrust::gather(thrust::device_ptr<unsigned>(ids), thrust::device_ptr<unsigned>(ids + n),
                           thrust::device_ptr<unsigned>(pid), thrust::device_ptr<unsigned>(pid2));
            std::swap(pid, pid2);
        }
        RT(cudaMemset(cs, 0xFF, 4 * (size_t)nc));
        RT(cudaMemset(ce, 0xFF, 4 * (size_t)nc));
        void* r[] = {&cs, &ce, &tpos, &tvel, &ids, &pos, &vel, &hashs, &n};
        launch(fReorder, n, r, smem);
        // computeDensities, computeAccelerations, integrate (Solver.cu:1142-1198)
        void* d[] = {&dens, &pres, &tpos, &cs, &ce, &n};
        launch(fDensity, n, d);
        void* a[] = {&acc, &dens, &pres, &tpos, &tvel, &cs, &ce, &bpos, &bcs, &bce, &n};
        launch(fAccel, n, a);
        if (s == 0) {
            RT(cudaDeviceSynchronize());
            wr(out, down(pid, n).data(), n);
            wr(out, down(hashs, n).data(), n);
            wr(out, down(cs, nc).data(), nc);
            wr(out, down(ce, nc).data(), nc);
            wr(out, down(dens, n).data(), n);
            wr(out, down(pres, n).data(), n);
            wr(out, down(acc, 3 * (size_t)n).data(), 3 * (size_t)n);
        }
        void* it[] = {&pos, &vel, &acc, &tpos, &tvel, &dt, &n};
        launch(fInt, n, it);
    }
    if (warm >= 0) {
        RT(cudaEventRecord(ev1));
        RT(cudaEventSynchronize(ev1));
        float ms = 0.0f;
        RT(cudaEventElapsedTime(&ms, ev0, ev1));
        std::printf("ref_harness_ms_per_step %.6f\n", steps ? ms / (float)steps : 0.0f);
    }
    RT(cudaDeviceSynchronize());
    wr(out, down(pos, 3 * (size_t)n).data(), 3 * (size_t)n);
    wr(out, down(vel, 3 * (size_t)n).data(), 3 * (size_t)n);
    wr(out, down(pid, n).data(), n);
    std::fclose(out);
    std::printf("ref_harness: %u particles, %u boundary, %u steps\n", n, nb, steps);
    return 0;
}
