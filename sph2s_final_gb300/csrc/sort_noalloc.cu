// sort_noalloc.cu -- sph_sort_pairs without any device allocation.
//
// Some callers of this sort cannot call cudaMalloc: a host application that
// owns a fixed device-memory budget and hands the library only its input and
// output buffers (an engine or visualiser embedding the solver, whose memory
// manager owns every device allocation), or a latency-critical loop that
// cannot afford the implicit device synchronisation an allocation may cause.
// For them this
// entry point takes its scratch -- the digit histograms, the look-back status
// words, the tile counters, the ping-pong key/value buffers and an error
// word -- from one file-scope static device array of fixed size, which every
// GPU that loads the library holds until the process exits.
//
// Limits and rules:
//  * at most kNoAllocMaxKeys pairs per call; larger calls return
//    SPH_E_CAPACITY without touching the device;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, once per device, with that device current), so
//    make that first call before any stream capture begins; the lookup is
//    repeated after the device's context is recreated (cudaDeviceReset),
//    recognised by the context's unique id;
//  * every call shares the one array and it keeps the last call's contents:
//    each call clears the parts that must start at zero, but calls whose
//    work overlaps on the GPU (different streams or host threads without
//    ordering between them) race on it and must be serialised by the caller.
#include <cuda.h>
#include <mutex>
#include "errors.h"
#include "radix_sort.cuh"

using namespace sph;

namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;       // 1,048,576 pairs
constexpr size_t kSortRegion = (size_t)2 << 20;      // >= sort_scratch_bytes(kNoAllocMaxKeys)
constexpr size_t kPairRegion = (size_t)8 * kNoAllocMaxKeys;  // ping-pong keys + values
constexpr size_t kScratchBytes = kSortRegion + kPairRegion + 256;  // + error word
constexpr int kMaxDevices = 64;
static_assert(sort_scratch_bytes(kNoAllocMaxKeys) <= kSortRegion,
              "the sort's scratch for kNoAllocMaxKeys pairs must fit its static region");

// Only device code may name this array directly; host code uses the address
// returned by cudaGetSymbolAddress (the host-side symbol is a stand-in, not a
// device address).
static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // id of the context the address belongs to

// Unique id of the calling thread's current context (0 if there is none yet,
// or if the driver cannot tell).  The two driver functions are fetched through
// the runtime, so the library does not link the driver library directly and
// still loads on machines without a GPU driver.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) !=
                cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) !=
                cudaSuccess ||
            qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return 0;
        }
        get_current = reinterpret_cast<GetCurrent>(a);
        get_id = reinterpret_cast<GetId>(b);
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

int scratch_for_current_device(void** out) {
    int dev = -1;
    SPH_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(SPH_E_INVALID, "sph_sort_pairs_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_scratch_ptr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
        void* p = nullptr;
        SPH_CUDA(cudaGetSymbolAddress(&p, g_sort_scratch));  // also creates the context if needed
        g_scratch_ptr[dev] = p;
        g_scratch_ctx[dev] = current_context_id();
    }
    *out = g_scratch_ptr[dev];
    return SPH_OK;
}

}  // namespace

extern "C" int sph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in,
                                      uint32_t* keys_out, uint32_t* vals_out, uint32_t n,
                                      int32_t key_bits, void* stream) {
    if (n == 0) return SPH_OK;
    if (!keys_in || !keys_out || !vals_out)
        return fail(SPH_E_INVALID, "sph_sort_pairs_noalloc: NULL key or output pointer");
    if (key_bits < 1 || key_bits > 32)
        return fail(SPH_E_INVALID, "sph_sort_pairs_noalloc: key_bits must be in 1..32");
    if (n > kNoAllocMaxKeys)
        return fail(SPH_E_CAPACITY,
                    "sph_sort_pairs_noalloc: more than 1,048,576 pairs (the static scratch limit); "
                    "use sph_sort_pairs");
    void* base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc != SPH_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char* b = static_cast<unsigned char*>(base);
    SortScratch s = sort_scratch_from(b, kNoAllocMaxKeys);
    uint32_t* tk = reinterpret_cast<uint32_t*>(b + kSortRegion);
    uint32_t* tv = tk + kNoAllocMaxKeys;
    uint32_t* err = reinterpret_cast<uint32_t*>(b + kSortRegion + kPairRegion);

    const int passes = sort_passes(key_bits);
    uint32_t* ka = (passes & 1) ? keys_out : tk;
    uint32_t* va = (passes & 1) ? vals_out : tv;
    uint32_t* kb = (passes & 1) ? tk : keys_out;
    uint32_t* vb = (passes & 1) ? tv : vals_out;
    SPH_CUDA(cudaMemsetAsync(err, 0, 4, st));
    sort_reset(s, st);  // histograms, tile counters and look-back words start at zero
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
    SPH_CUDA(cudaGetLastError());
    uint32_t herr = 0;
    SPH_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(cudaStreamSynchronize(st));
    if (herr)
        return fail(SPH_E_TIMEOUT, "sph_sort_pairs_noalloc: look-back timed out; output invalid");
    return SPH_OK;
}
