// errors.h -- status codes and the thread-local "last error" of the C ABI.
// The reference throws std::runtime_error with file and line from
// CUDA::SafeCall (SPH2S_FINAL_SINGLE_SCALE/cuda.h:115-129); across a C ABI
// that becomes a status code plus a message kept per calling thread.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include "../../include/sph2s.h"

namespace sph {

// Device error word bits (written by kernels, read at sync points).
constexpr unsigned kErrLookbackTimeout = 1u;
constexpr unsigned kErrCapacity = 2u;

void set_last_error(const std::string& msg);
int fail(int code, const std::string& msg);
// Maps a CUDA status to SPH_OK / SPH_E_CUDA, recording where it happened.
int check_cuda(cudaError_t e, const char* what, const char* file, int line);
// SPH_OK if p is device (or managed) memory usable on the current device; a
// host pointer handed to a kernel would fault, so device readback checks first.
int check_device_pointer(const void* p, const char* who);

}  // namespace sph

#define SPH_CUDA(call)                                                            \
    do {                                                                          \
        int _rc = ::sph::check_cuda((call), #call, __FILE__, __LINE__);           \
        if (_rc != SPH_OK) return _rc;                                            \
    } while (0)
