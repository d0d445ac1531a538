// noalloc.cu — facetcu_solve_noalloc: the reference-semantics Jacobi solve
// (the sweep of facetcu_solve) with no device allocation at all.
//
// Its working memory is one file-scope device array: the second radiosity
// buffer of the ping-pong pair (the caller's output is the first) followed
// by one max|dB| slot per sweep.  Host code must not use the array's name as
// a device address; every call looks the address up with
// cudaGetSymbolAddress on the current device (the context of that device may
// have been reset and the module reloaded since an earlier call, so a cached
// address could be stale) and passes it to the kernels.  Every call clears
// the parts that must start at zero.
#include <cmath>

#include "internal.h"

namespace {

constexpr uint32_t kMaxSurfaces = FACETCU_NOALLOC_MAX_SURFACES;
constexpr uint32_t kMaxIterations = FACETCU_NOALLOC_MAX_ITERATIONS;

// [0, kMaxSurfaces): radiosity buffer (float bits); then kMaxIterations
// max|dB| slots.  (1,048,576 + 4,096) x 4 B = 4.2 MB per device.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kMaxSurfaces + kMaxIterations];

// Device address of g_noalloc_scratch in the current device's context,
// looked up on every call (a host-side lookup, no device work).
int scratch_for_current_device(uint32_t** out)
{
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return FACETCU_NO_DEVICE;
    }
    void* ptr = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (rc != cudaSuccess || !ptr) {
        cudaGetLastError();
        return FACETCU_CUDA_ERROR;
    }
    *out = static_cast<uint32_t*>(ptr);
    return FACETCU_OK;
}

}  // namespace

extern "C" int facetcu_solve_noalloc(const uint32_t* row_offsets, const facetcu_csr_edge* edges,
                                     const uint32_t* denominators, const uint32_t* sky_counts,
                                     uint32_t surface_count, const facetcu_surface_optics* optics,
                                     float sky_radiosity, uint32_t iterations, float relaxation,
                                     float* radiosity, float* max_delta, void* stream)
{
    if (!row_offsets || !edges || !denominators || !sky_counts || !optics || !radiosity)
        return FACETCU_INVALID_ARGUMENT;
    if (surface_count == 0 || (surface_count & 1u)) return FACETCU_INVALID_ARGUMENT;
    if (surface_count > kMaxSurfaces) return FACETCU_OVERFLOW_ERROR;
    if (iterations == 0 || iterations > kMaxIterations) return FACETCU_INVALID_ARGUMENT;
    if (!(relaxation > 0.0f && relaxation <= 1.0f)) return FACETCU_INVALID_ARGUMENT;
    if (!std::isfinite(sky_radiosity) || sky_radiosity < 0.0f) return FACETCU_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (max_delta) {
        // reading max|dB| back waits for the stream, which a stream being
        // captured into a graph cannot do
        cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &capture) != cudaSuccess) {
            cudaGetLastError();
            return FACETCU_CUDA_ERROR;
        }
        if (capture != cudaStreamCaptureStatusNone) return FACETCU_INVALID_ARGUMENT;
    }
    uint32_t* scratch = nullptr;
    const int rc = scratch_for_current_device(&scratch);
    if (rc != FACETCU_OK) return rc;
    float* work = reinterpret_cast<float*>(scratch);
    uint32_t* residual = scratch + kMaxSurfaces;
    try {
        // Sweep i reads buffer i % 2 and writes (i + 1) % 2; the caller's
        // output is the buffer holding the final sweep, so no copy is needed.
        float* buf[2];
        buf[iterations & 1u] = radiosity;
        buf[(iterations + 1u) & 1u] = work;
        FCU_CHECK(cudaMemsetAsync(buf[0], 0, size_t(surface_count) * sizeof(float), s));
        FCU_CHECK(cudaMemsetAsync(residual, 0, size_t(iterations) * sizeof(uint32_t), s));
        for (uint32_t i = 0; i < iterations; ++i) {
            facetcu::jacobi_plain_sweep_raw(surface_count, row_offsets, edges, denominators,
                                            sky_counts, optics, sky_radiosity, relaxation,
                                            buf[i & 1u], buf[(i + 1u) & 1u], residual + i, s);
        }
        if (max_delta) {
            uint32_t bits = 0;
            FCU_CHECK(cudaMemcpyAsync(&bits, residual + iterations - 1u, sizeof(bits),
                                      cudaMemcpyDeviceToHost, s));
            FCU_CHECK(cudaStreamSynchronize(s));
            std::memcpy(max_delta, &bits, sizeof(bits));
        }
    } catch (const facetcu::Error& e) {
        return e.code;
    }
    return FACETCU_OK;
}
