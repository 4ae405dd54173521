// Helpers shared by the C entry points: exception -> status translation,
// the per-thread stream used by host-pointer entry points, and strided
// host <-> device matrix copies.
#pragma once
#include "rnla_internal.h"
#include <new>

namespace rnla {
int abi_error(int code, const char* msg);
int abi_ok();
cudaStream_t host_stream();
RngKey key_of(const rnla_rng* r);

inline void h2d_matrix(double* dev, int64_t ldd, const double* host, int64_t ldh, int64_t rows,
                       int64_t cols, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return;
    RNLA_CUDA(cudaMemcpy2DAsync(dev, ldd * sizeof(double), host, ldh * sizeof(double),
                                rows * sizeof(double), cols, cudaMemcpyHostToDevice, s));
}
inline void d2h_matrix(double* host, int64_t ldh, const double* dev, int64_t ldd, int64_t rows,
                       int64_t cols, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return;
    RNLA_CUDA(cudaMemcpy2DAsync(host, ldh * sizeof(double), dev, ldd * sizeof(double),
                                rows * sizeof(double), cols, cudaMemcpyDeviceToHost, s));
}
}  // namespace rnla

#define RNLA_API_BEGIN try {
#define RNLA_API_END                                                           \
    }                                                                          \
    catch (const ::rnla::Error& e) {                                           \
        return ::rnla::abi_error(e.code, e.what());                            \
    }                                                                          \
    catch (const std::bad_alloc&) {                                            \
        return ::rnla::abi_error(RNLA_ERR_COMPUTATION, "host allocation failed"); \
    }                                                                          \
    catch (const std::exception& e) {                                          \
        return ::rnla::abi_error(RNLA_ERR_COMPUTATION, e.what());              \
    }                                                                          \
    catch (...) {                                                              \
        return ::rnla::abi_error(RNLA_ERR_COMPUTATION, "unknown failure");     \
    }                                                                          \
    return ::rnla::abi_ok();
