// Shared runtime pieces of librandnla_gb300: status codes and exceptions,
// CUDA error checks, stream-ordered device buffers, a bounded grid barrier
// for cooperative persistent kernels, and small reduction helpers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <stdexcept>
#include "../../include/randnla_gb300.h"

namespace rnla {

// C++ exception carried up to the C ABI, where it becomes an rnla_status
// plus the thread-local message returned by rnla_last_error_message().
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, const std::string& msg) { throw Error(code, msg); }

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
    if (e != cudaSuccess) {
        char buf[512];
        snprintf(buf, sizeof buf, "CUDA error in %s (%s:%d): %s", what, file, line,
                 cudaGetErrorString(e));
        throw Error(RNLA_ERR_CUDA, buf);
    }
}
#define RNLA_CUDA(x) ::rnla::cuda_check((x), #x, __FILE__, __LINE__)
// Every kernel launch of the library is followed by RNLA_LAUNCH_CHECK(),
// which also counts it (rnla_kernel_launches()).
void count_launch();
#define RNLA_LAUNCH_CHECK()                                                          \
    do {                                                                             \
        ::rnla::count_launch();                                                      \
        ::rnla::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__); \
    } while (0)

// Per-call context: stream plus device facts used for grid sizing.
struct Ctx {
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;      // side stream of this context (null: the device's shared one)
    int device = 0;
    int sm_count = 0;                 // SMs the grids are sized for (a batched worker takes a share)
    unsigned int* status = nullptr;   // device word: nonzero = kernel-side failure code
    // Deferred mode: the status word is not cleared between kernels (the
    // first failure code sticks, and later kernels that poll it stop early)
    // and check_status does not synchronise; finish() does one check.
    bool deferred = false;
    const char* deferred_where = nullptr;
    explicit Ctx(cudaStream_t s);
    ~Ctx();
    Ctx(const Ctx&) = delete;
    Ctx& operator=(const Ctx&) = delete;
    // Clears the status word before a kernel that reports through it (no-op
    // in deferred mode).
    void clear_status();
    // Reads the device status word (synchronises the stream); in deferred
    // mode only remembers `where`.
    void check_status(const char* where);
    // Leaves deferred mode and performs the pending check (synchronises).
    void finish(const char* where);
};

// Device buffer allocated from the library's stream-ordered pool and freed
// on the same stream when it goes out of scope.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(size_t count, cudaStream_t stream) { alloc(count, stream); }
    void alloc(size_t count, cudaStream_t stream);
    ~DevBuf() { release(); }
    void release();
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p; n = o.n; s = o.s;
            o.p = nullptr; o.n = 0;
        }
        return *this;
    }
    T* get() const { return p; }
    operator T*() const { return p; }
};

// Second stream of a device, and an event-based dependency `to` -> `from`.
cudaStream_t side_stream(int device);
cudaStream_t worker_stream(int device, int idx);
int batched_workers();
void set_smem_limit(const void* fn, size_t bytes);
cudaStream_t copy_stream(int device);
void stream_wait(cudaStream_t to, cudaStream_t from);

void* pool_alloc(size_t bytes, cudaStream_t s);
void pool_free(void* p, cudaStream_t s);

template <typename T>
void DevBuf<T>::alloc(size_t count, cudaStream_t stream) {
    release();
    s = stream;
    n = count;
    p = count ? static_cast<T*>(pool_alloc(count * sizeof(T), stream)) : nullptr;
}
template <typename T>
void DevBuf<T>::release() {
    if (p) pool_free(p, s);
    p = nullptr;
    n = 0;
}

// Kernel-side failure codes written to Ctx::status.
enum : unsigned int {
    KSTATUS_OK = 0,
    KSTATUS_BARRIER_TIMEOUT = 1,   // a grid barrier waited longer than its limit
    KSTATUS_MBAR_TIMEOUT = 2,      // an mbarrier wait gave up
    KSTATUS_SINGULAR = 3,          // zero pivot where the algorithm needs a nonzero one
    KSTATUS_NOT_PD = 4,            // Cholesky met a non-positive pivot
};

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum; `red` must hold blockDim.x/32 doubles.  All threads get the result.
__device__ __forceinline__ double block_sum(double v, double* red) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
    if (w == 0) t = warp_sum(t);
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier for cooperative launches (all CTAs co-resident by contract
// of cudaLaunchCooperativeKernel).  The wait is bounded: after `limit_ns`
// it records KSTATUS_BARRIER_TIMEOUT in *status and returns false, and the
// caller leaves the kernel.  count/gen live in device memory zeroed before
// the launch.
struct GridBarrier {
    unsigned int* count;
    unsigned int* gen;
    unsigned int* status;
};

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned int atom_add_acqrel_gpu(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_release_gpu(unsigned int* p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One thread per CTA arrives with a release-acquire atomic (after the CTA's
// __syncthreads, so it publishes the whole CTA's writes); the last arriver
// resets the count and publishes the next generation with a release store;
// the others poll the generation with acquire loads.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b, unsigned long long limit_ns = 2000000000ull) {
    __syncthreads();
    __shared__ int ok_s;
    if (threadIdx.x == 0) {
        ok_s = 1;
        const unsigned int nblocks = gridDim.x * gridDim.y * gridDim.z;
        const unsigned int my_gen = ld_acquire_gpu(b.gen);
        const unsigned int arrived = atom_add_acqrel_gpu(b.count, 1u);
        if (arrived == nblocks - 1) {
            *b.count = 0;
            st_release_gpu(b.gen, my_gen + 1u);
        } else {
            unsigned long long t0 = 0;
            unsigned int spins = 0;
            while (ld_acquire_gpu(b.gen) == my_gen) {
                if ((++spins & 31u) == 0u) {
                    if (*((volatile unsigned int*)b.status) != 0u) { ok_s = 0; break; }
                    const unsigned long long now = globaltimer_ns();
                    if (t0 == 0) t0 = now;
                    else if (now - t0 > limit_ns) {
                        atomicCAS(b.status, 0u, (unsigned int)KSTATUS_BARRIER_TIMEOUT);
                        ok_s = 0;
                        break;
                    }
                }
            }
        }
    }
    __syncthreads();
    return ok_s != 0;
}
#endif

}  // namespace rnla
