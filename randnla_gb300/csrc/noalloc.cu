// LSQR entry point that allocates no device memory.
//
// Some callers cannot let a library allocate: applications that run under a
// fixed device-memory budget handed out by their own allocator (a cudaMalloc
// from inside a library can fail once that budget is committed, and it can
// synchronise the device at a moment the caller does not control), and
// latency-bound loops that must not pay a cudaMalloc/cudaFree pair per call.
// For them this file provides rnla_lsqr_noalloc_dev: the caller passes A, b,
// x0 and x (device pointers) and a stream; all scratch (the u/v/w/y vectors,
// per-CTA partial sums, the grid-barrier words, the status word and the
// result record) lives in the fixed array below.
//
// Limits and behaviour:
//   * the array holds RNLA_NOALLOC_SCRATCH_BYTES (32 MiB); every GPU that
//     loads this library keeps it reserved until the process exits;
//   * a problem needs 8 * (10 + 4G + m + 5n + G n) bytes, G = cooperative
//     grid size (up to 4 CTAs per SM); larger problems are rejected with
//     RNLA_ERR_INVALID_DIMENSIONS and a message giving both sizes;
//   * every call shares the array and leaves its contents behind; the words
//     that must start at zero are cleared by each call, the rest is written
//     before it is read;
//   * calls on one device are serialised: each holds that device's lock
//     from before its first launch until it has synchronised on its result,
//     so calls from several host threads or streams never overlap on the
//     array;
//   * n is at most 4096 (as for rnla_lsqr_dev); a larger n returns
//     RNLA_ERR_UNSUPPORTED;
//   * the first call on a device looks the array's device address up
//     (cudaGetSymbolAddress, with that device current) and caches it;
//   * every call clears its words with cudaMemsetAsync, queries the kernel's
//     occupancy and synchronises the stream it is given on its result
//     before it returns, so it must not be called on a stream that is being
//     captured into a graph.
#include "rnla_abi.h"
#include <mutex>

#define RNLA_NOALLOC_SCRATCH_BYTES (32u << 20)

namespace rnla {

static __device__ __align__(256) unsigned char g_noalloc_scratch[RNLA_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
std::mutex g_noalloc_call_mu[kMaxDevices];   // one call per device at a time
void* g_noalloc_ptr[kMaxDevices] = {};
int g_noalloc_sms[kMaxDevices] = {};

// Once per device, with that device current: the device address of the
// array (its host-side name is only a stand-in and must not reach a kernel).
void* noalloc_scratch(int dev, int* sms) {
    if (dev < 0 || dev >= kMaxDevices) fail(RNLA_ERR_CUDA, "device index out of range");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            fail(RNLA_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
        }
        int c = 0;
        RNLA_CUDA(cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev));
        g_noalloc_ptr[dev] = p;
        g_noalloc_sms[dev] = c;
    }
    *sms = g_noalloc_sms[dev];
    return g_noalloc_ptr[dev];
}
}  // namespace

}  // namespace rnla

using namespace rnla;

extern "C" int rnla_lsqr_noalloc_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda,
                                     const double* b_dev, double damp, double atol, double btol,
                                     double conlim, int64_t iter_lim, const double* x0_dev,
                                     double* x_dev, rnla_lsqr_result* result, void* stream) {
    RNLA_API_BEGIN
    if (m < 0 || n < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "negative dimension");
    if (m == 0 || n == 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    if (lda < m) fail(RNLA_ERR_INVALID_PARAMETERS, "leading dimension smaller than rows");
    int dev = 0;
    RNLA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) fail(RNLA_ERR_CUDA, "device index out of range");
    // held until lsqr_run_in_workspace has synchronised on the result
    std::lock_guard<std::mutex> call(g_noalloc_call_mu[dev]);
    // each of m and n alone must fit the array as doubles before the size
    // arithmetic below (which cannot overflow then: n <= 4096 is checked next)
    if ((uint64_t)m > RNLA_NOALLOC_SCRATCH_BYTES / 8 || (uint64_t)n > RNLA_NOALLOC_SCRATCH_BYTES / 8) {
        char buf[200];
        snprintf(buf, sizeof buf,
                 "rnla_lsqr_noalloc_dev: an %lld x %lld problem needs more than the %u bytes of scratch "
                 "the allocation-free entry point holds",
                 (long long)m, (long long)n, (unsigned)RNLA_NOALLOC_SCRATCH_BYTES);
        fail(RNLA_ERR_INVALID_DIMENSIONS, buf);
    }
    int sms = 0;
    void* ws = noalloc_scratch(dev, &sms);
    const size_t need = lsqr_workspace_bytes(m, n, sms, nullptr, nullptr, nullptr);
    if (need > RNLA_NOALLOC_SCRATCH_BYTES) {
        char buf[200];
        snprintf(buf, sizeof buf,
                 "rnla_lsqr_noalloc_dev: an %lld x %lld problem needs %zu bytes of scratch; the "
                 "allocation-free entry point holds %u",
                 (long long)m, (long long)n, need, (unsigned)RNLA_NOALLOC_SCRATCH_BYTES);
        fail(RNLA_ERR_INVALID_DIMENSIONS, buf);
    }
    LsqrParams p;
    p.damp = damp;
    p.atol = atol;
    p.btol = btol;
    p.conlim = conlim;
    p.iter_lim = iter_lim < 0 ? 2 * n : iter_lim;
    const LsqrResult r = lsqr_run_in_workspace((cudaStream_t)stream, sms, ws, RNLA_NOALLOC_SCRATCH_BYTES,
                                               a_dev, m, n, lda, b_dev, x0_dev, p, x_dev);
    if (result) {
        result->istop = r.istop;
        result->itn = r.itn;
        result->r1norm = r.r1norm;
        result->r2norm = r.r2norm;
        result->anorm = r.anorm;
        result->acond = r.acond;
        result->xnorm = r.xnorm;
    }
    RNLA_API_END
}
