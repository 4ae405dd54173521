// Diagnostic entry point that lets the library's bounded device waits run
// out on purpose, so a caller (and the test suite) can see that an expired
// wait comes back as RNLA_ERR_TIMEOUT with the CUDA context still usable.
//
// Two waits are exercised, with the same primitives the solvers use:
//   which = 0: the grid barrier (grid_sync) of a cooperative launch over
//              every SM; the barrier's arrival counter starts far above the
//              grid size, so no CTA is ever the last to arrive and every CTA
//              waits for a generation that never comes;
//   which = 1: an mbarrier phase (mbar_wait) that expects two arrivals and
//              receives one.
// Each wait gives up after `limit_us` microseconds of %globaltimer, records
// its status word and returns; nothing is left in flight (no bulk copy, no
// TMEM, no peer that waits on the failed CTA).
#include "rnla_abi.h"
#include "rnla_async.cuh"

namespace rnla {

__global__ void __launch_bounds__(128) barrier_expiry_kernel(GridBarrier bar, unsigned long long limit_ns,
                                                             unsigned int* arrived) {
    if (grid_sync(bar, limit_ns) && threadIdx.x == 0) atomicAdd(arrived, 1u);
}

__global__ void __launch_bounds__(32) mbar_expiry_kernel(unsigned long long limit_ns, unsigned int* status) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int err_s;
    if (threadIdx.x == 0) {
        err_s = 0;
        mbar_init(&bar, 2);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_arrive(&bar);                       // one of the two expected arrivals
        volatile int* err = &err_s;
        const unsigned long long t0 = globaltimer_ns();
        bool done = false;
        while (!(done = mbar_try(&bar, 0u)))
            if (globaltimer_ns() - t0 > limit_ns) break;
        if (!done) {
            *err = 1;
            atomicCAS(status, 0u, (unsigned int)KSTATUS_MBAR_TIMEOUT);
        }
    }
}

}  // namespace rnla

using namespace rnla;

extern "C" int rnla_check_bounded_wait(int32_t which, int64_t limit_us, void* stream) {
    RNLA_API_BEGIN
    if (which != 0 && which != 1) fail(RNLA_ERR_INVALID_PARAMETERS, "which must be 0 (grid barrier) or 1 (mbarrier)");
    if (limit_us <= 0 || limit_us > 2000000) fail(RNLA_ERR_INVALID_PARAMETERS, "limit_us must be in (0, 2e6]");
    Ctx ctx((cudaStream_t)stream);
    const unsigned long long limit_ns = (unsigned long long)limit_us * 1000ull;
    DevBuf<unsigned int> words(3, ctx.stream);   // barrier count, generation, CTAs that passed
    const unsigned int start[3] = {0x40000000u, 0u, 0u};
    RNLA_CUDA(cudaMemcpyAsync(words.get(), start, sizeof start, cudaMemcpyHostToDevice, ctx.stream));
    ctx.clear_status();
    if (which == 0) {
        GridBarrier bar{words.get(), words.get() + 1, ctx.status};
        unsigned int* arrived = words.get() + 2;
        void* args[] = {&bar, (void*)&limit_ns, &arrived};
        RNLA_CUDA(cudaLaunchCooperativeKernel((const void*)barrier_expiry_kernel, dim3(ctx.sm_count), dim3(128),
                                              args, 0, ctx.stream));
        count_launch();
    } else {
        mbar_expiry_kernel<<<1, 32, 0, ctx.stream>>>(limit_ns, ctx.status);
        RNLA_LAUNCH_CHECK();
    }
    unsigned int passed = 0;
    RNLA_CUDA(cudaMemcpyAsync(&passed, words.get() + 2, sizeof passed, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    if (passed != 0) fail(RNLA_ERR_COMPUTATION, "a CTA passed a barrier that cannot complete");
    ctx.check_status(which == 0 ? "grid barrier self-check" : "mbarrier self-check");
    RNLA_API_END
}
