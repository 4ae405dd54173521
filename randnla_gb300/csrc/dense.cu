// FP64 dense kernels on CUDA cores: the GEMM of the plain FP64 path
// (the reference's nalgebra `*` products, e.g. lora_helpers.rs:21,41,89,95
// and sketch_and_precondition.rs:51-52), plus copies and checks.
//
// GB300 executes FP64 at about 2 DFMA per clock per SM, so these kernels are
// bound by the FP64 pipe, not by memory; the tile below keeps 16 DFMA per
// thread per shared-memory step and splits K when the output has too few
// tiles to fill 152 SMs.
#include "rnla_internal.h"

namespace rnla {

constexpr int GB_M = 64, GB_N = 64, GB_K = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm_f64_kernel(int64_t M, int64_t N, int64_t K,
                                                      int64_t kchunk, double alpha,
                                                      const double* __restrict__ A, int64_t lda,
                                                      const double* __restrict__ B, int64_t ldb,
                                                      double beta, double* __restrict__ C,
                                                      int64_t ldc, double* __restrict__ W) {
    __shared__ __align__(16) double As[GB_K][GB_M];
    __shared__ __align__(16) double Bs[GB_K][GB_N];
    const int t = threadIdx.x;
    const int tx = t & 15, ty = t >> 4;
    const int64_t i0 = (int64_t)blockIdx.x * GB_M, j0 = (int64_t)blockIdx.y * GB_N;
    const int64_t kb = (int64_t)blockIdx.z * kchunk;
    const int64_t ke = min(K, kb + kchunk);
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

    for (int64_t k0 = kb; k0 < ke; k0 += GB_K) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            int ii, kk;
            if (!TA) { ii = t & 63; kk = (t >> 6) + 4 * r; }
            else     { kk = t & 15; ii = (t >> 4) + 16 * r; }
            const int64_t gi = i0 + ii, gk = k0 + kk;
            double v = 0.0;
            if (gi < M && gk < ke) v = TA ? A[gk + gi * lda] : A[gi + gk * lda];
            As[kk][ii] = v;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            int jj, kk;
            if (!TB) { kk = t & 15; jj = (t >> 4) + 16 * r; }
            else     { jj = t & 63; kk = (t >> 6) + 4 * r; }
            const int64_t gj = j0 + jj, gk = k0 + kk;
            double v = 0.0;
            if (gj < N && gk < ke) v = TB ? B[gj + gk * ldb] : B[gk + gj * ldb];
            Bs[kk][jj] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            const double2 a01 = *reinterpret_cast<const double2*>(&As[kk][ty * 4]);
            const double2 a23 = *reinterpret_cast<const double2*>(&As[kk][ty * 4 + 2]);
            const double2 b01 = *reinterpret_cast<const double2*>(&Bs[kk][tx * 4]);
            const double2 b23 = *reinterpret_cast<const double2*>(&Bs[kk][tx * 4 + 2]);
            const double av[4] = {a01.x, a01.y, a23.x, a23.y};
            const double bv[4] = {b01.x, b01.y, b23.x, b23.y};
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int64_t gj = j0 + tx * 4 + b;
        if (gj >= N) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int64_t gi = i0 + ty * 4 + a;
            if (gi >= M) continue;
            if (W) {
                W[(int64_t)blockIdx.z * M * N + gi + gj * M] = acc[a][b];
            } else {
                double* c = C + gi + gj * ldc;
                *c = (beta == 0.0) ? alpha * acc[a][b] : fma(alpha, acc[a][b], beta * *c);
            }
        }
    }
}

__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int splits, const double* __restrict__ W,
                                     double alpha, double beta, double* __restrict__ C, int64_t ldc) {
    const int64_t total = M * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int z = 0; z < splits; ++z) s += W[(int64_t)z * total + e];
        const int64_t i = e % M, j = e / M;
        double* c = C + i + j * ldc;
        *c = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * *c);
    }
}

void gemm_f64(Ctx& ctx, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
              const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
              int64_t ldc) {
    if (M <= 0 || N <= 0) return;
    if (K <= 0) {
        if (beta == 0.0) fill_zero(ctx, M, N, C, ldc);
        else if (beta != 1.0) {
            // scale C by beta: C = 0*C + beta*C via a reduce with zero splits
            splitk_reduce_kernel<<<div_up(M * N, 256) < 4096 ? div_up(M * N, 256) : 4096, 256, 0,
                                   ctx.stream>>>(M, N, 0, nullptr, 0.0, beta, C, ldc);
            RNLA_LAUNCH_CHECK();
        }
        return;
    }
    const int64_t tiles = (int64_t)div_up(M, GB_M) * div_up(N, GB_N);
    const int64_t want = 3LL * ctx.sm_count;
    int64_t splits = 1;
    if (tiles < want) {
        splits = (want + tiles - 1) / tiles;
        const int64_t kmax = (K + 255) / 256;
        if (splits > kmax) splits = kmax;
        if (splits < 1) splits = 1;
    }
    // keep the split-K workspace bounded (512 MB)
    while (splits > 1 && splits * M * N * (int64_t)sizeof(double) > (512LL << 20)) --splits;
    int64_t kchunk = (K + splits - 1) / splits;
    kchunk = ((kchunk + GB_K - 1) / GB_K) * GB_K;
    splits = (K + kchunk - 1) / kchunk;
    DevBuf<double> W;
    if (splits > 1) W.alloc((size_t)(splits * M * N), ctx.stream);
    dim3 grid(div_up(M, GB_M), div_up(N, GB_N), (unsigned)splits);
    const bool tA = (ta == 'T' || ta == 't'), tB = (tb == 'T' || tb == 't');
#define RNLA_GEMM_LAUNCH(TA_, TB_)                                                              \
    gemm_f64_kernel<TA_, TB_><<<grid, 256, 0, ctx.stream>>>(M, N, K, kchunk, alpha, A, lda, B,  \
                                                            ldb, beta, C, ldc, W.get())
    if (!tA && !tB) RNLA_GEMM_LAUNCH(false, false);
    else if (tA && !tB) RNLA_GEMM_LAUNCH(true, false);
    else if (!tA && tB) RNLA_GEMM_LAUNCH(false, true);
    else RNLA_GEMM_LAUNCH(true, true);
#undef RNLA_GEMM_LAUNCH
    RNLA_LAUNCH_CHECK();
    if (splits > 1) {
        int g = div_up(M * N, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        splitk_reduce_kernel<<<g, 256, 0, ctx.stream>>>(M, N, (int)splits, W.get(), alpha, beta, C,
                                                        ldc);
        RNLA_LAUNCH_CHECK();
    }
}

// ---------------------------------------------------------------------------
// Copies and fills
// ---------------------------------------------------------------------------
template <typename S>
__global__ void copy_kernel(int64_t rows, int64_t cols, const S* __restrict__ src, int64_t lds,
                            double* __restrict__ dst, int64_t ldd) {
    const int64_t total = rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % rows, j = e / rows;
        dst[i + j * ldd] = (double)src[i + j * lds];
    }
}

static int grid1d(Ctx& ctx, int64_t work) {
    int64_t g = (work + 255) / 256;
    if (g > 16LL * ctx.sm_count) g = 16LL * ctx.sm_count;
    return (int)(g < 1 ? 1 : g);
}

void copy_matrix(Ctx& ctx, int64_t rows, int64_t cols, const double* src, int64_t lds, double* dst,
                 int64_t ldd) {
    if (rows <= 0 || cols <= 0) return;
    copy_kernel<double><<<grid1d(ctx, rows * cols), 256, 0, ctx.stream>>>(rows, cols, src, lds, dst, ldd);
    RNLA_LAUNCH_CHECK();
}

void copy_matrix_f32_to_f64(Ctx& ctx, int64_t rows, int64_t cols, const float* src, int64_t lds,
                            double* dst, int64_t ldd) {
    if (rows <= 0 || cols <= 0) return;
    copy_kernel<float><<<grid1d(ctx, rows * cols), 256, 0, ctx.stream>>>(rows, cols, src, lds, dst, ldd);
    RNLA_LAUNCH_CHECK();
}

__global__ void transpose_kernel(int64_t rows, int64_t cols, const double* __restrict__ src,
                                 int64_t lds, double* __restrict__ dst, int64_t ldd) {
    __shared__ double tile[32][33];
    const int64_t bi = (int64_t)blockIdx.x * 32, bj = (int64_t)blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = bi + threadIdx.x, j = bj + r;
        if (i < rows && j < cols) tile[r][threadIdx.x] = src[i + j * lds];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t j = bj + threadIdx.x, i = bi + r;   // dst(j, i) = src(i, j)
        if (i < rows && j < cols) dst[j + i * ldd] = tile[threadIdx.x][r];
    }
}

void transpose(Ctx& ctx, int64_t rows, int64_t cols, const double* src, int64_t lds, double* dst,
               int64_t ldd) {
    if (rows <= 0 || cols <= 0) return;
    dim3 grid(div_up(rows, 32), div_up(cols, 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, ctx.stream>>>(rows, cols, src, lds, dst, ldd);
    RNLA_LAUNCH_CHECK();
}

__global__ void fill_kernel(int64_t rows, int64_t cols, double* dst, int64_t ld, int identity) {
    const int64_t total = rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % rows, j = e / rows;
        dst[i + j * ld] = (identity && i == j) ? 1.0 : 0.0;
    }
}

void fill_identity(Ctx& ctx, int64_t rows, int64_t cols, double* dst, int64_t ld) {
    if (rows <= 0 || cols <= 0) return;
    fill_kernel<<<grid1d(ctx, rows * cols), 256, 0, ctx.stream>>>(rows, cols, dst, ld, 1);
    RNLA_LAUNCH_CHECK();
}

void fill_zero(Ctx& ctx, int64_t rows, int64_t cols, double* dst, int64_t ld) {
    if (rows <= 0 || cols <= 0) return;
    fill_kernel<<<grid1d(ctx, rows * cols), 256, 0, ctx.stream>>>(rows, cols, dst, ld, 0);
    RNLA_LAUNCH_CHECK();
}

__global__ void finite_kernel(int64_t rows, int64_t cols, const double* __restrict__ a, int64_t lda,
                              unsigned int* flag) {
    const int64_t total = rows * cols;
    bool bad = false;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % rows, j = e / rows;
        if (!isfinite(a[i + j * lda])) bad = true;
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

bool all_finite(Ctx& ctx, int64_t rows, int64_t cols, const double* a, int64_t lda) {
    if (rows <= 0 || cols <= 0) return true;
    DevBuf<unsigned int> f(1, ctx.stream);
    RNLA_CUDA(cudaMemsetAsync(f.get(), 0, sizeof(unsigned int), ctx.stream));
    finite_kernel<<<grid1d(ctx, rows * cols), 256, 0, ctx.stream>>>(rows, cols, a, lda, f.get());
    RNLA_LAUNCH_CHECK();
    unsigned int h = 0;
    RNLA_CUDA(cudaMemcpyAsync(&h, f.get(), sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    return h == 0;
}

}  // namespace rnla
