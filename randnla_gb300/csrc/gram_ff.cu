// Float-float products of tall-skinny matrices on the FP32 pipe:
//
//   C (N1 x N2, FP64) = X^T Y,  X (K x N1), Y (K x N2) column-major FP64,
//
// K large (tens of thousands of rows), N1, N2 up to about a thousand.  Used
// where a product must be accurate to FP64 level but the FP64 pipe (1/64 of
// the FP32 rate on GB300) would take milliseconds: the Gram of the range
// basis before the projection of rand_svd (an FP32-accumulated Gram would
// leave the basis orthonormal only to ~1e-5 at K = 65536), and B B^T in the
// small-SVD finish.
//
// Each CTA computes a 64 x 64 tile of C over one K chunk: 32-row slices of X
// and Y are split into float-float (hi, lo) pairs in shared memory, each of
// the 256 threads accumulates a 4 x 4 block with exact products (FMA error
// terms) and TwoSum on packed f32x2 pairs (~48 significant bits), and the
// chunk's tile goes to a partial buffer; the chunks are summed in a fixed
// order, so the result is reproducible.
#include "rnla_internal.h"
#include "rnla_ff.cuh"

namespace rnla {
namespace gff {

constexpr int TM = 64;          // tile rows / columns
constexpr int KC = 32;          // K rows per shared-memory slice
constexpr int THREADS = 256;

// Tile (t1, t2) of C for a linear tile index: column-major over all tiles,
// or for a symmetric product X^T X over the upper triangle t1 <= t2 only.
__host__ __device__ __forceinline__ void tile_coords(int tile, int tiles1, int sym, int& t1, int& t2) {
    if (!sym) {
        t1 = tile % tiles1;
        t2 = tile / tiles1;
        return;
    }
    int c = (int)((sqrt(8.0 * tile + 1.0) - 1.0) * 0.5);
    while ((c + 1) * (c + 2) / 2 <= tile) ++c;
    while (c * (c + 1) / 2 > tile) --c;
    t2 = c;
    t1 = tile - c * (c + 1) / 2;
}

__global__ void __launch_bounds__(THREADS) gram_ff_kernel(const double* __restrict__ X, int64_t ldx, int64_t N1,
                                                          const double* __restrict__ Y, int64_t ldy, int64_t N2,
                                                          int64_t K, int64_t rows_per_chunk, int tiles1, int sym,
                                                          float4* __restrict__ part) {
    __shared__ float2 xs[KC][TM + 1];
    __shared__ float2 ys[KC][TM + 1];
    const int tile = blockIdx.x, chunk = blockIdx.y;
    int t1, t2;
    tile_coords(tile, tiles1, sym, t1, t2);
    const int64_t i0 = (int64_t)t1 * TM, j0 = (int64_t)t2 * TM;
    const int64_t k0 = (int64_t)chunk * rows_per_chunk;
    const int64_t k1 = min(K, k0 + rows_per_chunk);
    const int tid = threadIdx.x;
    const int ti = tid & 15, tj = tid >> 4;          // 4 x 4 block (rows 4 ti.., columns 4 tj..)
    f32x2 ah[4][2], al[4][2];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) { ah[a][b] = 0ull; al[a][b] = 0ull; }
    for (int64_t kb = k0; kb < k1; kb += KC) {
        // stage: element (k, c) of each 32 x 64 slice; consecutive threads take consecutive k
        for (int e = tid; e < KC * TM; e += THREADS) {
            const int k = e % KC, c = e / KC;
            const int64_t kg = kb + k;
            const bool kin = kg < k1;
            xs[k][c] = (kin && i0 + c < N1) ? ff_split(X[kg + (i0 + c) * ldx]) : make_float2(0.f, 0.f);
            ys[k][c] = (kin && j0 + c < N2) ? ff_split(Y[kg + (j0 + c) * ldy]) : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < KC; ++k) {
            f32x2 bh[2], nbh[2], bl[2];
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                const float2 y0 = ys[k][4 * tj + 2 * b], y1 = ys[k][4 * tj + 2 * b + 1];
                bh[b] = pk2(y0.x, y1.x);
                nbh[b] = pk2(-y0.x, -y1.x);
                bl[b] = pk2(y0.y, y1.y);
            }
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float2 x = xs[k][4 * ti + a];
                const f32x2 xh = pk2(x.x, x.x), xl = pk2(x.y, x.y);
#pragma unroll
                for (int b = 0; b < 2; ++b) ff2_madd(xh, xl, bh[b], nbh[b], bl[b], ah[a][b], al[a][b]);
            }
        }
        __syncthreads();
    }
    // partial tile: [chunk][tile][64 x 64] as (hi, lo) of two adjacent columns
    float4* out = part + ((size_t)chunk * gridDim.x + tile) * (TM * TM / 2);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const float2 H = upk2(ah[a][b]), L = upk2(al[a][b]);
            const float2 c0 = ff_norm(H.x, L.x), c1 = ff_norm(H.y, L.y);
            out[(4 * ti + a) * (TM / 2) + 2 * tj + b] = make_float4(c0.x, c0.y, c1.x, c1.y);
        }
}

// C[i + j ldc] = sum over chunks (fixed order, float-float) of the partials.
// (for a symmetric product the lower tiles are read from their mirror)
__global__ void gram_sum_kernel(const float4* __restrict__ part, int chunks, int tiles1, int tiles, int sym,
                                int64_t N1, int64_t N2, double* __restrict__ C, int64_t ldc) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < N1 * N2; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = e % N1, j = e / N1;
        const int64_t io = i, jo = j;
        int tile;
        if (sym) {
            if (i / TM > j / TM) { const int64_t t = i; i = j; j = t; }
            const int a = (int)(i / TM), b = (int)(j / TM);
            tile = b * (b + 1) / 2 + a;
        } else {
            tile = (int)(i / TM) + tiles1 * (int)(j / TM);
        }
        const int r = (int)(i % TM), c = (int)(j % TM);
        float h = 0.f, l = 0.f;
        for (int ch = 0; ch < chunks; ++ch) {
            const float4 v = part[((size_t)ch * tiles + tile) * (TM * TM / 2) + r * (TM / 2) + (c >> 1)];
            if (c & 1) ff_acc(h, l, v.z, v.w);
            else ff_acc(h, l, v.x, v.y);
        }
        const float2 s = ff_norm(h, l);
        C[io + jo * ldc] = (double)s.x + (double)s.y;
    }
}

}  // namespace gff

void gram_ff(Ctx& ctx, const double* X, int64_t ldx, int64_t N1, const double* Y, int64_t ldy, int64_t N2,
             int64_t K, double* C, int64_t ldc) {
    using namespace gff;
    if (N1 <= 0 || N2 <= 0) return;
    if (K <= 0) {
        fill_zero(ctx, N1, N2, C, ldc);
        return;
    }
    // X^T X: the upper tiles only, mirrored in the sum
    const int sym = (X == Y && ldx == ldy && N1 == N2) ? 1 : 0;
    const int tiles1 = div_up(N1, TM), tiles2 = div_up(N2, TM);
    const int tiles = sym ? tiles1 * (tiles1 + 1) / 2 : tiles1 * tiles2;
    // about eight CTAs per SM over (tile, K chunk), chunks a multiple of 32
    // rows: with ~2 per SM a tile count just above the SM count (153
    // symmetric tiles of a 1025-column Gram on 152 SMs) leaves a few SMs
    // with half again the work of the rest
    int chunks = div_up(8 * ctx.sm_count, tiles);
    const int64_t max_chunks = div_up(K, KC);
    if (chunks > max_chunks) chunks = (int)max_chunks;
    if (chunks > 4096) chunks = 4096;
    const int64_t rpc = ((div_up(K, chunks) + KC - 1) / KC) * KC;
    chunks = div_up(K, rpc);
    DevBuf<float4> part((size_t)chunks * tiles * (TM * TM / 2), ctx.stream);
    gram_ff_kernel<<<dim3((unsigned)tiles, (unsigned)chunks), THREADS, 0, ctx.stream>>>(X, ldx, N1, Y, ldy, N2, K, rpc,
                                                                                   tiles1, sym, part);
    RNLA_LAUNCH_CHECK();
    int g = div_up(N1 * N2, 256);
    if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
    gram_sum_kernel<<<g, 256, 0, ctx.stream>>>(part, chunks, tiles1, tiles, sym, N1, N2, C, ldc);
    RNLA_LAUNCH_CHECK();
}

}  // namespace rnla
