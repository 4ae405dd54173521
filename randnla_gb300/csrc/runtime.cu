// Library runtime: device memory pool, per-call context, error reporting,
// generator kernels and their C entry points.
#include <algorithm>
#include "rnla_internal.h"
#include "rnla_abi.h"
#include <mutex>
#include <map>
#include <cstring>
#include <atomic>

namespace rnla {

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// Stream-ordered pool (one per device, never shrinks between calls)
// ---------------------------------------------------------------------------
// One stream-ordered pool per device, created on first use.  Its release
// threshold is unlimited, so steady-state solves take every scratch buffer
// from memory the pool already holds; rnla_release_cached_memory() trims it.
static std::mutex g_pool_mu;
static std::map<int, cudaMemPool_t> g_pools;

static cudaMemPool_t device_pool(int dev) {
    std::mutex& mu = g_pool_mu;
    std::map<int, cudaMemPool_t>& pools = g_pools;
    std::lock_guard<std::mutex> g(mu);
    auto it = pools.find(dev);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props;
    memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    RNLA_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t thresh = ~0ull;
    RNLA_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thresh));
    // memory freed on one stream is reused on another only through event
    // dependencies the library made itself: the pool must not insert waits
    // between unrelated streams (the batched solver's workers would serialise)
    int no = 0;
    RNLA_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no));
    pools[dev] = pool;
    return pool;
}

void* pool_alloc(size_t bytes, cudaStream_t s) {
    int dev;
    RNLA_CUDA(cudaGetDevice(&dev));
    void* p = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, device_pool(dev), s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        char buf[160];
        snprintf(buf, sizeof buf, "device allocation of %zu bytes failed: %s", bytes,
                 cudaGetErrorString(e));
        throw Error(RNLA_ERR_CUDA, buf);
    }
    return p;
}

void pool_free(void* p, cudaStream_t s) { cudaFreeAsync(p, s); }

static int sm_count_of(int dev) {
    static std::mutex mu;
    static std::map<int, int> cache;
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int c = 0;
    RNLA_CUDA(cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev));
    cache[dev] = c;
    return c;
}

// One lazily created, never destroyed, non-blocking stream per device and
// purpose: `side` for work that overlaps the caller's stream (the sketch
// generator, the solver's input copies), `copy` for host <-> device copies.
static cudaStream_t device_stream(std::map<int, cudaStream_t>& cache, std::mutex& mu, int dev) {
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    cudaStream_t st = nullptr;
    RNLA_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cache[dev] = st;
    return st;
}

cudaStream_t side_stream(int dev) {
    static std::mutex mu;
    static std::map<int, cudaStream_t> cache;
    return device_stream(cache, mu, dev);
}

// Streams of the batched solver's workers: index 2 w (main) and 2 w + 1
// (side) of worker w, created on first use and kept.
cudaStream_t worker_stream(int dev, int idx) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, cudaStream_t> cache;
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find({dev, idx});
    if (it != cache.end()) return it->second;
    cudaStream_t st = nullptr;
    RNLA_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cache[{dev, idx}] = st;
    return st;
}

int batched_workers() { return 4; }

// The dynamic shared-memory limit of a kernel only ever grows: concurrent
// callers (the batched solver's workers) launching one kernel with different
// sizes must never see the limit lowered under them between their own
// setting and their launch.
void set_smem_limit(const void* fn, size_t bytes) {
    static std::mutex mu;
    static std::map<const void*, size_t> cur;
    std::lock_guard<std::mutex> g(mu);
    size_t& c = cur[fn];
    if (bytes <= c) return;
    RNLA_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    c = bytes;
}

cudaStream_t copy_stream(int dev) {
    static std::mutex mu;
    static std::map<int, cudaStream_t> cache;
    return device_stream(cache, mu, dev);
}

void h2d_columns_async(void* dev, const void* a, size_t esize, int64_t m, int64_t n, int64_t lda, int64_t chunk,
                       cudaStream_t s, ColumnFeed& feed) {
    int d = 0;
    RNLA_CUDA(cudaGetDevice(&d));
    const cudaStream_t cp = copy_stream(d);
    stream_wait(cp, s);                            // the device buffer exists
    feed.cols = chunk;
    feed.owner = s;
    for (int64_t j0 = 0; j0 < n; j0 += chunk) {
        const int64_t c = std::min(chunk, n - j0);
        RNLA_CUDA(cudaMemcpy2DAsync(static_cast<char*>(dev) + (size_t)j0 * m * esize, m * esize,
                                    static_cast<const char*>(a) + (size_t)j0 * lda * esize, lda * esize,
                                    m * esize, c, cudaMemcpyHostToDevice, cp));
        cudaEvent_t ev;
        RNLA_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        feed.ready.push_back(ev);
        RNLA_CUDA(cudaEventRecord(ev, cp));
    }
}

// `to` waits for the work enqueued on `from` so far.
void stream_wait(cudaStream_t to, cudaStream_t from) {
    cudaEvent_t ev;
    RNLA_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    RNLA_CUDA(cudaEventRecord(ev, from));
    RNLA_CUDA(cudaStreamWaitEvent(to, ev, 0));
    RNLA_CUDA(cudaEventDestroy(ev));
}

Ctx::Ctx(cudaStream_t s) : stream(s) {
    RNLA_CUDA(cudaGetDevice(&device));
    sm_count = sm_count_of(device);
    status = static_cast<unsigned int*>(pool_alloc(sizeof(unsigned int) * 4, s));
    RNLA_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned int) * 4, s));
}

Ctx::~Ctx() {
    if (status) pool_free(status, stream);
}

void Ctx::clear_status() {
    if (!deferred) RNLA_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned int), stream));
}

void Ctx::finish(const char* where) {
    deferred = false;
    check_status(deferred_where ? deferred_where : where);
    deferred_where = nullptr;
}

void Ctx::check_status(const char* where) {
    if (deferred) {
        if (!deferred_where) deferred_where = where;
        return;
    }
    unsigned int h = 0;
    RNLA_CUDA(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, stream));
    RNLA_CUDA(cudaStreamSynchronize(stream));
    if (h == KSTATUS_OK) return;
    char buf[256];
    if (h == KSTATUS_BARRIER_TIMEOUT || h == KSTATUS_MBAR_TIMEOUT) {
        snprintf(buf, sizeof buf, "%s: a device-side wait exceeded its limit (code %u)", where, h);
        throw Error(RNLA_ERR_TIMEOUT, buf);
    }
    if (h == KSTATUS_SINGULAR) {
        snprintf(buf, sizeof buf, "%s: zero pivot", where);
        throw Error(RNLA_ERR_SINGULAR_MATRIX, buf);
    }
    snprintf(buf, sizeof buf, "%s: device status %u", where, h);
    throw Error(RNLA_ERR_COMPUTATION, buf);
}

// ---------------------------------------------------------------------------
// Generator kernels
// ---------------------------------------------------------------------------
__global__ void rng_words_kernel(RngKey key, uint64_t first_word, int64_t n, uint32_t* out) {
    const uint64_t g0 = first_word >> 2;
    const uint64_t g1 = (first_word + (uint64_t)n - 1) >> 2;
    for (uint64_t g = g0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g <= g1;
         g += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t w[4];
        block_words(key, g, w);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const uint64_t L = 4 * g + t;
            if (L >= first_word && L < first_word + (uint64_t)n) out[L - first_word] = w[t];
        }
    }
}

template <typename T, bool QUANT>
__global__ void sketch_fill_kernel(RngKey key, int dist, int64_t rows, int64_t cols, T* out,
                                   int64_t ld) {
    const int64_t bpc = (rows + 3) >> 2;   // blocks per column (rows padded to a multiple of 4)
    const uint64_t total = (uint64_t)bpc * (uint64_t)cols;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < total;
         g += (uint64_t)gridDim.x * blockDim.x) {
        const int64_t j = (int64_t)(g / (uint64_t)bpc);
        const int64_t i0 = 4 * (int64_t)(g % (uint64_t)bpc);
        float v[4];
        if (QUANT) {
            uint32_t w[4];
            block_words(key, g, w);
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ldexpf((float)quant_t(dist, w[t], k_qgauss_table), -quant_shift(dist));
        } else {
            block_entries(key, dist, g, v);
        }
        T* col = out + j * ld;
#pragma unroll
        for (int t = 0; t < 4; ++t)
            if (i0 + t < rows) col[i0 + t] = (T)v[t];
    }
}

static int grid_for(Ctx& ctx, uint64_t work, int threads) {
    uint64_t want = (work + threads - 1) / threads;
    uint64_t cap = (uint64_t)ctx.sm_count * 16;
    return (int)(want < cap ? (want ? want : 1) : cap);
}

void rng_words(Ctx& ctx, const RngKey& key, uint64_t first_word, int64_t n, uint32_t* out) {
    if (n <= 0) return;
    const uint64_t blocks = ((first_word + n - 1) >> 2) - (first_word >> 2) + 1;
    rng_words_kernel<<<grid_for(ctx, blocks, 256), 256, 0, ctx.stream>>>(key, first_word, n, out);
    RNLA_LAUNCH_CHECK();
}

void sketch_fill_f64(Ctx& ctx, int dist, const RngKey& key, int64_t rows, int64_t cols,
                     double* out, int64_t ld) {
    const uint64_t blocks = (uint64_t)((rows + 3) >> 2) * (uint64_t)cols;
    sketch_fill_kernel<double, false><<<grid_for(ctx, blocks, 256), 256, 0, ctx.stream>>>(
        key, dist, rows, cols, out, ld);
    RNLA_LAUNCH_CHECK();
}

void sketch_fill_f32(Ctx& ctx, int dist, const RngKey& key, int64_t rows, int64_t cols,
                     bool quantized, float* out, int64_t ld) {
    const uint64_t blocks = (uint64_t)((rows + 3) >> 2) * (uint64_t)cols;
    if (quantized)
        sketch_fill_kernel<float, true><<<grid_for(ctx, blocks, 256), 256, 0, ctx.stream>>>(
            key, dist, rows, cols, out, ld);
    else
        sketch_fill_kernel<float, false><<<grid_for(ctx, blocks, 256), 256, 0, ctx.stream>>>(
            key, dist, rows, cols, out, ld);
    RNLA_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// ABI support
// ---------------------------------------------------------------------------
static thread_local std::string t_last_error;

int abi_error(int code, const char* msg) {
    t_last_error = msg ? msg : "";
    return code;
}
int abi_ok() {
    t_last_error.clear();
    return RNLA_OK;
}

cudaStream_t host_stream() {
    int dev;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(RNLA_ERR_CUDA, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
    }
    static thread_local std::map<int, cudaStream_t> streams;
    auto it = streams.find(dev);
    if (it != streams.end()) return it->second;
    cudaStream_t s;
    RNLA_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    streams[dev] = s;
    return s;
}

RngKey key_of(const rnla_rng* r) {
    RngKey k;
    if (!r) {
        k.gen = GEN_PHILOX4X32;
        k.k0 = 0;
        k.k1 = 0;
        return k;
    }
    if (r->generator != GEN_PHILOX4X32 && r->generator != GEN_THREEFRY2X64)
        fail(RNLA_ERR_INVALID_PARAMETERS, "unknown generator");
    k.gen = r->generator;
    k.k0 = r->key0;
    k.k1 = r->key1;
    return k;
}

}  // namespace rnla

using namespace rnla;

extern "C" {

const char* rnla_last_error_message(void) { return t_last_error.c_str(); }

const char* rnla_version(void) { return "0.1.0 sm_103a"; }

uint64_t rnla_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int rnla_release_cached_memory(void) {
    RNLA_API_BEGIN
    std::lock_guard<std::mutex> g(g_pool_mu);
    for (auto& kv : g_pools) RNLA_CUDA(cudaMemPoolTrimTo(kv.second, 0));
    RNLA_API_END
}

int rnla_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void rnla_options_default(rnla_options* o) {
    if (!o) return;
    memset(o, 0, sizeof *o);
    o->precision = RNLA_PREC_FP64;
    o->mode = RNLA_MODE_REFERENCE;
    o->inner_solver = RNLA_SOLVER_CGLS;
    o->power_iters = 2;
    o->rng.generator = RNLA_GEN_PHILOX4X32;
    o->conlim = 1e8;
}

int rnla_rng_words_dev(const rnla_rng* rng, uint64_t first_word, int64_t n, uint32_t* out_dev,
                       void* stream) {
    RNLA_API_BEGIN
    if (n < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "n must be non-negative");
    Ctx ctx((cudaStream_t)stream);
    rng_words(ctx, key_of(rng), first_word, n, out_dev);
    RNLA_API_END
}

int rnla_rng_words(const rnla_rng* rng, uint64_t first_word, int64_t n, uint32_t* out) {
    RNLA_API_BEGIN
    if (n < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "n must be non-negative");
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<uint32_t> d(n, s);
    rng_words(ctx, key_of(rng), first_word, n, d);
    RNLA_CUDA(cudaMemcpyAsync(out, d.get(), n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

static void check_sketch_args(int32_t dist, int64_t rows, int64_t cols, int64_t ld) {
    if (rows < 0 || cols < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "negative dimension");
    if (rows == 0 || cols == 0)
        fail(RNLA_ERR_INVALID_DIMENSIONS, "Rows and columns must be greater than 0");
    if (dist < 0 || dist > 2) fail(RNLA_ERR_INVALID_PARAMETERS, "unknown distribution");
    if (ld < rows) fail(RNLA_ERR_INVALID_PARAMETERS, "ld < rows");
}

int rnla_sketching_operator_dev(int32_t dist, int64_t rows, int64_t cols, const rnla_rng* rng,
                                double* out_dev, int64_t ld, void* stream) {
    RNLA_API_BEGIN
    check_sketch_args(dist, rows, cols, ld);
    Ctx ctx((cudaStream_t)stream);
    sketch_fill_f64(ctx, dist, key_of(rng), rows, cols, out_dev, ld);
    RNLA_API_END
}

int rnla_sketching_operator_f32_dev(int32_t dist, int64_t rows, int64_t cols, const rnla_rng* rng,
                                    int32_t quantized, float* out_dev, int64_t ld, void* stream) {
    RNLA_API_BEGIN
    check_sketch_args(dist, rows, cols, ld);
    Ctx ctx((cudaStream_t)stream);
    sketch_fill_f32(ctx, dist, key_of(rng), rows, cols, quantized != 0, out_dev, ld);
    RNLA_API_END
}

int rnla_sketching_operator_ex(int32_t dist, int64_t rows, int64_t cols, const rnla_rng* rng,
                               double* out, int64_t ld) {
    RNLA_API_BEGIN
    check_sketch_args(dist, rows, cols, ld);
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<double> d((size_t)rows * cols, s);
    sketch_fill_f64(ctx, dist, key_of(rng), rows, cols, d, rows);
    d2h_matrix(out, ld, d, rows, rows, cols, s);
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

int rnla_sketching_operator(int32_t dist, int64_t rows, int64_t cols, double* out, int64_t ld) {
    return rnla_sketching_operator_ex(dist, rows, cols, nullptr, out, ld);
}

}  // extern "C"
