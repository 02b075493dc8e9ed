// C ABI of libpylgpu (include/pylgpu.h): context, plans, host/device staging
// and the finalisation of the spectra.  The kernels live in deposit.cu,
// fft.cu and pk.cu.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <mutex>
#include <thread>

#include "async_copy.cuh"
#include "common.cuh"

using pyl::FftPlan;
using pyl::ModeTables;

namespace pyl {

int fail(pyl_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_fail(pyl_ctx *ctx, cudaError_t e, const char *what) {
    char buf[512];
    snprintf(buf, sizeof buf, "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    if (ctx) ctx->err = buf;
    return e == cudaErrorMemoryAllocation ? PYL_ERR_OOM : PYL_ERR_CUDA;
}

int status_check(pyl_ctx *ctx) {
    unsigned s = 0;
    PYL_CUDA(ctx, cudaMemcpyAsync(&s, ctx->d_status, sizeof s, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    PYL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (s) {
        PYL_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof s, ctx->stream));
        if (s & kStatusInternal)
            return fail(ctx, PYL_ERR_UNSUPPORTED, "a sort kernel met a bound its launch excludes; "
                                               "the result was not computed");
        if (s & kStatusInputChanged)
            return fail(ctx, PYL_ERR_ARG,
                        "the positions changed while they were sorted (is another stream still "
                        "writing them? synchronise it first); the result was not computed");
        return fail(ctx, PYL_ERR_TIMEOUT, "a device-side wait gave up (copy not completed)");
    }
    return PYL_OK;
}

void *ws_get(pyl_ctx *ctx, const char *name, size_t bytes, int *status) {
    pyl_ctx::Buf &b = ctx->ws[name];
    if (b.bytes >= bytes && b.p) return b.p;
    if (ctx->capturing) {
        *status = fail(ctx, PYL_ERR_STATE, std::string("workspace ") + name +
                                               " would grow during graph capture");
        return nullptr;
    }
    const size_t old = b.p ? b.bytes : 0;
    if (b.p) {
        // the stream may still use the old buffer
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "workspace sync"); return nullptr; }
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t want = bytes < 256 ? 256 : bytes;
    // growing workspaces grow by at least 25 %, so that requests of slowly
    // increasing size do not reallocate (and synchronise) every time
    if (old && want < old + old / 4) want = old + old / 4;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        b.p = nullptr;
        *status = cuda_fail(ctx, e, name);
        return nullptr;
    }
    b.bytes = want;
    return b.p;
}

int zero_beside(pyl_ctx *ctx, void *p, size_t bytes) {
    if (!ctx->side) {
        PYL_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        PYL_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
        PYL_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    }
    PYL_CUDA(ctx, cudaEventRecord(ctx->ev_fork, ctx->stream));
    PYL_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    PYL_CUDA(ctx, cudaMemsetAsync(p, 0, bytes, ctx->side));
    PYL_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
    ctx->grid_pending = true;
    return PYL_OK;
}

int wait_grid(pyl_ctx *ctx) {
    if (!ctx->grid_pending) return PYL_OK;
    ctx->grid_pending = false;
    PYL_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    return PYL_OK;
}

void stage_mark(pyl_ctx *ctx, int stage, bool begin) {
    if (!ctx->timing) return;
    cudaEvent_t ev;
    if (ctx->event_pool.empty()) {
        if (cudaEventCreate(&ev) != cudaSuccess) return;
    } else {
        ev = ctx->event_pool.back();
        ctx->event_pool.pop_back();
    }
    cudaEventRecord(ev, ctx->stream);
    if (begin) {
        ctx->pending.push_back({stage, ev, nullptr});
    } else {
        for (auto it = ctx->pending.rbegin(); it != ctx->pending.rend(); ++it)
            if (it->stage == stage && it->b == nullptr) { it->b = ev; return; }
        ctx->event_pool.push_back(ev);
    }
}

int stage_flush(pyl_ctx *ctx) {
    for (auto &p : ctx->pending) {
        if (p.b) {
            PYL_CUDA(ctx, cudaEventSynchronize(p.b));
            float ms = 0.f;
            PYL_CUDA(ctx, cudaEventElapsedTime(&ms, p.a, p.b));
            ctx->stage_ms[p.stage] += ms;
            ctx->stage_n[p.stage] += 1;
            ctx->event_pool.push_back(p.b);
        }
        ctx->event_pool.push_back(p.a);
    }
    ctx->pending.clear();
    return PYL_OK;
}

// tw[m] = exp(-2 pi i m / n), evaluated in double and rounded to float, for
// m < n; for lengths with a register FFT, that FFT's stage tables follow
// (copies of entries of the first n).
void twiddles_host(int n, std::vector<float2> &tw) {
    tw.resize(n);
    for (int m = 0; m < n; ++m) {
        const double a = 2.0 * M_PI * (double)m / (double)n;
        tw[m] = make_float2((float)cos(a), (float)(-sin(a)));
    }
    std::vector<int> src;
    if (reg_supported(n) && reg_stage_twiddle_sources(n, src) == PYL_OK) {
        tw.resize(n + src.size());
        for (size_t i = 0; i < src.size(); ++i) tw[n + i] = tw[src[i]];
    }
}

// MAS_correction (Pk_library.pyx:83-84) per grid index: 1 if x == 0 else
// (x / sin x)^p, x = pi * k / dims with k the signed frequency of index i.
void window_host(int dims, int mas, std::vector<float> &w) {
    if (mas < 1 || mas > 4) mas = 0;
    const int middle = dims / 2;
    w.resize(dims);
    const double prefact = M_PI / dims;
    for (int i = 0; i < dims; ++i) {
        const int k = i > middle ? i - dims : i;
        const double x = prefact * k;
        w[i] = (float)((x == 0.0) ? 1.0 : pow(x / sin(x), mas));
    }
}

static void factorize(int n, FftDesc &D) {
    D.n = n;
    D.nst = 0;
    int m = n;
    while (m % 8 == 0 && D.nst < kMaxStages) { D.radix[D.nst++] = 8; m /= 8; }
    if (m % 4 == 0) { D.radix[D.nst++] = 4; m /= 4; }
    if (m % 2 == 0) { D.radix[D.nst++] = 2; m /= 2; }
    for (int p : {3, 5, 7}) {
        while (m % p == 0) { D.radix[D.nst++] = p; m /= p; }
    }
    for (int p = 11; m > 1 && p <= m; p += 2) {
        while (m % p == 0) { D.radix[D.nst++] = p; m /= p; }
    }
    if (m > 1) D.radix[D.nst++] = m;
}

// FFT plans and window tables are small read-only device tables that depend
// only on (device, size[, scheme]): one cache for the whole process, so that
// contexts serving requests side by side do not create (and synchronise on)
// their own copies.  They live until the process exits.
static std::mutex g_tables_mu;
static std::map<std::pair<int, int>, FftPlan> g_fft;                 // (device, n)
static std::map<std::tuple<int, int, int>, float *> g_win;           // (device, dims, mas)

const FftPlan *fft_plan(pyl_ctx *ctx, int n, int *status) {
    const auto key = std::make_pair(ctx->device, n);
    std::lock_guard<std::mutex> lock(g_tables_mu);
    auto it = g_fft.find(key);
    if (it != g_fft.end()) return &it->second;
    FftPlan P;
    factorize(n, P.desc);
    std::vector<float2> tw;
    twiddles_host(n, tw);
    cudaError_t e = cudaMalloc(&P.d_tw, sizeof(float2) * tw.size());
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "twiddle table"); return nullptr; }
    e = cudaMemcpy(P.d_tw, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "twiddle upload"); return nullptr; }
    return &(g_fft[key] = P);
}

// MAS_correction (Pk_library.pyx:83-84): 1 if x == 0 else (x / sin x)^p,
// x = pi * k / dims with k the signed frequency of index i.
const float *window_table(pyl_ctx *ctx, int dims, int mas, int *status) {
    if (mas < 1 || mas > 4) mas = 0;
    const auto key = std::make_tuple(ctx->device, dims, mas);
    std::lock_guard<std::mutex> lock(g_tables_mu);
    auto it = g_win.find(key);
    if (it != g_win.end()) return it->second;
    std::vector<float> w;
    window_host(dims, mas, w);
    float *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float) * dims);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "window table"); return nullptr; }
    e = cudaMemcpy(d, w.data(), sizeof(float) * dims, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "window upload"); return nullptr; }
    g_win[key] = d;
    return d;
}

static void sizes(int dims, int &kmax, int &kmax_par, int &kmax_per) {
    const long long middle = dims / 2;
    kmax_par = (int)middle;
    kmax_per = isqrt_host(2 * middle * middle);
    kmax = isqrt_host(3 * middle * middle);
}

void mode_table_init(ModeTables &T, int dims, int axis, size_t &nn, size_t &n1, size_t &n2) {
    T = ModeTables();
    T.dims = dims;
    T.axis = (axis != 0 && axis != 1) ? 2 : axis;
    sizes(dims, T.kmax, T.kmax_par, T.kmax_per);
    const long long middle = dims / 2;
    nn = (size_t)(3 * middle * middle + 1);
    n1 = (size_t)(middle + 1);
    n2 = (size_t)(middle + 1) * (T.kmax_per + 1);
}

// Per-bin tables from the integer counts (counts per k^2, 1D, 2D).
void mode_table_fill(ModeTables &T, const unsigned long long *h, size_t nn, size_t n1,
                     size_t n2) {
    T.N3D.assign(T.kmax + 1, 0.0);
    T.k3Dsum.assign(T.kmax + 1, 0.0);
    T.total = 0;
    for (size_t v = 0; v < nn; ++v) {
        if (!h[v]) continue;
        const int b = isqrt_host((long long)v);
        T.N3D[b] += (double)h[v];
        T.k3Dsum[b] += (double)h[v] * sqrt((double)v);
        T.total += (long long)h[v];
    }
    T.N1D.resize(n1);
    T.k1Dsum.resize(n1);
    for (size_t i = 0; i < n1; ++i) {
        T.N1D[i] = (double)h[nn + i];
        T.k1Dsum[i] = (double)h[nn + i] * (double)i;
    }
    T.N2D.resize(n2);
    for (size_t i = 0; i < n2; ++i) T.N2D[i] = (double)h[nn + n1 + i];
}

// Mode tables are host data that depend only on (dims, axis): one cache for
// the whole process, filled by whichever context needs a table first.  std::map
// nodes are stable, so the returned pointers stay valid.
static std::mutex g_modes_mu;
static std::map<std::pair<int, int>, ModeTables> g_modes;

const ModeTables *mode_tables(pyl_ctx *ctx, int dims, int axis, int *status) {
    if (axis != 0 && axis != 1) axis = 2;
    auto key = std::make_pair(dims, axis);
    {
        std::lock_guard<std::mutex> lock(g_modes_mu);
        auto it = g_modes.find(key);
        if (it != g_modes.end()) return &it->second;
    }
    ModeTables T;
    size_t nn, n1, n2;
    mode_table_init(T, dims, axis, nn, n1, n2);
    int st = PYL_OK;
    unsigned long long *d = (unsigned long long *)ws_get(
        ctx, "mode_counts", sizeof(unsigned long long) * (nn + n1 + n2), &st);
    if (!d) { *status = st; return nullptr; }
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned long long) * (nn + n1 + n2), ctx->stream);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "mode count memset"); return nullptr; }
    if ((st = mode_counts(ctx, dims, axis, d, d + nn, d + nn + n1, T.kmax_per))) {
        *status = st;
        return nullptr;
    }
    std::vector<unsigned long long> h(nn + n1 + n2);
    e = cudaMemcpyAsync(h.data(), d, sizeof(unsigned long long) * h.size(),
                        cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "mode count download"); return nullptr; }
    mode_table_fill(T, h.data(), nn, n1, n2);
    std::lock_guard<std::mutex> lock(g_modes_mu);
    auto ins = g_modes.emplace(key, std::move(T));   // a concurrent filler may have won
    return &ins.first->second;
}

}  // namespace pyl

using namespace pyl;

// ====================================================================== ABI
extern "C" {

int pyl_ctx_create(pyl_ctx **out, int device, void *stream) {
    if (!out) return PYL_ERR_ARG;
    *out = nullptr;
    pyl_ctx *ctx = new pyl_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete ctx; return PYL_ERR_CUDA; }
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete ctx; return PYL_ERR_CUDA; }
        ctx->own_stream = true;
    }
    e = cudaMalloc(&ctx->d_status, 16);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_status, 0, 16, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        if (ctx->d_status) cudaFree(ctx->d_status);
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return PYL_ERR_CUDA;
    }
    *out = ctx;
    return PYL_OK;
}

static void release_all(pyl_ctx *ctx) {
    for (pyl_ctx *c : ctx->lanes) release_all(c);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    cudaStreamSynchronize(ctx->stream);
    for (auto &kv : ctx->ws) if (kv.second.p) cudaFree(kv.second.p);
    ctx->ws.clear();
}

int pyl_ctx_destroy(pyl_ctx *ctx) {
    if (!ctx) return PYL_OK;
    cudaSetDevice(ctx->device);
    release_all(ctx);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->done) cudaEventDestroy(ctx->done);
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    for (auto &p : ctx->pending) {
        cudaEventDestroy(p.a);
        if (p.b) cudaEventDestroy(p.b);
    }
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
    if (ctx->batch_pinned) cudaFreeHost(ctx->batch_pinned);
    for (pyl_ctx *c : ctx->lanes) pyl_ctx_destroy(c);
    for (cudaEvent_t e : ctx->lane_join) cudaEventDestroy(e);
    if (ctx->lane_fork) cudaEventDestroy(ctx->lane_fork);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PYL_OK;
}

int pyl_ctx_set_stream(pyl_ctx *ctx, void *stream) {
    if (!ctx) return PYL_ERR_ARG;
    PYL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
        ctx->own_stream = false;
    } else {
        PYL_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return PYL_OK;
}

int pyl_ctx_get_stream(const pyl_ctx *ctx, void **stream) {
    if (!ctx || !stream) return PYL_ERR_ARG;
    *stream = (void *)ctx->stream;
    return PYL_OK;
}

int pyl_synchronize(pyl_ctx *ctx) {
    if (!ctx) return PYL_ERR_ARG;
    return pyl::status_check(ctx);
}

const char *pyl_last_error(const pyl_ctx *ctx) {
    return ctx ? ctx->err.c_str() : "no context";
}

int pyl_ctx_workspace_bytes(const pyl_ctx *ctx, size_t *bytes) {
    if (!ctx || !bytes) return PYL_ERR_ARG;
    size_t s = 0;
    for (auto &kv : ctx->ws) s += kv.second.bytes;
    for (const pyl_ctx *c : ctx->lanes)
        for (auto &kv : c->ws) s += kv.second.bytes;
    *bytes = s;
    return PYL_OK;
}

int pyl_ctx_trim(pyl_ctx *ctx) {
    if (!ctx) return PYL_ERR_ARG;
    cudaSetDevice(ctx->device);
    release_all(ctx);
    return PYL_OK;
}

int pyl_ctx_set_timing(pyl_ctx *ctx, int on) {
    if (!ctx) return PYL_ERR_ARG;
    int st = stage_flush(ctx);
    ctx->timing = on != 0;
    return st;
}

int pyl_ctx_stage_times(pyl_ctx *ctx, double *ms, int64_t *counts, int n, int reset) {
    if (!ctx) return PYL_ERR_ARG;
    int st = stage_flush(ctx);
    if (st) return st;
    for (int i = 0; i < n && i < ST_NSTAGES; ++i) {
        if (ms) ms[i] = ctx->stage_ms[i];
        if (counts) counts[i] = ctx->stage_n[i];
    }
    if (reset) {
        for (int i = 0; i < ST_NSTAGES; ++i) { ctx->stage_ms[i] = 0.0; ctx->stage_n[i] = 0; }
    }
    return ST_NSTAGES;
}

const char *pyl_stage_name(int stage) {
    static const char *names[ST_NSTAGES] = {"h2d", "zero", "deposit", "partition", "fft_z",
                                            "fft_y", "fft_x", "pk_x", "d2h", "tile_count",
                                            "mass"};
    return (stage >= 0 && stage < ST_NSTAGES) ? names[stage] : "";
}

int pyl_ctx_last_sort(const pyl_ctx *ctx, int *count_free, unsigned *spilled) {
    if (!ctx || !count_free || !spilled) return PYL_ERR_ARG;
    *count_free = ctx->last_sort_cap;
    *spilled = ctx->last_spilled;
    return PYL_OK;
}

int pyl_ctx_launch_count(const pyl_ctx *ctx, int64_t *count) {
    if (!ctx || !count) return PYL_ERR_ARG;
    *count = ctx->launches;
    return PYL_OK;
}

int pyl_host_alloc(void **ptr, size_t bytes) {
    if (!ptr) return PYL_ERR_ARG;
    cudaError_t e = cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocPortable);
    if (e != cudaSuccess) { *ptr = nullptr; return PYL_ERR_OOM; }
    return PYL_OK;
}

int pyl_host_free(void *ptr) {
    if (ptr) cudaFreeHost(ptr);
    return PYL_OK;
}

int pyl_pk_sizes(int dims, int *kmax, int *kmax_par, int *kmax_per) {
    if (dims < 2 || !kmax || !kmax_par || !kmax_per) return PYL_ERR_ARG;
    sizes(dims, *kmax, *kmax_par, *kmax_per);
    return PYL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------- MA
template <typename G>
static int ma_impl(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                   G *grid, int dims, float BoxSize, int mas, int renormalize_2D, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (coord != 2 && coord != 3)
        return fail(ctx, PYL_ERR_ARG, "pos must have 2 or 3 columns");
    if (dims < 1) return fail(ctx, PYL_ERR_ARG, "dims must be positive");
    if (mas < PYL_MAS_NGP || mas > PYL_MAS_PCS)
        return fail(ctx, PYL_ERR_ARG, "option not valid!!!");
    if (n < 0 || (n > 0 && !pos) || !grid) return fail(ctx, PYL_ERR_ARG, "null array");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t cells = (int64_t)dims * dims * (coord == 3 ? dims : 1);
    const bool dev = flags & PYL_DEVICE_PTRS;
    int st = PYL_OK;
    const float *dpos = pos, *dW = W;
    G *dgrid = grid;
    if (!dev) {
        if (n > 0) {
            float *p = (float *)ws_get(ctx, "ma_pos", sizeof(float) * (size_t)(n * coord), &st);
            if (!p) return st;
            PYL_CUDA(ctx, cudaMemcpyAsync(p, pos, sizeof(float) * (size_t)(n * coord),
                                          cudaMemcpyHostToDevice, ctx->stream));
            dpos = p;
        }
        if (W && n > 0) {
            float *w = (float *)ws_get(ctx, "ma_w", sizeof(float) * (size_t)n, &st);
            if (!w) return st;
            PYL_CUDA(ctx, cudaMemcpyAsync(w, W, sizeof(float) * (size_t)n,
                                          cudaMemcpyHostToDevice, ctx->stream));
            dW = w;
        }
        dgrid = (G *)ws_get(ctx, "ma_grid", sizeof(G) * (size_t)cells, &st);
        if (!dgrid) return st;
        PYL_CUDA(ctx, cudaMemcpyAsync(dgrid, grid, sizeof(G) * (size_t)cells,
                                      cudaMemcpyHostToDevice, ctx->stream));
    }
    if ((st = deposit_any(ctx, dpos, n, coord, dW, dgrid, dims, BoxSize, mas, flags))) return st;
    if (coord == 2 && renormalize_2D && mas != PYL_MAS_NGP) {
        // MA divides the whole 2D grid by 2, 3, 4 (MAS_library.pyx:88-110)
        if ((st = scale_any(ctx, dgrid, cells, (double)mas))) return st;
    }
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(grid, dgrid, sizeof(G) * (size_t)cells,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        if ((st = status_check(ctx))) return st;
    }
    return PYL_OK;
}

extern "C" {

int pyl_ma(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
           float *grid, int dims, float BoxSize, int mas, int renormalize_2D, int flags) {
    return ma_impl<float>(ctx, pos, n, coord, W, grid, dims, BoxSize, mas, renormalize_2D, flags);
}

int pyl_ma_f64(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
               double *grid, int dims, float BoxSize, int mas, int renormalize_2D, int flags) {
    return ma_impl<double>(ctx, pos, n, coord, W, grid, dims, BoxSize, mas, renormalize_2D,
                           flags);
}

// --------------------------------------------------------------------- FFT
int pyl_fft_r2c(pyl_ctx *ctx, const float *in, float *out, int dims, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (dims < 2 || !in || !out) return fail(ctx, PYL_ERR_ARG, "bad FFT arguments");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const int h = dims / 2 + 1;
    const size_t rb = sizeof(float) * (size_t)dims * dims * dims;
    const size_t cb = sizeof(float2) * (size_t)dims * dims * h;
    const bool dev = flags & PYL_DEVICE_PTRS;
    int st = PYL_OK;
    const float *din = in;
    float2 *dout = (float2 *)out;
    if (!dev) {
        float *p = (float *)ws_get(ctx, "fft_real", rb, &st);
        if (!p) return st;
        PYL_CUDA(ctx, cudaMemcpyAsync(p, in, rb, cudaMemcpyHostToDevice, ctx->stream));
        din = p;
        dout = (float2 *)ws_get(ctx, "fft_cplx", cb, &st);
        if (!dout) return st;
    }
    if ((st = fft_rows_r2c(ctx, din, dout, (long long)dims * dims, dims, h))) return st;
    if ((st = fft_axis_c2c(ctx, dout, dims, h, h, 1, -1))) return st;
    if ((st = fft_axis_c2c(ctx, dout, dims, h, h, 0, -1))) return st;
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(out, dout, cb, cudaMemcpyDeviceToHost, ctx->stream));
        PYL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return PYL_OK;
}

int pyl_fft_c2r(pyl_ctx *ctx, const float *in, float *out, int dims, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (dims < 2 || !in || !out) return fail(ctx, PYL_ERR_ARG, "bad FFT arguments");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const int h = dims / 2 + 1;
    const size_t rb = sizeof(float) * (size_t)dims * dims * dims;
    const size_t cb = sizeof(float2) * (size_t)dims * dims * h;
    const bool dev = flags & PYL_DEVICE_PTRS;
    int st = PYL_OK;
    // the input is not modified: transform a copy (as the reference copies
    // into its aligned buffer, Pk_library.pyx:162)
    float2 *work = (float2 *)ws_get(ctx, "fft_cplx", cb, &st);
    if (!work) return st;
    PYL_CUDA(ctx, cudaMemcpyAsync(work, in, cb,
                                  dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  ctx->stream));
    float *dout = out;
    if (!dev) {
        dout = (float *)ws_get(ctx, "fft_real", rb, &st);
        if (!dout) return st;
    }
    if ((st = fft_axis_c2c(ctx, work, dims, h, h, 0, +1))) return st;
    if ((st = fft_axis_c2c(ctx, work, dims, h, h, 1, +1))) return st;
    const double norm = 1.0 / ((double)dims * dims * dims);
    if ((st = fft_rows_c2r(ctx, work, dout, (long long)dims * dims, dims, h, (float)norm)))
        return st;
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(out, dout, rb, cudaMemcpyDeviceToHost, ctx->stream));
        PYL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return PYL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------- Pk
namespace pyl {

AccLayout acc_layout(const ModeTables &T) {
    AccLayout L;
    L.n3 = 3 * (size_t)(T.kmax + 1);
    L.n1 = (size_t)T.kmax_par + 1;
    L.nph = (size_t)T.kmax + 1;
    L.n2 = (size_t)(T.kmax_par + 1) * (T.kmax_per + 1);
    return L;
}

PkAcc acc_view(void *base, const AccLayout &L) {
    PkAcc a;
    double *d = (double *)base;
    a.P3 = d;
    a.P1 = a.P3 + L.n3;
    a.Pph = a.P1 + L.n1;
    a.P2D = a.Pph + L.nph;
    a.dc = (float2 *)(a.P2D + L.n2);
    a.mass = (double *)(a.dc + 1);
    a.shift = (float *)(a.mass + 1);
    return a;
}

// Particle info for the fused particles -> spectrum path: the grid holds
// the deposited density rho; the FFT input is rho - shift with shift the
// mass per cell, so the large k = 0 term does not enter the other modes'
// round-off.
struct MassInfo {
    const float *W;
    int64_t n;
};

// z-r2c and y-c2c of a device grid into the half-complex workspace, then the
// fused x pass; sums are left in acc (device).
int pk_device(pyl_ctx *ctx, const float *dgrid, int dims, int axis, int mas, int what,
              const ModeTables &T, void **acc_out, AccLayout &L,
              const MassInfo *mi = nullptr) {
    int st = PYL_OK;
    const int h = dims / 2 + 1;
    const int rs = half_stride(dims);   // padded rows: 64-byte aligned column blocks
    const size_t cb = sizeof(float2) * (size_t)dims * dims * rs;
    float2 *half = (float2 *)ws_get(ctx, "pk_half", cb, &st);
    if (!half) return st;
    L = acc_layout(T);
    void *acc = ws_get(ctx, "pk_acc", L.bytes(), &st);
    if (!acc) return st;
    PYL_CUDA(ctx, cudaMemsetAsync(acc, 0, L.bytes(), ctx->stream));
    const PkAcc A = acc_view(acc, L);
    if (mi) {
        StageScope s(ctx, ST_MASS);
        const double cells = (double)dims * dims * dims;
        if ((st = mass_and_shift(ctx, mi->W, mi->n, cells, A.mass, A.shift))) return st;
    }
    {
        StageScope s(ctx, ST_FFT_Z);
        if ((st = fft_rows_r2c(ctx, dgrid, half, (long long)dims * dims, dims, rs,
                               mi ? A.shift : nullptr)))
            return st;
    }
    {
        StageScope s(ctx, ST_FFT_Y);
        if ((st = fft_axis_c2c(ctx, half, dims, h, rs, 1, -1))) return st;
    }
    {
        StageScope s(ctx, ST_PK_X);
        if ((st = pk_bin_x(ctx, half, dims, rs, axis, mas, what, acc_view(acc, L), T.kmax,
                           T.kmax_per)))
            return st;
    }
    *acc_out = acc;
    return PYL_OK;
}

// Finalisation of class Pk (Pk_library.pyx:384-418) from the raw float64
// sums.  inv_mean2 rescales the data sums (1 for a delta input).
int finalize(pyl_ctx *ctx, const ModeTables &T, const std::vector<double> &raw,
             const AccLayout &L, double BoxSize, int what, double inv_mean2,
             bool zero_dc2d, pyl_pk_out *out) {
    const int dims = T.dims;
    const long long own = (dims % 2 == 1) ? 1 : 8;
    const long long d3 = (long long)dims * dims * dims;
    const long long expected = (d3 - own) / 2 + own;
    if (T.total != expected) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "WARNING: Not all modes counted: counted %lld independent modes, expected %lld",
                 T.total, expected);
        return fail(ctx, PYL_ERR_MODES, buf);
    }
    const double kF = 2.0 * M_PI / BoxSize;
    const double kN = (dims / 2) * kF;
    const double unit = pow(BoxSize / (double)((long long)dims * dims), 3);
    const double *P3 = raw.data();
    const double *P1 = P3 + L.n3;
    const double *Pph = P1 + L.n1;
    const double *P2 = Pph + L.nph;
    for (int b = 1; b <= T.kmax; ++b) {
        const double N = T.N3D[b];
        if (out->k3D) out->k3D[b - 1] = (T.k3Dsum[b] / N) * kF;
        if (out->Nmodes3D) out->Nmodes3D[b - 1] = N;
        if (out->Pk) {
            // the device sums the moments S0, S1, S2 of |delta|^2 in mu^2;
            // the Legendre sums (Pk_library.pyx:362-365) follow from them
            const double S0 = P3[3 * b + 0], S1 = P3[3 * b + 1], S2 = P3[3 * b + 2];
            const double L2 = (3.0 * S1 - S0) / 2.0;
            const double L4 = (35.0 * S2 - 30.0 * S1 + 3.0 * S0) / 8.0;
            out->Pk[3 * (b - 1) + 0] = (S0 * inv_mean2 / N) * unit;
            out->Pk[3 * (b - 1) + 1] = (L2 * inv_mean2 * 5.0 / N) * unit;
            out->Pk[3 * (b - 1) + 2] = (L4 * inv_mean2 * 9.0 / N) * unit;
        }
        if ((what & PYL_PK_PHASE) && out->Pkphase) out->Pkphase[b - 1] = (Pph[b] / N) * unit;
    }
    if (what & PYL_PK_1D) {
        for (int i = 1; i <= T.kmax_par; ++i) {
            const double N = T.N1D[i];
            double pk = P1[i] * inv_mean2 * unit;
            const double k1 = (T.k1Dsum[i] / N) * kF;
            const double kmaxper = sqrt(kN * kN - k1 * k1);
            pk = pk * (M_PI * kmaxper * kmaxper / N) / ((2.0 * M_PI) * (2.0 * M_PI));
            if (out->k1D) out->k1D[i - 1] = k1;
            if (out->Pk1D) out->Pk1D[i - 1] = pk;
            if (out->Nmodes1D) out->Nmodes1D[i - 1] = N;
        }
    }
    if (what & PYL_PK_2D) {
        const int np = T.kmax_par + 1, nq = T.kmax_per + 1;
        for (int q = 0; q < nq; ++q)
            for (int p = 0; p < np; ++p) {
                const size_t i = (size_t)np * q + p;
                if (out->kpar) out->kpar[i] = 0.5 * (p + p + 1) * kF;
                if (out->kper) out->kper[i] = 0.5 * (q + q + 1) * kF;
                double s = P2[i] * inv_mean2;
                if (zero_dc2d && i == 0) s = 0.0;
                if (out->Pk2D) out->Pk2D[i] = s * unit / T.N2D[i];
                if (out->Nmodes2D) out->Nmodes2D[i] = T.N2D[i];
            }
    }
    return PYL_OK;
}

int check_particles(pyl_ctx *ctx, const pyl_pk_request &r) {
    if (r.dims < 2 || r.n <= 0 || !r.pos) return fail(ctx, PYL_ERR_ARG, "bad arguments");
    if (r.mas_deposit < PYL_MAS_NGP || r.mas_deposit > PYL_MAS_PCS)
        return fail(ctx, PYL_ERR_ARG, "option not valid!!!");
    return PYL_OK;
}

// Issues one particles -> spectrum request on the context stream: upload
// (host inputs), zero, deposit, the FFT passes and the fused binning, then
// the raw sums, the k = 0 mode and the mass copied to `dst` (host, pinned).
// Particle sets uploaded from host memory share one host link: on a device,
// each upload (from any context) waits for the one issued before it, so that
// one runs at a time at the link's full rate while the other contexts'
// requests compute (several uploads at once only share the link and then
// leave it idle while their requests all compute together).  Not applied
// while a sequence is captured into a graph (the event lives outside it).
static std::mutex g_upload_mu;
static std::map<int, cudaEvent_t> g_upload_ev;   // device -> after its last upload

int issue_particles(pyl_ctx *ctx, const pyl_pk_request &r, const ModeTables &T, int flags,
                    void *dst) {
    int st = PYL_OK;
    const int64_t n = r.n;
    const int dims = r.dims;
    const float *dpos = r.pos, *dW = r.W;
    if (!(flags & PYL_DEVICE_PTRS)) {
        StageScope s(ctx, ST_H2D);
        float *p = (float *)ws_get(ctx, "ma_pos", sizeof(float) * (size_t)(3 * n), &st);
        if (!p) return st;
        float *w = nullptr;
        if (r.W) {
            w = (float *)ws_get(ctx, "ma_w", sizeof(float) * (size_t)n, &st);
            if (!w) return st;
        }
        std::unique_lock<std::mutex> lock(g_upload_mu, std::defer_lock);
        cudaEvent_t *chain = nullptr;
        if (!ctx->capturing) {
            lock.lock();
            chain = &g_upload_ev[ctx->device];
            if (*chain) PYL_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, *chain, 0));
            else PYL_CUDA(ctx, cudaEventCreateWithFlags(chain, cudaEventDisableTiming));
        }
        PYL_CUDA(ctx, cudaMemcpyAsync(p, r.pos, sizeof(float) * (size_t)(3 * n),
                                      cudaMemcpyHostToDevice, ctx->stream));
        dpos = p;
        if (w) {
            PYL_CUDA(ctx, cudaMemcpyAsync(w, r.W, sizeof(float) * (size_t)n,
                                          cudaMemcpyHostToDevice, ctx->stream));
            dW = w;
        }
        if (chain) PYL_CUDA(ctx, cudaEventRecord(*chain, ctx->stream));
    }
    const size_t rb = sizeof(float) * (size_t)dims * dims * dims;
    float *grid = (float *)ws_get(ctx, "pk_grid", rb, &st);
    if (!grid) return st;
    // the grid is zeroed beside the sort (which is bound by shared memory,
    // not DRAM); the deposit waits for it
    if ((st = zero_beside(ctx, grid, rb))) return st;
    st = deposit(ctx, dpos, n, 3, dW, grid, dims, r.BoxSize, r.mas_deposit, flags);
    const int st2 = wait_grid(ctx);
    if (st) return st;
    if (st2) return st2;
    void *acc = nullptr;
    AccLayout L;
    const MassInfo mi{dW, n};
    if ((st = pk_device(ctx, grid, dims, r.axis, r.mas_window, r.what, T, &acc, L, &mi)))
        return st;
    const size_t nb = L.sums() + sizeof(float2) + sizeof(double);
    StageScope s(ctx, ST_D2H);
    PYL_CUDA(ctx, cudaMemcpyAsync(dst, acc, nb, cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->sort_hint && ctx->sort_used.valid && ctx->d_sort_info)
        PYL_CUDA(ctx, cudaMemcpyAsync((char *)dst + nb, ctx->d_sort_info, 4 * sizeof(unsigned),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    return PYL_OK;
}

// What the finished request's sorted deposit showed (its info words, copied
// after the sums) decides the sort of the next request of its kind: after
// an exact sort, slots sized from the largest tile and bucket counts (with a
// margin) unless the input is clustered; after a count-free sort whose slots
// overflowed, the exact sort again.
size_t result_bytes(const AccLayout &L) {
    return L.sums() + sizeof(float2) + sizeof(double) + 4 * sizeof(unsigned);
}

static std::mutex g_plans_mu;
static std::map<std::tuple<int, int, int, int>, pyl_ctx::SortPlan> g_plans;

pyl_ctx::SortPlan *shared_sort_plan(int device, int dims, int mas, int weighted) {
    std::lock_guard<std::mutex> lock(g_plans_mu);
    return &g_plans[std::make_tuple(device, dims, mas, weighted)];
}

pyl_ctx::SortPlan read_sort_plan(const pyl_ctx::SortPlan *p) {
    std::lock_guard<std::mutex> lock(g_plans_mu);
    return *p;
}

void learn_sort(const pyl_ctx::SortUsed &u, const unsigned *info) {
    if (!u.valid || !u.plan) return;
    std::lock_guard<std::mutex> lock(g_plans_mu);
    pyl_ctx::SortPlan &p = *u.plan;
    if (u.cap) {
        if (info[3] != 0) p.cap = false;
        return;
    }
    const double mean_t = (double)u.n / u.ntiles;
    const double phiT = info[0] / mean_t, phiC = info[1] / (mean_t * u.F);
    p.phiT = (float)std::max(1.05, 1.1 * phiT);
    p.phiC = (float)std::max(1.03, 1.05 * phiC);
    p.mode = (int)info[2];
    p.cap = p.phiT <= 2.0f && p.phiC <= 2.0f && mean_t >= 64.0;
}

// Spectrum of a request from the raw sums, k = 0 mode and mass at `src`.
// The FFT saw rho - shift (shift = mass per cell rounded to float, as on the
// device); the grid mean is shift + DC / dims^3, and P(delta = rho/mean - 1)
// = P(rho) / mean^2 for every k != 0.
int finalize_particles(pyl_ctx *ctx, const ModeTables &T, const AccLayout &L, const void *src,
                       int dims, double BoxSize, int what, pyl_pk_out *out) {
    std::vector<double> raw(L.n3 + L.n1 + L.nph + L.n2 + 8);
    memcpy(raw.data(), src, L.sums());
    float2 dc;
    double mass;
    memcpy(&dc, (const char *)src + L.sums(), sizeof(float2));
    memcpy(&mass, (const char *)src + L.sums() + sizeof(float2), sizeof(double));
    const double cells = (double)dims * dims * dims;
    const double shift = (double)(float)(mass * (1.0 / cells));
    const double mean = shift + (double)dc.x / cells;
    if (!(mean > 0.0) && !(mean < 0.0))
        return fail(ctx, PYL_ERR_ARG, "grid mean is zero: cannot form the overdensity");
    return finalize(ctx, T, raw, L, BoxSize, what, 1.0 / (mean * mean), true, out);
}

// Sums, the raw k = 0 mode and the deposited mass back to the host.
int download_raw(pyl_ctx *ctx, void *acc, const AccLayout &L, std::vector<double> &raw,
                 float2 *dc, double *mass) {
    raw.resize(L.n3 + L.n1 + L.nph + L.n2 + 8);
    const size_t sums = sizeof(double) * (L.n3 + L.n1 + L.nph + L.n2);
    {
        StageScope s(ctx, ST_D2H);
        PYL_CUDA(ctx, cudaMemcpyAsync(raw.data(), acc, sums + sizeof(float2) + sizeof(double),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    }
    int st = status_check(ctx);
    if (st) return st;
    memcpy(dc, (const char *)raw.data() + sums, sizeof(float2));
    memcpy(mass, (const char *)raw.data() + sums + sizeof(float2), sizeof(double));
    return PYL_OK;
}

}  // namespace pyl

extern "C" {

int pyl_pk(pyl_ctx *ctx, const float *delta, int dims, double BoxSize, int axis, int mas,
           int what, pyl_pk_out *out, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (dims < 2 || !delta || !out) return fail(ctx, PYL_ERR_ARG, "bad Pk arguments");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = PYL_OK;
    const ModeTables *T = mode_tables(ctx, dims, axis, &st);
    if (!T) return st;
    const float *dgrid = delta;
    if (!(flags & PYL_DEVICE_PTRS)) {
        const size_t rb = sizeof(float) * (size_t)dims * dims * dims;
        float *p = (float *)ws_get(ctx, "pk_grid", rb, &st);
        if (!p) return st;
        PYL_CUDA(ctx, cudaMemcpyAsync(p, delta, rb, cudaMemcpyHostToDevice, ctx->stream));
        dgrid = p;
    }
    void *acc = nullptr;
    AccLayout L;
    if ((st = pk_device(ctx, dgrid, dims, axis, mas, what, *T, &acc, L))) return st;
    std::vector<double> raw;
    float2 dc;
    double mass;
    if ((st = download_raw(ctx, acc, L, raw, &dc, &mass))) return st;
    return finalize(ctx, *T, raw, L, BoxSize, what, 1.0, false, out);
}

int pyl_pk_particles(pyl_ctx *ctx, const float *pos, int64_t n, const float *W, int dims,
                     float BoxSize, int mas_deposit, int axis, int mas_window, int what,
                     pyl_pk_out *out, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (!out) return fail(ctx, PYL_ERR_ARG, "null output");
    const int st = pyl_pk_particles_enqueue(ctx, pos, n, W, dims, BoxSize, mas_deposit, axis,
                                            mas_window, what, flags);
    if (st) return st;
    return pyl_pk_collect(ctx, out, -1);
}

int pyl_pk_particles_enqueue(pyl_ctx *ctx, const float *pos, int64_t n, const float *W,
                             int dims, float BoxSize, int mas_deposit, int axis, int mas_window,
                             int what, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (ctx->req.active)
        return fail(ctx, PYL_ERR_STATE, "a request is already in flight on this context");
    pyl_pk_request r{pos, n, W, dims, BoxSize, mas_deposit, axis, mas_window, what};
    int st = check_particles(ctx, r);
    if (st) return st;
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const ModeTables *T = mode_tables(ctx, dims, axis, &st);
    if (!T) return st;
    const AccLayout L = acc_layout(*T);
    const size_t nb = L.sums() + sizeof(float2) + sizeof(double) + 4 * sizeof(unsigned);
    if (ctx->pinned_bytes < nb) {
        if (ctx->pinned) {
            PYL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFreeHost(ctx->pinned);
            ctx->pinned = nullptr;
            ctx->pinned_bytes = 0;
        }
        PYL_CUDA(ctx, cudaHostAlloc(&ctx->pinned, nb, cudaHostAllocPortable));
        ctx->pinned_bytes = nb;
    }
    if (!ctx->done) PYL_CUDA(ctx, cudaEventCreateWithFlags(&ctx->done, cudaEventDisableTiming));
    ctx->sort_hint = shared_sort_plan(ctx->device, dims, mas_deposit, W ? 1 : 0);
    st = issue_particles(ctx, r, *T, flags, ctx->pinned);
    ctx->sort_hint = nullptr;
    if (st) return st;
    PYL_CUDA(ctx, cudaEventRecord(ctx->done, ctx->stream));
    ctx->req.sort = ctx->sort_used;
    ctx->req.active = true;
    ctx->req.dims = dims;
    ctx->req.axis = axis;
    ctx->req.what = what;
    ctx->req.BoxSize = BoxSize;
    ctx->req.T = T;
    ctx->req.L = L;
    return PYL_OK;
}

int pyl_pk_query(pyl_ctx *ctx) {
    if (!ctx) return PYL_ERR_ARG;
    if (!ctx->req.active) return fail(ctx, PYL_ERR_STATE, "no request in flight");
    const cudaError_t e = cudaEventQuery(ctx->done);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return cuda_fail(ctx, e, "cudaEventQuery");
}

}  // extern "C"

namespace {
// Wait for the event with a bound; timeout_ms < 0 waits without one.
int wait_done(pyl_ctx *ctx, int timeout_ms) {
    if (timeout_ms < 0) {
        PYL_CUDA(ctx, cudaEventSynchronize(ctx->done));
        return PYL_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaEventQuery(ctx->done);
        if (e == cudaSuccess) return PYL_OK;
        if (e != cudaErrorNotReady) return cuda_fail(ctx, e, "cudaEventQuery");
        const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
                            std::chrono::steady_clock::now() - t0).count();
        if (ms >= timeout_ms) return fail(ctx, PYL_ERR_TIMEOUT, "request not finished in time");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}
}  // namespace

extern "C" {

int pyl_pk_collect(pyl_ctx *ctx, pyl_pk_out *out, int timeout_ms) {
    if (!ctx) return PYL_ERR_ARG;
    if (!out) return fail(ctx, PYL_ERR_ARG, "null output");
    if (!ctx->req.active) return fail(ctx, PYL_ERR_STATE, "no request in flight");
    int st = wait_done(ctx, timeout_ms);
    if (st) return st;   // a timeout leaves the request in flight
    ctx->req.active = false;
    if ((st = status_check(ctx))) return st;
    const pyl_ctx::Request &R = ctx->req;
    const unsigned *info = (const unsigned *)((const char *)ctx->pinned + R.L.sums() +
                                              sizeof(float2) + sizeof(double));
    learn_sort(R.sort, info);
    ctx->last_sort_cap = R.sort.valid ? (R.sort.cap ? 1 : 0) : -1;
    ctx->last_spilled = (R.sort.valid && R.sort.cap) ? info[3] : 0u;
    return finalize_particles(ctx, *R.T, R.L, ctx->pinned, R.dims, R.BoxSize, R.what, out);
}

}  // extern "C"
