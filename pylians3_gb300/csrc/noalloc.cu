// pyl_pk_noalloc: the power spectrum of a grid that is already on the device,
// computed without allocating any device memory.
//
// Some callers cannot call cudaMalloc: a host application that has handed
// the whole device to its own pool allocator (any other allocation fails or
// breaks its accounting), a plugin host that forbids allocations outside its
// allocator, or a latency-critical loop in which cudaMalloc/cudaFree would
// synchronise the device.  This entry point serves them: it runs the same
// kernels as pyl_pk (z r2c, y c2c, fused x c2c + binning), but every
// intermediate -- the half-complex grid, the twiddle and window tables, the
// mode counts and the per-bin sums -- lives in one fixed array of device
// memory that is part of the library image itself.
//
// Limits and behaviour:
//  * The array is kNoAllocScratchBytes = 12 MiB, enough for power-of-two
//    grids with 16 <= dims <= 128; larger or other sizes are rejected with
//    PYL_ERR_UNSUPPORTED.  Every GPU that loads the library holds these
//    12 MiB until the process exits.
//  * The first call on a device resolves the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
//  * All calls share the one array and it keeps the last call's contents;
//    the sums are cleared at the start of every call.  The FFT twiddles and
//    the window of the last (dims, scheme) stay in the array: a call with the
//    same dims and scheme as the previous call on that device uploads
//    nothing.  Calls that overlap on the GPU (other streams, other host
//    threads) race on it: issue them one after another.
//  * The call allocates no device memory.  The context it runs on does: its
//    creation allocates a 16-byte device status word (and a stream, unless
//    the caller passes one), so create the context once, before the
//    allocation-free region.
//  * delta is a device pointer; the outputs are host arrays, as for pyl_pk.
#include <map>
#include <mutex>

#include "common.cuh"

static constexpr size_t kNoAllocScratchBytes = 12u << 20;
static constexpr int kNoAllocMaxDims = 128;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_mu;
std::map<int, unsigned char *> g_scratch_addr;             // device -> array address
std::map<int, std::pair<int, int>> g_tables_in_scratch;    // device -> (dims, mas) uploaded
std::map<std::pair<int, int>, pyl::ModeTables> g_tables;  // (dims, axis) -> host tables

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Device address of the scratch array on the current device (set-up on the
// first call per device).
int scratch_address(pyl_ctx *ctx, unsigned char **out) {
    int dev = 0;
    PYL_CUDA(ctx, cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_scratch_addr.find(dev);
    if (it != g_scratch_addr.end()) {
        *out = it->second;
        return PYL_OK;
    }
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return pyl::cuda_fail(ctx, e, "cudaGetSymbolAddress(scratch)");
    g_scratch_addr[dev] = (unsigned char *)p;
    *out = (unsigned char *)p;
    return PYL_OK;
}

}  // namespace

using namespace pyl;

extern "C" int pyl_pk_noalloc(pyl_ctx *ctx, const float *delta, int dims, double BoxSize,
                              int axis, int mas, int what, pyl_pk_out *out) {
    if (!ctx) return PYL_ERR_ARG;
    if (!delta || !out) return fail(ctx, PYL_ERR_ARG, "pyl_pk_noalloc: null delta or out");
    if (dims < 16 || dims > kNoAllocMaxDims || (dims & (dims - 1)) != 0)
        return fail(ctx, PYL_ERR_UNSUPPORTED,
                    "pyl_pk_noalloc: dims must be a power of two in [16, 128] (the fixed "
                    "12 MiB scratch); use pyl_pk for other grids");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned char *base = nullptr;
    int st = scratch_address(ctx, &base);
    if (st) return st;

    const int ax = (axis == 0 || axis == 1) ? axis : 2;
    const int h = dims / 2 + 1;
    const int rs = half_stride(dims);
    ModeTables T;
    size_t nn, n1, n2;
    mode_table_init(T, dims, ax, nn, n1, n2);
    const AccLayout L = acc_layout(T);

    std::vector<float2> htw;
    std::vector<float> hwin;
    twiddles_host(dims, htw);   // its size also fixes the scratch layout
    window_host(dims, mas, hwin);

    // carve the scratch array
    size_t off = 0;
    float2 *tw = (float2 *)(base + off);
    off = align256(off + sizeof(float2) * htw.size());
    float *win = (float *)(base + off);
    off = align256(off + sizeof(float) * dims);
    unsigned long long *counts = (unsigned long long *)(base + off);
    off = align256(off + sizeof(unsigned long long) * (nn + n1 + n2));
    void *acc = base + off;
    off = align256(off + L.bytes());
    float2 *half = (float2 *)(base + off);
    off = align256(off + sizeof(float2) * (size_t)dims * dims * rs);
    if (off > kNoAllocScratchBytes)
        return fail(ctx, PYL_ERR_UNSUPPORTED, "pyl_pk_noalloc: grid does not fit the scratch");

    // The tables depend on (dims, mas) only and sit at offsets that depend
    // on dims only: skip the upload when the previous call on this device
    // left the same ones (calls are issued one after another).
    const int key_mas = (mas >= 1 && mas <= 4) ? mas : 0;
    bool tables_current = false;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_tables_in_scratch.find(ctx->device);
        tables_current = it != g_tables_in_scratch.end() &&
                         it->second == std::make_pair(dims, key_mas);
        g_tables_in_scratch.erase(ctx->device);   // re-set once the upload is issued
    }
    if (!tables_current) {
        PYL_CUDA(ctx, cudaMemcpyAsync(tw, htw.data(), sizeof(float2) * htw.size(),
                                      cudaMemcpyHostToDevice, ctx->stream));
        PYL_CUDA(ctx, cudaMemcpyAsync(win, hwin.data(), sizeof(float) * dims,
                                      cudaMemcpyHostToDevice, ctx->stream));
    }
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_tables_in_scratch[ctx->device] = std::make_pair(dims, key_mas);
    }

    // mode tables: counted once per (dims, axis) on the device, kept on the host
    bool have = false;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_tables.find(std::make_pair(dims, ax));
        if (it != g_tables.end()) {
            T = it->second;
            have = true;
        }
    }
    if (!have) {
        const size_t cb = sizeof(unsigned long long) * (nn + n1 + n2);
        PYL_CUDA(ctx, cudaMemsetAsync(counts, 0, cb, ctx->stream));
        if ((st = mode_counts(ctx, dims, ax, counts, counts + nn, counts + nn + n1, T.kmax_per)))
            return st;
        std::vector<unsigned long long> hc(nn + n1 + n2);
        PYL_CUDA(ctx, cudaMemcpyAsync(hc.data(), counts, cb, cudaMemcpyDeviceToHost, ctx->stream));
        PYL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        mode_table_fill(T, hc.data(), nn, n1, n2);
        std::lock_guard<std::mutex> lock(g_mu);
        g_tables[std::make_pair(dims, ax)] = T;
    }

    PYL_CUDA(ctx, cudaMemsetAsync(acc, 0, L.bytes(), ctx->stream));
    const PkAcc A = acc_view(acc, L);
    if ((st = pow2_rows_r2c(ctx, delta, half, (int64_t)dims * dims, dims, rs, tw, nullptr)))
        return st;
    if ((st = pow2_cols(ctx, half, dims, h, rs, (int64_t)dims * rs, dims, -1, tw))) return st;
    if ((st = pow2_pk_x(ctx, half, dims, rs, ax, tw, win, T.kmax, A, what))) return st;
    std::vector<double> raw;
    float2 dc;
    double mass;
    if ((st = download_raw(ctx, acc, L, raw, &dc, &mass))) return st;
    return finalize(ctx, T, raw, L, BoxSize, what, 1.0, false, out);
}
