// Fast path (lengths 2^k and 3*2^k) of the 3D FFT passes and of the fused
// power-spectrum pass (the generic mixed-radix kernels in fft.cu / pk.cu
// handle every other length).  See fft_reg.cuh for the register-resident FFT.
//
//   rows r2c / c2r : a CTA transforms L row pairs (a + i b) of length N;
//                    loads and stores are contiguous runs along z.
//   columns c2c    : a CTA owns C consecutive columns (kz) of one outer
//                    index and transforms them along y or x; thread (c, t)
//                    loads x[t + s*P] of column c directly from global memory
//                    (C*8 contiguous bytes per element row) and stores its
//                    natural-order result the same way.
//   pk_x           : the x-column transform fused with the window, |delta|^2,
//                    Legendre weights and the integer-|k| binning, straight
//                    via a padded shared line; a CTA bins a few items into
//                    float32 shared histograms and adds them to the float64
//                    sums when it ends.
#include <vector>

#include "fft_reg.cuh"
#include "pk_common.cuh"

namespace pyl {

namespace {

template <int N>
struct RowsCfg {
    static constexpr int P = RegPlan<N>::P;
    static constexpr int L = P >= 256 ? 1 : 256 / P;   // row pairs per CTA
    static constexpr int THREADS = L * P;
};

template <int N>
struct ColsCfg {
    static constexpr int P = RegPlan<N>::P;
    static constexpr int C = P >= 512 ? 1 : (512 / P > 8 ? 8 : 512 / P);
    static constexpr int THREADS = C * P;
    // resident CTAs the fused Pk kernel is compiled for: E = 12 keeps two
    // register lines (the current item and the prefetched one) per thread
    static constexpr int PK_MINB =
        RegPlan<N>::E == 8 ? (THREADS >= 512 ? 2 : 4) : (THREADS >= 512 ? 1 : 2);
};

template <int N>
__global__ void __launch_bounds__(RowsCfg<N>::THREADS, 1)
k_rows_r2c_p2(const float *__restrict__ in, float2 *__restrict__ out, int64_t rows, int ostride,
              const float2 *__restrict__ g_tw, const float *__restrict__ shift) {
    using CF = RowsCfg<N>;
    constexpr int P = CF::P, LINE = RegPlan<N>::LINE16, H = N / 2 + 1;
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    const int l = threadIdx.x / P, t = threadIdx.x % P;
    float2 *line = sm + N + l * LINE;
    load_stage_twiddles<N>(tw, g_tw);
    const float sh = shift ? *shift : 0.f;
    const int64_t ra = 2 * ((int64_t)blockIdx.x * CF::L + l), rb = ra + 1;
    float2 v[RegPlan<N>::E];
#pragma unroll
    for (int s = 0; s < RegPlan<N>::E; ++s) {
        const float a = ra < rows ? __ldcs(in + ra * N + t + s * P) - sh : 0.f;
        const float b = rb < rows ? __ldcs(in + rb * N + t + s * P) - sh : 0.f;
        v[s] = make_float2(a, b);
    }
    __syncthreads();
    fft_line<N, -1, Pad16>(v, t, line, tw);
#pragma unroll
    for (int u = 0; u < RegPlan<N>::E; ++u) line[pad16(t + u * P)] = v[u];
    __syncthreads();
    for (int k = t; k < H; k += P) {
        const float2 Z = line[pad16(k)];
        const float2 Zm = line[pad16(k == 0 ? 0 : N - k)];
        if (ra < rows)
            out[ra * ostride + k] = make_float2(0.5f * (Z.x + Zm.x), 0.5f * (Z.y - Zm.y));
        if (rb < rows)
            out[rb * ostride + k] = make_float2(0.5f * (Z.y + Zm.y), -0.5f * (Z.x - Zm.x));
    }
}

template <int N>
__global__ void __launch_bounds__(RowsCfg<N>::THREADS, 1)
k_rows_c2r_p2(const float2 *__restrict__ in, float *__restrict__ out, int64_t rows, int istride,
              const float2 *__restrict__ g_tw, float scale) {
    using CF = RowsCfg<N>;
    constexpr int P = CF::P, LINE = RegPlan<N>::LINE16, H = N / 2 + 1;
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    const int l = threadIdx.x / P, t = threadIdx.x % P;
    float2 *line = sm + N + l * LINE;
    load_stage_twiddles<N>(tw, g_tw);
    const int64_t ra = 2 * ((int64_t)blockIdx.x * CF::L + l), rb = ra + 1;
    float2 v[RegPlan<N>::E];
#pragma unroll
    for (int s = 0; s < RegPlan<N>::E; ++s) {
        const int k = t + s * P;
        const bool lower = k < H;
        const int kk = lower ? k : N - k;
        float2 A = ra < rows ? in[ra * istride + kk] : make_float2(0.f, 0.f);
        float2 B = rb < rows ? in[rb * istride + kk] : make_float2(0.f, 0.f);
        if (kk == 0 || 2 * kk == N) { A.y = 0.f; B.y = 0.f; }
        if (!lower) { A.y = -A.y; B.y = -B.y; }
        v[s] = make_float2(A.x - B.y, A.y + B.x);
    }
    __syncthreads();
    fft_line<N, +1, Pad16>(v, t, line, tw);
#pragma unroll
    for (int u = 0; u < RegPlan<N>::E; ++u) {
        if (ra < rows) out[ra * N + t + u * P] = v[u].x * scale;
        if (rb < rows) out[rb * N + t + u * P] = v[u].y * scale;
    }
}

// In-place c2c along one axis.  Column (outer, kz0 + c): element e at
// data[outer * ostride + (kz0 + c) + e * estride]; columns >= ncol are idle.
template <int N, int DIR>
__global__ void __launch_bounds__(ColsCfg<N>::THREADS, 1)
k_cols_p2(float2 *__restrict__ data, int ncol, int64_t estride, int64_t ostride,
          const float2 *__restrict__ g_tw) {
    using CF = ColsCfg<N>;
    constexpr int P = CF::P, C = CF::C, LINE = RegPlan<N>::LINE8;
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    const int c = threadIdx.x % C, t = threadIdx.x / C;
    float2 *line = sm + N + c * LINE;
    load_stage_twiddles<N>(tw, g_tw);
    const int col = blockIdx.x * C + c;
    const bool valid = col < ncol;
    float2 *base = data + (int64_t)blockIdx.y * ostride + col;
    float2 v[RegPlan<N>::E];
#pragma unroll
    for (int s = 0; s < RegPlan<N>::E; ++s)
        v[s] = valid ? base[(int64_t)(t + s * P) * estride] : make_float2(0.f, 0.f);
    __syncthreads();
    fft_line<N, DIR>(v, t, line, tw);
    if (valid) {
#pragma unroll
        for (int u = 0; u < RegPlan<N>::E; ++u) base[(int64_t)(t + u * P) * estride] = v[u];
    }
}

// Fused x transform + binning.  A CTA bins `ipb` consecutive work items
// (kyy, kz block) into float32 shared histograms (a few hundred terms per bin
// at most) and adds them to the float64 sums when it ends.
template <int N, int WHAT>
__global__ void __launch_bounds__(ColsCfg<N>::THREADS, ColsCfg<N>::PK_MINB)
k_pk_x_p2(const float2 *__restrict__ data, int h, int rs, const float2 *__restrict__ g_tw,
          const float *__restrict__ g_win, int axis, int kmax, PkAcc acc, int nitems, int ipb) {
    using CF = ColsCfg<N>;
    constexpr int P = CF::P, C = CF::C, LINE = RegPlan<N>::LINE8;
    constexpr int MID = N / 2;
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    const int c = threadIdx.x % C, t = threadIdx.x / C;
    float2 *line = sm + N + c * LINE;
    float *win = reinterpret_cast<float *>(sm + N + C * LINE);
    FltHist H;
    H.setup(win + LINE, kmax, MID, WHAT);   // window padded like the lines
    load_stage_twiddles<N>(tw, g_tw);
    for (int i = threadIdx.x; i < N; i += blockDim.x) win[pad8(i)] = g_win[i];
    H.zero_all();
    __syncthreads();
    const int nzb = (h + C - 1) / C;
    const int it0 = blockIdx.x * ipb;
    const int it1 = min(nitems, it0 + ipb);
    // column c of item `item`, element s of thread t -> registers
    auto load = [&](int item, float2 (&v)[RegPlan<N>::E]) {
        const int kz = (item % nzb) * C + c;
        const bool valid = kz < h;
        const float2 *base = data + (int64_t)(item / nzb) * rs + kz;
        const int64_t es = (int64_t)N * rs;
#pragma unroll
        for (int s = 0; s < RegPlan<N>::E; ++s)
            v[s] = valid ? __ldcs(base + (int64_t)(t + s * P) * es) : make_float2(0.f, 0.f);
    };
    float2 v[RegPlan<N>::E];
    if (it0 < it1) load(it0, v);
    for (int it = it0; it < it1; ++it) {
        const int kyy = it / nzb;
        fft_line<N, -1>(v, t, line, tw);
        // natural order into the line, then each thread bins a run of E
        // consecutive kx of one column (neighbouring lanes -> different bins)
#pragma unroll
        for (int u = 0; u < RegPlan<N>::E; ++u) line[pad8(t + u * P)] = v[u];
        __syncthreads();
        // the next item's loads are in flight while this one is binned
        if (it + 1 < it1) load(it + 1, v);
        {
            const int cc = threadIdx.x / P, rr = threadIdx.x % P;
            const int kzc = (it % nzb) * C + cc;
            if (kzc < h) {
                const float2 *ln = sm + N + cc * LINE;
                const int ky = kyy > MID ? kyy - N : kyy;
                const float wyz = win[pad8(kyy)] * win[pad8(kzc)];
                constexpr int E = RegPlan<N>::E;
                bin_run<WHAT, E>(H, acc, ln, [](int i) { return pad8(i); }, E * rr, ky, kzc, N,
                                 axis, win, wyz, MID);
            }
        }
        __syncthreads();   // the shared lines are reused by the next item
    }
    H.flush(acc);
}

template <typename K>
int set_smem(pyl_ctx *ctx, K kernel, size_t bytes) {
    if (bytes > 40 * 1024)   // static shared memory counts toward the 48 KB default too
        PYL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
    return PYL_OK;
}

template <int N>
int rows_r2c_n(pyl_ctx *ctx, const float *in, float2 *out, int64_t rows, int ostride,
               const float2 *tw, const float *shift) {
    using CF = RowsCfg<N>;
    const size_t smem = sizeof(float2) * (N + (size_t)CF::L * RegPlan<N>::LINE16);
    int st;
    if ((st = set_smem(ctx, k_rows_r2c_p2<N>, smem))) return st;
    const int64_t pairs = (rows + 1) / 2;
    const int64_t grid = (pairs + CF::L - 1) / CF::L;
    k_rows_r2c_p2<N><<<(unsigned)grid, CF::THREADS, smem, ctx->stream>>>(in, out, rows, ostride, tw,
                                                                       shift);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

template <int N>
int rows_c2r_n(pyl_ctx *ctx, const float2 *in, float *out, int64_t rows, int istride,
               const float2 *tw, float scale) {
    using CF = RowsCfg<N>;
    const size_t smem = sizeof(float2) * (N + (size_t)CF::L * RegPlan<N>::LINE16);
    int st;
    if ((st = set_smem(ctx, k_rows_c2r_p2<N>, smem))) return st;
    const int64_t pairs = (rows + 1) / 2;
    const int64_t grid = (pairs + CF::L - 1) / CF::L;
    k_rows_c2r_p2<N><<<(unsigned)grid, CF::THREADS, smem, ctx->stream>>>(in, out, rows, istride,
                                                                       tw, scale);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

template <int N>
int cols_n(pyl_ctx *ctx, float2 *data, int ncol, int64_t estride, int64_t ostride, int nouter,
           int dir, const float2 *tw) {
    using CF = ColsCfg<N>;
    const size_t smem = sizeof(float2) * (N + (size_t)CF::C * RegPlan<N>::LINE8);
    int st;
    dim3 grid((ncol + CF::C - 1) / CF::C, nouter);
    if (dir < 0) {
        if ((st = set_smem(ctx, k_cols_p2<N, -1>, smem))) return st;
        k_cols_p2<N, -1><<<grid, CF::THREADS, smem, ctx->stream>>>(data, ncol, estride, ostride, tw);
    } else {
        if ((st = set_smem(ctx, k_cols_p2<N, +1>, smem))) return st;
        k_cols_p2<N, +1><<<grid, CF::THREADS, smem, ctx->stream>>>(data, ncol, estride, ostride, tw);
    }
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

template <int N, int WHAT>
int pk_n(pyl_ctx *ctx, const float2 *data, int h, int rs, int axis, const float2 *tw,
         const float *win, int kmax, const PkAcc &acc) {
    using CF = ColsCfg<N>;
    const size_t smem = sizeof(float2) * (N + (size_t)CF::C * RegPlan<N>::LINE8) +
                        sizeof(float) * RegPlan<N>::LINE8 + FltHist::bytes(kmax, N / 2, WHAT);
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "Pk histogram too large");
    int st;
    if ((st = set_smem(ctx, k_pk_x_p2<N, WHAT>, smem))) return st;
    // items per CTA: enough CTAs to fill the GPU several times over, few
    // enough that the per-CTA float64 flush stays small
    const int nitems = N * ((h + CF::C - 1) / CF::C);
    int ipb = nitems / (152 * 16);
    if (ipb < 1) ipb = 1;
    if (ipb > 8) ipb = 8;
    const int grid = (nitems + ipb - 1) / ipb;
    k_pk_x_p2<N, WHAT><<<grid, CF::THREADS, smem, ctx->stream>>>(data, h, rs, tw, win, axis, kmax,
                                                                 acc, nitems, ipb);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

template <int N>
int pk_what(pyl_ctx *ctx, const float2 *data, int h, int rs, int axis, const float2 *tw,
            const float *win, int kmax, const PkAcc &acc, int what) {
    switch (what & PYL_PK_ALL) {
        case 0: return pk_n<N, 0>(ctx, data, h, rs, axis, tw, win, kmax, acc);
        case 1: return pk_n<N, 1>(ctx, data, h, rs, axis, tw, win, kmax, acc);
        case 2: return pk_n<N, 2>(ctx, data, h, rs, axis, tw, win, kmax, acc);
        case 3: return pk_n<N, 3>(ctx, data, h, rs, axis, tw, win, kmax, acc);
        case 4: return pk_n<N, 4>(ctx, data, h, rs, axis, tw, win, kmax, acc);
        case 5: return pk_n<N, 5>(ctx, data, h, rs, axis, tw, win, kmax, acc);
        case 6: return pk_n<N, 6>(ctx, data, h, rs, axis, tw, win, kmax, acc);
        default: return pk_n<N, 7>(ctx, data, h, rs, axis, tw, win, kmax, acc);
    }
}

}  // namespace

bool reg_supported(int n) {
    switch (n) {
        case 16: case 32: case 64: case 128: case 256: case 512: case 1024: case 2048:
        case 4096: case 48: case 96: case 192: case 384: case 768: case 1536: case 3072:
            return true;
        default:
            return false;
    }
}

#define PYL_POW2_DISPATCH(n, CALL)                 \
    switch (n) {                                   \
        case 16: return CALL(16);                  \
        case 32: return CALL(32);                  \
        case 64: return CALL(64);                  \
        case 128: return CALL(128);                \
        case 256: return CALL(256);                \
        case 512: return CALL(512);                \
        case 1024: return CALL(1024);              \
        case 2048: return CALL(2048);              \
        case 4096: return CALL(4096);              \
        case 48: return CALL(48);                  \
        case 96: return CALL(96);                  \
        case 192: return CALL(192);                \
        case 384: return CALL(384);                \
        case 768: return CALL(768);                \
        case 1536: return CALL(1536);              \
        case 3072: return CALL(3072);              \
        default: return PYL_ERR_UNSUPPORTED;       \
    }

// tw: a table from twiddles_host(n); the kernels read the stage tables
// appended after its first n entries.
int pow2_rows_r2c(pyl_ctx *ctx, const float *in, float2 *out, int64_t rows, int n, int ostride,
                  const float2 *tw, const float *shift) {
#define CALL(N) rows_r2c_n<N>(ctx, in, out, rows, ostride, tw + N, shift)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

int pow2_rows_c2r(pyl_ctx *ctx, const float2 *in, float *out, int64_t rows, int n, int istride,
                  const float2 *tw, float scale) {
#define CALL(N) rows_c2r_n<N>(ctx, in, out, rows, istride, tw + N, scale)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

int pow2_cols(pyl_ctx *ctx, float2 *data, int n, int ncol, int64_t estride, int64_t ostride,
              int nouter, int dir, const float2 *tw) {
#define CALL(N) cols_n<N>(ctx, data, ncol, estride, ostride, nouter, dir, tw + N)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

int pow2_pk_x(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
              const float *win, int kmax, const PkAcc &acc, int what) {
    const int h = n / 2 + 1;
#define CALL(N) pk_what<N>(ctx, data, h, rs, axis, tw + N, win, kmax, acc, what)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

template <int N>
int stage_sources_n(std::vector<int> &src) {
    src.resize(TwStages<N>::SIZE);
    for (int i = 0; i < TwStages<N>::SIZE; ++i) src[i] = stage_tw_src<N, 0>(i);
    return PYL_OK;
}

int reg_stage_twiddle_sources(int n, std::vector<int> &src) {
#define CALL(N) stage_sources_n<N>(src)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

}  // namespace pyl
