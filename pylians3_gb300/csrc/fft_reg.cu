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
//                    Legendre weights and the integer-|k| binning
//                    (fft_reg_pk.cuh, instantiated in fft_reg_pk0..3.cu).
#include <vector>

#include "fft_reg_cfg.cuh"

namespace pyl {

namespace {

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
    const int w = what & PYL_PK_ALL;
    if (w == 0) return pk_x_what0(ctx, data, n, rs, axis, tw, win, kmax, acc);
    if (w <= 3) return pk_x_what13(ctx, data, n, rs, axis, tw, win, kmax, acc, w);
    if (w <= 5) return pk_x_what45(ctx, data, n, rs, axis, tw, win, kmax, acc, w);
    return pk_x_what67(ctx, data, n, rs, axis, tw, win, kmax, acc, w);
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
