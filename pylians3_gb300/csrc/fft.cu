// Stockham FFT passes of the 3D r2c / c2r transforms (replacing FFTW's
// FFT3Dr_f / IFFT3Dr_f, library/Pk_library/Pk_library.pyx:117-130, 149-162).
//
// Layout in HBM: real grid (n, n, n) row-major (z fastest); half-complex
// grid (n, n, h), h = n/2 + 1, interleaved complex64 -- FFTW's r2c layout.
//   pass z : rows r2c.  Two real rows a, b form one complex line a + i b; one
//            complex FFT gives both half spectra (A = (Z + conj Z-)/2,
//            B = (Z - conj Z-)/2i), for any n.
//   pass y, x : batched strided c2c.  A CTA owns one outer index and a block
//            of B consecutive kz columns, so every global access is a run of
//            B*8 contiguous bytes; the lines are transposed into shared
//            memory (padded stride n+1) and transformed there.
#include "fft_core.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;
constexpr size_t kLineBudget = 64 * 1024;  // bytes of one line buffer per CTA

template <int DIR>
__global__ void __launch_bounds__(kThreads)
k_rows_r2c(const float *__restrict__ in, float2 *__restrict__ out, int64_t rows,
           FftDesc D, const float2 *__restrict__ g_tw, int pairs,
           const float *__restrict__ shift) {
    extern __shared__ float2 sm[];
    const int n = D.n;
    const int h = n / 2 + 1;
    float2 *tw = sm;
    float2 *b0 = tw + n;
    float2 *b1 = b0 + (size_t)pairs * n;
    load_twiddles(tw, g_tw, n);
    const float sh = shift ? *shift : 0.f;
    const long long row0 = (long long)blockIdx.x * pairs * 2;
    for (int idx = threadIdx.x; idx < pairs * n; idx += blockDim.x) {
        const int p = idx / n, i = idx - p * n;
        const long long ra = row0 + 2 * p, rb = ra + 1;
        const float a = ra < rows ? __ldcs(in + ra * n + i) - sh : 0.f;
        const float b = rb < rows ? __ldcs(in + rb * n + i) - sh : 0.f;
        b0[idx] = make_float2(a, b);
    }
    __syncthreads();
    float2 *res = fft_smem<DIR>(b0, b1, n, pairs, D, tw);
    for (int idx = threadIdx.x; idx < pairs * h; idx += blockDim.x) {
        const int p = idx / h, k = idx - p * h;
        const long long ra = row0 + 2 * p, rb = ra + 1;
        const float2 Z = res[p * n + k];
        const float2 Zm = res[p * n + (k == 0 ? 0 : n - k)];
        if (ra < rows)
            out[ra * h + k] = make_float2(0.5f * (Z.x + Zm.x), 0.5f * (Z.y - Zm.y));
        if (rb < rows)
            out[rb * h + k] = make_float2(0.5f * (Z.y + Zm.y), -0.5f * (Z.x - Zm.x));
    }
}

__global__ void __launch_bounds__(kThreads)
k_rows_c2r(const float2 *__restrict__ in, float *__restrict__ out, int64_t rows,
           FftDesc D, const float2 *__restrict__ g_tw, int pairs, float scale) {
    extern __shared__ float2 sm[];
    const int n = D.n;
    const int h = n / 2 + 1;
    float2 *tw = sm;
    float2 *b0 = tw + n;
    float2 *b1 = b0 + (size_t)pairs * n;
    load_twiddles(tw, g_tw, n);
    const long long row0 = (long long)blockIdx.x * pairs * 2;
    for (int idx = threadIdx.x; idx < pairs * n; idx += blockDim.x) {
        const int p = idx / n, k = idx - p * n;
        const long long ra = row0 + 2 * p, rb = ra + 1;
        const bool lower = k < h;
        const int kk = lower ? k : n - k;
        float2 A = ra < rows ? in[ra * h + kk] : make_float2(0.f, 0.f);
        float2 B = rb < rows ? in[rb * h + kk] : make_float2(0.f, 0.f);
        // the imaginary parts of the DC and Nyquist terms do not enter a c2r
        if (kk == 0 || (2 * kk == n)) { A.y = 0.f; B.y = 0.f; }
        if (!lower) { A.y = -A.y; B.y = -B.y; }
        b0[idx] = make_float2(A.x - B.y, A.y + B.x);  // A + iB
    }
    __syncthreads();
    float2 *res = fft_smem<+1>(b0, b1, n, pairs, D, tw);
    for (int idx = threadIdx.x; idx < pairs * n; idx += blockDim.x) {
        const int p = idx / n, i = idx - p * n;
        const long long ra = row0 + 2 * p, rb = ra + 1;
        const float2 z = res[idx];
        if (ra < rows) out[ra * n + i] = z.x * scale;
        if (rb < rows) out[rb * n + i] = z.y * scale;
    }
}

template <int DIR>
__global__ void __launch_bounds__(kThreads)
k_axis_c2c(float2 *__restrict__ data, int h, int axis, FftDesc D,
           const float2 *__restrict__ g_tw, int B) {
    extern __shared__ float2 sm[];
    const int n = D.n;
    const int ld = n + 1;
    float2 *tw = sm;
    float2 *b0 = tw + n;
    float2 *b1 = b0 + (size_t)B * ld;
    load_twiddles(tw, g_tw, n);
    const int kz0 = blockIdx.x * B;
    const int nb = min(B, h - kz0);
    const long long outer = blockIdx.y;
    long long base, stride;
    if (axis == 1) { base = outer * n * (long long)h + kz0; stride = h; }
    else           { base = outer * h + kz0;               stride = (long long)n * h; }
    for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) {
        const int i = idx / B, c = idx - i * B;
        if (c < nb) b0[c * ld + i] = data[base + i * stride + c];
    }
    __syncthreads();
    float2 *res = fft_smem<DIR>(b0, b1, ld, nb, D, tw);
    for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) {
        const int i = idx / B, c = idx - i * B;
        if (c < nb) data[base + i * stride + c] = res[c * ld + i];
    }
}

template <typename K>
int set_smem(pyl_ctx *ctx, K kernel, size_t bytes) {
    if (bytes > 40 * 1024)   // static shared memory counts toward the 48 KB default too
        PYL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
    return PYL_OK;
}

}  // namespace

int fft_rows_r2c(pyl_ctx *ctx, const float *in, float2 *out, int64_t rows, int n,
                 int ostride, const float *shift) {
    int st = PYL_OK;
    const FftPlan *P = fft_plan(ctx, n, &st);
    if (!P) return st;
    if (reg_supported(n)) return pow2_rows_r2c(ctx, in, out, rows, n, ostride, P->d_tw, shift);
    if (ostride != n / 2 + 1) return fail(ctx, PYL_ERR_UNSUPPORTED, "padded rows need 2^k");
    int pairs = (int)(kLineBudget / (sizeof(float2) * (size_t)n));
    if (pairs < 1) pairs = 1;
    const int64_t npairs = (rows + 1) / 2;
    if (pairs > npairs) pairs = (int)npairs;
    const size_t smem = sizeof(float2) * ((size_t)n + 2 * (size_t)pairs * n);
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "FFT length too large");
    if ((st = set_smem(ctx, k_rows_r2c<-1>, smem))) return st;
    const int64_t grid = (npairs + pairs - 1) / pairs;
    k_rows_r2c<-1><<<(unsigned)grid, kThreads, smem, ctx->stream>>>(in, out, rows, P->desc,
                                                                  P->d_tw, pairs, shift);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

int fft_rows_c2r(pyl_ctx *ctx, const float2 *in, float *out, int64_t rows, int n,
                 int istride, float scale) {
    int st = PYL_OK;
    const FftPlan *P = fft_plan(ctx, n, &st);
    if (!P) return st;
    if (reg_supported(n)) return pow2_rows_c2r(ctx, in, out, rows, n, istride, P->d_tw, scale);
    if (istride != n / 2 + 1) return fail(ctx, PYL_ERR_UNSUPPORTED, "padded rows need 2^k");
    int pairs = (int)(kLineBudget / (sizeof(float2) * (size_t)n));
    if (pairs < 1) pairs = 1;
    const int64_t npairs = (rows + 1) / 2;
    if (pairs > npairs) pairs = (int)npairs;
    const size_t smem = sizeof(float2) * ((size_t)n + 2 * (size_t)pairs * n);
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "FFT length too large");
    if ((st = set_smem(ctx, k_rows_c2r, smem))) return st;
    const int64_t grid = (npairs + pairs - 1) / pairs;
    k_rows_c2r<<<(unsigned)grid, kThreads, smem, ctx->stream>>>(in, out, rows, P->desc,
                                                              P->d_tw, pairs, scale);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

int fft_plane_c2c(pyl_ctx *ctx, float2 *data, int n, int h, int rs, int dir) {
    int st = PYL_OK;
    const FftPlan *P = fft_plan(ctx, n, &st);
    if (!P) return st;
    if (reg_supported(n)) return pow2_cols(ctx, data, n, h, rs, 0, 1, dir, P->d_tw);
    if (rs != h) return fail(ctx, PYL_ERR_UNSUPPORTED, "padded rows need 2^k or 3*2^k");
    int B = 16;
    while (B > 1 && sizeof(float2) * (size_t)B * (n + 1) > kLineBudget) B >>= 1;
    while (B > 1 && B / 2 >= h) B >>= 1;
    const size_t smem = sizeof(float2) * ((size_t)n + 2 * (size_t)B * (n + 1));
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "FFT length too large");
    // one outer index: axis 1 of a (1, n, h) array is axis 0 of the plane
    dim3 grid((h + B - 1) / B, 1);
    if (dir < 0) {
        if ((st = set_smem(ctx, k_axis_c2c<-1>, smem))) return st;
        k_axis_c2c<-1><<<grid, kThreads, smem, ctx->stream>>>(data, h, 1, P->desc, P->d_tw, B);
    } else {
        if ((st = set_smem(ctx, k_axis_c2c<+1>, smem))) return st;
        k_axis_c2c<+1><<<grid, kThreads, smem, ctx->stream>>>(data, h, 1, P->desc, P->d_tw, B);
    }
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

int fft_axis_c2c(pyl_ctx *ctx, float2 *data, int n, int h, int rs, int axis, int dir) {
    int st = PYL_OK;
    const FftPlan *P = fft_plan(ctx, n, &st);
    if (!P) return st;
    if (reg_supported(n)) {
        const int64_t plane = (int64_t)n * rs;
        return axis == 1 ? pow2_cols(ctx, data, n, h, rs, plane, n, dir, P->d_tw)
                         : pow2_cols(ctx, data, n, h, plane, rs, n, dir, P->d_tw);
    }
    if (rs != h) return fail(ctx, PYL_ERR_UNSUPPORTED, "padded rows need 2^k");
    // largest power of two <= 16 whose B lines fit the line budget
    int B = 16;
    while (B > 1 && sizeof(float2) * (size_t)B * (n + 1) > kLineBudget) B >>= 1;
    while (B > 1 && B / 2 >= h) B >>= 1;
    const size_t smem = sizeof(float2) * ((size_t)n + 2 * (size_t)B * (n + 1));
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "FFT length too large");
    dim3 grid((h + B - 1) / B, n);
    if (dir < 0) {
        if ((st = set_smem(ctx, k_axis_c2c<-1>, smem))) return st;
        k_axis_c2c<-1><<<grid, kThreads, smem, ctx->stream>>>(data, h, axis, P->desc, P->d_tw, B);
    } else {
        if ((st = set_smem(ctx, k_axis_c2c<+1>, smem))) return st;
        k_axis_c2c<+1><<<grid, kThreads, smem, ctx->stream>>>(data, h, axis, P->desc, P->d_tw, B);
    }
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

}  // namespace pyl
