// Power-spectrum pass: x-axis FFT fused with the MAS window deconvolution,
// |delta_k|^2, the Legendre weights along the line of sight and the integer
// |k| shell binning.  Replaces the mode loop of class Pk,
// library/Pk_library/Pk_library.pyx:311-378.  The per-mode work is
// bin_mode() in pk_common.cuh.
//
// Input: the (n, n, h) half-complex grid already transformed along z and y.
// Lengths 2^k and 3*2^k take the register-resident kernel of fft_reg.cu; this file
// holds the generic (any n) kernel: a CTA owns one ky row and a block of B
// consecutive kz columns, loads the B pencils along x (runs of B*8
// contiguous bytes), transforms them in shared memory and bins every mode.
// The number of modes and the sum of |k| per bin do not depend on the data:
// they come from mode_counts(), once per (dims, axis).
#include "fft_core.cuh"
#include "pk_common.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;
constexpr size_t kLineBudget = 64 * 1024;

template <int WHAT>
__global__ void __launch_bounds__(kThreads)
k_pk_x(const float2 *__restrict__ data, int h, int axis, FftDesc D,
       const float2 *__restrict__ g_tw, const float *__restrict__ g_win, int B, int kmax,
       PkAcc acc) {
    extern __shared__ float2 sm[];
    const int n = D.n;
    const int ld = n + 1;
    const int middle = n / 2;
    float2 *tw = sm;
    float2 *b0 = tw + n;
    float2 *b1 = b0 + (size_t)B * ld;
    float *win = reinterpret_cast<float *>(b1 + (size_t)B * ld);
    BinHist H;
    H.setup(win + n, kmax, middle, WHAT);

    load_twiddles(tw, g_tw, n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) win[i] = g_win[i];
    H.zero_all();

    const int kz0 = blockIdx.x * B;
    const int nb = min(B, h - kz0);
    const int kyy = blockIdx.y;
    const long long base = (long long)kyy * h + kz0;
    const long long stride = (long long)n * h;
    for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) {
        const int i = idx / B, c = idx - i * B;
        if (c < nb) b0[c * ld + i] = __ldcs(data + base + i * stride + c);
    }
    __syncthreads();
    float2 *res = fft_smem<-1>(b0, b1, ld, nb, D, tw);

    const int ky = kyy > middle ? kyy - n : kyy;
    const float wy = win[kyy];
    for (int idx = threadIdx.x; idx < n * nb; idx += blockDim.x) {
        const int c = idx / n, kxx = idx - c * n;
        const int kz = kz0 + c;  // kzz in [0, middle]: kz = kzz
        bin_mode<WHAT>(H, acc, res[c * ld + kxx], kxx, ky, kz, n, axis, win[kxx], wy * win[kz],
                       middle);
    }
    __syncthreads();
    H.fold();
    __syncthreads();
    H.flush(acc, middle, WHAT);
}

// Integer mode counts of the independent half space of an n^3 grid.
__global__ void k_mode_counts(int n, int axis, int kmax_per,
                              unsigned long long *__restrict__ cnt_n,
                              unsigned long long *__restrict__ cnt1,
                              unsigned long long *__restrict__ cnt2) {
    const int middle = n / 2;
    const bool even = (n % 2) == 0;
    const long long total = (long long)n * n;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        const int kxx = (int)(p / n), kyy = (int)(p % n);
        const int kx = kxx > middle ? kxx - n : kxx;
        const int ky = kyy > middle ? kyy - n : kyy;
        for (int kz = 0; kz <= middle; ++kz) {
            if (kz == 0 || (kz == middle && even)) {
                if (kx < 0) continue;
                if (kx == 0 || (kx == middle && even)) {
                    if (ky < 0) continue;
                }
            }
            const int n2 = kx * kx + ky * ky + kz * kz;
            atomicAdd(&cnt_n[n2], 1ull);
            const int kpar = axis == 0 ? kx : (axis == 1 ? ky : kz);
            const int ap = abs(kpar);
            if (n2 <= middle * middle) atomicAdd(&cnt1[ap], 1ull);
            const int kper = isqrt_dev(n2 - kpar * kpar);
            atomicAdd(&cnt2[(long long)(middle + 1) * kper + ap], 1ull);
        }
    }
}

template <typename K>
int set_smem(pyl_ctx *ctx, K kernel, size_t bytes) {
    if (bytes > 40 * 1024)   // static shared memory counts toward the 48 KB default too
        PYL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
    return PYL_OK;
}

template <int WHAT>
int launch_pk(pyl_ctx *ctx, const float2 *data, int n, int h, int axis, const FftPlan *P,
              const float *win, int B, int kmax, const PkAcc &acc, size_t smem) {
    int st;
    if ((st = set_smem(ctx, k_pk_x<WHAT>, smem))) return st;
    dim3 grid((h + B - 1) / B, n);
    k_pk_x<WHAT><<<grid, kThreads, smem, ctx->stream>>>(data, h, axis, P->desc, P->d_tw, win, B,
                                                        kmax, acc);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

}  // namespace

int pk_bin_x(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, int mas, int what,
             const PkAcc &acc, int kmax, int kmax_per) {
    (void)kmax_per;
    int st = PYL_OK;
    const FftPlan *P = fft_plan(ctx, n, &st);
    if (!P) return st;
    const float *win = window_table(ctx, n, mas, &st);
    if (!win) return st;
    if (reg_supported(n)) return pow2_pk_x(ctx, data, n, rs, axis, P->d_tw, win, kmax, acc, what);
    const int h = n / 2 + 1;
    if (rs != h) return fail(ctx, PYL_ERR_UNSUPPORTED, "padded rows need 2^k");
    int B = 16;
    while (B > 1 && sizeof(float2) * (size_t)B * (n + 1) > kLineBudget) B >>= 1;
    while (B > 1 && B / 2 >= h) B >>= 1;
    const size_t smem = sizeof(float2) * ((size_t)n + 2 * (size_t)B * (n + 1)) +
                        sizeof(float) * (size_t)n + BinHist::bytes(kmax, n / 2, what);
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "FFT length too large");
    switch (what & PYL_PK_ALL) {
        case 0: return launch_pk<0>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
        case 1: return launch_pk<1>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
        case 2: return launch_pk<2>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
        case 3: return launch_pk<3>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
        case 4: return launch_pk<4>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
        case 5: return launch_pk<5>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
        case 6: return launch_pk<6>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
        default: return launch_pk<7>(ctx, data, n, h, axis, P, win, B, kmax, acc, smem);
    }
}

int mode_counts(pyl_ctx *ctx, int dims, int axis, unsigned long long *cnt_n,
                unsigned long long *cnt1, unsigned long long *cnt2, int kmax_per) {
    const long long total = (long long)dims * dims;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_mode_counts<<<blocks, 256, 0, ctx->stream>>>(dims, axis, kmax_per, cnt_n, cnt1, cnt2);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

}  // namespace pyl
