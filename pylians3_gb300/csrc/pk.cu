// Power-spectrum pass: x-axis FFT fused with the MAS window deconvolution,
// |delta_k|^2, the Legendre weights along the line of sight and the integer
// |k| shell binning.  Replaces the mode loop of class Pk,
// library/Pk_library/Pk_library.pyx:311-378.
//
// Input: the (n, n, h) half-complex grid already transformed along z and y.
// A CTA owns one ky row and a block of B consecutive kz columns; it loads the
// B pencils along x (runs of B*8 contiguous bytes), transforms them in shared
// memory and never writes them back.  Per mode (kx, ky, kz):
//   Hermitian half space as the reference (:324-327): on the kz = 0 and
//   (even n) kz = n/2 planes skip kx < 0, and on their kx = 0 / kx = n/2
//   lines skip ky < 0;
//   n2 = kx^2 + ky^2 + kz^2 (integer), bin = floor(sqrt(n2)) exactly;
//   f = w[kx] w[ky] w[kz] (float window table), re = f Re, im = f Im,
//   d2 = re^2 + im^2, mu^2 = k_par^2 / n2;
//   P0 += d2, P2 += d2 (3 mu^2 - 1)/2, P4 += d2 (35 mu^4 - 30 mu^2 + 3)/8.
// Per-mode arithmetic is float32; each CTA accumulates its modes in a
// shared-memory float32 histogram and adds it to the float64 global sums
// (one double atomic per non-empty bin and quantity).  The number of modes
// and the sum of |k| per bin do not depend on the data: they come from
// mode_counts(), once per (dims, axis).
#include "fft_core.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;
constexpr size_t kLineBudget = 64 * 1024;

__device__ __forceinline__ int isqrt_dev(int v) {
    int r = (int)sqrtf((float)v);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

template <int WHAT>
__global__ void __launch_bounds__(kThreads)
k_pk_x(const float2 *__restrict__ data, int h, int axis, FftDesc D,
       const float2 *__restrict__ g_tw, const float *__restrict__ g_win, int B,
       int kmax, int kmax_per, PkAcc acc) {
    extern __shared__ float2 sm[];
    const int n = D.n;
    const int ld = n + 1;
    const int middle = n / 2;
    const bool even = (n % 2) == 0;
    float2 *tw = sm;
    float2 *b0 = tw + n;
    float2 *b1 = b0 + (size_t)B * ld;
    float *win = reinterpret_cast<float *>(b1 + (size_t)B * ld);
    float *hP = win + n;                    // 3*(kmax+1)
    float *h1 = hP + 3 * (kmax + 1);        // middle+1
    float *hph = h1 + (middle + 1);         // kmax+1
    const int nh = 3 * (kmax + 1) + (middle + 1) + (kmax + 1);

    load_twiddles(tw, g_tw, n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) win[i] = g_win[i];
    for (int i = threadIdx.x; i < nh; i += blockDim.x) hP[i] = 0.f;

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
        const int kx = kxx > middle ? kxx - n : kxx;
        if (kz == 0 || (kz == middle && even)) {
            if (kx < 0) continue;
            if (kx == 0 || (kx == middle && even)) {
                if (ky < 0) continue;
            }
        }
        const float2 v = res[c * ld + kxx];
        if (kx == 0 && ky == 0 && kz == 0) *acc.dc = v;
        const int n2 = kx * kx + ky * ky + kz * kz;
        const int bin = isqrt_dev(n2);
        const int kpar = axis == 0 ? kx : (axis == 1 ? ky : kz);
        const float f = win[kxx] * wy * win[kz];
        const float re = v.x * f, im = v.y * f;
        const float d2 = re * re + im * im;
        const float mu2 = n2 > 0 ? (float)(kpar * kpar) / (float)n2 : 0.f;
        atomicAdd(&hP[3 * bin + 0], d2);
        atomicAdd(&hP[3 * bin + 1], d2 * (3.f * mu2 - 1.f) * 0.5f);
        atomicAdd(&hP[3 * bin + 2], d2 * ((35.f * mu2 - 30.f) * mu2 + 3.f) * 0.125f);
        if (WHAT & PYL_PK_1D) {
            if (n2 <= middle * middle) atomicAdd(&h1[abs(kpar)], d2);
        }
        if (WHAT & PYL_PK_PHASE) {
            const float ph = atan2f(re, sqrtf(d2));
            atomicAdd(&hph[bin], ph * ph);
        }
        if (WHAT & PYL_PK_2D) {
            const int ap = abs(kpar);
            const int kper = isqrt_dev(n2 - kpar * kpar);
            atomicAdd(&acc.P2D[(long long)(middle + 1) * kper + ap], (double)d2);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * (kmax + 1); i += blockDim.x) {
        const float v = hP[i];
        if (v != 0.f) atomicAdd(&acc.P3[i], (double)v);
    }
    if (WHAT & PYL_PK_1D) {
        for (int i = threadIdx.x; i <= middle; i += blockDim.x) {
            const float v = h1[i];
            if (v != 0.f) atomicAdd(&acc.P1[i], (double)v);
        }
    }
    if (WHAT & PYL_PK_PHASE) {
        for (int i = threadIdx.x; i <= kmax; i += blockDim.x) {
            const float v = hph[i];
            if (v != 0.f) atomicAdd(&acc.Pph[i], (double)v);
        }
    }
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
    if (bytes > 48 * 1024)
        PYL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
    return PYL_OK;
}

template <int WHAT>
int launch_pk(pyl_ctx *ctx, const float2 *data, int n, int h, int axis, const FftPlan *P,
              const float *win, int B, int kmax, int kmax_per, const PkAcc &acc,
              size_t smem) {
    int st;
    if ((st = set_smem(ctx, k_pk_x<WHAT>, smem))) return st;
    dim3 grid((h + B - 1) / B, n);
    k_pk_x<WHAT><<<grid, kThreads, smem, ctx->stream>>>(data, h, axis, P->desc, P->d_tw, win,
                                                        B, kmax, kmax_per, acc);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

}  // namespace

int pk_bin_x(pyl_ctx *ctx, const float2 *data, int n, int axis, int mas, int what,
             const PkAcc &acc, int kmax, int kmax_per) {
    int st = PYL_OK;
    const FftPlan *P = fft_plan(ctx, n, &st);
    if (!P) return st;
    const float *win = window_table(ctx, n, mas, &st);
    if (!win) return st;
    const int h = n / 2 + 1;
    int B = 16;
    while (B > 1 && sizeof(float2) * (size_t)B * (n + 1) > kLineBudget) B >>= 1;
    while (B > 1 && B / 2 >= h) B >>= 1;
    const size_t smem = sizeof(float2) * ((size_t)n + 2 * (size_t)B * (n + 1)) +
                        sizeof(float) * ((size_t)n + 3 * (kmax + 1) + (n / 2 + 1) + (kmax + 1));
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "FFT length too large");
    switch (what & PYL_PK_ALL) {
        case 0: return launch_pk<0>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
        case 1: return launch_pk<1>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
        case 2: return launch_pk<2>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
        case 3: return launch_pk<3>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
        case 4: return launch_pk<4>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
        case 5: return launch_pk<5>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
        case 6: return launch_pk<6>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
        default: return launch_pk<7>(ctx, data, n, h, axis, P, win, B, kmax, kmax_per, acc, smem);
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
