// Auto- and cross-power spectra of several fields (class XPk,
// library/Pk_library/Pk_library.pyx:529-735).  Each field is transformed in
// full (z r2c, y and x c2c) into its own half-complex grid; one binning pass
// then reads all fields at each independent mode, applies each field's MAS
// window and accumulates, per bin, the auto terms |delta_i|^2 and the cross
// terms Re(delta_i conj(delta_j)) = re_i re_j + im_i im_j with the Legendre
// weights (3D), per k_par (1D, |k| <= middle) and per (k_par, k_per) (2D).
// Mode counts and the sums of |k| come from the cached mode tables, as for
// class Pk.
#include <math.h>
#include <string.h>

#include "pk_common.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxFields = 8;
constexpr int kModesPerCta = 16384;

struct XPkArgs {
    const float2 *half[kMaxFields];   // per field: (d, d, rs) complex, fully transformed
    int nf, ns;                       // fields, series (fields + pairs)
    int d, h, rs, axis, kmax, kmax_par, kmax_per;
    const float *win;                 // nf * d window factors
    double *P3;                       // (kmax+1) * 3 * ns
    double *P1;                       // (kmax_par+1) * ns
    double *P2;                       // (kmax_par+1)*(kmax_per+1) * ns
};

// One CTA bins kModesPerCta consecutive modes (z fastest, so the reads of
// every field are coalesced) into float32 shared bins (3D and 1D; a few
// hundred terms per bin at most), added to the float64 sums when it ends;
// the 2D bins go straight to the float64 sums.
__global__ void __launch_bounds__(kThreads)
k_xpk_bin(XPkArgs A) {
    extern __shared__ float s_x[];
    const int ns = A.ns, nf = A.nf, d = A.d;
    float *win = s_x;                                   // nf * d
    float *h3 = win + nf * d;                           // (kmax+1) * 3 * ns
    float *h1 = h3 + (A.kmax + 1) * 3 * ns;             // (kmax_par+1) * ns
    const int n3 = (A.kmax + 1) * 3 * ns, n1 = (A.kmax_par + 1) * ns;
    for (int i = threadIdx.x; i < nf * d; i += blockDim.x) win[i] = A.win[i];
    for (int i = threadIdx.x; i < n3 + n1; i += blockDim.x) h3[i] = 0.f;
    __syncthreads();
    const int mid = d / 2;
    const bool even = (d & 1) == 0;
    const long long total = (long long)d * d * A.h;
    const long long m0 = (long long)blockIdx.x * kModesPerCta;
    const long long m1 = min(total, m0 + kModesPerCta);
    for (long long m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
        const int kzz = (int)(m % A.h);
        const long long row = m / A.h;
        const int kyy = (int)(row % d), kxx = (int)(row / d);
        const int kx = kxx > mid ? kxx - d : kxx;
        const int ky = kyy > mid ? kyy - d : kyy;
        const int kz = kzz;
        if (kz == 0 || (kz == mid && even)) {
            if (kx < 0) continue;
            if ((kx == 0 || (kx == mid && even)) && ky < 0) continue;
        }
        const int n2 = kx * kx + ky * ky + kz * kz;
        const int bin = isqrt_dev(n2);
        const int kpar = A.axis == 0 ? kx : (A.axis == 1 ? ky : kz);
        const int kper = isqrt_dev(n2 - kpar * kpar);
        const float mu2 = n2 > 0 ? (float)(kpar * kpar) / (float)n2 : 0.f;
        const float l2 = (3.f * mu2 - 1.f) * 0.5f;
        const float l4 = ((35.f * mu2 - 30.f) * mu2 + 3.f) * 0.125f;
        const int ap = abs(kpar);
        const bool in1 = n2 <= mid * mid;
        const long long i2 = (long long)(A.kmax_par + 1) * kper + ap;
        const long long off = ((long long)kxx * d + kyy) * A.rs + kzz;
        float re[kMaxFields], im[kMaxFields];
#pragma unroll
        for (int i = 0; i < kMaxFields; ++i) {
            if (i < nf) {
                const float *w = win + i * d;
                const float f = w[kxx] * (w[kyy] * w[kzz]);
                const float2 v = A.half[i][off];
                re[i] = v.x * f;
                im[i] = v.y * f;
            }
        }
        int s = 0;
        auto add = [&](float t) {
            float *b = h3 + (bin * 3) * ns + s;
            atomicAdd(b, t);
            atomicAdd(b + ns, t * l2);
            atomicAdd(b + 2 * ns, t * l4);
            if (in1) atomicAdd(&h1[ap * ns + s], t);
            atomicAdd(&A.P2[i2 * ns + s], (double)t);
            ++s;
        };
#pragma unroll
        for (int i = 0; i < kMaxFields; ++i)
            if (i < nf) add(re[i] * re[i] + im[i] * im[i]);
#pragma unroll
        for (int i = 0; i < kMaxFields; ++i)
#pragma unroll
            for (int j = i + 1; j < kMaxFields; ++j)
                if (j < nf) add(re[i] * re[j] + im[i] * im[j]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n3; i += blockDim.x)
        if (h3[i] != 0.f) atomicAdd(&A.P3[i], (double)h3[i]);
    for (int i = threadIdx.x; i < n1; i += blockDim.x)
        if (h1[i] != 0.f) atomicAdd(&A.P1[i], (double)h1[i]);
}

}  // namespace

}  // namespace pyl

using namespace pyl;

extern "C" {

int pyl_xpk(pyl_ctx *ctx, const float *const *deltas, int nfields, int dims, double BoxSize,
            int axis, const int *mas, pyl_xpk_out *out, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (!deltas || !mas || !out || nfields < 1 || nfields > kMaxFields || dims < 2)
        return fail(ctx, PYL_ERR_ARG, "bad XPk arguments (1 to 8 fields)");
    for (int i = 0; i < nfields; ++i)
        if (!deltas[i]) return fail(ctx, PYL_ERR_ARG, "null field");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool dev = flags & PYL_DEVICE_PTRS;
    int st = PYL_OK;
    const ModeTables *T = mode_tables(ctx, dims, axis, &st);
    if (!T) return st;
    const int h = dims / 2 + 1, rs = half_stride(dims);
    const long long cells = (long long)dims * dims * dims;
    const int nx = nfields * (nfields - 1) / 2, ns = nfields + nx;
    XPkArgs A;
    memset(&A, 0, sizeof A);
    A.nf = nfields;
    A.ns = ns;
    A.d = dims;
    A.h = h;
    A.rs = rs;
    A.axis = T->axis;
    A.kmax = T->kmax;
    A.kmax_par = T->kmax_par;
    A.kmax_per = T->kmax_per;
    const size_t hb = sizeof(float2) * (size_t)dims * dims * rs;
    char *halves = (char *)ws_get(ctx, "xpk_half", hb * nfields, &st);
    if (!halves) return st;
    float *in = nullptr;
    if (!dev) {
        in = (float *)ws_get(ctx, "xpk_in", sizeof(float) * (size_t)cells, &st);
        if (!in) return st;
    }
    float *win = (float *)ws_get(ctx, "xpk_win", sizeof(float) * (size_t)nfields * dims, &st);
    if (!win) return st;
    for (int i = 0; i < nfields; ++i) {
        float2 *half = reinterpret_cast<float2 *>(halves + hb * i);
        const float *src = deltas[i];
        if (!dev) {
            PYL_CUDA(ctx, cudaMemcpyAsync(in, deltas[i], sizeof(float) * (size_t)cells,
                                          cudaMemcpyHostToDevice, ctx->stream));
            src = in;
        }
        if ((st = fft_rows_r2c(ctx, src, half, (long long)dims * dims, dims, rs))) return st;
        if ((st = fft_axis_c2c(ctx, half, dims, h, rs, 1, -1))) return st;
        if ((st = fft_axis_c2c(ctx, half, dims, h, rs, 0, -1))) return st;
        A.half[i] = half;
        const float *w = window_table(ctx, dims, mas[i], &st);
        if (!w) return st;
        PYL_CUDA(ctx, cudaMemcpyAsync(win + (size_t)i * dims, w, sizeof(float) * dims,
                                      cudaMemcpyDeviceToDevice, ctx->stream));
    }
    A.win = win;
    const size_t n3 = (size_t)(T->kmax + 1) * 3 * ns, n1 = (size_t)(T->kmax_par + 1) * ns;
    const size_t n2 = (size_t)(T->kmax_par + 1) * (T->kmax_per + 1) * ns;
    double *acc = (double *)ws_get(ctx, "xpk_acc", sizeof(double) * (n3 + n1 + n2), &st);
    if (!acc) return st;
    PYL_CUDA(ctx, cudaMemsetAsync(acc, 0, sizeof(double) * (n3 + n1 + n2), ctx->stream));
    A.P3 = acc;
    A.P1 = acc + n3;
    A.P2 = acc + n3 + n1;
    const size_t smem = sizeof(float) * ((size_t)nfields * dims + n3 + n1);
    if (smem > 220 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "XPk: too many bins for one CTA");
    if (smem > 40 * 1024)
        PYL_CUDA(ctx, cudaFuncSetAttribute(k_xpk_bin, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
    const long long total = (long long)dims * dims * h;
    k_xpk_bin<<<(unsigned)((total + kModesPerCta - 1) / kModesPerCta), kThreads, smem,
                ctx->stream>>>(A);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    std::vector<double> raw(n3 + n1 + n2);
    PYL_CUDA(ctx, cudaMemcpyAsync(raw.data(), acc, sizeof(double) * raw.size(),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    if ((st = status_check(ctx))) return st;

    // ---- finalisation, Pk_library.pyx:737-803 (formulas and order kept)
    const long long own = (dims % 2 == 1) ? 1 : 8;
    const long long expected = (cells - own) / 2 + own;
    if (T->total != expected) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "WARNING: Not all modes counted: counted %lld independent modes, expected %lld",
                 T->total, expected);
        return fail(ctx, PYL_ERR_MODES, buf);
    }
    const double kF = 2.0 * M_PI / BoxSize;
    const double kN = (dims / 2) * kF;
    const double fact = pow(BoxSize / ((double)dims * dims), 3);
    const double *P3 = raw.data(), *P1 = P3 + n3, *P2 = P1 + n1;
    auto col = [&](int s) { return s < nfields ? s : s - nfields; };
    for (int i = 1; i <= T->kmax_par; ++i) {
        const double N = T->N1D[i];
        const double k1 = (T->k1Dsum[i] / N) * kF;
        const double kmaxper = sqrt(kN * kN - k1 * k1);
        if (out->k1D) out->k1D[i - 1] = k1;
        if (out->Nmodes1D) out->Nmodes1D[i - 1] = N;
        for (int s = 0; s < ns; ++s) {
            double v = P1[(size_t)i * ns + s] * fact;
            v = v * (M_PI * kmaxper * kmaxper / N) / ((2.0 * M_PI) * (2.0 * M_PI));
            double *dst = s < nfields ? out->Pk1D : out->PkX1D;
            const int w = s < nfields ? nfields : nx;
            if (dst) dst[(size_t)(i - 1) * w + col(s)] = v;
        }
    }
    const int np = T->kmax_par + 1, nq = T->kmax_per + 1;
    for (int q = 0; q < nq; ++q)
        for (int p = 0; p < np; ++p) {
            const size_t i = (size_t)np * q + p;
            if (out->kpar) out->kpar[i] = 0.5 * (p + p + 1) * kF;
            if (out->kper) out->kper[i] = 0.5 * (q + q + 1) * kF;
            if (out->Nmodes2D) out->Nmodes2D[i] = T->N2D[i];
            for (int s = 0; s < ns; ++s) {
                double *dst = s < nfields ? out->Pk2D : out->PkX2D;
                const int w = s < nfields ? nfields : nx;
                if (dst) dst[i * w + col(s)] = P2[i * ns + s] * fact / T->N2D[i];
            }
        }
    for (int b = 1; b <= T->kmax; ++b) {
        const double N = T->N3D[b];
        if (out->k3D) out->k3D[b - 1] = (T->k3Dsum[b] / N) * kF;
        if (out->Nmodes3D) out->Nmodes3D[b - 1] = N;
        for (int s = 0; s < ns; ++s) {
            double *dst = s < nfields ? out->Pk : out->XPk;
            const int w = s < nfields ? nfields : nx;
            if (!dst) continue;
            const size_t base = ((size_t)(b - 1) * 3) * w + col(s);
            dst[base] = (P3[((size_t)b * 3 + 0) * ns + s] / N) * fact;
            dst[base + w] = (P3[((size_t)b * 3 + 1) * ns + s] * 5.0 / N) * fact;
            dst[base + 2 * (size_t)w] = (P3[((size_t)b * 3 + 2) * ns + s] * 9.0 / N) * fact;
        }
    }
    return PYL_OK;
}

}  // extern "C"
