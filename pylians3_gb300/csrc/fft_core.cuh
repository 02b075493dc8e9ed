// Shared-memory Stockham FFT used by the FFT and power-spectrum kernels.
//
// A CTA transforms `nlines` lines of length n held in shared memory (line l
// at buf[l*ld + i]).  Each stage of radix r performs, for every line and
// every j in [0, n/r):
//     k = j mod Ns,  x_t = src[j + t*n/r] * W^(k*t),  W = exp(dir*2*pi*i/(Ns*r))
//     dst[(j - k)*r + k + u*Ns] = sum_t x_t * exp(dir*2*pi*i*u*t/r)
// (Stockham autosort: the result of the last stage is in natural order), then
// Ns *= r.  Radices 2, 4 and 8 have hand-written butterflies; 3, 5 and 7 use
// a register DFT with table constants; any other prime uses a direct DFT
// that reads its inputs from shared memory (slow, but any n works).
#pragma once

#include "common.cuh"

namespace pyl {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    return make_float2(a.x - b.x, a.y - b.y);
}
// multiply by dir*i  (dir = -1 forward, +1 inverse)
template <int DIR>
__device__ __forceinline__ float2 mul_i(float2 a) {
    return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}
template <int DIR>
__device__ __forceinline__ float2 tw_get(const float2 *tw, int m) {
    float2 w = tw[m];
    if (DIR > 0) w.y = -w.y;
    return w;
}

template <int DIR>
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
    float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <int DIR>
__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3) {
    float2 s02 = cadd(a0, a2), d02 = csub(a0, a2);
    float2 s13 = cadd(a1, a3), d13 = mul_i<DIR>(csub(a1, a3));
    a0 = cadd(s02, s13);
    a2 = csub(s02, s13);
    a1 = cadd(d02, d13);
    a3 = csub(d02, d13);
}

template <int DIR>
__device__ __forceinline__ void dft8(float2 *x) {
    const float h = 0.70710678118654752440f;
    // a_t = x_t + x_{t+4};  b_t = (x_t - x_{t+4}) * W8^t
    float2 a0 = cadd(x[0], x[4]), a1 = cadd(x[1], x[5]);
    float2 a2 = cadd(x[2], x[6]), a3 = cadd(x[3], x[7]);
    float2 b0 = csub(x[0], x[4]), b1 = csub(x[1], x[5]);
    float2 b2 = csub(x[2], x[6]), b3 = csub(x[3], x[7]);
    // W8^1 = h*(1 + dir*i), W8^2 = dir*i, W8^3 = h*(-1 + dir*i)
    b1 = DIR < 0 ? make_float2(h * (b1.x + b1.y), h * (b1.y - b1.x))
                 : make_float2(h * (b1.x - b1.y), h * (b1.y + b1.x));
    b2 = mul_i<DIR>(b2);
    b3 = DIR < 0 ? make_float2(h * (b3.y - b3.x), -h * (b3.x + b3.y))
                 : make_float2(-h * (b3.x + b3.y), h * (b3.x - b3.y));
    dft4<DIR>(a0, a1, a2, a3);
    dft4<DIR>(b0, b1, b2, b3);
    x[0] = a0; x[2] = a1; x[4] = a2; x[6] = a3;
    x[1] = b0; x[3] = b1; x[5] = b2; x[7] = b3;
}

// r-point DFT in registers with constants from the table (r = 3, 5, 7).
template <int DIR, int R>
__device__ __forceinline__ void dft_small(float2 *x, const float2 *tw, int n) {
    float2 y[R];
    const int step = n / R;
#pragma unroll
    for (int u = 0; u < R; ++u) {
        float2 acc = x[0];
#pragma unroll
        for (int t = 1; t < R; ++t) {
            float2 w = tw_get<DIR>(tw, ((u * t) % R) * step);
            acc = cadd(acc, cmul(x[t], w));
        }
        y[u] = acc;
    }
#pragma unroll
    for (int u = 0; u < R; ++u) x[u] = y[u];
}

template <int DIR, int R>
__device__ __forceinline__ void stage_reg(const float2 *src, float2 *dst, int ld,
                                          int nlines, int n, int Ns,
                                          const float2 *tw) {
    const int m = n / R;
    const int total = nlines * m;
    const int step = n / (Ns * R);
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int line = idx / m;
        const int j = idx - line * m;
        const float2 *in = src + line * ld;
        float2 *out = dst + line * ld;
        const int k = j % Ns;
        float2 x[R];
#pragma unroll
        for (int t = 0; t < R; ++t) x[t] = in[j + t * m];
        if (Ns > 1) {
#pragma unroll
            for (int t = 1; t < R; ++t) x[t] = cmul(x[t], tw_get<DIR>(tw, k * t * step));
        }
        if (R == 2) dft2<DIR>(x[0], x[1]);
        else if (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
        else if (R == 8) dft8<DIR>(x);
        else dft_small<DIR, R>(x, tw, n);
        const int ob = (j - k) * R + k;
#pragma unroll
        for (int u = 0; u < R; ++u) out[ob + u * Ns] = x[u];
    }
}

// Direct DFT stage for an arbitrary radix (large primes).
template <int DIR>
__device__ void stage_generic(const float2 *src, float2 *dst, int ld, int nlines,
                              int n, int Ns, int R, const float2 *tw) {
    const int m = n / R;
    const int total = nlines * m * R;
    const int step = n / (Ns * R);
    const int rstep = n / R;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int u = idx % R;
        const int jj = idx / R;
        const int line = jj / m;
        const int j = jj - line * m;
        const float2 *in = src + line * ld;
        const int k = j % Ns;
        float2 acc = make_float2(0.f, 0.f);
        for (int t = 0; t < R; ++t) {
            float2 x = in[j + t * m];
            // W^(k t) * exp(dir 2 pi i u t / R) = table[(k t step + u t rstep) mod n]
            long long e = (long long)k * t * step + (long long)((u * t) % R) * rstep;
            x = cmul(x, tw_get<DIR>(tw, (int)(e % n)));
            acc = cadd(acc, x);
        }
        dst[line * ld + (j - k) * R + k + u * Ns] = acc;
    }
}

// Transform all lines; returns the buffer holding the result (src or dst).
// Must be called by every thread of the CTA; ends with __syncthreads().
template <int DIR>
__device__ float2 *fft_smem(float2 *src, float2 *dst, int ld, int nlines,
                            const FftDesc &D, const float2 *tw) {
    int Ns = 1;
    const int n = D.n;
    for (int s = 0; s < D.nst; ++s) {
        const int r = D.radix[s];
        switch (r) {
            case 2: stage_reg<DIR, 2>(src, dst, ld, nlines, n, Ns, tw); break;
            case 3: stage_reg<DIR, 3>(src, dst, ld, nlines, n, Ns, tw); break;
            case 4: stage_reg<DIR, 4>(src, dst, ld, nlines, n, Ns, tw); break;
            case 5: stage_reg<DIR, 5>(src, dst, ld, nlines, n, Ns, tw); break;
            case 7: stage_reg<DIR, 7>(src, dst, ld, nlines, n, Ns, tw); break;
            case 8: stage_reg<DIR, 8>(src, dst, ld, nlines, n, Ns, tw); break;
            default: stage_generic<DIR>(src, dst, ld, nlines, n, Ns, r, tw); break;
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
        Ns *= r;
    }
    return src;
}

__device__ __forceinline__ void load_twiddles(float2 *s_tw, const float2 *g_tw, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_tw[i] = g_tw[i];
}

}  // namespace pyl
