// Register-resident radix-8 Stockham FFT for power-of-two lengths N >= 8.
//
// A line of N complex values is held by P = N/8 threads, thread t owning
// x[t + s*P], s = 0..7 ("strided" layout).  The stages are radix R0 in
// {2, 4, 8} (so that the remaining length is a power of 8) followed by
// radix-8 stages.  A stage of radix R with Ns = product of the earlier radices
// performs, for every butterfly j in [0, N/R),
//     k = j mod Ns,  x_q = in[j + q*N/R] * W^(k*q),  W = exp(dir*2*pi*i/(Ns*R))
//     out[(j - k)*R + k + u*Ns] = sum_q x_q exp(dir*2*pi*i*u*q/R)
// Thread t runs butterflies j = t + b*P (b < 8/R), whose inputs are exactly
// its registers v[b + q*(8/R)]; outputs go through shared memory to the next
// stage.  The last stage has R = 8 and Ns = P, so its outputs land in the
// strided layout again, in natural order: thread t ends with X[t + u*P] and no
// final exchange is needed.  Shared-memory indices are padded by one element
// every 8 (pad8) so that the stride-8 stores of the first stage do not
// conflict on banks.
#pragma once

#include "fft_core.cuh"

namespace pyl {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int N>
struct Pow2 {
    static constexpr int P = N / 8;
    static constexpr int LOG = ilog2c(N);
    static constexpr int R0 = (LOG % 3 == 0) ? 8 : (LOG % 3 == 1 ? 2 : 4);
    static constexpr int NST = (LOG % 3 == 0) ? LOG / 3 : LOG / 3 + 1;
    static constexpr int LINE = N + N / 8 + 1;   // padded line stride in shared memory
};

__device__ __forceinline__ int pad8(int i) { return i + (i >> 3); }

template <int DIR>
__device__ __forceinline__ float2 twl(const float2 *tw, int m) {
    float2 w = tw[m];
    if (DIR > 0) w.y = -w.y;
    return w;
}

// One butterfly group of a stage, in registers.
template <int N, int R, int NS, int DIR>
__device__ __forceinline__ void stage_compute(float2 (&v)[8], int t, const float2 *tw) {
    constexpr int P = N / 8;
    constexpr int NB = 8 / R;
    constexpr int ST = N / (NS * R);   // table stride of W
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * P;
        const int k = j & (NS - 1);
        float2 x[R];
#pragma unroll
        for (int q = 0; q < R; ++q) x[q] = v[b + q * NB];
        if (NS > 1) {
            if (R == 2) {
                x[1] = cmul(x[1], twl<DIR>(tw, k * ST));
            } else if (R == 4) {
                const float2 w1 = twl<DIR>(tw, k * ST), w2 = twl<DIR>(tw, 2 * k * ST);
                x[1] = cmul(x[1], w1);
                x[2] = cmul(x[2], w2);
                x[3] = cmul(x[3], cmul(w1, w2));
            } else {
                const float2 w1 = twl<DIR>(tw, k * ST), w2 = twl<DIR>(tw, 2 * k * ST);
                const float2 w4 = twl<DIR>(tw, 4 * k * ST);
                const float2 w3 = cmul(w1, w2);
                x[1] = cmul(x[1], w1);
                x[2] = cmul(x[2], w2);
                x[3] = cmul(x[3], w3);
                x[4] = cmul(x[4], w4);
                x[5] = cmul(x[5], cmul(w1, w4));
                x[6] = cmul(x[6], cmul(w2, w4));
                x[7] = cmul(x[7], cmul(w3, w4));
            }
        }
        if (R == 2) dft2<DIR>(x[0], x[1]);
        else if (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
        else dft8<DIR>(x);
#pragma unroll
        for (int u = 0; u < R; ++u) v[b + u * NB] = x[u];
    }
}

// Scatter the stage outputs to their Stockham positions in the shared line.
template <int N, int R, int NS>
__device__ __forceinline__ void stage_store(const float2 (&v)[8], int t, float2 *line) {
    constexpr int P = N / 8;
    constexpr int NB = 8 / R;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * P;
        const int k = j & (NS - 1);
        const int ob = (j - k) * R + k;
#pragma unroll
        for (int u = 0; u < R; ++u) line[pad8(ob + u * NS)] = v[b + u * NB];
    }
}

template <int N>
__device__ __forceinline__ void strided_load(float2 (&v)[8], int t, const float2 *line) {
    constexpr int P = N / 8;
#pragma unroll
    for (int s = 0; s < 8; ++s) v[s] = line[pad8(t + s * P)];
}

// Stage S of the plan (compile-time recursion).  Each exchange between
// stages is bracketed by __syncthreads(), so every thread of the CTA must
// call this the same number of times.
template <int N, int DIR, int S>
__device__ __forceinline__ void run_stages(float2 (&v)[8], int t, float2 *line, const float2 *tw) {
    using PL = Pow2<N>;
    constexpr int R = (S == 0) ? PL::R0 : 8;
    constexpr int NS = (S == 0) ? 1 : PL::R0 * (1 << (3 * (S - 1)));
    stage_compute<N, R, NS, DIR>(v, t, tw);
    if constexpr (S + 1 < PL::NST) {
        stage_store<N, R, NS>(v, t, line);
        __syncthreads();
        strided_load<N>(v, t, line);
        __syncthreads();
        run_stages<N, DIR, S + 1>(v, t, line, tw);
    }
}

// Full FFT of the thread's line: input and output in the strided layout.
template <int N, int DIR>
__device__ __forceinline__ void fft_line(float2 (&v)[8], int t, float2 *line, const float2 *tw) {
    run_stages<N, DIR, 0>(v, t, line, tw);
}

}  // namespace pyl
