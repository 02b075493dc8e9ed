// Register-resident Stockham FFT for lengths N = 2^k (N >= 16) and
// N = 3 * 2^k (N >= 48).
//
// A line of N complex values is held by P = N/E threads, thread t owning
// x[t + s*P], s = 0..E-1 ("strided" layout); E = 8 for powers of two and
// E = 12 for 3 * 2^k.  A stage of radix R (R divides E) with Ns = product of
// the earlier radices performs, for every butterfly j in [0, N/R),
//     k = j mod Ns,  x_q = in[j + q*N/R] * W^(k*q),  W = exp(dir*2*pi*i/(Ns*R))
//     out[(j - k)*R + k + u*Ns] = sum_q x_q exp(dir*2*pi*i*u*q/R)
// Thread t runs butterflies j = t + b*P (b < E/R), whose inputs are exactly
// its registers v[b + q*(E/R)]; outputs go through shared memory to the next
// stage.  In the last stage Ns = N/R, so its outputs land in the strided
// layout again in natural order: thread t ends with X[t + u*P] and no final
// exchange is needed.  Stage radices:
//   2^k    : one 2 or 4 first when k is not a multiple of 3, then 8s;
//   3*2^k  : a 3 first, then 4s, then a 2 when k is odd.
// Shared-memory indices are padded (Pad8: one element every 8, Pad16: one
// every 16) so that the stage exchanges of a half-warp (16 lanes of 8-byte
// elements) fall on distinct banks.  The row kernels, whose lanes run along
// one line, use Pad16 (the strided loads read 16 consecutive elements); the
// column kernels, whose lanes interleave C lines, use Pad8 with a line stride
// that spreads the lines over the banks (LINE8 / LINE16 below).
#pragma once

#include "fft_core.cuh"

namespace pyl {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int N>
struct RegPlan {
    static constexpr bool POW2 = (N & (N - 1)) == 0;
    static constexpr int E = POW2 ? 8 : 12;
    static constexpr int P = N / E;
    // padded line strides in shared memory (elements): for Pad8 with C
    // interleaved lines, for Pad16 with lanes along one line.  The extra
    // elements per length minimise the bank-conflict wavefronts of all the
    // exchange accesses (stage stores, strided loads, r2c split, binning
    // reads), counted per half-warp of 8-byte elements for each length.
    static constexpr int LINE8 = N + N / 8 + ((N == 16 || N == 48 || N == 1024 || N == 1536) ? 4 : 2);
    static constexpr int LINE16 = N + N / 16 + (N == 64 ? 0 : (N == 96 ? 2 : 1));
    static constexpr int K = POW2 ? ilog2c(N) : ilog2c(N / 3);   // power of two part
    static constexpr int NST = POW2 ? (K % 3 == 0 ? K / 3 : K / 3 + 1)
                                    : 1 + K / 2 + (K % 2);
    static constexpr int radix(int s) {
        if (POW2) return (s == 0 && K % 3 != 0) ? (K % 3 == 1 ? 2 : 4) : 8;
        if (s == 0) return 3;
        return (s == NST - 1 && (K % 2)) ? 2 : 4;
    }
    static constexpr int ns(int s) { return s == 0 ? 1 : ns(s - 1) * radix(s - 1); }
};

// Twiddles of the stages with NS > 1, stage after stage: stage s holds
// T_s[q * NS + k] = W_N^(m_q * k * ST), k < NS, with m_q = 2^q for q <
// mults(R) (W^k, W^2k and W^4k for radix 8; W^k, W^2k for radix 4 and 3;
// W^k for radix 2).  A half-warp then reads consecutive k (or one k by
// broadcast) instead of k * ST-strided entries of an N-entry table, which
// fall on few banks.  SIZE < N for every supported length.
template <int N>
struct TwStages {
    using PL = RegPlan<N>;
    static constexpr int mults(int R) { return R == 8 ? 3 : (R == 2 ? 1 : 2); }
    static constexpr int count(int s) { return PL::ns(s) > 1 ? mults(PL::radix(s)) * PL::ns(s) : 0; }
    static constexpr int off(int s) { return s == 0 ? 0 : off(s - 1) + count(s - 1); }
    static constexpr int SIZE = off(PL::NST);
    static_assert(SIZE <= N, "stage twiddles fit the N-entry slot");
};

// Entry i of the stage tables as an index of the N-entry table W_N^m (the
// host appends the stage tables after that table: twiddles_host).
template <int N, int S>
__host__ __device__ inline int stage_tw_src(int i) {
    if constexpr (S >= RegPlan<N>::NST) {
        return 0;
    } else {
        constexpr int NS = RegPlan<N>::ns(S), R = RegPlan<N>::radix(S), ST = N / (NS * R);
        constexpr int O0 = TwStages<N>::off(S), O1 = TwStages<N>::off(S + 1);
        if (O1 > O0 && i >= O0 && i < O1) {
            const int r = i - O0;
            return (1 << (r / NS)) * (r % NS) * ST;
        }
        return stage_tw_src<N, S + 1>(i);
    }
}

// Shared stage tables from their global copy (all threads).
template <int N>
__device__ __forceinline__ void load_stage_twiddles(float2 *tw, const float2 *__restrict__ g_stw) {
    for (int i = threadIdx.x; i < TwStages<N>::SIZE; i += blockDim.x) tw[i] = g_stw[i];
}

template <int N>
constexpr bool reg_fft_length() {
    return (N >= 16 && (N & (N - 1)) == 0) ||
           (N >= 48 && N % 3 == 0 && ((N / 3) & (N / 3 - 1)) == 0);
}

__device__ __forceinline__ int pad8(int i) { return i + (i >> 3); }
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }
struct Pad8 {
    __device__ __forceinline__ int operator()(int i) const { return pad8(i); }
};
struct Pad16 {
    __device__ __forceinline__ int operator()(int i) const { return pad16(i); }
};

template <int DIR>
__device__ __forceinline__ float2 twl(const float2 *tw, int m) {
    float2 w = tw[m];
    if (DIR > 0) w.y = -w.y;
    return w;
}

template <int DIR>
__device__ __forceinline__ void dft3(float2 &a0, float2 &a1, float2 &a2) {
    const float h3 = 0.86602540378443864676f;   // sqrt(3)/2
    const float2 t1 = cadd(a1, a2), t2 = csub(a1, a2);
    const float2 m = make_float2(a0.x - 0.5f * t1.x, a0.y - 0.5f * t1.y);
    const float2 r = mul_i<DIR>(make_float2(h3 * t2.x, h3 * t2.y));
    a0 = cadd(a0, t1);
    a1 = cadd(m, r);
    a2 = csub(m, r);
}

// One stage in registers; tw: this stage's table (TwStages).
template <int N, int R, int NS, int DIR>
__device__ __forceinline__ void stage_compute(float2 (&v)[RegPlan<N>::E], int t, const float2 *tw) {
    constexpr int E = RegPlan<N>::E;
    constexpr int P = RegPlan<N>::P;
    constexpr int NB = E / R;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * P;
        const int k = j % NS;
        float2 x[R];
#pragma unroll
        for (int q = 0; q < R; ++q) x[q] = v[b + q * NB];
        if constexpr (NS > 1) {
            if constexpr (R == 2) {
                x[1] = cmul(x[1], twl<DIR>(tw, k));
            } else if constexpr (R == 3) {
                x[1] = cmul(x[1], twl<DIR>(tw, k));
                x[2] = cmul(x[2], twl<DIR>(tw, NS + k));
            } else if constexpr (R == 4) {
                const float2 w1 = twl<DIR>(tw, k), w2 = twl<DIR>(tw, NS + k);
                x[1] = cmul(x[1], w1);
                x[2] = cmul(x[2], w2);
                x[3] = cmul(x[3], cmul(w1, w2));
            } else {
                const float2 w1 = twl<DIR>(tw, k), w2 = twl<DIR>(tw, NS + k);
                const float2 w4 = twl<DIR>(tw, 2 * NS + k);
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
        if constexpr (R == 2) dft2<DIR>(x[0], x[1]);
        else if constexpr (R == 3) dft3<DIR>(x[0], x[1], x[2]);
        else if constexpr (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
        else dft8<DIR>(x);
#pragma unroll
        for (int u = 0; u < R; ++u) v[b + u * NB] = x[u];
    }
}

// Scatter the stage outputs to their Stockham positions in the shared line.
template <int N, int R, int NS, class IDX>
__device__ __forceinline__ void stage_store(const float2 (&v)[RegPlan<N>::E], int t, float2 *line) {
    constexpr int E = RegPlan<N>::E;
    constexpr int P = RegPlan<N>::P;
    constexpr int NB = E / R;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * P;
        const int k = j % NS;
        const int ob = (j - k) * R + k;
#pragma unroll
        for (int u = 0; u < R; ++u) line[IDX()(ob + u * NS)] = v[b + u * NB];
    }
}

template <int N, class IDX>
__device__ __forceinline__ void strided_load(float2 (&v)[RegPlan<N>::E], int t, const float2 *line) {
    constexpr int E = RegPlan<N>::E;
    constexpr int P = RegPlan<N>::P;
#pragma unroll
    for (int s = 0; s < E; ++s) v[s] = line[IDX()(t + s * P)];
}

// Stage S of the plan (compile-time recursion).  Each exchange between
// stages is bracketed by __syncthreads(), so every thread of the CTA must
// call this the same number of times.
template <int N, int DIR, int S, class IDX>
__device__ __forceinline__ void run_stages(float2 (&v)[RegPlan<N>::E], int t, float2 *line,
                                           const float2 *tw) {
    using PL = RegPlan<N>;
    constexpr int R = PL::radix(S);
    constexpr int NS = PL::ns(S);
    stage_compute<N, R, NS, DIR>(v, t, tw + TwStages<N>::off(S));
    if constexpr (S + 1 < PL::NST) {
        stage_store<N, R, NS, IDX>(v, t, line);
        __syncthreads();
        strided_load<N, IDX>(v, t, line);
        __syncthreads();
        run_stages<N, DIR, S + 1, IDX>(v, t, line, tw);
    }
}

// Full FFT of the thread's line: input and output in the strided layout;
// IDX maps line positions to padded shared-memory indices; tw holds the
// stage tables (load_stage_twiddles).
template <int N, int DIR, class IDX = Pad8>
__device__ __forceinline__ void fft_line(float2 (&v)[RegPlan<N>::E], int t, float2 *line,
                                         const float2 *tw) {
    static_assert(reg_fft_length<N>(), "register FFT length must be 2^k or 3*2^k");
    static_assert(RegPlan<N>::ns(RegPlan<N>::NST - 1) * RegPlan<N>::radix(RegPlan<N>::NST - 1) == N,
                  "stage radices must multiply to N");
    run_stages<N, DIR, 0, IDX>(v, t, line, tw);
}

}  // namespace pyl
