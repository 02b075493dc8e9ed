// The fused x transform + power-spectrum binning of the register-FFT path
// (lengths 2^k and 3*2^k): one template, instantiated for the output sets
// in fft_reg_pk0.cu .. fft_reg_pk3.cu.
//
//   pk_x : the x-column transform fused with the window, |delta|^2,
//          Legendre weights and the integer-|k| binning, straight via a
//          padded shared line; a CTA bins a few items into float32 shared
//          histograms and adds them to the float64 sums when it ends.  The
//          3D sums alone (what = 0) are binned by mirrored pairs into
//          per-warp histograms where the lengths allow (k_pk_x_pairs).
#pragma once

#include "fft_reg_cfg.cuh"

namespace pyl {
namespace {

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
            RunAcc R;
            if (kzc < h) {
                const float2 *ln = sm + N + cc * LINE;
                const int ky = kyy > MID ? kyy - N : kyy;
                const float wyz = win[pad8(kyy)] * win[pad8(kzc)];
                constexpr int E = RegPlan<N>::E;
                bin_run<WHAT, E>(R, H, acc, ln, [](int i) { return pad8(i); }, E * rr, ky, kzc,
                                 N, axis, win, wyz, MID);
            }
            warp_flush_runs(H, R);   // every lane of the warp, valid column or not
        }
        __syncthreads();   // the shared lines are reused by the next item
    }
    H.flush(acc);
}

// Lengths whose 3D sums (what = 0) are binned by mirrored pairs: one warp
// per column of a work item, N/64 values of |kx| per lane, and items of 8
// columns (with fewer, too few warps bin: 1024^3 pk_x 4.3 -> 4.5 ms).
template <int N>
constexpr bool pair_binning() {
    return ColsCfg<N>::THREADS >= 32 * ColsCfg<N>::C && ColsCfg<N>::C >= 8 && N % 64 == 0;
}

// Fused x transform + binning of the 3D sums by mirrored pairs (the mode
// loop of class Pk, library/Pk_library/Pk_library.pyx:311-378, for the 3D
// multipoles: the same half-space selection :324-327, exact integer bins,
// window and mu^2 as bin_run).  The modes at +kx and -kx of a pencil (ky, kz
// fixed) share |k|, its bin and mu^2 (and the window), so warp w bins column
// w of the item alone: lane l takes |kx|
// in [L l, L l + L) (L = N / 64) and adds |v(+kx)|^2 + |v(-kx)|^2 with one
// bin and mu^2 evaluation; lane 31 also takes |kx| = N/2 (no mirror), and
// |kx| = 0 has none either.  On the half-space planes kz = 0 and kz = N/2
// only kx >= 0 counts (and kx = 0, N/2 only for ky >= 0), as in bin_run.
// Along the warp the bins rise with |kx|, so the runs it flushes (after the
// warp merge) never share a bin: each warp adds them to its own float
// histogram with plain read-modify-writes, no shared atomics; the C
// histograms are summed and added to the float64 sums when the CTA ends.
template <int N>
__global__ void __launch_bounds__(ColsCfg<N>::THREADS, ColsCfg<N>::PK_MINB)
k_pk_x_pairs(const float2 *__restrict__ data, int h, int rs, const float2 *__restrict__ g_tw,
             const float *__restrict__ g_win, int axis, int kmax, PkAcc acc, int nitems,
             int ipb) {
    using CF = ColsCfg<N>;
    constexpr int P = CF::P, C = CF::C, LINE = RegPlan<N>::LINE8;
    constexpr int MID = N / 2, E = RegPlan<N>::E, L = N / 64;
    static_assert(pair_binning<N>(), "one binning warp per column, whole |kx| runs per lane");
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    const int c = threadIdx.x % C, t = threadIdx.x / C;
    float2 *line = sm + N + c * LINE;
    float *win = reinterpret_cast<float *>(sm + N + C * LINE);
    const int n3 = 3 * (kmax + 1);
    float *hall = win + LINE;                         // C histograms of n3 floats
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpHist H{hall + warp * n3};                     // used by warps < C only
    load_stage_twiddles<N>(tw, g_tw);
    for (int i = threadIdx.x; i < N; i += blockDim.x) win[pad8(i)] = g_win[i];
    for (int i = threadIdx.x; i < C * n3; i += blockDim.x) hall[i] = 0.f;
    __syncthreads();
    const int nzb = (h + C - 1) / C;
    const int it0 = blockIdx.x * ipb;
    const int it1 = min(nitems, it0 + ipb);
    auto load = [&](int item, float2 (&v)[E]) {
        const int kz = (item % nzb) * C + c;
        const bool valid = kz < h;
        const float2 *base = data + (int64_t)(item / nzb) * rs + kz;
        const int64_t es = (int64_t)N * rs;
#pragma unroll
        for (int s = 0; s < E; ++s)
            v[s] = valid ? __ldcs(base + (int64_t)(t + s * P) * es) : make_float2(0.f, 0.f);
    };
    float2 v[E];
    if (it0 < it1) load(it0, v);
    for (int it = it0; it < it1; ++it) {
        const int kyy = it / nzb;
        fft_line<N, -1>(v, t, line, tw);
#pragma unroll
        for (int u = 0; u < E; ++u) line[pad8(t + u * P)] = v[u];
        __syncthreads();
        // the next item's loads are in flight while this one is binned
        if (it + 1 < it1) load(it + 1, v);
        if (warp < C) {
            const int kzc = (it % nzb) * C + warp;
            RunAcc R;
            if (kzc < h) {
                const float2 *ln = sm + N + warp * LINE;
                const int ky = kyy > MID ? kyy - N : kyy;
                const float wyz = win[pad8(kyy)] * win[pad8(kzc)];
                const float wyz2 = wyz * wyz;
                const bool plane = (kzc == 0 || kzc == MID);
                const int r2 = ky * ky + kzc * kzc;
                const int kpar_c = axis == 1 ? ky : kzc;
                const float r2f = (float)r2, kpc2f = (float)(kpar_c * kpar_c);
                const int j0 = L * lane;
                int bin = isqrt_dev(j0 * j0 + r2);
                const int nj = L + (lane == 31 ? 1 : 0);
                for (int q = 0; q < nj; ++q) {
                    const int j = j0 + q;
                    const int n2 = j * j + r2;
                    bin += ((bin + 1) * (bin + 1) <= n2) - (bin * bin > n2);
                    const float2 a = ln[pad8(j)];
                    const float wx = win[pad8(j)];
                    const float f2 = wx * wx * wyz2;
                    float d2;
                    if (!plane) {
                        float s2 = a.x * a.x + a.y * a.y;
                        if (j != 0 && j != MID) {
                            const float2 m = ln[pad8(N - j)];   // kx = -j
                            s2 += m.x * m.x + m.y * m.y;
                        }
                        d2 = s2 * f2;
                    } else {
                        if ((j == 0 || j == MID) && ky < 0) continue;
                        if (n2 == 0) *acc.dc = a;
                        d2 = (a.x * a.x + a.y * a.y) * f2;
                    }
                    const float jf = (float)j;
                    const float kpar2f = axis == 0 ? jf * jf : kpc2f;
                    const float mu2 = n2 > 0 ? __fdividef(kpar2f, fmaf(jf, jf, r2f)) : 0.f;
                    R.add(H, bin, d2, mu2);
                }
            }
            warp_flush_runs(H, R);   // every lane of the warp, valid column or not
        }
        __syncthreads();   // the shared lines are reused by the next item
    }
    for (int i = threadIdx.x; i < n3; i += blockDim.x) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < C; ++w) s += hall[w * n3 + i];
        if (s != 0.f) atomicAdd(&acc.P3[i], (double)s);
    }
}

template <int N, int WHAT>
int pk_n(pyl_ctx *ctx, const float2 *data, int h, int rs, int axis, const float2 *tw,
         const float *win, int kmax, const PkAcc &acc) {
    using CF = ColsCfg<N>;
    const size_t base = sizeof(float2) * (N + (size_t)CF::C * RegPlan<N>::LINE8) +
                        sizeof(float) * RegPlan<N>::LINE8;
    // items per CTA: enough CTAs to fill the GPU several times over, few
    // enough that the per-CTA float64 flush stays small
    const int nitems = N * ((h + CF::C - 1) / CF::C);
    int ipb = nitems / (152 * 16);
    if (ipb < 1) ipb = 1;
    if (ipb > 8) ipb = 8;
    const int grid = (nitems + ipb - 1) / ipb;
    int st;
    if constexpr (WHAT == 0 && pair_binning<N>()) {
        const size_t smem = base + sizeof(float) * (size_t)CF::C * 3 * (kmax + 1);
        if (smem <= 227 * 1024) {
            if ((st = set_smem(ctx, k_pk_x_pairs<N>, smem))) return st;
            k_pk_x_pairs<N><<<grid, CF::THREADS, smem, ctx->stream>>>(data, h, rs, tw, win, axis,
                                                                      kmax, acc, nitems, ipb);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
            return PYL_OK;
        }
    }
    const size_t smem = base + FltHist::bytes(kmax, N / 2, WHAT);
    if (smem > 227 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "Pk histogram too large");
    if ((st = set_smem(ctx, k_pk_x_p2<N, WHAT>, smem))) return st;
    k_pk_x_p2<N, WHAT><<<grid, CF::THREADS, smem, ctx->stream>>>(data, h, rs, tw, win, axis, kmax,
                                                                 acc, nitems, ipb);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

}  // namespace
}  // namespace pyl
