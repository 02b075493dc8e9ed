// The fused x transform + power-spectrum binning of the register-FFT path
// (lengths 2^k and 3*2^k): one template, instantiated for the output sets
// in fft_reg_pk0.cu .. fft_reg_pk3.cu.
//
//   pk_x : the x-column transform fused with the window, |delta|^2,
//          Legendre weights and the integer-|k| binning, straight via a
//          padded shared line; a CTA bins a few items into float32 shared
//          histograms and adds them to the float64 sums when it ends.
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

}  // namespace
}  // namespace pyl
