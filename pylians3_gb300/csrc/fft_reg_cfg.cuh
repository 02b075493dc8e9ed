// Launch configuration shared by the register-FFT translation units
// (fft_reg.cu and the fused power-spectrum pass in fft_reg_pk*.cu).
#pragma once

#include "fft_reg.cuh"
#include "pk_common.cuh"

namespace pyl {

template <int N>
struct RowsCfg {
    static constexpr int P = RegPlan<N>::P;
    static constexpr int L = P >= 256 ? 1 : 256 / P;   // row pairs per CTA
    static constexpr int THREADS = L * P;
};

template <int N>
struct ColsCfg {
    static constexpr int P = RegPlan<N>::P;
    static constexpr int C = P >= 512 ? 1 : (512 / P > 8 ? 8 : 512 / P);
    static constexpr int THREADS = C * P;
    // resident CTAs the fused Pk kernel is compiled for: E = 12 keeps two
    // register lines (the current item and the prefetched one) per thread
    static constexpr int PK_MINB =
        RegPlan<N>::E == 8 ? (THREADS >= 512 ? 2 : 4) : (THREADS >= 512 ? 1 : 2);
};

template <typename K>
int set_smem(pyl_ctx *ctx, K kernel, size_t bytes) {
    if (bytes > 40 * 1024)   // static shared memory counts toward the 48 KB default too
        PYL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
    return PYL_OK;
}

#define PYL_POW2_DISPATCH(n, CALL)                 \
    switch (n) {                                   \
        case 16: return CALL(16);                  \
        case 32: return CALL(32);                  \
        case 64: return CALL(64);                  \
        case 128: return CALL(128);                \
        case 256: return CALL(256);                \
        case 512: return CALL(512);                \
        case 1024: return CALL(1024);              \
        case 2048: return CALL(2048);              \
        case 4096: return CALL(4096);              \
        case 48: return CALL(48);                  \
        case 96: return CALL(96);                  \
        case 192: return CALL(192);                \
        case 384: return CALL(384);                \
        case 768: return CALL(768);                \
        case 1536: return CALL(1536);              \
        case 3072: return CALL(3072);              \
        default: return PYL_ERR_UNSUPPORTED;       \
    }

// The fused x transform + binning for the output sets what = 0, 1..3, 4..5
// and 6..7 (one translation unit each, fft_reg_pk0..3.cu, so that they
// compile in parallel); tw: the table from twiddles_host(n).
int pk_x_what0(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
               const float *win, int kmax, const PkAcc &acc);
int pk_x_what13(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
                const float *win, int kmax, const PkAcc &acc, int what);
int pk_x_what45(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
                const float *win, int kmax, const PkAcc &acc, int what);
int pk_x_what67(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
                const float *win, int kmax, const PkAcc &acc, int what);

}  // namespace pyl
