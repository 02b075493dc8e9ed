// The fused x transform + binning (fft_reg_pk.cuh) for the output sets
// what = 4, 5.
#include "fft_reg_pk.cuh"

namespace pyl {
namespace {

template <int N>
int pk_group(pyl_ctx *ctx, const float2 *data, int h, int rs, int axis, const float2 *stw,
             const float *win, int kmax, const PkAcc &acc, int what) {
    switch (what) {
        case 4: return pk_n<N, 4>(ctx, data, h, rs, axis, stw, win, kmax, acc);
        case 5: return pk_n<N, 5>(ctx, data, h, rs, axis, stw, win, kmax, acc);
        default: return PYL_ERR_ARG;
    }
}

}  // namespace

int pk_x_what45(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
                const float *win, int kmax, const PkAcc &acc, int what) {
    const int h = n / 2 + 1;
#define CALL(N) pk_group<N>(ctx, data, h, rs, axis, tw + N, win, kmax, acc, what)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

}  // namespace pyl
