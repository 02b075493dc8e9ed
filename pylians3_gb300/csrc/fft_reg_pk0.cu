// The fused x transform + binning (fft_reg_pk.cuh) for the output sets
// what = 0.
#include "fft_reg_pk.cuh"

namespace pyl {

int pk_x_what0(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
               const float *win, int kmax, const PkAcc &acc) {
    const int h = n / 2 + 1;
#define CALL(N) pk_n<N, 0>(ctx, data, h, rs, axis, tw + N, win, kmax, acc)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

}  // namespace pyl
