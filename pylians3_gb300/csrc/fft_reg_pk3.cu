// The fused x transform + binning (fft_reg_pk.cuh) for the output sets
// what = 6, 7.
#include "fft_reg_pk.cuh"

namespace pyl {
namespace {

template <int N>
int pk_group(pyl_ctx *ctx, const float2 *data, int h, int rs, int axis, const float2 *stw,
             const float *win, int kmax, const PkAcc &acc, int what) {
    switch (what) {
        case 6: return pk_n<N, 6>(ctx, data, h, rs, axis, stw, win, kmax, acc);
        case 7: return pk_n<N, 7>(ctx, data, h, rs, axis, stw, win, kmax, acc);
        default: return PYL_ERR_ARG;
    }
}

}  // namespace

int pk_x_what67(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
                const float *win, int kmax, const PkAcc &acc, int what) {
    const int h = n / 2 + 1;
#define CALL(N) pk_group<N>(ctx, data, h, rs, axis, tw + N, win, kmax, acc, what)
    PYL_POW2_DISPATCH(n, CALL)
#undef CALL
}

}  // namespace pyl
