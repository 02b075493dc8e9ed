// Particle deposit (mass assignment) NGP / CIC / TSC / PCS, with optional
// weights, 3D and 2D.  Replaces MAS_library.pyx:123-545 (NGP..PCSW) and the
// C kernels of MAS_c.c:8-266.
//
// Per axis the cell indices and weights follow the reference's arithmetic
// exactly where it decides which cell a particle lands in:
//   dist = pos * (dims / BoxSize)          float32 product
//   NGP: index = trunc(dist + 0.5) evaluated exactly (the reference adds 0.5
//        in double): c = trunc(dist), index = c + (dist - c >= 0.5)
//   CIC: c = trunc(dist), u = dist - c, d = 1 - u, taps c, c+1
//   TSC: minimum = floor(dist - 1.5) evaluated exactly as c - 1 - (frac < 0.5),
//        taps minimum+1..+3, diff = |float(tap) - dist|,
//        w = 0.75 - diff^2 | 0.5 (1.5 - diff)^2 | 0
//   PCS: minimum = floor(dist - 2) = c - 2, taps minimum+1..+4,
//        w = (4 - 6 d^2 + 3 d^3)/6 | (2 - d)^3 / 6 | 0
// and the tap weight is the float product ((w_x w_y) w_z) [* W], as in the
// reference.  The spline polynomials are evaluated in float32 here (the
// reference evaluates them in double and rounds to float): at most one ulp
// per weight.  Indices wrap periodically (also for inputs outside
// [0, BoxSize], where the reference's behaviour is not defined).
//
// 2D (coord = 2) follows MA's expand_dims path: the third axis has extent 1,
// index 0 and weight 1 for every tap, so a particle is deposited 2/3/4 times
// onto the same plane for CIC/TSC/PCS (and renormalised by the caller).
#include "common.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;

template <int MAS>
struct Taps { static constexpr int N = MAS == PYL_MAS_NGP ? 1 : MAS; };

__device__ __forceinline__ int wrap(int i, int dims) {
    i %= dims;
    return i < 0 ? i + dims : i;
}

template <int MAS>
__device__ __forceinline__ void axis_taps(float p, float inv, int dims, int *idx, float *w) {
    const float dist = __fmul_rn(p, inv);
    if (MAS == PYL_MAS_NGP) {
        int c = (int)dist;  // truncation, as (int) in C
        int i;
        if (dist >= 0.f) i = c + ((dist - (float)c) >= 0.5f ? 1 : 0);
        else i = (int)((double)dist + 0.5);
        idx[0] = wrap(i, dims);
        w[0] = 1.f;
    } else if (MAS == PYL_MAS_CIC) {
        const int c = (int)dist;
        const float u = dist - (float)c;
        idx[0] = wrap(c, dims);
        idx[1] = wrap(c + 1, dims);
        w[0] = 1.f - u;
        w[1] = u;
    } else if (MAS == PYL_MAS_TSC) {
        const float fl = floorf(dist);
        const int c = (int)fl;
        const int minimum = (dist - fl) < 0.5f ? c - 2 : c - 1;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int t = minimum + j + 1;
            const float diff = fabsf((float)t - dist);
            float C;
            if (diff < 0.5f) C = 0.75f - diff * diff;
            else if (diff < 1.5f) { const float q = 1.5f - diff; C = 0.5f * q * q; }
            else C = 0.f;
            idx[j] = wrap(t, dims);
            w[j] = C;
        }
    } else {  // PCS
        const int minimum = (int)floorf(dist) - 2;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int t = minimum + j + 1;
            const float diff = fabsf((float)t - dist);
            float C;
            if (diff < 1.f) C = (4.f - 6.f * diff * diff + 3.f * diff * diff * diff) / 6.f;
            else if (diff < 2.f) { const float q = 2.f - diff; C = q * q * q / 6.f; }
            else C = 0.f;
            idx[j] = wrap(t, dims);
            w[j] = C;
        }
    }
}

// One thread per particle, one global float atomic (RED) per tap.
template <int MAS, bool HAS_W, typename G>
__global__ void __launch_bounds__(kThreads)
k_deposit_atomic(const float *__restrict__ pos, long long n, int coord,
                 const float *__restrict__ W, G *__restrict__ grid, int dims,
                 float inv) {
    constexpr int NT = Taps<MAS>::N;
    const long long sy = coord == 3 ? dims : 1;
    const long long sx = sy * dims;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int ix[NT], iy[NT], iz[NT];
        float wx[NT], wy[NT], wz[NT];
        const float *p = pos + i * coord;
        axis_taps<MAS>(__ldg(p + 0), inv, dims, ix, wx);
        axis_taps<MAS>(__ldg(p + 1), inv, dims, iy, wy);
        if (coord == 3) {
            axis_taps<MAS>(__ldg(p + 2), inv, dims, iz, wz);
        } else {
#pragma unroll
            for (int j = 0; j < NT; ++j) { iz[j] = 0; wz[j] = 1.f; }
        }
        const float wt = HAS_W ? __ldg(W + i) : 1.f;
#pragma unroll
        for (int l = 0; l < NT; ++l) {
#pragma unroll
            for (int m = 0; m < NT; ++m) {
                const float wxy = wx[l] * wy[m];
                G *row = grid + ix[l] * sx + iy[m] * sy;
#pragma unroll
                for (int q = 0; q < NT; ++q) {
                    float v = wxy * wz[q];
                    if (HAS_W) v *= wt;
                    atomicAdd(row + iz[q], (G)v);
                }
            }
        }
    }
}

// g /= d elementwise (IEEE division, as numpy's `number2 /= 2.0` on float32)
template <typename G>
__global__ void k_scale(G *__restrict__ g, long long count, G d) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        g[i] = g[i] / d;
}

template <typename G>
int scale_t(pyl_ctx *ctx, G *grid, int64_t count, G s) {
    long long blocks = (count + kThreads - 1) / kThreads;
    if (blocks > 152LL * 32) blocks = 152LL * 32;
    if (blocks < 1) blocks = 1;
    k_scale<G><<<(unsigned)blocks, kThreads, 0, ctx->stream>>>(grid, count, s);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

template <int MAS, typename G>
int launch_atomic(pyl_ctx *ctx, const float *pos, long long n, int coord, const float *W,
                  G *grid, int dims, float inv) {
    long long blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 152LL * 64) blocks = 152LL * 64;
    if (blocks < 1) blocks = 1;
    if (W)
        k_deposit_atomic<MAS, true, G><<<(unsigned)blocks, kThreads, 0, ctx->stream>>>(
            pos, n, coord, W, grid, dims, inv);
    else
        k_deposit_atomic<MAS, false, G><<<(unsigned)blocks, kThreads, 0, ctx->stream>>>(
            pos, n, coord, W, grid, dims, inv);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

}  // namespace

template <typename G>
static int deposit_t(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                     G *grid, int dims, float BoxSize, int mas) {
    if (n == 0) return PYL_OK;
    // inv_cell_size = dims/BoxSize as a float division (MAS_library.pyx:135)
    const float inv = (float)dims / BoxSize;
    switch (mas) {
        case PYL_MAS_NGP: return launch_atomic<PYL_MAS_NGP>(ctx, pos, n, coord, W, grid, dims, inv);
        case PYL_MAS_CIC: return launch_atomic<PYL_MAS_CIC>(ctx, pos, n, coord, W, grid, dims, inv);
        case PYL_MAS_TSC: return launch_atomic<PYL_MAS_TSC>(ctx, pos, n, coord, W, grid, dims, inv);
        case PYL_MAS_PCS: return launch_atomic<PYL_MAS_PCS>(ctx, pos, n, coord, W, grid, dims, inv);
        default: return fail(ctx, PYL_ERR_ARG, "option not valid!!! (MAS must be NGP, CIC, TSC or PCS)");
    }
}

int deposit(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
            float *grid, int dims, float BoxSize, int mas, int flags) {
    (void)flags;
    return deposit_t(ctx, pos, n, coord, W, grid, dims, BoxSize, mas);
}

int deposit_f64(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                double *grid, int dims, float BoxSize, int mas) {
    return deposit_t(ctx, pos, n, coord, W, grid, dims, BoxSize, mas);
}

int scale_grid(pyl_ctx *ctx, float *grid, int64_t count, float s) {
    return scale_t<float>(ctx, grid, count, s);
}

int scale_grid_f64(pyl_ctx *ctx, double *grid, int64_t count, double s) {
    return scale_t<double>(ctx, grid, count, s);
}

}  // namespace pyl
