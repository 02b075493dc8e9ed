// The rows around the spectrum that reuse its FFT and mode conventions:
//   correct_MAS  Pk_library.pyx:1882-1939  (r2c, window on the independent
//                modes, c2r)
//   Pk_plane     Pk_library.pyx:435-511    (2D r2c, window, |k| bins) with
//                FFT2Dr_f / IFFT2Dr_f       Pk_library.pyx:181-228
//   CIC_interp   MAS_library.pyx:558-599   (gather of a grid at positions)
//   pos_redshift_space  redshift_space_library.pyx:29-50 (the RSD shift of
//                the snapshot driver, Pk_snapshot.py:63-67)
#include <math.h>
#include <string.h>

#include <mutex>
#include <tuple>

#include "pk_common.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;

// correct_MAS: every independent mode of the (d, d, rs) half grid times
// float(w(kx) * w(ky) * w(kz)), the product formed in double and rounded
// once to float as the reference's `cdef float MAS_factor`.  The modes its
// loop skips (the redundant halves of the kz = 0 and kz = d/2 planes) are
// left as they are; the c2r that follows reads them as the reference's does.
__global__ void k_correct_mas(float2 *__restrict__ data, int d, int h, int rs,
                              const double *__restrict__ wd) {
    const int mid = d / 2;
    const bool even = (d & 1) == 0;
    const long long total = (long long)d * d * h;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < total;
         m += (long long)gridDim.x * blockDim.x) {
        const int kzz = (int)(m % h);
        const long long row = m / h;
        const int kyy = (int)(row % d), kxx = (int)(row / d);
        const int kx = kxx > mid ? kxx - d : kxx;
        const int ky = kyy > mid ? kyy - d : kyy;
        if (kzz == 0 || (kzz == mid && even)) {
            if (kx < 0) continue;
            if ((kx == 0 || (kx == mid && even)) && ky < 0) continue;
        }
        const float f = (float)(wd[kxx] * wd[kyy] * wd[kzz]);
        float2 *p = data + ((long long)kxx * d + kyy) * rs + kzz;
        float2 v = *p;
        v.x = v.x * f;
        v.y = v.y * f;
        *p = v;
    }
}

// Pk_plane binning: a CTA bins kPlaneChunk consecutive modes of the (g, rs)
// half plane into float64 shared bins (the reference sums |delta|^2 in
// double), added to the global sums when it ends.
constexpr int kPlaneChunk = 8192;

__global__ void __launch_bounds__(kThreads)
k_pk_plane(const float2 *__restrict__ data, int g, int h, int rs,
           const double *__restrict__ wd, int kmax, double *__restrict__ P) {
    extern __shared__ double s_bins[];
    for (int b = threadIdx.x; b <= kmax; b += blockDim.x) s_bins[b] = 0.0;
    __syncthreads();
    const int mid = g / 2;
    const bool even = (g & 1) == 0;
    const long long total = (long long)g * h;
    const long long m0 = (long long)blockIdx.x * kPlaneChunk;
    const long long m1 = min(total, m0 + kPlaneChunk);
    for (long long m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
        const int kyy = (int)(m % h), kxx = (int)(m / h);
        const int kx = kxx > mid ? kxx - g : kxx;
        const int ky = kyy;   // kyy in [0, middle]
        if ((ky == 0 || (ky == mid && even)) && kx < 0) continue;
        const int bin = isqrt_dev(kx * kx + ky * ky);
        const float f = (float)(wd[kxx] * wd[kyy]);
        const float2 v = data[(long long)kxx * rs + kyy];
        const double re = (double)(v.x * f), im = (double)(v.y * f);
        atomicAdd(&s_bins[bin], re * re + im * im);
    }
    __syncthreads();
    for (int b = threadIdx.x; b <= kmax; b += blockDim.x)
        if (s_bins[b] != 0.0) atomicAdd(&P[b], s_bins[b]);
}

// CIC_interp: the eight-cell trilinear gather, float32 throughout in the
// reference's order (products left to right, the eight terms summed left to
// right; no fused multiply-adds).
__global__ void __launch_bounds__(kThreads)
k_cic_interp(const float *__restrict__ grid, int dims, float inv,
             const float *__restrict__ pos, long long n, float *__restrict__ den) {
    const long long sx = (long long)dims * dims, sy = dims;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float u[3], d[3];
        long long id[3], iu[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float dist = __fmul_rn(__ldg(pos + 3 * i + a), inv);
            if (!(fabsf(dist) < 1.0e9f)) dist = 0.f;   // keeps every index bounded
            const int c = (int)dist;
            u[a] = __fsub_rn(dist, (float)c);
            d[a] = __fsub_rn(1.0f, u[a]);
            // C remainder as the reference; a negative remainder (positions
            // below 0, out of bounds there) is wrapped into the grid
            int lo = c % dims;
            if (lo < 0) lo += dims;
            id[a] = lo;
            iu[a] = (lo + 1) % dims;
        }
        auto g = [&](long long x, long long y, long long z) {
            return __ldg(grid + x * sx + y * sy + z);
        };
        auto t = [&](float v, float a, float b, float c) {
            return __fmul_rn(__fmul_rn(__fmul_rn(v, a), b), c);
        };
        float s = t(g(id[0], id[1], id[2]), d[0], d[1], d[2]);
        s = __fadd_rn(s, t(g(id[0], id[1], iu[2]), d[0], d[1], u[2]));
        s = __fadd_rn(s, t(g(id[0], iu[1], id[2]), d[0], u[1], d[2]));
        s = __fadd_rn(s, t(g(id[0], iu[1], iu[2]), d[0], u[1], u[2]));
        s = __fadd_rn(s, t(g(iu[0], id[1], id[2]), u[0], d[1], d[2]));
        s = __fadd_rn(s, t(g(iu[0], id[1], iu[2]), u[0], d[1], u[2]));
        s = __fadd_rn(s, t(g(iu[0], iu[1], id[2]), u[0], u[1], d[2]));
        s = __fadd_rn(s, t(g(iu[0], iu[1], iu[2]), u[0], u[1], u[2]));
        den[i] = s;
    }
}

// pos_redshift_space (redshift_space_library.pyx:29-50): along `axis`,
// s = r + v (1 + z) / H(z), then wrapped into [0, BoxSize]: BoxSize is added
// while s < 0 (particles that crossed the box several times), and s above
// BoxSize is replaced by fmod(s, BoxSize); float32 steps as written (no
// fused multiply-add).  The loop of additions is bounded: past 1024 box
// lengths below 0 the wrap is done with fmod instead.
__global__ void __launch_bounds__(kThreads)
k_rsd(float *__restrict__ pos, const float *__restrict__ vel, long long n, float box,
      float factor, int axis) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float p = __fadd_rn(pos[3 * i + axis], __fmul_rn(vel[3 * i + axis], factor));
        int it = 0;
        while (p < 0.f && it < 1024) {
            p = __fadd_rn(p, box);
            ++it;
        }
        if (p < 0.f) {
            p = fmodf(p, box);
            if (p < 0.f) p = __fadd_rn(p, box);
        }
        if (p > box) p = fmodf(p, box);
        pos[3 * i + axis] = p;
    }
}

unsigned grid_for(long long work) {
    long long b = (work + kThreads - 1) / kThreads;
    if (b > 152LL * 32) b = 152LL * 32;
    if (b < 1) b = 1;
    return (unsigned)b;
}

// Per-axis MAS_correction(pi k / d, p) in double (index i -> k = i or i - d).
std::mutex g_wd_mu;
std::map<std::tuple<int, int, int>, double *> g_wd;

const double *window_table_d(pyl_ctx *ctx, int dims, int mas, int *status) {
    if (mas < 1 || mas > 4) mas = 0;
    const auto key = std::make_tuple(ctx->device, dims, mas);
    std::lock_guard<std::mutex> lock(g_wd_mu);
    auto it = g_wd.find(key);
    if (it != g_wd.end()) return it->second;
    std::vector<double> w(dims);
    const int middle = dims / 2;
    const double prefact = M_PI / dims;
    for (int i = 0; i < dims; ++i) {
        const int k = i > middle ? i - dims : i;
        const double x = prefact * k;
        w[i] = (x == 0.0) ? 1.0 : pow(x / sin(x), mas);
    }
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * dims);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "window table"); return nullptr; }
    e = cudaMemcpy(d, w.data(), sizeof(double) * dims, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "window upload"); return nullptr; }
    g_wd[key] = d;
    return d;
}

// Copies n bytes to a device workspace unless the pointer already is one.
template <typename T>
const T *stage_in(pyl_ctx *ctx, const T *p, size_t count, bool dev, const char *name,
                  int *status) {
    if (dev) return p;
    T *d = (T *)ws_get(ctx, name, sizeof(T) * count, status);
    if (!d) return nullptr;
    cudaError_t e = cudaMemcpyAsync(d, p, sizeof(T) * count, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) { *status = cuda_fail(ctx, e, "stage in"); return nullptr; }
    return d;
}

}  // namespace

}  // namespace pyl

using namespace pyl;

extern "C" {

int pyl_correct_mas(pyl_ctx *ctx, const float *delta, float *out, int dims, int mas, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (dims < 2 || !delta || !out) return fail(ctx, PYL_ERR_ARG, "bad correct_MAS arguments");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool dev = flags & PYL_DEVICE_PTRS;
    const int h = dims / 2 + 1;
    const int rs = half_stride(dims);
    const long long cells = (long long)dims * dims * dims;
    int st = PYL_OK;
    const float *din = stage_in(ctx, delta, (size_t)cells, dev, "cm_in", &st);
    if (!din) return st;
    float2 *half = (float2 *)ws_get(ctx, "cm_half", sizeof(float2) * (size_t)dims * dims * rs, &st);
    if (!half) return st;
    const double *wd = window_table_d(ctx, dims, mas, &st);
    if (!wd) return st;
    float *dout = out;
    if (!dev) {
        dout = (float *)ws_get(ctx, "cm_out", sizeof(float) * (size_t)cells, &st);
        if (!dout) return st;
    }
    if ((st = fft_rows_r2c(ctx, din, half, (long long)dims * dims, dims, rs))) return st;
    if ((st = fft_axis_c2c(ctx, half, dims, h, rs, 1, -1))) return st;
    if ((st = fft_axis_c2c(ctx, half, dims, h, rs, 0, -1))) return st;
    k_correct_mas<<<grid_for((long long)dims * dims * h), kThreads, 0, ctx->stream>>>(
        half, dims, h, rs, wd);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    if ((st = fft_axis_c2c(ctx, half, dims, h, rs, 0, +1))) return st;
    if ((st = fft_axis_c2c(ctx, half, dims, h, rs, 1, +1))) return st;
    const double norm = 1.0 / ((double)dims * dims * dims);
    if ((st = fft_rows_c2r(ctx, half, dout, (long long)dims * dims, dims, rs, (float)norm)))
        return st;
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)cells,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        return status_check(ctx);
    }
    return PYL_OK;
}

int pyl_fft2_r2c(pyl_ctx *ctx, const float *in, float *out, int grid, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (grid < 2 || !in || !out) return fail(ctx, PYL_ERR_ARG, "bad FFT2D arguments");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool dev = flags & PYL_DEVICE_PTRS;
    const int h = grid / 2 + 1;
    int st = PYL_OK;
    const float *din = stage_in(ctx, in, (size_t)grid * grid, dev, "f2_in", &st);
    if (!din) return st;
    float2 *dout = reinterpret_cast<float2 *>(out);
    if (!dev) {
        dout = (float2 *)ws_get(ctx, "f2_cplx", sizeof(float2) * (size_t)grid * h, &st);
        if (!dout) return st;
    }
    if ((st = fft_rows_r2c(ctx, din, dout, grid, grid, h))) return st;
    if ((st = fft_plane_c2c(ctx, dout, grid, h, h, -1))) return st;
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(out, dout, sizeof(float2) * (size_t)grid * h,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        return status_check(ctx);
    }
    return PYL_OK;
}

int pyl_fft2_c2r(pyl_ctx *ctx, const float *in, float *out, int grid, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (grid < 2 || !in || !out) return fail(ctx, PYL_ERR_ARG, "bad FFT2D arguments");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool dev = flags & PYL_DEVICE_PTRS;
    const int h = grid / 2 + 1;
    int st = PYL_OK;
    // the input is not modified: transform a copy
    float2 *work = (float2 *)ws_get(ctx, "f2_work", sizeof(float2) * (size_t)grid * h, &st);
    if (!work) return st;
    PYL_CUDA(ctx, cudaMemcpyAsync(work, in, sizeof(float2) * (size_t)grid * h,
                                  dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  ctx->stream));
    float *dout = out;
    if (!dev) {
        dout = (float *)ws_get(ctx, "f2_real", sizeof(float) * (size_t)grid * grid, &st);
        if (!dout) return st;
    }
    if ((st = fft_plane_c2c(ctx, work, grid, h, h, +1))) return st;
    const double norm = 1.0 / ((double)grid * grid);
    if ((st = fft_rows_c2r(ctx, work, dout, grid, grid, h, (float)norm))) return st;
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(out, dout, sizeof(float) * (size_t)grid * grid,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        return status_check(ctx);
    }
    return PYL_OK;
}

int pyl_pk_plane(pyl_ctx *ctx, const float *delta, int grid, double BoxSize, int mas, double *k,
                 double *Pk, double *Nmodes, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (grid < 2 || !delta) return fail(ctx, PYL_ERR_ARG, "bad Pk_plane arguments");
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool dev = flags & PYL_DEVICE_PTRS;
    const int h = grid / 2 + 1;
    const int rs = half_stride(grid);
    const int middle = grid / 2;
    const int kmax = isqrt_host(2LL * middle * middle);
    int st = PYL_OK;
    const float *din = stage_in(ctx, delta, (size_t)grid * grid, dev, "pp_in", &st);
    if (!din) return st;
    float2 *half = (float2 *)ws_get(ctx, "pp_half", sizeof(float2) * (size_t)grid * rs, &st);
    if (!half) return st;
    double *P = (double *)ws_get(ctx, "pp_sums", sizeof(double) * (size_t)(kmax + 1), &st);
    if (!P) return st;
    const double *wd = window_table_d(ctx, grid, mas, &st);
    if (!wd) return st;
    PYL_CUDA(ctx, cudaMemsetAsync(P, 0, sizeof(double) * (size_t)(kmax + 1), ctx->stream));
    if ((st = fft_rows_r2c(ctx, din, half, grid, grid, rs))) return st;
    if ((st = fft_plane_c2c(ctx, half, grid, h, rs, -1))) return st;
    const long long total = (long long)grid * h;
    const size_t smem = sizeof(double) * (size_t)(kmax + 1);
    if (smem > 200 * 1024) return fail(ctx, PYL_ERR_UNSUPPORTED, "Pk_plane grid too large");
    if (smem > 40 * 1024)
        PYL_CUDA(ctx, cudaFuncSetAttribute(k_pk_plane, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
    k_pk_plane<<<(unsigned)((total + kPlaneChunk - 1) / kPlaneChunk), kThreads, smem,
                 ctx->stream>>>(half, grid, h, rs, wd, kmax, P);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    std::vector<double> sums(kmax + 1);
    PYL_CUDA(ctx, cudaMemcpyAsync(sums.data(), P, sizeof(double) * (size_t)(kmax + 1),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    // mode counts and sum of |k| per bin, in the reference's loop order
    std::vector<double> N(kmax + 1, 0.0), ksum(kmax + 1, 0.0);
    const bool even = (grid % 2) == 0;
    for (int kxx = 0; kxx < grid; ++kxx) {
        const int kx = kxx > middle ? kxx - grid : kxx;
        for (int kyy = 0; kyy <= middle; ++kyy) {
            const int ky = kyy;
            if ((ky == 0 || (ky == middle && even)) && kx < 0) continue;
            const double kk = sqrt((double)(kx * kx + ky * ky));
            const int b = (int)kk;
            ksum[b] += kk;
            N[b] += 1.0;
        }
    }
    if ((st = status_check(ctx))) return st;
    double total_modes = 0.0;
    for (double v : N) total_modes += v;
    const long long own = even ? 4 : 1;
    const long long expected = ((long long)grid * grid - own) / 2 + own;
    if ((long long)total_modes != expected) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "WARNING: Not all modes counted: counted %lld independent modes, expected %lld",
                 (long long)total_modes, expected);
        return fail(ctx, PYL_ERR_MODES, buf);
    }
    const double kF = 2.0 * M_PI / BoxSize;
    const double unit = pow(BoxSize / ((double)grid * grid), 2);
    for (int b = 1; b <= kmax; ++b) {
        if (k) k[b - 1] = (ksum[b] / N[b]) * kF;
        if (Pk) Pk[b - 1] = (sums[b] / N[b]) * unit;
        if (Nmodes) Nmodes[b - 1] = N[b];
    }
    return PYL_OK;
}

int pyl_rsd(pyl_ctx *ctx, float *pos, const float *vel, int64_t n, float BoxSize, float Hubble,
            float redshift, int axis, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (n < 0 || axis < 0 || axis > 2 || (n > 0 && (!pos || !vel)))
        return fail(ctx, PYL_ERR_ARG, "bad pos_redshift_space arguments");
    if (n == 0) return PYL_OK;
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool dev = flags & PYL_DEVICE_PTRS;
    int st = PYL_OK;
    float *dp = pos;
    if (!dev) {
        dp = (float *)ws_get(ctx, "rsd_pos", sizeof(float) * 3 * (size_t)n, &st);
        if (!dp) return st;
        PYL_CUDA(ctx, cudaMemcpyAsync(dp, pos, sizeof(float) * 3 * (size_t)n,
                                      cudaMemcpyHostToDevice, ctx->stream));
    }
    const float *dv = stage_in(ctx, vel, (size_t)n * 3, dev, "rsd_vel", &st);
    if (!dv) return st;
    // factor = (1.0 + redshift) / Hubble in double, stored as float (:34)
    const float factor = (float)((1.0 + (double)redshift) / (double)Hubble);
    k_rsd<<<grid_for(n), kThreads, 0, ctx->stream>>>(dp, dv, n, BoxSize, factor, axis);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(pos, dp, sizeof(float) * 3 * (size_t)n,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        return status_check(ctx);
    }
    return PYL_OK;
}

int pyl_cic_interp(pyl_ctx *ctx, const float *density, int dims, float BoxSize, const float *pos,
                   int64_t n, float *den, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (dims < 1 || n < 0 || (n > 0 && (!density || !pos || !den)))
        return fail(ctx, PYL_ERR_ARG, "bad CIC_interp arguments");
    if (n == 0) return PYL_OK;
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool dev = flags & PYL_DEVICE_PTRS;
    int st = PYL_OK;
    const long long cells = (long long)dims * dims * dims;
    const float *dg = stage_in(ctx, density, (size_t)cells, dev, "ci_grid", &st);
    if (!dg) return st;
    const float *dp = stage_in(ctx, pos, (size_t)n * 3, dev, "ci_pos", &st);
    if (!dp) return st;
    float *dd = den;
    if (!dev) {
        dd = (float *)ws_get(ctx, "ci_den", sizeof(float) * (size_t)n, &st);
        if (!dd) return st;
    }
    // inv_cell_size = dims/BoxSize (int / float, MAS_library.pyx:573)
    const float inv = (float)dims / BoxSize;
    k_cic_interp<<<grid_for(n), kThreads, 0, ctx->stream>>>(dg, dims, inv, dp, n, dd);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    if (!dev) {
        PYL_CUDA(ctx, cudaMemcpyAsync(den, dd, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        return status_check(ctx);
    }
    return PYL_OK;
}

}  // extern "C"
