// Per-mode work of the power-spectrum pass and its per-CTA histograms,
// shared by the power-of-two and the generic kernels.  Restates the body of
// the mode loop of class Pk (library/Pk_library/Pk_library.pyx:311-378).
#pragma once

#include "common.cuh"

namespace pyl {

__device__ __forceinline__ int isqrt_dev(int v) {
    int r = (int)sqrtf((float)v);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

// Shared-memory histograms of one CTA: float32 bins updated with shared
// atomics, folded into float64 bins (owner-computes, no atomics) every few
// items, and added to the global float64 sums once at the end.
struct BinHist {
    float *h3, *h1, *hph;    // 3*(kmax+1), mid+1, kmax+1
    double *d3, *d1, *dph;
    int n3, n1, nph;

    __host__ __device__ static int count1(int mid, int what) { return (what & PYL_PK_1D) ? mid + 1 : 0; }
    __host__ __device__ static int countph(int kmax, int what) { return (what & PYL_PK_PHASE) ? kmax + 1 : 0; }
    __host__ static size_t bytes(int kmax, int mid, int what) {
        const size_t n = 3 * (size_t)(kmax + 1) + count1(mid, what) + countph(kmax, what);
        return 8 + n * (sizeof(double) + sizeof(float));
    }
    __device__ void setup(void *base, int kmax, int mid, int what) {
        uintptr_t p = ((uintptr_t)base + 7) & ~(uintptr_t)7;
        n3 = 3 * (kmax + 1);
        n1 = count1(mid, what);
        nph = countph(kmax, what);
        d3 = (double *)p;
        d1 = d3 + n3;
        dph = d1 + n1;
        h3 = (float *)(dph + nph);
        h1 = h3 + n3;
        hph = h1 + n1;
    }
    __device__ void zero_all() {
        const int n = n3 + n1 + nph;
        for (int i = threadIdx.x; i < n; i += blockDim.x) { d3[i] = 0.0; h3[i] = 0.f; }
    }
    // d += h; h = 0   (the arrays are contiguous: one loop covers all three)
    __device__ void fold() {
        const int n = n3 + n1 + nph;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const float v = h3[i];
            if (v != 0.f) { d3[i] += (double)v; h3[i] = 0.f; }
        }
    }
    __device__ void flush(const PkAcc &acc, int mid, int what) {
        for (int i = threadIdx.x; i < n3; i += blockDim.x)
            if (d3[i] != 0.0) atomicAdd(&acc.P3[i], d3[i]);
        for (int i = threadIdx.x; i < n1; i += blockDim.x)
            if (d1[i] != 0.0) atomicAdd(&acc.P1[i], d1[i]);
        for (int i = threadIdx.x; i < nph; i += blockDim.x)
            if (dph[i] != 0.0) atomicAdd(&acc.Pph[i], dph[i]);
    }
};

// The extra (non-3D) outputs of one mode: 1D and phase into the shared
// histograms, 2D into the global float64 sums.
template <int WHAT, class Hist>
__device__ __forceinline__ void mode_extras(Hist &H, const PkAcc &acc, int n2, int bin,
                                            int kpar, float re, float d2, int mid) {
    if (WHAT & PYL_PK_1D) {
        if (n2 <= mid * mid) atomicAdd(&H.h1[abs(kpar)], d2);
    }
    if (WHAT & PYL_PK_PHASE) {
        const float ph = atan2f(re, sqrtf(d2));
        atomicAdd(&H.hph[bin], ph * ph);
    }
    if (WHAT & PYL_PK_2D) {
        const int kper = isqrt_dev(n2 - kpar * kpar);
        atomicAdd(&acc.P2D[(long long)(mid + 1) * kper + abs(kpar)], (double)d2);
    }
}

// Adds a run's moments to bin b of a CTA histogram (float shared atomics: the
// warps of a CTA share it).
template <class Hist>
__device__ __forceinline__ void hist_add3(Hist &H, int b, float c0, float c1, float c2) {
    atomicAdd(&H.h3[3 * b + 0], c0);
    atomicAdd(&H.h3[3 * b + 1], c1);
    atomicAdd(&H.h3[3 * b + 2], c2);
}

// A histogram private to one warp whose flushed runs never share a bin (the
// warp's modes have monotone |k|): plain read-modify-writes.
struct WarpHist {
    float *h3;
};
template <>
__device__ __forceinline__ void hist_add3<WarpHist>(WarpHist &H, int b, float c0, float c1,
                                                    float c2) {
    H.h3[3 * b + 0] += c0;
    H.h3[3 * b + 1] += c1;
    H.h3[3 * b + 2] += c2;
}

// Runs of consecutive modes of one lane that fall into the same |k| bin:
// the sums of the current run are kept in registers.  A bin's three sums
// are the moments S0 = sum |delta|^2, S1 = sum |delta|^2 mu^2 and S2 = sum
// |delta|^2 mu^4; the Legendre sums of Pk_library.pyx:362-365 are formed
// from them in float64 when the spectrum is finalised (finalize).  The lane's
// first run (head) and its last run (tail) may continue in the neighbouring
// lanes' modes, so they are kept for the warp merge (warp_flush_runs); the
// runs in between are complete and go to the shared histogram as they close.
struct RunAcc {
    int hb = -1, cb = -1;                 // head bin, current (tail) bin; -1: none
    float h0 = 0.f, h1 = 0.f, h2 = 0.f;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    template <class Hist>
    __device__ __forceinline__ void add(Hist &H, int b, float d2, float mu2) {
        if (b != cb) {
            if (cb >= 0) {
                if (hb < 0) {
                    hb = cb;
                    h0 = c0; h1 = c1; h2 = c2;
                } else {
                    hist_add3(H, cb, c0, c1, c2);
                }
            }
            cb = b;
            c0 = c1 = c2 = 0.f;
        }
        const float t = d2 * mu2;
        c0 += d2;
        c1 += t;
        c2 = fmaf(t, mu2, c2);
    }
};

// Adds the head and tail runs of the 32 lanes of a warp to the shared
// histogram, merging runs of neighbouring lanes that share a bin first, so
// that lanes hitting one bin (along a pencil |k| often changes by less than
// one over many modes) make one set of shared atomics instead of one each.
// A segmented inclusive scan over the lanes sums the tails of each maximal
// stretch of lanes whose tails share a bin (a lane with a head run starts a
// new stretch); the last lane of a stretch also takes the next lane's head
// when its bin matches, and adds the total.  Every run is added exactly once
// whatever the bins are.  Every thread of the warp must call it (a CTA of
// fewer than 32 threads, as for 16-point lines, is one partial warp).
template <class Hist>
__device__ __forceinline__ void warp_flush_runs(Hist &H, const RunAcc &R) {
    const int lane = threadIdx.x & 31;
    const int nl = min(32, (int)blockDim.x - (int)(threadIdx.x & ~31u));   // lanes present
    const unsigned FULL = nl == 32 ? 0xffffffffu : ((1u << nl) - 1u);
    const int last = nl - 1;
    const int prev_tb = __shfl_up_sync(FULL, R.cb, 1);
    const int start = (lane == 0 || R.hb >= 0 || R.cb < 0 || R.cb != prev_tb) ? 1 : 0;
    float v0 = R.c0, v1 = R.c1, v2 = R.c2;
    int f = start;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float u0 = __shfl_up_sync(FULL, v0, d);
        const float u1 = __shfl_up_sync(FULL, v1, d);
        const float u2 = __shfl_up_sync(FULL, v2, d);
        const int uf = __shfl_up_sync(FULL, f, d);
        if (lane >= d) {
            if (!f) {
                v0 += u0;
                v1 += u1;
                v2 += u2;
            }
            f |= uf;
        }
    }
    const int next_start = __shfl_down_sync(FULL, start, 1);
    const int nb = __shfl_down_sync(FULL, R.hb, 1);
    const float n0 = __shfl_down_sync(FULL, R.h0, 1);
    const float n1 = __shfl_down_sync(FULL, R.h1, 1);
    const float n2 = __shfl_down_sync(FULL, R.h2, 1);
    if (R.cb >= 0 && (lane == last || next_start)) {
        if (lane < last && nb == R.cb) {     // the next lane's head continues this stretch
            v0 += n0;
            v1 += n1;
            v2 += n2;
        }
        hist_add3(H, R.cb, v0, v1, v2);
    }
    __syncwarp(FULL);
    if (R.hb >= 0 && !(lane > 0 && R.hb == prev_tb)) hist_add3(H, R.hb, R.h0, R.h1, R.h2);
}

// L consecutive modes kxx0 .. kxx0+L-1 of one pencil (ky, kz fixed), read
// from shared memory at ln[pad(kxx)], the window at win[pad(kxx)] (the pad
// spreads the L-strided accesses of a warp over the banks): the per-mode
// work of bin_mode, into the lane's runs R (the caller ends with
// warp_flush_runs), with the bin index updated incrementally instead of one
// square root per mode.  Between neighbours |kx| changes by one, so
// sqrt(kx^2 + ky^2 + kz^2) changes by at most one and the bin by -1, 0 or +1.
// Pencils off the kz = 0 and kz = mid planes (all but two planes) need none
// of the half-space checks and hold no DC mode: they take a branch-free body.
template <int WHAT, int L, class Hist, class Pad>
__device__ __forceinline__ void bin_run(RunAcc &R, Hist &H, const PkAcc &acc, const float2 *ln,
                                        Pad pad, int kxx0, int ky, int kz, int n, int axis,
                                        const float *win, float wyz, int mid) {
    const bool even = (n & 1) == 0;
    const bool plane = (kz == 0 || (kz == mid && even));
    const int r2 = ky * ky + kz * kz;
    const int kx0 = kxx0 > mid ? kxx0 - n : kxx0;
    int bin = isqrt_dev(kx0 * kx0 + r2);
    if (!plane) {
        const int kpar_c = axis == 1 ? ky : kz;   // kpar when it is not kx
        // |k|^2 and k_par^2 also in float, exact (< 2^24), from kxx in
        // float: no integer-to-float conversions per mode
        const float r2f = (float)r2, kpc2f = (float)(kpar_c * kpar_c);
        const float kxx0f = (float)kxx0, nf = (float)n;
#pragma unroll
        for (int i = 0; i < L; ++i) {
            const int kxx = kxx0 + i;
            const bool wrap = kxx > mid;
            const int kx = wrap ? kxx - n : kxx;
            const int n2 = kx * kx + r2;          // > 0: kz != 0 here
            bin += ((bin + 1) * (bin + 1) <= n2) - (bin * bin > n2);
            const float2 v = ln[pad(kxx)];
            const float kxf = (kxx0f + (float)i) - (wrap ? nf : 0.f);
            const float n2f = fmaf(kxf, kxf, r2f);
            const float kpar2f = axis == 0 ? kxf * kxf : kpc2f;
            const float f = win[pad(kxx)] * wyz;
            const float re = v.x * f, im = v.y * f;
            const float d2 = re * re + im * im;
            const float mu2 = __fdividef(kpar2f, n2f);
            R.add(H, bin, d2, mu2);
            if (WHAT) mode_extras<WHAT>(H, acc, n2, bin, axis == 0 ? kx : kpar_c, re, d2, mid);
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < L; ++i) {
        const int kxx = kxx0 + i;
        const int kx = kxx > mid ? kxx - n : kxx;
        const int n2 = kx * kx + r2;
        bin += ((bin + 1) * (bin + 1) <= n2) - (bin * bin > n2);
        if (kx < 0) continue;
        if ((kx == 0 || (kx == mid && even)) && ky < 0) continue;
        const float2 v = ln[pad(kxx)];
        if (n2 == 0) *acc.dc = v;
        const int kpar = axis == 0 ? kx : (axis == 1 ? ky : kz);
        const float f = win[pad(kxx)] * wyz;
        const float re = v.x * f, im = v.y * f;
        const float d2 = re * re + im * im;
        const float mu2 = n2 > 0 ? __fdividef((float)(kpar * kpar), (float)n2) : 0.f;
        R.add(H, bin, d2, mu2);
        if (WHAT) mode_extras<WHAT>(H, acc, n2, bin, kpar, re, d2, mid);
    }
}

// Float32-only shared histograms of one CTA, added to the global float64
// sums when the CTA ends (used where a CTA bins a bounded number of modes).
struct FltHist {
    float *h3, *h1, *hph;
    int n3, n1, nph;
    __host__ static size_t bytes(int kmax, int mid, int what) {
        return sizeof(float) * (3 * (size_t)(kmax + 1) + BinHist::count1(mid, what) +
                                BinHist::countph(kmax, what));
    }
    __device__ void setup(float *base, int kmax, int mid, int what) {
        n3 = 3 * (kmax + 1);
        n1 = BinHist::count1(mid, what);
        nph = BinHist::countph(kmax, what);
        h3 = base;
        h1 = h3 + n3;
        hph = h1 + n1;
    }
    __device__ void zero_all() {
        for (int i = threadIdx.x; i < n3 + n1 + nph; i += blockDim.x) h3[i] = 0.f;
    }
    __device__ void flush(const PkAcc &acc) {
        for (int i = threadIdx.x; i < n3; i += blockDim.x)
            if (h3[i] != 0.f) atomicAdd(&acc.P3[i], (double)h3[i]);
        for (int i = threadIdx.x; i < n1; i += blockDim.x)
            if (h1[i] != 0.f) atomicAdd(&acc.P1[i], (double)h1[i]);
        for (int i = threadIdx.x; i < nph; i += blockDim.x)
            if (hph[i] != 0.f) atomicAdd(&acc.Pph[i], (double)hph[i]);
    }
};

// One independent mode (kxx, ky, kz) with raw value v: Hermitian half-space
// selection (:324-327), |k| bin = floor(sqrt(kx^2 + ky^2 + kz^2)) exactly,
// window f = w(kx) w(ky) w(kz) in float32 applied to the complex64 mode
// (:351-352), |delta|^2 and the Legendre weights of mu^2 = k_par^2 / k^2
// (:355-375).  wx = w(kx), wyz = w(ky) w(kz).
template <int WHAT>
__device__ __forceinline__ void bin_mode(BinHist &H, const PkAcc &acc, float2 v, int kxx, int ky,
                                         int kz, int n, int axis, float wx, float wyz, int mid) {
    const bool even = (n & 1) == 0;
    const int kx = kxx > mid ? kxx - n : kxx;
    if (kz == 0 || (kz == mid && even)) {
        if (kx < 0) return;
        if (kx == 0 || (kx == mid && even)) {
            if (ky < 0) return;
        }
    }
    if (kx == 0 && ky == 0 && kz == 0) *acc.dc = v;
    const int n2 = kx * kx + ky * ky + kz * kz;
    const int bin = isqrt_dev(n2);
    const int kpar = axis == 0 ? kx : (axis == 1 ? ky : kz);
    const float f = wx * wyz;
    const float re = v.x * f, im = v.y * f;
    const float d2 = re * re + im * im;
    const float mu2 = n2 > 0 ? (float)(kpar * kpar) / (float)n2 : 0.f;
    atomicAdd(&H.h3[3 * bin + 0], d2);                // moments S0, S1, S2 (see RunAcc)
    atomicAdd(&H.h3[3 * bin + 1], d2 * mu2);
    atomicAdd(&H.h3[3 * bin + 2], d2 * mu2 * mu2);
    if (WHAT & PYL_PK_1D) {
        if (n2 <= mid * mid) atomicAdd(&H.h1[abs(kpar)], d2);
    }
    if (WHAT & PYL_PK_PHASE) {
        const float ph = atan2f(re, sqrtf(d2));
        atomicAdd(&H.hph[bin], ph * ph);
    }
    if (WHAT & PYL_PK_2D) {
        const int kper = isqrt_dev(n2 - kpar * kpar);
        atomicAdd(&acc.P2D[(long long)(mid + 1) * kper + abs(kpar)], (double)d2);
    }
}

}  // namespace pyl
