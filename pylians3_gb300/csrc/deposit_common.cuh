// Per-axis stencil of the four mass-assignment schemes, shared by the
// unsorted (global atomic) and tile-sorted (shared memory) deposits.
//
// For one coordinate, dist = pos * (dims / BoxSize) (float32 product) and
//   c = trunc(dist) for NGP/CIC, floor(dist) for TSC/PCS  ("home" cell),
// every tap lies at c + off with off in [-LO, HI]:
//   NGP: one tap at c + (frac >= 0.5)   trunc(dist + 0.5) evaluated exactly
//        (the reference adds 0.5 in double, MAS_library.pyx:290)
//   CIC: taps c, c+1 with weights 1-u, u, u = dist - c   (:151-157)
//   TSC: minimum = floor(dist - 1.5) = c - 2 + (frac >= 0.5), taps
//        minimum+1 .. minimum+3, diff = |float(tap) - dist|,
//        w = 0.75 - diff^2 | 0.5 (1.5 - diff)^2 | 0          (:391-399)
//   PCS: minimum = floor(dist - 2) = c - 2, taps minimum+1 .. minimum+4,
//        w = (4 - 6 diff^2 + 3 diff^3)/6 | (2 - diff)^3 / 6 | 0  (:484-492)
// The cell choice is exact (the reference decides it with the same float
// product and exact integer comparisons).  The NGP, CIC and TSC weights are
// the reference's float values exactly (their double steps are exact or
// rounded once); the PCS cubics are evaluated in float32 (the reference: in
// double, rounded to float), within a couple of ulps per weight.
#pragma once

#include "common.cuh"

namespace pyl {

template <int MAS>
struct Stencil {
    static constexpr int NT = MAS == PYL_MAS_NGP ? 1 : MAS;   // taps per axis
    static constexpr int LO = (MAS == PYL_MAS_TSC || MAS == PYL_MAS_PCS) ? 1 : 0;
    static constexpr int HI = MAS == PYL_MAS_NGP ? 1 : (MAS == PYL_MAS_CIC ? 1 : 2);
};

__device__ __forceinline__ int wrap_idx(int i, int dims) {
    if ((unsigned)i < (unsigned)dims) return i;   // the common, in-box case
    i %= dims;
    return i < 0 ? i + dims : i;
}

// Position in cell units.  A non-finite or absurdly large value (|dist| >=
// 1e9 cells, where the reference's int conversions overflow) is taken as 0
// so that every index computed from it stays bounded.
__device__ __forceinline__ float cell_dist(float p, float inv) {
    const float d = __fmul_rn(p, inv);
    return fabsf(d) < 1.0e9f ? d : 0.f;
}

// home cell (unwrapped) of a coordinate
template <int MAS>
__device__ __forceinline__ int home_cell(float dist) {
    if (MAS == PYL_MAS_TSC || MAS == PYL_MAS_PCS) return (int)floorf(dist);
    return (int)dist;
}

// Taps of one coordinate: off[j] (relative to the home cell) and w[j].
template <int MAS>
__device__ __forceinline__ void axis_stencil(float dist, int c, int *off, float *w) {
    if (MAS == PYL_MAS_NGP) {
        int i;
        if (dist >= 0.f) i = c + ((dist - (float)c) >= 0.5f ? 1 : 0);
        else i = (int)((double)dist + 0.5);   // outside the box: as the reference
        off[0] = i - c;
        w[0] = 1.f;
    } else if (MAS == PYL_MAS_CIC) {
        const float u = dist - (float)c;
        off[0] = 0;
        off[1] = 1;
        w[0] = 1.f - u;
        w[1] = u;
    } else if (MAS == PYL_MAS_TSC) {
        const int minimum = (dist - (float)c) < 0.5f ? c - 2 : c - 1;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int t = minimum + j + 1;
            const float diff = fabsf((float)t - dist);
            float C;
            // 0.75 - diff*diff with the product rounded first, as the reference
            // (float product, double subtraction exact here, one rounding)
            if (diff < 0.5f) C = __fsub_rn(0.75f, __fmul_rn(diff, diff));
            else if (diff < 1.5f) { const float q = 1.5f - diff; C = 0.5f * q * q; }
            else C = 0.f;
            off[j] = t - c;
            w[j] = C;
        }
    } else {  // PCS
        const int minimum = c - 2;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int t = minimum + j + 1;
            const float diff = fabsf((float)t - dist);
            float C;
            if (diff < 1.f) C = (4.f - 6.f * diff * diff + 3.f * diff * diff * diff) / 6.f;
            else if (diff < 2.f) { const float q = 2.f - diff; C = q * q * q / 6.f; }
            else C = 0.f;
            off[j] = t - c;
            w[j] = C;
        }
    }
}

// Compensated accumulation (PYL_COMPENSATED): adds v to *hi with an atomic,
// recomputes the rounded sum the atomic formed from the value it read, and
// adds the rounding error of that addition (Knuth's TwoSum) to *lo.  hi + lo
// then holds the exact sum of everything added, up to the rounding of the
// much smaller lo sums.  Works on shared and global addresses.
__device__ __forceinline__ void comp_add(float *hi, float *lo, float v) {
    const float old = atomicAdd(hi, v);
    const float s = __fadd_rn(old, v);
    const float bv = __fsub_rn(s, old);
    const float err = __fadd_rn(__fsub_rn(old, __fsub_rn(s, bv)), __fsub_rn(v, bv));
    if (err != 0.f) atomicAdd(lo, err);
}

}  // namespace pyl
