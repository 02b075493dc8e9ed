/*
 * CPU restatement of the Pylians3 density-field + power-spectrum hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is
 * checked against; it is compiled into oracle/_build/liborc.so and may only be
 * loaded by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py.  The product path (pylians3_gb300) never links or calls it.
 *
 * Every routine restates one reference routine (paths relative to the Pylians3
 * source tree) with the same floating-point types at each step:
 *   orc_ngp / orc_cic / orc_tsc / orc_pcs  <- library/MAS_library/MAS_library.pyx
 *        NGP :273-292, NGPW :305-325, CIC :123-166, CICW :179-216,
 *        TSC :369-404, TSCW :417-452, PCS :463-497, PCSW :510-545
 *   orc_*_d (float64 grid)                 <- NGPW_d :338-358, CICW_d :229-266
 *        (extended here to TSC/PCS for the float64 precision oracle)
 *   orc_deposit_d_omp                      the orc_*_d taps on all cores (3D),
 *        float64 atomics; for the precision oracle on large grids
 *   orc_deposit_omp                        <- library/MAS_library/MAS_c.c:8-266
 *        (OpenMP particle loop with an atomic add per tap)
 *   orc_pk_bin                             <- library/Pk_library/Pk_library.pyx:311-378
 *        (the independent-mode loop of class Pk); orc_pk_bin_mt runs its rows
 *        on all cores, orc_mode_counts its index part alone (no data)
 * Parity of this file with the compiled reference is pinned by the golden
 * vectors under tests/golden/ (generated by tests/golden/make_golden.py from
 * the reference compiled by oracle/build_ref.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Mass assignment.  pos is a C-contiguous (n, coord) float32 array, coord 2
 * or 3; for coord == 2 the grid is (dims, dims, 1) as MA's expand_dims does
 * (MAS_library.pyx:84-110) and the third axis keeps index 0 / weight 1.      */
/* ------------------------------------------------------------------------ */

#define DEPOSIT_BODY_CIC(GRID_T)                                                \
    long i;                                                                     \
    int axis;                                                                   \
    float inv_cell_size = dims / box; /* int / float -> float, :135 */         \
    float u[3] = {1.0f, 1.0f, 1.0f}, d[3] = {1.0f, 1.0f, 1.0f};                \
    int iu[3] = {0, 0, 0}, id[3] = {0, 0, 0};                                  \
    long sx = (long)dims * dz, sy = dz;                                         \
    for (i = 0; i < n; i++) {                                                   \
        float w = W ? W[i] : 1.0f;                                              \
        for (axis = 0; axis < coord; axis++) {                                  \
            float dist = pos[i * coord + axis] * inv_cell_size;                 \
            u[axis] = dist - (float)(int)dist;                                  \
            d[axis] = (float)(1.0 - (double)u[axis]);                           \
            id[axis] = ((int)dist) % dims;                                      \
            iu[axis] = (id[axis] + 1) % dims;                                   \
        }                                                                       \
        if (coord == 2) { id[2] = 0; iu[2] = 0; u[2] = 1.0f; d[2] = 1.0f; }     \
        int zu = (coord == 2) ? 0 : iu[2];                                      \
        if (W) {                                                                \
            g[id[0]*sx + id[1]*sy + id[2]] += d[0]*d[1]*d[2]*w;                 \
            g[id[0]*sx + id[1]*sy + zu]    += d[0]*d[1]*u[2]*w;                 \
            g[id[0]*sx + iu[1]*sy + id[2]] += d[0]*u[1]*d[2]*w;                 \
            g[id[0]*sx + iu[1]*sy + zu]    += d[0]*u[1]*u[2]*w;                 \
            g[iu[0]*sx + id[1]*sy + id[2]] += u[0]*d[1]*d[2]*w;                 \
            g[iu[0]*sx + id[1]*sy + zu]    += u[0]*d[1]*u[2]*w;                 \
            g[iu[0]*sx + iu[1]*sy + id[2]] += u[0]*u[1]*d[2]*w;                 \
            g[iu[0]*sx + iu[1]*sy + zu]    += u[0]*u[1]*u[2]*w;                 \
        } else {                                                                \
            g[id[0]*sx + id[1]*sy + id[2]] += d[0]*d[1]*d[2];                   \
            g[id[0]*sx + id[1]*sy + zu]    += d[0]*d[1]*u[2];                   \
            g[id[0]*sx + iu[1]*sy + id[2]] += d[0]*u[1]*d[2];                   \
            g[id[0]*sx + iu[1]*sy + zu]    += d[0]*u[1]*u[2];                   \
            g[iu[0]*sx + id[1]*sy + id[2]] += u[0]*d[1]*d[2];                   \
            g[iu[0]*sx + id[1]*sy + zu]    += u[0]*d[1]*u[2];                   \
            g[iu[0]*sx + iu[1]*sy + id[2]] += u[0]*u[1]*d[2];                   \
            g[iu[0]*sx + iu[1]*sy + zu]    += u[0]*u[1]*u[2];                   \
        }                                                                       \
    }

/* In 2D the reference passes number2 = expand_dims(number, 2) whose third
 * extent is 1 (MAS_library.pyx:85); dz is that extent (dims in 3D, 1 in 2D). */

void orc_cic(const float *pos, long n, int coord, const float *W, float *g,
             int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_CIC(float)
}

void orc_cic_d(const float *pos, long n, int coord, const float *W, double *g,
               int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_CIC(double)
}

#define DEPOSIT_BODY_NGP                                                        \
    long i;                                                                     \
    int axis;                                                                   \
    float inv_cell_size = dims / box;                                           \
    int idx[3] = {0, 0, 0};                                                     \
    long sx = (long)dims * dz, sy = dz;                                         \
    for (i = 0; i < n; i++) {                                                   \
        for (axis = 0; axis < coord; axis++) {                                  \
            /* float product, + 0.5 in double, truncation (:290) */             \
            idx[axis] = (int)((double)(pos[i * coord + axis] * inv_cell_size)   \
                              + 0.5);                                           \
            idx[axis] = (idx[axis] + dims) % dims;                              \
        }                                                                       \
        g[idx[0]*sx + idx[1]*sy + idx[2]] += W ? W[i] : 1.0f;                   \
    }

void orc_ngp(const float *pos, long n, int coord, const float *W, float *g,
             int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_NGP
}

void orc_ngp_d(const float *pos, long n, int coord, const float *W, double *g,
               int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_NGP
}

/* TSC (:369-404) and PCS (:463-497): the window is built per axis with
 * `minimum = (int)floor(dist - c)` in double, `diff = fabs(float(min+j+1) -
 * dist)` in float and the polynomial in double, rounded to float on store.  */
static inline void tsc_axis(float dist, int dims, int *index, float *C)
{
    int minimum = (int)floor((double)dist - 1.5);
    for (int j = 0; j < 3; j++) {
        index[j] = (minimum + j + 1 + dims) % dims;
        float diff = (float)fabs((double)((float)(minimum + j + 1) - dist));
        if (diff < 0.5)      C[j] = (float)(0.75 - (double)(diff * diff));
        else if (diff < 1.5) C[j] = (float)(0.5 * (1.5 - diff) * (1.5 - diff));
        else                 C[j] = 0.0f;
    }
}

static inline void pcs_axis(float dist, int dims, int *index, float *C)
{
    int minimum = (int)floor((double)dist - 2.0);
    for (int j = 0; j < 4; j++) {
        index[j] = (minimum + j + 1 + dims) % dims;
        float diff = (float)fabs((double)((float)(minimum + j + 1) - dist));
        double dd = diff;
        if (diff < 1.0)
            C[j] = (float)((4.0 - 6.0 * dd * dd + 3.0 * dd * dd * dd) / 6.0);
        else if (diff < 2.0)
            C[j] = (float)((2.0 - dd) * (2.0 - dd) * (2.0 - dd) / 6.0);
        else
            C[j] = 0.0f;
    }
}

#define DEPOSIT_BODY_SPLINE(NT, AXISFN)                                         \
    long i;                                                                     \
    int axis, l, m, q;                                                          \
    float inv_cell_size = dims / box;                                           \
    float C[3][NT];                                                             \
    int index[3][NT];                                                           \
    long sx = (long)dims * dz, sy = dz;                                         \
    for (axis = 0; axis < 3; axis++)                                            \
        for (l = 0; l < NT; l++) { C[axis][l] = 1.0f; index[axis][l] = 0; }     \
    for (i = 0; i < n; i++) {                                                   \
        for (axis = 0; axis < coord; axis++) {                                  \
            float dist = pos[i * coord + axis] * inv_cell_size;                 \
            AXISFN(dist, dims, index[axis], C[axis]);                           \
        }                                                                       \
        float w = W ? W[i] : 1.0f;                                              \
        for (l = 0; l < NT; l++)                                                \
            for (m = 0; m < NT; m++)                                            \
                for (q = 0; q < NT; q++) {                                      \
                    long o = index[0][l]*sx + index[1][m]*sy + index[2][q];     \
                    if (W) g[o] += C[0][l]*C[1][m]*C[2][q]*w;                   \
                    else   g[o] += C[0][l]*C[1][m]*C[2][q];                     \
                }                                                               \
    }

void orc_tsc(const float *pos, long n, int coord, const float *W, float *g,
             int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_SPLINE(3, tsc_axis)
}

void orc_tsc_d(const float *pos, long n, int coord, const float *W, double *g,
               int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_SPLINE(3, tsc_axis)
}

void orc_pcs(const float *pos, long n, int coord, const float *W, float *g,
             int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_SPLINE(4, pcs_axis)
}

void orc_pcs_d(const float *pos, long n, int coord, const float *W, double *g,
               int dims, float box)
{
    int dz = (coord == 3) ? dims : 1;
    DEPOSIT_BODY_SPLINE(4, pcs_axis)
}

/* ------------------------------------------------------------------------ */
/* Float64 grid deposit on all cores, 3D only (precision oracle for large
 * grids): the per-tap values of orc_ngp_d .. orc_pcs_d above, each added with
 * `#pragma omp atomic`; the result differs from the serial functions only by
 * the float64 rounding order.  mas: 1 NGP 2 CIC 3 TSC 4 PCS                */
/* ------------------------------------------------------------------------ */
void orc_deposit_d_omp(int mas, const float *pos, long n, const float *W,
                       double *g, int dims, float box, int threads)
{
    const float inv_cell_size = dims / box;
    const long sx = (long)dims * dims, sy = dims;
#ifdef _OPENMP
    if (threads < 1) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(static, 4096)
#endif
    for (long i = 0; i < n; i++) {
        const float w = W ? W[i] : 1.0f;
        float C[3][4];
        int index[3][4];
        int nt = 4;
        for (int ax = 0; ax < 3; ax++) {
            const float dist = pos[3*i+ax] * inv_cell_size;
            if (mas == 1) {
                nt = 1;
                index[ax][0] = ((int)((double)dist + 0.5) + dims) % dims;
                C[ax][0] = 1.0f;
            } else if (mas == 2) {
                nt = 2;
                C[ax][1] = dist - (float)(int)dist;
                C[ax][0] = (float)(1.0 - (double)C[ax][1]);
                index[ax][0] = ((int)dist) % dims;
                index[ax][1] = (index[ax][0] + 1) % dims;
            } else if (mas == 3) {
                nt = 3;
                tsc_axis(dist, dims, index[ax], C[ax]);
            } else {
                pcs_axis(dist, dims, index[ax], C[ax]);
            }
        }
        for (int l = 0; l < nt; l++)
            for (int m = 0; m < nt; m++)
                for (int q = 0; q < nt; q++) {
                    float v = C[0][l]*C[1][m]*C[2][q];
                    if (W) v = v * w;
#ifdef _OPENMP
#pragma omp atomic
#endif
                    g[index[0][l]*sx + index[1][m]*sy + index[2][q]] += v;
                }
    }
}

/* ------------------------------------------------------------------------ */
/* OpenMP deposit, 3D only: the reference's threaded C kernels (MAS_c.c:8-266,
 * reached through NGPc3D..PCSWc3D, MAS_library.pyx:1305-1389): a parallel
 * loop over particles with `#pragma omp atomic` on every tap (MAS_c.c:41,64).
 * Used as the timed CPU baseline of the deposit.  mas: 1 NGP 2 CIC 3 TSC 4 PCS */
/* ------------------------------------------------------------------------ */
void orc_deposit_omp(int mas, const float *pos, long n, const float *W,
                     float *g, int dims, float box, int threads)
{
    const float inv_cell_size = dims * 1.0f / box;
    const long a = (long)dims * dims, b = dims;
#ifdef _OPENMP
    if (threads < 1) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(static)
#endif
    for (long i = 0; i < n; i++) {
        float WW = W ? W[i] : 1.0f;
        if (mas == 1) {
            int idx[3];
            for (int ax = 0; ax < 3; ax++)
                idx[ax] = ((int)(pos[3*i+ax] * inv_cell_size + 0.5)) % dims;
#ifdef _OPENMP
#pragma omp atomic
#endif
            g[idx[0]*a + idx[1]*b + idx[2]] += WW;
        } else if (mas == 2) {
            float C[3][2];
            int index[3][2];
            for (int ax = 0; ax < 3; ax++) {
                float dist = pos[3*i+ax] * inv_cell_size;
                C[ax][1] = dist - (int)dist;
                C[ax][0] = 1.0f - C[ax][1];
                index[ax][0] = ((int)dist) % dims;
                index[ax][1] = (index[ax][0] + 1) % dims;
            }
            for (int l = 0; l < 2; l++)
                for (int m = 0; m < 2; m++)
                    for (int q = 0; q < 2; q++) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                        g[index[0][l]*a + index[1][m]*b + index[2][q]] +=
                            C[0][l]*C[1][m]*C[2][q]*WW;
                    }
        } else if (mas == 3) {
            float C[3][3];
            int index[3][3];
            for (int ax = 0; ax < 3; ax++)
                tsc_axis(pos[3*i+ax] * inv_cell_size, dims, index[ax], C[ax]);
            for (int l = 0; l < 3; l++)
                for (int m = 0; m < 3; m++)
                    for (int q = 0; q < 3; q++) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                        g[index[0][l]*a + index[1][m]*b + index[2][q]] +=
                            C[0][l]*C[1][m]*C[2][q]*WW;
                    }
        } else {
            float C[3][4];
            int index[3][4];
            for (int ax = 0; ax < 3; ax++)
                pcs_axis(pos[3*i+ax] * inv_cell_size, dims, index[ax], C[ax]);
            for (int l = 0; l < 4; l++)
                for (int m = 0; m < 4; m++)
                    for (int q = 0; q < 4; q++) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                        g[index[0][l]*a + index[1][m]*b + index[2][q]] +=
                            C[0][l]*C[1][m]*C[2][q]*WW;
                    }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Pk mode loop (Pk_library.pyx:311-378).  dk is the unnormalised r2c output
 * (dims, dims, dims//2+1) complex64 stored as interleaved float pairs; it is
 * read, not modified (the reference rescales it in place, :352).  Output
 * arrays are zero-initialised by the caller with the reference's sizes:
 *   k1D, Pk1D, N1D            kmax_par+1         (:292-294)
 *   Pk2D, N2D                 (kmax_par+1)*(kmax_per+1)  (:297-298)
 *   k3D, Pk3D[.,3], Pkphase, N3D   kmax+1        (:302-305)
 * `row0, row1` restrict the outer kxx loop to [row0, row1) so that the CPU
 * baseline can time a bounded sample of the loop; pass 0, dims for all.    */
/* ------------------------------------------------------------------------ */
static double mas_correction(double x, int p)
{
    return (x == 0.0) ? 1.0 : pow(x / sin(x), p);   /* :83-84 */
}

void orc_pk_bin(const float *dk, int dims, int axis, int MAS_index,
                int row0, int row1,
                double *k1D, double *Pk1D, double *N1D,
                double *Pk2D, double *N2D,
                double *k3D, double *Pk3D, double *Pkphase, double *N3D)
{
    const int middle = dims / 2;
    const int kmax_par = middle;
    const int h = middle + 1;
    const double prefact = M_PI / dims;
    double MAS_corr[3];
    for (int kxx = row0; kxx < row1; kxx++) {
        int kx = (kxx > middle) ? kxx - dims : kxx;
        MAS_corr[0] = mas_correction(prefact * kx, MAS_index);
        for (int kyy = 0; kyy < dims; kyy++) {
            int ky = (kyy > middle) ? kyy - dims : kyy;
            MAS_corr[1] = mas_correction(prefact * ky, MAS_index);
            for (int kzz = 0; kzz < middle + 1; kzz++) {
                int kz = (kzz > middle) ? kzz - dims : kzz;
                MAS_corr[2] = mas_correction(prefact * kz, MAS_index);

                /* Hermitian half-space: kz=0 and kz=middle planes, :324-327 */
                if (kz == 0 || (kz == middle && dims % 2 == 0)) {
                    if (kx < 0) continue;
                    else if (kx == 0 || (kx == middle && dims % 2 == 0)) {
                        if (ky < 0.0) continue;
                    }
                }
                double k = sqrt((double)(kx*kx + ky*ky + kz*kz));
                int k_index = (int)k;
                int k_par, k_per;
                if (axis == 0)      { k_par = kx; k_per = (int)sqrt((double)(ky*ky + kz*kz)); }
                else if (axis == 1) { k_par = ky; k_per = (int)sqrt((double)(kx*kx + kz*kz)); }
                else                { k_par = kz; k_per = (int)sqrt((double)(kx*kx + ky*ky)); }
                double mu = (k == 0) ? 0.0 : k_par / k;
                double mu2 = mu * mu;
                if (k_par < 0) k_par = -k_par;

                /* float window factor times the complex64 mode, :351-352 */
                float MAS_factor = (float)(MAS_corr[0] * MAS_corr[1] * MAS_corr[2]);
                size_t o = (((size_t)kxx * dims + kyy) * h + kzz) * 2;
                float re_f = dk[o] * MAS_factor, im_f = dk[o + 1] * MAS_factor;
                double real = re_f, imag = im_f;
                double delta2 = real * real + imag * imag;
                double phase = atan2(real, sqrt(delta2));

                if (k <= middle) {
                    k1D[k_par] += k_par;
                    Pk1D[k_par] += delta2;
                    N1D[k_par] += 1.0;
                }
                int index_2D = (kmax_par + 1) * k_per + k_par;
                Pk2D[index_2D] += delta2;
                N2D[index_2D] += 1.0;

                k3D[k_index] += k;
                Pk3D[3*k_index + 0] += delta2;
                Pk3D[3*k_index + 1] += (delta2 * (3.0 * mu2 - 1.0) / 2.0);
                Pk3D[3*k_index + 2] += (delta2 * (35.0 * mu2 * mu2 - 30.0 * mu2 + 3.0) / 8.0);
                Pkphase[k_index] += phase * phase;
                N3D[k_index] += 1.0;
            }
        }
    }
}

/* The same loop with its kxx rows split over `threads` OpenMP threads (0:
 * all cores), each summing into private arrays that are added at the end.
 * Every per-mode value is the serial loop's; only the order of the float64
 * sums differs (for large grids in tests, where the serial loop is slow).  */
void orc_pk_bin_mt(const float *dk, int dims, int axis, int MAS_index, int threads,
                   double *k1D, double *Pk1D, double *N1D,
                   double *Pk2D, double *N2D,
                   double *k3D, double *Pk3D, double *Pkphase, double *N3D)
{
    const int middle = dims / 2;
    const long n1 = middle + 1;
    const long kmax_per = (long)sqrt((double)(2L * middle * middle));
    const long kmax = (long)sqrt((double)(3L * middle * middle));
    const long n2 = n1 * (kmax_per + 1), n3 = kmax + 1;
    const long per = 3 * n1 + 2 * n2 + 6 * n3;   /* doubles per thread */
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    threads = 1;
#endif
    if (threads > dims) threads = dims;
    double *buf = (double *)calloc((size_t)threads * per, sizeof(double));
    if (!buf) return;
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static, 1)
#endif
    for (int t = 0; t < threads; t++) {
        double *b = buf + (size_t)t * per;
        const int r0 = (int)((long)dims * t / threads), r1 = (int)((long)dims * (t + 1) / threads);
        orc_pk_bin(dk, dims, axis, MAS_index, r0, r1, b, b + n1, b + 2 * n1,
                   b + 3 * n1, b + 3 * n1 + n2, b + 3 * n1 + 2 * n2,
                   b + 3 * n1 + 2 * n2 + n3, b + 3 * n1 + 2 * n2 + 4 * n3,
                   b + 3 * n1 + 2 * n2 + 5 * n3);
    }
    double *outs[9] = {k1D, Pk1D, N1D, Pk2D, N2D, k3D, Pk3D, Pkphase, N3D};
    const long lens[9] = {n1, n1, n1, n2, n2, n3, 3 * n3, n3, n3};
    for (int t = 0; t < threads; t++) {
        const double *b = buf + (size_t)t * per;
        for (int a = 0; a < 9; a++) {
            for (long i = 0; i < lens[a]; i++) outs[a][i] += b[i];
            b += lens[a];
        }
    }
    free(buf);
}

/* The index part of the mode loop alone (Pk_library.pyx:318-345, 360-378
 * without the data): per-bin mode counts N1D, N2D, N3D and the sums of k
 * (k1D, k3D), over all cores.  The float64 counts are exact integers.     */
void orc_mode_counts(int dims, int axis, int threads, double *k1D, double *N1D,
                     double *N2D, double *k3D, double *N3D)
{
    const int middle = dims / 2;
    const int kmax_par = middle;
    const long n1 = middle + 1;
    const long kmax_per = (long)sqrt((double)(2L * middle * middle));
    const long kmax = (long)sqrt((double)(3L * middle * middle));
    const long n2 = n1 * (kmax_per + 1), n3 = kmax + 1;
    const long per = 2 * n1 + n2 + 2 * n3;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    threads = 1;
#endif
    if (threads > dims) threads = dims;
    double *buf = (double *)calloc((size_t)threads * per, sizeof(double));
    if (!buf) return;
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static, 1)
#endif
    for (int t = 0; t < threads; t++) {
        double *bk1 = buf + (size_t)t * per, *bn1 = bk1 + n1, *bn2 = bn1 + n1;
        double *bk3 = bn2 + n2, *bn3 = bk3 + n3;
        const int r0 = (int)((long)dims * t / threads), r1 = (int)((long)dims * (t + 1) / threads);
        for (int kxx = r0; kxx < r1; kxx++) {
            int kx = (kxx > middle) ? kxx - dims : kxx;
            for (int kyy = 0; kyy < dims; kyy++) {
                int ky = (kyy > middle) ? kyy - dims : kyy;
                for (int kzz = 0; kzz < middle + 1; kzz++) {
                    int kz = (kzz > middle) ? kzz - dims : kzz;
                    if (kz == 0 || (kz == middle && dims % 2 == 0)) {
                        if (kx < 0) continue;
                        else if (kx == 0 || (kx == middle && dims % 2 == 0)) {
                            if (ky < 0.0) continue;
                        }
                    }
                    double k = sqrt((double)(kx*kx + ky*ky + kz*kz));
                    int k_index = (int)k;
                    int k_par, k_per;
                    if (axis == 0)      { k_par = kx; k_per = (int)sqrt((double)(ky*ky + kz*kz)); }
                    else if (axis == 1) { k_par = ky; k_per = (int)sqrt((double)(kx*kx + kz*kz)); }
                    else                { k_par = kz; k_per = (int)sqrt((double)(kx*kx + ky*ky)); }
                    if (k_par < 0) k_par = -k_par;
                    if (k <= middle) {
                        bk1[k_par] += k_par;
                        bn1[k_par] += 1.0;
                    }
                    bn2[(kmax_par + 1) * k_per + k_par] += 1.0;
                    bk3[k_index] += k;
                    bn3[k_index] += 1.0;
                }
            }
        }
    }
    for (int t = 0; t < threads; t++) {
        const double *b = buf + (size_t)t * per;
        for (long i = 0; i < n1; i++) { k1D[i] += b[i]; N1D[i] += b[n1 + i]; }
        for (long i = 0; i < n2; i++) N2D[i] += b[2 * n1 + i];
        for (long i = 0; i < n3; i++) { k3D[i] += b[2 * n1 + n2 + i]; N3D[i] += b[2 * n1 + n2 + n3 + i]; }
    }
    free(buf);
}

/* Same loop in float64 throughout for the precision oracle: dk is complex128
 * and the window is applied in double.  Rows [row0, row1) of kxx.         */
static void pk_bin_d_rows(const double *dk, int dims, int axis, int MAS_index,
                          int row0, int row1, double *k3D, double *Pk3D, double *N3D)
{
    const int middle = dims / 2;
    const int h = middle + 1;
    const double prefact = M_PI / dims;
    for (int kxx = row0; kxx < row1; kxx++) {
        int kx = (kxx > middle) ? kxx - dims : kxx;
        double c0 = mas_correction(prefact * kx, MAS_index);
        for (int kyy = 0; kyy < dims; kyy++) {
            int ky = (kyy > middle) ? kyy - dims : kyy;
            double c1 = mas_correction(prefact * ky, MAS_index);
            for (int kzz = 0; kzz < middle + 1; kzz++) {
                int kz = kzz;
                double c2 = mas_correction(prefact * kz, MAS_index);
                if (kz == 0 || (kz == middle && dims % 2 == 0)) {
                    if (kx < 0) continue;
                    else if (kx == 0 || (kx == middle && dims % 2 == 0)) {
                        if (ky < 0) continue;
                    }
                }
                double k = sqrt((double)(kx*kx + ky*ky + kz*kz));
                int k_index = (int)k;
                int k_par = (axis == 0) ? kx : (axis == 1) ? ky : kz;
                double mu = (k == 0) ? 0.0 : k_par / k;
                double mu2 = mu * mu;
                double f = c0 * c1 * c2;
                size_t o = (((size_t)kxx * dims + kyy) * h + kzz) * 2;
                double re = dk[o] * f, im = dk[o + 1] * f;
                double delta2 = re * re + im * im;
                k3D[k_index] += k;
                Pk3D[3*k_index + 0] += delta2;
                Pk3D[3*k_index + 1] += delta2 * (3.0 * mu2 - 1.0) / 2.0;
                Pk3D[3*k_index + 2] += delta2 * (35.0 * mu2 * mu2 - 30.0 * mu2 + 3.0) / 8.0;
                N3D[k_index] += 1.0;
            }
        }
    }
}

void orc_pk_bin_d(const double *dk, int dims, int axis, int MAS_index,
                  double *k3D, double *Pk3D, double *N3D)
{
    pk_bin_d_rows(dk, dims, axis, MAS_index, 0, dims, k3D, Pk3D, N3D);
}

/* orc_pk_bin_d with the kxx rows over `threads` OpenMP threads (0: all). */
void orc_pk_bin_d_mt(const double *dk, int dims, int axis, int MAS_index, int threads,
                     double *k3D, double *Pk3D, double *N3D)
{
    const int middle = dims / 2;
    const long n3 = (long)sqrt((double)(3L * middle * middle)) + 1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#else
    threads = 1;
#endif
    if (threads > dims) threads = dims;
    double *buf = (double *)calloc((size_t)threads * 5 * n3, sizeof(double));
    if (!buf) return;
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static, 1)
#endif
    for (int t = 0; t < threads; t++) {
        double *b = buf + (size_t)t * 5 * n3;
        const int r0 = (int)((long)dims * t / threads), r1 = (int)((long)dims * (t + 1) / threads);
        pk_bin_d_rows(dk, dims, axis, MAS_index, r0, r1, b, b + n3, b + 4 * n3);
    }
    for (int t = 0; t < threads; t++) {
        const double *b = buf + (size_t)t * 5 * n3;
        for (long i = 0; i < n3; i++) { k3D[i] += b[i]; N3D[i] += b[4 * n3 + i]; }
        for (long i = 0; i < 3 * n3; i++) Pk3D[i] += b[n3 + i];
    }
    free(buf);
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
