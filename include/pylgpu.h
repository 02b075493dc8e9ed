/*
 * pylgpu.h -- C ABI of libpylgpu.so, the GB300 (sm_103a) implementation of
 * Pylians3's density-field + power-spectrum hot path.
 *
 * Conventions
 *   - Every entry point returns 0 (PYL_OK) or a negative pyl_status; no
 *     exception or exit() crosses the ABI.  pyl_last_error() gives the text.
 *   - Plain pointers and sizes only.  With PYL_DEVICE_PTRS the array
 *     arguments are device pointers (e.g. torch CUDA tensors, zero copy);
 *     otherwise they are host pointers (pinned host memory copies fastest,
 *     see pyl_host_alloc) and the library stages them through device memory.
 *   - Arrays are C-contiguous: positions (n, coord) float32, grids
 *     (dims, dims, dims) float32 (2D: (dims, dims)), spectra float64.
 *   - Work is issued on the context's stream.  Calls with host outputs return
 *     after the results are on the host; calls with device outputs return
 *     once the work is enqueued (pyl_synchronize waits for it).
 *   - A context is used by one host thread at a time; concurrent requests
 *     use one context each (pyl_pk_particles_enqueue / pyl_pk_collect).
 *
 * The reference interface each entry point replaces is cited beside it,
 * as path:line in the Pylians3 source tree.
 */
#ifndef PYLGPU_H
#define PYLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PYL_OK = 0,
    PYL_ERR_ARG = -1,         /* bad argument (shape, MAS, size)            */
    PYL_ERR_CUDA = -2,        /* a CUDA runtime call failed                  */
    PYL_ERR_OOM = -3,         /* device or pinned allocation failed          */
    PYL_ERR_MODES = -4,       /* mode-count self check failed (Pk :87-99)    */
    PYL_ERR_TIMEOUT = -5,     /* a bounded wait gave up                      */
    PYL_ERR_BUDGET = -6,      /* request larger than the HBM budget          */
    PYL_ERR_UNSUPPORTED = -7, /* size or option this build does not handle   */
    PYL_ERR_STATE = -8        /* call made in the wrong state                */
} pyl_status;

/* Mass-assignment schemes; the numbering is the reference's MAS_index
 * (library/Pk_library/Pk_library.pyx:72-78): anything else = no window.  */
enum { PYL_MAS_NONE = 0, PYL_MAS_NGP = 1, PYL_MAS_CIC = 2, PYL_MAS_TSC = 3,
       PYL_MAS_PCS = 4 };

/* flags */
#define PYL_DEVICE_PTRS  0x01  /* array arguments are device pointers          */
#define PYL_COMPENSATED  0x02  /* deposit: two-sum compensated accumulation    */
#define PYL_DEPOSIT_ATOMIC 0x04 /* deposit: force the unsorted global-atomic path */
#define PYL_DEPOSIT_SORTED 0x08 /* deposit: force the tile-sorted shared path  */
/* The tile sort picks, on the device, one pass with per-tile global cursors
 * for spatially coherent input order, two staged partition passes
 * otherwise; these flags force one of them.                                */
#define PYL_SORT_TWO_PASS  0x10
#define PYL_SORT_FRONTIER  0x20
/* The tile-sorted NGP/CIC/TSC deposit of unit-weight particles accumulates
 * each tile in 32-bit fixed point: each tap is rounded once to a scale
 * chosen per tile from its densest region (so that no cell can overflow),
 * and the tile's sums are then exact.  This flag keeps float32 shared
 * atomics instead (always used for PCS and for weighted particles).        */
#define PYL_DEPOSIT_FLOAT  0x40
/* pyl_pk_batch: issue the requests directly instead of through the cached
 * CUDA graph (the same work, launch by launch).                           */
#define PYL_NO_GRAPH       0x80
/* pyl_pk_particles: sort with the exact counting sort even where the
 * previous request of the same kind would allow the count-free one (see
 * pyl_ctx_last_sort).                                                     */
#define PYL_SORT_EXACT     0x100

/* Which Pk outputs to compute (bit mask); the 3D multipoles always are.   */
#define PYL_PK_3D     0x00
#define PYL_PK_1D     0x01     /* k1D, Pk1D, Nmodes1D                        */
#define PYL_PK_2D     0x02     /* kpar, kper, Pk2D, Nmodes2D                 */
#define PYL_PK_PHASE  0x04     /* Pkphase                                    */
#define PYL_PK_ALL    0x07

typedef struct pyl_ctx pyl_ctx;

/* ---------------------------------------------------------------- context */
/* device: CUDA ordinal; stream: a cudaStream_t to issue on, or NULL for a
 * stream owned by the context.                                             */
int pyl_ctx_create(pyl_ctx **out, int device, void *stream);
int pyl_ctx_destroy(pyl_ctx *ctx);
int pyl_ctx_set_stream(pyl_ctx *ctx, void *stream);
/* The cudaStream_t the context issues on.                                  */
int pyl_ctx_get_stream(const pyl_ctx *ctx, void **stream);
int pyl_synchronize(pyl_ctx *ctx);
const char *pyl_last_error(const pyl_ctx *ctx);
/* Device bytes currently held by the context's workspaces and plans.      */
int pyl_ctx_workspace_bytes(const pyl_ctx *ctx, size_t *bytes);
/* Free cached workspaces and plans (they are rebuilt on demand).          */
int pyl_ctx_trim(pyl_ctx *ctx);
/* Number of kernel launches this context has issued (for accounting).     */
int pyl_ctx_launch_count(const pyl_ctx *ctx, int64_t *count);
/* The tile sort of the last collected pyl_pk_particles request (no
 * reference counterpart; for tests and tuning): *count_free = 1 when it ran
 * without a counting pass (fixed slots sized from the previous request of
 * the same dims, scheme and weighting), 0 for the exact counting sort, -1
 * when the deposit was not sorted; *spilled = particles that overflowed
 * their slots and were added by a global-atomic deposit instead (the next
 * request of that kind then takes the exact sort).                         */
int pyl_ctx_last_sort(const pyl_ctx *ctx, int *count_free, unsigned *spilled);
/* Stage timing with CUDA events on the context stream (off by default).
 * pyl_ctx_stage_times waits for recorded events, writes the accumulated
 * milliseconds and launch counts of the first n stages (names from
 * pyl_stage_name) and returns the number of stages; reset != 0 clears them. */
int pyl_ctx_set_timing(pyl_ctx *ctx, int on);
int pyl_ctx_stage_times(pyl_ctx *ctx, double *ms, int64_t *counts, int n, int reset);
const char *pyl_stage_name(int stage);

/* Pinned host memory (cudaHostAlloc) for fast host<->device staging.     */
int pyl_host_alloc(void **ptr, size_t bytes);
int pyl_host_free(void *ptr);

/* ------------------------------------------------------ mass assignment */
/* Deposit n particles onto grid with scheme mas, ACCUMULATING into grid
 * (grid += ...), as MA does.  coord = 3: grid (dims,dims,dims);
 * coord = 2: grid (dims,dims) -- the reference's expand_dims path -- and,
 * when renormalize_2D != 0, the whole grid is then divided by 2/3/4 for
 * CIC/TSC/PCS.  W (nullable) holds one weight per particle.
 * Replaces: MA            library/MAS_library/MAS_library.pyx:57-112
 *           NGP..PCSW     library/MAS_library/MAS_library.pyx:123-545
 *           NGP..PCS (C)  library/MAS_library/MAS_c.h:3-10 (MAS_c.c:8-266) */
int pyl_ma(pyl_ctx *ctx, const float *pos, int64_t n, int coord,
           const float *W, float *grid, int dims, float BoxSize, int mas,
           int renormalize_2D, int flags);

/* Same deposit into a float64 grid (accumulated with float64 atomics; the
 * per-tap weight is still the float32 product, as in the reference).
 * Replaces: NGPW_d        library/MAS_library/MAS_library.pyx:338-358
 *           CICW_d        library/MAS_library/MAS_library.pyx:229-266
 * (any scheme and coord are accepted; renormalize_2D as pyl_ma).          */
int pyl_ma_f64(pyl_ctx *ctx, const float *pos, int64_t n, int coord,
               const float *W, double *grid, int dims, float BoxSize, int mas,
               int renormalize_2D, int flags);

/* ----------------------------------------------------------------- FFTs */
/* r2c over all three axes, unnormalised; out is (dims,dims,dims/2+1)
 * complex64 (interleaved float pairs).
 * Replaces: FFT3Dr_f  library/Pk_library/Pk_library.pyx:117-130          */
int pyl_fft_r2c(pyl_ctx *ctx, const float *in, float *out, int dims, int flags);
/* c2r over all three axes, normalised by 1/dims^3 (pyFFTW's default).
 * Replaces: IFFT3Dr_f library/Pk_library/Pk_library.pyx:149-162          */
int pyl_fft_c2r(pyl_ctx *ctx, const float *in, float *out, int dims, int flags);

/* -------------------------------------------------------- power spectrum */
/* Output arrays, finalised exactly as class Pk leaves them (DC bin dropped,
 * units applied, :384-418).  Sizes, with middle = dims/2:
 *   kmax     = int(sqrt(3*middle^2)), kmax_par = middle,
 *   kmax_per = int(sqrt(2*middle^2))
 *   k3D, Nmodes3D, Pkphase : kmax entries;  Pk : kmax*3 (row-major [k][ell])
 *   k1D, Pk1D, Nmodes1D    : kmax_par entries
 *   kpar, kper, Pk2D, Nmodes2D : (kmax_par+1)*(kmax_per+1) entries
 * Pointers of outputs not requested by `what` may be NULL.  All host memory. */
typedef struct {
    double *k3D, *Pk, *Nmodes3D;
    double *k1D, *Pk1D, *Nmodes1D;
    double *kpar, *kper, *Pk2D, *Nmodes2D;
    double *Pkphase;
} pyl_pk_out;

/* Sizes of the output arrays for a grid of dims^3.                         */
int pyl_pk_sizes(int dims, int *kmax, int *kmax_par, int *kmax_per);

/* Power spectrum of an overdensity grid delta (dims^3 float32; not modified).
 * mas is the window to deconvolve (PYL_MAS_*; other values: none).  axis is
 * the line of sight (0, 1, 2; other values behave as 2, as in the
 * reference).  Returns PYL_ERR_MODES when the mode count check fails.
 * Replaces: class Pk  library/Pk_library/Pk_library.pyx:263-418          */
int pyl_pk(pyl_ctx *ctx, const float *delta, int dims, double BoxSize,
           int axis, int mas, int what, pyl_pk_out *out, int flags);

/* Particles to spectrum in one call: zero a resident grid, deposit with
 * mas_deposit, form delta = rho/mean - 1 (mean = grid mean, as the
 * reference's callers compute it), and run Pk with window mas_window.  The
 * overdensity step is folded into the spectrum (P(k!=0) of rho/mean - 1 is
 * P(k) of rho divided by mean^2) so no extra pass over the grid is made.
 * Replaces the canonical caller Pk_comp
 *           library/Pk_library/Pk_snapshot.py:81-89
 * (MA -> delta/=mean; delta-=1 -> Pk).                                    */
int pyl_pk_particles(pyl_ctx *ctx, const float *pos, int64_t n,
                     const float *W, int dims, float BoxSize, int mas_deposit,
                     int axis, int mas_window, int what, pyl_pk_out *out,
                     int flags);

/* The same request split in two, for overlapping requests (one context per
 * request in flight, each on its own stream):
 *   enqueue -- issues all device work and the copy of the raw sums into
 *              context-owned pinned memory, and returns at once (host
 *              positions should then be pinned for the copy to be async);
 *   query   -- 1 when the request has finished, 0 while in flight;
 *   collect -- waits (timeout_ms >= 0 bounds the wait: PYL_ERR_TIMEOUT leaves
 *              the request in flight; < 0 waits without bound) and writes the
 *              finalised spectra into out.
 * PYL_ERR_STATE: enqueue with a request already in flight, or query/collect
 * without one.                                                             */
int pyl_pk_particles_enqueue(pyl_ctx *ctx, const float *pos, int64_t n,
                             const float *W, int dims, float BoxSize,
                             int mas_deposit, int axis, int mas_window,
                             int what, int flags);
int pyl_pk_query(pyl_ctx *ctx);
int pyl_pk_collect(pyl_ctx *ctx, pyl_pk_out *out, int timeout_ms);

/* Power spectrum of a device grid without allocating device memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- a host application whose pool allocator owns the whole
 * device, a plugin host that forbids allocations outside its allocator, or
 * a latency-critical loop where cudaMalloc/cudaFree would synchronise the
 * device.  Same arguments and outputs as pyl_pk, except: delta must be a
 * device pointer; dims must be a power of two in [16, 128], other sizes
 * return PYL_ERR_UNSUPPORTED.  All intermediates live in one fixed 12 MiB
 * array of device memory inside the library, which every GPU that loads the
 * library holds until the process exits.  The first call on a device looks
 * up that array's address (make it before any stream capture).  Calls share
 * the array and it keeps the last call's contents (the sums are cleared on
 * every call; the FFT and window tables of the last dims and scheme are
 * kept, so a call repeating them uploads nothing); calls that overlap on the
 * GPU race, so issue them one after another.  The call itself allocates no
 * device memory.  The context does once, when it is created: a 16-byte
 * device status word (and a stream unless the caller passes one), so create
 * it before the region where allocation is not allowed.                   */
int pyl_pk_noalloc(pyl_ctx *ctx, const float *delta, int dims, double BoxSize,
                   int axis, int mas, int what, pyl_pk_out *out);

/* Tile shape of the sorted deposit for (dims, mas): tiles of TX x TY x TZ
 * cells (powers of two, at most 64) and F tiles per coarse bucket of the
 * first partition pass (a power of two <= 256; 0 = about sqrt(tiles)).  No
 * reference counterpart: set by the autotuner (pylians3_gb300.autotune) for
 * the whole process; TX = 0 restores the built-in rule.  Returns
 * PYL_ERR_UNSUPPORTED for shapes whose footprint or tile histogram does not
 * fit in shared memory or that need more than 256 coarse buckets.
 * pyl_get_tile_shape reports the shape in use.                             */
int pyl_set_tile_shape(int dims, int mas, int TX, int TY, int TZ, int F);
int pyl_get_tile_shape(int dims, int mas, int *TX, int *TY, int *TZ, int *F);

/* One particles -> spectrum request (the arguments of pyl_pk_particles). */
typedef struct {
    const float *pos;   /* (n, 3) positions                                */
    int64_t n;
    const float *W;     /* (n,) weights or NULL                             */
    int dims;
    float BoxSize;
    int mas_deposit, axis, mas_window, what;
} pyl_pk_request;

/* Spectra of `count` requests issued at once and waited for once (no
 * reference counterpart: the batched form of pyl_pk_particles).  The
 * requests are spread over lanes -- child contexts with their own streams
 * and workspaces that run side by side (PYL_BATCH_LANES(k) in flags, 1..15;
 * 0 = 4 lanes) -- longest first onto the least loaded lane.  The sequence is
 * captured into a CUDA graph (the lanes as parallel branches) the first
 * time a given list of requests (same pointers, sizes and options) is seen:
 * that first call issues the requests directly with the exact counting sort,
 * which also sizes the workspaces, and learns from each request the slots of
 * the count-free sort the graph then uses; later calls with the same list
 * launch the graph: one launch for the whole batch.  outs[i] receives
 * request i (arrays as for pyl_pk).  All requests use device pointers
 * (PYL_DEVICE_PTRS) or all host pointers; PYL_NO_GRAPH skips the graph.     */
#define PYL_BATCH_LANES(k) (((k) & 0xF) << 16)
int pyl_pk_batch(pyl_ctx *ctx, const pyl_pk_request *reqs, int count,
                 pyl_pk_out *outs, int flags);

/* ---------------------------------------------------------------------
 * Rows around the spectrum (same FFT, window and mode conventions).
 * ------------------------------------------------------------------- */

/* correct_MAS (library/Pk_library/Pk_library.pyx:1882-1939): out = the
 * field with its independent Fourier modes divided by the MAS window
 * (r2c, window, c2r normalised by 1/dims^3).  delta is not modified.      */
int pyl_correct_mas(pyl_ctx *ctx, const float *delta, float *out, int dims,
                    int mas, int flags);

/* FFT2Dr_f / IFFT2Dr_f (Pk_library.pyx:181-196, 213-228): (grid, grid)
 * float32 <-> (grid, grid/2+1) complex64 (interleaved floats); the inverse
 * is normalised by 1/grid^2 and does not modify its input.                */
int pyl_fft2_r2c(pyl_ctx *ctx, const float *in, float *out, int grid, int flags);
int pyl_fft2_c2r(pyl_ctx *ctx, const float *in, float *out, int grid, int flags);

/* class Pk_plane (Pk_library.pyx:435-511): spectrum of a (grid, grid)
 * float32 field; k, Pk, Nmodes have kmax = int(sqrt(2 (grid/2)^2)) entries
 * (the DC bin dropped).  Returns PYL_ERR_MODES when check_number_modes_2D
 * (:102-115) would exit.                                                   */
int pyl_pk_plane(pyl_ctx *ctx, const float *delta, int grid, double BoxSize,
                 int mas, double *k, double *Pk, double *Nmodes, int flags);

/* CIC_interp (library/MAS_library/MAS_library.pyx:558-599): den[i] = the
 * trilinear (CIC) interpolation of density (dims^3 float32) at pos[i]
 * ((n, 3) float32), float32 arithmetic in the reference's order.          */
int pyl_cic_interp(pyl_ctx *ctx, const float *density, int dims, float BoxSize,
                   const float *pos, int64_t n, float *den, int flags);

/* pos_redshift_space (library/redshift_space_library/
 * redshift_space_library.pyx:29-50), in place on the (n, 3) positions:
 * pos[:, axis] += vel[:, axis] (1 + redshift) / Hubble, wrapped into
 * [0, BoxSize].                                                            */
int pyl_rsd(pyl_ctx *ctx, float *pos, const float *vel, int64_t n, float BoxSize,
            float Hubble, float redshift, int axis, int flags);

/* class XPk (Pk_library.pyx:529-735): auto- and cross-spectra of nfields
 * (1..8) float32 fields of the same dims^3 grid, mas[i] the window of field
 * i.  With X = nfields (nfields - 1) / 2 pairs (i < j in row order), the
 * row-major arrays are: Pk (kmax, 3, nfields), XPk (kmax, 3, X), k3D and
 * Nmodes3D (kmax); k1D, Nmodes1D (kmax_par), Pk1D (kmax_par, nfields), PkX1D
 * (kmax_par, X); kpar, kper, Nmodes2D (n2D), Pk2D (n2D, nfields), PkX2D
 * (n2D, X), n2D = (kmax_par + 1)(kmax_per + 1).  Null pointers skip an
 * output.  deltas[i] are host pointers, or device pointers with
 * PYL_DEVICE_PTRS.                                                         */
typedef struct {
    double *k3D, *Pk, *XPk, *Nmodes3D;
    double *k1D, *Pk1D, *PkX1D, *Nmodes1D;
    double *kpar, *kper, *Pk2D, *PkX2D, *Nmodes2D;
} pyl_xpk_out;
int pyl_xpk(pyl_ctx *ctx, const float *const *deltas, int nfields, int dims,
            double BoxSize, int axis, const int *mas, pyl_xpk_out *out, int flags);

#ifdef __cplusplus
}
#endif
#endif /* PYLGPU_H */
