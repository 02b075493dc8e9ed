// Shared declarations of libpylgpu: the context, plans and the internal
// launchers each translation unit provides.  Device code targets sm_103a.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <tuple>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pylgpu.h"

namespace pyl {

// ------------------------------------------------------------------ FFT plan
// A length-n complex FFT is a sequence of Stockham stages of the given radices
// (product = n).  tw[m] = exp(-2*pi*i*m/n), computed on the host in double.
constexpr int kMaxStages = 24;
struct FftDesc {
    int n;
    int nst;
    int radix[kMaxStages];
};

struct FftPlan {
    FftDesc desc;
    float2 *d_tw = nullptr;  // n entries
};

// Mode-count tables of one (dims, axis): integer counts of independent modes
// per bin, and the sum of |k| per 3D bin, made once and cached.  Indices
// include the DC bin (index 0), as the reference's raw arrays do.
struct ModeTables {
    int dims = 0, axis = 0, kmax = 0, kmax_par = 0, kmax_per = 0;
    std::vector<double> N3D, k3Dsum;     // kmax+1
    std::vector<double> N1D, k1Dsum;     // kmax_par+1
    std::vector<double> N2D;             // (kmax_par+1)*(kmax_per+1)
    long long total = 0;
};

// Device layout of the float64 sums of one Pk evaluation, followed by the raw
// k = 0 mode (float2), the deposited mass (double) and the FFT shift (float).
struct AccLayout {
    size_t n3 = 0, n1 = 0, nph = 0, n2 = 0;
    size_t sums() const { return sizeof(double) * (n3 + n1 + nph + n2); }
    size_t bytes() const { return sums() + 64; }
};

// Accumulators of one Pk evaluation on the device (float64 sums).
struct PkAcc {
    double *P3 = nullptr;     // (kmax+1)*3   sum of delta2 * L_ell(mu)
    double *P1 = nullptr;     // kmax_par+1   sum of delta2 for k <= middle
    double *Pph = nullptr;    // kmax+1       sum of phase^2
    double *P2D = nullptr;    // (kmax_par+1)*(kmax_per+1)
    float2 *dc = nullptr;     // the raw (k=0) mode, for the grid mean
    double *mass = nullptr;   // total deposited mass (particles path)
    float *shift = nullptr;   // constant subtracted from the grid before the FFT
};

}  // namespace pyl

// Pipeline stages timed (on request) with CUDA events on the context stream.
// The stages do not overlap: ST_BINS is the tile histogram and the scans of
// the sorted deposit, ST_SORT its partition passes, ST_DEPOSIT the deposit
// kernel proper, ST_MASS the total mass and FFT shift of the fused path.
enum PylStage {
    ST_H2D = 0, ST_ZERO, ST_DEPOSIT, ST_SORT, ST_FFT_Z, ST_FFT_Y, ST_FFT_X, ST_PK_X,
    ST_D2H, ST_BINS, ST_MASS, ST_NSTAGES
};

// ------------------------------------------------------------------ context
struct pyl_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int64_t launches = 0;

    bool timing = false;
    struct Pending { int stage; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    double stage_ms[ST_NSTAGES] = {};
    int64_t stage_n[ST_NSTAGES] = {};

    // Count-free ("capacity") tile sort of the fused particles path: per
    // (device, dims, scheme, weighted), what the last request showed, shared
    // by all contexts of the process (shared_sort_plan).  After an exact
    // sort, the largest tile and coarse-bucket counts relative to their means
    // (phiT, phiC) size fixed slots for the next request, which then needs
    // no counting pass; a request whose slots overflowed (its particles went
    // to the spill list) sends the next one back to the exact sort.  mode:
    // the sort the exact pass chose (frontier/two-pass).  Plans are read and
    // written under one lock (read_sort_plan, learn_sort).
    struct SortPlan { bool cap = false; float phiT = 0.f, phiC = 0.f; int mode = -1; };
    SortPlan *sort_hint = nullptr;     // set by the particles path around deposit()
    struct SortUsed {
        bool valid = false, cap = false;
        int ntiles = 0, F = 0;
        long long n = 0;
        SortPlan *plan = nullptr;
    } sort_used;                       // what the last sorted deposit did
    unsigned *d_sort_info = nullptr;   // its 4 info words on the device
    int last_sort_cap = -1;            // the last collected request's sort (pyl_ctx_last_sort)
    unsigned last_spilled = 0;

    // The request issued by pyl_pk_particles_enqueue and not yet collected:
    // its raw sums are copied to `pinned` and `done` is recorded after them.
    struct Request {
        bool active = false;
        int dims = 0, axis = 0, what = 0;
        double BoxSize = 0.0;
        const pyl::ModeTables *T = nullptr;
        pyl::AccLayout L;
        SortUsed sort;        // its sorted deposit; its info words follow the sums
    } req;
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    cudaEvent_t done = nullptr;

    struct Buf { void *p = nullptr; size_t bytes = 0; };
    std::map<std::string, Buf> ws;                       // named workspaces

    // A second stream for work that can run beside the sort: the grid of
    // the fused particles path is zeroed there (created on first use).
    // grid_pending: that zeroing is issued and the context stream has not
    // yet waited for it (wait_grid).
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool grid_pending = false;

    // Status word the kernels set when a bounded wait gives up (bits of
    // kStatusWaitTimeout, async_copy.cuh); read and cleared by status_check.
    unsigned *d_status = nullptr;

    // pyl_pk_batch: while a sequence is captured no workspace may grow (a
    // reallocation synchronises the stream); the last captured batch, its
    // key (the request list and flags) and the pinned buffer it writes.
    bool capturing = false;
    // pyl_pk_batch's lanes: child contexts (own stream, own workspaces) whose
    // requests run side by side, forked from and joined back to this
    // context's stream by events; the sort plans learned per request of the
    // batch (keyed by batch_plans_key) and the sorts its graph was captured
    // with (batch_used).
    std::vector<pyl_ctx *> lanes;
    std::vector<cudaEvent_t> lane_join;
    cudaEvent_t lane_fork = nullptr;
    std::vector<SortPlan> batch_plans;
    std::vector<char> batch_plans_key;
    std::vector<SortUsed> batch_used;
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<char> batch_key;
    void *batch_pinned = nullptr;
    size_t batch_pinned_bytes = 0;
};

namespace pyl {

// Error helpers: record a message on the context and return a status.
int fail(pyl_ctx *ctx, int code, const std::string &msg);
int cuda_fail(pyl_ctx *ctx, cudaError_t e, const char *what);
#define PYL_CUDA(ctx, call)                                                  \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return pyl::cuda_fail((ctx), e_, #call);      \
    } while (0)

// Waits for the context stream, then reads and clears the device status
// word: PYL_ERR_TIMEOUT if a kernel's bounded wait gave up since the last
// check.
int status_check(pyl_ctx *ctx);

// Workspace of at least `bytes`, kept across calls under `name`.
void *ws_get(pyl_ctx *ctx, const char *name, size_t bytes, int *status);

// Stage timing: events recorded around a stage when ctx->timing is set;
// stage_flush() waits for them and accumulates the elapsed times.
void stage_mark(pyl_ctx *ctx, int stage, bool begin);
int stage_flush(pyl_ctx *ctx);
struct StageScope {
    pyl_ctx *ctx;
    int stage;
    StageScope(pyl_ctx *c, int s) : ctx(c), stage(s) { stage_mark(ctx, stage, true); }
    ~StageScope() { stage_mark(ctx, stage, false); }
};

// Plans (ctx.cu)
const FftPlan *fft_plan(pyl_ctx *ctx, int n, int *status);
const ModeTables *mode_tables(pyl_ctx *ctx, int dims, int axis, int *status);
const float *window_table(pyl_ctx *ctx, int dims, int mas, int *status);

// ---------------------------------------------------------------- launchers
// deposit.cu: grid += deposit of n particles (grid extent dims^2 * dz where
// dz = dims for coord 3 and 1 for coord 2).  All pointers are device pointers.
// Zeroes `bytes` at p on the context's side stream after the work already
// on the context stream, so that it overlaps what the context stream does
// next; wait_grid makes the context stream wait for it (a no-op when nothing
// is pending).  Every kernel that touches the grid calls wait_grid first.
int zero_beside(pyl_ctx *ctx, void *p, size_t bytes);
int wait_grid(pyl_ctx *ctx);

int deposit(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
            float *grid, int dims, float BoxSize, int mas, int flags);
int deposit_f64(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                double *grid, int dims, float BoxSize, int mas);
// grid /= d over `count` elements
int scale_grid(pyl_ctx *ctx, float *grid, int64_t count, float s);
int scale_grid_f64(pyl_ctx *ctx, double *grid, int64_t count, double s);
inline int deposit_any(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                       float *grid, int dims, float BoxSize, int mas, int flags) {
    return deposit(ctx, pos, n, coord, W, grid, dims, BoxSize, mas, flags);
}
inline int deposit_any(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                       double *grid, int dims, float BoxSize, int mas, int) {
    return deposit_f64(ctx, pos, n, coord, W, grid, dims, BoxSize, mas);
}
inline int scale_any(pyl_ctx *ctx, float *g, int64_t c, double s) {
    return scale_grid(ctx, g, c, (float)s);
}
inline int scale_any(pyl_ctx *ctx, double *g, int64_t c, double s) {
    return scale_grid_f64(ctx, g, c, s);
}

// fft.cu (lengths 2^k and 3*2^k go to fft_reg.cu)
// r2c along the last axis of rows (rows x n real -> rows x (n/2+1) complex,
// output row stride ostride >= n/2+1; padding needs n = 2^k or 3*2^k).  When
// shift is not null, *shift (device) is subtracted from every input value
// (changes only the k = 0 mode, and keeps its round-off out of the others).
int fft_rows_r2c(pyl_ctx *ctx, const float *in, float2 *out, int64_t rows, int n, int ostride,
                 const float *shift = nullptr);
// c2r along the last axis, times `scale` (input row stride istride)
int fft_rows_c2r(pyl_ctx *ctx, const float2 *in, float *out, int64_t rows, int n, int istride,
                 float scale);
// in-place c2c along axis 0 (x) or 1 (y) of an (n, n, h) complex array whose
// rows have stride rs >= h
int fft_axis_c2c(pyl_ctx *ctx, float2 *data, int n, int h, int rs, int axis, int dir);
// in-place c2c along axis 0 of an (n, rs) complex plane (its first h columns)
int fft_plane_c2c(pyl_ctx *ctx, float2 *data, int n, int h, int rs, int dir);

// fft_reg.cu: lengths 2^k (16..4096) and 3*2^k (48..3072)
bool reg_supported(int n);
// Entries of the register FFT's stage twiddle tables for length n, as
// indices of the n-entry table (PYL_ERR_UNSUPPORTED if n has no register FFT).
int reg_stage_twiddle_sources(int n, std::vector<int> &src);
int pow2_rows_r2c(pyl_ctx *ctx, const float *in, float2 *out, int64_t rows, int n, int ostride,
                  const float2 *tw, const float *shift);
// total mass (sum of W, or n) into *mass, then *shift = mass / cells
int mass_and_shift(pyl_ctx *ctx, const float *W, int64_t n, double cells, double *mass,
                   float *shift);
int pow2_rows_c2r(pyl_ctx *ctx, const float2 *in, float *out, int64_t rows, int n, int istride,
                  const float2 *tw, float scale);
int pow2_cols(pyl_ctx *ctx, float2 *data, int n, int ncol, int64_t estride, int64_t ostride,
              int nouter, int dir, const float2 *tw);
int pow2_pk_x(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, const float2 *tw,
              const float *win, int kmax, const PkAcc &acc, int what);

// pk.cu
// x-axis FFT of the (n, n, h) half-complex array (already transformed along
// z and y) fused with the window, |delta_k|^2, Legendre weights and binning.
int pk_bin_x(pyl_ctx *ctx, const float2 *data, int n, int rs, int axis, int mas,
             int what, const PkAcc &acc, int kmax, int kmax_per);
// padded row stride of the internal half-complex grid (64-byte aligned rows
// on the power-of-two path)
inline int half_stride(int n) {
    const int h = n / 2 + 1;
    return reg_supported(n) ? (h + 7) / 8 * 8 : h;
}
// integer mode counts of (dims, axis) into device histograms
int mode_counts(pyl_ctx *ctx, int dims, int axis, unsigned long long *cnt_n,
                unsigned long long *cnt1, unsigned long long *cnt2, int kmax_per);

inline int isqrt_host(long long v) { return (int)__builtin_sqrt((double)v); }

// ------------------------------------------------- spectrum bookkeeping (ctx.cu)
// Device layout of the float64 sums of one Pk evaluation, followed by the raw
// k = 0 mode (float2), the deposited mass (double) and the FFT shift (float).
AccLayout acc_layout(const ModeTables &T);
PkAcc acc_view(void *base, const AccLayout &L);
// Finalisation of class Pk from the raw sums (host, float64).
int finalize(pyl_ctx *ctx, const ModeTables &T, const std::vector<double> &raw,
             const AccLayout &L, double BoxSize, int what, double inv_mean2, bool zero_dc2d,
             pyl_pk_out *out);
int download_raw(pyl_ctx *ctx, void *acc, const AccLayout &L, std::vector<double> &raw,
                 float2 *dc, double *mass);
// The particles -> spectrum request (ctx.cu): argument check, issue on the
// context stream with the result copied to host `dst`, finalisation.
int check_particles(pyl_ctx *ctx, const pyl_pk_request &r);
int issue_particles(pyl_ctx *ctx, const pyl_pk_request &r, const ModeTables &T, int flags,
                    void *dst);
int finalize_particles(pyl_ctx *ctx, const ModeTables &T, const AccLayout &L, const void *src,
                       int dims, double BoxSize, int what, pyl_pk_out *out);
// Bytes a request's result takes in pinned memory: the raw sums, the k = 0
// mode, the mass and the 4 info words of its sort (copied when the request
// was issued with a sort plan).
size_t result_bytes(const AccLayout &L);
// Updates the sort plan of a finished request from its sort's info words.
void learn_sort(const pyl_ctx::SortUsed &u, const unsigned *info);
// The process-wide plan of (device, dims, scheme, weighted) (a stable
// pointer), and a copy of a plan taken under the plans' lock.
pyl_ctx::SortPlan *shared_sort_plan(int device, int dims, int mas, int weighted);
pyl_ctx::SortPlan read_sort_plan(const pyl_ctx::SortPlan *p);
void twiddles_host(int n, std::vector<float2> &tw);
void window_host(int dims, int mas, std::vector<float> &w);
// Mode tables: sizes of the count arrays, and the tables from the counts.
void mode_table_init(ModeTables &T, int dims, int axis, size_t &nn, size_t &n1, size_t &n2);
void mode_table_fill(ModeTables &T, const unsigned long long *h, size_t nn, size_t n1,
                     size_t n2);

}  // namespace pyl
