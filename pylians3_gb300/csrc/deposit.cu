// Particle deposit (mass assignment) NGP / CIC / TSC / PCS, with optional
// weights, 3D and 2D.  Replaces MAS_library.pyx:123-545 (NGP..PCSW) and the
// C kernels of MAS_c.c:8-266.  The per-axis stencil is in deposit_common.cuh.
//
// Two paths:
//  * unsorted: one thread per particle, one global float atomic (RED) per
//    tap.  Used for small inputs, 2D and float64 grids.
//  * tile-sorted (3D float32): particles are sorted by the tile of their
//    home cell (tiles of TX*TY*TZ cells), each tile's footprint (tile + the
//    stencil halo) is accumulated in shared memory with shared atomics, and
//    added to the grid with vectorised global reductions (red.global.add.v4).
//    The sort is a counting sort done in two partition passes so that every
//    write to HBM is a contiguous run: pass 1 splits the particles into
//    "coarse" buckets of F consecutive tiles, pass 2 splits each bucket into
//    its tiles.  A pass stages KP particles in shared memory, orders them by
//    key there, reserves one contiguous range per key with a single global
//    atomic on that key's cursor, and writes each key's run in one go.
//    Tile start offsets come from a counting pass and an exclusive scan.
//    Tiles holding very many particles (clusters) are split into several
//    work items, so one CTA never serialises a dense halo.
//
// 2D (coord = 2) follows MA's expand_dims path: the third axis has extent 1,
// index 0 and weight 1 for every tap, so a particle is deposited 2/3/4 times
// onto the same plane for CIC/TSC/PCS (and renormalised by the caller).
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

#include "async_copy.cuh"
#include "deposit_common.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;

// ------------------------------------------------------------ unsorted path
// COMP: compensated float adds, errors into lo (same layout as the grid).
// n_dev (may be null): the particle count is min(n, *n_dev), read on the
// device (the spill list of the count-free sort).
template <int MAS, bool HAS_W, typename G, bool COMP>
__global__ void __launch_bounds__(kThreads)
k_deposit_atomic(const float *__restrict__ pos, long long n, int coord,
                 const float *__restrict__ W, G *__restrict__ grid, int dims,
                 float inv, float *__restrict__ lo, const unsigned *__restrict__ n_dev) {
    static_assert(!COMP || sizeof(G) == sizeof(float), "compensation is for float32 grids");
    using S = Stencil<MAS>;
    constexpr int NT = S::NT;
    if (n_dev && (long long)*n_dev < n) n = (long long)*n_dev;
    const long long sy = coord == 3 ? dims : 1;
    const long long sx = sy * dims;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int ix[NT], iy[NT], iz[NT];
        float wx[NT], wy[NT], wz[NT];
        const float *p = pos + i * coord;
        {
            const float d = cell_dist(__ldg(p + 0), inv);
            const int c = home_cell<MAS>(d);
            int off[NT];
            axis_stencil<MAS>(d, c, off, wx);
#pragma unroll
            for (int j = 0; j < NT; ++j) ix[j] = wrap_idx(c + off[j], dims);
        }
        {
            const float d = cell_dist(__ldg(p + 1), inv);
            const int c = home_cell<MAS>(d);
            int off[NT];
            axis_stencil<MAS>(d, c, off, wy);
#pragma unroll
            for (int j = 0; j < NT; ++j) iy[j] = wrap_idx(c + off[j], dims);
        }
        if (coord == 3) {
            const float d = cell_dist(__ldg(p + 2), inv);
            const int c = home_cell<MAS>(d);
            int off[NT];
            axis_stencil<MAS>(d, c, off, wz);
#pragma unroll
            for (int j = 0; j < NT; ++j) iz[j] = wrap_idx(c + off[j], dims);
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
                const long long row = ix[l] * sx + iy[m] * sy;
#pragma unroll
                for (int q = 0; q < NT; ++q) {
                    float v = wxy * wz[q];
                    if (HAS_W) v *= wt;
                    if constexpr (COMP)
                        comp_add(reinterpret_cast<float *>(grid) + row + iz[q], lo + row + iz[q], v);
                    else
                        atomicAdd(grid + row + iz[q], (G)v);
                }
            }
        }
    }
}

// g += lo elementwise (one rounding): folds the compensation into the grid
__global__ void k_fold_lo(float *__restrict__ g, const float *__restrict__ lo, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        g[i] = __fadd_rn(g[i], lo[i]);
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

// lo != nullptr (float grids only): compensated adds, errors into lo.
template <int MAS, typename G>
int launch_atomic(pyl_ctx *ctx, const float *pos, long long n, int coord, const float *W,
                  G *grid, int dims, float inv, float *lo) {
    long long blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 152LL * 64) blocks = 152LL * 64;
    if (blocks < 1) blocks = 1;
    int st = wait_grid(ctx);
    if (st) return st;
    StageScope s(ctx, ST_DEPOSIT);
    auto go = [&](auto kernel) {
        kernel<<<(unsigned)blocks, kThreads, 0, ctx->stream>>>(pos, n, coord, W, grid, dims, inv,
                                                               lo, nullptr);
    };
    if constexpr (sizeof(G) == sizeof(float)) {
        if (lo) {
            if (W) go(k_deposit_atomic<MAS, true, G, true>);
            else go(k_deposit_atomic<MAS, false, G, true>);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
            return PYL_OK;
        }
    }
    if (W) go(k_deposit_atomic<MAS, true, G, false>);
    else go(k_deposit_atomic<MAS, false, G, false>);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

// ------------------------------------------------------------------- scan
// Exclusive scan of a uint32 array in place (three passes: block sums, scan
// of block sums, block-local scan + offset).
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;
constexpr int kScanChunk = kScanThreads * kScanPer;

// Block-wide exclusive scan of one value per thread.  Uses s_warp[32]; two
// consecutive calls must be separated by a __syncthreads().
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned *s_warp,
                                                         unsigned *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        unsigned s = lane < nw ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) s_warp[lane] = s;
    }
    __syncthreads();
    const unsigned warp_off = wid > 0 ? s_warp[wid - 1] : 0u;
    if (total) *total = s_warp[(blockDim.x >> 5) - 1];
    return warp_off + x - v;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_sums(const unsigned *__restrict__ a, long long n, unsigned *__restrict__ sums) {
    __shared__ unsigned s_warp[32];
    const long long base = (long long)blockIdx.x * kScanChunk + (long long)threadIdx.x * kScanPer;
    unsigned s = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k)
        if (base + k < n) s += a[base + k];
    unsigned total;
    block_exclusive_scan(s, s_warp, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_top(unsigned *__restrict__ sums, int nb) {
    __shared__ unsigned s_warp[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const unsigned v = i < nb ? sums[i] : 0u;
        unsigned total;
        const unsigned ex = block_exclusive_scan(v, s_warp, &total);
        const unsigned c = carry;
        if (i < nb) sums[i] = c + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_apply(unsigned *__restrict__ a, long long n, const unsigned *__restrict__ sums) {
    __shared__ unsigned s_warp[32];
    const long long base = (long long)blockIdx.x * kScanChunk + (long long)threadIdx.x * kScanPer;
    unsigned v[kScanPer];
    unsigned s = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        v[k] = base + k < n ? a[base + k] : 0u;
        s += v[k];
    }
    unsigned run = block_exclusive_scan(s, s_warp, nullptr) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        if (base + k < n) a[base + k] = run;
        run += v[k];
    }
}

int scan_exclusive(pyl_ctx *ctx, unsigned *a, long long n) {
    const long long nb = (n + kScanChunk - 1) / kScanChunk;
    int st = PYL_OK;
    unsigned *sums = (unsigned *)ws_get(ctx, "scan_sums", sizeof(unsigned) * (size_t)nb, &st);
    if (!sums) return st;
    k_scan_sums<<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(a, n, sums);
    k_scan_top<<<1, kScanThreads, 0, ctx->stream>>>(sums, (int)nb);
    k_scan_apply<<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(a, n, sums);
    ctx->launches += 3;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

// -------------------------------------------------------- tile-sorted path
struct TileGeom {
    int dims;
    int TX, TY, TZ;      // tile extent in cells (powers of two)
    int sx, sy, sz;      // log2 of the tile extents
    int ntx, nty, ntz;   // tiles per axis
    int RX, RY, RZ;      // shared footprint extent = T + LO + HI
    int ntiles;
    int F;               // tiles per coarse bucket (power of two)
    int sF;              // log2 F
    int ncoarse;         // coarse buckets = ceil(ntiles / F)
    int dmask;           // dims - 1 when dims is a power of two, else -1
};

// Periodic wrap of a cell index: for a power-of-two grid one mask (equal to
// wrap_idx for every int), else wrap_idx's in-box test and remainder.
__device__ __forceinline__ int wrap_cell(int i, const TileGeom &g) {
    return g.dmask >= 0 ? (i & g.dmask) : wrap_idx(i, g.dims);
}

// The same with the grid's kind known at compile time (P2: power of two).
template <class P2>
__device__ __forceinline__ int wrap_as(P2, int i, const TileGeom &g) {
    return P2::value ? (i & g.dmask) : wrap_idx(i, g.dims);
}

// Partition shape (compile-time; the defaults are the measured best):
// particles staged per chunk, threads per CTA (>= kMaxKeys: one scan value
// per thread), resident CTAs per SM the registers are sized for.  2048
// particles per chunk on 512 threads (two CTAs per SM) gives each key longer
// runs per chunk than 1024 on 256 threads (four CTAs per SM): both count-free
// passes at 512^3 CIC 1.73 -> 1.67 ms; 2048 on 256 threads: 1.81 ms.
#ifndef PYL_PART_KP
#define PYL_PART_KP 2048
#endif
#ifndef PYL_PART_THREADS
#define PYL_PART_THREADS 512
#endif
#ifndef PYL_PART_MINB
#define PYL_PART_MINB 2
#endif
constexpr int KP = PYL_PART_KP;
constexpr int kPartThreads = PYL_PART_THREADS;
static_assert(KP % 4 == 0, "bulk copies move whole 16-byte groups");
constexpr int kMaxKeys = 256;     // buckets of one partition step
constexpr int kChunkTab = 8192;   // fine partition: chunks per CTA it can map
constexpr unsigned kItemCap = 65536;  // particles per deposit work item

template <int MAS>
__device__ __forceinline__ int tile_of(float x, float y, float z, float inv, const TileGeom &g) {
    const int hx = wrap_cell(home_cell<MAS>(cell_dist(x, inv)), g);
    const int hy = wrap_cell(home_cell<MAS>(cell_dist(y, inv)), g);
    const int hz = wrap_cell(home_cell<MAS>(cell_dist(z, inv)), g);
    return ((hx >> g.sx) * g.nty + (hy >> g.sy)) * g.ntz + (hz >> g.sz);
}

// The same with the grid's kind known at compile time (P2: power of two).
template <int MAS, class P2>
__device__ __forceinline__ int tile_of_as(P2 p2, float x, float y, float z, float inv,
                                          const TileGeom &g) {
    const int hx = wrap_as(p2, home_cell<MAS>(cell_dist(x, inv)), g);
    const int hy = wrap_as(p2, home_cell<MAS>(cell_dist(y, inv)), g);
    const int hz = wrap_as(p2, home_cell<MAS>(cell_dist(z, inv)), g);
    return ((hx >> g.sx) * g.nty + (hy >> g.sy)) * g.ntz + (hz >> g.sz);
}

// Counting pass: particles per tile (shared histogram, then global adds).
// It also counts tile changes between neighbouring particles of each warp
// (particle i vs i-1): few changes mean the input order is already spatially
// coherent (e.g. a displaced lattice), and the single-pass frontier scatter
// is then the cheaper sort.  A warp whose 32 particles share one tile adds
// them with one shared atomic.
constexpr int kCountUnroll = 4;

template <int MAS>
__global__ void __launch_bounds__(1024, 1)
k_tile_count(const float *__restrict__ pos, long long n, float inv, TileGeom g,
             unsigned *__restrict__ count, unsigned *__restrict__ distinct) {
    extern __shared__ unsigned s_cnt[];
    __shared__ unsigned s_distinct;
    for (int t = threadIdx.x; t < g.ntiles; t += blockDim.x) s_cnt[t] = 0u;
    if (threadIdx.x == 0) s_distinct = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    unsigned changes = 0;
    // kCountUnroll rows of blockDim.x particles per iteration, all loads
    // issued before any is used (the pass is bound by load latency)
    const long long step = (long long)gridDim.x * blockDim.x * kCountUnroll;
    for (long long b = (long long)blockIdx.x * blockDim.x * kCountUnroll; b < n; b += step) {
        float x[kCountUnroll], y[kCountUnroll], z[kCountUnroll];
#pragma unroll
        for (int u = 0; u < kCountUnroll; ++u) {
            const long long i = b + (long long)u * blockDim.x + threadIdx.x;
            if (i < n) {
                x[u] = __ldcs(pos + 3 * i);
                y[u] = __ldcs(pos + 3 * i + 1);
                z[u] = __ldcs(pos + 3 * i + 2);
            }
        }
#pragma unroll
        for (int u = 0; u < kCountUnroll; ++u) {
            const long long i = b + (long long)u * blockDim.x + threadIdx.x;
            const bool active = i < n;
            const int t = active ? tile_of<MAS>(x[u], y[u], z[u], inv, g) : -1;
            const int prev = __shfl_up_sync(0xffffffffu, t, 1);
            const int first = __shfl_sync(0xffffffffu, t, 0);
            const bool same = __all_sync(0xffffffffu, t == first);
            if (same) {
                if (lane == 0 && t >= 0) atomicAdd(&s_cnt[t], 32u);
                changes += (lane == 0 && t >= 0) ? 1u : 0u;
            } else if (active) {
                atomicAdd(&s_cnt[t], 1u);
                changes += (lane == 0 || t != prev) ? 1u : 0u;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) changes += __shfl_down_sync(0xffffffffu, changes, o);
    if (lane == 0 && changes) atomicAdd(&s_distinct, changes);
    __syncthreads();
    for (int t = threadIdx.x; t < g.ntiles; t += blockDim.x)
        if (s_cnt[t]) atomicAdd(&count[t], s_cnt[t]);
    if (threadIdx.x == 0 && s_distinct) atomicAdd(distinct, s_distinct);
}

// The same count with 16-byte loads (positions 16-byte aligned): a thread
// takes four consecutive particles as three float4 (a warp reads 1536
// contiguous bytes per load instruction), two groups in flight; runs of one
// tile inside a thread take one shared atomic, a warp whose 128 particles
// share a tile takes one.  Tile changes are counted between consecutive
// particles (inside a thread and across neighbouring lanes), plus one per
// warp group.  The last n % 4 particles are counted by block 0 one by one.
template <int MAS>
__global__ void __launch_bounds__(1024, 1)
k_tile_count4(const float4 *__restrict__ pos4, const float *__restrict__ pos, long long n,
              float inv, TileGeom g, unsigned *__restrict__ count,
              unsigned *__restrict__ distinct) {
    extern __shared__ unsigned s_cnt[];
    __shared__ unsigned s_distinct;
    for (int t = threadIdx.x; t < g.ntiles; t += blockDim.x) s_cnt[t] = 0u;
    if (threadIdx.x == 0) s_distinct = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    unsigned changes = 0;
    const long long groups = n / 4;          // groups of four particles
    constexpr int U = 2;
    const long long step = (long long)gridDim.x * blockDim.x * U;
    for (long long b = (long long)blockIdx.x * blockDim.x * U; b < groups; b += step) {
        float4 a[U][3];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long gi = b + (long long)u * blockDim.x + threadIdx.x;
            if (gi < groups) {
                a[u][0] = __ldcs(pos4 + 3 * gi);
                a[u][1] = __ldcs(pos4 + 3 * gi + 1);
                a[u][2] = __ldcs(pos4 + 3 * gi + 2);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long gi = b + (long long)u * blockDim.x + threadIdx.x;
            const bool active = gi < groups;
            int t[4] = {-1, -1, -1, -1};
            if (active) {
                const float4 p0 = a[u][0], p1 = a[u][1], p2 = a[u][2];
                t[0] = tile_of<MAS>(p0.x, p0.y, p0.z, inv, g);
                t[1] = tile_of<MAS>(p0.w, p1.x, p1.y, inv, g);
                t[2] = tile_of<MAS>(p1.z, p1.w, p2.x, inv, g);
                t[3] = tile_of<MAS>(p2.y, p2.z, p2.w, inv, g);
            }
            const int prev_last = __shfl_up_sync(0xffffffffu, t[3], 1);
            const int first = __shfl_sync(0xffffffffu, t[0], 0);
            const bool same = __all_sync(0xffffffffu, t[0] == first && t[1] == first &&
                                                          t[2] == first && t[3] == first);
            if (same) {
                if (lane == 0 && first >= 0) {
                    atomicAdd(&s_cnt[first], 128u);
                    changes += 1u;
                }
            } else if (active) {
                changes += (lane == 0 || t[0] != prev_last) ? 1u : 0u;
                unsigned run = 1u;
#pragma unroll
                for (int k = 1; k < 4; ++k) {
                    if (t[k] == t[k - 1]) {
                        ++run;
                    } else {
                        atomicAdd(&s_cnt[t[k - 1]], run);
                        run = 1u;
                        ++changes;
                    }
                }
                atomicAdd(&s_cnt[t[3]], run);
            }
        }
    }
    if (blockIdx.x == 0) {
        for (long long i = groups * 4 + threadIdx.x; i < n; i += blockDim.x)
            atomicAdd(&s_cnt[tile_of<MAS>(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], inv, g)], 1u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) changes += __shfl_down_sync(0xffffffffu, changes, o);
    if (lane == 0 && changes) atomicAdd(&s_distinct, changes);
    __syncthreads();
    for (int t = threadIdx.x; t < g.ntiles; t += blockDim.x)
        if (s_cnt[t]) atomicAdd(&count[t], s_cnt[t]);
    if (threadIdx.x == 0 && s_distinct) atomicAdd(distinct, s_distinct);
}

// After the scan (start[0..ntiles] exclusive, start[ntiles] = n): the key
// cursors of both passes and the deposit work items (tile, chunk) of every
// non-empty tile, chunk = kItemCap particles.  nchunk is scanned separately.
// Sort mode: 0 = frontier scatter, 1 = two partition passes; forced >= 0
// overrides the choice made from the distinct-tiles-per-warp count (frontier
// when a warp's 32 particles span at most 8 tiles on average).
constexpr int kSortFrontier = 0, kSortTwoPass = 1;

// info (4 words, zeroed): [0] the largest tile count, [1] the largest coarse
// bucket count, [2] the sort chosen -- what the count-free sort of the next
// request sizes its slots from.
__global__ void k_sort_setup(const unsigned *__restrict__ start, int ntiles, int F, int ncoarse,
                             unsigned *__restrict__ fine_cur, unsigned *__restrict__ coarse_cur,
                             unsigned *__restrict__ nchunk, long long n,
                             const unsigned *__restrict__ distinct, int forced,
                             unsigned *__restrict__ mode, unsigned *__restrict__ info) {
    const unsigned m = forced >= 0 ? (unsigned)forced
                                   : ((long long)*distinct * 4 <= n ? kSortFrontier : kSortTwoPass);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *mode = m;
        info[2] = m;
    }
    unsigned mt = 0, mc = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
        fine_cur[t] = start[t];
        const unsigned cnt = start[t + 1] - start[t];
        nchunk[t] = (cnt + kItemCap - 1) / kItemCap;
        mt = max(mt, cnt);
        if (t % F == 0) {
            coarse_cur[t / F] = start[t];
            mc = max(mc, start[min(t + F, ntiles)] - start[t]);
        }
    }
    if (mt) atomicMax(&info[0], mt);
    if (mc) atomicMax(&info[1], mc);
}

__global__ void k_items(const unsigned *__restrict__ nchunk_ex, const unsigned *__restrict__ start,
                        int ntiles, uint2 *__restrict__ items, unsigned *__restrict__ nitems) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
        const unsigned cnt = start[t + 1] - start[t];
        const unsigned k = (cnt + kItemCap - 1) / kItemCap;
        for (unsigned c = 0; c < k; ++c) items[nchunk_ex[t] + c] = make_uint2(t, c);
        if (t == ntiles - 1) *nitems = nchunk_ex[t] + k;
    }
}

// One partition pass.  FINE = false: keys are coarse buckets (tile / F) of
// the particles in input order; FINE = true: the input is grouped by coarse
// bucket and each bucket is split into its F tiles.
//
// Persistent CTAs walk the input in chunks of KP particles (chunk c, c +
// gridDim.x, ...).  The next chunk is fetched into the other of two shared
// buffers by a bulk copy (cp.async.bulk + mbarrier) while the current one is
// partitioned, so the load latency is off the critical path.  Chunks that
// are not whole or not 16-byte aligned (the tail; unaligned user pointers)
// are read with plain loads.  A chunk is processed as segments that do not
// straddle a coarse bucket (one segment in the coarse pass): keys, a shared
// histogram, one global atomic per key on that key's cursor, a shared
// counting sort, then each key's run is written out contiguously.
template <int MAS, bool HAS_W, bool FINE>
__global__ void __launch_bounds__(kPartThreads, PYL_PART_MINB)
k_partition(const float *__restrict__ src, const float *__restrict__ srcw,
            float *__restrict__ dst, float *__restrict__ dstw, long long n, float inv,
            TileGeom g, unsigned *__restrict__ cursor, const unsigned *__restrict__ start,
            const unsigned *__restrict__ mode, int bulk, unsigned *__restrict__ status) {
    if (*mode != kSortTwoPass) return;   // the whole grid takes the same branch
    const long long nchunks = (n + KP - 1) / KP;
    long long c = blockIdx.x;
    if (c >= nchunks) return;
    extern __shared__ __align__(16) float sm[];
    constexpr int WS = HAS_W ? KP : 0;
    // buffer b: positions at sm + 3*KP*b, weights at sm + 6*KP + WS*b
    float *sp2 = sm + 6 * KP + 2 * WS;                   // 3*KP in key order
    float *sw2 = sp2 + 3 * KP;
    unsigned short *skey = reinterpret_cast<unsigned short *>(sw2 + WS);
    unsigned short *skey2 = skey + KP;
    unsigned *hist = reinterpret_cast<unsigned *>(skey2 + KP);   // kMaxKeys each
    unsigned *loff = hist + kMaxKeys;
    unsigned *lcur = loff + kMaxKeys;
    unsigned *gbase = lcur + kMaxKeys;
    unsigned *groom = gbase + kMaxKeys;   // elements of the key's run that fit its region
    __shared__ unsigned s_warp[32];
    __shared__ long long s_seg[2];
    __shared__ __align__(8) uint64_t s_bar[2];

    auto whole = [&](long long cc) { return bulk && (cc + 1) * KP <= n; };
    // thread 0: start the copy of chunk cc into buffer b
    auto issue = [&](long long cc, int b) {
        fence_proxy_async_smem();
        const long long r0 = cc * KP;
        mbar_arrive_expect_tx(&s_bar[b], (12u + (HAS_W ? 4u : 0u)) * KP);
        bulk_copy_g2s(sm + 3 * KP * b, src + 3 * r0, 12u * KP, &s_bar[b]);
        if (HAS_W) bulk_copy_g2s(sm + 6 * KP + WS * b, srcw + r0, 4u * KP, &s_bar[b]);
    };
    if (threadIdx.x == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        mbar_init_fence();
    }
    __syncthreads();
    unsigned parity = 0u;   // bit b: parity of the next phase of s_bar[b]
    unsigned pend = 0u;     // bit b: a copy into buffer b is in flight
    if (whole(c)) {
        if (threadIdx.x == 0) issue(c, 0);
        pend |= 1u;
    }
    int b = 0;
    for (; c < nchunks; c += gridDim.x, b ^= 1) {
        const long long cn = c + gridDim.x;
        // buffer b^1 was released by the barrier that ended the last chunk
        if (cn < nchunks && whole(cn)) {
            if (threadIdx.x == 0) issue(cn, b ^ 1);
            pend |= 2u >> b;   // bit b^1
        }
        const long long r0 = c * KP;
        const int cnt = (int)min((long long)KP, n - r0);
        float *sp = sm + 3 * KP * b;
        float *sw = sm + 6 * KP + WS * b;
        if (pend & (1u << b)) {
            const unsigned ph = (parity >> b) & 1u;
            const bool ok = mbar_wait_parity(&s_bar[b], ph);
            parity ^= 1u << b;
            pend &= ~(1u << b);
            if (__syncthreads_or(!ok)) {
                // a copy did not complete: record it, give each copy in
                // flight one more bounded wait, and leave
                if (threadIdx.x == 0) atomicOr(status, kStatusWaitTimeout);
                mbar_wait_parity(&s_bar[b], ph);
                if (pend) mbar_wait_parity(&s_bar[b ^ 1], (parity >> (b ^ 1)) & 1u);
                return;
            }
        } else {
            for (int j = threadIdx.x; j < 3 * cnt; j += blockDim.x) sp[j] = __ldcs(src + 3 * r0 + j);
            if (HAS_W)
                for (int j = threadIdx.x; j < cnt; j += blockDim.x) sw[j] = __ldcs(srcw + r0 + j);
            __syncthreads();
        }
        const long long r1 = r0 + cnt;
        long long seg0 = r0;
        while (seg0 < r1) {
            // ---- segment [seg0, seg1) with keys in [keybase, keybase + nkeys)
            long long seg1 = r1;
            int keybase = 0, nkeys = g.ncoarse;
            if (FINE) {
                if (threadIdx.x == 0) {
                    // coarse bucket holding position seg0: last c with start[c*F] <= seg0
                    int lo = 0, hi = g.ncoarse - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) / 2;
                        if ((long long)start[min(mid * g.F, g.ntiles)] <= seg0) lo = mid;
                        else hi = mid - 1;
                    }
                    const long long bend = start[min((lo + 1) * g.F, g.ntiles)];
                    s_seg[0] = lo;
                    s_seg[1] = bend < r1 ? bend : r1;
                }
                __syncthreads();
                const int cb = (int)s_seg[0];
                seg1 = s_seg[1];
                keybase = cb * g.F;
                nkeys = min(g.F, g.ntiles - keybase);
            }
            const int o = (int)(seg0 - r0);
            const int cs = (int)(seg1 - seg0);
            for (int k = threadIdx.x; k < nkeys; k += blockDim.x) hist[k] = 0u;
            __syncthreads();
            for (int i = threadIdx.x; i < cs; i += blockDim.x) {
                const float *q = sp + 3 * (o + i);
                const int t = tile_of<MAS>(q[0], q[1], q[2], inv, g);
                int key = FINE ? t - keybase : t >> g.sF;
                if (FINE && (unsigned)key >= (unsigned)nkeys) {
                    // not of this bucket: a slot the first pass left unwritten
                    // because the positions changed after the counting pass
                    atomicOr(status, kStatusInputChanged);
                    key = 0;
                }
                skey[i] = (unsigned short)key;
                atomicAdd(&hist[key], 1u);
            }
            __syncthreads();
            const unsigned hv = threadIdx.x < nkeys ? hist[threadIdx.x] : 0u;
            // Reserve the key's run in the destination now; the write-out is
            // the first to need it, so the atomic's round trip overlaps the
            // scan and the shared counting sort.
            unsigned my_base = 0u;
            if (hv) my_base = atomicAdd(&cursor[keybase + threadIdx.x], hv);
            const unsigned ex = block_exclusive_scan(hv, s_warp, nullptr);
            if (threadIdx.x < nkeys) {
                loff[threadIdx.x] = ex;
                lcur[threadIdx.x] = ex;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < cs; i += blockDim.x) {
                const int key = skey[i];
                const unsigned r = atomicAdd(&lcur[key], 1u);
                const float *q = sp + 3 * (o + i);
                sp2[3 * r] = q[0];
                sp2[3 * r + 1] = q[1];
                sp2[3 * r + 2] = q[2];
                if (HAS_W) sw2[r] = sw[o + i];
                skey2[r] = (unsigned short)key;
            }
            if (threadIdx.x < nkeys) {
                gbase[threadIdx.x] = my_base;
                // the key's region ends where the counting pass put the next
                // one; a run that would cross it (only when the positions
                // changed between the passes) is cut there and flagged
                const int kt = keybase + threadIdx.x;
                const unsigned end = FINE ? start[kt + 1] : start[min((kt + 1) * g.F, g.ntiles)];
                const unsigned room = my_base >= end ? 0u : min(hv, end - my_base);
                if (room < hv) atomicOr(status, kStatusInputChanged);
                groom[threadIdx.x] = room;
            }
            __syncthreads();
            // key runs are contiguous both here and in the destination; one
            // particle per thread: consecutive threads hold consecutive slots
            // of a run, so each of the three stores covers one span
            for (int e = threadIdx.x; e < cs; e += blockDim.x) {
                const int key = skey2[e];
                const unsigned j = (unsigned)e - loff[key];
                if (j >= groom[key]) continue;
                const size_t d = (size_t)gbase[key] + j;
                const float x = sp2[3 * e], y = sp2[3 * e + 1], z = sp2[3 * e + 2];
                dst[3 * d] = x;
                dst[3 * d + 1] = y;
                dst[3 * d + 2] = z;
                if (HAS_W) dstw[d] = sw2[e];
            }
            __syncthreads();
            seg0 = seg1;
        }
    }
}

// Count-free partition pass into fixed-capacity slots (the "capacity" sort,
// used when the previous request of the same kind showed the occupancy of
// tiles and coarse buckets; no counting pass, no scan).
//   FINE = false: keys are coarse buckets of the input particles; bucket c
//     owns dst[c * cap, (c + 1) * cap).
//   FINE = true: the input is the coarse pass's output -- bucket c's
//     particles are src[c * cap_in, c * cap_in + min(count_in[c], cap_in)) --
//     and the keys are the bucket's tiles; tile t owns dst[t * cap, ...).
// A key's cursor counts all its particles; the part of a run beyond the
// key's capacity goes to the spill list (spill[*spill_n ...]), which a
// global-atomic deposit adds to the grid.  Chunks never straddle buckets.
// Otherwise as k_partition: persistent CTAs, the next chunk fetched by a
// bulk copy while the current one is partitioned (bounded mbarrier waits),
// a shared counting sort, each key's run written contiguously.  Software
// pipelined over chunks: a chunk's key-ordered particles are written out
// during the next chunk, after that chunk's key phase, so each chunk's slot
// reservations (one global atomic per key) return while the previous chunk
// is written, its keys are scanned and its particles sorted; a chunk costs
// two CTA barriers (after its key phase, after its scan).
template <int MAS, bool HAS_W, bool FINE>
__global__ void __launch_bounds__(kPartThreads, PYL_PART_MINB)
k_partition_cap(const float *__restrict__ src, const float *__restrict__ srcw,
                const unsigned *__restrict__ count_in, unsigned cap_in, long long n,
                float *__restrict__ dst, float *__restrict__ dstw, unsigned cap,
                unsigned *__restrict__ cursor, float inv, TileGeom g, int bulk,
                float *__restrict__ spill, float *__restrict__ spillw,
                unsigned *__restrict__ spill_n, unsigned *__restrict__ status) {
    extern __shared__ __align__(16) float sm[];
    constexpr int WS = HAS_W ? KP : 0;
    constexpr int PT = KP / kPartThreads;   // particles of a chunk per thread
    static_assert(KP % kPartThreads == 0, "whole chunks per thread");
    static_assert(PT % 4 == 0, "four particles per group of three 16-byte loads");
    static_assert(kMaxKeys % 128 == 0 && kMaxKeys <= kPartThreads,
                  "the one-warp scan reads whole uint4 groups; one key per thread");
    float *sp2 = sm + 6 * KP + 2 * WS;                   // 3*KP in key order
    float *sw2 = sp2 + 3 * KP;
    unsigned short *skey = reinterpret_cast<unsigned short *>(sw2 + WS);
    unsigned short *skey2 = skey + KP;
    // key histograms, one per chunk parity (a chunk's histogram is cleared
    // after its scan, two barriers before the chunk after next uses it)
    unsigned *histb = reinterpret_cast<unsigned *>(skey2 + KP);   // 2 * kMaxKeys
    unsigned *gdiff = histb + 2 * kMaxKeys;   // slot of key-ordered element e: gdiff[key] + e
    unsigned *glim = gdiff + kMaxKeys;   // elements e < glim[key] fit their slots
    unsigned *gsp = glim + kMaxKeys;     // spill index of the others: gsp[key] + e
    unsigned *hex = gsp + kMaxKeys;      // each key's first position in key order
    unsigned *cpre = hex + kMaxKeys;                     // kMaxKeys + 1 (fine pass)
    unsigned *mcnt = cpre + kMaxKeys + 1;    // fine pass: particles of each bucket
    // fine pass: bucket of this CTA's k-th chunk (blockIdx.x + k * gridDim.x)
    unsigned char *ctab = reinterpret_cast<unsigned char *>(mcnt + kMaxKeys);
    __shared__ unsigned s_warp[32];
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ int s_fail;               // a bulk-copy wait gave up

    // chunks: the input in KP pieces (coarse), or each bucket's particles in
    // KP pieces (fine; cpre = exclusive prefix of the chunks per bucket)
    long long nchunks;
    if (FINE) {
        const int c = threadIdx.x;
        const unsigned cnt = c < g.ncoarse ? min(count_in[c], cap_in) : 0u;
        unsigned tot = 0;
        const unsigned ex = block_exclusive_scan((cnt + KP - 1) / KP, s_warp, &tot);
        if (c < g.ncoarse) {
            cpre[c] = ex;
            mcnt[c] = cnt;
        }
        if (c == 0) cpre[g.ncoarse] = tot;
        __syncthreads();
        nchunks = tot;
        // every chunk of this CTA mapped to its bucket up front, in parallel
        // (a binary search over the chunk prefix each), so that no thread
        // waits on one thread's search between chunks
        if ((long long)blockIdx.x < nchunks &&
            (nchunks - blockIdx.x + gridDim.x - 1) / gridDim.x > kChunkTab) {
            // (the host sizes the grid for the table: this does not happen)
            if (threadIdx.x == 0) atomicOr(status, kStatusInternal);
            return;
        }
        for (int k = threadIdx.x; k < kChunkTab; k += blockDim.x) {
            const long long v = blockIdx.x + (long long)k * gridDim.x;
            if (v >= nchunks) break;
            int lo = 0, hi = g.ncoarse - 1;            // last bucket b with cpre[b] <= v
            while (lo < hi) {
                const int mid = (lo + hi + 1) / 2;
                if ((long long)cpre[mid] <= v) lo = mid;
                else hi = mid - 1;
            }
            ctab[k] = (unsigned char)lo;
        }
    } else {
        nchunks = (n + KP - 1) / KP;
    }
    long long c = blockIdx.x;
    if (c >= nchunks) return;
    // chunk v (this CTA's kk-th) -> first particle, count, key base and key count
    auto map_chunk = [&](long long v, int kk, long long &r0, int &cnt, int &keybase, int &nkeys) {
        if (FINE) {
            const int lo = ctab[kk];
            const long long k = v - cpre[lo];
            const long long m = mcnt[lo];
            r0 = (long long)lo * cap_in + k * KP;
            cnt = (int)min((long long)KP, m - k * KP);
            keybase = lo * g.F;
            nkeys = min(g.F, g.ntiles - keybase);
        } else {
            r0 = v * KP;
            cnt = (int)min((long long)KP, n - r0);
            keybase = 0;
            nkeys = g.ncoarse;
        }
    };
    auto issue = [&](long long r0, int b) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&s_bar[b], (12u + (HAS_W ? 4u : 0u)) * KP);
        bulk_copy_g2s(sm + 3 * KP * b, src + 3 * r0, 12u * KP, &s_bar[b]);
        if (HAS_W) bulk_copy_g2s(sm + 6 * KP + WS * b, srcw + r0, 4u * KP, &s_bar[b]);
    };
    if (threadIdx.x == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        mbar_init_fence();
        s_fail = 0;
    }
    for (int k = threadIdx.x; k < 2 * kMaxKeys; k += blockDim.x) histb[k] = 0u;
    __syncthreads();   // (also publishes the fine pass's chunk table)
    unsigned parity = 0u, pend = 0u;
    long long r0;
    int cnt, keybase, nkeys;
    map_chunk(c, 0, r0, cnt, keybase, nkeys);
    if (bulk && cnt == KP) {
        if (threadIdx.x == 0) issue(r0, 0);
        pend |= 1u;
    }
    // a chunk's key-ordered particles -> their slots (or the spill list)
    auto write_out = [&](int wcnt, bool spilled) {
        if (!spilled) {
            // every run fits its slots (the common case)
            for (int e = threadIdx.x; e < wcnt; e += blockDim.x) {
                const int key = skey2[e];
                const size_t d = gdiff[key] + (unsigned)e;
                dst[3 * d] = sp2[3 * e];
                dst[3 * d + 1] = sp2[3 * e + 1];
                dst[3 * d + 2] = sp2[3 * e + 2];
                if (HAS_W) dstw[d] = sw2[e];
            }
            return;
        }
        for (int e = threadIdx.x; e < wcnt; e += blockDim.x) {
            const int key = skey2[e];
            const float x = sp2[3 * e], y = sp2[3 * e + 1], z = sp2[3 * e + 2];
            if ((unsigned)e < glim[key]) {
                const size_t d = gdiff[key] + (unsigned)e;
                dst[3 * d] = x;
                dst[3 * d + 1] = y;
                dst[3 * d + 2] = z;
                if (HAS_W) dstw[d] = sw2[e];
            } else {
                const size_t d = gsp[key] + (unsigned)e;
                spill[3 * d] = x;
                spill[3 * d + 1] = y;
                spill[3 * d + 2] = z;
                if (HAS_W) spillw[d] = sw2[e];
            }
        }
    };
    int prev_cnt = 0;   // particles of the previous chunk still to be written
    int my_spill = 0;   // this thread's key of that chunk overflowed its slots
    int b = 0, kk = 0;
    for (; c < nchunks; c += gridDim.x, b ^= 1, ++kk) {
        const long long cn = c + gridDim.x;
        long long nr0 = 0;
        int ncnt = 0, nkb = 0, nnk = 0;
        if (cn < nchunks) {
            map_chunk(cn, kk + 1, nr0, ncnt, nkb, nnk);
            if (bulk && ncnt == KP) {
                if (threadIdx.x == 0) issue(nr0, b ^ 1);
                pend |= 2u >> b;
            }
        }
        float *sp = sm + 3 * KP * b;
        float *sw = sm + 6 * KP + WS * b;
        unsigned *hist = histb + kMaxKeys * b;
        // Each thread waits for the bulk copy itself (its completed wait
        // makes the copied data visible to it) and goes on to the key phase;
        // a wait that gave up is reported through s_fail and the whole CTA
        // leaves after the next barrier.
        const bool was_bulk = (pend & (1u << b)) != 0;
        const unsigned ph = (parity >> b) & 1u;
        bool ok = true;
        if (was_bulk) {
            ok = mbar_wait_parity(&s_bar[b], ph);
            parity ^= 1u << b;
            pend &= ~(1u << b);
            if (!ok) s_fail = 1;
        } else {
            for (int j = threadIdx.x; j < 3 * cnt; j += blockDim.x) sp[j] = __ldcs(src + 3 * r0 + j);
            if (HAS_W)
                for (int j = threadIdx.x; j < cnt; j += blockDim.x) sw[j] = __ldcs(srcw + r0 + j);
            __syncthreads();
        }
        // (hist is zero here: cleared before the loop and after the scan of
        // the chunk before the previous one)
        // each thread's PT particles stay in registers from here to the
        // counting sort, with their key and their rank within the key (the
        // histogram atomic's old value)
        // (thread j takes the PT consecutive particles from PT * j: four
        // particles are three aligned 16-byte shared loads)
        // (weights too: the next bulk copy into this buffer may be issued
        // before the sort below is done)
        float px[PT], py[PT], pz[PT], pw[HAS_W ? PT : 1];
        int pk[PT];
        unsigned pr[PT];
        // (a whole chunk, the common case, takes the loop without the
        // per-particle bounds test)
        auto key_phase = [&](auto whole, auto p2) {
#pragma unroll
            for (int q4 = 0; q4 < PT / 4; ++q4) {
                const int i0 = PT * threadIdx.x + 4 * q4;
                const float4 *q = reinterpret_cast<const float4 *>(sp + 3 * i0);
                const float4 a = q[0], b4 = q[1], c4 = q[2];
                const float xs[4] = {a.x, a.w, b4.z, c4.y};
                const float ys[4] = {a.y, b4.x, b4.w, c4.z};
                const float zs[4] = {a.z, b4.y, c4.x, c4.w};
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int u = 4 * q4 + v;
                    pk[u] = -1;
                    if (decltype(whole)::value || i0 + v < cnt) {
                        px[u] = xs[v];
                        py[u] = ys[v];
                        pz[u] = zs[v];
                        if (HAS_W) pw[u] = sw[i0 + v];
                        const int t = tile_of_as<MAS>(p2, px[u], py[u], pz[u], inv, g);
                        pk[u] = FINE ? t - keybase : t >> g.sF;
                        pr[u] = atomicAdd(&hist[pk[u]], 1u);
                    }
                }
            }
        };
        if (!ok) {
#pragma unroll
            for (int u = 0; u < PT; ++u) pk[u] = -1;   // nothing of this chunk is read
        } else if (cnt == KP) {
            if (g.dmask >= 0) key_phase(std::true_type(), std::true_type());
            else key_phase(std::true_type(), std::false_type());
        } else {
            key_phase(std::false_type(), std::false_type());
        }
        // (the barrier also tells whether any run of the previous chunk
        // overflowed its slots)
        const bool spilled = __syncthreads_or(my_spill) != 0;
        if (s_fail) {
            // a bulk-copy wait gave up: wait (bounded) for the copies still
            // in flight into this CTA's buffers, then leave
            if (threadIdx.x == 0) atomicOr(status, kStatusWaitTimeout);
            if (was_bulk && !ok) mbar_wait_parity(&s_bar[b], ph);
            if (pend) mbar_wait_parity(&s_bar[b ^ 1], (parity >> (b ^ 1)) & 1u);
            return;
        }
        const unsigned hv = threadIdx.x < nkeys ? hist[threadIdx.x] : 0u;
        // reserve the key's run now; its value is first needed after the
        // counting sort, so the atomic's round trip overlaps the previous
        // chunk's write-out, the scan and the sort
        unsigned my_base = 0u;
        if (hv) my_base = atomicAdd(&cursor[keybase + threadIdx.x], hv);
        if (prev_cnt > 0) write_out(prev_cnt, spilled);
        if (threadIdx.x < 32) {
            // one warp scans the key counts (KPL consecutive keys per lane):
            // each key's first position in key order -> hex
            constexpr int KPL = kMaxKeys / 32;
            const int lane = threadIdx.x;
            unsigned cv[KPL], sum = 0u;
#pragma unroll
            for (int j = 0; j < KPL; j += 4) {
                const uint4 h4 = *reinterpret_cast<const uint4 *>(hist + lane * KPL + j);
                cv[j] = h4.x;
                cv[j + 1] = h4.y;
                cv[j + 2] = h4.z;
                cv[j + 3] = h4.w;
            }
#pragma unroll
            for (int j = 0; j < KPL; ++j) sum += cv[j];
            unsigned incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            unsigned run = incl - sum;
#pragma unroll
            for (int j = 0; j < KPL; j += 4) {
                uint4 e4;
                e4.x = run;
                run += cv[j];
                e4.y = run;
                run += cv[j + 1];
                e4.z = run;
                run += cv[j + 2];
                e4.w = run;
                run += cv[j + 3];
                *reinterpret_cast<uint4 *>(hex + lane * KPL + j) = e4;
            }
        }
        __syncthreads();
        // every read of this chunk's histogram and of the previous chunk's
        // key-ordered buffer and tables is behind the barrier
        for (int k = threadIdx.x; k < kMaxKeys; k += blockDim.x) hist[k] = 0u;   // chunk after next
#pragma unroll
        for (int u = 0; u < PT; ++u) {
            if (pk[u] >= 0) {
                const unsigned r = hex[pk[u]] + pr[u];
                sp2[3 * r] = px[u];
                sp2[3 * r + 1] = py[u];
                sp2[3 * r + 2] = pz[u];
                if (HAS_W) sw2[r] = pw[u];
                skey2[r] = (unsigned short)pk[u];
            }
        }
        my_spill = 0;
        if (threadIdx.x < nkeys) {
            const unsigned ex = hex[threadIdx.x];
            const unsigned room = my_base >= cap ? 0u : min(hv, cap - my_base);
            unsigned sb = 0u;
            if (hv > room) sb = atomicAdd(spill_n, hv - room);
            my_spill = hv > room;
            // unsigned arithmetic modulo 2^32: every slot and spill index is
            // below 2^32 (the host checks the slot arrays' sizes)
            gdiff[threadIdx.x] = (unsigned)(keybase + threadIdx.x) * cap + my_base - ex;
            glim[threadIdx.x] = ex + room;
            gsp[threadIdx.x] = sb - (ex + room);
        }
        // this chunk is written out during the next one (after its key
        // phase and barrier), or after the loop
        prev_cnt = cnt;
        r0 = nr0;
        cnt = ncnt;
        keybase = nkb;
        nkeys = nnk;
    }
    const bool spilled = __syncthreads_or(my_spill) != 0;
    if (prev_cnt > 0) write_out(prev_cnt, spilled);
}

// Single-pass alternative to the two partition passes: every particle takes
// the next slot of its tile with one atomic on the tile's global cursor
// (lanes of a warp that share a tile take one atomic for all of them).
// All writes of a tile happen at its advancing frontier, so the partially
// written sectors stay in L2 until they are complete.
// cap > 0 (the count-free sort): tile t owns dst[t * cap, (t + 1) * cap),
// cursor[t] counts its particles from 0, and a particle beyond the capacity
// goes to the spill list; mode is then not read.
template <int MAS, bool HAS_W>
__global__ void __launch_bounds__(256)
k_scatter_frontier(const float *__restrict__ src, const float *__restrict__ srcw, long long n,
                   float inv, TileGeom g, unsigned *__restrict__ cursor,
                   float *__restrict__ dst, float *__restrict__ dstw,
                   const unsigned *__restrict__ mode, unsigned cap,
                   float *__restrict__ spill, float *__restrict__ spillw,
                   unsigned *__restrict__ spill_n, const unsigned *__restrict__ start,
                   unsigned *__restrict__ status) {
    if (!cap && *mode != kSortFrontier) return;   // the whole grid takes the same branch
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (long long b = (long long)blockIdx.x * blockDim.x; b < n;
         b += (long long)gridDim.x * blockDim.x) {
        const long long i = b + threadIdx.x;
        const bool active = i < n;
        const unsigned live = __ballot_sync(0xffffffffu, active);
        if (!active) continue;
        const float x = __ldcs(src + 3 * i), y = __ldcs(src + 3 * i + 1),
                    z = __ldcs(src + 3 * i + 2);
        const int t = tile_of<MAS>(x, y, z, inv, g);
        const unsigned peers = __match_any_sync(live, t);
        const int leader = __ffs(peers) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&cursor[t], (unsigned)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        const unsigned r = base + __popc(peers & lt);
        if (!cap && r >= start[t + 1]) {
            // beyond the tile's counted region: the positions changed after
            // the counting pass
            atomicOr(status, kStatusInputChanged);
            continue;
        }
        if (!cap || r < cap) {
            const size_t slot = cap ? (size_t)t * cap + r : (size_t)r;
            dst[3 * slot] = x;
            dst[3 * slot + 1] = y;
            dst[3 * slot + 2] = z;
            if (HAS_W) dstw[slot] = __ldcs(srcw + i);
        } else {
            const size_t slot = atomicAdd(spill_n, 1u);
            spill[3 * slot] = x;
            spill[3 * slot + 1] = y;
            spill[3 * slot + 2] = z;
            if (HAS_W) spillw[slot] = __ldcs(srcw + i);
        }
    }
}

__device__ __forceinline__ void red_v4(float *addr, float a, float b, float c, float d) {
    asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};"
                 :: "l"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// Largest weight of one tap (product of the three axis weights) per scheme.
template <int MAS>
struct TapBound {
    static constexpr float WMAX = MAS == PYL_MAS_TSC ? 0.421875f          // 0.75^3
                                : MAS == PYL_MAS_PCS ? 0.2962963f         // (2/3)^3
                                                     : 1.0f;
};

// In place along one line of n ints (stride st):
//     a[j] <- sum of a[k] for k in [j - HI, j + LO]   (0 outside the line),
// the cells whose taps can reach cell j (taps lie at home + [-LO, HI]).
// The last LO + HI inputs are kept in registers while the line is rewritten.
// Counts (int) or sums of |W| (float, then each window is summed afresh so
// that no rounding drift builds up along the line).
template <int LO, int HI, typename T>
__device__ __forceinline__ T box_line(T *a, int n, int st, bool write) {
    constexpr int R = LO + HI + 1;
    T r[R];
#pragma unroll
    for (int q = 0; q < R; ++q) r[q] = T(0);
    T best = T(0);
    for (int k = 0; k < n + LO; ++k) {
        const T x = k < n ? a[k * st] : T(0);
#pragma unroll
        for (int q = 0; q + 1 < R; ++q) r[q] = r[q + 1];
        r[R - 1] = x;
        T sum = r[0];
#pragma unroll
        for (int q = 1; q < R; ++q) sum += r[q];
        const int j = k - LO;
        if (j >= 0) {
            if (write) a[j * st] = sum;
            // the largest window; a NaN (a NaN weight) sticks
            if (best == best && (sum > best || sum != sum)) best = sum;
        }
    }
    return best;
}

// Deposit: work items (tile, chunk) over a persistent grid; shared
// footprint, shared atomics, then a global flush of the footprint.
//
// FIXED: the footprint is accumulated in 32-bit integers, each tap rounded
// to a fixed point of scale 2^e.  A first pass over the item's particles
// histograms their home cells (counts, or sums of |W| for weighted
// particles).  A footprint cell can only be reached from the R^3 home cells
// around it, so no cell can exceed WMAX * R^3 * (largest home cell); where
// that leaves at least 21 fractional bits it sets the scale.  Otherwise
// (dense clumps) a box sum of the histogram over the stencil's reach gives,
// for every footprint cell, how much mass can reach it, and the largest box
// sum sets it.  2^e is the largest power of two keeping WMAX times the bound
// under 2^30.  An item whose bound is not finite (weights of inf or NaN)
// falls back to float atomics.
// Integer shared atomics run at about twice the rate of float ones, and the
// sums are exact (independent of the order of the atomics); the flush
// converts each cell once (int -> float rounding, then an exact scaling by
// 2^-e).
//
// COMP (PYL_COMPENSATED): float shared accumulators with a second footprint
// of TwoSum rounding errors (comp_add), merged into the grid and into the
// error grid glo with compensated global atomics.
constexpr int kAccFloat = 0, kAccFixed = 1, kAccComp = 2;

// Largest value over the CTA (a NaN anywhere gives NaN); all threads get it.
__device__ __forceinline__ float block_max_nan(float m, float *s_max) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float b = __shfl_xor_sync(0xffffffffu, m, o);
        m = (b > m || b != b) ? b : m;
    }
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    m = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
        m = (s_max[w] > m || s_max[w] != s_max[w]) ? s_max[w] : m;
    __syncthreads();   // s_max may be written again
    return m;
}

// Fixed-point exponent for footprint cells whose mass is at most m: the
// largest e with WMAX * m * 2^e < 2^30 (at most 30).  Float sums of |W| get
// a margin for their rounding.  False when m is not finite (inf or NaN
// weights): the item then accumulates in float.
template <int MAS, bool HAS_W>
__device__ __forceinline__ bool fixed_exponent(float m, int &e) {
    const float raw = TapBound<MAS>::WMAX * m * (HAS_W ? 1.001f : 1.f);
    if (!(raw < 1.0e30f)) return false;
    frexpf(fmaxf(raw, 1.f), &e);   // bound < 2^e
    e = min(30 - e, 30);
    return true;
}

// Work items: items[0 .. *nitems) over the exact sort's tile starts, or
// with cap_count (the count-free sort) the fixed grid of ntiles * ipt items
// (tile it / ipt, chunk it % ipt) over the tile slots of capT particles,
// tile t holding min(cap_count[t], capT) of them.
// Resident CTAs per SM the registers are held to: three for NGP / CIC
// (their footprints fit three to an SM), two for TSC / PCS and the
// compensated form (whose taps need up to 64 registers).
template <int MAS, int ACC>
constexpr int deposit_min_blocks() {
    return (ACC != kAccComp && (MAS == PYL_MAS_NGP || MAS == PYL_MAS_CIC)) ? 3 : 2;
}

template <int MAS, bool HAS_W, int ACC>
__global__ void __launch_bounds__(512, deposit_min_blocks<MAS, ACC>())
k_tile_deposit(const float *__restrict__ spos, const float *__restrict__ sw,
               const unsigned *__restrict__ start, const uint2 *__restrict__ items,
               const unsigned *__restrict__ nitems, float inv, TileGeom g,
               float *__restrict__ grid, int vec4, float *__restrict__ glo,
               const unsigned *__restrict__ cap_count, unsigned capT, unsigned ipt,
               const unsigned *__restrict__ status) {
    // the sort found that the positions changed under it: its tiles may hold
    // unwritten slots, so nothing is deposited (the call reports the error)
    if (*status & (kStatusInputChanged | kStatusInternal)) return;
    constexpr bool FIXED = ACC == kAccFixed;
    constexpr bool COMP = ACC == kAccComp;
    // Fewest fractional bits a fixed-point item may keep; an item whose bound
    // leaves fewer accumulates in float.  PCS: the deconvolution amplifies
    // the grid's rounding noise ~5e4-fold in the corner bins beyond the
    // Nyquist wavenumber, so a PCS item takes fixed point only where its
    // quantization noise (64 taps of at most 2^-25 each per cell) stays
    // below that of float32 accumulation; tiles holding dense halos keep
    // float atomics.  TSC keeps fixed point at any scale: requiring 25 bits
    // sent most 512^3 Zel'dovich tiles to float atomics (deposit 2.4 ->
    // 5.8 ms) and left the corner bins where they were -- those bins hold a
    // handful of modes and sit at the float32 noise of the FFT as much as of
    // the grid (the last bin: 3e-5 to 3e-4 of P0 over deposit variants and
    // runs, the reference's own summation orders 1e-5 to 5e-5).
    constexpr int MIN_BITS = MAS == PYL_MAS_PCS ? 24 : 0;
    using S = Stencil<MAS>;
    constexpr int NT = S::NT;
    extern __shared__ __align__(16) float s_reg[];
    int *s_int = reinterpret_cast<int *>(s_reg);
    // zeroes the first nf floats of the footprint (16-byte stores)
    auto zero_fp = [&](int nf) {
        float4 *s4 = reinterpret_cast<float4 *>(s_reg);
        for (int i = threadIdx.x; i < nf / 4; i += blockDim.x) s4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int i = (nf & ~3) + threadIdx.x; i < nf; i += blockDim.x) s_reg[i] = 0.f;
    };
    __shared__ float s_max[32];
    const int RX = g.RX, RY = g.RY, RZ = g.RZ;
    const int cells = RX * RY * RZ;
    const unsigned total = cap_count ? (unsigned)g.ntiles * ipt : *nitems;
    for (unsigned it = blockIdx.x; it < total; it += gridDim.x) {
        int t;
        long long p0, p1;
        if (cap_count) {
            t = (int)(it / ipt);
            const long long base = (long long)t * capT;
            p0 = base + (long long)(it % ipt) * kItemCap;
            p1 = min(base + (long long)min(cap_count[t], capT), p0 + (long long)kItemCap);
            if (p0 >= p1) continue;          // the whole CTA skips an empty chunk
        } else {
            const uint2 item = items[it];
            t = (int)item.x;
            p0 = (long long)start[t] + (long long)item.y * kItemCap;
            p1 = min((long long)start[t + 1], p0 + (long long)kItemCap);
        }
        zero_fp((COMP ? 2 : 1) * cells);
        const int tx = t / (g.nty * g.ntz), ty = (t / g.ntz) % g.nty, tz = t % g.ntz;
        const int ox = tx * g.TX, oy = ty * g.TY, oz = tz * g.TZ;   // tile origin (cells)
        __syncthreads();
        float scale = 1.f, inv_scale = 1.f;
        bool fixed = FIXED;   // this item in fixed point
        bool exact_mass = false;   // ... with per-particle mass-exact rounding
        if (FIXED) {
            // ---- home-cell occupancy (counts, or sums of |W|), the largest
            // home cell, and from it (or from box sums) the scale
            int lmi = 0;       // largest count this thread has seen
            float lmf = 0.f;   // ... or largest sum of |W| (a NaN sticks)
            auto occupy = [&](auto p2, float x, float y, float z, float w) {
                const int hx = wrap_as(p2, home_cell<MAS>(cell_dist(x, inv)), g);
                const int hy = wrap_as(p2, home_cell<MAS>(cell_dist(y, inv)), g);
                const int hz = wrap_as(p2, home_cell<MAS>(cell_dist(z, inv)), g);
                const int c = ((hx - ox + S::LO) * RY + (hy - oy + S::LO)) * RZ + (hz - oz + S::LO);
                if (HAS_W) {
                    const float o = atomicAdd(&s_reg[c], fabsf(w)) + fabsf(w);
                    lmf = (o > lmf || o != o) ? o : lmf;
                } else {
                    lmi = max(lmi, atomicAdd(&s_int[c], 1) + 1);
                }
            };
            // two particles per thread and step, both loaded first; the
            // grid's wrap chosen once per item
            auto occupy_all = [&](auto p2) {
            for (long long i = p0 + threadIdx.x; i < p1; i += 2 * blockDim.x) {
                const long long i2 = i + blockDim.x;
                const float x = __ldg(spos + 3 * i), y = __ldg(spos + 3 * i + 1),
                            z = __ldg(spos + 3 * i + 2);
                const float w = HAS_W ? __ldg(sw + i) : 1.f;
                float x2 = 0.f, y2 = 0.f, z2 = 0.f, w2 = 1.f;
                if (i2 < p1) {
                    x2 = __ldg(spos + 3 * i2);
                    y2 = __ldg(spos + 3 * i2 + 1);
                    z2 = __ldg(spos + 3 * i2 + 2);
                    if (HAS_W) w2 = __ldg(sw + i2);
                }
                occupy(p2, x, y, z, w);
                if (i2 < p1) occupy(p2, x2, y2, z2, w2);
            }
            };
            if (g.dmask >= 0) occupy_all(std::true_type());
            else occupy_all(std::false_type());
            // A footprint cell takes taps from the home cells of an R^3 box
            // only, so R^3 times the largest home cell bounds every cell.
            // Where that bound leaves fewer than FAST_BITS fractional bits,
            // the box sums of the histogram give the tight bound.  TSC and
            // PCS need 24 bits there: with R^3 = 27 or 64 the loose bound
            // costs them about two bits, and the 512^3 TSC corner bins beyond
            // the Nyquist wavenumber then moved from 1.4e-4 to 3.8e-4 of P0;
            // NGP / CIC keep the loose bound from 21 bits on (512^3 CIC:
            // worst bin 3.0e-6 -> 5.4e-6 of P0).
            constexpr int R = S::LO + S::HI + 1;
            constexpr int FAST_BITS = (MAS == PYL_MAS_TSC || MAS == PYL_MAS_PCS) ? 24 : 21;
            int e = 0;
            fixed = fixed_exponent<MAS, HAS_W>(
                block_max_nan(HAS_W ? lmf : (float)lmi, s_max) * (float)(R * R * R), e);
            if (fixed && e < FAST_BITS) {
                // separable box sums: z lines, y lines, then x lines (max only)
                using T = typename std::conditional<HAS_W, float, int>::type;
                T *hs = reinterpret_cast<T *>(s_reg);
                for (int l = threadIdx.x; l < RX * RY; l += blockDim.x)
                    box_line<S::LO, S::HI, T>(hs + l * RZ, RZ, 1, true);
                __syncthreads();
                for (int l = threadIdx.x; l < RX * RZ; l += blockDim.x)
                    box_line<S::LO, S::HI, T>(hs + (l / RZ) * RY * RZ + (l % RZ), RY, RZ, true);
                __syncthreads();
                float m = 0.f;
                for (int l = threadIdx.x; l < RY * RZ; l += blockDim.x) {
                    const float b = (float)box_line<S::LO, S::HI, T>(hs + l, RX, RY * RZ, false);
                    m = (b > m || b != b) ? b : m;        // keeps a NaN
                }
                fixed = fixed_exponent<MAS, HAS_W>(block_max_nan(m, s_max), e);
            }
            if (e < MIN_BITS) fixed = false;   // too coarse: float for this item
            zero_fp(cells);
            __syncthreads();
            if (fixed) {
                scale = ldexpf(1.f, e);
                inv_scale = ldexpf(1.f, -e);
                exact_mass = MIN_BITS < 20 && e < 20;
            }
        }
        // one particle: P2 -- power-of-two grid (mask wrap); M -- 0 fixed point,
        // 1 fixed point with mass-exact rounding, 2 float / compensated
        auto deposit_one = [&](auto p2, auto mode, float px, float py, float pz, float wt) {
            constexpr int M = decltype(mode)::value;
            int lx[NT], ly[NT], lz[NT];
            float wx[NT], wy[NT], wz[NT];
            {
                const float d = cell_dist(px, inv);
                const int c = home_cell<MAS>(d);
                const int base = wrap_as(p2, c, g) - ox + S::LO;
                int o[NT];
                axis_stencil<MAS>(d, c, o, wx);
#pragma unroll
                for (int j = 0; j < NT; ++j) lx[j] = base + o[j];
            }
            {
                const float d = cell_dist(py, inv);
                const int c = home_cell<MAS>(d);
                const int base = wrap_as(p2, c, g) - oy + S::LO;
                int o[NT];
                axis_stencil<MAS>(d, c, o, wy);
#pragma unroll
                for (int j = 0; j < NT; ++j) ly[j] = base + o[j];
            }
            {
                const float d = cell_dist(pz, inv);
                const int c = home_cell<MAS>(d);
                const int base = wrap_as(p2, c, g) - oz + S::LO;
                int o[NT];
                axis_stencil<MAS>(d, c, o, wz);
#pragma unroll
                for (int j = 0; j < NT; ++j) lz[j] = base + o[j];
            }
            if (M < 2) {
                // Each tap rounded to the item's fixed point.  In items whose
                // scale is coarse (dense clumps, 2^e < 2^20), the particle's
                // rounding residue -- its quantized mass minus the sum of its
                // quantized taps -- also goes to its largest tap, so that the
                // many tiny outer taps rounding to zero cannot bias the mass.
                if (M == 0) {
                    // the scale (a power of two) folded into the x weights:
                    // the same products, exactly, with NT^3 fewer multiplies
                    float wxs[NT];
#pragma unroll
                    for (int l = 0; l < NT; ++l) wxs[l] = wx[l] * scale;
#pragma unroll
                    for (int l = 0; l < NT; ++l)
#pragma unroll
                        for (int m = 0; m < NT; ++m) {
                            const float wxy = wxs[l] * wy[m];
                            const int row = (lx[l] * RY + ly[m]) * RZ;
#pragma unroll
                            for (int q = 0; q < NT; ++q) {
                                float v = wxy * wz[q];
                                if (HAS_W) v *= wt;
                                atomicAdd(s_int + row + lz[q], __float2int_rn(v));
                            }
                        }
                    return;
                }
                int sum = 0;
#pragma unroll
                for (int l = 0; l < NT; ++l)
#pragma unroll
                    for (int m = 0; m < NT; ++m) {
                        const float wxy = wx[l] * wy[m];
#pragma unroll
                        for (int q = 0; q < NT; ++q) {
                            float v = wxy * wz[q];
                            if (HAS_W) v *= wt;
                            sum += __float2int_rn(v * scale);
                        }
                    }
                int al = 0, am = 0, aq = 0;
#pragma unroll
                for (int j = 1; j < NT; ++j) {
                    if (wx[j] > wx[al]) al = j;
                    if (wy[j] > wy[am]) am = j;
                    if (wz[j] > wz[aq]) aq = j;
                }
                const int residue = (HAS_W ? __float2int_rn(wt * scale) : (int)scale) - sum;
#pragma unroll
                for (int l = 0; l < NT; ++l)
#pragma unroll
                    for (int m = 0; m < NT; ++m) {
                        const float wxy = wx[l] * wy[m];
                        const int row = (lx[l] * RY + ly[m]) * RZ;
#pragma unroll
                        for (int q = 0; q < NT; ++q) {
                            float v = wxy * wz[q];
                            if (HAS_W) v *= wt;
                            int iv = __float2int_rn(v * scale);
                            if (l == al && m == am && q == aq) iv += residue;
                            atomicAdd(s_int + row + lz[q], iv);
                        }
                    }
                return;
            }
#pragma unroll
            for (int l = 0; l < NT; ++l) {
#pragma unroll
                for (int m = 0; m < NT; ++m) {
                    const float wxy = wx[l] * wy[m];
                    const int row = (lx[l] * RY + ly[m]) * RZ;
#pragma unroll
                    for (int q = 0; q < NT; ++q) {
                        float v = wxy * wz[q];
                        if (HAS_W) v *= wt;
                        if (COMP) comp_add(s_reg + row + lz[q], s_reg + cells + row + lz[q], v);
                        else atomicAdd(s_reg + row + lz[q], v);
                    }
                }
            }
        };
        // two particles per thread and step, both loaded first; the form
        // of the item and the grid's wrap chosen once per item
        auto deposit_all = [&](auto p2, auto mode) {
        for (long long i = p0 + threadIdx.x; i < p1; i += 2 * blockDim.x) {
            const long long i2 = i + blockDim.x;
            const float x = __ldcs(spos + 3 * i), y = __ldcs(spos + 3 * i + 1),
                        z = __ldcs(spos + 3 * i + 2);
            const float w = HAS_W ? __ldcs(sw + i) : 1.f;
            float x2 = 0.f, y2 = 0.f, z2 = 0.f, w2 = 1.f;
            if (i2 < p1) {
                x2 = __ldcs(spos + 3 * i2);
                y2 = __ldcs(spos + 3 * i2 + 1);
                z2 = __ldcs(spos + 3 * i2 + 2);
                if (HAS_W) w2 = __ldcs(sw + i2);
            }
            deposit_one(p2, mode, x, y, z, w);
            if (i2 < p1) deposit_one(p2, mode, x2, y2, z2, w2);
        }
        };
        using Fix = std::integral_constant<int, 0>;
        using FixMass = std::integral_constant<int, 1>;
        using Flt = std::integral_constant<int, 2>;
        if (FIXED && fixed && (MIN_BITS >= 20 || !exact_mass)) {
            if (g.dmask >= 0) deposit_all(std::true_type(), Fix());
            else deposit_all(std::false_type(), Fix());
        } else if (FIXED && fixed) {
            deposit_all(std::false_type(), FixMass());
        } else {
            deposit_all(std::false_type(), Flt());
        }
        __syncthreads();
        // footprint cell value as a float
        auto cell = [&](int c) {
            return (FIXED && fixed) ? (float)s_int[c] * inv_scale : s_reg[c];
        };
        const int d = g.dims;
        const long long dd = (long long)d * d;
        const int zs = oz - S::LO;  // unwrapped global z of footprint column 0
        if (COMP) {
            for (int c = threadIdx.x; c < cells; c += blockDim.x) {
                const float v = s_reg[c], e = s_reg[cells + c];
                if (v == 0.f && e == 0.f) continue;
                const int lz = c % RZ, ly = (c / RZ) % RY, lx = c / (RZ * RY);
                const int gx = wrap_idx(ox - S::LO + lx, d);
                const int gy = wrap_idx(oy - S::LO + ly, d);
                const int gz = wrap_idx(zs + lz, d);
                const long long gi = gx * dd + (long long)gy * d + gz;
                comp_add(grid + gi, glo + gi, v);
                if (e != 0.f) atomicAdd(glo + gi, e);
            }
        } else if (vec4) {
            // quads aligned to the global z index (dims % 4 == 0: never wraps inside)
            const int q0 = (zs >= 0 ? zs : zs - 3) / 4;          // floor(zs / 4)
            const int q1 = (zs + RZ - 1 >= 0 ? zs + RZ - 1 : zs + RZ - 4) / 4;
            const int nq = q1 - q0 + 1;
            const int work = RX * RY * nq;
            // quad w = (lx * RY + ly) * nq + q; each step advances w by
            // blockDim.x, carried through (q, ly, lx) without divisions
            int q = threadIdx.x % nq, ly, lx;
            {
                const int r = threadIdx.x / nq;
                ly = r % RY;
                lx = r / RY;
            }
            const int sq = blockDim.x % nq, sr = blockDim.x / nq;
            const int sly = sr % RY, slx = sr / RY;
            for (int w = threadIdx.x; w < work; w += blockDim.x) {
                const int zq = 4 * (q0 + q);                      // unwrapped quad start
                const int row = (lx * RY + ly) * RZ;
                float v[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int lz = zq + e - zs;
                    v[e] = (lz >= 0 && lz < RZ) ? cell(row + lz) : 0.f;
                }
                if (v[0] != 0.f || v[1] != 0.f || v[2] != 0.f || v[3] != 0.f) {
                    const int gx = wrap_cell(ox - S::LO + lx, g);
                    const int gy = wrap_cell(oy - S::LO + ly, g);
                    const int gz = wrap_cell(zq, g);
                    red_v4(grid + gx * dd + (long long)gy * d + gz, v[0], v[1], v[2], v[3]);
                }
                q += sq;
                int carry = 0;
                if (q >= nq) { q -= nq; carry = 1; }
                ly += sly + carry;
                carry = 0;
                if (ly >= RY) { ly -= RY; carry = 1; }
                lx += slx + carry;
            }
        } else {
            for (int c = threadIdx.x; c < cells; c += blockDim.x) {
                const float v = cell(c);
                if (v == 0.f) continue;
                const int lz = c % RZ, ly = (c / RZ) % RY, lx = c / (RZ * RY);
                const int gx = wrap_idx(ox - S::LO + lx, d);
                const int gy = wrap_idx(oy - S::LO + ly, d);
                const int gz = wrap_idx(zs + lz, d);
                atomicAdd(grid + gx * dd + (long long)gy * d + gz, v);
            }
        }
        __syncthreads();   // the footprint is zeroed again by the next item
    }
}

template <typename K>
int set_smem(pyl_ctx *ctx, K kernel, size_t bytes) {
    if (bytes > 40 * 1024)   // static shared memory counts toward the 48 KB default too
        PYL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
    return PYL_OK;
}

// Tile shapes chosen by the autotuner (pyl_set_tile_shape), per (dims, MAS);
// make_geom's rule applies where none is set.
struct TileShape {
    int TX, TY, TZ, F;
};
std::mutex g_shape_mu;
std::map<std::pair<int, int>, TileShape> g_shape;

int ilog2_ceil(int v) {
    int s = 0;
    while ((1 << s) < v) ++s;
    return s;
}

// Fills the derived fields of a geometry with tile extents TX, TY, TZ and F
// tiles per coarse bucket (F = 0: ~sqrt(ntiles)).
void finish_geom(TileGeom &g, int dims, int mas, int F) {
    g.dims = dims;
    g.ntx = (dims + g.TX - 1) / g.TX;
    g.nty = (dims + g.TY - 1) / g.TY;
    g.ntz = (dims + g.TZ - 1) / g.TZ;
    g.ntiles = g.ntx * g.nty * g.ntz;
    g.sx = ilog2_ceil(g.TX);
    g.sy = ilog2_ceil(g.TY);
    g.sz = ilog2_ceil(g.TZ);
    const int lo = (mas == PYL_MAS_TSC || mas == PYL_MAS_PCS) ? 1 : 0;
    const int hi = (mas == PYL_MAS_TSC || mas == PYL_MAS_PCS) ? 2 : 1;
    g.RX = g.TX + lo + hi;
    g.RY = g.TY + lo + hi;
    g.RZ = g.TZ + lo + hi;
    if (F > 0) {
        g.F = F;
    } else {
        // coarse buckets: ~sqrt(ntiles) tiles each, at most kMaxKeys buckets
        g.F = 1;
        while ((long long)g.F * g.F < g.ntiles) g.F *= 2;
        while ((g.ntiles + g.F - 1) / g.F > kMaxKeys) g.F *= 2;
        if (g.F > kMaxKeys) g.F = kMaxKeys;
    }
    g.sF = ilog2_ceil(g.F);
    g.ncoarse = (g.ntiles + g.F - 1) / g.F;
    g.dmask = (dims & (dims - 1)) == 0 ? dims - 1 : -1;
}

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

TileGeom make_geom(int dims, int mas) {
    {
        std::lock_guard<std::mutex> lock(g_shape_mu);
        auto it = g_shape.find(std::make_pair(dims, mas));
        if (it != g_shape.end()) {
            TileGeom g;
            g.TX = it->second.TX;
            g.TY = it->second.TY;
            g.TZ = it->second.TZ;
            finish_geom(g, dims, mas, it->second.F);
            return g;
        }
    }
    TileGeom g;
    g.dims = dims;
    int p2 = 1;   // largest power of two <= dims, at most 32
    while (p2 * 2 <= dims && p2 < 32) p2 *= 2;
    g.TZ = p2;
    g.TY = p2;
    g.TX = dims >= 1024 ? 32 : (p2 >= 16 ? 16 : p2);
    auto count = [&](TileGeom &q) {
        q.ntx = (dims + q.TX - 1) / q.TX;
        q.nty = (dims + q.TY - 1) / q.TY;
        q.ntz = (dims + q.TZ - 1) / q.TZ;
        q.ntiles = q.ntx * q.nty * q.ntz;
    };
    count(g);
    // enough tiles to fill the GPU on small grids
    while (g.ntiles < 4 * 152 && (g.TY > 8 || g.TX > 8)) {
        if (g.TY >= g.TX && g.TY > 8) g.TY /= 2;
        else g.TX /= 2;
        count(g);
    }
    auto lg = [](int v) { int s = 0; while ((1 << s) < v) ++s; return s; };
    g.sx = lg(g.TX);
    g.sy = lg(g.TY);
    g.sz = lg(g.TZ);
    const int lo = (mas == PYL_MAS_TSC || mas == PYL_MAS_PCS) ? 1 : 0;
    const int hi = (mas == PYL_MAS_TSC || mas == PYL_MAS_PCS) ? 2 : 1;
    g.RX = g.TX + lo + hi;
    g.RY = g.TY + lo + hi;
    g.RZ = g.TZ + lo + hi;
    // coarse buckets: ~sqrt(ntiles) tiles each, at most kMaxKeys buckets
    g.F = 1;
    while ((long long)g.F * g.F < g.ntiles) g.F *= 2;
    while ((g.ntiles + g.F - 1) / g.F > kMaxKeys) g.F *= 2;
    if (g.F > kMaxKeys) g.F = kMaxKeys;
    g.sF = lg(g.F);
    g.ncoarse = (g.ntiles + g.F - 1) / g.F;
    g.dmask = (dims & (dims - 1)) == 0 ? dims - 1 : -1;
    return g;
}

// two input buffers, the key-ordered buffer, keys and per-key tables
size_t partition_smem(bool weighted) {
    return sizeof(float) * (9 * (size_t)KP + (weighted ? 3 * (size_t)KP : 0)) +
           sizeof(unsigned short) * 2 * (size_t)KP + sizeof(unsigned) * 5 * kMaxKeys;
}

// k_partition_cap: the same buffers, two key histograms, four per-key
// tables, the bucket chunk prefix and counts and the fine pass's chunk ->
// bucket table
size_t partition_cap_smem(bool weighted) {
    return sizeof(float) * (9 * (size_t)KP + (weighted ? 3 * (size_t)KP : 0)) +
           sizeof(unsigned short) * 2 * (size_t)KP + sizeof(unsigned) * (8 * kMaxKeys + 1) +
           kChunkTab;
}

unsigned round_up4(double v) {
    const unsigned u = (unsigned)ceil(v);
    return (u + 3u) & ~3u;
}

// The count-free sort (see pyl_ctx::SortPlan): fixed slots of capT particles
// per tile and capC per coarse bucket, sized from the occupancy the last
// exact sort of the same kind showed, a spill list for what does not fit.
template <int MAS, bool HAS_W>
int launch_capacity_t(pyl_ctx *ctx, const float *pos, long long n, const float *W,
                      float *grid, int dims, float inv, const TileGeom &g, int mode,
                      unsigned capT, unsigned capC, int acc, int sms) {
    int st = PYL_OK;
    const int nt = g.ntiles;
    const bool two_pass = mode != kSortFrontier;
    unsigned *info = (unsigned *)ws_get(ctx, "dep_info", 4 * sizeof(unsigned), &st);
    if (!info) return st;
    unsigned *spill_n = info + 3;
    unsigned *fcur = (unsigned *)ws_get(ctx, "dep_fcur", sizeof(unsigned) * (size_t)nt, &st);
    if (!fcur) return st;
    unsigned *ccur = (unsigned *)ws_get(ctx, "dep_ccur", sizeof(unsigned) * (size_t)g.ncoarse, &st);
    if (!ccur) return st;
    float *b1 = nullptr, *w1 = nullptr, *w2 = nullptr, *spw = nullptr;
    const size_t nb1 = (size_t)g.ncoarse * capC, nb2 = (size_t)nt * capT;
    if (two_pass) {
        b1 = (float *)ws_get(ctx, "dep_b1", sizeof(float) * 3 * nb1, &st);
        if (!b1) return st;
    }
    float *b2 = (float *)ws_get(ctx, "dep_b2", sizeof(float) * 3 * nb2, &st);
    if (!b2) return st;
    float *sp = (float *)ws_get(ctx, "dep_spill", sizeof(float) * 3 * (size_t)n, &st);
    if (!sp) return st;
    if (HAS_W) {
        if (two_pass) {
            w1 = (float *)ws_get(ctx, "dep_w1", sizeof(float) * nb1, &st);
            if (!w1) return st;
        }
        w2 = (float *)ws_get(ctx, "dep_w2", sizeof(float) * nb2, &st);
        if (!w2) return st;
        spw = (float *)ws_get(ctx, "dep_spillw", sizeof(float) * (size_t)n, &st);
        if (!spw) return st;
    }
    PYL_CUDA(ctx, cudaMemsetAsync(info, 0, 4 * sizeof(unsigned), ctx->stream));
    PYL_CUDA(ctx, cudaMemsetAsync(fcur, 0, sizeof(unsigned) * (size_t)nt, ctx->stream));
    {
        StageScope s(ctx, ST_SORT);
        if (two_pass) {
            PYL_CUDA(ctx, cudaMemsetAsync(ccur, 0, sizeof(unsigned) * (size_t)g.ncoarse,
                                          ctx->stream));
            const size_t psm = partition_cap_smem(HAS_W);
            if ((st = set_smem(ctx, k_partition_cap<MAS, HAS_W, false>, psm))) return st;
            if ((st = set_smem(ctx, k_partition_cap<MAS, HAS_W, true>, psm))) return st;
            static int per_sm = 0;
            if (!per_sm) {
                PYL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                  &per_sm, k_partition_cap<MAS, HAS_W, true>, kPartThreads, psm));
                if (per_sm < 1) per_sm = 1;
            }
            const unsigned nblk = (unsigned)std::min<long long>((n + KP - 1) / KP,
                                                                (long long)per_sm * sms);
            // the fine pass maps at most kChunkTab chunks per CTA: it has at
            // most n / KP + ncoarse chunks (every bucket's last one partial)
            if ((n / KP + g.ncoarse + 1 + nblk - 1) / nblk > kChunkTab)
                return fail(ctx, PYL_ERR_UNSUPPORTED, "too many particles for the count-free sort");
            const int bulk_in = ((uintptr_t)pos & 15) == 0 && (!W || ((uintptr_t)W & 15) == 0);
            k_partition_cap<MAS, HAS_W, false><<<nblk, kPartThreads, psm, ctx->stream>>>(
                pos, W, nullptr, 0u, n, b1, w1, capC, ccur, inv, g, bulk_in, sp, spw, spill_n,
                ctx->d_status);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
            k_partition_cap<MAS, HAS_W, true><<<nblk, kPartThreads, psm, ctx->stream>>>(
                b1, w1, ccur, capC, n, b2, w2, capT, fcur, inv, g, 1, sp, spw, spill_n,
                ctx->d_status);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
        } else {
            long long blocks = (n + 255) / 256;
            if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
            k_scatter_frontier<MAS, HAS_W><<<(unsigned)blocks, 256, 0, ctx->stream>>>(
                pos, W, n, inv, g, fcur, b2, w2, nullptr, capT, sp, spw, spill_n, nullptr,
                ctx->d_status);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
        }
    }
    const int vec4 = (dims % 4 == 0 && ((uintptr_t)grid & 15) == 0) ? 1 : 0;
    const size_t rsm = sizeof(float) * (size_t)g.RX * g.RY * g.RZ;
    const unsigned ipt = (capT + kItemCap - 1) / kItemCap;
    auto run = [&](auto kernel) -> int {
        int st2;
        if ((st2 = set_smem(ctx, kernel, rsm))) return st2;
        int per_sm = 0;
        PYL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 512, rsm));
        long long grid_n = (long long)(per_sm > 0 ? per_sm : 1) * sms * 4;
        if (grid_n > (long long)nt * ipt) grid_n = (long long)nt * ipt;
        if ((st2 = wait_grid(ctx))) return st2;
        StageScope s(ctx, ST_DEPOSIT);
        kernel<<<(unsigned)grid_n, 512, rsm, ctx->stream>>>(b2, w2, nullptr, nullptr, nullptr, inv,
                                                           g, grid, vec4, nullptr, fcur, capT, ipt,
                                                           ctx->d_status);
        ctx->launches++;
        PYL_CUDA(ctx, cudaGetLastError());
        return PYL_OK;
    };
    if ((st = acc == kAccFixed ? run(k_tile_deposit<MAS, HAS_W, kAccFixed>)
                               : run(k_tile_deposit<MAS, HAS_W, kAccFloat>)))
        return st;
    // the particles beyond their slots (none unless the occupancy grew)
    k_deposit_atomic<MAS, HAS_W, float, false><<<152 * 8, kThreads, 0, ctx->stream>>>(
        sp, n, 3, spw, grid, dims, inv, nullptr, spill_n);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    ctx->sort_used.cap = true;
    ctx->d_sort_info = info;
    return PYL_OK;
}

template <int MAS, bool HAS_W>
int launch_sorted_t(pyl_ctx *ctx, const float *pos, long long n, const float *W, float *grid,
                    int dims, float inv, const TileGeom &g, int forced_mode, int acc,
                    float *glo) {
    int st = PYL_OK;
    const int nt = g.ntiles;
    const bool two_pass = forced_mode != kSortFrontier;   // may be chosen on the device
    // device scratch: counts/starts (nt+1), cursors, item bookkeeping
    unsigned *start = (unsigned *)ws_get(ctx, "dep_start", sizeof(unsigned) * (size_t)(nt + 1), &st);
    if (!start) return st;
    unsigned *flags2 = (unsigned *)ws_get(ctx, "dep_mode", 2 * sizeof(unsigned), &st);
    if (!flags2) return st;
    unsigned *distinct = flags2, *mode = flags2 + 1;
    unsigned *fcur = (unsigned *)ws_get(ctx, "dep_fcur", sizeof(unsigned) * (size_t)nt, &st);
    if (!fcur) return st;
    unsigned *ccur = (unsigned *)ws_get(ctx, "dep_ccur", sizeof(unsigned) * (size_t)g.ncoarse, &st);
    if (!ccur) return st;
    unsigned *nchunk = (unsigned *)ws_get(ctx, "dep_nchunk", sizeof(unsigned) * (size_t)(nt + 1), &st);
    if (!nchunk) return st;
    const size_t max_items = (size_t)nt + (size_t)(n / kItemCap) + 1;
    uint2 *items = (uint2 *)ws_get(ctx, "dep_items", sizeof(uint2) * max_items, &st);
    if (!items) return st;
    unsigned *nitems = (unsigned *)ws_get(ctx, "dep_nitems", sizeof(unsigned), &st);
    if (!nitems) return st;
    unsigned *info = (unsigned *)ws_get(ctx, "dep_info", 4 * sizeof(unsigned), &st);
    if (!info) return st;
    float *b1 = nullptr, *w1 = nullptr, *w2 = nullptr;
    if (two_pass) {
        b1 = (float *)ws_get(ctx, "dep_b1", sizeof(float) * 3 * (size_t)n, &st);
        if (!b1) return st;
    }
    float *b2 = (float *)ws_get(ctx, "dep_b2", sizeof(float) * 3 * (size_t)n, &st);
    if (!b2) return st;
    if (HAS_W) {
        if (two_pass) {
            w1 = (float *)ws_get(ctx, "dep_w1", sizeof(float) * (size_t)n, &st);
            if (!w1) return st;
        }
        w2 = (float *)ws_get(ctx, "dep_w2", sizeof(float) * (size_t)n, &st);
        if (!w2) return st;
    }
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    {
        StageScope s(ctx, ST_BINS);
        PYL_CUDA(ctx, cudaMemsetAsync(start, 0, sizeof(unsigned) * (size_t)(nt + 1), ctx->stream));
        PYL_CUDA(ctx, cudaMemsetAsync(flags2, 0, 2 * sizeof(unsigned), ctx->stream));
        PYL_CUDA(ctx, cudaMemsetAsync(info, 0, 4 * sizeof(unsigned), ctx->stream));
        const size_t hsm = sizeof(unsigned) * (size_t)nt;
        if (((uintptr_t)pos & 15) == 0) {
            if ((st = set_smem(ctx, k_tile_count4<MAS>, hsm))) return st;
            k_tile_count4<MAS><<<sms, 1024, hsm, ctx->stream>>>(
                reinterpret_cast<const float4 *>(pos), pos, n, inv, g, start, distinct);
        } else {
            if ((st = set_smem(ctx, k_tile_count<MAS>, hsm))) return st;
            k_tile_count<MAS><<<sms, 1024, hsm, ctx->stream>>>(pos, n, inv, g, start, distinct);
        }
        ctx->launches++;
        PYL_CUDA(ctx, cudaGetLastError());
        // exclusive scan over nt+1 entries (the extra 0 becomes the total n)
        if ((st = scan_exclusive(ctx, start, nt + 1))) return st;
        k_sort_setup<<<(nt + 255) / 256, 256, 0, ctx->stream>>>(start, nt, g.F, g.ncoarse, fcur,
                                                                ccur, nchunk, n, distinct,
                                                                forced_mode, mode, info);
        ctx->launches++;
        PYL_CUDA(ctx, cudaGetLastError());
        PYL_CUDA(ctx, cudaMemsetAsync(nchunk + nt, 0, sizeof(unsigned), ctx->stream));
        if ((st = scan_exclusive(ctx, nchunk, nt + 1))) return st;
        k_items<<<(nt + 255) / 256, 256, 0, ctx->stream>>>(nchunk, start, nt, items, nitems);
        ctx->launches++;
        PYL_CUDA(ctx, cudaGetLastError());
    }
    {
        StageScope s(ctx, ST_SORT);
        // Both sorts are enqueued unless one is forced; each kernel reads the
        // mode chosen on the device and the other one returns at once.
        if (two_pass) {
            const size_t psm = partition_smem(HAS_W);
            if ((st = set_smem(ctx, k_partition<MAS, HAS_W, false>, psm))) return st;
            if ((st = set_smem(ctx, k_partition<MAS, HAS_W, true>, psm))) return st;
            static int per_sm = 0;   // resident partition CTAs per SM (same for both passes)
            if (!per_sm) {
                PYL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                                  &per_sm, k_partition<MAS, HAS_W, true>, kPartThreads, psm));
                if (per_sm < 1) per_sm = 1;
            }
            const long long nchunks = (n + KP - 1) / KP;
            const unsigned nblk = (unsigned)std::min<long long>(nchunks, (long long)per_sm * sms);
            // bulk copies need 16-byte aligned sources (the workspaces are)
            const int bulk_in = ((uintptr_t)pos & 15) == 0 && (!W || ((uintptr_t)W & 15) == 0);
            k_partition<MAS, HAS_W, false><<<nblk, kPartThreads, psm, ctx->stream>>>(
                pos, W, b1, w1, n, inv, g, ccur, start, mode, bulk_in, ctx->d_status);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
            k_partition<MAS, HAS_W, true><<<nblk, kPartThreads, psm, ctx->stream>>>(
                b1, w1, b2, w2, n, inv, g, fcur, start, mode, 1, ctx->d_status);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
        }
        if (forced_mode != kSortTwoPass) {
            long long blocks = (n + 255) / 256;
            if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
            k_scatter_frontier<MAS, HAS_W><<<(unsigned)blocks, 256, 0, ctx->stream>>>(
                pos, W, n, inv, g, fcur, b2, w2, mode, 0u, nullptr, nullptr, nullptr, start,
                ctx->d_status);
            ctx->launches++;
            PYL_CUDA(ctx, cudaGetLastError());
        }
    }
    const int vec4 = (dims % 4 == 0 && ((uintptr_t)grid & 15) == 0) ? 1 : 0;
    const size_t rsm =
        sizeof(float) * (size_t)g.RX * g.RY * g.RZ * (acc == kAccComp ? 2 : 1);
    auto run = [&](auto kernel) -> int {
        int st2;
        if ((st2 = set_smem(ctx, kernel, rsm))) return st2;
        int per_sm = 0;
        PYL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 512, rsm));
        long long grid_n = (long long)(per_sm > 0 ? per_sm : 1) * sms * 4;
        if (grid_n > (long long)max_items) grid_n = (long long)max_items;
        if ((st2 = wait_grid(ctx))) return st2;
        StageScope s(ctx, ST_DEPOSIT);
        kernel<<<(unsigned)grid_n, 512, rsm, ctx->stream>>>(b2, w2, start, items, nitems, inv, g,
                                                           grid, vec4, glo, nullptr, 0u, 1u,
                                                           ctx->d_status);
        ctx->launches++;
        PYL_CUDA(ctx, cudaGetLastError());
        return PYL_OK;
    };
    ctx->sort_used.cap = false;
    ctx->d_sort_info = info;
    if (acc == kAccComp) return run(k_tile_deposit<MAS, HAS_W, kAccComp>);
    if (acc == kAccFixed) return run(k_tile_deposit<MAS, HAS_W, kAccFixed>);
    return run(k_tile_deposit<MAS, HAS_W, kAccFloat>);
}

template <int MAS>
int launch_sorted(pyl_ctx *ctx, const float *pos, long long n, const float *W, float *grid,
                  int dims, float inv, int flags, float *glo) {
    const TileGeom g = make_geom(dims, MAS);
    const int forced = (flags & PYL_SORT_TWO_PASS) ? kSortTwoPass
                       : (flags & PYL_SORT_FRONTIER) ? kSortFrontier : -1;
    // Compensated if asked for; else fixed point (PCS: per item, where the
    // scale keeps at least 24 fractional bits) unless float atomics are
    // asked for.
    const int acc = glo ? kAccComp : !(flags & PYL_DEPOSIT_FLOAT) ? kAccFixed : kAccFloat;
    ctx->sort_used = pyl_ctx::SortUsed();
    ctx->sort_used.valid = true;
    ctx->sort_used.n = n;
    ctx->sort_used.ntiles = g.ntiles;
    ctx->sort_used.F = g.F;
    ctx->sort_used.plan = ctx->sort_hint;
    // the count-free sort where the last request of this kind allows it
    const pyl_ctx::SortPlan plan = ctx->sort_hint ? read_sort_plan(ctx->sort_hint)
                                                  : pyl_ctx::SortPlan();
    if (plan.cap && acc != kAccComp && !(flags & PYL_SORT_EXACT)) {
        const double mean_t = (double)n / g.ntiles;
        const unsigned capT = round_up4(plan.phiT * mean_t + 32.0);
        const unsigned capC = round_up4(plan.phiC * mean_t * g.F + KP);
        const int mode = forced >= 0 ? forced : plan.mode;
        if ((double)capT * g.ntiles < 4.0e9 && (double)capC * g.ncoarse < 4.0e9 &&
            (mode == kSortFrontier || mode == kSortTwoPass)) {
            int sms = 152;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
            return W ? launch_capacity_t<MAS, true>(ctx, pos, n, W, grid, dims, inv, g, mode, capT,
                                                    capC, acc, sms)
                     : launch_capacity_t<MAS, false>(ctx, pos, n, W, grid, dims, inv, g, mode,
                                                     capT, capC, acc, sms);
        }
    }
    return W ? launch_sorted_t<MAS, true>(ctx, pos, n, W, grid, dims, inv, g, forced, acc, glo)
             : launch_sorted_t<MAS, false>(ctx, pos, n, W, grid, dims, inv, g, forced, acc, glo);
}

bool use_sorted(long long n, int coord, int dims, int mas, int flags) {
    if (coord != 3) return false;
    if (flags & PYL_DEPOSIT_ATOMIC) return false;
    const TileGeom g = make_geom(dims, mas);
    const size_t rsm = sizeof(float) * (size_t)g.RX * g.RY * g.RZ *
                       ((flags & PYL_COMPENSATED) ? 2 : 1);
    if (rsm > 200 * 1024 || (size_t)g.ntiles * 4 > 200 * 1024) return false;
    if (g.F > 65535 || g.ncoarse > kMaxKeys) return false;
    if (n >= (1LL << 32) - 1) return false;
    if (flags & PYL_DEPOSIT_SORTED) return true;
    return n >= (1LL << 20) && dims >= 32;
}

}  // namespace

template <typename G>
static int deposit_t(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                     G *grid, int dims, float BoxSize, int mas, int flags) {
    if (mas < PYL_MAS_NGP || mas > PYL_MAS_PCS)
        return fail(ctx, PYL_ERR_ARG, "option not valid!!! (MAS must be NGP, CIC, TSC or PCS)");
    ctx->sort_used = pyl_ctx::SortUsed();   // set by the sorted path below
    if (n == 0) return PYL_OK;
    // inv_cell_size = dims/BoxSize as a float division (MAS_library.pyx:135)
    const float inv = (float)dims / BoxSize;
    int st = PYL_OK;
    // compensated float32 deposit: rounding errors into lo, folded at the end
    float *lo = nullptr;
    const long long cells = (long long)dims * dims * (coord == 3 ? dims : 1);
    if (sizeof(G) == sizeof(float) && (flags & PYL_COMPENSATED)) {
        lo = (float *)ws_get(ctx, "dep_lo", sizeof(float) * (size_t)cells, &st);
        if (!lo) return st;
        PYL_CUDA(ctx, cudaMemsetAsync(lo, 0, sizeof(float) * (size_t)cells, ctx->stream));
    }
    if (sizeof(G) == sizeof(float) && use_sorted(n, coord, dims, mas, flags)) {
        float *gf = reinterpret_cast<float *>(grid);
        switch (mas) {
            case PYL_MAS_NGP: st = launch_sorted<PYL_MAS_NGP>(ctx, pos, n, W, gf, dims, inv, flags, lo); break;
            case PYL_MAS_CIC: st = launch_sorted<PYL_MAS_CIC>(ctx, pos, n, W, gf, dims, inv, flags, lo); break;
            case PYL_MAS_TSC: st = launch_sorted<PYL_MAS_TSC>(ctx, pos, n, W, gf, dims, inv, flags, lo); break;
            default: st = launch_sorted<PYL_MAS_PCS>(ctx, pos, n, W, gf, dims, inv, flags, lo); break;
        }
    } else {
        switch (mas) {
            case PYL_MAS_NGP: st = launch_atomic<PYL_MAS_NGP>(ctx, pos, n, coord, W, grid, dims, inv, lo); break;
            case PYL_MAS_CIC: st = launch_atomic<PYL_MAS_CIC>(ctx, pos, n, coord, W, grid, dims, inv, lo); break;
            case PYL_MAS_TSC: st = launch_atomic<PYL_MAS_TSC>(ctx, pos, n, coord, W, grid, dims, inv, lo); break;
            default: st = launch_atomic<PYL_MAS_PCS>(ctx, pos, n, coord, W, grid, dims, inv, lo); break;
        }
    }
    if (st || !lo) return st;
    long long blocks = (cells + kThreads - 1) / kThreads;
    if (blocks > 152LL * 32) blocks = 152LL * 32;
    k_fold_lo<<<(unsigned)blocks, kThreads, 0, ctx->stream>>>(reinterpret_cast<float *>(grid), lo,
                                                             cells);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

int deposit(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
            float *grid, int dims, float BoxSize, int mas, int flags) {
    return deposit_t(ctx, pos, n, coord, W, grid, dims, BoxSize, mas, flags);
}

int deposit_f64(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                double *grid, int dims, float BoxSize, int mas) {
    return deposit_t(ctx, pos, n, coord, W, grid, dims, BoxSize, mas, PYL_DEPOSIT_ATOMIC);
}

int scale_grid(pyl_ctx *ctx, float *grid, int64_t count, float s) {
    return scale_t<float>(ctx, grid, count, s);
}

namespace {

__global__ void __launch_bounds__(256)
k_wsum(const float *__restrict__ W, long long n, double *__restrict__ mass) {
    // float partial sums per thread (the mass only sets the FFT shift, whose
    // rounding the k = 0 mode corrects exactly), double across threads, one
    // atomic per CTA
    __shared__ double s_w[32];
    float f = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        f += __ldcs(W + i);
    double s = (double)f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_w[w];
        if (t != 0.0) atomicAdd(mass, t);
    }
}

__global__ void k_shift(double *mass, long long n, int weighted, double inv_cells,
                        float *shift) {
    if (!weighted) *mass = (double)n;
    *shift = (float)(*mass * inv_cells);
}

}  // namespace

int mass_and_shift(pyl_ctx *ctx, const float *W, int64_t n, double cells, double *mass,
                   float *shift) {
    if (W) {
        long long blocks = (n + 255) / 256;
        if (blocks > 152LL * 8) blocks = 152LL * 8;
        if (blocks < 1) blocks = 1;
        k_wsum<<<(unsigned)blocks, 256, 0, ctx->stream>>>(W, n, mass);
        ctx->launches++;
    }
    k_shift<<<1, 1, 0, ctx->stream>>>(mass, n, W ? 1 : 0, 1.0 / cells, shift);
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

int scale_grid_f64(pyl_ctx *ctx, double *grid, int64_t count, double s) {
    return scale_t<double>(ctx, grid, count, s);
}

}  // namespace pyl

using pyl::TileGeom;

extern "C" {

int pyl_set_tile_shape(int dims, int mas, int TX, int TY, int TZ, int F) {
    if (dims < 2 || mas < PYL_MAS_NGP || mas > PYL_MAS_PCS) return PYL_ERR_ARG;
    const auto key = std::make_pair(dims, mas);
    std::lock_guard<std::mutex> lock(pyl::g_shape_mu);
    if (TX == 0) {
        pyl::g_shape.erase(key);
        return PYL_OK;
    }
    if (!pyl::pow2(TX) || !pyl::pow2(TY) || !pyl::pow2(TZ) || TX > 64 || TY > 64 || TZ > 64 ||
        (F != 0 && (!pyl::pow2(F) || F > pyl::kMaxKeys)))
        return PYL_ERR_ARG;
    TileGeom g;
    g.TX = TX;
    g.TY = TY;
    g.TZ = TZ;
    pyl::finish_geom(g, dims, mas, F);
    // the sorted deposit's limits: footprint and tile histogram in shared
    // memory, at most kMaxKeys keys per partition pass
    if (sizeof(float) * (size_t)g.RX * g.RY * g.RZ > 200 * 1024 ||
        (size_t)g.ntiles * 4 > 200 * 1024 || g.ncoarse > pyl::kMaxKeys || g.F > pyl::kMaxKeys)
        return PYL_ERR_UNSUPPORTED;
    pyl::g_shape[key] = pyl::TileShape{TX, TY, TZ, g.F};
    return PYL_OK;
}

int pyl_get_tile_shape(int dims, int mas, int *TX, int *TY, int *TZ, int *F) {
    if (dims < 2 || !TX || !TY || !TZ || !F) return PYL_ERR_ARG;
    const TileGeom g = pyl::make_geom(dims, mas);
    *TX = g.TX;
    *TY = g.TY;
    *TZ = g.TZ;
    *F = g.F;
    return PYL_OK;
}

}  // extern "C"
