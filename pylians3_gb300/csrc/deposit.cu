// Particle deposit (mass assignment) NGP / CIC / TSC / PCS, with optional
// weights, 3D and 2D.  Replaces MAS_library.pyx:123-545 (NGP..PCSW) and the
// C kernels of MAS_c.c:8-266.  The per-axis stencil is in deposit_common.cuh.
//
// Two paths:
//  * unsorted: one thread per particle, one global float atomic (RED) per
//    tap.  Used for small inputs, 2D, float64 grids, and inputs whose order is
//    already spatially coherent enough for L2 to absorb the atomics.
//  * tile-sorted (3D float32): particles are counting-sorted by the tile of
//    their home cell (tiles of TX*TY*TZ cells), each tile's footprint
//    (tile + stencil halo) is accumulated in shared memory with shared
//    atomics, and the footprint is added to the grid with vectorised global
//    reductions (red.global.add.v4.f32).  Sort: per-block tile histograms
//    (block-major chunks of the particle array), one exclusive scan over the
//    tile-major (tile, block) count matrix, and a scatter whose destination is
//    offset[tile][block] + a shared-memory cursor -- no global atomics.
//
// 2D (coord = 2) follows MA's expand_dims path: the third axis has extent 1,
// index 0 and weight 1 for every tap, so a particle is deposited 2/3/4 times
// onto the same plane for CIC/TSC/PCS (and renormalised by the caller).
#include "deposit_common.cuh"

namespace pyl {

namespace {

constexpr int kThreads = 256;

// ------------------------------------------------------------ unsorted path
template <int MAS, bool HAS_W, typename G>
__global__ void __launch_bounds__(kThreads)
k_deposit_atomic(const float *__restrict__ pos, long long n, int coord,
                 const float *__restrict__ W, G *__restrict__ grid, int dims,
                 float inv) {
    using S = Stencil<MAS>;
    constexpr int NT = S::NT;
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

// -------------------------------------------------------- tile-sorted path
struct TileGeom {
    int dims;
    int TX, TY, TZ;      // tile extent in cells
    int ntx, nty, ntz;   // tiles per axis
    int RX, RY, RZ;      // shared footprint extent = T + LO + HI
    int ntiles;
};

template <int MAS>
__device__ __forceinline__ int tile_of(const float *p, float inv, const TileGeom &g) {
    const int hx = wrap_idx(home_cell<MAS>(cell_dist(p[0], inv)), g.dims);
    const int hy = wrap_idx(home_cell<MAS>(cell_dist(p[1], inv)), g.dims);
    const int hz = wrap_idx(home_cell<MAS>(cell_dist(p[2], inv)), g.dims);
    return ((hx / g.TX) * g.nty + hy / g.TY) * g.ntz + hz / g.TZ;
}

// Phase A: per-block tile histograms -> hist[tile * B + block]
template <int MAS>
__global__ void __launch_bounds__(1024)
k_tile_hist(const float *__restrict__ pos, long long n, long long chunk, float inv,
            TileGeom g, unsigned *__restrict__ hist) {
    extern __shared__ unsigned s_cnt[];
    for (int t = threadIdx.x; t < g.ntiles; t += blockDim.x) s_cnt[t] = 0u;
    __syncthreads();
    const long long b0 = blockIdx.x * chunk;
    const long long b1 = min(n, b0 + chunk);
    for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x)
        atomicAdd(&s_cnt[tile_of<MAS>(pos + 3 * i, inv, g)], 1u);
    __syncthreads();
    const int B = gridDim.x;
    for (int t = threadIdx.x; t < g.ntiles; t += blockDim.x)
        hist[(size_t)t * B + blockIdx.x] = s_cnt[t];
}

// Phase C: scatter particles (and weights) to their tile-sorted slots.
template <int MAS, bool HAS_W>
__global__ void __launch_bounds__(1024)
k_tile_scatter(const float *__restrict__ pos, const float *__restrict__ W, long long n,
               long long chunk, float inv, TileGeom g, const unsigned *__restrict__ off,
               float *__restrict__ spos, float *__restrict__ sw) {
    extern __shared__ unsigned s_cur[];
    const int B = gridDim.x;
    for (int t = threadIdx.x; t < g.ntiles; t += blockDim.x)
        s_cur[t] = off[(size_t)t * B + blockIdx.x];
    __syncthreads();
    const long long b0 = blockIdx.x * chunk;
    const long long b1 = min(n, b0 + chunk);
    for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const float x = __ldcs(pos + 3 * i), y = __ldcs(pos + 3 * i + 1),
                    z = __ldcs(pos + 3 * i + 2);
        const float p[3] = {x, y, z};
        const unsigned slot = atomicAdd(&s_cur[tile_of<MAS>(p, inv, g)], 1u);
        spos[3 * (size_t)slot + 0] = x;
        spos[3 * (size_t)slot + 1] = y;
        spos[3 * (size_t)slot + 2] = z;
        if (HAS_W) sw[slot] = __ldcs(W + i);
    }
}

__device__ __forceinline__ void red_v4(float *addr, float a, float b, float c, float d) {
    asm volatile("red.relaxed.gpu.global.add.v4.f32 [%0], {%1, %2, %3, %4};"
                 :: "l"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// Phase D: one CTA per tile: shared footprint, shared atomics, global flush.
template <int MAS, bool HAS_W>
__global__ void __launch_bounds__(512)
k_tile_deposit(const float *__restrict__ spos, const float *__restrict__ sw,
               const unsigned *__restrict__ off, int B, long long n, float inv, TileGeom g,
               float *__restrict__ grid, int vec4) {
    using S = Stencil<MAS>;
    constexpr int NT = S::NT;
    extern __shared__ float s_reg[];
    const int t = blockIdx.x;
    const int RX = g.RX, RY = g.RY, RZ = g.RZ;
    const int cells = RX * RY * RZ;
    for (int i = threadIdx.x; i < cells; i += blockDim.x) s_reg[i] = 0.f;
    const int tx = t / (g.nty * g.ntz), ty = (t / g.ntz) % g.nty, tz = t % g.ntz;
    const int ox = tx * g.TX, oy = ty * g.TY, oz = tz * g.TZ;   // tile origin (cells)
    const long long p0 = off[(size_t)t * B];
    const long long p1 = (t + 1 < g.ntiles) ? (long long)off[(size_t)(t + 1) * B] : n;
    __syncthreads();
    for (long long i = p0 + threadIdx.x; i < p1; i += blockDim.x) {
        int lx[NT], ly[NT], lz[NT];
        float wx[NT], wy[NT], wz[NT];
        {
            const float d = cell_dist(__ldcs(spos + 3 * i + 0), inv);
            const int c = home_cell<MAS>(d);
            const int base = wrap_idx(c, g.dims) - ox + S::LO;
            int o[NT];
            axis_stencil<MAS>(d, c, o, wx);
#pragma unroll
            for (int j = 0; j < NT; ++j) lx[j] = base + o[j];
        }
        {
            const float d = cell_dist(__ldcs(spos + 3 * i + 1), inv);
            const int c = home_cell<MAS>(d);
            const int base = wrap_idx(c, g.dims) - oy + S::LO;
            int o[NT];
            axis_stencil<MAS>(d, c, o, wy);
#pragma unroll
            for (int j = 0; j < NT; ++j) ly[j] = base + o[j];
        }
        {
            const float d = cell_dist(__ldcs(spos + 3 * i + 2), inv);
            const int c = home_cell<MAS>(d);
            const int base = wrap_idx(c, g.dims) - oz + S::LO;
            int o[NT];
            axis_stencil<MAS>(d, c, o, wz);
#pragma unroll
            for (int j = 0; j < NT; ++j) lz[j] = base + o[j];
        }
        const float wt = HAS_W ? __ldcs(sw + i) : 1.f;
#pragma unroll
        for (int l = 0; l < NT; ++l) {
#pragma unroll
            for (int m = 0; m < NT; ++m) {
                const float wxy = wx[l] * wy[m];
                float *row = s_reg + (lx[l] * RY + ly[m]) * RZ;
#pragma unroll
                for (int q = 0; q < NT; ++q) {
                    float v = wxy * wz[q];
                    if (HAS_W) v *= wt;
                    atomicAdd(row + lz[q], v);
                }
            }
        }
    }
    __syncthreads();
    const int d = g.dims;
    const long long dd = (long long)d * d;
    const int zs = oz - S::LO;  // unwrapped global z of footprint column 0
    if (vec4) {
        // quads aligned to the global z index (dims % 4 == 0: never wraps inside)
        const int q0 = (zs >= 0 ? zs : zs - 3) / 4;          // floor(zs / 4)
        const int q1 = (zs + RZ - 1 >= 0 ? zs + RZ - 1 : zs + RZ - 4) / 4;
        const int nq = q1 - q0 + 1;
        const int work = RX * RY * nq;
        for (int w = threadIdx.x; w < work; w += blockDim.x) {
            const int q = w % nq;
            const int r = w / nq;
            const int ly = r % RY, lx = r / RY;
            const int zq = 4 * (q0 + q);                      // unwrapped quad start
            float v[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int lz = zq + e - zs;
                v[e] = (lz >= 0 && lz < RZ) ? s_reg[(lx * RY + ly) * RZ + lz] : 0.f;
            }
            if (v[0] != 0.f || v[1] != 0.f || v[2] != 0.f || v[3] != 0.f) {
                const int gx = wrap_idx(ox - S::LO + lx, d);
                const int gy = wrap_idx(oy - S::LO + ly, d);
                const int gz = wrap_idx(zq, d);
                red_v4(grid + gx * dd + (long long)gy * d + gz, v[0], v[1], v[2], v[3]);
            }
        }
    } else {
        for (int c = threadIdx.x; c < cells; c += blockDim.x) {
            const float v = s_reg[c];
            if (v == 0.f) continue;
            const int lz = c % RZ, ly = (c / RZ) % RY, lx = c / (RZ * RY);
            const int gx = wrap_idx(ox - S::LO + lx, d);
            const int gy = wrap_idx(oy - S::LO + ly, d);
            const int gz = wrap_idx(zs + lz, d);
            atomicAdd(grid + gx * dd + (long long)gy * d + gz, v);
        }
    }
}

// ------------------------------------------------------------------- scan
// Exclusive scan of a uint32 array in place (three passes: block sums, scan
// of block sums, block-local scan + offset).
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;
constexpr int kScanChunk = kScanThreads * kScanPer;

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

template <typename K>
int set_smem(pyl_ctx *ctx, K kernel, size_t bytes) {
    if (bytes > 48 * 1024)
        PYL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes));
    return PYL_OK;
}

TileGeom make_geom(int dims, int mas) {
    TileGeom g;
    g.dims = dims;
    g.TZ = dims >= 32 ? 32 : dims;
    g.TY = dims >= 32 ? 32 : dims;
    g.TX = dims >= 1024 ? 32 : (dims >= 16 ? 16 : dims);
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
    const int lo = (mas == PYL_MAS_TSC || mas == PYL_MAS_PCS) ? 1 : 0;
    const int hi = (mas == PYL_MAS_TSC || mas == PYL_MAS_PCS) ? 2 : 1;
    g.RX = g.TX + lo + hi;
    g.RY = g.TY + lo + hi;
    g.RZ = g.TZ + lo + hi;
    return g;
}

template <int MAS>
int launch_sorted(pyl_ctx *ctx, const float *pos, long long n, const float *W, float *grid,
                  int dims, float inv) {
    const TileGeom g = make_geom(dims, MAS);
    int st = PYL_OK;
    int B = 4 * 152;
    long long chunk = (n + B - 1) / B;
    if (chunk < 1024) { chunk = 1024; B = (int)((n + chunk - 1) / chunk); }
    const size_t hsm = sizeof(unsigned) * (size_t)g.ntiles;
    const size_t rsm = sizeof(float) * (size_t)g.RX * g.RY * g.RZ;
    const long long nh = (long long)g.ntiles * B;
    unsigned *hist = (unsigned *)ws_get(ctx, "dep_hist", sizeof(unsigned) * (size_t)nh, &st);
    if (!hist) return st;
    float *spos = (float *)ws_get(ctx, "dep_spos", sizeof(float) * 3 * (size_t)n, &st);
    if (!spos) return st;
    float *sw = nullptr;
    if (W) {
        sw = (float *)ws_get(ctx, "dep_sw", sizeof(float) * (size_t)n, &st);
        if (!sw) return st;
    }
    {
        StageScope s(ctx, ST_SORT);
        if ((st = set_smem(ctx, k_tile_hist<MAS>, hsm))) return st;
        k_tile_hist<MAS><<<B, 1024, hsm, ctx->stream>>>(pos, n, chunk, inv, g, hist);
        ctx->launches++;
        PYL_CUDA(ctx, cudaGetLastError());
        if ((st = scan_exclusive(ctx, hist, nh))) return st;
        if (W) {
            if ((st = set_smem(ctx, k_tile_scatter<MAS, true>, hsm))) return st;
            k_tile_scatter<MAS, true><<<B, 1024, hsm, ctx->stream>>>(pos, W, n, chunk, inv, g,
                                                                     hist, spos, sw);
        } else {
            if ((st = set_smem(ctx, k_tile_scatter<MAS, false>, hsm))) return st;
            k_tile_scatter<MAS, false><<<B, 1024, hsm, ctx->stream>>>(pos, W, n, chunk, inv, g,
                                                                      hist, spos, sw);
        }
        ctx->launches++;
        PYL_CUDA(ctx, cudaGetLastError());
    }
    // vector reductions need 16-byte aligned quads: dims % 4 == 0 and an
    // aligned grid base (a user tensor may be a view with an offset)
    const int vec4 = (dims % 4 == 0 && ((uintptr_t)grid & 15) == 0) ? 1 : 0;
    if (W) {
        if ((st = set_smem(ctx, k_tile_deposit<MAS, true>, rsm))) return st;
        k_tile_deposit<MAS, true><<<g.ntiles, 512, rsm, ctx->stream>>>(spos, sw, hist, B, n, inv,
                                                                       g, grid, vec4);
    } else {
        if ((st = set_smem(ctx, k_tile_deposit<MAS, false>, rsm))) return st;
        k_tile_deposit<MAS, false><<<g.ntiles, 512, rsm, ctx->stream>>>(spos, sw, hist, B, n,
                                                                        inv, g, grid, vec4);
    }
    ctx->launches++;
    PYL_CUDA(ctx, cudaGetLastError());
    return PYL_OK;
}

bool use_sorted(long long n, int coord, int dims, int mas, int flags) {
    if (coord != 3) return false;
    if (flags & PYL_DEPOSIT_ATOMIC) return false;
    const TileGeom g = make_geom(dims, mas);
    const size_t rsm = sizeof(float) * (size_t)g.RX * g.RY * g.RZ;
    if (rsm > 200 * 1024 || (size_t)g.ntiles * 4 > 200 * 1024) return false;
    if ((long long)g.ntiles * 4 * 152 >= (1LL << 31)) return false;
    if (n >= (1LL << 32) - 1) return false;
    if (flags & PYL_DEPOSIT_SORTED) return true;
    return n >= (1LL << 20) && dims >= 32;
}

}  // namespace

template <typename G>
static int deposit_t(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                     G *grid, int dims, float BoxSize, int mas, int flags) {
    if (n == 0) return PYL_OK;
    // inv_cell_size = dims/BoxSize as a float division (MAS_library.pyx:135)
    const float inv = (float)dims / BoxSize;
    if (sizeof(G) == sizeof(float) && use_sorted(n, coord, dims, mas, flags)) {
        float *gf = reinterpret_cast<float *>(grid);
        switch (mas) {
            case PYL_MAS_NGP: return launch_sorted<PYL_MAS_NGP>(ctx, pos, n, W, gf, dims, inv);
            case PYL_MAS_CIC: return launch_sorted<PYL_MAS_CIC>(ctx, pos, n, W, gf, dims, inv);
            case PYL_MAS_TSC: return launch_sorted<PYL_MAS_TSC>(ctx, pos, n, W, gf, dims, inv);
            case PYL_MAS_PCS: return launch_sorted<PYL_MAS_PCS>(ctx, pos, n, W, gf, dims, inv);
            default: break;
        }
    }
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
    return deposit_t(ctx, pos, n, coord, W, grid, dims, BoxSize, mas, flags);
}

int deposit_f64(pyl_ctx *ctx, const float *pos, int64_t n, int coord, const float *W,
                double *grid, int dims, float BoxSize, int mas) {
    return deposit_t(ctx, pos, n, coord, W, grid, dims, BoxSize, mas, PYL_DEPOSIT_ATOMIC);
}

int scale_grid(pyl_ctx *ctx, float *grid, int64_t count, float s) {
    return scale_t<float>(ctx, grid, count, s);
}

int scale_grid_f64(pyl_ctx *ctx, double *grid, int64_t count, double s) {
    return scale_t<double>(ctx, grid, count, s);
}

}  // namespace pyl
