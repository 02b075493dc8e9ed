// pyl_pk_batch: many particles -> spectrum requests issued back to back on
// one stream and waited for once, the sequence captured into a CUDA graph
// and relaunched as a single graph launch when the same batch comes again.
//
// The requests share the context's workspaces (sort buffers, grid,
// half-complex grid, sums): the stream orders request i+1's zeroing after
// request i's copy of its sums to its own slot of one pinned buffer.  The
// first call with a new batch issues it directly (this sizes every
// workspace, loads every kernel and fills the plan caches), then captures
// the same sequence; capture never grows a workspace (ws_get refuses while
// ctx->capturing), so the graph holds no allocation.
#include <string.h>

#include <vector>

#include "common.cuh"

using namespace pyl;

namespace {

std::vector<char> batch_key(const pyl_pk_request *reqs, int count, int flags) {
    std::vector<char> k(sizeof(int) + sizeof(pyl_pk_request) * (size_t)count);
    memcpy(k.data(), &flags, sizeof(int));
    memcpy(k.data() + sizeof(int), reqs, sizeof(pyl_pk_request) * (size_t)count);
    return k;
}

int issue_all(pyl_ctx *ctx, const pyl_pk_request *reqs, int count,
              const std::vector<const ModeTables *> &T, const std::vector<size_t> &off, int flags) {
    for (int i = 0; i < count; ++i) {
        const int st =
            issue_particles(ctx, reqs[i], *T[i], flags, (char *)ctx->batch_pinned + off[i]);
        if (st) return st;
    }
    return PYL_OK;
}

}  // namespace

extern "C" int pyl_pk_batch(pyl_ctx *ctx, const pyl_pk_request *reqs, int count,
                            pyl_pk_out *outs, int flags) {
    if (!ctx) return PYL_ERR_ARG;
    if (count < 0 || (count > 0 && (!reqs || !outs)))
        return fail(ctx, PYL_ERR_ARG, "bad batch arguments");
    if (count == 0) return PYL_OK;
    if (ctx->req.active)
        return fail(ctx, PYL_ERR_STATE, "a request is already in flight on this context");
    int st = PYL_OK;
    for (int i = 0; i < count; ++i)
        if ((st = check_particles(ctx, reqs[i]))) return st;
    PYL_CUDA(ctx, cudaSetDevice(ctx->device));
    // tables and the pinned result slots (one per request)
    std::vector<const ModeTables *> T(count);
    std::vector<AccLayout> L(count);
    std::vector<size_t> off(count);
    size_t total = 0;
    for (int i = 0; i < count; ++i) {
        T[i] = mode_tables(ctx, reqs[i].dims, reqs[i].axis, &st);
        if (!T[i]) return st;
        L[i] = acc_layout(*T[i]);
        off[i] = total;
        total += (L[i].sums() + sizeof(float2) + sizeof(double) + 255) / 256 * 256;
    }
    std::vector<char> key = batch_key(reqs, count, flags);
    const bool hit = ctx->batch_exec && key == ctx->batch_key && total <= ctx->batch_pinned_bytes;
    if (!hit) {
        if (ctx->batch_pinned_bytes < total) {
            PYL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            if (ctx->batch_pinned) cudaFreeHost(ctx->batch_pinned);
            ctx->batch_pinned = nullptr;
            ctx->batch_pinned_bytes = 0;
            PYL_CUDA(ctx, cudaHostAlloc(&ctx->batch_pinned, total, cudaHostAllocPortable));
            ctx->batch_pinned_bytes = total;
        }
        // issue directly: these are this call's results
        if ((st = issue_all(ctx, reqs, count, T, off, flags))) return st;
        if ((st = status_check(ctx))) return st;
        for (int i = 0; i < count; ++i)
            if ((st = finalize_particles(ctx, *T[i], L[i], (char *)ctx->batch_pinned + off[i],
                                         reqs[i].dims, reqs[i].BoxSize, reqs[i].what, &outs[i])))
                return st;
        if (flags & PYL_NO_GRAPH) return PYL_OK;
        // capture the same sequence for the next call with this batch
        if (ctx->batch_exec) {
            cudaGraphExecDestroy(ctx->batch_exec);
            ctx->batch_exec = nullptr;
            ctx->batch_key.clear();
        }
        // (this call's results are already in outs: a capture that fails
        // only leaves the next call without a graph, which then captures
        // again)
        const bool timing = ctx->timing;
        ctx->timing = false;
        if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            ctx->timing = timing;
            cudaGetLastError();
            return PYL_OK;
        }
        ctx->capturing = true;
        st = issue_all(ctx, reqs, count, T, off, flags);
        ctx->capturing = false;
        ctx->timing = timing;
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        if (st || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return PYL_OK;
        }
        const cudaError_t ei = cudaGraphInstantiate(&ctx->batch_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            ctx->batch_exec = nullptr;
            cudaGetLastError();
            return PYL_OK;
        }
        ctx->batch_key = std::move(key);
        return PYL_OK;
    }
    PYL_CUDA(ctx, cudaGraphLaunch(ctx->batch_exec, ctx->stream));
    ctx->launches += 1;
    if ((st = status_check(ctx))) return st;
    for (int i = 0; i < count; ++i)
        if ((st = finalize_particles(ctx, *T[i], L[i], (char *)ctx->batch_pinned + off[i],
                                     reqs[i].dims, reqs[i].BoxSize, reqs[i].what, &outs[i])))
            return st;
    return PYL_OK;
}
