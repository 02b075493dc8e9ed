// pyl_pk_batch: many particles -> spectrum requests issued at once and
// waited for once, the sequence captured into a CUDA graph and relaunched as
// a single graph launch when the same batch comes again.
//
// The requests are spread over lanes: child contexts, each with its own
// stream and workspaces (sort buffers, grid, half-complex grid, sums),
// forked from and joined back to the context's stream by events.  Requests
// of one lane run one after another; the lanes run side by side, so the
// small grids and short kernels of uneven realizations share the GPU (in the
// graph they are parallel branches).  Requests go to lanes longest first,
// each to the lane with the least work so far.  Every request copies its
// sums to its own slot of one pinned buffer.
//
// The first call with a new batch issues it directly with the exact
// counting sort (this also sizes every workspace, loads every kernel and
// fills the plan caches) and learns from each request's sort the slots of
// the count-free sort; then it captures the same sequence with those sorts.
// Capture never grows a workspace (ws_get refuses while capturing), so the
// graph holds no allocation.  A replay whose count-free slots overflowed
// (the same pointers with new contents) is still exact -- the overflow goes
// through the spill deposit -- and drops the graph, so that the next call
// learns and captures again.
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"

using namespace pyl;

namespace {

constexpr int kDefaultLanes = 4;

std::vector<char> batch_key(const pyl_pk_request *reqs, int count, int flags) {
    std::vector<char> k(sizeof(int) + sizeof(pyl_pk_request) * (size_t)count);
    memcpy(k.data(), &flags, sizeof(int));
    memcpy(k.data() + sizeof(int), reqs, sizeof(pyl_pk_request) * (size_t)count);
    return k;
}

int lanes_wanted(int flags, int count) {
    int k = (flags >> 16) & 0xF;
    if (k == 0) k = kDefaultLanes;
    return std::max(1, std::min(k, count));
}

int ensure_lanes(pyl_ctx *ctx, int k) {
    if (!ctx->lane_fork)
        PYL_CUDA(ctx, cudaEventCreateWithFlags(&ctx->lane_fork, cudaEventDisableTiming));
    while ((int)ctx->lanes.size() < k) {
        pyl_ctx *c = nullptr;
        const int st = pyl_ctx_create(&c, ctx->device, nullptr);
        if (st) return fail(ctx, st, "cannot create a batch lane context");
        ctx->lanes.push_back(c);
        cudaEvent_t e = nullptr;
        PYL_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->lane_join.push_back(e);
    }
    return PYL_OK;
}

// Longest first, each to the least loaded lane (cost ~ bytes a request moves).
std::vector<int> assign_lanes(const pyl_pk_request *reqs, int count, int k) {
    std::vector<double> cost(count);
    for (int i = 0; i < count; ++i)
        cost[i] = (double)reqs[i].n * (reqs[i].W ? 16.0 : 12.0) * 5.0 +
                  40.0 * (double)reqs[i].dims * reqs[i].dims * reqs[i].dims;
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<double> load(k, 0.0);
    std::vector<int> lane(count);
    for (int i : order) {
        const int j = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        lane[i] = j;
        load[j] += cost[i];
    }
    return lane;
}

// Issues every request on its lane between a fork and a join on the
// context's stream; used[i] receives request i's sort.
int issue_all(pyl_ctx *ctx, const pyl_pk_request *reqs, int count,
              const std::vector<const ModeTables *> &T, const std::vector<size_t> &off, int flags,
              const std::vector<int> &lane, int k, std::vector<pyl_ctx::SortUsed> &used) {
    PYL_CUDA(ctx, cudaEventRecord(ctx->lane_fork, ctx->stream));
    for (int j = 0; j < k; ++j)
        PYL_CUDA(ctx, cudaStreamWaitEvent(ctx->lanes[j]->stream, ctx->lane_fork, 0));
    int st = PYL_OK;
    for (int i = 0; i < count && !st; ++i) {
        pyl_ctx *c = ctx->lanes[lane[i]];
        c->capturing = ctx->capturing;
        c->sort_hint = &ctx->batch_plans[i];
        st = issue_particles(c, reqs[i], *T[i], flags, (char *)ctx->batch_pinned + off[i]);
        c->sort_hint = nullptr;
        used[i] = c->sort_used;
        if (st) {
            ctx->err = c->err;
        }
    }
    // join every lane, also after an error (a capture must end joined)
    for (int j = 0; j < k; ++j) {
        ctx->lanes[j]->capturing = false;
        PYL_CUDA(ctx, cudaEventRecord(ctx->lane_join[j], ctx->lanes[j]->stream));
        PYL_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->lane_join[j], 0));
    }
    return st;
}

// After the batch's work: the lanes' status words, the sorts' lessons and
// the spectra.  Returns whether a count-free sort overflowed its slots.
int finish_all(pyl_ctx *ctx, const pyl_pk_request *reqs, int count,
               const std::vector<const ModeTables *> &T, const std::vector<AccLayout> &L,
               const std::vector<size_t> &off, const std::vector<pyl_ctx::SortUsed> &used,
               int k, pyl_pk_out *outs, bool *spilled) {
    int st = status_check(ctx);
    if (st) return st;
    for (int j = 0; j < k; ++j)
        if ((st = status_check(ctx->lanes[j]))) {
            ctx->err = ctx->lanes[j]->err;
            return st;
        }
    *spilled = false;
    for (int i = 0; i < count; ++i) {
        const char *slot = (const char *)ctx->batch_pinned + off[i];
        const unsigned *info =
            (const unsigned *)(slot + L[i].sums() + sizeof(float2) + sizeof(double));
        if (used[i].valid) {
            if (used[i].cap && info[3] != 0) *spilled = true;
            learn_sort(used[i], info);
        }
        if ((st = finalize_particles(ctx, *T[i], L[i], slot, reqs[i].dims, reqs[i].BoxSize,
                                     reqs[i].what, &outs[i])))
            return st;
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
    const int k = lanes_wanted(flags, count);
    if ((st = ensure_lanes(ctx, k))) return st;
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
        total += (result_bytes(L[i]) + 255) / 256 * 256;
    }
    std::vector<char> key = batch_key(reqs, count, flags);
    const std::vector<int> lane = assign_lanes(reqs, count, k);
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
        if (key != ctx->batch_plans_key) {         // a new batch: learn its sorts afresh
            ctx->batch_plans.assign(count, pyl_ctx::SortPlan());
            ctx->batch_plans_key = key;
        }
        // issue directly: these are this call's results
        std::vector<pyl_ctx::SortUsed> used(count);
        if ((st = issue_all(ctx, reqs, count, T, off, flags, lane, k, used))) return st;
        bool spilled = false;
        if ((st = finish_all(ctx, reqs, count, T, L, off, used, k, outs, &spilled))) return st;
        if (flags & PYL_NO_GRAPH) return PYL_OK;
        // capture the same sequence, with the sorts just learned, for the
        // next call with this batch
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
        ctx->batch_used.assign(count, pyl_ctx::SortUsed());
        st = issue_all(ctx, reqs, count, T, off, flags, lane, k, ctx->batch_used);
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
    bool spilled = false;
    if ((st = finish_all(ctx, reqs, count, T, L, off, ctx->batch_used, k, outs, &spilled)))
        return st;
    if (spilled) {   // the slots no longer fit: learn and capture again next time
        cudaGraphExecDestroy(ctx->batch_exec);
        ctx->batch_exec = nullptr;
        ctx->batch_key.clear();
    }
    return PYL_OK;
}
