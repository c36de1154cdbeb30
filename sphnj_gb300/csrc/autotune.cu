// Autotuner of the neighbour-sweep launch shape.
//
// The fastest way to sweep neighbours depends on the scene: the cells per
// tile (how many home cells share one shared-memory staging of their
// neighbour strips), and whether the pair pass stores per-step neighbour
// lists for the shifting passes or every pass walks the 3x3 stencil again
// (lists pay off with many shifting passes and dense cells).  All candidates
// compute the same sums in the same order - the result does not depend on
// the choice - so the tuner times them on the caller's own state: it copies
// every context's arena on the device, runs each candidate from that copy,
// and puts the state back, so tuning leaves the run exactly where it was.
// The block size is fixed at 256 threads (8 warps): the tile height sets how
// much work a block has.
#include "context.h"

using namespace sphnj;

namespace {

const TileConfig kCandidates[] = {
    {false, 16, false},                                          // one thread per particle
    {true, 8, true},  {true, 12, true}, {true, 16, true}, {true, 24, true}, {true, 32, true},
    {true, 8, false}, {true, 16, false}, {true, 32, false},      // tiles without stored lists
};

struct Saved {
    sphnj_ctx *ctx;
    char *copy;
    int step, parity;
    bool virt_sorted, virt_cells_valid;
};

void release(std::vector<Saved> &s) {
    for (auto &x : s)
        if (x.copy) cudaFree(x.copy);
    s.clear();
}

cudaError_t take(const std::vector<sphnj_ctx *> &ctxs, cudaStream_t st, std::vector<Saved> &out) {
    for (sphnj_ctx *c : ctxs) {
        Saved s{c, nullptr, c->step, c->parity, c->virt_sorted, c->virt_cells_valid};
        cudaError_t e = cudaMalloc(&s.copy, c->arena_bytes);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s.copy, c->arena, c->arena_bytes, cudaMemcpyDeviceToDevice, st);
        out.push_back(s);
        if (e != cudaSuccess) return e;
    }
    return cudaStreamSynchronize(st);
}

cudaError_t put_back(const std::vector<Saved> &saved, cudaStream_t st) {
    for (const Saved &s : saved) {
        cudaError_t e = cudaMemcpyAsync(s.ctx->arena, s.copy, s.ctx->arena_bytes, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
        s.ctx->step = s.step;
        s.ctx->parity = s.parity;
        s.ctx->virt_sorted = s.virt_sorted;
        s.ctx->virt_cells_valid = s.virt_cells_valid;
    }
    return cudaStreamSynchronize(st);
}

}  // namespace

namespace sphnj {

int tune_sweeps(const std::vector<sphnj_ctx *> &ctxs, cudaStream_t st, int steps,
                int (*apply)(void *, const TileConfig &), int (*step)(void *, int), void *obj, TuneResult *out) {
    std::vector<Saved> saved;
    cudaError_t e = take(ctxs, st, saved);
    if (e != cudaSuccess) {
        release(saved);
        cudaGetLastError();
        return SPHNJ_ERR_CUDA;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    TuneResult best{kCandidates[0], 1e300, 0};
    int rc = SPHNJ_OK;
    for (const TileConfig &cand : kCandidates) {
        if ((rc = apply(obj, cand))) break;
        if ((e = put_back(saved, st)) != cudaSuccess) break;
        if ((rc = step(obj, steps))) break;  // captures this configuration's graphs
        if ((e = put_back(saved, st)) != cudaSuccess) break;
        cudaEventRecord(e0, st);
        if ((rc = step(obj, steps))) break;
        cudaEventRecord(e1, st);
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        best.tried++;
        if (ms / steps < best.ms_per_step) {
            best.best = cand;
            best.ms_per_step = ms / steps;
        }
    }
    if (e == cudaSuccess && rc == SPHNJ_OK) {
        e = put_back(saved, st);
        if (e == cudaSuccess) rc = apply(obj, best.best);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release(saved);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SPHNJ_ERR_CUDA;
    }
    if (rc == SPHNJ_OK && out) *out = best;
    return rc;
}

}  // namespace sphnj

namespace {

int apply_ctx(void *o, const TileConfig &t) {
    sphnj_ctx *c = static_cast<sphnj_ctx *>(o);
    int rc = sphnj_set_tiling(c, t.tiled ? 1 : 0, t.tile_h);
    return rc ? rc : sphnj_set_neighbour_lists(c, t.lists ? 1 : 0);
}
int step_ctx(void *o, int n) { return sphnj_step(static_cast<sphnj_ctx *>(o), n); }

}  // namespace

extern "C" int sphnj_autotune(sphnj_ctx *ctx, int steps, sphnj_tuning *out) {
    if (!ctx || steps < 1) return SPHNJ_ERR_ARG;
    if (!ctx->uploaded) {
        ctx->msg = "sphnj_autotune before sphnj_upload";
        return SPHNJ_ERR_ARG;
    }
    if (ctx->batch) {
        ctx->msg = "the scene is in a batch: tune the batch";
        return SPHNJ_ERR_ARG;
    }
    cudaSetDevice(ctx->device);
    if (cudaStreamSynchronize(ctx->st) != cudaSuccess) return SPHNJ_ERR_CUDA;
    TuneResult r{};
    const int rc = tune_sweeps({ctx}, ctx->st, steps, apply_ctx, step_ctx, ctx, &r);
    if (rc == SPHNJ_OK && out) {
        out->tiled = r.best.tiled ? 1 : 0;
        out->tile_h = r.best.tile_h;
        out->lists = r.best.lists ? 1 : 0;
        out->candidates = r.tried;
        out->ms_per_step = r.ms_per_step;
    }
    return rc;
}
