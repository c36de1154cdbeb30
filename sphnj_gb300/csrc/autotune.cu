// Autotuner of the neighbour-sweep launch shape.
//
// The fastest way to sweep neighbours depends on the scene: the cells per
// tile (how many home cells share one shared-memory staging of their
// neighbour strips), whether the pair pass stores per-step neighbour lists
// for the shifting passes or every pass walks the 3x3 stencil again (lists
// pay off with many shifting passes and dense cells), and the threads per
// block of the shifting passes and of the pair pass.  All candidates compute
// the same sums in the same order - the result does not depend on the
// choice - so the tuner times them on the caller's own state: it copies
// every context's arena on the device, runs each candidate from that copy,
// and puts the state back, so tuning leaves the run exactly where it was.
//
// The search is coordinate-wise: the tile height and the list switch first
// (one thread per particle, tiles of 8-32 cells with and without lists), then
// the shifting passes' block size (64, 128, 256 threads), then the pair
// pass's (128, 256).  In a batch the scenes with fluid are then split into
// two size classes at their median particle count, and each class's tile
// height (8, 12, 16, 24, 32 cells) is tuned with the other class's fixed:
// one launch covers every scene, but each scene sweeps tiles of its class's
// height.
#include "context.h"

#include <algorithm>

using namespace sphnj;

namespace {

const TileConfig kCandidates[] = {
    {false, 16, false},                                          // one thread per particle
    {true, 8, true},  {true, 12, true}, {true, 16, true}, {true, 24, true}, {true, 32, true},
    {true, 8, false}, {true, 16, false}, {true, 32, false},      // tiles without stored lists
};
const int kShiftBlocks[] = {64, 128, 256};
const int kPairBlocks[] = {128, 256};
const int kClassTiles[] = {8, 12, 16, 24, 32};

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

int tune_sweeps(const std::vector<sphnj_ctx *> &ctxs, cudaStream_t st, int steps, bool classes,
                int (*apply)(void *, const Tuned &), int (*step)(void *, int), void *obj, TuneResult *out) {
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
    // size classes: the scenes with fluid at or above the median fluid count
    // form class 1 (a single scene, or a batch of equal scenes, has one class)
    std::vector<int> counts;
    for (const sphnj_ctx *c : ctxs)
        if (c->p.fluid_number_total > 0) counts.push_back(c->p.fluid_number_total);
    std::sort(counts.begin(), counts.end());
    Tuned cur;
    cur.split = 0;
    if (classes && counts.size() >= 2 && counts.front() < counts.back()) cur.split = counts[counts.size() / 2];
    for (const sphnj_ctx *c : ctxs) cur.cls.push_back(cur.split > 0 && c->p.fluid_number_total >= cur.split ? 1 : 0);
    TuneResult best{cur, 1e300, 0};
    int rc = SPHNJ_OK;
    // one trial: capture the candidate's graphs on a copy of the state, then
    // time `steps` steps from the same state
    auto trial = [&](const Tuned &cand) -> bool {
        if ((rc = apply(obj, cand))) return false;
        if ((e = put_back(saved, st)) != cudaSuccess) return false;
        if ((rc = step(obj, steps))) return false;
        if ((e = put_back(saved, st)) != cudaSuccess) return false;
        cudaEventRecord(e0, st);
        if ((rc = step(obj, steps))) return false;
        cudaEventRecord(e1, st);
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return false;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        best.tried++;
        if (ms / steps < best.ms_per_step) {
            best.best = cand;
            best.ms_per_step = ms / steps;
        }
        return true;
    };
    bool ok = true;
    for (const TileConfig &t : kCandidates) {  // tile height and lists, the same for every scene
        Tuned c = cur;
        c.launch = t;
        c.tile_h[0] = c.tile_h[1] = t.tile_h;
        c.lists[0] = c.lists[1] = t.lists;
        if (!(ok = trial(c))) break;
    }
    if (ok && best.best.launch.tiled) {
        const Tuned base = best.best;
        for (int b : kShiftBlocks) {  // threads per block of the shifting passes
            Tuned c = base;
            c.launch.shift_block = b;
            if (!(ok = trial(c))) break;
        }
    }
    if (ok && best.best.launch.tiled) {
        const Tuned base = best.best;
        for (int b : kPairBlocks) {  // of the pair pass
            Tuned c = base;
            c.launch.pair_block = b;
            if (!(ok = trial(c))) break;
        }
    }
    if (ok && best.best.launch.tiled && best.best.split > 0) {
        for (int k = 0; k < 2 && ok; ++k) {  // each size class's tile height, the other class fixed
            const Tuned base = best.best;
            for (int h : kClassTiles) {
                if (h == base.tile_h[k]) continue;
                Tuned c = base;
                c.tile_h[k] = h;
                if (!(ok = trial(c))) break;
            }
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

void tuning_out(const TuneResult &r, sphnj_tuning *out) {
    if (!out) return;
    const Tuned &t = r.best;
    out->tiled = t.launch.tiled ? 1 : 0;
    out->tile_h = t.tile_h[0];
    out->lists = t.lists[0] ? 1 : 0;
    out->candidates = r.tried;
    out->ms_per_step = r.ms_per_step;
    out->shift_block = t.launch.shift_block;
    out->pair_block = t.launch.pair_block;
    out->size_classes = t.split > 0 ? 2 : 1;
    out->class_split = t.split;
    for (int k = 0; k < 2; ++k) {
        out->class_tile_h[k] = t.tile_h[k];
        out->class_lists[k] = t.lists[k] ? 1 : 0;
    }
}

}  // namespace sphnj

namespace {

int apply_ctx(void *o, const Tuned &t) {
    sphnj_ctx *c = static_cast<sphnj_ctx *>(o);
    int rc = sphnj_set_tiling(c, t.launch.tiled ? 1 : 0, t.tile_h[0]);
    if (!rc) rc = sphnj_set_neighbour_lists(c, t.lists[0] ? 1 : 0);
    return rc ? rc : sphnj_set_block_sizes(c, t.launch.shift_block, t.launch.pair_block);
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
    const int rc = tune_sweeps({ctx}, ctx->st, steps, false, apply_ctx, step_ctx, ctx, &r);
    if (rc == SPHNJ_OK) tuning_out(r, out);
    return rc;
}
