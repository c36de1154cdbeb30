// Batched stepping: many independent scenes (each an ordinary context with
// its own arena, uploaded and downloaded on its own) advanced together.
//
// Every stage of a step is ONE launch over all scenes of the batch: a block
// finds its scene in a per-launch block table (scene k owns a run of
// consecutive blocks, in proportion to its own particle / cell / tile
// counts; one 16-byte entry per block) and reads the scene's record -
// parameters, state pointers, cell lists and scratch - from device memory.  So a batch of 256 small scenes costs the
// same ~30 launches per step as one large scene, every launch fills the GPU,
// and scenes of uneven size share it in proportion to their work.  Each kind
// of step is captured once as a CUDA graph and replayed.
//
// The scenes of a batch step in lockstep: they must share sort_every_step
// and sit at the same step index with the same list buffer.  Scenes may
// differ in everything else (sizes, grids, materials, time steps, shifting
// passes and solid sub-steps per step: a scene with fewer passes owns no
// block of the later ones).
#include "context.h"

#include <algorithm>
#include <cstdio>
#include <set>

using namespace sphnj;

struct sphnj_batch {
    std::vector<sphnj_ctx *> scenes;
    int device = 0;
    cudaStream_t own = nullptr, st = nullptr;
    GroupMany g;
    // host records, list buffer 0 / 1 bound: the n scenes, then the same with
    // their position buffers exchanged (GroupMany::d_scenes)
    std::vector<Scene> recs[2];
    Scene *d_recs[2] = {nullptr, nullptr};
    TileConfig tiles;
    bool use_graphs = true;
    bool pdl = true;  // programmatic dependent launch between the kernels of a step
    std::map<int, StepGraph> graphs;
    std::set<int> planned;             // step kinds whose block tables exist
    Profiler prof;
    uint64_t launches = 0;
    std::string msg = "ok";
};

namespace {

int bfail(sphnj_batch *b, int code, const std::string &m) {
    if (b) b->msg = m;
    return code;
}

int bcuda(sphnj_batch *b, cudaError_t e, const char *where) {
    return bfail(b, SPHNJ_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define BCK(call)                                                  \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return bcuda(b, e_, #call);         \
    } while (0)

void drop_graphs(sphnj_batch *b) {
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.second.exec);
    b->graphs.clear();
}

// Builds the block tables of one kind of step (no launch).
int plan(sphnj_batch *b, const StepKind &k) {
    if (b->planned.count(k.key())) return SPHNJ_OK;
    b->g.planning = true;
    issue_step(b->g, k, b->st, b->tiles, nullptr);
    b->g.planning = false;
    if (b->g.error != cudaSuccess) {
        cudaError_t e = b->g.error;
        b->g.error = cudaSuccess;
        return bcuda(b, e, "batch launch planning");
    }
    b->planned.insert(k.key());
    return SPHNJ_OK;
}

void set_scene_streams(sphnj_batch *b, cudaStream_t st) {
    for (sphnj_ctx *c : b->scenes) c->st = st;
}

// The device records of every scene, list buffer 0 / 1 bound: the n scenes,
// then the same with their position buffers exchanged.
cudaError_t write_records(sphnj_batch *b) {
    const int n = (int)b->scenes.size();
    for (int par = 0; par < 2; ++par) {
        b->recs[par].clear();
        b->recs[par].reserve(2 * (size_t)n);
        for (sphnj_ctx *c : b->scenes) b->recs[par].push_back(scene_of(c, par));
        for (int k = 0; k < n; ++k) {
            Scene s = b->recs[par][k];
            exchange_positions(s, b->g.form);
            b->recs[par].push_back(s);
        }
        if (!b->d_recs[par]) {
            cudaError_t e = cudaMalloc(&b->d_recs[par], sizeof(Scene) * 2 * n);
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = cudaMemcpy(b->d_recs[par], b->recs[par].data(), sizeof(Scene) * 2 * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// After a scene's sweep shape changed: new records, new block tables, new graphs.
int refresh_records(sphnj_batch *b) {
    drop_graphs(b);
    b->planned.clear();
    b->g.free_tables();
    BCK(write_records(b));
    return SPHNJ_OK;
}

}  // namespace

extern "C" {

int sphnj_batch_create(sphnj_ctx *const *scenes, int n, sphnj_batch **out) {
    if (!scenes || n < 1 || !out) return SPHNJ_ERR_ARG;
    *out = nullptr;
    const sphnj_ctx *c0 = scenes[0];
    if (!c0) return SPHNJ_ERR_ARG;
    for (int i = 0; i < n; ++i) {
        const sphnj_ctx *c = scenes[i];
        if (!c || !c->uploaded || c->batch) return SPHNJ_ERR_ARG;
        for (int j = 0; j < i; ++j)
            if (scenes[j] == c) return SPHNJ_ERR_ARG;  // a scene appears once
        if (c->device != c0->device || c->form != c0->form || c->p.sort_every_step != c0->p.sort_every_step ||
            c->step != c0->step || c->parity != c0->parity)
            return SPHNJ_ERR_ARG;
    }
    sphnj_batch *b = new sphnj_batch;
    b->device = c0->device;
    cudaSetDevice(b->device);
    b->scenes.assign(scenes, scenes + n);
    for (sphnj_ctx *c : b->scenes)
        if (cudaStreamSynchronize(c->st) != cudaSuccess) {
            cudaGetLastError();
            delete b;
            return SPHNJ_ERR_CUDA;
        }
    if (cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return SPHNJ_ERR_CUDA;
    }
    b->st = b->own;
    b->g.n = n;
    b->g.form = c0->form;
    // the batch's launch shape starts as its first scene's
    b->tiles = c0->tiles;
    if (write_records(b) != cudaSuccess) {
        cudaGetLastError();
        for (Scene *r : b->d_recs)
            if (r) cudaFree(r);
        cudaStreamDestroy(b->own);
        delete b;
        return SPHNJ_ERR_CUDA;
    }
    if (configure_sweeps(b->tiles) != cudaSuccess) {
        cudaGetLastError();
        for (Scene *r : b->d_recs) cudaFree(r);
        cudaStreamDestroy(b->own);
        delete b;
        return SPHNJ_ERR_CUDA;
    }
    for (sphnj_ctx *c : b->scenes) c->batch = b;
    set_scene_streams(b, b->st);
    *out = b;
    return SPHNJ_OK;
}

void sphnj_batch_destroy(sphnj_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->st) cudaStreamSynchronize(b->st);
    drop_graphs(b);
    b->g.free_tables();
    b->prof.release();
    for (Scene *r : b->d_recs)
        if (r) cudaFree(r);
    for (sphnj_ctx *c : b->scenes) {
        c->st = c->own;
        c->batch = nullptr;
    }
    if (b->own) cudaStreamDestroy(b->own);
    delete b;
}

int sphnj_batch_set_stream(sphnj_batch *b, void *stream) {
    if (!b) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->st = stream ? static_cast<cudaStream_t>(stream) : b->own;
    set_scene_streams(b, b->st);
    return SPHNJ_OK;
}

int sphnj_batch_set_tiling(sphnj_batch *b, int tiled, int tile_h) {
    if (!b || tile_h < 1 || tile_h > 64) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->tiles.tiled = tiled != 0;
    b->tiles.tile_h = tile_h;
    for (sphnj_ctx *c : b->scenes) {  // every scene takes the batch's shape
        c->tiles.tiled = b->tiles.tiled;
        c->tiles.tile_h = tile_h;
    }
    BCK(configure_sweeps(b->tiles));
    return refresh_records(b);
}

int sphnj_batch_set_neighbour_lists(sphnj_batch *b, int on) {
    if (!b) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->tiles.lists = on != 0;
    for (sphnj_ctx *c : b->scenes) c->tiles.lists = b->tiles.lists;
    return refresh_records(b);
}

int sphnj_batch_set_scene_tiling(sphnj_batch *b, int scene, int tile_h, int lists) {
    if (!b || scene < 0 || scene >= (int)b->scenes.size() || tile_h < 1 || tile_h > 64) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->scenes[scene]->tiles.tile_h = tile_h;
    b->scenes[scene]->tiles.lists = lists != 0;
    return refresh_records(b);
}

int sphnj_batch_get_scene_tiling(const sphnj_batch *b, int scene, int *tile_h, int *lists) {
    if (!b || scene < 0 || scene >= (int)b->scenes.size()) return SPHNJ_ERR_ARG;
    if (tile_h) *tile_h = b->scenes[scene]->tiles.tile_h;
    if (lists) *lists = b->scenes[scene]->tiles.lists ? 1 : 0;
    return SPHNJ_OK;
}

int sphnj_batch_set_block_sizes(sphnj_batch *b, int shift_threads, int pair_threads) {
    if (!b) return SPHNJ_ERR_ARG;
    if (!(shift_threads == 0 || shift_threads == 64 || shift_threads == 128 || shift_threads == 256) ||
        !(pair_threads == 0 || pair_threads == 128 || pair_threads == 256))
        return bfail(b, SPHNJ_ERR_ARG, "block sizes: shifting pass 0, 64, 128 or 256; pair pass 0, 128 or 256");
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->tiles.shift_block = shift_threads;
    b->tiles.pair_block = pair_threads;
    for (sphnj_ctx *c : b->scenes) {
        c->tiles.shift_block = shift_threads;
        c->tiles.pair_block = pair_threads;
    }
    return refresh_records(b);
}

int sphnj_batch_get_sweeps(const sphnj_batch *b, int *tiled, int *tile_h, int *lists) {
    if (!b) return SPHNJ_ERR_ARG;
    if (tiled) *tiled = b->tiles.tiled ? 1 : 0;
    if (tile_h) *tile_h = b->tiles.tile_h;
    if (lists) *lists = b->tiles.lists ? 1 : 0;
    return SPHNJ_OK;
}

int sphnj_batch_set_launch_chaining(sphnj_batch *b, int on) {
    if (!b) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->pdl = on != 0;
    drop_graphs(b);
    return SPHNJ_OK;
}

int sphnj_batch_set_graphs(sphnj_batch *b, int on) {
    if (!b) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->use_graphs = on != 0;
    drop_graphs(b);
    return SPHNJ_OK;
}

int sphnj_batch_step(sphnj_batch *b, int n) {
    if (!b || n < 0) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    cudaStream_t st = b->st;
    for (int it = 0; it < n; ++it) {
        const sphnj_ctx *c0 = b->scenes[0];
        for (const sphnj_ctx *c : b->scenes)
            if (!c->uploaded || c->step != c0->step || c->parity != c0->parity)
                return bfail(b, SPHNJ_ERR_ARG, "batch scenes are not at the same step");
        StepKind k{};
        std::vector<StepKind> kinds(b->scenes.size());
        for (size_t i = 0; i < b->scenes.size(); ++i) {
            const StepKind ki = kinds[i] = next_kind(b->scenes[i]);
            if (i == 0) {
                k = ki;
            } else {
                // re-binning or re-sorting virtual particles that are already
                // binned and sorted changes nothing, so these are OR-ed
                k.bin_virt = k.bin_virt || ki.bin_virt;
                k.sort_virt = k.sort_virt || ki.sort_virt;
            }
        }
        GroupMany &g = b->g;
        g.pdl = b->pdl;
        g.h_scenes = b->recs[k.parity].data();
        g.d_scenes = b->d_recs[k.parity];
        int rc = plan(b, k);
        if (rc) return rc;
        if (b->use_graphs && !b->prof.on) {
            auto it_g = b->graphs.find(k.key());
            if (it_g == b->graphs.end()) {
                cudaGraph_t graph = nullptr;
                BCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                const int launched = issue_step(g, k, st, b->tiles, nullptr);
                cudaError_t e = cudaStreamEndCapture(st, &graph);
                cudaGraphExec_t exec = nullptr;
                if (e == cudaSuccess) e = g.error;
                if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
                if (graph) cudaGraphDestroy(graph);
                g.error = cudaSuccess;
                if (e != cudaSuccess) return bcuda(b, e, "batch step graph capture");
                it_g = b->graphs.emplace(k.key(), StepGraph{exec, launched}).first;
            }
            BCK(cudaGraphLaunch(it_g->second.exec, st));
            b->launches += (uint64_t)it_g->second.kernels;
        } else {
            b->launches += (uint64_t)issue_step(g, k, st, b->tiles, b->prof.on ? &b->prof : nullptr);
            if (g.error != cudaSuccess) {
                cudaError_t e = g.error;
                g.error = cudaSuccess;
                return bcuda(b, e, "batch step");
            }
        }
        BCK(cudaGetLastError());
        // the step is issued: only now does every scene's step state move
        for (size_t i = 0; i < b->scenes.size(); ++i) commit_step(b->scenes[i], kinds[i]);
    }
    return SPHNJ_OK;
}

int sphnj_batch_synchronize(sphnj_batch *b) {
    if (!b) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    for (sphnj_ctx *c : b->scenes)
        BCK(cudaMemcpyAsync(c->h_err, c->d.err, sizeof(DevErr), cudaMemcpyDeviceToHost, b->st));
    BCK(cudaStreamSynchronize(b->st));
    for (size_t i = 0; i < b->scenes.size(); ++i) {
        const int rc = device_error_status(b->scenes[i]);
        if (rc) {
            char buf[48];
            snprintf(buf, sizeof buf, "scene %d: ", (int)i);
            return bfail(b, rc, buf + b->scenes[i]->msg);
        }
    }
    return SPHNJ_OK;
}

int sphnj_batch_profile_enable(sphnj_batch *b, int on) {
    if (!b) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->prof.enable(on != 0);
    return SPHNJ_OK;
}

int sphnj_batch_profile_read(sphnj_batch *b, double *ms, int64_t *calls, int64_t *kernels) {
    if (!b) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    BCK(b->prof.collect());
    for (int s = 0; s < ST_COUNT; ++s) {
        if (ms) ms[s] = b->prof.ms[s];
        if (calls) calls[s] = b->prof.calls[s];
        if (kernels) kernels[s] = b->prof.kernels[s];
    }
    return SPHNJ_OK;
}

int sphnj_batch_stat_launches(const sphnj_batch *b, uint64_t *launches) {
    if (!b || !launches) return SPHNJ_ERR_ARG;
    *launches = b->launches;
    return SPHNJ_OK;
}

const char *sphnj_batch_last_error(const sphnj_batch *b) { return b ? b->msg.c_str() : "null batch"; }

}  // extern "C"

namespace {

// Installs a candidate: the launch shape for the batch, and each scene its
// size class's tile height and list switch (one record refresh).
int apply_batch(void *o, const Tuned &t) {
    sphnj_batch *b = static_cast<sphnj_batch *>(o);
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    b->tiles = t.launch;
    for (size_t k = 0; k < b->scenes.size(); ++k) {
        TileConfig &c = b->scenes[k]->tiles;
        const int cls = k < t.cls.size() ? t.cls[k] : 0;
        c = t.launch;
        c.tile_h = t.tile_h[cls];
        c.lists = t.lists[cls];
    }
    BCK(configure_sweeps(b->tiles));
    return refresh_records(b);
}
int step_batch(void *o, int n) { return sphnj_batch_step(static_cast<sphnj_batch *>(o), n); }

}  // namespace

extern "C" {

int sphnj_batch_autotune(sphnj_batch *b, int steps, sphnj_tuning *out) {
    if (!b || steps < 1) return SPHNJ_ERR_ARG;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->st));
    TuneResult r{};
    const int rc = tune_sweeps(b->scenes, b->st, steps, true, apply_batch, step_batch, b, &r);
    if (rc) return rc == SPHNJ_ERR_CUDA ? bfail(b, rc, "batch autotune: CUDA error") : rc;
    tuning_out(r, out);
    return SPHNJ_OK;
}

}  // extern "C"
