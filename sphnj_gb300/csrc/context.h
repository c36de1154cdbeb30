// Internal state of a libsphnj context (one scene) and the pieces of the step
// sequencer that a batch of scenes shares with it.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "kernels.h"

namespace sphnj {

enum Stage {
    ST_BIN, ST_SORT, ST_REBUILD, ST_CAPACITY, ST_SOLID_COUPLE, ST_VIRT_DATA, ST_FLUID_PAIR, ST_FLUID_UPDATE,
    ST_SOLID_DEFORM, ST_SOLID_FORCE, ST_SOLID_UPDATE, ST_SHIFT_PASS, ST_SHIFT_COPY_BACK, ST_COUNT
};
extern const char *const kStageNames[ST_COUNT];

// Per-stage device times from CUDA events recorded around each stage on the
// launching stream (steps are issued directly, not as graphs, while on).
struct Profiler {
    struct Rec {
        int stage, kernels;
        cudaEvent_t a, b;
    };
    bool on = false;
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double ms[ST_COUNT] = {};
    int64_t calls[ST_COUNT] = {}, kernels[ST_COUNT] = {};
    cudaEvent_t take();
    void enable(bool v);                  // stream synchronised by the caller
    cudaError_t collect();                // stream synchronised by the caller
    void release();
};

struct StepGraph {
    cudaGraphExec_t exec;
    int kernels;
};

// What distinguishes the launch sequence of one step from another.
struct StepKind {
    bool is_sort, bin_virt, sort_virt;
    int parity;  // list buffer that this step writes and reads
    // host transfers overlapping the step (sphnj_step_exchange): bit 0, wait
    // for StepIO::in before the first stage that reads fluid velocities,
    // densities or pressures; bit 1, record StepIO::rho_p after the fluid
    // update, which writes the step's last densities and pressures
    int io = 0;
    int key() const {
        return (is_sort ? 1 : 0) | (bin_virt ? 2 : 0) | (sort_virt ? 4 : 0) | (parity << 3) | (io << 4);
    }
};
struct StepIO {
    cudaEvent_t in = nullptr, rho_p = nullptr;
};

// Issues the launches of one step of every scene of g on stream st; returns
// the number of kernels launched.  Reads no host state that changes from
// step to step except through `k`, so the sequence can be captured (with
// the events of `io` as external event nodes).
template <class G>
int issue_step(G &g, const StepKind &k, cudaStream_t st, const TileConfig &tc, Profiler *prof,
               const StepIO *io = nullptr);

}  // namespace sphnj

struct sphnj_ctx {
    sphnj_params p;
    sphnj::Profiler prof;
    uint64_t launches = 0;
    int form = SPHNJ_FORM_PLAIN;
    int device = 0;
    cudaStream_t own = nullptr, st = nullptr;
    // sphnj_step_exchange: the stream of its overlapped transfers and their
    // events (created on first use)
    cudaStream_t io_st = nullptr;
    cudaEvent_t ev_start = nullptr, ev_in = nullptr, ev_rho_p = nullptr, ev_out = nullptr;
    char *arena = nullptr;
    size_t arena_bytes = 0;
    sphnj::DevState d{};
    sphnj::CellList lf[2]{}, ls[2]{}, lv{};
    sphnj::ListScratch sc{};
    void *payload = nullptr;
    sphnj::DevErr *h_err = nullptr;  // pinned
    int step = 0;
    int parity = 0;
    bool virt_sorted = false;
    bool virt_cells_valid = false;  // virtual cell ids computed since the last upload
    bool uploaded = false;
    int *f_listed_total = nullptr;
    double *diag_part = nullptr;       // device: per-block diagnostic partials
    sphnj_diag *diag_out = nullptr;    // device: the last diagnostics
    void *probe_buf = nullptr;         // device: probe points and results (grown on demand)
    int probe_cap = 0;
    sphnj::TileConfig tiles;
    bool use_graphs = true;  // replay each kind of step as a captured CUDA graph
    bool pdl = true;         // programmatic dependent launch between the kernels of a step
    std::map<int, sphnj::StepGraph> graphs;
    sphnj_batch *batch = nullptr;  // the batch this scene belongs to, if any
    std::string msg = "ok";
};

namespace sphnj {

// The scene record of ctx with the cell lists of buffer `parity` bound.
Scene scene_of(const sphnj_ctx *ctx, int parity);
// The kind of launch sequence the next step of ctx needs, from its host-side
// step state, which is left unchanged.
StepKind next_kind(const sphnj_ctx *ctx);
// Advances the host-side step state of ctx past a step of kind k (its
// next_kind), once that step's launches have been issued: a step whose
// capture or launch fails leaves the state where it was, so a retry repeats
// the same step.
void commit_step(sphnj_ctx *ctx, const StepKind &k);
// Copies the device error record of ctx to the host (synchronising its
// stream) and turns it into a status and message.
int check_device_error(sphnj_ctx *ctx);
// The status and message of the device error record last copied to the host.
int device_error_status(sphnj_ctx *ctx);

// Trial runs of the sweep configurations (autotune.cu): from a device copy
// of the contexts' complete state, each candidate runs `steps` steps twice
// (the first captures its graphs), the second timed with CUDA events on `st`;
// the state is put back after every trial and at the end.  `apply` installs a
// candidate, `step` advances every context; with `classes` the scenes are
// split into two size classes whose tile heights are tuned apart.  Returns
// the fastest candidate.
struct Tuned {
    TileConfig launch;              // tiled switch and block sizes
    int tile_h[2] = {16, 16};       // per size class
    bool lists[2] = {true, true};
    int split = 0;                  // fluid count at which class 1 starts (0: one class)
    std::vector<int> cls;           // class of each context
};
struct TuneResult {
    Tuned best;
    double ms_per_step;
    int tried;
};
int tune_sweeps(const std::vector<sphnj_ctx *> &ctxs, cudaStream_t st, int steps, bool classes,
                int (*apply)(void *, const Tuned &), int (*step)(void *, int), void *obj, TuneResult *out);
void tuning_out(const TuneResult &r, sphnj_tuning *out);

}  // namespace sphnj
