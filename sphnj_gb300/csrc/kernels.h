// Host-side launchers for the sm_103a kernels of libsphnj.  Each wraps one
// or more kernel launches on the given stream, returns how many kernels it
// launched, and never synchronises.
//
// Every launcher is a template over the group of scenes it advances:
//   GroupOne   one scene; its record travels as a kernel parameter.
//   GroupMany  a batch of independent scenes advanced by the same launches:
//              the records live in device memory and each launch gets a
//              block table (scene k owns a run of consecutive blocks; each
//              block's entry names its scene and its place in the run), so
//              one launch covers every scene and a scene with no work for it
//              owns no block.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <utility>
#include <vector>

#include "device_common.cuh"

namespace sphnj {

// How the fluid neighbour sweeps are launched: tiled (a block per column
// segment of tile_h cells, neighbours staged in shared memory) or one thread
// per particle, and the block sizes of the tiled sweeps.  Every choice gives
// identical results.  tile_h and lists are a scene's own (copied into its
// record, so the scenes of a batch may differ); tiled and the block sizes
// belong to a launch.
struct TileConfig {
    bool tiled = true;
    int tile_h = 16;
    bool lists = true;    // tiled: store per-step neighbour lists (else walk the stencil in every pass)
    int shift_block = 0;  // threads per block of the tiled shifting passes: 64, 128, 256 (0: per launch kind)
    int pair_block = 0;   // threads per block of the tiled pair pass: 128, 256 (0: per launch kind)
};

// Launch sites: a batch keeps one block table per (site, argument).
enum Site : int {
    SITE_BIN, SITE_SORT_CLEAR, SITE_SORT_N, SITE_SORT_TILES, SITE_SORT_ONE, SITE_SORT_CELLS32,
    SITE_REBUILD_CELLS, SITE_REBUILD_TILES, SITE_REBUILD_ONE, SITE_REBUILD_ZERO, SITE_CAPACITY, SITE_COUPLE,
    SITE_VIRT_NORMAL, SITE_VIRT_DATA, SITE_PAIR_TILED, SITE_PAIR_EACH, SITE_PAIR_FALLBACK, SITE_FLUID_UPDATE, SITE_SOLID_DEFORM,
    SITE_SOLID_FORCE, SITE_SOLID_UPDATE, SITE_SHIFT_TILED, SITE_SHIFT_EACH, SITE_SHIFT_FALLBACK,
    SITE_SHIFT_COPY_BACK, SITE_TILE_COMPACT, SITE_TILE_SUMS, SITE_TILE_SCATTER, SITE_VIRT_BIN, SITE_SHIFT_GATHER,
    SITE_SHIFT_SCATTER
};
inline long long site_key(int site, int arg = 0) { return ((long long)site << 32) | (unsigned)arg; }

// The record with its fluid position buffer (f_pos, or f_off in the mixed
// form) and the shifting passes' second buffer f_x_alt exchanged.
inline void exchange_positions(Scene &s, int form) {
    float2 *&x = form == SPHNJ_FORM_MIXED ? s.d.f_off : s.d.f_pos;
    float2 *t = x;
    x = s.d.f_x_alt;
    s.d.f_x_alt = t;
    t = s.d.f_xl;  // the list-order pair of the shifting passes
    s.d.f_xl = s.d.f_xl_alt;
    s.d.f_xl_alt = t;
}

// exchange_positions() switches the group's records between the two buffer
// assignments (called in pairs around the launches of an odd shifting pass).
struct GroupOne {
    using Dev = One;
    Scene s;
    int form = SPHNJ_FORM_PLAIN;
    bool pdl = false;  // launch with programmatic stream serialisation
    template <class F> bool prepare(long long, F &&blocks_of, unsigned &blocks, Dev &dev) {
        blocks = blocks_of(s);
        dev.s = s;
        return blocks > 0;
    }
    template <class Pred> bool any(Pred &&pr) const { return pr(s.p); }
    void exchange_positions() { sphnj::exchange_positions(s, form); }
};

struct GroupMany {
    using Dev = Many;
    const Scene *h_scenes = nullptr;  // host copies of the first n records of d_scenes
    int n = 0;
    int form = SPHNJ_FORM_PLAIN;      // every scene of a group has the same form
    bool pdl = false;                 // launch with programmatic stream serialisation
    // device records of the current list parity: n records, then the same n
    // with their position buffers exchanged
    const Scene *d_scenes = nullptr;
    bool exchanged = false;
    void exchange_positions() { exchanged = !exchanged; }
    // With `planning` set, prepare() builds the block table of each launch
    // (synchronous allocation and copy) and launches nothing; a launch
    // sequence is planned once before it is captured into a graph.
    bool planning = false;
    struct Table {
        int4 *blocks;  // per block: {scene, index within the scene's run, run length, 0}
        unsigned total;
    };
    std::map<long long, Table> tables;
    cudaError_t error = cudaSuccess;
    template <class F> bool prepare(long long key, F &&blocks_of, unsigned &blocks, Dev &dev) {
        auto it = tables.find(key);
        if (it == tables.end()) {
            if (!planning) {
                if (error == cudaSuccess) error = cudaErrorNotReady;  // launch not planned
                return false;
            }
            std::vector<unsigned> run((size_t)n, 0u);
            long long acc = 0;
            for (int k = 0; k < n; ++k) {
                run[k] = blocks_of(h_scenes[k]);
                acc += run[k];
            }
            Table t{nullptr, (unsigned)acc};
            if (acc > 0x7fffffffLL) {
                error = cudaErrorInvalidValue;
                return false;
            }
            cudaError_t e = cudaSuccess;
            if (acc > 0) {
                std::vector<int4> table((size_t)acc);
                size_t b = 0;
                for (int k = 0; k < n; ++k)
                    for (unsigned j = 0; j < run[k]; ++j) table[b++] = make_int4(k, (int)j, (int)run[k], 0);
                e = cudaMalloc(&t.blocks, sizeof(int4) * table.size());
                if (e == cudaSuccess)
                    e = cudaMemcpy(t.blocks, table.data(), sizeof(int4) * table.size(), cudaMemcpyHostToDevice);
            }
            if (e != cudaSuccess) {
                if (t.blocks) cudaFree(t.blocks);
                error = e;
                return false;
            }
            it = tables.emplace(key, t).first;
        }
        if (planning) return false;
        blocks = it->second.total;
        dev.scenes = d_scenes + (exchanged ? n : 0);
        dev.blocks = it->second.blocks;
        dev.n = n;
        return blocks > 0;
    }
    template <class Pred> bool any(Pred &&pr) const {
        for (int k = 0; k < n; ++k)
            if (pr(h_scenes[k].p)) return true;
        return false;
    }
    void free_tables() {
        for (auto &t : tables)
            if (t.second.blocks) cudaFree(t.second.blocks);
        tables.clear();
    }
};

// Launches `kern` over the blocks that blocks_of(scene) gives each scene of
// the group; returns 1 when something was launched.
template <class G, class F, class... P, class... A>
int launch(G &g, long long key, F &&blocks_of, void (*kern)(typename G::Dev, P...), int threads, size_t smem,
           cudaStream_t st, A &&...a) {
    unsigned blocks = 0;
    typename G::Dev dev;
    if (!g.prepare(key, blocks_of, blocks, dev)) return 0;
    if (g.pdl) {
        // programmatic dependent launch: the kernel waits for its predecessor
        // in pdl_enter (SPHNJ_SCENE), so its blocks may be scheduled early
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(blocks);
        cfg.blockDim = dim3(threads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, kern, dev, std::forward<A>(a)...);  // errors: cudaGetLastError of the caller
    } else {
        kern<<<blocks, threads, smem, st>>>(dev, std::forward<A>(a)...);
    }
    return 1;
}

__host__ __device__ inline int count_of(const sphnj_params &p, Kind k) {
    return k == KF ? p.fluid_number_total : k == KS ? p.solid_number : p.virt_number;
}

// Tiles of the neighbour sweeps of one scene (column segments of tile_h cells).
__host__ __device__ inline int sweep_tiles(const sphnj_params &p, int tile_h) {
    return p.cell_number[0] * ((p.cell_number[1] + tile_h - 1) / tile_h);
}
// A scene whose fluid fills few of its tiles - under 64 particles per tile on
// average (a dam break before the surge fills a small corner of its tank) -
// sweeps only the tiles listed active this step; a dense scene swept alone
// gives every tile a block (an empty one returns at once), which saves the
// list's dependent loads at the start of every block.  Batched launches sweep
// every scene through its list.
__host__ __device__ inline bool sweep_compacted(const sphnj_params &p, int tile_h) {
    return p.fluid_number_total > 0 && (long)p.fluid_number_total < 64L * sweep_tiles(p, tile_h);
}

// cells: cell ids of every particle (pair.cu:20-64); also resets the
// per-step accumulators and advances the list stamp.
template <class G> int launch_bin(cudaStream_t st, G &g, bool with_virt);

// stable sort of one kind by cell id + identity cell lists written to list
// buffer `parity` (sort.cu:10-137)
template <class G> int launch_sort_kind(cudaStream_t st, G &g, Kind k, int parity);

// cell ids of the virtual particles and their per-cell index lists in
// ascending order (ranges in lv.rng, indices in the sort scratch sc.sorted),
// the arrays left in their order: the lists of the wall normals at upload
template <class G> int launch_virt_index(cudaStream_t st, G &g);

// incremental cell-list rebuild of one kind from list buffer parity ^ 1 into
// list buffer `parity` (pair.cu:66-181)
template <class G> int launch_rebuild_kind(cudaStream_t st, G &g, Kind k, int parity);

// this step's active tiles of the tiled sweeps (each scene's own tile
// height) into d.tile_list / d.tile_count, in tile order: for every scene
// with fluid (all_scenes) or for the scenes that sweep_compacted() selects
template <class G> int launch_tile_compact(cudaStream_t st, G &g, bool all_scenes);

// per-cell capacity check against the reference's 64 slots
template <class G> int launch_capacity_check(cudaStream_t st, G &g);

// Function attributes the sweeps need for this configuration (dynamic shared
// memory above 48 KB); called outside any stream capture.
cudaError_t configure_sweeps(const TileConfig &tc);

// fluid passes (fluid.cu)
template <class G> int launch_fluid_pair(cudaStream_t st, G &g, const TileConfig &tc);
template <class G> int launch_fluid_update(cudaStream_t st, G &g);
// Shifting pass `pass` of the step (gradient and position update in one
// sweep; scenes with fewer shifting passes per step own no block of it; pass
// 0 first gathers the listed particles' positions into list order), and,
// after the last pass, the positions back to f_pos / f_off: from f_x_alt in
// the scenes whose number of passes is odd, then from list order.
template <class G> int launch_shift_pass(cudaStream_t st, G &g, const TileConfig &tc, int pass);
template <class G> int launch_shift_copy_back(cudaStream_t st, G &g);

// virtual particles (virt.cu).  launch_virt_normal builds the per-cell index
// lists it reads (launch_virt_index: v_cell, lv.rng and the sort scratch);
// the caller empties lv.rng again where the step expects empty lists.
template <class G> int launch_virt_normal(cudaStream_t st, G &g);
template <class G> int launch_virt_data(cudaStream_t st, G &g);

// solid (solid.cu); sub = index of the solid sub-step within the fluid step
template <class G> int launch_solid_couple(cudaStream_t st, G &g);
template <class G> int launch_solid_deformation(cudaStream_t st, G &g, int sub);
template <class G> int launch_solid_force(cudaStream_t st, G &g, int sub);
template <class G> int launch_solid_update(cudaStream_t st, G &g, int sub);

// mixed form: host layout -> mixed state for the kinds in `kinds` (bit 0
// fluid, bit 1 solid, bit 2 virtual), and mixed state -> host layout
// (absolute positions, FP64 solid position / velocity / acceleration)
void launch_mixed_split(cudaStream_t st, const GroupOne &g, int kinds);
void launch_mixed_join(cudaStream_t st, const GroupOne &g, int kinds);  // bit 0 fluid, bit 1 solid

// Fluid fields in device-mapped host memory (null: not moved), moved in
// place by one kernel: from_host writes the device state (the mixed form
// splits the positions as launch_mixed_split does), to_host reads it (the
// mixed form joins them as launch_mixed_join does, refreshing f_pos too).
struct FluidHost {
    float2 *pos, *vel;
    float *rho, *p;
    bool any() const { return pos || vel || rho || p; }
};
void launch_fluid_from_host(cudaStream_t st, const GroupOne &g, const FluidHost &h);
void launch_fluid_to_host(cudaStream_t st, const GroupOne &g, const FluidHost &h);
// whether [ptr, ptr + bytes) lies inside one sphnj_host_alloc allocation
bool host_mapped(const void *ptr, size_t bytes);

// global diagnostics (kernels_diag.cu): kDiagBlocks x kDiagSlots doubles of
// per-block partials, then the result in *out (device memory)
constexpr int kDiagBlocks = 304;
constexpr int kDiagSlots = 16;
void launch_diagnostics(cudaStream_t st, const GroupOne &g, double *part, int step, sphnj_diag *out);
// Shepard probes at n points (device arrays): out = {vx, vy, p, rho}
void launch_probe(cudaStream_t st, const GroupOne &g, int n, const float2 *pts, float4 *out);

// state conversion helpers (upload / download of 32-bit enums)
void launch_u8_from_i32(cudaStream_t st, uint8_t *dst, const int32_t *src, int n);
void launch_i32_from_u8(cudaStream_t st, int32_t *dst, const uint8_t *src, int n);
void launch_fill_u8(cudaStream_t st, uint8_t *dst, uint8_t v, int n);
void launch_fill_dmat2(cudaStream_t st, dmat2 *dst, dmat2 v, int n);
void launch_fill_f32(cudaStream_t st, float *dst, float v, int n);

#define SPHNJ_INSTANTIATE_GROUPS(fn, ...)                 \
    template int fn<GroupOne>(cudaStream_t, GroupOne &, ##__VA_ARGS__); \
    template int fn<GroupMany>(cudaStream_t, GroupMany &, ##__VA_ARGS__)

}  // namespace sphnj
