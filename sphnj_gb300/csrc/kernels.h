// Host-side launchers for the sm_103a kernels of libsphnj.  Each wraps one
// or more kernel launches on the given stream; none synchronises.
#pragma once

#include <cuda_runtime.h>

#include "device_common.cuh"

namespace sphnj {

// CSR cell list of one particle kind
struct CellList {
    int2 *rng;  // [C] {start, count}
    int *lst;   // [N] particle indices, cell by cell
};

// Scratch for sorting / list rebuilding of one particle kind
struct ListScratch {
    int *cnt9;    // [9*C] per (destination cell, neighbour slot) counts
    int *cnt;     // [C]
    int *local;   // [C] tile-local exclusive prefix
    int *sums;    // [SCAN_MAX_TILES] tile sums (scanned in place)
    int *cursor;  // [C]
    int *bucket;  // [N]
    int *sorted;  // [N]
};

// kinds
enum Kind { KF = 0, KS = 1, KV = 2 };

// Which particles a list build placed in some cell list: listed[i] = stamp
// for each of them, and *total = their number.  The tiled neighbour sweeps
// process listed particles cell by cell; particles that dropped out of every
// list (a jump of more than one cell between sorts) are processed by the
// per-particle fallback kernels.  Null members: nothing recorded.
struct Listing {
    int *listed = nullptr;
    const int *stamp = nullptr;  // device value of this step's stamp
    int *total = nullptr;
};

// cells: cell ids of every particle (pair.cu:20-64); also resets the
// per-step max-speed accumulator.
void launch_bin(cudaStream_t st, const sphnj_params &p, const DevState &d, bool with_virt);

// stable sort of one kind by cell id + identity cell lists (sort.cu:10-137)
void launch_sort_kind(cudaStream_t st, const sphnj_params &p, const DevState &d, Kind k, int n, int *cell,
                      ListScratch sc, CellList cur, void *payload_scratch, Listing lg = Listing());

// incremental cell-list rebuild of one kind from its previous lists
// (pair.cu:66-181)
void launch_rebuild_kind(cudaStream_t st, const sphnj_params &p, int n, const int *cell, CellList prev,
                         CellList cur, ListScratch sc, DevErr *err, Listing lg = Listing());

// per-cell capacity check against the reference's 64 slots
void launch_capacity_check(cudaStream_t st, const sphnj_params &p, const DevState &d);

// How the fluid neighbour sweeps are launched: tiled (a block per column
// segment of tile_h cells, neighbours staged in shared memory) or one thread
// per particle.  Both give identical results.
struct TileConfig {
    bool tiled = true;
    int tile_h = 16;
};

// Function attributes the sweeps need for this configuration (dynamic shared
// memory above 48 KB); called outside any stream capture.
cudaError_t configure_sweeps(const TileConfig &tc);

// fluid passes (fluid.cu)
void launch_fluid_pair(cudaStream_t st, const sphnj_params &p, const DevState &d, const TileConfig &tc);
void launch_fluid_update(cudaStream_t st, const sphnj_params &p, const DevState &d);
// pass = index of the shifting pass within the step (0..shift_per_step-1)
void launch_shift_gradient(cudaStream_t st, const sphnj_params &p, const DevState &d, const TileConfig &tc,
                           int pass);
void launch_shift_update(cudaStream_t st, const sphnj_params &p, const DevState &d, int pass);

// virtual particles (virt.cu)
void launch_virt_normal(cudaStream_t st, const sphnj_params &p, const DevState &d);
void launch_virt_data(cudaStream_t st, const sphnj_params &p, const DevState &d);

// solid (solid.cu)
void launch_solid_couple(cudaStream_t st, const sphnj_params &p, const DevState &d);
void launch_solid_deformation(cudaStream_t st, const sphnj_params &p, const DevState &d);
void launch_solid_force(cudaStream_t st, const sphnj_params &p, const DevState &d);
void launch_solid_update(cudaStream_t st, const sphnj_params &p, const DevState &d);

// state conversion helpers (upload / download of 32-bit enums)
void launch_u8_from_i32(cudaStream_t st, uint8_t *dst, const int32_t *src, int n);
void launch_i32_from_u8(cudaStream_t st, int32_t *dst, const uint8_t *src, int n);
void launch_fill_u8(cudaStream_t st, uint8_t *dst, uint8_t v, int n);
void launch_fill_dmat2(cudaStream_t st, dmat2 *dst, dmat2 v, int n);
void launch_fill_f32(cudaStream_t st, float *dst, float v, int n);

}  // namespace sphnj
