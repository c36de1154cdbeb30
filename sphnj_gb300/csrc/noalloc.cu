// Incremental cell-list rebuild for callers that cannot allocate device
// memory.
//
// Some callers of this library may not call cudaMalloc: code that runs while
// a host framework owns all device memory through its own pool allocator,
// plugin hosts that forbid allocation after start-up, and real-time loops
// that must not hit the driver's allocator (it can block and synchronise).
// They hand in every input and output buffer themselves.  The rebuild's
// scratch (per destination cell and neighbour slot counts, tile-local
// prefixes and tile sums) therefore lives in the file-scope array below,
// sized for at most SPHNJ_NOALLOC_MAX_CELLS cells.  Every GPU that loads this
// library holds that array until the process exits.
//
// The kernels are the ones the context path uses (launch_rebuild_kind); only
// the scratch pointers differ.
#include "kernels.h"

#include <mutex>

namespace {

constexpr int kMaxCells = SPHNJ_NOALLOC_MAX_CELLS;
constexpr int kMaxTiles = (kMaxCells + sphnj::SCAN_TILE - 1) / sphnj::SCAN_TILE;
// cnt9 (9 per cell) + tile-local prefix (1 per cell) + tile sums
constexpr size_t kScratchInts = (size_t)10 * kMaxCells + kMaxTiles;

// Shared by every call on a device: each call overwrites all of it before
// reading it (every (cell, valid slot) count, every prefix, every tile sum),
// so nothing has to be cleared between calls, but two calls that overlap on
// the GPU race on it.
static __device__ __align__(256) int g_rebuild_scratch[kScratchInts];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
int *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_rebuild_scratch in the current context.  In host code
// the array's name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, called with the device current.  Outside a stream
// capture it is looked up on every call, so that a caller on another context
// of the same device, or after a cudaDeviceReset (which reloads the module),
// gets the address of its own context; during a capture, where the lookup
// could load the module, the address cached per device by an earlier call
// is used (the first call on a device must therefore come before any
// capture, as the header states).
int scratch_for_current_device(cudaStream_t st, int **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SPHNJ_ERR_NO_DEVICE;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();
        return SPHNJ_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
        if (cap != cudaStreamCaptureStatusNone) return SPHNJ_ERR_ARG;  // first call inside a capture
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_rebuild_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return SPHNJ_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<int *>(ptr);
    }
    *out = g_scratch_ptr[dev];
    return SPHNJ_OK;
}

}  // namespace

extern "C" int sphnj_rebuild_cell_lists_noalloc(int nx, int ny, int n_particles, const int32_t *cell_id,
                                                const int32_t *prev_range, const int32_t *prev_list,
                                                int32_t *range_out, int32_t *list_out, void *stream) {
    if (nx < 3 || ny < 3 || n_particles < 0) return SPHNJ_ERR_ARG;
    if ((long)nx * ny > kMaxCells) return SPHNJ_ERR_UNSUPPORTED;  // beyond the static scratch
    if (!prev_range || !range_out || (n_particles > 0 && (!cell_id || !prev_list || !list_out)))
        return SPHNJ_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(prev_range) | reinterpret_cast<uintptr_t>(range_out)) & 7u)
        return SPHNJ_ERR_ARG;  // {start, count} pairs are read as 8-byte int2
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int *scratch = nullptr;
    int rc = scratch_for_current_device(st, &scratch);
    if (rc) return rc;
    const int C = nx * ny;
    if (n_particles == 0) {
        // no particles: every cell starts at 0 and holds none
        cudaError_t e = cudaMemsetAsync(range_out, 0, sizeof(int32_t) * 2 * (size_t)C, st);
        return e == cudaSuccess ? SPHNJ_OK : SPHNJ_ERR_CUDA;
    }
    // A scene record holding only what the rebuild reads: the grid, the
    // particles' cell ids (as fluid, with no listing), the two list buffers
    // (previous = 0, output = 1) and the static scratch.
    sphnj::GroupOne g{};
    sphnj::Scene &s = g.s;
    s.p.cell_number[0] = nx;
    s.p.cell_number[1] = ny;
    s.p.cell_number_total = C;
    s.p.fluid_number_total = n_particles;
    s.d.f_cell = const_cast<int32_t *>(cell_id);
    s.sc.cnt9 = scratch;
    s.sc.local = scratch + (size_t)9 * kMaxCells;
    s.sc.sums = scratch + (size_t)10 * kMaxCells;
    s.lf[0] = {reinterpret_cast<int2 *>(const_cast<int32_t *>(prev_range)), const_cast<int32_t *>(prev_list)};
    s.lf[1] = {reinterpret_cast<int2 *>(range_out), list_out};
    sphnj::launch_rebuild_kind(st, g, sphnj::KF, 1);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SPHNJ_OK : SPHNJ_ERR_CUDA;
}
