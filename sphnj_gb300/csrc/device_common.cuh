// Device-side building blocks of libsphnj: the SoA pointer table passed to
// every kernel, the cell grid, error flagging and small vector helpers.
//
// HBM layout (one arena per context, every sub-buffer 256-byte aligned):
//   fluid  : pos float2, vel float2, rho float, p float, phase/boundary/near
//            uint8, du_dx float4 (column-major 2x2), gradient float2,
//            du_dt float2, color float, drho_dt float, cell int32
//   solid  : pos/ref/vel/du_dt double2, F/P/L/max_strain dmat2 (32 B),
//            pressure float, normal/couple float2, boundary/material uint8,
//            cell int32
//   virtual: pos/normal/vel float2, p/rho float, phase/boundary uint8,
//            cell int32
//   cells  : per particle kind a CSR range table int2{start,count}[C] and
//            an index list int32[N]; fluid and solid tables are double
//            buffered (previous/current) for the incremental rebuild.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sphnj.h"

namespace sphnj {

struct __align__(32) dmat2 {
    double m00, m10, m01, m11;  // column-major, as Eigen::Matrix2d
};

struct DevErr {
    int code;       // first error wins (atomicCAS from 0)
    int info[3];
};

// Pointers to one scene's device state.  Passed by value to kernels.
struct DevState {
    // fluid
    float2 *f_pos, *f_vel, *f_grad, *f_dudt;
    float *f_rho, *f_p, *f_color, *f_drho;
    float4 *f_dudx;
    uint8_t *f_phase, *f_fbt, *f_near;
    int *f_cell;
    // second fluid position buffer of the shifting passes: a pass reads the
    // positions (f_pos, or f_off in the mixed form) and writes the shifted
    // ones here; the launches of odd passes exchange the two pointers
    float2 *f_x_alt;
    // The shifting passes in list order: before the first pass the positions
    // (f_pos, or f_off) and cell ids of the listed fluid particles are
    // gathered by their position h in the fluid CSR list into f_xl and
    // f_celll; every pass reads and writes them there (f_xl, f_xl_alt,
    // exchanged like f_pos / f_x_alt), so that staging a tile's neighbours
    // reads contiguous ranges and a home particle's position and cell need
    // no gather through the list; after the last pass they are scattered
    // back.  Particles in no list stay in the particle arrays.
    float2 *f_xl, *f_xl_alt;
    int *f_celll;
    uint8_t *f_btl;  // boundary types the shifting update assigns, gathered with them
    // solid
    double2 *s_pos, *s_ref, *s_vel, *s_dudt;
    dmat2 *s_F, *s_P, *s_L, *s_maxstrain;
    float *s_p;
    float2 *s_normal, *s_couple;
    uint8_t *s_bt, *s_mat;
    int *s_cell;
    // virtual
    float2 *v_pos, *v_normal, *v_vel;
    float *v_p, *v_rho;
    uint8_t *v_phase, *v_bt;
    int *v_cell;
    // current cell lists (CSR) used by the neighbour sweeps
    const int2 *rng_f, *rng_s, *rng_v;
    const int *lst_f, *lst_s, *lst_v;
    // which fluid particles the current lists hold (listed[i] == *stamp) and
    // how many; the stamp is advanced on the device at the start of every step
    // (so that a captured step graph replays correctly)
    int *f_listed;
    const int *f_listed_total;
    int *stamp;
    // neighbour lists of this step, indexed by the particle's position h in
    // the fluid CSR list: the tile slots t (as uint16 byte offsets 8 t into
    // the tile's staged positions) of the fluid entries - and, next to a
    // wall, of the virtual entries, staged after the fluid ones - that
    // were within the cutoff plus skin when the pair pass ran, in the
    // reference's order, up to 128 bytes per particle moved in 16-byte chunks
    // of 8 slots, chunk c of particle h at f_nbr[c nf + h] (a warp's
    // consecutive particles read one contiguous run per chunk), and their count
    // (kNbrNone: no list - the stencil holds solid entries, the tile's
    // strips were not staged, or the list would exceed kNbrCap)
    uint4 *f_nbr;
    uint8_t *f_nbr_cnt;
    // max |displacement|^2 (float bits) of each position update since the
    // pair pass: [0] fluid update, [1 + k] shifting pass k
    unsigned int *disp2_bits;
    // tiles of the neighbour sweeps that hold fluid this step (in tile order)
    // and their number; reset by binning, filled after the cell lists are built
    int *tile_list, *tile_count;
    // scalars
    unsigned int *max_speed2_bits;  // max over fluid of |v|^2 (float bits)
    DevErr *err;
    // ---- mixed-precision form only (null in the plain form) ----------------
    // Positions are an integer cell (f_cell, s_cell, v_cell: the cell the
    // particle is listed in) plus an FP32 offset from that cell's lower-left
    // corner; fluid positions and velocities carry Kahan compensations.
    float2 *f_off, *f_offc, *f_velc;
    // the listed fluid particles' offsets and their compensations before the
    // step's first shifting pass, in list order (the velocity correction of
    // all passes is applied once, from the total displacement, after the last)
    float2 *f_x0l, *f_xc0l;
    // the listed particles' offset compensations during the shifting passes,
    // in list order (back to f_offc after the last pass)
    float2 *f_offcl;
    // Solids: reference position = reference cell (x, y) + FP32 offset;
    // current position = reference position + FP32 displacement u (Kahan);
    // s_off is the current offset from the corner of s_cell (set by binning).
    int2 *s_rc;
    float2 *s_roff, *s_u, *s_uc, *s_v, *s_vc, *s_off, *s_acc;
    float4 *s_PL, *s_FL;  // P L and F L of the last deformation pass (FP32, column-major)
    // per solid particle, the solid neighbours that passed the deformation
    // pass's reference-distance test, in its order (the force pass visits
    // the same ones): entry k of particle i at s_nbr[k ns + i], their number
    // in s_nbr_cnt (kNbrNone: more than kSolidNbrCap, walk the stencil)
    int *s_nbr;
    uint8_t *s_nbr_cnt;
    float2 *v_off;
};

__device__ __forceinline__ void raise_error(DevErr *e, int code, int a = 0, int b = 0, int c = 0) {
    if (atomicCAS(&e->code, 0, code) == 0) {
        e->info[0] = a;
        e->info[1] = b;
        e->info[2] = c;
    }
}

// Non-finite state: the update kernels raise SPHNJ_ERR_NONFINITE (kind,
// particle index) for the first particle whose updated position, velocity or
// density is NaN or infinite.  The reference steps on silently; values are
// left as they are, so the check changes no result.
__device__ __forceinline__ bool finite2(float2 a) { return isfinite(a.x) && isfinite(a.y); }
__device__ __forceinline__ bool finite2(double2 a) { return isfinite(a.x) && isfinite(a.y); }

// findPositionCell, pair.cu:8-18: x-major cell id from the float position,
// (y - ymin) * inv_dy truncated toward zero plus the column index times ny.
// Explicit round-to-nearest intrinsics keep the result independent of
// contraction, so ids are bit-identical to the reference's host/device math.
__device__ __forceinline__ int cell_of(const sphnj_params &p, float x, float y) {
    int iy = (int)__fmul_rn(__fsub_rn(y, p.cell_xmin[1]), p.interval_inv[1]);
    int ix = (int)__fmul_rn(__fsub_rn(x, p.cell_xmin[0]), p.interval_inv[0]);
    return iy + ix * p.cell_number[1];
}

// Neighbour slot n (0..8) of cell c: n = 3*(di+1) + (dj+1), di the column
// (x) offset, dj the row (y) offset, -1 outside the grid - the table built
// by Sim::createCell, sim.cu:175-193.
__device__ __forceinline__ int neighbour_cell(int c, int n, int nx, int ny) {
    int ci = c / ny, cj = c - ci * ny;
    int i = ci + n / 3 - 1, j = cj + n % 3 - 1;
    if (i < 0 || i >= nx || j < 0 || j >= ny) return -1;
    return i * ny + j;
}

// Calls fn(t, n) for every slot t of the CSR list `rng` in the nine cells
// around cell c, in the order of the loop over neighbour slots n = 0..8.
// Cells are numbered column-major and a list's ranges follow the cell order,
// so rows cj-1..cj+1 of one column are one contiguous range of slots: three
// ranges instead of nine, their bounds loaded together up front.  With kSlot
// the slot n of each entry's cell is passed too (row cj starts at m1 and row
// cj+1 at m2 in the column's range); otherwise n is 0.
template <bool kSlot, class Fn>
__device__ __forceinline__ void for_each_in_stencil(const int2 *rng, int c, int nx, int ny, Fn &&fn) {
    const int ci = c / ny, cj = c - ci * ny;
    const int r0 = max(cj - 1, 0), r1 = min(cj + 1, ny - 1);
    int2 lo[3], mid[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int col = ci + k - 1;
        lo[k] = mid[k] = hi[k] = make_int2(0, 0);
        if (col >= 0 && col < nx) {
            lo[k] = __ldg(&rng[col * ny + r0]);
            hi[k] = __ldg(&rng[col * ny + r1]);
            if constexpr (kSlot) mid[k] = __ldg(&rng[col * ny + cj]);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int b = lo[k].x, e = hi[k].x + hi[k].y;
        const int m1 = mid[k].x, m2 = cj + 1 < ny ? hi[k].x : e;
        for (int t = b; t < e; ++t) {
            if constexpr (kSlot) fn(t, 3 * k + (t >= m1) + (t >= m2));
            else fn(t, 0);
        }
    }
}

// Gaussian kernel-gradient factor exp(-q^2) * Kd * C32 (fluid.cu:44-46)
__device__ __forceinline__ float grad_w(const sphnj_params &p, float q2) {
    return expf(-q2) * p.kernel_differential * p.coefficient_3d_to_2d;
}
// Truncated-Gaussian Shepard weight (exp(-q^2) - e^{-R^2}) * C2 * C32
// (virt.cu:71-74, solid.cu:381-386)
__device__ __forceinline__ float shepard_w(const sphnj_params &p, float q2) {
    return (expf(-q2) - p.kernel_coefficient_1) * p.kernel_coefficient_2 * p.coefficient_3d_to_2d;
}

// Sums of two products are written with explicit round-to-nearest
// intrinsics: left to the compiler, `a*b + c*d` may be contracted into an FMA
// around either product, and the choice can differ between the kernels a
// helper is inlined into - which would make the tiled and per-particle sweeps
// differ in the last bit.
__device__ __forceinline__ float sum2(float a, float b, float c, float d) { return __fmaf_rn(c, d, __fmul_rn(a, b)); }
__device__ __forceinline__ float sqn(float2 a) { return sum2(a.x, a.x, a.y, a.y); }
__device__ __forceinline__ float dot2(float2 a, float2 b) { return sum2(a.x, b.x, a.y, b.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// Eigen normalized(): zero vector returned unchanged
__device__ __forceinline__ float2 normalized(float2 a) {
    float z = sqn(a);
    if (z > 0.0f) {
        float s = sqrtf(z);
        return make_float2(a.x / s, a.y / s);
    }
    return a;
}
__device__ __forceinline__ float2 to_f2(double2 a) { return make_float2((float)a.x, (float)a.y); }

__device__ __forceinline__ dmat2 dmul(const dmat2 &a, const dmat2 &b) {
    return {a.m00 * b.m00 + a.m01 * b.m10, a.m10 * b.m00 + a.m11 * b.m10,
            a.m00 * b.m01 + a.m01 * b.m11, a.m10 * b.m01 + a.m11 * b.m11};
}
__device__ __forceinline__ double2 dmv(const dmat2 &a, double2 v) {
    return make_double2(a.m00 * v.x + a.m01 * v.y, a.m10 * v.x + a.m11 * v.y);
}
__device__ __forceinline__ dmat2 dtrans(const dmat2 &a) { return {a.m00, a.m01, a.m10, a.m11}; }
__device__ __forceinline__ double ddet(const dmat2 &a) { return a.m00 * a.m11 - a.m10 * a.m01; }
__device__ __forceinline__ dmat2 dinv(const dmat2 &a) {
    double inv = 1.0 / ddet(a);
    return {a.m11 * inv, -a.m10 * inv, -a.m01 * inv, a.m00 * inv};
}

constexpr int kMaskShifts = 32;       // shifting passes tracked by disp2_bits
constexpr float kSkin = 0.05f;        // list radius = cutoff * (1 + kSkin)
constexpr int kNbrCap = 64;           // neighbour-list entries per particle
constexpr int kNbrChunks = kNbrCap / 8;  // 16-byte chunks per list
constexpr int kSolidNbrCap = 64;      // listed solid neighbours per solid particle (mixed form)
constexpr uint8_t kNbrNone = 0xFF;
constexpr float EPS_FOR_SUM = 0.1f;   // global.h:6
constexpr float LARGE_FLOAT = 1.0E6f; // global.h:7
constexpr int SCAN_TILE = 1024;       // cells per block in the two-level scans
constexpr int SCAN_MAX_TILES = 4096;  // => up to 4M cells per scene

inline unsigned grid_for(long n, int block) { return (unsigned)((n + block - 1) / block); }

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

// Everything a kernel reads about one scene: its parameters, its state (with
// the current cell lists bound in `d`), both list buffers of each kind, and
// its sort / rebuild scratch.
struct Scene {
    sphnj_params p;
    DevState d;
    CellList lf[2], ls[2], lv;
    ListScratch sc;
    char *payload;        // sort payload staging
    int *f_listed_total;  // fluid particles in the current lists (written by the list scans)
    // sweep shape of this scene: cells per tile of the tiled neighbour sweeps
    // and whether its pair pass stores neighbour lists (the scenes of a batch
    // may have different shapes, chosen by size)
    int tile_h, lists, pad_[4];
};

__device__ __forceinline__ void pdl_enter();

// Where a block finds its scene.  Every kernel of the step is a template over
// one of the two, and starts with SPHNJ_SCENE(g), which defines
//   blk, nblk  the block's index among its scene's blocks, and their number
//   S, p, d    the scene record, its parameters and its state.
//
// One: a launch over one scene, the record a __grid_constant__ kernel
// parameter (read in place from parameter space).
struct One {
    Scene s;
    __device__ __forceinline__ const Scene *locate(int &blk, int &nblk) const {
        blk = blockIdx.x;
        nblk = gridDim.x;
        return &s;
    }
    // a block of a sweep over the scene's active-tile list: waits for the
    // launch's predecessor (pdl_enter), then reads the list's length; null
    // when the block has no tile of it
    __device__ __forceinline__ const Scene *locate_listed(int &blk, int &nblk, int &n_active) const {
        blk = blockIdx.x;
        nblk = gridDim.x;
        pdl_enter();
        n_active = *s.d.tile_count;
        return blk < n_active ? &s : nullptr;
    }
};

// Many: one launch over many scenes.  Each scene owns a run of consecutive
// blocks (a scene with no work for this launch owns none); the launch's block
// table gives block b its scene, its index within the scene's run and the
// run's length in one 16-byte entry, so a block finds its scene with one
// load.  The block copies its scene's record into shared memory, so that the
// kernel reads its fields with shared loads at fixed addresses (as a
// one-scene launch reads them from parameter space) rather than holding
// global addresses in registers.
struct Many {
    const Scene *scenes;
    const int4 *blocks;  // [grid size]: {scene, blk, nblk, 0}
    int n;
    __device__ __forceinline__ const Scene *locate(int &blk, int &nblk) const {
        __shared__ __align__(16) Scene s_scene;
        static_assert(sizeof(Scene) % 16 == 0, "the record is copied in 16-byte words");
        const int4 t = __ldg(&blocks[blockIdx.x]);
        blk = t.y;
        nblk = t.z;
        const int4 *src = reinterpret_cast<const int4 *>(scenes + t.x);
        int4 *dst = reinterpret_cast<int4 *>(&s_scene);
        for (int w = threadIdx.x; w < (int)(sizeof(Scene) / 16); w += blockDim.x) dst[w] = __ldg(&src[w]);
        __syncthreads();
        return &s_scene;
    }
    // As One::locate_listed.  A batched list launch has more blocks than its
    // scenes have active tiles; a block without a tile reads only its
    // scene's list length (two dependent loads) and returns before copying
    // the record.
    __device__ __forceinline__ const Scene *locate_listed(int &blk, int &nblk, int &n_active) const {
        const int4 t = __ldg(&blocks[blockIdx.x]);
        blk = t.y;
        nblk = t.z;
        pdl_enter();
        const int *count = scenes[t.x].d.tile_count;
        n_active = *count;
        if (blk >= n_active) return nullptr;
        __shared__ __align__(16) Scene s_scene;
        const int4 *src = reinterpret_cast<const int4 *>(scenes + t.x);
        int4 *dst = reinterpret_cast<int4 *>(&s_scene);
        for (int w = threadIdx.x; w < (int)(sizeof(Scene) / 16); w += blockDim.x) dst[w] = __ldg(&src[w]);
        __syncthreads();
        return &s_scene;
    }
};

// Programmatic dependent launch: every kernel of a step is launched with
// programmatic stream serialisation (when the context has it on), so that its
// blocks can be scheduled while the previous kernel's last blocks still run.
// Before a kernel reads anything an earlier kernel wrote it waits for the
// previous grid to complete and its writes to be visible
// (griddepcontrol.wait; a no-op in a launch without the attribute); then it
// lets the next kernel's blocks be scheduled.  Only the block's scene lookup
// (constant records and block tables) comes before the wait.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The neighbour sweeps: with kList (blocks loop over the scene's active-tile
// list) the block reads the list's length first and, when it has no tile of
// it, returns before loading anything else (locate_listed).
template <bool kList, class G>
__device__ __forceinline__ const Scene *locate_sweep(const G &g, int &blk, int &nblk, int &n_active) {
    if constexpr (kList) {
        return g.locate_listed(blk, nblk, n_active);
    } else {
        const Scene *s = g.locate(blk, nblk);
        pdl_enter();
        return s;
    }
}
#define SPHNJ_SCENE_SWEEP(g, kList, n_active)                                          \
    int blk, nblk;                                                                    \
    const ::sphnj::Scene *S_ptr_ = ::sphnj::locate_sweep<kList>(g, blk, nblk, n_active); \
    if (!S_ptr_) return;                                                              \
    const ::sphnj::Scene &S = *S_ptr_;                                                \
    const sphnj_params &p = S.p;                                                      \
    const ::sphnj::DevState &d = S.d;                                                 \
    (void)nblk;                                                                       \
    (void)p;                                                                          \
    (void)d

#define SPHNJ_SCENE(g)                                   \
    int blk, nblk;                                       \
    const ::sphnj::Scene &S = *(g).locate(blk, nblk);    \
    ::sphnj::pdl_enter();                                \
    const sphnj_params &p = S.p;                         \
    const ::sphnj::DevState &d = S.d;                    \
    (void)nblk;                                          \
    (void)p;                                             \
    (void)d

}  // namespace sphnj
