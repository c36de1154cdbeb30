// Cell-list construction on sm_103a: binning, the stable sort done every
// sort_every_step steps, and the per-step incremental list rebuild.
//
// Reference behaviour reproduced (bit-exact lists and sorted order):
//   - cell ids                 pair.cu:8-64
//   - stable sort by cell id   sort.cu:10-45 (thrust::sort_by_key; payload
//                              per kind from particle.cuh:93-96,176-179,
//                              238-241) and the per-cell ranges written by
//                              updateCell* (sort.cu:59-137)
//   - incremental rebuild      pair.cu:66-181: the new list of cell c is, for
//                              neighbour slot n = 0..8 in order, the entries
//                              of neighbour n's previous list whose new cell
//                              is c.  Because slot order equals increasing
//                              neighbour-cell id (ny >= 3), that list is the
//                              stable partition of the previous list order
//                              by new cell id, restricted to particles that
//                              moved at most one cell; particles that jumped
//                              further drop out of every list until the next
//                              sort, exactly as in the reference.
//
// GB300 design:
//   - sort = histogram + two-level scan + atomic bucket fill + a warp rank
//     sort inside each cell (indices are unique, so rank = number of smaller
//     indices); stable by construction, no radix passes, no library calls.
//   - rebuild = each old cell m scatters its non-zero outgoing counts to
//     cnt9[c][slot], zeroed first (every (c,slot) pair has at most one
//     writer, so no atomics), a tiled scan gives the new cell starts, and
//     m writes its particles to their destinations in previous-list order.
//   - every kernel runs over one scene or a batch of scenes (SPHNJ_SCENE):
//     each scene's scan, sort and rebuild use that scene's own scratch, so
//     the scenes of a batch share launches but no data.
#include "forms.cuh"
#include "kernels.h"

#include <climits>

namespace sphnj {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ int *cells_of(const DevState &d, int k) {
    return k == KF ? d.f_cell : k == KS ? d.s_cell : d.v_cell;
}
__device__ __forceinline__ const CellList &list_of(const Scene &S, int k, int parity) {
    return k == KF ? S.lf[parity] : k == KS ? S.ls[parity] : S.lv;
}

// Mixed form: the cell of a position given as offset `off` from the corner of
// cell (cx, cy), with `off` moved into that cell (off - k w in one rounding).
// A cell outside the grid is reported as the reference's out-of-bounds read
// would not be (SPHNJ_ERR_OUT_OF_GRID) and clamped to the grid, the offset
// kept relative to the clamped cell.
__device__ __forceinline__ int rebase(const sphnj_params &p, const DevState &d, int kind, int i, int cx, int cy,
                                      float2 &off) {
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float wx = p.interval[0], wy = p.interval[1];
    if (!(off.x >= 0.0f && off.x < wx)) {
        const float k = fminf(fmaxf(floorf(__fdiv_rn(off.x, wx)), -1.0e6f), 1.0e6f);
        if (k == k) {
            off.x = __fmaf_rn(-k, wx, off.x);
            cx += (int)k;
        }
    }
    if (!(off.y >= 0.0f && off.y < wy)) {
        const float k = fminf(fmaxf(floorf(__fdiv_rn(off.y, wy)), -1.0e6f), 1.0e6f);
        if (k == k) {
            off.y = __fmaf_rn(-k, wy, off.y);
            cy += (int)k;
        }
    }
    if (cx < 0 || cx >= nx || cy < 0 || cy >= ny) {
        raise_error(d.err, SPHNJ_ERR_OUT_OF_GRID, kind, i, cx * ny + cy);
        const int qx = min(max(cx, 0), nx - 1), qy = min(max(cy, 0), ny - 1);
        off.x = __fmaf_rn((float)(cx - qx), wx, off.x);
        off.y = __fmaf_rn((float)(cy - qy), wy, off.y);
        cx = qx;
        cy = qy;
    }
    return cx * ny + cy;
}

template <class G> __global__ void k_bin(const __grid_constant__ G g, int with_virt) {
    SPHNJ_SCENE(g);
    const int nf = p.fluid_number_total, ns = p.solid_number, nv = with_virt ? p.virt_number : 0;
    const int C = p.cell_number_total;
    long t = (long)blk * blockDim.x + threadIdx.x;
    if (t == 0) {
        *d.max_speed2_bits = 0u;
        *d.stamp += 1;  // this step's stamp (read by kernels launched after this one)
        *d.tile_count = 0;
    }
    if (t < 1 + kMaskShifts) d.disp2_bits[t] = 0u;  // every scene has >= 256 threads
    int kind, i, c;
    if (d.f_off) {  // mixed form
        if (t < nf) {
            i = (int)t;
            const int c0 = d.f_cell[i];
            float2 off = d.f_off[i];
            c = rebase(p, d, 0, i, c0 / p.cell_number[1], c0 % p.cell_number[1], off);
            if (c != c0) {
                d.f_off[i] = off;
                d.f_cell[i] = c;
            }
        } else if (t < (long)nf + ns) {
            i = (int)(t - nf);
            const int2 rc = d.s_rc[i];
            const float2 roff = d.s_roff[i], u = d.s_u[i];
            float2 off = add2_rn(roff, u);
            c = rebase(p, d, 1, i, rc.x, rc.y, off);
            d.s_off[i] = solid_offset(p, rc, roff, u, c);
            d.s_cell[i] = c;
        }
        return;  // virtual particles keep the cells and offsets set at upload
    }
    if (t < nf) {
        kind = 0;
        i = (int)t;
        float2 x = d.f_pos[i];
        c = cell_of(p, x.x, x.y);
    } else if (t < (long)nf + ns) {
        kind = 1;
        i = (int)(t - nf);
        double2 x = d.s_pos[i];
        c = cell_of(p, (float)x.x, (float)x.y);
    } else if (t < (long)nf + ns + nv) {
        kind = 2;
        i = (int)(t - nf - ns);
        float2 x = d.v_pos[i];
        c = cell_of(p, x.x, x.y);
    } else {
        return;
    }
    if (c < 0 || c >= C) {
        // The reference indexes its cell array with this id unchecked.
        raise_error(d.err, SPHNJ_ERR_OUT_OF_GRID, kind, i, c);
        c = c < 0 ? 0 : C - 1;  // keep every later index in bounds
    }
    (kind == 0 ? d.f_cell : kind == 1 ? d.s_cell : d.v_cell)[i] = c;
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ int block_excl_scan(int v, int *total) {
    __shared__ int ws[kBlock / 32 + 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        int x = lane < kBlock / 32 ? ws[lane] : 0;
        int xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += y;
        }
        if (lane < kBlock / 32) ws[lane] = xi - x;
        if (lane == kBlock / 32 - 1) ws[kBlock / 32] = xi;  // uses spare slot below
    }
    __syncthreads();
    int r = inc - v + ws[w];
    if (total) *total = ws[kBlock / 32];
    return r;
}

// Valid neighbour slots of cell (ci, cj): those whose neighbour exists.
__device__ __forceinline__ bool slot_valid(int ci, int cj, int s, int nx, int ny) {
    int i = ci + s / 3 - 1, j = cj + s % 3 - 1;
    return i >= 0 && i < nx && j >= 0 && j < ny;
}

// Tile scan: tile = 1024 cells, 4 per thread.  Source is either per-cell
// counts (sort) or the per-(cell,slot) counts of a rebuild, whose per-cell
// totals also become the counts of list buffer `parity` of kind k.
template <class G, bool kFromCnt9>
__global__ void __launch_bounds__(kBlock) k_scan_tile(const __grid_constant__ G g, int k, int parity) {
    SPHNJ_SCENE(g);
    const int C = p.cell_number_total, nx = p.cell_number[0], ny = p.cell_number[1];
    const ListScratch &sc = S.sc;
    int2 *rng = list_of(S, k, parity).rng;
    const int c0 = blk * SCAN_TILE + threadIdx.x * 4;
    int v[4];
    int tsum = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int c = c0 + q;
        int x = 0;
        if (c < C) {
            if (kFromCnt9) {
                int ci = c / ny, cj = c - ci * ny;
#pragma unroll
                for (int s = 0; s < 9; ++s)
                    if (slot_valid(ci, cj, s, nx, ny)) x += sc.cnt9[(long)c * 9 + s];
                rng[c].y = x;
            } else {
                x = sc.cnt[c];
            }
        }
        v[q] = x;
        tsum += x;
    }
    int total;
    int ex = block_excl_scan(tsum, &total);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int c = c0 + q;
        if (c < C) sc.local[c] = ex;
        ex += v[q];
    }
    if (threadIdx.x == 0) sc.sums[blk] = total;
}

// In-place exclusive scan of the tile sums (<= SCAN_MAX_TILES) by one block:
// of the cell scans (sweep_tiles == 0: one sum per 1024 cells) or of the
// sweep-tile compaction (one sum per 1024 sweep tiles of the scene's tile
// height).
// The grand total goes to the scene's listed-particle count (total_to 1), its
// active-tile count (2) or nowhere (0).
template <class G>
__global__ void __launch_bounds__(1024) k_scan_sums(const __grid_constant__ G g, int total_to, int sweep_tiles_) {
    SPHNJ_SCENE(g);
    __shared__ int ws[33];
    const int units = sweep_tiles_ ? sweep_tiles(p, S.tile_h) : p.cell_number_total;
    const int ntiles = (units + SCAN_TILE - 1) / SCAN_TILE;
    int *sums = S.sc.sums;
    int *total = total_to == 1 ? S.f_listed_total : total_to == 2 ? d.tile_count : nullptr;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v[4], tsum = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int t = threadIdx.x * 4 + q;
        v[q] = t < ntiles ? sums[t] : 0;
        tsum += v[q];
    }
    int inc = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        int x = ws[lane], xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += y;
        }
        ws[lane] = xi - x;
    }
    __syncthreads();
    int ex = inc - tsum + ws[w];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int t = threadIdx.x * 4 + q;
        if (t < ntiles) sums[t] = ex;
        if (total && t == ntiles - 1) *total = ex + v[q];
        ex += v[q];
    }
}

__device__ __forceinline__ int cell_start(const int *local, const int *sums, int c) {
    return local[c] + sums[c / SCAN_TILE];
}

// ---- active sweep tiles ------------------------------------------------------
// Tile t of the neighbour sweeps (column segments of tile_h cells) holds fluid
// this step.  The active tiles are listed in tile order - an order-preserving
// compaction (flag scan per 1024 tiles, scan of the tile sums, scatter) - so
// that blocks sweeping consecutive list entries share staged strips in L2.
__device__ __forceinline__ bool tile_active(const sphnj_params &p, const DevState &d, int t, int tile_h) {
    const int ny = p.cell_number[1], tiles_y = (ny + tile_h - 1) / tile_h;
    const int ci = t / tiles_y, cj0 = (t - ci * tiles_y) * tile_h, cj1 = min(cj0 + tile_h, ny);
    const int2 h0 = __ldg(&d.rng_f[ci * ny + cj0]), h1 = __ldg(&d.rng_f[ci * ny + cj1 - 1]);
    return h1.x + h1.y > h0.x;
}

template <class G> __global__ void __launch_bounds__(kBlock) k_tile_flag_scan(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int tile_h = S.tile_h;
    const int nt = sweep_tiles(p, tile_h);
    const ListScratch &sc = S.sc;
    const int t0 = blk * SCAN_TILE + threadIdx.x * 4;
    int v[4], tsum = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int t = t0 + q;
        v[q] = t < nt && tile_active(p, d, t, tile_h) ? 1 : 0;
        tsum += v[q];
    }
    int total;
    int ex = block_excl_scan(tsum, &total);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (t0 + q < nt) sc.local[t0 + q] = ex;
        ex += v[q];
    }
    if (threadIdx.x == 0) sc.sums[blk] = total;
}

template <class G> __global__ void k_tile_scatter(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int tile_h = S.tile_h;
    const int t = blk * blockDim.x + threadIdx.x;
    if (t < sweep_tiles(p, tile_h) && tile_active(p, d, t, tile_h))
        d.tile_list[cell_start(S.sc.local, S.sc.sums, t)] = t;
}

// ---- sort ------------------------------------------------------------------
template <class G> __global__ void k_sort_clear(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int c = blk * blockDim.x + threadIdx.x;
    if (c >= p.cell_number_total) return;
    S.sc.cnt[c] = 0;
    S.sc.cursor[c] = 0;
}

template <class G> __global__ void k_hist(const __grid_constant__ G g, int k) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i < count_of(p, (Kind)k)) atomicAdd(&S.sc.cnt[cells_of(d, k)[i]], 1);
}

template <class G> __global__ void k_bucket(const __grid_constant__ G g, int k) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= count_of(p, (Kind)k)) return;
    const ListScratch &sc = S.sc;
    const int c = cells_of(d, k)[i];
    const int slot = atomicAdd(&sc.cursor[c], 1);
    sc.bucket[cell_start(sc.local, sc.sums, c) + slot] = i;
}

// One warp per cell: rank sort of the cell's bucket by particle index.
template <class G> __global__ void k_cellsort(const __grid_constant__ G g, int k, int parity) {
    SPHNJ_SCENE(g);
    const ListScratch &sc = S.sc;
    const int lane = threadIdx.x & 31;
    const long c = ((long)blk * blockDim.x + threadIdx.x) >> 5;
    if (c >= p.cell_number_total) return;
    const int n = sc.cnt[c];
    const int base = cell_start(sc.local, sc.sums, (int)c);
    if (lane == 0) list_of(S, k, parity).rng[c] = make_int2(base, n);
    for (int k0 = 0; k0 < n; k0 += 32) {
        int q = k0 + lane;
        int v = q < n ? sc.bucket[base + q] : INT_MAX;
        int rank = 0;
        for (int q0 = 0; q0 < n; q0 += 32) {
            int w = q0 + lane < n ? sc.bucket[base + q0 + lane] : INT_MAX;
#pragma unroll 8
            for (int t = 0; t < 32; ++t) rank += (__shfl_sync(0xffffffffu, w, t) < v) ? 1 : 0;
        }
        if (q < n) sc.sorted[base + rank] = v;
    }
}

// Payload gathers (sort.cu:10-45): new[k] = old[sorted[k]], lists = identity.
__device__ __forceinline__ size_t align256_d(size_t x) { return (x + 255) & ~size_t(255); }
template <class T> __device__ __forceinline__ T *carve(char *&q, size_t n) {
    T *r = reinterpret_cast<T *>(q);
    q += align256_d(n * sizeof(T));
    return r;
}

// Mixed form (`mixed`): the position is the cell + offset pair with its
// compensation, and the velocity compensation travels too.
struct FluidPayload {
    float2 *pos, *vel;
    float *rho, *p;
    uint8_t *phase, *fbt;
    int *cell;
    float2 *off, *offc, *velc;
    __device__ FluidPayload(char *q, int n, bool mixed) {
        pos = carve<float2>(q, n); vel = carve<float2>(q, n);
        rho = carve<float>(q, n); p = carve<float>(q, n);
        phase = carve<uint8_t>(q, n); fbt = carve<uint8_t>(q, n);
        cell = carve<int>(q, n);
        off = offc = velc = nullptr;
        if (mixed) {
            off = carve<float2>(q, n); offc = carve<float2>(q, n); velc = carve<float2>(q, n);
        }
    }
};
template <class G> __global__ void k_gather_fluid(const __grid_constant__ G g, int parity) {
    SPHNJ_SCENE(g);
    const int n = p.fluid_number_total;
    const int k = blk * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const FluidPayload o(S.payload, n, d.f_off != nullptr);
    if (d.f_listed) d.f_listed[k] = *d.stamp;
    const int s = S.sc.sorted[k];
    if (o.off) {
        o.off[k] = d.f_off[s];
        o.offc[k] = d.f_offc[s];
        o.velc[k] = d.f_velc[s];
    } else {
        o.pos[k] = d.f_pos[s];
    }
    o.vel[k] = d.f_vel[s];
    o.rho[k] = d.f_rho[s];
    o.p[k] = d.f_p[s];
    o.phase[k] = d.f_phase[s];
    o.fbt[k] = d.f_fbt[s];
    o.cell[k] = d.f_cell[s];
    S.lf[parity].lst[k] = k;
}
template <class G> __global__ void k_scatter_back_fluid(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int n = p.fluid_number_total;
    const int k = blk * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const FluidPayload o(S.payload, n, d.f_off != nullptr);
    if (o.off) {
        d.f_off[k] = o.off[k];
        d.f_offc[k] = o.offc[k];
        d.f_velc[k] = o.velc[k];
    } else {
        d.f_pos[k] = o.pos[k];
    }
    d.f_vel[k] = o.vel[k];
    d.f_rho[k] = o.rho[k];
    d.f_p[k] = o.p[k];
    d.f_phase[k] = o.phase[k];
    d.f_fbt[k] = o.fbt[k];
    d.f_cell[k] = o.cell[k];
}

// Mixed form (`mixed`): the reference cell + offset, displacement and
// velocity (with their compensations) replace the FP64 position and velocity.
struct SolidPayload {
    double2 *ref, *pos, *vel;
    dmat2 *maxstrain;
    uint8_t *mat, *bt;
    int *cell;
    int2 *rc;
    float2 *roff, *u, *uc, *v, *vc, *off;
    __device__ SolidPayload(char *q, int n, bool mixed) {
        ref = carve<double2>(q, n); pos = carve<double2>(q, n); vel = carve<double2>(q, n);
        maxstrain = carve<dmat2>(q, n);
        mat = carve<uint8_t>(q, n); bt = carve<uint8_t>(q, n);
        cell = carve<int>(q, n);
        rc = nullptr;
        roff = u = uc = v = vc = off = nullptr;
        if (mixed) {
            rc = carve<int2>(q, n);
            roff = carve<float2>(q, n); u = carve<float2>(q, n); uc = carve<float2>(q, n);
            v = carve<float2>(q, n); vc = carve<float2>(q, n);
            off = carve<float2>(q, n);  // set by this step's binning, before the sort
        }
    }
};
template <class G> __global__ void k_gather_solid(const __grid_constant__ G g, int parity) {
    SPHNJ_SCENE(g);
    const int n = p.solid_number;
    const int k = blk * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const SolidPayload o(S.payload, n, d.s_rc != nullptr);
    const int s = S.sc.sorted[k];
    o.ref[k] = d.s_ref[s];
    if (o.rc) {
        o.rc[k] = d.s_rc[s];
        o.roff[k] = d.s_roff[s];
        o.u[k] = d.s_u[s];
        o.uc[k] = d.s_uc[s];
        o.v[k] = d.s_v[s];
        o.vc[k] = d.s_vc[s];
        o.off[k] = d.s_off[s];
    } else {
        o.pos[k] = d.s_pos[s];
        o.vel[k] = d.s_vel[s];
    }
    o.maxstrain[k] = d.s_maxstrain[s];
    o.mat[k] = d.s_mat[s];
    o.bt[k] = d.s_bt[s];
    o.cell[k] = d.s_cell[s];
    S.ls[parity].lst[k] = k;
}
template <class G> __global__ void k_scatter_back_solid(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int n = p.solid_number;
    const int k = blk * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const SolidPayload o(S.payload, n, d.s_rc != nullptr);
    d.s_ref[k] = o.ref[k];
    if (o.rc) {
        d.s_rc[k] = o.rc[k];
        d.s_roff[k] = o.roff[k];
        d.s_u[k] = o.u[k];
        d.s_uc[k] = o.uc[k];
        d.s_v[k] = o.v[k];
        d.s_vc[k] = o.vc[k];
        d.s_off[k] = o.off[k];
    } else {
        d.s_pos[k] = o.pos[k];
        d.s_vel[k] = o.vel[k];
    }
    d.s_maxstrain[k] = o.maxstrain[k];
    d.s_mat[k] = o.mat[k];
    d.s_bt[k] = o.bt[k];
    d.s_cell[k] = o.cell[k];
}

struct VirtPayload {
    float2 *pos, *normal;
    uint8_t *bt;
    int *cell;
    float2 *off;  // mixed form
    __device__ VirtPayload(char *q, int n, bool mixed) {
        pos = carve<float2>(q, n); normal = carve<float2>(q, n);
        bt = carve<uint8_t>(q, n);
        cell = carve<int>(q, n);
        off = mixed ? carve<float2>(q, n) : nullptr;
    }
};
template <class G> __global__ void k_gather_virt(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int n = p.virt_number;
    const int k = blk * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const VirtPayload o(S.payload, n, d.v_off != nullptr);
    const int s = S.sc.sorted[k];
    if (o.off) o.off[k] = d.v_off[s];
    o.pos[k] = d.v_pos[s];
    o.normal[k] = d.v_normal[s];
    o.bt[k] = d.v_bt[s];
    o.cell[k] = d.v_cell[s];
    S.lv.lst[k] = k;
}
template <class G> __global__ void k_scatter_back_virt(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int n = p.virt_number;
    const int k = blk * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const VirtPayload o(S.payload, n, d.v_off != nullptr);
    if (o.off) d.v_off[k] = o.off[k];
    d.v_pos[k] = o.pos[k];
    d.v_normal[k] = o.normal[k];
    d.v_bt[k] = o.bt[k];
    d.v_cell[k] = o.cell[k];
}

// ---- incremental rebuild ---------------------------------------------------
// Slot of old cell m as seen from new cell c, or -1 when c is not within
// one cell of m.
__device__ __forceinline__ int slot_from(int mi, int mj, int c, int ny) {
    int ci = c / ny, cj = c - ci * ny;
    int di = mi - ci, dj = mj - cj;
    if (di < -1 || di > 1 || dj < -1 || dj > 1) return -1;
    return 3 * (di + 1) + (dj + 1);
}

// The per-(cell, slot) counts start at zero, so that k_rebuild_count writes
// only the non-zero ones: most cells of a sparse scene are empty, and a
// particle that stays in its cell leaves its cell's eight other slots at
// zero.  A count kernel that wrote all nine (each to another cell's row)
// spent most of its time on those scattered stores of zeros.
template <class G> __global__ void __launch_bounds__(kBlock) k_zero_cnt9(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const long n = 9L * p.cell_number_total;
    int *cnt9 = S.sc.cnt9;
    for (long t = (long)blk * blockDim.x + threadIdx.x; t < n; t += (long)nblk * blockDim.x) cnt9[t] = 0;
}

template <class G> __global__ void k_rebuild_count(const __grid_constant__ G g, int k, int parity) {
    SPHNJ_SCENE(g);
    const int C = p.cell_number_total, nx = p.cell_number[0], ny = p.cell_number[1];
    const int m = blk * blockDim.x + threadIdx.x;
    if (m >= C) return;
    const CellList &prev = list_of(S, k, parity ^ 1);
    const int *cell = cells_of(d, k);
    int *cnt9 = S.sc.cnt9;
    const int mi = m / ny, mj = m - mi * ny;
    const int2 r = prev.rng[m];
    int run[9];
#pragma unroll
    for (int s = 0; s < 9; ++s) run[s] = 0;
    for (int q = r.x; q < r.x + r.y; ++q) {
        int s = slot_from(mi, mj, __ldg(&cell[__ldg(&prev.lst[q])]), ny);
#pragma unroll
        for (int t = 0; t < 9; ++t) run[t] += (s == t);
    }
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        int ci = mi - (s / 3 - 1), cj = mj - (s % 3 - 1);
        if (run[s] && ci >= 0 && ci < nx && cj >= 0 && cj < ny) cnt9[(long)(ci * ny + cj) * 9 + s] = run[s];
    }
}

template <class G> __global__ void k_rebuild_write(const __grid_constant__ G g, int k, int parity) {
    SPHNJ_SCENE(g);
    const int C = p.cell_number_total, nx = p.cell_number[0], ny = p.cell_number[1];
    const int m = blk * blockDim.x + threadIdx.x;
    if (m >= C) return;
    const CellList &prev = list_of(S, k, parity ^ 1), &cur = list_of(S, k, parity);
    const int *cell = cells_of(d, k);
    const ListScratch &sc = S.sc;
    int *listed = k == KF ? d.f_listed : nullptr;
    const int mi = m / ny, mj = m - mi * ny;
    cur.rng[m].x = cell_start(sc.local, sc.sums, m);
    const int2 r = prev.rng[m];
    if (r.y == 0) return;  // no particle of cell m to place
    int base[9];
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        int ci = mi - (s / 3 - 1), cj = mj - (s % 3 - 1);
        int b = 0;
        if (ci >= 0 && ci < nx && cj >= 0 && cj < ny) {
            int c = ci * ny + cj;
            b = cell_start(sc.local, sc.sums, c);
            for (int q = 0; q < s; ++q)
                if (slot_valid(ci, cj, q, nx, ny)) b += sc.cnt9[(long)c * 9 + q];
        }
        base[s] = b;
    }
    const int stamp = listed ? *d.stamp : 0;
    for (int q = r.x; q < r.x + r.y; ++q) {
        int pidx = __ldg(&prev.lst[q]);
        int s = slot_from(mi, mj, __ldg(&cell[pidx]), ny);
        if (s < 0) continue;
        int dst = 0;
#pragma unroll
        for (int t = 0; t < 9; ++t)
            if (t == s) dst = base[t]++;
        cur.lst[dst] = pidx;
        if (listed) listed[pidx] = stamp;
    }
}

template <class G> __global__ void k_capacity(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int c = blk * blockDim.x + threadIdx.x;
    if (c >= p.cell_number_total) return;
    const int t = d.rng_f[c].y + d.rng_s[c].y + d.rng_v[c].y;
    if (t > SPHNJ_CELL_SIZE) raise_error(d.err, SPHNJ_ERR_CELL_OVERFLOW, c, t, 0);
}

}  // namespace

template <class G> int launch_bin(cudaStream_t st, G &g, bool with_virt) {
    return launch(
        g, site_key(SITE_BIN, with_virt ? 1 : 0),
        [&](const Scene &s) {
            long n = (long)s.p.fluid_number_total + s.p.solid_number + (with_virt ? s.p.virt_number : 0);
            return grid_for(n > 0 ? n : 1, kBlock);
        },
        k_bin<typename G::Dev>, kBlock, 0, st, with_virt ? 1 : 0);
}

// Cell ids of the virtual particles from their positions (the virtual part
// of k_bin, with its out-of-grid check), for the cell lists of the wall
// normals at upload.
template <class G> __global__ void __launch_bounds__(kBlock) k_virt_bin(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.virt_number) return;
    const float2 x = d.v_pos[i];
    int c = cell_of(p, x.x, x.y);
    if (c < 0 || c >= p.cell_number_total) {
        raise_error(d.err, SPHNJ_ERR_OUT_OF_GRID, 2, i, c);
        c = c < 0 ? 0 : p.cell_number_total - 1;
    }
    d.v_cell[i] = c;
}

// Per-cell lists of kind k, the particle arrays not reordered: cell c's
// particle indices in ascending order at sc.sorted[r.x .. r.x + r.y), r the
// cell's range in list buffer `parity` (the sort's first stages; the list
// entries themselves are written by the gathers that follow in a sort).
template <class G> int launch_index_kind(cudaStream_t st, G &g, Kind k, int parity) {
    using D = typename G::Dev;
    auto has = [k](const Scene &s) { return count_of(s.p, k) > 0; };
    auto cells = [&](const Scene &s) { return has(s) ? grid_for(s.p.cell_number_total, kBlock) : 0u; };
    auto parts = [&](const Scene &s) { return has(s) ? grid_for(count_of(s.p, k), kBlock) : 0u; };
    auto tiles = [&](const Scene &s) { return has(s) ? grid_for(s.p.cell_number_total, SCAN_TILE) : 0u; };
    auto one = [&](const Scene &s) { return has(s) ? 1u : 0u; };
    auto warps = [&](const Scene &s) { return has(s) ? grid_for((long)s.p.cell_number_total * 32, kBlock) : 0u; };
    const int ki = (int)k;
    int n = 0;
    n += launch(g, site_key(SITE_SORT_CLEAR, ki), cells, k_sort_clear<D>, kBlock, 0, st);
    n += launch(g, site_key(SITE_SORT_N, ki), parts, k_hist<D>, kBlock, 0, st, ki);
    n += launch(g, site_key(SITE_SORT_TILES, ki), tiles, k_scan_tile<D, false>, kBlock, 0, st, ki, parity);
    n += launch(g, site_key(SITE_SORT_ONE, ki), one, k_scan_sums<D>, 1024, 0, st, k == KF ? 1 : 0, 0);
    n += launch(g, site_key(SITE_SORT_N, ki), parts, k_bucket<D>, kBlock, 0, st, ki);
    n += launch(g, site_key(SITE_SORT_CELLS32, ki), warps, k_cellsort<D>, kBlock, 0, st, ki, parity);
    return n;
}

template <class G> int launch_virt_index(cudaStream_t st, G &g) {
    int n = launch(
        g, site_key(SITE_VIRT_BIN), [](const Scene &s) { return grid_for(s.p.virt_number, kBlock); },
        k_virt_bin<typename G::Dev>, kBlock, 0, st);
    return n + launch_index_kind(st, g, KV, 0);
}

template <class G> int launch_sort_kind(cudaStream_t st, G &g, Kind k, int parity) {
    using D = typename G::Dev;
    auto has = [k](const Scene &s) { return count_of(s.p, k) > 0; };
    auto parts = [&](const Scene &s) { return has(s) ? grid_for(count_of(s.p, k), kBlock) : 0u; };
    const int ki = (int)k;
    int n = launch_index_kind(st, g, k, parity);
    if (k == KF) {
        n += launch(g, site_key(SITE_SORT_N, ki), parts, k_gather_fluid<D>, kBlock, 0, st, parity);
        n += launch(g, site_key(SITE_SORT_N, ki), parts, k_scatter_back_fluid<D>, kBlock, 0, st);
    } else if (k == KS) {
        n += launch(g, site_key(SITE_SORT_N, ki), parts, k_gather_solid<D>, kBlock, 0, st, parity);
        n += launch(g, site_key(SITE_SORT_N, ki), parts, k_scatter_back_solid<D>, kBlock, 0, st);
    } else {
        n += launch(g, site_key(SITE_SORT_N, ki), parts, k_gather_virt<D>, kBlock, 0, st);
        n += launch(g, site_key(SITE_SORT_N, ki), parts, k_scatter_back_virt<D>, kBlock, 0, st);
    }
    return n;
}

template <class G> int launch_rebuild_kind(cudaStream_t st, G &g, Kind k, int parity) {
    using D = typename G::Dev;
    auto has = [k](const Scene &s) { return count_of(s.p, k) > 0; };
    auto cells = [&](const Scene &s) { return has(s) ? grid_for(s.p.cell_number_total, kBlock) : 0u; };
    auto tiles = [&](const Scene &s) { return has(s) ? grid_for(s.p.cell_number_total, SCAN_TILE) : 0u; };
    auto one = [&](const Scene &s) { return has(s) ? 1u : 0u; };
    // zeroing: eight counts a thread (the scene's 9 per cell)
    auto zero = [&](const Scene &s) { return has(s) ? grid_for(9L * s.p.cell_number_total, 8 * kBlock) : 0u; };
    const int ki = (int)k;
    int n = 0;
    n += launch(g, site_key(SITE_REBUILD_ZERO, ki), zero, k_zero_cnt9<D>, kBlock, 0, st);
    n += launch(g, site_key(SITE_REBUILD_CELLS, ki), cells, k_rebuild_count<D>, kBlock, 0, st, ki, parity);
    n += launch(g, site_key(SITE_REBUILD_TILES, ki), tiles, k_scan_tile<D, true>, kBlock, 0, st, ki, parity);
    n += launch(g, site_key(SITE_REBUILD_ONE, ki), one, k_scan_sums<D>, 1024, 0, st, k == KF ? 1 : 0, 0);
    n += launch(g, site_key(SITE_REBUILD_CELLS, ki), cells, k_rebuild_write<D>, kBlock, 0, st, ki, parity);
    return n;
}

template <class G> int launch_tile_compact(cudaStream_t st, G &g, bool all_scenes) {
    using D = typename G::Dev;
    auto has = [all_scenes](const Scene &s) {
        return all_scenes ? s.p.fluid_number_total > 0 : sweep_compacted(s.p, s.tile_h);
    };
    int n = launch(
        g, site_key(SITE_TILE_COMPACT),
        [&](const Scene &s) { return has(s) ? grid_for(sweep_tiles(s.p, s.tile_h), SCAN_TILE) : 0u; },
        k_tile_flag_scan<D>, kBlock, 0, st);
    n += launch(
        g, site_key(SITE_TILE_SUMS), [&](const Scene &s) { return has(s) ? 1u : 0u; }, k_scan_sums<D>, 1024, 0, st, 2,
        1);
    n += launch(
        g, site_key(SITE_TILE_SCATTER),
        [&](const Scene &s) { return has(s) ? grid_for(sweep_tiles(s.p, s.tile_h), kBlock) : 0u; }, k_tile_scatter<D>,
        kBlock, 0, st);
    return n;
}

template <class G> int launch_capacity_check(cudaStream_t st, G &g) {
    return launch(
        g, site_key(SITE_CAPACITY), [](const Scene &s) { return grid_for(s.p.cell_number_total, kBlock); },
        k_capacity<typename G::Dev>, kBlock, 0, st);
}

SPHNJ_INSTANTIATE_GROUPS(launch_bin, bool);
SPHNJ_INSTANTIATE_GROUPS(launch_sort_kind, Kind, int);
SPHNJ_INSTANTIATE_GROUPS(launch_virt_index);
SPHNJ_INSTANTIATE_GROUPS(launch_rebuild_kind, Kind, int);
SPHNJ_INSTANTIATE_GROUPS(launch_capacity_check);
SPHNJ_INSTANTIATE_GROUPS(launch_tile_compact, bool);

}  // namespace sphnj
