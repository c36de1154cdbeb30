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
//   - rebuild = each old cell m scatters its 9 outgoing counts to
//     cnt9[c][slot] (every (c,slot) pair has exactly one writer, so no
//     atomics and no zeroing), a tiled scan gives the new cell starts, and
//     m writes its particles to their destinations in previous-list order.
#include "kernels.h"

#include <climits>

namespace sphnj {

namespace {

constexpr int kBlock = 256;

__global__ void k_bin(sphnj_params p, DevState d, int with_virt) {
    const int nf = p.fluid_number_total, ns = p.solid_number, nv = with_virt ? p.virt_number : 0;
    const int C = p.cell_number_total;
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        *d.max_speed2_bits = 0u;
        *d.stamp += 1;  // this step's stamp (read by kernels launched after this one)
    }
    if (t < 1 + kMaskShifts) d.disp2_bits[t] = 0u;  // grid has >= 256 threads
    int kind, i, c;
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
// counts (cnt) or the per-(cell,slot) counts of a rebuild (cnt9).
template <bool kFromCnt9>
__global__ void __launch_bounds__(kBlock) k_scan_tile(int C, int nx, int ny, const int *cnt, const int *cnt9,
                                                      int2 *rng, int *local, int *sums) {
    const int c0 = blockIdx.x * SCAN_TILE + threadIdx.x * 4;
    int v[4];
    int tsum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int c = c0 + k;
        int x = 0;
        if (c < C) {
            if (kFromCnt9) {
                int ci = c / ny, cj = c - ci * ny;
#pragma unroll
                for (int s = 0; s < 9; ++s)
                    if (slot_valid(ci, cj, s, nx, ny)) x += cnt9[(long)c * 9 + s];
                rng[c].y = x;
            } else {
                x = cnt[c];
            }
        }
        v[k] = x;
        tsum += x;
    }
    int total;
    int ex = block_excl_scan(tsum, &total);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int c = c0 + k;
        if (c < C) local[c] = ex;
        ex += v[k];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// In-place exclusive scan of the tile sums (<= SCAN_MAX_TILES) by one block;
// the grand total goes to *total when given.
__global__ void __launch_bounds__(1024) k_scan_sums(int ntiles, int *sums, int *total = nullptr) {
    __shared__ int ws[33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v[4], tsum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int t = threadIdx.x * 4 + k;
        v[k] = t < ntiles ? sums[t] : 0;
        tsum += v[k];
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
    for (int k = 0; k < 4; ++k) {
        int t = threadIdx.x * 4 + k;
        if (t < ntiles) sums[t] = ex;
        if (total && t == ntiles - 1) *total = ex + v[k];
        ex += v[k];
    }
}

__device__ __forceinline__ int cell_start(const int *local, const int *sums, int c) {
    return local[c] + sums[c / SCAN_TILE];
}

// ---- sort ------------------------------------------------------------------
__global__ void k_hist(int n, const int *cell, int *cnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&cnt[cell[i]], 1);
}

__global__ void k_bucket(int n, const int *cell, const int *local, const int *sums, int *cursor, int *bucket) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell[i];
    int slot = atomicAdd(&cursor[c], 1);
    bucket[cell_start(local, sums, c) + slot] = i;
}

// One warp per cell: rank sort of the cell's bucket by particle index.
__global__ void k_cellsort(int C, const int *cnt, const int *local, const int *sums, const int *bucket,
                           int *sorted, int2 *rng) {
    const int lane = threadIdx.x & 31;
    const long c = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= C) return;
    const int n = cnt[c];
    const int base = cell_start(local, sums, (int)c);
    if (lane == 0) rng[c] = make_int2(base, n);
    for (int k0 = 0; k0 < n; k0 += 32) {
        int k = k0 + lane;
        int v = k < n ? bucket[base + k] : INT_MAX;
        int rank = 0;
        for (int q0 = 0; q0 < n; q0 += 32) {
            int w = q0 + lane < n ? bucket[base + q0 + lane] : INT_MAX;
#pragma unroll 8
            for (int t = 0; t < 32; ++t) rank += (__shfl_sync(0xffffffffu, w, t) < v) ? 1 : 0;
        }
        if (k < n) sorted[base + rank] = v;
    }
}

// Payload gathers (sort.cu:10-45): new[k] = old[sorted[k]], lists = identity.
struct FluidPayload {
    float2 *pos, *vel;
    float *rho, *p;
    uint8_t *phase, *fbt;
    int *cell;
};
__global__ void k_gather_fluid(int n, const int *sorted, DevState d, FluidPayload o, int *lst, int *listed,
                               const int *stamp) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (listed) listed[k] = *stamp;
    int s = sorted[k];
    o.pos[k] = d.f_pos[s];
    o.vel[k] = d.f_vel[s];
    o.rho[k] = d.f_rho[s];
    o.p[k] = d.f_p[s];
    o.phase[k] = d.f_phase[s];
    o.fbt[k] = d.f_fbt[s];
    o.cell[k] = d.f_cell[s];
    lst[k] = k;
}
__global__ void k_scatter_back_fluid(int n, DevState d, FluidPayload o) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    d.f_pos[k] = o.pos[k];
    d.f_vel[k] = o.vel[k];
    d.f_rho[k] = o.rho[k];
    d.f_p[k] = o.p[k];
    d.f_phase[k] = o.phase[k];
    d.f_fbt[k] = o.fbt[k];
    d.f_cell[k] = o.cell[k];
}

struct SolidPayload {
    double2 *ref, *pos, *vel;
    dmat2 *maxstrain;
    uint8_t *mat, *bt;
    int *cell;
};
__global__ void k_gather_solid(int n, const int *sorted, DevState d, SolidPayload o, int *lst) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int s = sorted[k];
    o.ref[k] = d.s_ref[s];
    o.pos[k] = d.s_pos[s];
    o.vel[k] = d.s_vel[s];
    o.maxstrain[k] = d.s_maxstrain[s];
    o.mat[k] = d.s_mat[s];
    o.bt[k] = d.s_bt[s];
    o.cell[k] = d.s_cell[s];
    lst[k] = k;
}
__global__ void k_scatter_back_solid(int n, DevState d, SolidPayload o) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    d.s_ref[k] = o.ref[k];
    d.s_pos[k] = o.pos[k];
    d.s_vel[k] = o.vel[k];
    d.s_maxstrain[k] = o.maxstrain[k];
    d.s_mat[k] = o.mat[k];
    d.s_bt[k] = o.bt[k];
    d.s_cell[k] = o.cell[k];
}

struct VirtPayload {
    float2 *pos, *normal;
    uint8_t *bt;
    int *cell;
};
__global__ void k_gather_virt(int n, const int *sorted, DevState d, VirtPayload o, int *lst) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int s = sorted[k];
    o.pos[k] = d.v_pos[s];
    o.normal[k] = d.v_normal[s];
    o.bt[k] = d.v_bt[s];
    o.cell[k] = d.v_cell[s];
    lst[k] = k;
}
__global__ void k_scatter_back_virt(int n, DevState d, VirtPayload o) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
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

__global__ void k_rebuild_count(int C, int nx, int ny, const int2 *prng, const int *plst, const int *cell,
                                int *cnt9) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= C) return;
    const int mi = m / ny, mj = m - mi * ny;
    const int2 r = prng[m];
    int run[9];
#pragma unroll
    for (int s = 0; s < 9; ++s) run[s] = 0;
    for (int k = r.x; k < r.x + r.y; ++k) {
        int s = slot_from(mi, mj, __ldg(&cell[__ldg(&plst[k])]), ny);
#pragma unroll
        for (int q = 0; q < 9; ++q) run[q] += (s == q);
    }
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        int ci = mi - (s / 3 - 1), cj = mj - (s % 3 - 1);
        if (ci >= 0 && ci < nx && cj >= 0 && cj < ny) cnt9[(long)(ci * ny + cj) * 9 + s] = run[s];
    }
}

__global__ void k_rebuild_write(int C, int nx, int ny, const int2 *prng, const int *plst, const int *cell,
                                const int *cnt9, const int *local, const int *sums, int2 *crng, int *clst,
                                int *listed, const int *stamp) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= C) return;
    const int mi = m / ny, mj = m - mi * ny;
    crng[m].x = cell_start(local, sums, m);
    int base[9];
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        int ci = mi - (s / 3 - 1), cj = mj - (s % 3 - 1);
        int b = 0;
        if (ci >= 0 && ci < nx && cj >= 0 && cj < ny) {
            int c = ci * ny + cj;
            b = cell_start(local, sums, c);
            for (int q = 0; q < s; ++q)
                if (slot_valid(ci, cj, q, nx, ny)) b += cnt9[(long)c * 9 + q];
        }
        base[s] = b;
    }
    const int2 r = prng[m];
    for (int k = r.x; k < r.x + r.y; ++k) {
        int pidx = __ldg(&plst[k]);
        int s = slot_from(mi, mj, __ldg(&cell[pidx]), ny);
        if (s < 0) continue;
        int dst = 0;
#pragma unroll
        for (int q = 0; q < 9; ++q)
            if (q == s) dst = base[q]++;
        clst[dst] = pidx;
        if (listed) listed[pidx] = *stamp;
    }
}

__global__ void k_capacity(int C, const int2 *rf, const int2 *rs, const int2 *rv, DevErr *err) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    int t = rf[c].y + rs[c].y + rv[c].y;
    if (t > SPHNJ_CELL_SIZE) raise_error(err, SPHNJ_ERR_CELL_OVERFLOW, c, t, 0);
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
template <class T> T *carve(char *&p, size_t n) {
    T *r = reinterpret_cast<T *>(p);
    p += align256(n * sizeof(T));
    return r;
}

}  // namespace

void launch_bin(cudaStream_t st, const sphnj_params &p, const DevState &d, bool with_virt) {
    long n = (long)p.fluid_number_total + p.solid_number + (with_virt ? p.virt_number : 0);
    k_bin<<<grid_for(n > 0 ? n : 1, kBlock), kBlock, 0, st>>>(p, d, with_virt ? 1 : 0);
}

static void scan_counts(cudaStream_t st, int C, const int *cnt, int *local, int *sums, int *total) {
    int tiles = (C + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tile<false><<<tiles, kBlock, 0, st>>>(C, 0, 1, cnt, nullptr, nullptr, local, sums);
    k_scan_sums<<<1, 1024, 0, st>>>(tiles, sums, total);
}

void launch_sort_kind(cudaStream_t st, const sphnj_params &p, const DevState &d, Kind k, int n, int *cell,
                      ListScratch sc, CellList cur, void *payload_scratch, Listing lg) {
    const int C = p.cell_number_total;
    cudaMemsetAsync(sc.cnt, 0, sizeof(int) * C, st);
    cudaMemsetAsync(sc.cursor, 0, sizeof(int) * C, st);
    if (n > 0) k_hist<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, cell, sc.cnt);
    scan_counts(st, C, sc.cnt, sc.local, sc.sums, lg.total);
    if (n > 0) k_bucket<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, cell, sc.local, sc.sums, sc.cursor, sc.bucket);
    k_cellsort<<<grid_for((long)C * 32, kBlock), kBlock, 0, st>>>(C, sc.cnt, sc.local, sc.sums, sc.bucket,
                                                                    sc.sorted, cur.rng);
    if (n <= 0) return;
    char *q = static_cast<char *>(payload_scratch);
    if (k == KF) {
        FluidPayload o;
        o.pos = carve<float2>(q, n); o.vel = carve<float2>(q, n);
        o.rho = carve<float>(q, n); o.p = carve<float>(q, n);
        o.phase = carve<uint8_t>(q, n); o.fbt = carve<uint8_t>(q, n);
        o.cell = carve<int>(q, n);
        k_gather_fluid<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, sc.sorted, d, o, cur.lst, lg.listed, lg.stamp);
        k_scatter_back_fluid<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, d, o);
    } else if (k == KS) {
        SolidPayload o;
        o.ref = carve<double2>(q, n); o.pos = carve<double2>(q, n); o.vel = carve<double2>(q, n);
        o.maxstrain = carve<dmat2>(q, n);
        o.mat = carve<uint8_t>(q, n); o.bt = carve<uint8_t>(q, n);
        o.cell = carve<int>(q, n);
        k_gather_solid<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, sc.sorted, d, o, cur.lst);
        k_scatter_back_solid<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, d, o);
    } else {
        VirtPayload o;
        o.pos = carve<float2>(q, n); o.normal = carve<float2>(q, n);
        o.bt = carve<uint8_t>(q, n);
        o.cell = carve<int>(q, n);
        k_gather_virt<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, sc.sorted, d, o, cur.lst);
        k_scatter_back_virt<<<grid_for(n, kBlock), kBlock, 0, st>>>(n, d, o);
    }
}

void launch_rebuild_kind(cudaStream_t st, const sphnj_params &p, int n, const int *cell, CellList prev,
                         CellList cur, ListScratch sc, DevErr *err, Listing lg) {
    (void)n;
    (void)err;
    const int C = p.cell_number_total, nx = p.cell_number[0], ny = p.cell_number[1];
    const int tiles = (C + SCAN_TILE - 1) / SCAN_TILE;
    k_rebuild_count<<<grid_for(C, kBlock), kBlock, 0, st>>>(C, nx, ny, prev.rng, prev.lst, cell, sc.cnt9);
    k_scan_tile<true><<<tiles, kBlock, 0, st>>>(C, nx, ny, nullptr, sc.cnt9, cur.rng, sc.local, sc.sums);
    k_scan_sums<<<1, 1024, 0, st>>>(tiles, sc.sums, lg.total);
    k_rebuild_write<<<grid_for(C, kBlock), kBlock, 0, st>>>(C, nx, ny, prev.rng, prev.lst, cell, sc.cnt9, sc.local,
                                                            sc.sums, cur.rng, cur.lst, lg.listed, lg.stamp);
}

void launch_capacity_check(cudaStream_t st, const sphnj_params &p, const DevState &d) {
    const int C = p.cell_number_total;
    k_capacity<<<grid_for(C, kBlock), kBlock, 0, st>>>(C, d.rng_f, d.rng_s, d.rng_v, d.err);
}

}  // namespace sphnj
