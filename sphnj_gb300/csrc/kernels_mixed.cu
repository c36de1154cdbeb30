// Conversions between the host layout (absolute positions, the plain form's
// arrays) and the mixed-precision form's state, for upload and download.
//
//   split  absolute position x  ->  cell (floor((x - cell_min) / width), in
//          FP64) + FP32 offset from that cell's corner (x - corner in FP64,
//          rounded once); solid displacement u = x - X and velocity rounded
//          to FP32 with the rounding error kept as the Kahan compensation
//          (value = main part - compensation).
//   join   the inverse, in FP64: x = corner + offset - compensation.
#include "forms.cuh"
#include "kernels.h"

namespace sphnj {

namespace {

constexpr int kBlock = 256;

// The cell grid in FP64; iwx, iwy are 1 / width, computed on the host.
struct Grid2 {
    double x0, y0, wx, wy, iwx, iwy;
    int nx, ny;
};
__device__ __forceinline__ Grid2 grid_of(const sphnj_params &p, double iwx = 0.0, double iwy = 0.0) {
    return {(double)p.cell_xmin[0], (double)p.cell_xmin[1], (double)p.interval[0], (double)p.interval[1], iwx, iwy,
            p.cell_number[0], p.cell_number[1]};
}

// floor((x - x0) / w) without an FP64 division (slow on this GPU): the
// product with the reciprocal, corrected by one step so that the corner
// satisfies x0 + c w <= x < x0 + (c + 1) w as evaluated in FP64.
__device__ __forceinline__ double cell_floor(double x, double x0, double w, double iw) {
    double c = floor((x - x0) * iw);
    if (x0 + c * w > x) c -= 1.0;
    else if (x0 + (c + 1.0) * w <= x) c += 1.0;
    return c;
}

// Cell (x, y) holding absolute position (x, y) and the FP32 offset from its
// corner; positions outside the grid are reported and clamped into it.
__device__ __forceinline__ int2 split_pos(const Grid2 &g, double x, double y, float2 &off, DevErr *err, int kind,
                                          int i) {
    double fx = cell_floor(x, g.x0, g.wx, g.iwx), fy = cell_floor(y, g.y0, g.wy, g.iwy);
    if (!(fx >= 0.0 && fx < g.nx && fy >= 0.0 && fy < g.ny)) {
        raise_error(err, SPHNJ_ERR_OUT_OF_GRID, kind, i, -1);
        fx = fx == fx ? fmin(fmax(fx, 0.0), (double)(g.nx - 1)) : 0.0;
        fy = fy == fy ? fmin(fmax(fy, 0.0), (double)(g.ny - 1)) : 0.0;
    }
    off = make_float2((float)(x - (g.x0 + fx * g.wx)), (float)(y - (g.y0 + fy * g.wy)));
    return make_int2((int)fx, (int)fy);
}

__device__ __forceinline__ float2 round_f2(double2 v, float2 &comp) {
    const float2 r = make_float2((float)v.x, (float)v.y);
    comp = make_float2((float)((double)r.x - v.x), (float)((double)r.y - v.y));
    return r;
}

// kinds: bit 0 fluid, bit 1 solid, bit 2 virtual
__global__ void k_split(const __grid_constant__ One g, int kinds, double iwx, double iwy) {
    const Scene &S = g.s;
    const sphnj_params &p = S.p;
    const DevState &d = S.d;
    const Grid2 gr = grid_of(p, iwx, iwy);
    const int nf = p.fluid_number_total, ns = p.solid_number, nv = p.virt_number;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nf) {
        if (!(kinds & 1)) return;
        const int i = (int)t;
        const float2 x = d.f_pos[i];
        float2 off;
        const int2 c = split_pos(gr, x.x, x.y, off, d.err, 0, i);
        d.f_cell[i] = c.x * gr.ny + c.y;
        d.f_off[i] = off;
        d.f_offc[i] = make_float2(0.f, 0.f);
        d.f_velc[i] = make_float2(0.f, 0.f);
    } else if (t < (long)nf + ns) {
        if (!(kinds & 2)) return;
        const int i = (int)(t - nf);
        const double2 X = d.s_ref[i], x = d.s_pos[i];
        float2 roff;
        const int2 rc = split_pos(gr, X.x, X.y, roff, d.err, 1, i);
        d.s_rc[i] = rc;
        d.s_roff[i] = roff;
        float2 comp;
        d.s_u[i] = round_f2(make_double2(x.x - X.x, x.y - X.y), comp);
        d.s_uc[i] = comp;
        d.s_v[i] = round_f2(d.s_vel[i], comp);
        d.s_vc[i] = comp;
        const double2 a = d.s_dudt[i];
        d.s_acc[i] = make_float2((float)a.x, (float)a.y);
    } else if (t < (long)nf + ns + nv) {
        if (!(kinds & 4)) return;
        const int i = (int)(t - nf - ns);
        const float2 x = d.v_pos[i];
        float2 off;
        const int2 c = split_pos(gr, x.x, x.y, off, d.err, 2, i);
        d.v_cell[i] = c.x * gr.ny + c.y;
        d.v_off[i] = off;
    }
}

// kinds: bit 0 fluid, bit 1 solid
__global__ void k_join(const __grid_constant__ One g, int kinds) {
    const Scene &S = g.s;
    const sphnj_params &p = S.p;
    const DevState &d = S.d;
    const Grid2 gr = grid_of(p);
    const int nf = p.fluid_number_total, ns = p.solid_number;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nf) {
        if (!(kinds & 1)) return;
        const int i = (int)t;
        const int c = d.f_cell[i];
        const int cx = c / gr.ny, cy = c - cx * gr.ny;
        const float2 off = d.f_off[i], oc = d.f_offc[i];
        d.f_pos[i] = make_float2((float)(gr.x0 + cx * gr.wx + ((double)off.x - (double)oc.x)),
                                 (float)(gr.y0 + cy * gr.wy + ((double)off.y - (double)oc.y)));
    } else if (t < (long)nf + ns) {
        if (!(kinds & 2)) return;
        const int i = (int)(t - nf);
        const double2 X = d.s_ref[i];
        const float2 u = d.s_u[i], uc = d.s_uc[i], v = d.s_v[i], vc = d.s_vc[i], a = d.s_acc[i];
        d.s_pos[i] = make_double2(X.x + ((double)u.x - (double)uc.x), X.y + ((double)u.y - (double)uc.y));
        d.s_vel[i] = make_double2((double)v.x - (double)vc.x, (double)v.y - (double)vc.y);
        d.s_dudt[i] = make_double2((double)a.x, (double)a.y);
    }
}

// Fluid fields between the device state and device-mapped host arrays, one
// thread per particle: every host load is issued before any store, so a
// warp keeps its reads of the host link in flight together.  Positions are
// split (in) or joined (out) with k_split / k_join's fluid arithmetic, and
// f_pos is written as those kernels leave it.
template <bool kMixed>
__global__ void __launch_bounds__(kBlock) k_fluid_from_host(const __grid_constant__ One g, FluidHost h, double iwx,
                                                            double iwy) {
    const Scene &S = g.s;
    const sphnj_params &p = S.p;
    const DevState &d = S.d;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.fluid_number_total) return;
    const int i = (int)t;
    float2 x = make_float2(0.f, 0.f), v = make_float2(0.f, 0.f);
    float rho = 0.f, pr = 0.f;
    if (h.pos) x = h.pos[i];
    if (h.vel) v = h.vel[i];
    if (h.rho) rho = h.rho[i];
    if (h.p) pr = h.p[i];
    if (h.pos) {
        d.f_pos[i] = x;
        if constexpr (kMixed) {
            const Grid2 gr = grid_of(p, iwx, iwy);
            float2 off;
            const int2 c = split_pos(gr, x.x, x.y, off, d.err, 0, i);
            d.f_cell[i] = c.x * gr.ny + c.y;
            d.f_off[i] = off;
            d.f_offc[i] = make_float2(0.f, 0.f);
        }
    }
    if (h.vel) d.f_vel[i] = v;
    // new positions or velocities start without compensation
    if (kMixed && (h.pos || h.vel)) d.f_velc[i] = make_float2(0.f, 0.f);
    if (h.rho) d.f_rho[i] = rho;
    if (h.p) d.f_p[i] = pr;
}

template <bool kMixed>
__global__ void __launch_bounds__(kBlock) k_fluid_to_host(const __grid_constant__ One g, FluidHost h) {
    const Scene &S = g.s;
    const sphnj_params &p = S.p;
    const DevState &d = S.d;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.fluid_number_total) return;
    const int i = (int)t;
    if (h.pos) {
        float2 x;
        if constexpr (kMixed) {
            const Grid2 gr = grid_of(p);
            const int c = d.f_cell[i];
            const int cx = c / gr.ny, cy = c - cx * gr.ny;
            const float2 off = d.f_off[i], oc = d.f_offc[i];
            x = make_float2((float)(gr.x0 + cx * gr.wx + ((double)off.x - (double)oc.x)),
                            (float)(gr.y0 + cy * gr.wy + ((double)off.y - (double)oc.y)));
            d.f_pos[i] = x;
        } else {
            x = d.f_pos[i];
        }
        h.pos[i] = x;
    }
    if (h.vel) h.vel[i] = d.f_vel[i];
    if (h.rho) h.rho[i] = d.f_rho[i];
    if (h.p) h.p[i] = d.f_p[i];
}

}  // namespace

void launch_fluid_from_host(cudaStream_t st, const GroupOne &g, const FluidHost &h) {
    const sphnj_params &p = g.s.p;
    if (p.fluid_number_total <= 0 || !h.any()) return;
    const unsigned blocks = grid_for(p.fluid_number_total, kBlock);
    if (g.form == SPHNJ_FORM_MIXED)
        k_fluid_from_host<true><<<blocks, kBlock, 0, st>>>(One{g.s}, h, 1.0 / (double)p.interval[0],
                                                           1.0 / (double)p.interval[1]);
    else
        k_fluid_from_host<false><<<blocks, kBlock, 0, st>>>(One{g.s}, h, 0.0, 0.0);
}

void launch_fluid_to_host(cudaStream_t st, const GroupOne &g, const FluidHost &h) {
    const sphnj_params &p = g.s.p;
    if (p.fluid_number_total <= 0 || !h.any()) return;
    const unsigned blocks = grid_for(p.fluid_number_total, kBlock);
    if (g.form == SPHNJ_FORM_MIXED)
        k_fluid_to_host<true><<<blocks, kBlock, 0, st>>>(One{g.s}, h);
    else
        k_fluid_to_host<false><<<blocks, kBlock, 0, st>>>(One{g.s}, h);
}

void launch_mixed_split(cudaStream_t st, const GroupOne &g, int kinds) {
    const sphnj_params &p = g.s.p;
    const long n = (long)p.fluid_number_total + p.solid_number + p.virt_number;
    if (n > 0 && kinds)
        k_split<<<grid_for(n, kBlock), kBlock, 0, st>>>(One{g.s}, kinds, 1.0 / (double)p.interval[0],
                                                        1.0 / (double)p.interval[1]);
}

void launch_mixed_join(cudaStream_t st, const GroupOne &g, int kinds) {
    const sphnj_params &p = g.s.p;
    const long n = (long)p.fluid_number_total + p.solid_number;
    if (n > 0 && kinds) k_join<<<grid_for(n, kBlock), kBlock, 0, st>>>(One{g.s}, kinds);
}

}  // namespace sphnj
