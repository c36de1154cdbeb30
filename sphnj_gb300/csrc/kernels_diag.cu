// Global diagnostics reduced on the device in FP64 (sphnj_diagnostics).
//
// The reference computes its global outputs on the host from full copies of
// the state every step (output.cu:283-560).  Here a grid-stride kernel forms
// every particle's contribution in FP64 and reduces per block; one block then
// sums the block partials in a fixed order (so the result does not depend on
// scheduling) and finds the beam tip.  Both forms are read: the plain form's
// absolute / FP64 arrays, or the mixed form's cell + offset and displacement
// state (value = main part - Kahan compensation).
#include "context.h"
#include "forms.cuh"

namespace sphnj {

namespace {

enum Slot {
    // sums
    D_MOMX, D_MOMY, D_EKF, D_MASS, D_EKS, D_EPS, D_FX, D_FY, D_PSUM, D_REFY, D_NLIQ,
    // maxima
    D_FRONT, D_VMLIN, D_VMAUX, D_REFXMAX,
    D_SLOTS
};
constexpr int kSums = D_FRONT;
constexpr int kThreads = 256;

__device__ __forceinline__ double comb(int s, double a, double b) { return s < kSums ? a + b : fmax(a, b); }
__device__ __forceinline__ double ident(int s) { return s < kSums ? 0.0 : -1.0e300; }

__device__ __forceinline__ double2 fluid_pos(const sphnj_params &p, const DevState &d, int i) {
    if (d.f_off) {
        const int ny = p.cell_number[1], c = d.f_cell[i], cx = c / ny, cy = c - cx * ny;
        const float2 o = d.f_off[i], oc = d.f_offc[i];
        return make_double2((double)p.cell_xmin[0] + cx * (double)p.interval[0] + ((double)o.x - (double)oc.x),
                            (double)p.cell_xmin[1] + cy * (double)p.interval[1] + ((double)o.y - (double)oc.y));
    }
    const float2 x = d.f_pos[i];
    return make_double2(x.x, x.y);
}
__device__ __forceinline__ double2 fluid_vel(const DevState &d, int i) {
    const float2 v = d.f_vel[i];
    if (d.f_velc) {
        const float2 c = d.f_velc[i];
        return make_double2((double)v.x - (double)c.x, (double)v.y - (double)c.y);
    }
    return make_double2(v.x, v.y);
}
__device__ __forceinline__ double2 solid_pos(const DevState &d, int i) {
    if (d.s_u) {
        const double2 X = d.s_ref[i];
        const float2 u = d.s_u[i], uc = d.s_uc[i];
        return make_double2(X.x + ((double)u.x - (double)uc.x), X.y + ((double)u.y - (double)uc.y));
    }
    return d.s_pos[i];
}
__device__ __forceinline__ double2 solid_vel(const DevState &d, int i) {
    if (d.s_v) {
        const float2 v = d.s_v[i], c = d.s_vc[i];
        return make_double2((double)v.x - (double)c.x, (double)v.y - (double)c.y);
    }
    return d.s_vel[i];
}

// Block-wide combine of acc[] into out[] (thread 0 writes).
__device__ void block_combine(double (&acc)[D_SLOTS], double *out) {
    __shared__ double sm[kThreads / 32][D_SLOTS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < D_SLOTS; ++s) {
        double v = acc[s];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = comb(s, v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0) sm[w][s] = v;
    }
    __syncthreads();
    if (threadIdx.x < D_SLOTS) {
        const int s = threadIdx.x;
        double v = sm[0][s];
        for (int k = 1; k < kThreads / 32; ++k) v = comb(s, v, sm[k][s]);
        out[s] = v;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads) k_diag_partials(const __grid_constant__ One g, double *part) {
    const Scene &S = g.s;
    const sphnj_params &p = S.p;
    const DevState &d = S.d;
    const int nf = p.fluid_number_total, ns = p.solid_number;
    const double dd = (double)p.particle_diameter, dv = dd * dd;
    double acc[D_SLOTS];
#pragma unroll
    for (int s = 0; s < D_SLOTS; ++s) acc[s] = ident(s);
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += stride) {
        const int ph = d.f_phase[i];
        const double m = (double)(ph == SPHNJ_GAS ? p.reference_density[1] : p.reference_density[0]) * dv;
        const double2 x = fluid_pos(p, d, i), v = fluid_vel(d, i);
        acc[D_MOMX] += m * v.x;
        acc[D_MOMY] += m * v.y;
        acc[D_EKF] += 0.5 * m * (v.x * v.x + v.y * v.y);
        acc[D_MASS] += (double)d.f_rho[i] * dv;
        if (ph == SPHNJ_LIQUID) {
            acc[D_NLIQ] += 1.0;
            acc[D_FRONT] = fmax(acc[D_FRONT], x.x);
        }
    }
    const double lam = (double)p.lambda, mu = (double)p.nu;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += stride) {
        const double2 X = d.s_ref[i], v = solid_vel(d, i);
        const dmat2 F = d.s_F[i], P = d.s_P[i];
        const int mat = d.s_mat[i];
        // outputTotalEnergy (output.cu:426-455): Ep over every particle, Ek
        // over reference x >= 0 only, both with the linear-elastic density
        const double e00 = 0.5 * (F.m00 * F.m00 + F.m10 * F.m10 - 1.0);
        const double e11 = 0.5 * (F.m01 * F.m01 + F.m11 * F.m11 - 1.0);
        const double e01 = 0.5 * (F.m00 * F.m01 + F.m10 * F.m11);
        const double tr = e00 + e11;
        acc[D_EPS] += (0.5 * lam * tr * tr + mu * (e00 * e00 + e11 * e11 + 2.0 * e01 * e01)) * dv;
        if (X.x >= 0.0) acc[D_EKS] += 0.5 * (double)p.solid_reference_density * dv * (v.x * v.x + v.y * v.y);
        // outputTotalForce (output.cu:283-305)
        const double rho = mat == SPHNJ_LINEAR_ELASTIC ? (double)p.solid_reference_density : (double)p.auxetic_density;
        const float2 cf = d.s_couple[i];
        acc[D_FX] += (double)cf.x * dv * rho;
        acc[D_FY] += (double)cf.y * dv * rho;
        // outputVonMisesStress (output.cu:503-544): sigma = F^-1 P
        const double det = F.m00 * F.m11 - F.m10 * F.m01;
        if (det != 0.0) {
            const double i00 = F.m11 / det, i10 = -F.m10 / det, i01 = -F.m01 / det, i11 = F.m00 / det;
            const double s00 = i00 * P.m00 + i01 * P.m10, s11 = i10 * P.m01 + i11 * P.m11;
            const double s01 = i00 * P.m01 + i01 * P.m11;
            const double vm = sqrt(0.5 * (s00 - s11) * (s00 - s11) + 3.0 * s01 * s01);
            if (mat == SPHNJ_LINEAR_ELASTIC) acc[D_VMLIN] = fmax(acc[D_VMLIN], vm);
            else if (mat == SPHNJ_AUXETIC) acc[D_VMAUX] = fmax(acc[D_VMAUX], vm);
        }
        acc[D_PSUM] += (double)d.s_p[i];
        acc[D_REFY] += X.y;
        acc[D_REFXMAX] = fmax(acc[D_REFXMAX], X.x);
    }
    block_combine(acc, part + (size_t)blockIdx.x * D_SLOTS);
}

// One block: the partials in block order, then the tip particle.
__global__ void __launch_bounds__(kThreads) k_diag_final(const __grid_constant__ One g, const double *part,
                                                         int nblocks, int step, sphnj_diag *out) {
    const Scene &S = g.s;
    const sphnj_params &p = S.p;
    const DevState &d = S.d;
    const int ns = p.solid_number;
    double acc[D_SLOTS];
#pragma unroll
    for (int s = 0; s < D_SLOTS; ++s) acc[s] = ident(s);
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int s = 0; s < D_SLOTS; ++s) acc[s] = comb(s, acc[s], part[(size_t)b * D_SLOTS + s]);
    __shared__ double tot[D_SLOTS];
    block_combine(acc, tot);
    // tip: largest reference x (within 1e-12), then closest to the mean reference y
    const double xmax = tot[D_REFXMAX], ymean = ns > 0 ? tot[D_REFY] / ns : 0.0;
    double best = 1.0e300;
    int besti = -1;
    for (int i = threadIdx.x; i < ns; i += blockDim.x) {
        const double2 X = d.s_ref[i];
        if (X.x >= xmax - 1e-12) {
            const double e = fabs(X.y - ymean);
            if (e < best || (e == best && i < besti)) {
                best = e;
                besti = i;
            }
        }
    }
    __shared__ double sb[kThreads];
    __shared__ int si[kThreads];
    sb[threadIdx.x] = best;
    si[threadIdx.x] = besti;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const double b2 = sb[threadIdx.x + o];
            const int i2 = si[threadIdx.x + o];
            if (i2 >= 0 && (si[threadIdx.x] < 0 || b2 < sb[threadIdx.x] ||
                            (b2 == sb[threadIdx.x] && i2 < si[threadIdx.x]))) {
                sb[threadIdx.x] = b2;
                si[threadIdx.x] = i2;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        sphnj_diag r;
        r.step = step;
        r.n_liquid = (int)tot[D_NLIQ];
        r.front = tot[D_NLIQ] > 0.0 ? tot[D_FRONT] + 0.5 * (double)p.particle_diameter : -1.0e300;
        r.fluid_momentum[0] = tot[D_MOMX];
        r.fluid_momentum[1] = tot[D_MOMY];
        r.fluid_kinetic = tot[D_EKF];
        r.fluid_mass = tot[D_MASS];
        r.tip_disp[0] = r.tip_disp[1] = 0.0;
        if (si[0] >= 0) {
            const double2 x = solid_pos(d, si[0]), X = d.s_ref[si[0]];
            r.tip_disp[0] = x.x - X.x;
            r.tip_disp[1] = x.y - X.y;
        }
        r.solid_kinetic = tot[D_EKS];
        r.solid_strain = tot[D_EPS];
        r.total_force[0] = tot[D_FX];
        r.total_force[1] = tot[D_FY];
        r.von_mises[0] = tot[D_VMLIN] > 0.0 ? tot[D_VMLIN] : 0.0;
        r.von_mises[1] = tot[D_VMAUX] > 0.0 ? tot[D_VMAUX] : 0.0;
        r.mean_pressure = ns > 0 ? tot[D_PSUM] / ns : 0.0;
        *out = r;
    }
}

static_assert(D_SLOTS <= kDiagSlots, "diagnostic partials overflow their arena slots");

// getProbeData (probe.cu:7-107): Shepard interpolation of velocity, pressure
// and density at a point from the fluid and solid entries of its 3x3 cells
// (solid density taken as 0, as there).  The reference walks neighbour cell j
// with the probe cell's own counts (probe.cu:51,74); here each cell's own
// entries are walked.  One thread per probe; the point's cell is found as
// findProbeCell does, and a point outside the grid gives the no-neighbour
// result.
template <class F>
__global__ void k_probe(const __grid_constant__ One g, int n, const float2 *pts, float4 *out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const Scene &S = g.s;
    const sphnj_params &p = S.p;
    const DevState &d = S.d;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float2 x = pts[k];
    const int cx = (int)__fmul_rn(__fsub_rn(x.x, p.cell_xmin[0]), p.interval_inv[0]);
    const int cy = (int)__fmul_rn(__fsub_rn(x.y, p.cell_xmin[1]), p.interval_inv[1]);
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    float sum = 0.f, pr = 0.f, rho = 0.f;
    float2 vel = make_float2(0.f, 0.f);
    if (cx >= 0 && cx < nx && cy >= 0 && cy < ny) {
        // the probe in the frame of its own cell (mixed form)
        const float2 xi = F::kMixed
                              ? make_float2(__fsub_rn(x.x, __fmaf_rn((float)cx, p.interval[0], p.cell_xmin[0])),
                                            __fsub_rn(x.y, __fmaf_rn((float)cy, p.interval[1], p.cell_xmin[1])))
                              : x;
        const int c = cx * ny + cy;
        for (int nb = 0; nb < 9; ++nb) {
            const int m = neighbour_cell(c, nb, nx, ny);
            if (m < 0) continue;
            const float2 sh = F::shift(p, Frame{0, 0}, nb);
            const int2 rf = d.rng_f[m];
            for (int t = rf.x; t < rf.x + rf.y; ++t) {
                const int j = d.lst_f[t];
                const float2 dx = sub2(F::f_nbr(d, j, sh), xi);
                const float q = sqn(dx);
                if (!(q < R2)) continue;
                const float w = (expf(-q * hinv2) - p.kernel_coefficient_1) * p.kernel_coefficient_2 *
                                p.coefficient_3d_to_2d;
                sum += w;
                const float2 v = d.f_vel[j];
                vel.x += v.x * w;
                vel.y += v.y * w;
                pr += d.f_p[j] * w;
                rho += d.f_rho[j] * w;
            }
            const int2 rs = d.rng_s[m];
            for (int t = rs.x; t < rs.x + rs.y; ++t) {
                const int j = d.lst_s[t];
                const float2 dx = sub2(F::s_nbr(d, j, sh), xi);
                const float q = sqn(dx);
                if (!(q < R2)) continue;
                const float w = (expf(-q * hinv2) - p.kernel_coefficient_1) * p.kernel_coefficient_2 *
                                p.coefficient_3d_to_2d;
                sum += w;
                const float2 v = F::s_vel(d, j);
                vel.x += v.x * w;
                vel.y += v.y * w;
                pr += d.s_p[j] * w;
            }
        }
    }
    out[k] = sum != 0.0f ? make_float4(vel.x / sum, vel.y / sum, pr / sum, rho / sum)
                         : make_float4(0.f, 0.f, 0.f, p.reference_density[0]);
}

}  // namespace

void launch_probe(cudaStream_t st, const GroupOne &g, int n, const float2 *pts, float4 *out) {
    if (n <= 0) return;
    if (g.form == SPHNJ_FORM_MIXED) k_probe<FormMixed><<<grid_for(n, 128), 128, 0, st>>>(One{g.s}, n, pts, out);
    else k_probe<FormPlain><<<grid_for(n, 128), 128, 0, st>>>(One{g.s}, n, pts, out);
}

void launch_diagnostics(cudaStream_t st, const GroupOne &g, double *part, int step, sphnj_diag *out) {
    k_diag_partials<<<kDiagBlocks, kThreads, 0, st>>>(One{g.s}, part);
    k_diag_final<<<1, kThreads, 0, st>>>(One{g.s}, part, kDiagBlocks, step, out);
}

}  // namespace sphnj
