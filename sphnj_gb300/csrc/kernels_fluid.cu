// Fluid passes on sm_103a, reference precision (FP32 fluid state).
//
//   k_fluid_pair     findFluidPair + fluidFluid/Solid/VirtCalculate
//                    (fluid.cu:25-254): Riemann continuity and momentum,
//                    velocity gradient, colour, kernel-gradient sum and the
//                    near-free-surface flag, summed over the 3x3 stencil in
//                    the reference's list order (fluid, solid, virtual per
//                    neighbour cell, slots 0..8).
//   k_fluid_update   fluidUpdate (fluid.cu:256-287) fused with getMaxSpeed
//                    (fluid.cu:429-440): the max of |v| is reduced on the
//                    device (the reference copies every velocity to the host
//                    each step).  |v|^2 is formed with round-to-nearest
//                    multiplies and adds and compared as float bits, which
//                    equals the reference's host loop over |v| (sqrt is
//                    monotone), so max_speed is bit-identical.
//   k_shift_gradient correctionCalculate (fluid.cu:304-367)
//   k_shift_update   shiftDisplacementCalculate + correctionUpdate
//                    (fluid.cu:369-427)
//
// Math: the neighbour sweeps use __expf and __fdividef, the approximations
// that the reference's -use_fast_math build uses for expf and '/'
// (CMakeLists.txt:16-19); the equation of state keeps powf, whose fast form
// loses ~1e-4 relative pressure accuracy near the reference density.
#include "kernels.h"

namespace sphnj {

namespace {

constexpr int kPairBlock = 128;
constexpr int kBlock = 256;

__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float gw(const sphnj_params &p, float q2) {
    return __expf(-q2) * p.kernel_differential * p.coefficient_3d_to_2d;
}
__device__ __forceinline__ float2 nrm_fast(float2 a) {
    float z = sqn(a);
    if (z > 0.0f) {
        float s = sqrtf(z);
        return make_float2(fdiv(a.x, s), fdiv(a.y, s));
    }
    return a;
}
__device__ __forceinline__ float by_phase(const float (&a)[2], int ph) { return ph ? a[1] : a[0]; }

struct FAcc {
    float velo_div, color;
    float2 du_dt, grad;
    float4 du_dx;  // m00 m10 m01 m11
    int near;
};

// Riemann pair term shared by fluid, solid and virtual neighbours
// (fluid.cu:48-58, 115-124, 167-177).
__device__ __forceinline__ void riemann(float2 u_i, float2 u_j, float p_i, float p_j, float rho_i, float rho_j,
                                        float cs, float2 dx, float kc, FAcc &a) {
    const float rs = rho_i + rho_j;
    float ps = fdiv(rho_i * p_j + rho_j * p_i, rs);
    float2 n = nrm_fast(dx);
    float du = dot2(sub2(u_i, u_j), n);
    if (du >= 0.0f) ps += fdiv(rho_i * rho_j * du, rs) * fminf(3.0f * du, cs);
    float2 vs = make_float2(fdiv(rho_i * u_i.x + rho_j * u_j.x, rs), fdiv(rho_i * u_i.y + rho_j * u_j.y, rs));
    float t = fdiv(fdiv(p_i - p_j, rs), cs);
    vs.x += t * n.x;
    vs.y += t * n.y;
    float am = fdiv(-2.0f * ps, rho_i);
    a.du_dt.x += am * dx.x * kc;
    a.du_dt.y += am * dx.y * kc;
    a.velo_div += 2.0f * rho_i * dot2(sub2(u_i, vs), dx) * kc;
    float2 w = sub2(u_j, u_i);
    a.du_dx.x += w.x * dx.x * kc;
    a.du_dx.y += w.y * dx.x * kc;
    a.du_dx.z += w.x * dx.y * kc;
    a.du_dx.w += w.y * dx.y * kc;
}

__device__ __forceinline__ void viscous(const sphnj_params &p, float2 u_i, float2 u_j, float rho_i, int ph_i,
                                        float2 dx, float kc, FAcc &a) {
    float vis = dot2(sub2(u_j, u_i), dx);
    vis = fdiv(vis, sqn(dx) + 0.01f * p.smoothing_length_square);
    float am = fdiv(8.0f * by_phase(p.viscosity, ph_i) * vis, rho_i);
    a.du_dt.x += am * dx.x * kc;
    a.du_dt.y += am * dx.y * kc;
}

__global__ void __launch_bounds__(kPairBlock) k_fluid_pair(sphnj_params p, DevState d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nf = p.fluid_number_total;
    if (i >= nf) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const bool viscid = p.is_fluid_viscid != 0;
    const float2 x_i = d.f_pos[i], u_i = d.f_vel[i];
    const float p_i = d.f_p[i], rho_i = d.f_rho[i];
    const int ph_i = d.f_phase[i];
    const float cs = by_phase(p.sound_speed, ph_i);
    const int c = d.f_cell[i];
    FAcc a;
    a.velo_div = 0.f; a.color = 0.f;
    a.du_dt = make_float2(0.f, 0.f); a.grad = make_float2(0.f, 0.f);
    a.du_dx = make_float4(0.f, 0.f, 0.f, 0.f);
    a.near = SPHNJ_NO_PARTICLE;
    for (int n = 0; n < 9; ++n) {
        const int m = neighbour_cell(c, n, nx, ny);
        if (m < 0) continue;
        const int2 rf = __ldg(&d.rng_f[m]);
        for (int t = rf.x; t < rf.x + rf.y; ++t) {
            const int j = __ldg(&d.lst_f[t]);
            const float2 x_j = __ldg(&d.f_pos[j]);
            const float2 dx = sub2(x_j, x_i);
            if (!(sqn(dx) < R2)) continue;
            const float kc = gw(p, sqn(dx) * hinv2);
            const float2 u_j = __ldg(&d.f_vel[j]);
            riemann(u_i, u_j, p_i, __ldg(&d.f_p[j]), rho_i, __ldg(&d.f_rho[j]), cs, dx, kc, a);
            const int ph_j = __ldg(&d.f_phase[j]);
            if (!(ph_i == SPHNJ_LIQUID && ph_j == SPHNJ_GAS)) {
                a.color += dot2(dx, dx) * kc;
                a.grad.x += dx.x * kc;
                a.grad.y += dx.y * kc;
            }
            if (__ldg(&d.f_fbt[j]) == SPHNJ_FREE_SURFACE && ph_i == SPHNJ_LIQUID && i != j) {
                if (sqn(dx) < 0.25f * R2) a.near = SPHNJ_HAS_NEAR_PARTICLE;
                else if (a.near == SPHNJ_NO_PARTICLE) a.near = SPHNJ_HAS_PARTICLE;
            }
            if (viscid) viscous(p, u_i, u_j, rho_i, ph_i, dx, kc, a);
        }
        const int2 rs = __ldg(&d.rng_s[m]);
        for (int t = rs.x; t < rs.x + rs.y; ++t) {
            const int j = __ldg(&d.lst_s[t]);
            const float2 x_j = to_f2(d.s_pos[j]);
            const float2 dx = sub2(x_j, x_i);
            if (!(sqn(dx) < R2)) continue;
            const float kc = gw(p, sqn(dx) * hinv2);
            const float2 u_j = to_f2(d.s_vel[j]);
            riemann(u_i, u_j, p_i, __ldg(&d.s_p[j]), rho_i, rho_i, cs, dx, kc, a);
            a.grad.x += dx.x * kc;
            a.grad.y += dx.y * kc;
            if (viscid) viscous(p, u_i, u_j, rho_i, ph_i, dx, kc, a);
        }
        const int2 rv = __ldg(&d.rng_v[m]);
        for (int t = rv.x; t < rv.x + rv.y; ++t) {
            const int j = __ldg(&d.lst_v[t]);
            const float2 x_j = __ldg(&d.v_pos[j]);
            const float2 dx = sub2(x_j, x_i);
            if (!(sqn(dx) < R2)) continue;
            const float kc = gw(p, sqn(dx) * hinv2);
            const float rho_j = by_phase(p.reference_density, __ldg(&d.v_phase[j]));
            const float2 u_j = __ldg(&d.v_vel[j]);
            riemann(u_i, u_j, p_i, __ldg(&d.v_p[j]), rho_i, rho_j, cs, dx, kc, a);
            // fluid.cu:179 reads the fluid phase array with the virtual
            // index; past the fluid count it is taken as LIQUID.
            const int ph_j = j < nf ? (int)__ldg(&d.f_phase[j]) : SPHNJ_LIQUID;
            if (!(ph_i == SPHNJ_LIQUID && ph_j == SPHNJ_GAS)) {
                a.color += dot2(dx, dx) * kc;
                a.grad.x += dx.x * kc;
                a.grad.y += dx.y * kc;
            }
            if (viscid) viscous(p, u_i, u_j, rho_i, ph_i, dx, kc, a);
        }
    }
    d.f_drho[i] = a.velo_div;
    d.f_dudt[i] = a.du_dt;
    d.f_near[i] = (uint8_t)a.near;
    d.f_color[i] = a.color;
    d.f_grad[i] = a.grad;
    d.f_dudx[i] = a.du_dx;
}

// densityToPressure, fluid.cu:15-23
__device__ __forceinline__ float density_to_pressure(const sphnj_params &p, float rho, int ph) {
    float pr = (powf(rho * by_phase(p.reference_density_inverse, ph), by_phase(p.gamma, ph)) - 1.0f) *
               by_phase(p.coefficient_rho2p, ph);
    return fmaxf(pr, p.min_pressure);
}

__global__ void __launch_bounds__(kBlock) k_fluid_update(sphnj_params p, DevState d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int sp2 = 0u;
    if (i < p.fluid_number_total) {
        const int ph = d.f_phase[i];
        const float dt = p.dt;
        float2 x = d.f_pos[i], v = d.f_vel[i], a = d.f_dudt[i];
        if (p.transient_type == SPHNJ_STEADY) {
            a.x += -0.1f * v.x;
            a.y += -0.1f * v.y;
            d.f_dudt[i] = a;
        }
        x.x += v.x * dt;
        x.y += v.y * dt;
        v.x += (a.x + p.gravity[0]) * dt;
        v.y += (a.y + p.gravity[1]) * dt;
        float rho = d.f_rho[i] + d.f_drho[i] * dt;
        rho = fmaxf(rho, by_phase(p.min_density, ph));
        d.f_rho[i] = rho;
        d.f_p[i] = density_to_pressure(p, rho, ph);
        x.x = fminf(fmaxf(x.x, p.domain_xmin[0]), p.domain_xmax[0]);
        x.y = fminf(fmaxf(x.y, p.domain_xmin[1]), p.domain_xmax[1]);
        d.f_pos[i] = x;
        d.f_vel[i] = v;
        float s2 = __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
        if (s2 == s2) sp2 = __float_as_uint(s2);  // NaN never wins, as on the host
    }
    // block max of non-negative float bits, one atomic per block
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sp2 = max(sp2, __shfl_xor_sync(0xffffffffu, sp2, o));
    __shared__ unsigned int wmax[kBlock / 32];
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = sp2;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned int v = threadIdx.x < kBlock / 32 ? wmax[threadIdx.x] : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0 && v) atomicMax(d.max_speed2_bits, v);
    }
}

__global__ void __launch_bounds__(kPairBlock) k_shift_gradient(sphnj_params p, DevState d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.fluid_number_total) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const float2 x_i = d.f_pos[i];
    const int c = d.f_cell[i];
    float2 g = make_float2(0.f, 0.f);
    for (int n = 0; n < 9; ++n) {
        const int m = neighbour_cell(c, n, nx, ny);
        if (m < 0) continue;
        const int2 rf = __ldg(&d.rng_f[m]);
        for (int t = rf.x; t < rf.x + rf.y; ++t) {
            const float2 dx = sub2(__ldg(&d.f_pos[__ldg(&d.lst_f[t])]), x_i);
            if (sqn(dx) < R2) {
                const float kc = gw(p, sqn(dx) * hinv2);
                g.x += dx.x * kc;
                g.y += dx.y * kc;
            }
        }
        const int2 rs = __ldg(&d.rng_s[m]);
        for (int t = rs.x; t < rs.x + rs.y; ++t) {
            const float2 dx = sub2(to_f2(d.s_pos[__ldg(&d.lst_s[t])]), x_i);
            if (sqn(dx) < R2) {
                const float kc = gw(p, sqn(dx) * hinv2);
                g.x += dx.x * kc;
                g.y += dx.y * kc;
            }
        }
        const int2 rv = __ldg(&d.rng_v[m]);
        for (int t = rv.x; t < rv.x + rv.y; ++t) {
            const float2 dx = sub2(__ldg(&d.v_pos[__ldg(&d.lst_v[t])]), x_i);
            if (sqn(dx) < R2) {
                const float kc = gw(p, sqn(dx) * hinv2);
                g.x += dx.x * kc;
                g.y += dx.y * kc;
            }
        }
    }
    d.f_grad[i] = g;
}

// (I - n n^T) d with n = normalize(g), zeroed below EPS_FOR_SUM
// (fluid.cu:394-397)
__device__ __forceinline__ float2 project(float2 g, float2 disp) {
    float2 n = normalized(g);
    if (sqrtf(sqn(n)) < EPS_FOR_SUM) n = make_float2(0.f, 0.f);
    float m00 = 1.0f - n.x * n.x, m10 = 0.0f - n.y * n.x, m01 = 0.0f - n.x * n.y, m11 = 1.0f - n.y * n.y;
    return make_float2(m00 * disp.x + m01 * disp.y, m10 * disp.x + m11 * disp.y);
}

__global__ void __launch_bounds__(kBlock) k_shift_update(sphnj_params p, DevState d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.fluid_number_total) return;
    // getMaxSpeed's clamp, fluid.cu:438-439
    const float vmax = __fsqrt_rn(__uint_as_float(*d.max_speed2_bits));
    const float max_speed = fminf(vmax, __fmul_rn(0.1f, fminf(p.sound_speed[0], p.sound_speed[1])));
    const float s = -p.particle_shift_coef * p.smoothing_length * p.dt;
    const float2 g = d.f_grad[i];
    const float2 disp = make_float2(s * g.x, s * g.y);
    const int ph = d.f_phase[i];
    const float color = d.f_color[i];
    const int near = d.f_near[i];
    float2 dd;
    uint8_t bt;
    if (ph == SPHNJ_GAS) {
        bt = SPHNJ_INNER;
        dd = disp;
    } else if (color < 1.5f) {
        if (near == SPHNJ_NO_PARTICLE) {
            bt = SPHNJ_SPLASH;
            dd = make_float2(0.f, 0.f);
        } else {
            bt = SPHNJ_FREE_SURFACE;
            dd = project(g, disp);
        }
    } else if (color < 2.0f && near == SPHNJ_HAS_NEAR_PARTICLE) {
        bt = SPHNJ_VICINITY;
        dd = project(g, disp);
    } else {
        bt = SPHNJ_INNER;
        dd = disp;
    }
    d.f_fbt[i] = bt;
    const float2 sh = make_float2(max_speed * dd.x, max_speed * dd.y);
    float2 x = d.f_pos[i];
    x.x += sh.x;
    x.y += sh.y;
    d.f_pos[i] = x;
    const float4 m = d.f_dudx[i];
    float2 v = d.f_vel[i];
    v.x += m.x * sh.x + m.z * sh.y;
    v.y += m.y * sh.x + m.w * sh.y;
    d.f_vel[i] = v;
}

}  // namespace

void launch_fluid_pair(cudaStream_t st, const sphnj_params &p, const DevState &d) {
    const int n = p.fluid_number_total;
    if (n > 0) k_fluid_pair<<<grid_for(n, kPairBlock), kPairBlock, 0, st>>>(p, d);
}
void launch_fluid_update(cudaStream_t st, const sphnj_params &p, const DevState &d) {
    const int n = p.fluid_number_total;
    if (n > 0) k_fluid_update<<<grid_for(n, kBlock), kBlock, 0, st>>>(p, d);
}
void launch_shift_gradient(cudaStream_t st, const sphnj_params &p, const DevState &d) {
    const int n = p.fluid_number_total;
    if (n > 0) k_shift_gradient<<<grid_for(n, kPairBlock), kPairBlock, 0, st>>>(p, d);
}
void launch_shift_update(cudaStream_t st, const sphnj_params &p, const DevState &d) {
    const int n = p.fluid_number_total;
    if (n > 0) k_shift_update<<<grid_for(n, kBlock), kBlock, 0, st>>>(p, d);
}

}  // namespace sphnj
