// Virtual (wall) and solid passes on sm_103a, reference precision:
// virtual/fluid FP32, solid state FP64 with FP32 kernel weights
// (include/particle.cuh:104-115, solid.cu:18-19,271-272).
//
//   k_virt_normal      getVirtNormal (virt.cu:8-48): wall normals (setup
//                      only), the reference's index-order sum over the
//                      per-cell lists of the nine stencil cells.
//   k_virt_data        getVirtData + virtDataCalculate (virt.cu:61-149)
//   k_solid_couple     solidCoupleUpdate (solid.cu:355-444)
//   k_solid_deform     solidDeformationCalculate (solid.cu:7-23,169-209)
//                      with the SVK / auxetic-plastic stress (solid.cu:80-167)
//   k_solid_force      solidForceCalculate (solid.cu:211-353)
//   k_solid_update     solidUpdate (solid.cu:446-471)
#include "forms.cuh"
#include "kernels.h"

namespace sphnj {

namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ float gw(const sphnj_params &p, float q2) {
    return __expf(-q2) * p.kernel_differential * p.coefficient_3d_to_2d;
}
__device__ __forceinline__ float sw(const sphnj_params &p, float q2) {
    return (__expf(-q2) - p.kernel_coefficient_1) * p.kernel_coefficient_2 * p.coefficient_3d_to_2d;
}
__device__ __forceinline__ float by_phase(const float (&a)[2], int ph) { return ph ? a[1] : a[0]; }

// The reference sums over every virtual particle j in index order, those
// within the cutoff contributing.  All of them lie in the nine cells around
// particle i (cells are at least a cutoff wide), and each cell's particles
// are listed in ascending index order (launch_virt_index: ranges in lv.rng,
// indices in the sort scratch sc.sorted), so a nine-way merge of those lists
// visits the same j in the same order: the same sum, from about a hundred
// candidates instead of N_v.
template <class G> __global__ void __launch_bounds__(kBlock) k_virt_normal(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.virt_number) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const float2 x_i = d.v_pos[i];
    const int2 *rng = S.lv.rng;
    const int *lst = S.sc.sorted;
    const int c = d.v_cell[i];
    constexpr int kDone = 0x7fffffff;
    int cur[9], end[9], head[9];  // per stencil cell: next slot, end slot, index at the next slot
#pragma unroll
    for (int n = 0; n < 9; ++n) {
        const int m = neighbour_cell(c, n, nx, ny);
        const int2 r = m >= 0 ? __ldg(&rng[m]) : make_int2(0, 0);
        cur[n] = r.x;
        end[n] = r.x + r.y;
        head[n] = cur[n] < end[n] ? __ldg(&lst[cur[n]]) : kDone;
    }
    float2 nrm = make_float2(0.f, 0.f);
    for (;;) {
        int j = kDone, nj = 0;
#pragma unroll
        for (int n = 0; n < 9; ++n)
            if (head[n] < j) {
                j = head[n];
                nj = n;
            }
        if (j == kDone) break;
        const float2 dx = sub2(__ldg(&d.v_pos[j]), x_i);
        if (sqn(dx) < R2) {
            const float kc = gw(p, sqn(dx) * hinv2);
            nrm.x -= dx.x * kc;
            nrm.y -= dx.y * kc;
        }
#pragma unroll
        for (int n = 0; n < 9; ++n)  // advance the cell j came from (unrolled: the arrays stay in registers)
            if (n == nj) {
                ++cur[n];
                head[n] = cur[n] < end[n] ? __ldg(&lst[cur[n]]) : kDone;
            }
    }
    d.v_normal[i] = sqrtf(sqn(nrm)) < EPS_FOR_SUM ? make_float2(0.f, 0.f) : normalized(nrm);
}

template <class G, class F> __global__ void __launch_bounds__(kBlock) k_virt_data(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.virt_number) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const float gx = p.gravity[0], gy = p.gravity[1];
    const Frame fr{0, 0};
    const float2 x_i = F::v_home(p, d, fr, i);
    float2 vel = make_float2(0.f, 0.f);
    float pr = 0.f, sum = 0.f, nearest = LARGE_FLOAT;
    int phase = d.v_phase[i];
    for_each_in_stencil<F::kMixed>(d.rng_f, d.v_cell[i], nx, ny, [&](int t, int n) {
        const int j = __ldg(&d.lst_f[t]);
        const float2 dx = sub2(F::f_nbr(d, j, F::shift(p, fr, n)), x_i);
        const float d2 = sqn(dx);
        if (!(d2 < R2)) return;
        const float kc = sw(p, d2 * hinv2);
        sum += kc;
        const float2 vj = __ldg(&d.f_vel[j]);
        vel.x += vj.x * kc;
        vel.y += vj.y * kc;
        pr += (__ldg(&d.f_p[j]) - __ldg(&d.f_rho[j]) * (gx * dx.x + gy * dx.y)) * kc;
        if (d2 < nearest) {
            phase = __ldg(&d.f_phase[j]);
            nearest = d2;
        }
    });
    float2 v;
    float pv;
    if (sum != 0.0f) {
        v = make_float2(vel.x / sum, vel.y / sum);
        pv = pr / sum;
    } else {
        v = make_float2(0.f, 0.f);
        pv = 0.f;
    }
    const int bt = d.v_bt[i];
    if (bt == SPHNJ_SLIP) {
        const float2 nn = d.v_normal[i];
        const float t = 2.0f * dot2(v, nn);
        v = make_float2(v.x - t * nn.x, v.y - t * nn.y);
    } else if (bt == SPHNJ_NO_SLIP) {
        v = make_float2(-v.x, -v.y);
    }
    if (nearest == LARGE_FLOAT) phase = SPHNJ_LIQUID;
    d.v_vel[i] = v;
    d.v_p[i] = pv;
    d.v_phase[i] = (uint8_t)phase;
    // pressureToDensity, fluid.cu:6-13
    d.v_rho[i] = by_phase(p.reference_density, phase) *
                 powf(pv * by_phase(p.coefficient_p2rho, phase) + 1.0f, by_phase(p.gamma_inv, phase));
}

template <class G, class F> __global__ void __launch_bounds__(kBlock) k_solid_couple(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.solid_number) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const Frame fr{0, 0};
    const float2 x_i = F::s_home(p, d, fr, i);
    float2 nrm = make_float2(0.f, 0.f);
    float pr = 0.f, sum = 0.f;
    // fluid and solid neighbours feed separate sums, each in stencil order
    const int c = d.s_cell[i];
    for_each_in_stencil<F::kMixed>(d.rng_f, c, nx, ny, [&](int t, int n) {
        const int j = __ldg(&d.lst_f[t]);
        const float2 dx = sub2(F::f_nbr(d, j, F::shift(p, fr, n)), x_i);
        if (!(sqn(dx) < R2)) return;
        const float kc = sw(p, sqn(dx) * hinv2);
        sum += kc;
        pr += __ldg(&d.f_p[j]) * kc;
    });
    for_each_in_stencil<F::kMixed>(d.rng_s, c, nx, ny, [&](int t, int n) {
        const int j = __ldg(&d.lst_s[t]);
        const float2 dx = sub2(F::s_nbr(d, j, F::shift(p, fr, n)), x_i);
        if (!(sqn(dx) < R2)) return;
        const float kc = gw(p, sqn(dx) * hinv2);
        nrm.x -= dx.x * kc;
        nrm.y -= dx.y * kc;
    });
    d.s_normal[i] = sqrtf(sqn(nrm)) < EPS_FOR_SUM ? make_float2(0.f, 0.f) : normalized(nrm);
    d.s_p[i] = sum != 0.0f ? fmaxf(pr / sum, p.min_pressure) : 0.0f;
}

// ---- stress (solid.cu:80-167) ---------------------------------------------
__device__ double plastic_elastic(const sphnj_params &p, double strain, double &max_strain) {
    const float modulus = p.auxetic_modulus, yield_stress = p.yield_stress;
    const float harden_strain = p.harden_strain, harden_coef = p.harden_coef;
    const double ts = strain > -0.5 ? sqrt(1.0 + 2.0 * strain) - 1.0 : -1.0;
    if (ts > max_strain) return modulus * (ts - max_strain) - yield_stress;
    if (ts > -harden_strain) {
        if (max_strain > ts && p.plastic_type == SPHNJ_PLASTIC) max_strain = ts;
        return -yield_stress;
    }
    if (max_strain > ts && p.plastic_type == SPHNJ_PLASTIC) max_strain = ts;
    const double dd = fabs(-harden_strain - ts);
    return -(harden_coef * (dd * dd) + yield_stress);
}

__device__ dmat2 green(const dmat2 &F) {
    const dmat2 ftf = dmul(dtrans(F), F);
    return {0.5 * (ftf.m00 - 1.0), 0.5 * (ftf.m10 - 0.0), 0.5 * (ftf.m01 - 0.0), 0.5 * (ftf.m11 - 1.0)};
}

// g: the Green strain of F
__device__ dmat2 auxetic_stress(const sphnj_params &p, const dmat2 &F, const dmat2 &g, dmat2 &max_strain) {
    const double mid = 0.5 * (g.m00 + g.m11);
    const double df = g.m00 - g.m11;
    const double rad = sqrt(0.25 * (df * df) + g.m01 * g.m10);
    const double alpha = 0.5 * atan2(g.m01 + g.m10, g.m00 - g.m11);
    double sa, ca;
    sincos(alpha, &sa, &ca);
    const dmat2 rot = {ca, sa, -sa, ca};
    const dmat2 rinv = dinv(rot);
    dmat2 msp = dmul(dmul(rinv, max_strain), rot);
    dmat2 ps = {0.0, 0.0, 0.0, 0.0};
    ps.m00 = plastic_elastic(p, mid + rad, msp.m00);
    ps.m11 = plastic_elastic(p, mid - rad, msp.m11);
    max_strain = dmul(dmul(rot, msp), rinv);
    return dmul(dmul(dmul(F, rot), ps), rinv);
}

__device__ dmat2 linear_stress(const sphnj_params &p, const dmat2 &F, const dmat2 &g) {
    const double lambda = p.lambda, nu = p.nu;
    const double a = 2.0 * nu, b = lambda * (g.m00 + g.m11);
    const dmat2 S = {a * g.m00 + b * 1.0, a * g.m10 + b * 0.0, a * g.m01 + b * 0.0, a * g.m11 + b * 1.0};
    return dmul(F, S);
}

__device__ __forceinline__ float ref_q2(const sphnj_params &p, double2 dref) {
    return __double2float_rn((dref.x * dref.x + dref.y * dref.y) * (double)p.smoothing_length_inverse_square);
}
__device__ __forceinline__ bool ref_within(const sphnj_params &p, double2 dref) {
    return __double2float_rn(dref.x * dref.x + dref.y * dref.y) < p.impact_distance_square;
}

template <class G> __global__ void __launch_bounds__(kBlock) k_solid_deform(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.solid_number) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    dmat2 L = {0, 0, 0, 0}, Ft = {0, 0, 0, 0};
    const double2 xr_i = d.s_ref[i], x_i = d.s_pos[i];
    for_each_in_stencil<false>(d.rng_s, d.s_cell[i], nx, ny, [&](int t, int) {
        const int j = __ldg(&d.lst_s[t]);
        const double2 xr_j = d.s_ref[j];
        const double2 dref = make_double2(xr_j.x - xr_i.x, xr_j.y - xr_i.y);
        if (!ref_within(p, dref)) return;
        const double2 x_j = d.s_pos[j];
        const double2 dx = make_double2(x_j.x - x_i.x, x_j.y - x_i.y);
        const double kc = (double)gw(p, ref_q2(p, dref));
        Ft.m00 += dx.x * dref.x * kc;
        Ft.m10 += dx.y * dref.x * kc;
        Ft.m01 += dx.x * dref.y * kc;
        Ft.m11 += dx.y * dref.y * kc;
        L.m00 += dref.x * dref.x * kc;
        L.m10 += dref.y * dref.x * kc;
        L.m01 += dref.x * dref.y * kc;
        L.m11 += dref.y * dref.y * kc;
    });
    if (ddet(L) != 0.0) L = dinv(L);
    else L = {1.0, 0.0, 0.0, 1.0};
    const dmat2 F = dmul(Ft, L);
    d.s_F[i] = F;
    dmat2 ms = d.s_maxstrain[i];
    const int mat = d.s_mat[i];
    dmat2 P = {0, 0, 0, 0};
    if (mat == SPHNJ_AUXETIC) {
        P = auxetic_stress(p, F, green(F), ms);
        d.s_maxstrain[i] = ms;
    } else if (mat == SPHNJ_LINEAR_ELASTIC) {
        P = linear_stress(p, F, green(F));
    }
    d.s_P[i] = P;
    d.s_L[i] = L;
}

template <class G> __global__ void __launch_bounds__(kBlock) k_solid_force(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.solid_number) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const float alpha = p.artificial_viscosity[0], beta = p.artificial_viscosity[1];
    const float eps = 0.01f * p.smoothing_length_square;
    const float cs_s = p.solid_sound_speed, hs = p.smoothing_length;
    const double2 x_id = d.s_pos[i], v_id = d.s_vel[i], xr_i = d.s_ref[i];
    const float2 x_i = to_f2(x_id), u_i = to_f2(v_id);
    const float rho_ref = d.s_mat[i] == SPHNJ_AUXETIC ? p.auxetic_density : p.solid_reference_density;
    const double rho_ref_d = (double)rho_ref;
    const dmat2 F_i = d.s_F[i], L_i = d.s_L[i];
    const dmat2 PL_i = dmul(d.s_P[i], L_i);
    const float p_i = d.s_p[i];
    float2 couple = make_float2(0.f, 0.f);
    double2 acc = make_double2(0.0, 0.0);
    // fluid (couple) and solid (acc) neighbours feed separate sums, each in
    // stencil order
    const int c = d.s_cell[i];
    for_each_in_stencil<false>(d.rng_f, c, nx, ny, [&](int t, int) {  // solidFluidCouple, solid.cu:211-255
        const int j = __ldg(&d.lst_f[t]);
        const float2 dx = sub2(__ldg(&d.f_pos[j]), x_i);
        if (!(sqn(dx) < R2)) return;
        const float kc = gw(p, sqn(dx) * hinv2);
        const float p_j = __ldg(&d.f_p[j]);
        const float cs = by_phase(p.sound_speed, __ldg(&d.f_phase[j]));
        const float rho_j = __ldg(&d.f_rho[j]), rho_i = rho_j;
        const float2 u_j = __ldg(&d.f_vel[j]);
        float ps = fdiv(rho_i * p_j + rho_j * p_i, rho_i + rho_j);
        float2 nn = sqn(dx) > 0.f ? make_float2(fdiv(dx.x, sqrtf(sqn(dx))), fdiv(dx.y, sqrtf(sqn(dx)))) : dx;
        const float du = dot2(sub2(u_i, u_j), nn);
        if (du >= 0.0f) ps += fdiv(rho_i * rho_j * du, rho_i + rho_j) * fminf(3.0f * du, cs);
        const float am = fdiv(-2.0f * ps, rho_ref);
        couple.x += am * dx.x * kc;
        couple.y += am * dx.y * kc;
    });
    for_each_in_stencil<false>(d.rng_s, c, nx, ny, [&](int t, int) {  // solidSolidForce, solid.cu:257-305
        const int j = __ldg(&d.lst_s[t]);
        const double2 xr_j = d.s_ref[j];
        const double2 dref = make_double2(xr_j.x - xr_i.x, xr_j.y - xr_i.y);
        if (!ref_within(p, dref)) return;
        const double kc = (double)gw(p, ref_q2(p, dref));
        const dmat2 PL = dmul(d.s_P[j], d.s_L[j]);
        const dmat2 M = {PL.m00 + PL_i.m00, PL.m10 + PL_i.m10, PL.m01 + PL_i.m01, PL.m11 + PL_i.m11};
        const double2 tv = dmv(M, dref);
        acc.x += tv.x * kc / rho_ref_d;
        acc.y += tv.y * kc / rho_ref_d;
        const double2 x_j = d.s_pos[j], v_j = d.s_vel[j];
        const double2 dx = make_double2(x_j.x - x_id.x, x_j.y - x_id.y);
        const double2 dv = make_double2(v_j.x - v_id.x, v_j.y - v_id.y);
        const float dvdx = __double2float_rn(dv.x * dx.x + dv.y * dx.y);
        const float dis2 = __double2float_rn(dx.x * dx.x + dx.y * dx.y);
        const float nuv = hs * dvdx / (dis2 + eps);
        float visc = alpha * nuv * cs_s;
        visc -= beta * nuv * nuv;
        const double vd = (double)visc;
        const dmat2 Fv = {F_i.m00 * vd, F_i.m10 * vd, F_i.m01 * vd, F_i.m11 * vd};
        const double2 w = dmv(dmul(Fv, L_i), dref);
        acc.x += w.x * kc;
        acc.y += w.y * kc;
    });
    d.s_couple[i] = couple;
    d.s_dudt[i] = make_double2(acc.x + (double)couple.x, acc.y + (double)couple.y);
}

template <class G> __global__ void __launch_bounds__(256) k_solid_update(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.solid_number) return;
    const double dt = (double)(p.dt / (float)p.solid_sub_step);
    const int bt = d.s_bt[i];
    double2 x = d.s_pos[i], v = d.s_vel[i];
    if (bt == SPHNJ_FIXED) {
        v = make_double2(p.fixed_speed[0], p.fixed_speed[1]);
        x.x += v.x * dt;
        x.y += v.y * dt;
        d.s_dudt[i] = make_double2(0.0, 0.0);
    } else if (bt == SPHNJ_UNCONSTRAINED) {
        double2 a = d.s_dudt[i];
        if (p.transient_type == SPHNJ_STEADY) {
            a.x += -0.1 * v.x;
            a.y += -0.1 * v.y;
            d.s_dudt[i] = a;
        }
        x.x += v.x * dt;
        x.y += v.y * dt;
        v.x += (a.x + (double)p.gravity[0]) * dt;
        v.y += (a.y + (double)p.gravity[1]) * dt;
    }
    d.s_pos[i] = x;
    d.s_vel[i] = v;
    if (!(finite2(x) && finite2(v))) raise_error(d.err, SPHNJ_ERR_NONFINITE, KS, i);
}

// ---- mixed form -------------------------------------------------------------
// Reference separation X_j - X_i from reference cells + FP32 offsets.
__device__ __forceinline__ float2 ref_delta(const sphnj_params &p, int2 rc_i, float2 ro_i, int2 rc_j, float2 ro_j) {
    return make_float2(__fmaf_rn((float)(rc_j.x - rc_i.x), p.interval[0], ro_j.x - ro_i.x),
                       __fmaf_rn((float)(rc_j.y - rc_i.y), p.interval[1], ro_j.y - ro_i.y));
}

__device__ __forceinline__ float4 to_f4(const dmat2 &a) {
    return make_float4((float)a.m00, (float)a.m10, (float)a.m01, (float)a.m11);
}

// solidDeformationCalculate (solid.cu:169-209) in displacement form.  The
// pair loop sums in FP32, over the same neighbours as the plain form
// (current-position stencil, reference-distance filter),
//   H~ = sum (u_j - u_i) (x) dX W'   and   M = sum dX (x) dX W';
// then in FP64: L = M^-1, H = H~ L, F = I + H (the plain form's F~ L, since
// F~ = M + H~), the Green strain E = (H + H^T + H^T H) / 2 without the
// cancellation of F^T F - I, and the PK1 stress.  P L and F L are stored in
// FP32 for the force loop.
template <class G> __global__ void __launch_bounds__(kBlock) k_solid_deform_mixed(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.solid_number) return;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const int2 rc_i = d.s_rc[i];
    const float2 ro_i = d.s_roff[i], u_i = d.s_u[i];
    float h00 = 0.f, h10 = 0.f, h01 = 0.f, h11 = 0.f, m00 = 0.f, m10 = 0.f, m01 = 0.f, m11 = 0.f;
    const int ns = p.solid_number;
    int listed = 0;  // the neighbours that pass, recorded for the force pass
    for_each_in_stencil<false>(d.rng_s, d.s_cell[i], nx, ny, [&](int t, int) {
        const int j = __ldg(&d.lst_s[t]);
        const float2 dX = ref_delta(p, rc_i, ro_i, __ldg(&d.s_rc[j]), __ldg(&d.s_roff[j]));
        const float q = sqn(dX);
        if (!(q < R2)) return;
        if (listed < kSolidNbrCap) d.s_nbr[(size_t)listed * ns + i] = j;
        ++listed;
        const float kc = gw(p, q * hinv2);
        const float2 du = sub2(__ldg(&d.s_u[j]), u_i);
        const float ax = dX.x * kc, ay = dX.y * kc;
        h00 += du.x * ax;
        h10 += du.y * ax;
        h01 += du.x * ay;
        h11 += du.y * ay;
        m00 += dX.x * ax;
        m10 += dX.y * ax;
        m01 += dX.x * ay;
        m11 += dX.y * ay;
    });
    d.s_nbr_cnt[i] = listed <= kSolidNbrCap ? (uint8_t)listed : kNbrNone;
    const dmat2 M = {m00, m10, m01, m11};
    const dmat2 L = ddet(M) != 0.0 ? dinv(M) : dmat2{1.0, 0.0, 0.0, 1.0};
    const dmat2 H = dmul(dmat2{h00, h10, h01, h11}, L);
    const dmat2 F = {1.0 + H.m00, H.m10, H.m01, 1.0 + H.m11};
    const dmat2 HtH = dmul(dtrans(H), H);
    const dmat2 E = {0.5 * (2.0 * H.m00 + HtH.m00), 0.5 * (H.m10 + H.m01 + HtH.m10),
                     0.5 * (H.m01 + H.m10 + HtH.m01), 0.5 * (2.0 * H.m11 + HtH.m11)};
    dmat2 ms = d.s_maxstrain[i];
    const int mat = d.s_mat[i];
    dmat2 P = {0, 0, 0, 0};
    if (mat == SPHNJ_AUXETIC) {
        P = auxetic_stress(p, F, E, ms);
        d.s_maxstrain[i] = ms;
    } else if (mat == SPHNJ_LINEAR_ELASTIC) {
        P = linear_stress(p, F, E);
    }
    d.s_F[i] = F;
    d.s_P[i] = P;
    d.s_L[i] = L;
    d.s_PL[i] = to_f4(dmul(P, L));
    d.s_FL[i] = to_f4(dmul(F, L));
}

// solidForceCalculate (solid.cu:211-353), FP32: the stress divergence from
// the stored P L, the artificial viscosity with dx = dX + du, and the fluid
// coupling in the solid particle's cell frame.
template <class G> __global__ void __launch_bounds__(kBlock) k_solid_force_mixed(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.solid_number) return;
    using F = FormMixed;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square, hinv2 = p.smoothing_length_inverse_square;
    const float alpha = p.artificial_viscosity[0], beta = p.artificial_viscosity[1];
    const float eps = 0.01f * p.smoothing_length_square;
    const float cs_s = p.solid_sound_speed, hs = p.smoothing_length;
    const Frame fr{0, 0};
    const float2 x_i = F::s_home(p, d, fr, i);
    const float2 v_i = d.s_v[i], u_i = d.s_u[i], ro_i = d.s_roff[i];
    const int2 rc_i = d.s_rc[i];
    const float rho_ref = d.s_mat[i] == SPHNJ_AUXETIC ? p.auxetic_density : p.solid_reference_density;
    const float rinv = 1.0f / rho_ref;
    const float4 PL_i = d.s_PL[i], FL_i = d.s_FL[i];
    const float p_i = d.s_p[i];
    float2 couple = make_float2(0.f, 0.f), acc = make_float2(0.f, 0.f);
    // fluid (couple) and solid (acc) neighbours feed separate sums, each in
    // stencil order
    const int c = d.s_cell[i];
    for_each_in_stencil<true>(d.rng_f, c, nx, ny, [&](int t, int n) {  // solidFluidCouple, solid.cu:211-255
        const int j = __ldg(&d.lst_f[t]);
        const float2 dx = sub2(F::f_nbr(d, j, F::shift(p, fr, n)), x_i);
        if (!(sqn(dx) < R2)) return;
        const float kc = gw(p, sqn(dx) * hinv2);
        const float p_j = __ldg(&d.f_p[j]);
        const float cs = by_phase(p.sound_speed, __ldg(&d.f_phase[j]));
        const float rho_j = __ldg(&d.f_rho[j]), rho_f = rho_j;
        const float2 u_j = __ldg(&d.f_vel[j]);
        float ps = fdiv(rho_f * p_j + rho_j * p_i, rho_f + rho_j);
        float2 nn = sqn(dx) > 0.f ? make_float2(fdiv(dx.x, sqrtf(sqn(dx))), fdiv(dx.y, sqrtf(sqn(dx)))) : dx;
        const float du = dot2(sub2(v_i, u_j), nn);
        if (du >= 0.0f) ps += fdiv(rho_f * rho_j * du, rho_f + rho_j) * fminf(3.0f * du, cs);
        const float am = fdiv(-2.0f * ps, rho_ref);
        couple.x += am * dx.x * kc;
        couple.y += am * dx.y * kc;
    });
    auto solid_pair = [&](int j) {  // solidSolidForce, solid.cu:257-305
        const float2 dX = ref_delta(p, rc_i, ro_i, __ldg(&d.s_rc[j]), __ldg(&d.s_roff[j]));
        const float q = sqn(dX);
        if (!(q < R2)) return;
        const float kc = gw(p, q * hinv2);
        const float4 PL_j = __ldg(&d.s_PL[j]);
        const float4 M = make_float4(PL_j.x + PL_i.x, PL_j.y + PL_i.y, PL_j.z + PL_i.z, PL_j.w + PL_i.w);
        const float kr = kc * rinv;
        acc.x += sum2(M.x, dX.x, M.z, dX.y) * kr;
        acc.y += sum2(M.y, dX.x, M.w, dX.y) * kr;
        const float2 dx = add2(dX, sub2(__ldg(&d.s_u[j]), u_i));
        const float2 dv = sub2(__ldg(&d.s_v[j]), v_i);
        const float nuv = hs * dot2(dv, dx) / (sqn(dx) + eps);
        const float visc = sum2(alpha * nuv, cs_s, -beta * nuv, nuv) * kc;
        acc.x += sum2(FL_i.x, dX.x, FL_i.z, dX.y) * visc;
        acc.y += sum2(FL_i.y, dX.x, FL_i.w, dX.y) * visc;
    };
    // The solid neighbours this sub-step's deformation pass accepted, in its
    // (stencil) order: each thread loops over its own ~40 rather than testing
    // ~117 candidates with most lanes masked off; the cutoff test repeats on
    // the same inputs, so the sum is the stencil walk's.
    const int listed = d.s_nbr_cnt[i];
    if (listed != kNbrNone) {
        const int ns = p.solid_number;
        for (int k = 0; k < listed; ++k) solid_pair(__ldg(&d.s_nbr[(size_t)k * ns + i]));
    } else {
        for_each_in_stencil<false>(d.rng_s, c, nx, ny, [&](int t, int) { solid_pair(__ldg(&d.lst_s[t])); });
    }
    d.s_couple[i] = couple;
    d.s_acc[i] = add2(acc, couple);
}

// solidUpdate (solid.cu:446-471): displacement and velocity integrated with
// Kahan compensation over the sub-step dt / k.
template <class G> __global__ void __launch_bounds__(256) k_solid_update_mixed(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i >= p.solid_number) return;
    const float dt = p.dt / (float)p.solid_sub_step;
    const int bt = d.s_bt[i];
    float2 u = d.s_u[i], uc = d.s_uc[i], v = d.s_v[i], vc = d.s_vc[i];
    if (bt == SPHNJ_FIXED) {
        v = make_float2((float)p.fixed_speed[0], (float)p.fixed_speed[1]);
        vc = make_float2(0.f, 0.f);
        kahan_add2(u, uc, make_float2(v.x * dt, v.y * dt));
        d.s_acc[i] = make_float2(0.f, 0.f);
    } else if (bt == SPHNJ_UNCONSTRAINED) {
        float2 a = d.s_acc[i];
        if (p.transient_type == SPHNJ_STEADY) {
            a.x += -0.1f * v.x;
            a.y += -0.1f * v.y;
            d.s_acc[i] = a;
        }
        kahan_add2(u, uc, make_float2(v.x * dt, v.y * dt));
        kahan_add2(v, vc, make_float2((a.x + p.gravity[0]) * dt, (a.y + p.gravity[1]) * dt));
    }
    d.s_u[i] = u;
    d.s_uc[i] = uc;
    d.s_v[i] = v;
    d.s_vc[i] = vc;
    if (!(finite2(u) && finite2(v))) raise_error(d.err, SPHNJ_ERR_NONFINITE, KS, i);
    d.s_off[i] = solid_offset(p, d.s_rc[i], d.s_roff[i], u, d.s_cell[i]);
}

}  // namespace


template <class G> int launch_virt_normal(cudaStream_t st, G &g) {
    const int n = launch_virt_index(st, g);
    return n + launch(
                   g, site_key(SITE_VIRT_NORMAL), [](const Scene &s) { return grid_for(s.p.virt_number, kBlock); },
                   k_virt_normal<typename G::Dev>, kBlock, 0, st);
}
template <class G> int launch_virt_data(cudaStream_t st, G &g) {
    using D = typename G::Dev;
    auto blocks = [](const Scene &s) { return grid_for(s.p.virt_number, kBlock); };
    return g.form == SPHNJ_FORM_MIXED
               ? launch(g, site_key(SITE_VIRT_DATA), blocks, k_virt_data<D, FormMixed>, kBlock, 0, st)
               : launch(g, site_key(SITE_VIRT_DATA), blocks, k_virt_data<D, FormPlain>, kBlock, 0, st);
}
template <class G> int launch_solid_couple(cudaStream_t st, G &g) {
    using D = typename G::Dev;
    auto blocks = [](const Scene &s) { return s.p.fluid_number_total > 0 ? grid_for(s.p.solid_number, kBlock) : 0u; };
    return g.form == SPHNJ_FORM_MIXED
               ? launch(g, site_key(SITE_COUPLE), blocks, k_solid_couple<D, FormMixed>, kBlock, 0, st)
               : launch(g, site_key(SITE_COUPLE), blocks, k_solid_couple<D, FormPlain>, kBlock, 0, st);
}
// scenes with fewer solid sub-steps per fluid step own no block of sub-step `sub`
inline unsigned solid_blocks(const sphnj_params &p, int sub, int block) {
    return sub < p.solid_sub_step ? grid_for(p.solid_number, block) : 0u;
}
template <class G> int launch_solid_deformation(cudaStream_t st, G &g, int sub) {
    using D = typename G::Dev;
    auto blocks = [sub](const Scene &s) { return solid_blocks(s.p, sub, kBlock); };
    return g.form == SPHNJ_FORM_MIXED
               ? launch(g, site_key(SITE_SOLID_DEFORM, sub), blocks, k_solid_deform_mixed<D>, kBlock, 0, st)
               : launch(g, site_key(SITE_SOLID_DEFORM, sub), blocks, k_solid_deform<D>, kBlock, 0, st);
}
template <class G> int launch_solid_force(cudaStream_t st, G &g, int sub) {
    using D = typename G::Dev;
    auto blocks = [sub](const Scene &s) { return solid_blocks(s.p, sub, kBlock); };
    return g.form == SPHNJ_FORM_MIXED
               ? launch(g, site_key(SITE_SOLID_FORCE, sub), blocks, k_solid_force_mixed<D>, kBlock, 0, st)
               : launch(g, site_key(SITE_SOLID_FORCE, sub), blocks, k_solid_force<D>, kBlock, 0, st);
}
template <class G> int launch_solid_update(cudaStream_t st, G &g, int sub) {
    using D = typename G::Dev;
    auto blocks = [sub](const Scene &s) { return solid_blocks(s.p, sub, 256); };
    return g.form == SPHNJ_FORM_MIXED
               ? launch(g, site_key(SITE_SOLID_UPDATE, sub), blocks, k_solid_update_mixed<D>, 256, 0, st)
               : launch(g, site_key(SITE_SOLID_UPDATE, sub), blocks, k_solid_update<D>, 256, 0, st);
}

SPHNJ_INSTANTIATE_GROUPS(launch_virt_normal);
SPHNJ_INSTANTIATE_GROUPS(launch_virt_data);
SPHNJ_INSTANTIATE_GROUPS(launch_solid_couple);
SPHNJ_INSTANTIATE_GROUPS(launch_solid_deformation, int);
SPHNJ_INSTANTIATE_GROUPS(launch_solid_force, int);
SPHNJ_INSTANTIATE_GROUPS(launch_solid_update, int);

}  // namespace sphnj
