// ORACLE - test infrastructure only.  A CPU restatement of SPHNJ's
// particle-step hot path, used by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py as the checker and the CPU baseline.  It is
// never linked into, loaded by, or called from libsphnj.
//
// Every stage follows the reference source line by line (file:line cited at
// each function).  Cell lists are kept in the reference's own fixed-capacity
// form (class Cell, include/cell.cuh:11-47: 9 neighbour ids, 64-slot current
// and previous lists), so that the GPU library's CSR reformulation is checked
// against an independent restatement of the original data structure.
//
// Precision: template parameter R is the type of fluid / virtual state and of
// the kernel weights; solid state is always double, as in the reference
// (include/particle.cuh:23-32,104-115).  R = float is the reference precision
// (the plain CPU baseline); R = double is the FP64 oracle.  Arithmetic is
// written in the evaluation order of the reference's Eigen expressions.
// Build with -ffp-contract=off so that results do not depend on the host
// (x86-64 and aarch64 give identical output).
//
// Parity pin: the reference publishes no test vectors; this restatement is
// pinned against state dumps of the reference's own CUDA build (see
// oracle/ref/ and tests/golden/).
#include "../include/sphnj.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

template <class T> struct V2 { T x, y; };
template <class T> struct M2 { T m00, m10, m01, m11; };  // column-major, Eigen layout

template <class T> static inline T sqn(V2<T> a) { return a.x * a.x + a.y * a.y; }
template <class T> static inline T dot(V2<T> a, V2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> static inline V2<T> sub(V2<T> a, V2<T> b) { return {a.x - b.x, a.y - b.y}; }
// Eigen normalized(): zero vector returned unchanged (Eigen 3.4 semantics)
template <class T> static inline V2<T> normalized(V2<T> a) {
    T z = sqn(a);
    if (z > T(0)) {
        T s = std::sqrt(z);
        return {a.x / s, a.y / s};
    }
    return a;
}
template <class T> static inline T vnorm(V2<T> a) { return std::sqrt(sqn(a)); }
template <class T> static inline M2<T> mmul(const M2<T> &a, const M2<T> &b) {
    return {a.m00 * b.m00 + a.m01 * b.m10, a.m10 * b.m00 + a.m11 * b.m10,
            a.m00 * b.m01 + a.m01 * b.m11, a.m10 * b.m01 + a.m11 * b.m11};
}
template <class T> static inline V2<T> mvec(const M2<T> &a, V2<T> v) {
    return {a.m00 * v.x + a.m01 * v.y, a.m10 * v.x + a.m11 * v.y};
}
template <class T> static inline M2<T> mtrans(const M2<T> &a) { return {a.m00, a.m01, a.m10, a.m11}; }
template <class T> static inline T mdet(const M2<T> &a) { return a.m00 * a.m11 - a.m10 * a.m01; }
// 2x2 inverse as adjugate times the reciprocal determinant
template <class T> static inline M2<T> minv(const M2<T> &a) {
    T inv = T(1) / mdet(a);
    return {a.m11 * inv, -a.m10 * inv, -a.m01 * inv, a.m00 * inv};
}
template <class T> static inline M2<T> mI() { return {T(1), T(0), T(0), T(1)}; }
template <class T> static inline M2<T> mZ() { return {T(0), T(0), T(0), T(0)}; }

static inline float fmaxf_(float a, float b) { return std::fmax(a, b); }
static inline double fmaxf_(double a, double b) { return std::fmax(a, b); }

constexpr int CELL_SIZE = 64;
constexpr float EPS_FOR_SUM = 0.1f;
constexpr float LARGE_FLOAT = 1.0E6f;

// class Cell, cell.cuh:11-47
struct Cell {
    int neighbor_cell_id[9];
    int fluid_num, solid_num, virt_num;
    int particle_list[CELL_SIZE];
    int fluid_num_previous, solid_num_previous, virt_num_previous;
    int particle_list_previous[CELL_SIZE];
    Cell() {
        for (int i = 0; i < 9; i++) neighbor_cell_id[i] = -1;
        fluid_num = solid_num = virt_num = 0;
        fluid_num_previous = solid_num_previous = virt_num_previous = 0;
        for (int i = 0; i < CELL_SIZE; i++) particle_list[i] = particle_list_previous[i] = -1;
    }
};

// Derived constants in precision R.  For R = float they are the exact
// float values of sphnj_params (reference precision).  For R = double they
// are re-derived in double from the same float inputs (FP64 oracle).
template <class R> struct Consts {
    R h, h2, h_inv2, R2, coef1, coef2, kdiff, c32;
    R rho0[2], rho0_inv[2], gamma[2], gamma_inv[2], p2rho[2], rho2p[2], cs[2], visc[2], min_density[2];
    R min_pressure, shift_coef, dt, g[2];
};

template <class R> static Consts<R> make_consts(const sphnj_params &p) {
    Consts<R> c;
    if (sizeof(R) == sizeof(float)) {
        c.h = p.smoothing_length;
        c.h2 = p.smoothing_length_square;
        c.h_inv2 = p.smoothing_length_inverse_square;
        c.R2 = p.impact_distance_square;
        c.coef1 = p.kernel_coefficient_1;
        c.coef2 = p.kernel_coefficient_2;
        c.kdiff = p.kernel_differential;
        c.c32 = p.coefficient_3d_to_2d;
        for (int i = 0; i < 2; ++i) {
            c.rho0[i] = p.reference_density[i];
            c.rho0_inv[i] = p.reference_density_inverse[i];
            c.gamma[i] = p.gamma[i];
            c.gamma_inv[i] = p.gamma_inv[i];
            c.p2rho[i] = p.coefficient_p2rho[i];
            c.rho2p[i] = p.coefficient_rho2p[i];
            c.min_density[i] = p.min_density[i];
        }
    } else {
        const double h = p.smoothing_length, d = p.particle_diameter, Rr = p.impact_length_hsml_ratio;
        c.h = h;
        c.h2 = h * h;
        c.h_inv2 = 1.0 / (h * h);
        c.R2 = Rr * Rr * h * h;
        c.coef1 = std::exp(-Rr * Rr);
        c.coef2 = 1.0 / 5.551921 * std::pow(h / d, -3.0);
        c.kdiff = 2.0 / 5.551921 * std::pow(h / d, -3.0) * std::pow(h, -2.0);
        c.c32 = 2.120729;
        for (int i = 0; i < 2; ++i) {
            c.rho0[i] = p.reference_density[i];
            c.rho0_inv[i] = 1.0 / (double)p.reference_density[i];
            c.gamma[i] = p.gamma[i];
            c.gamma_inv[i] = 1.0 / (double)p.gamma[i];
            c.p2rho[i] = (double)p.gamma[i] / ((double)p.sound_speed[i] * p.sound_speed[i]) / p.reference_density[i];
            c.rho2p[i] = 1.0 / (double)c.p2rho[i];
            c.min_density[i] = 0.6 * (double)p.reference_density[i];
        }
    }
    for (int i = 0; i < 2; ++i) {
        c.cs[i] = p.sound_speed[i];
        c.visc[i] = p.viscosity[i];
    }
    c.min_pressure = p.min_pressure;
    c.shift_coef = p.particle_shift_coef;
    c.dt = p.dt;
    c.g[0] = p.gravity[0];
    c.g[1] = p.gravity[1];
    return c;
}

struct Base {
    virtual ~Base() {}
    virtual int upload(const sphnj_host_state &) = 0;
    virtual int step(int n) = 0;
    virtual int download(uint32_t mask, sphnj_host_state &) = 0;
    virtual int cells(int type, int32_t *start, int32_t *count, int32_t *list, int32_t *n_listed) = 0;
    virtual float max_speed() const = 0;
    virtual int get_step() const = 0;
    virtual int error() const = 0;
    virtual int set_cells(const int32_t *cnt[3], const int32_t *lst[3]) = 0;
    virtual void set_step(int s) = 0;
};

template <class R> struct Sim : Base {
    typedef V2<R> VR;
    typedef M2<R> MR;
    typedef V2<double> VD;
    typedef M2<double> MD;

    sphnj_params p;
    Consts<R> k;
    int nf, ns, nv, C, nx, ny;
    int step_i;
    int err = SPHNJ_OK;
    float last_max_speed = 0.0f;

    // fluid (particle.cuh:20-32)
    std::vector<VR> f_pos, f_vel, f_grad, f_dudt;
    std::vector<R> f_rho, f_p, f_color, f_drho;
    std::vector<int> f_phase, f_fbt, f_near, f_cell;
    std::vector<MR> f_dudx;
    // solid (particle.cuh:101-116)
    std::vector<VD> s_pos, s_ref, s_vel, s_dudt;
    std::vector<int> s_bt, s_mat, s_cell;
    std::vector<MD> s_maxstrain, s_F, s_P, s_L;
    std::vector<R> s_p;
    std::vector<VR> s_normal, s_couple;
    // virtual (particle.cuh:184-192)
    std::vector<VR> v_pos, v_normal, v_vel;
    std::vector<R> v_p, v_rho;
    std::vector<int> v_phase, v_bt, v_cell;

    std::vector<Cell> cells_;

    explicit Sim(const sphnj_params &pp) : p(pp) {
        k = make_consts<R>(p);
        nf = p.fluid_number_total;
        ns = p.solid_number;
        nv = p.virt_number;
        nx = p.cell_number[0];
        ny = p.cell_number[1];
        C = p.cell_number_total;
        step_i = p.istart;
        create_cells();
    }

    // Sim::createCell, sim.cu:163-197
    void create_cells() {
        cells_.assign((size_t)C, Cell());
        for (int i = 0; i < nx; i++)
            for (int j = 0; j < ny; j++) {
                Cell &t = cells_[(size_t)i * ny + j];
                int id = i * ny + j;
                t.neighbor_cell_id[4] = id;
                if (i != 0) t.neighbor_cell_id[1] = id - ny;
                if (i != nx - 1) t.neighbor_cell_id[7] = id + ny;
                if (j != 0) t.neighbor_cell_id[3] = id - 1;
                if (j != ny - 1) t.neighbor_cell_id[5] = id + 1;
                if (i != 0 && j != 0) t.neighbor_cell_id[0] = id - 1 - ny;
                if (i != 0 && j != ny - 1) t.neighbor_cell_id[2] = id + 1 - ny;
                if (i != nx - 1 && j != 0) t.neighbor_cell_id[6] = id - 1 + ny;
                if (i != nx - 1 && j != ny - 1) t.neighbor_cell_id[8] = id + 1 + ny;
            }
    }

    int upload(const sphnj_host_state &s) override {
        // initial values of the host lists, host_data.cuh:24-115
        f_pos.assign(nf, VR{0, 0}); f_vel.assign(nf, VR{0, 0});
        f_rho.assign(nf, 0); f_p.assign(nf, 0); f_phase.assign(nf, 0);
        f_fbt.assign(nf, SPHNJ_FREE_SURFACE); f_near.assign(nf, SPHNJ_NO_PARTICLE);
        f_dudx.assign(nf, mZ<R>()); f_grad.assign(nf, VR{0, 0}); f_dudt.assign(nf, VR{0, 0});
        f_color.assign(nf, 0); f_drho.assign(nf, 0); f_cell.assign(nf, -1);
        for (int i = 0; i < nf; ++i) {
            if (s.fluid_position) f_pos[i] = {(R)s.fluid_position[2 * i], (R)s.fluid_position[2 * i + 1]};
            if (s.fluid_velocity) f_vel[i] = {(R)s.fluid_velocity[2 * i], (R)s.fluid_velocity[2 * i + 1]};
            if (s.fluid_density) f_rho[i] = s.fluid_density[i];
            if (s.fluid_pressure) f_p[i] = s.fluid_pressure[i];
            if (s.fluid_phase) f_phase[i] = s.fluid_phase[i];
            if (s.fluid_boundary_type) f_fbt[i] = s.fluid_boundary_type[i];
            if (s.fluid_has_near_particle) f_near[i] = s.fluid_has_near_particle[i];
            if (s.fluid_du_dx)
                f_dudx[i] = {(R)s.fluid_du_dx[4 * i], (R)s.fluid_du_dx[4 * i + 1], (R)s.fluid_du_dx[4 * i + 2],
                             (R)s.fluid_du_dx[4 * i + 3]};
            if (s.fluid_gradient) f_grad[i] = {(R)s.fluid_gradient[2 * i], (R)s.fluid_gradient[2 * i + 1]};
            if (s.fluid_du_dt) f_dudt[i] = {(R)s.fluid_du_dt[2 * i], (R)s.fluid_du_dt[2 * i + 1]};
            if (s.fluid_color) f_color[i] = s.fluid_color[i];
            if (s.fluid_drho_dt) f_drho[i] = s.fluid_drho_dt[i];
        }
        s_pos.assign(ns, VD{0, 0}); s_ref.assign(ns, VD{0, 0}); s_vel.assign(ns, VD{0, 0});
        s_dudt.assign(ns, VD{0, 0}); s_bt.assign(ns, 0); s_mat.assign(ns, 0); s_cell.assign(ns, -1);
        MD ms0 = {-(double)p.yield_strain, 0.0, 0.0, -(double)p.yield_strain};
        s_maxstrain.assign(ns, ms0);
        s_F.assign(ns, mI<double>()); s_P.assign(ns, mZ<double>()); s_L.assign(ns, mI<double>());
        s_p.assign(ns, 0); s_normal.assign(ns, VR{0, 0}); s_couple.assign(ns, VR{0, 0});
        for (int i = 0; i < ns; ++i) {
            if (s.solid_position) s_pos[i] = {s.solid_position[2 * i], s.solid_position[2 * i + 1]};
            if (s.solid_reference_position)
                s_ref[i] = {s.solid_reference_position[2 * i], s.solid_reference_position[2 * i + 1]};
            if (s.solid_velocity) s_vel[i] = {s.solid_velocity[2 * i], s.solid_velocity[2 * i + 1]};
            if (s.solid_boundary_type) s_bt[i] = s.solid_boundary_type[i];
            if (s.solid_material_type) s_mat[i] = s.solid_material_type[i];
            if (s.solid_max_strain)
                s_maxstrain[i] = {s.solid_max_strain[4 * i], s.solid_max_strain[4 * i + 1],
                                  s.solid_max_strain[4 * i + 2], s.solid_max_strain[4 * i + 3]};
            if (s.solid_pressure) s_p[i] = s.solid_pressure[i];
            if (s.solid_deformation)
                s_F[i] = {s.solid_deformation[4 * i], s.solid_deformation[4 * i + 1], s.solid_deformation[4 * i + 2],
                          s.solid_deformation[4 * i + 3]};
            if (s.solid_stress_1st_piola)
                s_P[i] = {s.solid_stress_1st_piola[4 * i], s.solid_stress_1st_piola[4 * i + 1],
                          s.solid_stress_1st_piola[4 * i + 2], s.solid_stress_1st_piola[4 * i + 3]};
            if (s.solid_correction)
                s_L[i] = {s.solid_correction[4 * i], s.solid_correction[4 * i + 1], s.solid_correction[4 * i + 2],
                          s.solid_correction[4 * i + 3]};
            if (s.solid_du_dt) s_dudt[i] = {s.solid_du_dt[2 * i], s.solid_du_dt[2 * i + 1]};
            if (s.solid_normal) s_normal[i] = {(R)s.solid_normal[2 * i], (R)s.solid_normal[2 * i + 1]};
            if (s.solid_couple_dudt) s_couple[i] = {(R)s.solid_couple_dudt[2 * i], (R)s.solid_couple_dudt[2 * i + 1]};
        }
        v_pos.assign(nv, VR{0, 0}); v_normal.assign(nv, VR{0, 0}); v_vel.assign(nv, VR{0, 0});
        v_p.assign(nv, 0); v_rho.assign(nv, (R)p.reference_density[0]); v_phase.assign(nv, SPHNJ_LIQUID);
        v_bt.assign(nv, 0); v_cell.assign(nv, -1);
        for (int i = 0; i < nv; ++i) {
            if (s.virt_position) v_pos[i] = {(R)s.virt_position[2 * i], (R)s.virt_position[2 * i + 1]};
            if (s.virt_normal) v_normal[i] = {(R)s.virt_normal[2 * i], (R)s.virt_normal[2 * i + 1]};
            if (s.virt_velocity) v_vel[i] = {(R)s.virt_velocity[2 * i], (R)s.virt_velocity[2 * i + 1]};
            if (s.virt_pressure) v_p[i] = s.virt_pressure[i];
            if (s.virt_density) v_rho[i] = s.virt_density[i];
            if (s.virt_phase) v_phase[i] = s.virt_phase[i];
            if (s.virt_boundary_type) v_bt[i] = s.virt_boundary_type[i];
        }
        create_cells();
        step_i = p.istart;
        err = SPHNJ_OK;
        if (!s.virt_normal && nv > 0) virt_normal_calculation();
        return SPHNJ_OK;
    }

    // ---- kernel weights (kernel.cpp:25-41) --------------------------------
    R grad_w(R q2) const { return std::exp(-q2) * k.kdiff * k.c32; }
    R shepard_w(R q2) const { return (std::exp(-q2) - k.coef1) * k.coef2 * k.c32; }

    // ---- EOS (fluid.cu:6-23) -------------------------------------------------
    R pressure_to_density(R pr, int ph) const {
        return k.rho0[ph] * std::pow(pr * k.p2rho[ph] + R(1), k.gamma_inv[ph]);
    }
    R density_to_pressure(R rho, int ph) const {
        R pr = (std::pow(rho * k.rho0_inv[ph], k.gamma[ph]) - R(1)) * k.rho2p[ph];
        return fmaxf_(pr, k.min_pressure);
    }

    // ---- getVirtNormal, virt.cu:8-59 (O(N_v^2), index order) ------------------
    void virt_normal_calculation() {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nv; ++i) {
            VR xi = v_pos[i];
            VR nrm = {0, 0};
            for (int j = 0; j < nv; ++j) {
                VR dx = sub(v_pos[j], xi);
                if (sqn(dx) < k.R2) {
                    R q2 = sqn(dx) * k.h_inv2;
                    R kc = grad_w(q2);
                    nrm.x -= dx.x * kc;
                    nrm.y -= dx.y * kc;
                }
            }
            if (vnorm(nrm) < (R)EPS_FOR_SUM) v_normal[i] = {0, 0};
            else v_normal[i] = normalized(nrm);
        }
    }

    // ---- findPositionCell, pair.cu:8-18 -------------------------------------
    // Float arithmetic on the float-cast position, truncation toward zero.
    int cell_of(float x, float y) const {
        return (int)((y - p.cell_xmin[1]) * p.interval_inv[1]) + (int)((x - p.cell_xmin[0]) * p.interval_inv[0]) * ny;
    }
    bool in_grid(int c) const { return c >= 0 && c < C; }

    // particleCellUpdate, pair.cu:20-64
    void particle_cell_update() {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nf; ++i) f_cell[i] = cell_of((float)f_pos[i].x, (float)f_pos[i].y);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < ns; ++i) s_cell[i] = cell_of((float)s_pos[i].x, (float)s_pos[i].y);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nv; ++i) v_cell[i] = cell_of((float)v_pos[i].x, (float)v_pos[i].y);
        for (int i = 0; i < nf; ++i) if (!in_grid(f_cell[i])) err = SPHNJ_ERR_OUT_OF_GRID;
        for (int i = 0; i < ns; ++i) if (!in_grid(s_cell[i])) err = SPHNJ_ERR_OUT_OF_GRID;
        for (int i = 0; i < nv; ++i) if (!in_grid(v_cell[i])) err = SPHNJ_ERR_OUT_OF_GRID;
    }

    // thrust::sort_by_key is a stable sort: permutation by (key, old index)
    static std::vector<int> stable_perm(const std::vector<int> &key) {
        std::vector<int> perm(key.size());
        std::iota(perm.begin(), perm.end(), 0);
        std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
        return perm;
    }
    template <class T> static void apply(std::vector<T> &v, const std::vector<int> &perm) {
        std::vector<T> t(v.size());
        for (size_t q = 0; q < perm.size(); ++q) t[q] = v[perm[q]];
        v.swap(t);
    }
    // reduce_by_key with constant 1 + exclusive_scan (sort.cu:15-19)
    static void runs(const std::vector<int> &key, std::vector<int> &ids, std::vector<int> &cnt, std::vector<int> &idx) {
        ids.clear(); cnt.clear(); idx.clear();
        for (size_t q = 0; q < key.size(); ++q) {
            if (ids.empty() || ids.back() != key[q]) { ids.push_back(key[q]); cnt.push_back(0); }
            cnt.back()++;
        }
        int acc = 0;
        for (size_t r = 0; r < cnt.size(); ++r) { idx.push_back(acc); acc += cnt[r]; }
    }

    // Fluid/Solid/Virtual_List::sort + updateCell, sort.cu:10-137
    void sort_particle() {
        std::vector<int> fid, fcnt, fidx, sid, scnt, sidx, vid, vcnt, vidx;
        if (nf > 0) {  // payload: position, velocity, density, pressure, phase, boundary type
            auto perm = stable_perm(f_cell);
            apply(f_pos, perm); apply(f_vel, perm); apply(f_rho, perm); apply(f_p, perm);
            apply(f_phase, perm); apply(f_fbt, perm); apply(f_cell, perm);
            runs(f_cell, fid, fcnt, fidx);
        }
        if (ns > 0) {  // payload: reference position, position, velocity, material, boundary (+ max_strain)
            auto perm = stable_perm(s_cell);
            apply(s_ref, perm); apply(s_pos, perm); apply(s_vel, perm); apply(s_mat, perm);
            apply(s_bt, perm); apply(s_maxstrain, perm); apply(s_cell, perm);
            runs(s_cell, sid, scnt, sidx);
        }
        if (nv > 0) {  // payload: position, normal, boundary type
            auto perm = stable_perm(v_cell);
            apply(v_pos, perm); apply(v_normal, perm); apply(v_bt, perm); apply(v_cell, perm);
            runs(v_cell, vid, vcnt, vidx);
        }
        // clearCellNumber, sort.cu:47-57
        for (auto &c : cells_) c.fluid_num = c.solid_num = c.virt_num = 0;
        // updateCellFluid/Solid/Virt, sort.cu:59-92 (the reference has no
        // bound check there; a cell past 64 entries corrupts memory, so the
        // restatement stops writing at 64 and reports the overflow)
        for (size_t r = 0; r < fid.size(); ++r) {
            if (!in_grid(fid[r])) continue;
            Cell &c = cells_[fid[r]];
            c.fluid_num = fcnt[r];
            for (int q = 0; q < fcnt[r]; ++q) {
                if (q >= CELL_SIZE) { err = SPHNJ_ERR_CELL_OVERFLOW; break; }
                c.particle_list[q] = fidx[r] + q;
            }
        }
        for (size_t r = 0; r < sid.size(); ++r) {
            if (!in_grid(sid[r])) continue;
            Cell &c = cells_[sid[r]];
            c.solid_num = scnt[r];
            for (int q = 0; q < scnt[r]; ++q) {
                if (q + c.fluid_num >= CELL_SIZE) { err = SPHNJ_ERR_CELL_OVERFLOW; break; }
                c.particle_list[q + c.fluid_num] = sidx[r] + q;
            }
        }
        for (size_t r = 0; r < vid.size(); ++r) {
            if (!in_grid(vid[r])) continue;
            Cell &c = cells_[vid[r]];
            c.virt_num = vcnt[r];
            for (int q = 0; q < vcnt[r]; ++q) {
                if (q + c.fluid_num + c.solid_num >= CELL_SIZE) { err = SPHNJ_ERR_CELL_OVERFLOW; break; }
                c.particle_list[q + c.fluid_num + c.solid_num] = vidx[r] + q;
            }
        }
    }

    // copyCellList + fillCellList, pair.cu:66-181
    void fill_cell() {
#pragma omp parallel for schedule(static)
        for (int id = 0; id < C; ++id) {
            Cell &c = cells_[id];
            c.fluid_num_previous = c.fluid_num;
            c.solid_num_previous = c.solid_num;
            c.virt_num_previous = c.virt_num;
            int tot = std::min(c.fluid_num + c.solid_num + c.virt_num, CELL_SIZE);
            for (int i = 0; i < tot; i++) c.particle_list_previous[i] = c.particle_list[i];
        }
        int overflow = 0;
#pragma omp parallel for schedule(static) reduction(| : overflow)
        for (int id = 0; id < C; ++id) overflow |= fill_cell_list(id);
        if (overflow) err = SPHNJ_ERR_CELL_OVERFLOW;
    }
    int fill_cell_list(int id) {
        Cell &ci = cells_[id];
        int fnum = 0, snum = 0, vnum = 0;
        for (int n = 0; n < 9; n++) {
            int nb = ci.neighbor_cell_id[n];
            if (nb == -1) continue;
            const Cell &cj = cells_[nb];
            for (int q = 0; q < cj.fluid_num_previous && q < CELL_SIZE; q++) {
                int pid = cj.particle_list_previous[q];
                if (f_cell[pid] == id) {
                    if (fnum >= CELL_SIZE) return 1;  // printf + return, pair.cu:90-93
                    ci.particle_list[fnum] = pid;
                    fnum++;
                }
            }
        }
        ci.fluid_num = fnum;
        for (int n = 0; n < 9; n++) {
            int nb = ci.neighbor_cell_id[n];
            if (nb == -1) continue;
            const Cell &cj = cells_[nb];
            int f0 = cj.fluid_num_previous, s0 = cj.solid_num_previous;
            for (int q = f0; q < f0 + s0 && q < CELL_SIZE; q++) {
                int pid = cj.particle_list_previous[q];
                if (s_cell[pid] == id) {
                    if (fnum + snum >= CELL_SIZE) return 1;
                    ci.particle_list[fnum + snum] = pid;
                    snum++;
                }
            }
        }
        ci.solid_num = snum;
        for (int n = 0; n < 9; n++) {
            int nb = ci.neighbor_cell_id[n];
            if (nb == -1) continue;
            const Cell &cj = cells_[nb];
            int f0 = cj.fluid_num_previous, s0 = cj.solid_num_previous, v0 = cj.virt_num_previous;
            for (int q = f0 + s0; q < f0 + s0 + v0 && q < CELL_SIZE; q++) {
                int pid = cj.particle_list_previous[q];
                if (v_cell[pid] == id) {
                    if (fnum + snum + vnum >= CELL_SIZE) return 1;
                    ci.particle_list[fnum + snum + vnum] = pid;
                    vnum++;
                }
            }
        }
        ci.virt_num = vnum;
        return 0;
    }

    // iteration helpers over the 3x3 stencil of the cell of a particle
    template <class F> void for_fluid(int cell, F f) const {
        const Cell &ci = cells_[cell];
        for (int n = 0; n < 9; ++n) {
            int nb = ci.neighbor_cell_id[n];
            if (nb == -1) continue;
            const Cell &cj = cells_[nb];
            for (int q = 0; q < cj.fluid_num && q < CELL_SIZE; ++q) f(cj.particle_list[q]);
        }
    }

    // ---- fluid pair functions, fluid.cu:25-191 --------------------------------
    struct Acc {
        R velo_div = 0, color = 0;
        VR du_dt{0, 0}, grad{0, 0};
        MR du_dx{0, 0, 0, 0};
        int near = SPHNJ_NO_PARTICLE;
    };

    // The Riemann pair term shared by the three neighbour kinds.
    void riemann(VR u_i, VR u_j, R p_i, R p_j, R rho_i, R rho_j, R cs, VR dx, R kc, Acc &a) const {
        R ps = (rho_i * p_j + rho_j * p_i) / (rho_i + rho_j);
        VR nrm = normalized(dx);
        R du = dot(sub(u_i, u_j), nrm);
        if (du >= R(0)) ps += rho_i * rho_j * du / (rho_i + rho_j) * std::fmin(R(3) * du, cs);
        VR vs = {(rho_i * u_i.x + rho_j * u_j.x) / (rho_i + rho_j), (rho_i * u_i.y + rho_j * u_j.y) / (rho_i + rho_j)};
        R t = (p_i - p_j) / (rho_i + rho_j) / cs;
        vs.x += t * nrm.x;
        vs.y += t * nrm.y;
        R am = R(-2) * ps / rho_i;
        a.du_dt.x += am * dx.x * kc;
        a.du_dt.y += am * dx.y * kc;
        a.velo_div += R(2) * rho_i * dot(sub(u_i, vs), dx) * kc;
        VR w = sub(u_j, u_i);
        a.du_dx.m00 += w.x * dx.x * kc;
        a.du_dx.m10 += w.y * dx.x * kc;
        a.du_dx.m01 += w.x * dx.y * kc;
        a.du_dx.m11 += w.y * dx.y * kc;
    }
    void viscous(VR u_i, VR u_j, R rho_i, int phase_i, VR dx, R kc, Acc &a) const {
        if (!p.is_fluid_viscid) return;
        R vis = dot(sub(u_j, u_i), dx);
        vis /= sqn(dx) + R(0.01f) * k.h2;
        R am = R(8) * k.visc[phase_i] * vis / rho_i;
        a.du_dt.x += am * dx.x * kc;
        a.du_dt.y += am * dx.y * kc;
    }

    // findFluidPair, fluid.cu:193-254
    void find_fluid_pair() {
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < nf; ++i) {
            Acc a;
            VR x_i = f_pos[i], u_i = f_vel[i];
            R p_i = f_p[i], rho_i = f_rho[i];
            int ph_i = f_phase[i];
            R cs = k.cs[ph_i];
            const Cell &ci = cells_[f_cell[i]];
            for (int n = 0; n < 9; ++n) {
                int nb = ci.neighbor_cell_id[n];
                if (nb == -1) continue;
                const Cell &cj = cells_[nb];
                int fn = cj.fluid_num, sn = cj.solid_num, vn = cj.virt_num;
                for (int q = 0; q < fn && q < CELL_SIZE; ++q) {
                    int j = cj.particle_list[q];
                    VR x_j = f_pos[j];
                    if (sqn(sub(x_j, x_i)) < k.R2) {  // fluidFluidCalculate, fluid.cu:25-80
                        VR dx = sub(x_j, x_i);
                        R kc = grad_w(sqn(dx) * k.h_inv2);
                        R rho_j = f_rho[j];
                        riemann(u_i, f_vel[j], p_i, f_p[j], rho_i, rho_j, cs, dx, kc, a);
                        int ph_j = f_phase[j];
                        if (!(ph_i == SPHNJ_LIQUID && ph_j == SPHNJ_GAS)) {
                            a.color += dot(dx, dx) * kc;
                            a.grad.x += dx.x * kc;
                            a.grad.y += dx.y * kc;
                        }
                        if (f_fbt[j] == SPHNJ_FREE_SURFACE && ph_i == SPHNJ_LIQUID && i != j) {
                            if (sqn(dx) < R(0.25f) * k.R2) a.near = SPHNJ_HAS_NEAR_PARTICLE;
                            else if (a.near == SPHNJ_NO_PARTICLE) a.near = SPHNJ_HAS_PARTICLE;
                        }
                        viscous(u_i, f_vel[j], rho_i, ph_i, dx, kc, a);
                    }
                }
                for (int q = fn; q < fn + sn && q < CELL_SIZE; ++q) {
                    int j = cj.particle_list[q];
                    VR x_j = {(R)(float)s_pos[j].x, (R)(float)s_pos[j].y};
                    if (sizeof(R) == sizeof(double)) x_j = {(R)s_pos[j].x, (R)s_pos[j].y};
                    if (sqn(sub(x_j, x_i)) < k.R2) {  // fluidSolidCalculate, fluid.cu:82-134
                        VR dx = sub(x_j, x_i);
                        VR u_j = {(R)(float)s_vel[j].x, (R)(float)s_vel[j].y};
                        if (sizeof(R) == sizeof(double)) u_j = {(R)s_vel[j].x, (R)s_vel[j].y};
                        R kc = grad_w(sqn(dx) * k.h_inv2);
                        riemann(u_i, u_j, p_i, s_p[j], rho_i, rho_i, cs, dx, kc, a);
                        a.grad.x += dx.x * kc;
                        a.grad.y += dx.y * kc;
                        viscous(u_i, u_j, rho_i, ph_i, dx, kc, a);
                    }
                }
                for (int q = fn + sn; q < fn + sn + vn && q < CELL_SIZE; ++q) {
                    int j = cj.particle_list[q];
                    VR x_j = v_pos[j];
                    if (sqn(sub(x_j, x_i)) < k.R2) {  // fluidVirtCalculate, fluid.cu:136-191
                        VR dx = sub(x_j, x_i);
                        R kc = grad_w(sqn(dx) * k.h_inv2);
                        R rho_j = k.rho0[v_phase[j]];
                        riemann(u_i, v_vel[j], p_i, v_p[j], rho_i, rho_j, cs, dx, kc, a);
                        // fluid.cu:179 reads the FLUID phase array with the
                        // virtual particle's index (quirk reproduced);
                        // beyond the fluid count the reference reads out of
                        // bounds - treated here as LIQUID.
                        int ph_j = j < nf ? f_phase[j] : SPHNJ_LIQUID;
                        if (!(ph_i == SPHNJ_LIQUID && ph_j == SPHNJ_GAS)) {
                            a.color += dot(dx, dx) * kc;
                            a.grad.x += dx.x * kc;
                            a.grad.y += dx.y * kc;
                        }
                        viscous(u_i, v_vel[j], rho_i, ph_i, dx, kc, a);
                    }
                }
            }
            f_drho[i] = a.velo_div;
            f_dudt[i] = a.du_dt;
            f_near[i] = a.near;
            f_color[i] = a.color;
            f_grad[i] = a.grad;
            f_dudx[i] = a.du_dx;
        }
    }

    // fluidUpdate, fluid.cu:256-287
    void fluid_update() {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nf; ++i) {
            int ph = f_phase[i];
            R dt = k.dt;
            if (p.transient_type == SPHNJ_STEADY) {
                f_dudt[i].x += R(-0.1f) * f_vel[i].x;
                f_dudt[i].y += R(-0.1f) * f_vel[i].y;
            }
            f_pos[i].x += f_vel[i].x * dt;
            f_pos[i].y += f_vel[i].y * dt;
            f_vel[i].x += (f_dudt[i].x + k.g[0]) * dt;
            f_vel[i].y += (f_dudt[i].y + k.g[1]) * dt;
            f_rho[i] += f_drho[i] * dt;
            f_rho[i] = fmaxf_(f_rho[i], k.min_density[ph]);
            f_p[i] = density_to_pressure(f_rho[i], ph);
            f_pos[i].x = fmaxf_(f_pos[i].x, (R)p.domain_xmin[0]);
            f_pos[i].x = std::fmin(f_pos[i].x, (R)p.domain_xmax[0]);
            f_pos[i].y = fmaxf_(f_pos[i].y, (R)p.domain_xmin[1]);
            f_pos[i].y = std::fmin(f_pos[i].y, (R)p.domain_xmax[1]);
        }
    }

    // getMaxSpeed, fluid.cu:429-440 (host loop over |v|)
    R get_max_speed() const {
        R ms = 0;
        for (int i = 0; i < nf; ++i) {
            R nrm = vnorm(f_vel[i]);
            if (nrm > ms) ms = nrm;
        }
        R mc = std::fmin((R)p.sound_speed[0], (R)p.sound_speed[1]);
        return std::fmin(ms, R(0.1f) * mc);
    }

    // correctionCalculate, fluid.cu:304-367
    void correction_calculate() {
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < nf; ++i) {
            VR x_i = f_pos[i];
            VR g = {0, 0};
            const Cell &ci = cells_[f_cell[i]];
            for (int n = 0; n < 9; ++n) {
                int nb = ci.neighbor_cell_id[n];
                if (nb == -1) continue;
                const Cell &cj = cells_[nb];
                int fn = cj.fluid_num, sn = cj.solid_num, vn = cj.virt_num;
                auto add = [&](VR x_j) {
                    if (sqn(sub(x_j, x_i)) < k.R2) {
                        VR dx = sub(x_j, x_i);
                        R kc = grad_w(sqn(dx) * k.h_inv2);
                        g.x += dx.x * kc;
                        g.y += dx.y * kc;
                    }
                };
                for (int q = 0; q < fn && q < CELL_SIZE; ++q) add(f_pos[cj.particle_list[q]]);
                for (int q = fn; q < fn + sn && q < CELL_SIZE; ++q) {
                    const VD &sp = s_pos[cj.particle_list[q]];
                    VR x_j = sizeof(R) == sizeof(double) ? VR{(R)sp.x, (R)sp.y} : VR{(R)(float)sp.x, (R)(float)sp.y};
                    add(x_j);
                }
                for (int q = fn + sn; q < fn + sn + vn && q < CELL_SIZE; ++q) add(v_pos[cj.particle_list[q]]);
            }
            f_grad[i] = g;
        }
    }

    // shiftDisplacementCalculate + correctionUpdate, fluid.cu:369-427
    VR project(VR g, VR disp) const {
        VR n = normalized(g);
        if (vnorm(n) < (R)EPS_FOR_SUM) n = {0, 0};
        MR m = {R(1) - n.x * n.x, R(0) - n.y * n.x, R(0) - n.x * n.y, R(1) - n.y * n.y};
        return mvec(m, disp);
    }
    void correction_update(R max_speed) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nf; ++i) {
            R s = -k.shift_coef * k.h * k.dt;
            VR disp = {s * f_grad[i].x, s * f_grad[i].y};
            VR d;
            if (f_phase[i] == SPHNJ_GAS) {
                f_fbt[i] = SPHNJ_INNER;
                d = disp;
            } else if (f_color[i] < R(1.5f)) {
                if (f_near[i] == SPHNJ_NO_PARTICLE) {
                    f_fbt[i] = SPHNJ_SPLASH;
                    d = {0, 0};
                } else {
                    f_fbt[i] = SPHNJ_FREE_SURFACE;
                    d = project(f_grad[i], disp);
                }
            } else if (f_color[i] < R(2.0f) && f_near[i] == SPHNJ_HAS_NEAR_PARTICLE) {
                f_fbt[i] = SPHNJ_VICINITY;
                d = project(f_grad[i], disp);
            } else {
                f_fbt[i] = SPHNJ_INNER;
                d = disp;
            }
            VR sh = {max_speed * d.x, max_speed * d.y};
            f_pos[i].x += sh.x;
            f_pos[i].y += sh.y;
            VR dv = mvec(f_dudx[i], sh);
            f_vel[i].x += dv.x;
            f_vel[i].y += dv.y;
        }
    }

    // getVirtData, virt.cu:61-149
    void virt_update() {
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < nv; ++i) {
            VR x_i = v_pos[i];
            VR vel = {0, 0};
            R pr = 0, sum = 0;
            R nearest = (R)LARGE_FLOAT;
            int phase = v_phase[i];
            R gx = k.g[0], gy = k.g[1];
            for_fluid(v_cell[i], [&](int j) {
                VR x_j = f_pos[j];
                if (sqn(sub(x_j, x_i)) < k.R2) {
                    VR dx = sub(x_j, x_i);
                    R kc = shepard_w(sqn(dx) * k.h_inv2);
                    sum += kc;
                    vel.x += f_vel[j].x * kc;
                    vel.y += f_vel[j].y * kc;
                    pr += (f_p[j] - f_rho[j] * (gx * dx.x + gy * dx.y)) * kc;
                    if (sqn(dx) < nearest) {
                        phase = f_phase[j];
                        nearest = sqn(dx);
                    }
                }
            });
            VR v;
            R pv;
            if (sum != R(0)) {
                v = {vel.x / sum, vel.y / sum};
                pv = pr / sum;
            } else {
                v = {0, 0};
                pv = 0;
            }
            VR n = v_normal[i];
            if (v_bt[i] == SPHNJ_SLIP) {
                R t = R(2) * dot(v, n);
                v = {v.x - t * n.x, v.y - t * n.y};
            } else if (v_bt[i] == SPHNJ_NO_SLIP) {
                v = {-v.x, -v.y};
            }
            if (nearest == (R)1.0e6) phase = SPHNJ_LIQUID;
            v_vel[i] = v;
            v_p[i] = pv;
            v_phase[i] = phase;
            v_rho[i] = pressure_to_density(pv, phase);
        }
    }

    // solidCoupleUpdate, solid.cu:355-444
    void solid_couple_update() {
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < ns; ++i) {
            VR x_i = sizeof(R) == sizeof(double) ? VR{(R)s_pos[i].x, (R)s_pos[i].y}
                                                 : VR{(R)(float)s_pos[i].x, (R)(float)s_pos[i].y};
            VR nrm = {0, 0};
            R pr = 0, sum = 0;
            const Cell &ci = cells_[s_cell[i]];
            for (int n = 0; n < 9; ++n) {
                int nb = ci.neighbor_cell_id[n];
                if (nb == -1) continue;
                const Cell &cj = cells_[nb];
                int fn = cj.fluid_num, sn = cj.solid_num;
                for (int q = 0; q < fn && q < CELL_SIZE; ++q) {
                    int j = cj.particle_list[q];
                    VR x_j = f_pos[j];
                    if (sqn(sub(x_j, x_i)) < k.R2) {
                        VR dx = sub(x_j, x_i);
                        R kc = shepard_w(sqn(dx) * k.h_inv2);
                        sum += kc;
                        pr += f_p[j] * kc;
                    }
                }
                for (int q = fn; q < fn + sn && q < CELL_SIZE; ++q) {
                    int j = cj.particle_list[q];
                    VR x_j = sizeof(R) == sizeof(double) ? VR{(R)s_pos[j].x, (R)s_pos[j].y}
                                                         : VR{(R)(float)s_pos[j].x, (R)(float)s_pos[j].y};
                    if (sqn(sub(x_j, x_i)) < k.R2) {
                        VR dx = sub(x_j, x_i);
                        R kc = grad_w(sqn(dx) * k.h_inv2);
                        nrm.x -= dx.x * kc;
                        nrm.y -= dx.y * kc;
                    }
                }
            }
            if (vnorm(nrm) < (R)EPS_FOR_SUM) s_normal[i] = {0, 0};
            else s_normal[i] = normalized(nrm);
            if (sum != R(0)) s_p[i] = fmaxf_(pr / sum, k.min_pressure);
            else s_p[i] = 0;
        }
    }

    // ---- solid stress, solid.cu:80-167 ---------------------------------------
    double plastic_elastic(double strain, double &max_strain) const {
        float modulus = p.auxetic_modulus, yield_stress = p.yield_stress;
        float harden_strain = p.harden_strain, harden_coef = p.harden_coef;
        double ts = strain > -0.5 ? std::sqrt(1.0 + 2.0 * strain) - 1.0 : -1.0;
        if (ts > max_strain) return modulus * (ts - max_strain) - yield_stress;
        if (ts > -harden_strain) {
            if (max_strain > ts && p.plastic_type == SPHNJ_PLASTIC) max_strain = ts;
            return -yield_stress;
        }
        if (max_strain > ts && p.plastic_type == SPHNJ_PLASTIC) max_strain = ts;
        return -(harden_coef * std::pow(std::fabs(-harden_strain - ts), 2.0) + yield_stress);
    }
    MD auxetic_stress(const MD &F, MD &max_strain) const {
        MD ftf = mmul(mtrans(F), F);
        MD g = {0.5 * (ftf.m00 - 1.0), 0.5 * (ftf.m10 - 0.0), 0.5 * (ftf.m01 - 0.0), 0.5 * (ftf.m11 - 1.0)};
        double mid = 0.5 * (g.m00 + g.m11);
        double rad = std::sqrt(0.25 * std::pow(g.m00 - g.m11, 2.0) + g.m01 * g.m10);
        double e0 = mid + rad, e1 = mid - rad;
        double alpha = 0.5 * std::atan2(g.m01 + g.m10, g.m00 - g.m11);
        MD rot = {std::cos(alpha), std::sin(alpha), -std::sin(alpha), std::cos(alpha)};
        MD rinv = minv(rot);
        MD msp = mmul(mmul(rinv, max_strain), rot);
        MD ps = mZ<double>();
        ps.m00 = plastic_elastic(e0, msp.m00);
        ps.m11 = plastic_elastic(e1, msp.m11);
        max_strain = mmul(mmul(rot, msp), rinv);
        return mmul(mmul(mmul(F, rot), ps), rinv);
    }
    MD linear_stress(const MD &F) const {
        double lambda = p.lambda, nu = p.nu;
        MD ftf = mmul(mtrans(F), F);
        MD g = {0.5 * (ftf.m00 - 1.0), 0.5 * (ftf.m10 - 0.0), 0.5 * (ftf.m01 - 0.0), 0.5 * (ftf.m11 - 1.0)};
        double a = 2.0 * nu;
        double b = lambda * (g.m00 + g.m11);
        MD S = {a * g.m00 + b * 1.0, a * g.m10 + b * 0.0, a * g.m01 + b * 0.0, a * g.m11 + b * 1.0};
        return mmul(F, S);
    }
    MD stress(const MD &F, MD &max_strain, int material) const {
        if (material == SPHNJ_AUXETIC) return auxetic_stress(F, max_strain);
        if (material == SPHNJ_LINEAR_ELASTIC) return linear_stress(F);
        return mZ<double>();
    }

    R ref_q2(VD dref) const {
        // `float q_2 = dx_ref.squaredNorm() * h_inv_2;` (double product, float result)
        if (sizeof(R) == sizeof(float)) return (R)(float)(sqn(dref) * (double)p.smoothing_length_inverse_square);
        return (R)(sqn(dref) * (double)k.h_inv2);
    }
    bool ref_within(VD dref) const {
        if (sizeof(R) == sizeof(float)) return (float)sqn(dref) < p.impact_distance_square;
        return sqn(dref) < (double)k.R2;
    }

    // solidDeformationCalculate, solid.cu:7-23,169-209
    void solid_deformation() {
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < ns; ++i) {
            MD L = mZ<double>(), Ft = mZ<double>();
            VD xr_i = s_ref[i];
            const Cell &ci = cells_[s_cell[i]];
            for (int n = 0; n < 9; ++n) {
                int nb = ci.neighbor_cell_id[n];
                if (nb == -1) continue;
                const Cell &cj = cells_[nb];
                int fn = cj.fluid_num, sn = cj.solid_num;
                for (int q = fn; q < fn + sn && q < CELL_SIZE; ++q) {
                    int j = cj.particle_list[q];
                    VD dref = sub(s_ref[j], xr_i);
                    if (!ref_within(dref)) continue;
                    VD dx = sub(s_pos[j], s_pos[i]);
                    double kc = (double)grad_w(ref_q2(dref));
                    Ft.m00 += dx.x * dref.x * kc; Ft.m10 += dx.y * dref.x * kc;
                    Ft.m01 += dx.x * dref.y * kc; Ft.m11 += dx.y * dref.y * kc;
                    L.m00 += dref.x * dref.x * kc; L.m10 += dref.y * dref.x * kc;
                    L.m01 += dref.x * dref.y * kc; L.m11 += dref.y * dref.y * kc;
                }
            }
            if (mdet(L) != 0.0) L = minv(L);
            else L = mI<double>();
            MD F = mmul(Ft, L);
            s_F[i] = F;
            s_P[i] = stress(F, s_maxstrain[i], s_mat[i]);
            s_L[i] = L;
        }
    }

    // solidForceCalculate, solid.cu:211-353
    void solid_force() {
        const float alpha = p.artificial_viscosity[0], beta = p.artificial_viscosity[1];
        const float eps = 0.01f * p.smoothing_length_square;
        const float cs_s = p.solid_sound_speed, hs = p.smoothing_length;
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < ns; ++i) {
            VR couple = {0, 0};
            VD acc = {0, 0};
            VR x_i = sizeof(R) == sizeof(double) ? VR{(R)s_pos[i].x, (R)s_pos[i].y}
                                                 : VR{(R)(float)s_pos[i].x, (R)(float)s_pos[i].y};
            VD xr_i = s_ref[i];
            double rho_ref = s_mat[i] == SPHNJ_AUXETIC ? (double)p.auxetic_density : (double)p.solid_reference_density;
            VR u_i = sizeof(R) == sizeof(double) ? VR{(R)s_vel[i].x, (R)s_vel[i].y}
                                                 : VR{(R)(float)s_vel[i].x, (R)(float)s_vel[i].y};
            MD PL_i = mmul(s_P[i], s_L[i]);
            const Cell &ci = cells_[s_cell[i]];
            for (int n = 0; n < 9; ++n) {
                int nb = ci.neighbor_cell_id[n];
                if (nb == -1) continue;
                const Cell &cj = cells_[nb];
                int fn = cj.fluid_num, sn = cj.solid_num;
                for (int q = 0; q < fn && q < CELL_SIZE; ++q) {  // solidFluidCouple, solid.cu:211-255
                    int j = cj.particle_list[q];
                    VR x_j = f_pos[j];
                    if (!(sqn(sub(x_j, x_i)) < k.R2)) continue;
                    VR dx = sub(x_j, x_i);
                    R kc = grad_w(sqn(dx) * k.h_inv2);
                    R p_i = s_p[i], p_j = f_p[j];
                    R cs = k.cs[f_phase[j]];
                    R rho_j = f_rho[j], rho_i = rho_j;
                    VR u_j = f_vel[j];
                    R ps = (rho_i * p_j + rho_j * p_i) / (rho_i + rho_j);
                    R du = dot(sub(u_i, u_j), normalized(dx));
                    if (du >= R(0)) ps += rho_i * rho_j * du / (rho_i + rho_j) * std::fmin(R(3) * du, cs);
                    R am = R(-2) * ps / (R)rho_ref;
                    couple.x += am * dx.x * kc;
                    couple.y += am * dx.y * kc;
                }
                for (int q = fn; q < fn + sn && q < CELL_SIZE; ++q) {  // solidSolidForce, solid.cu:257-305
                    int j = cj.particle_list[q];
                    VD dref = sub(s_ref[j], xr_i);
                    if (!ref_within(dref)) continue;
                    double kc = (double)grad_w(ref_q2(dref));
                    MD PL = mmul(s_P[j], s_L[j]);
                    MD M = {PL.m00 + PL_i.m00, PL.m10 + PL_i.m10, PL.m01 + PL_i.m01, PL.m11 + PL_i.m11};
                    VD t = mvec(M, dref);
                    acc.x += t.x * kc / rho_ref;
                    acc.y += t.y * kc / rho_ref;
                    VD dx = sub(s_pos[j], s_pos[i]);
                    VD dv = sub(s_vel[j], s_vel[i]);
                    if (sizeof(R) == sizeof(float)) {
                        float dvdx = (float)dot(dv, dx);
                        float dis2 = (float)sqn(dx);
                        float nuv = hs * dvdx / (dis2 + eps);
                        float visc = alpha * nuv * cs_s;
                        visc -= beta * nuv * nuv;
                        MD Fv = {s_F[i].m00 * visc, s_F[i].m10 * visc, s_F[i].m01 * visc, s_F[i].m11 * visc};
                        VD w = mvec(mmul(Fv, s_L[i]), dref);
                        acc.x += w.x * kc;
                        acc.y += w.y * kc;
                    } else {
                        double dvdx = dot(dv, dx);
                        double dis2 = sqn(dx);
                        double nuv = (double)hs * dvdx / (dis2 + 0.01 * (double)hs * hs);
                        double visc = (double)alpha * nuv * cs_s;
                        visc -= (double)beta * nuv * nuv;
                        MD Fv = {s_F[i].m00 * visc, s_F[i].m10 * visc, s_F[i].m01 * visc, s_F[i].m11 * visc};
                        VD w = mvec(mmul(Fv, s_L[i]), dref);
                        acc.x += w.x * kc;
                        acc.y += w.y * kc;
                    }
                }
            }
            s_couple[i] = couple;
            s_dudt[i] = {acc.x + (double)couple.x, acc.y + (double)couple.y};
        }
    }

    // solidUpdate, solid.cu:446-471
    void solid_update() {
        float dtf = p.dt / (float)p.solid_sub_step;
        double dt = sizeof(R) == sizeof(float) ? (double)dtf : (double)p.dt / (double)p.solid_sub_step;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < ns; ++i) {
            if (s_bt[i] == SPHNJ_FIXED) {
                s_vel[i] = {p.fixed_speed[0], p.fixed_speed[1]};
                s_pos[i].x += s_vel[i].x * dt;
                s_pos[i].y += s_vel[i].y * dt;
                s_dudt[i] = {0, 0};
            } else if (s_bt[i] == SPHNJ_UNCONSTRAINED) {
                if (p.transient_type == SPHNJ_STEADY) {
                    s_dudt[i].x += -0.1 * s_vel[i].x;
                    s_dudt[i].y += -0.1 * s_vel[i].y;
                }
                s_pos[i].x += s_vel[i].x * dt;
                s_pos[i].y += s_vel[i].y * dt;
                s_vel[i].x += (s_dudt[i].x + (double)p.gravity[0]) * dt;
                s_vel[i].y += (s_dudt[i].y + (double)p.gravity[1]) * dt;
            }
        }
    }

    // One iteration of the loop in DeviceCalculation::calculation,
    // calculation.cu:28-43 (outputs excluded: they only read state).
    void one_step() {
        step_i++;  // SimTime::addStep, sim_time.cpp:34-40
        particle_cell_update();
        if (err) return;
        if (!((step_i - 1) % p.sort_every_step)) sort_particle();  // SimTime::isSort
        fill_cell();
        if (err) return;
        if (nf > 0 && ns > 0) solid_couple_update();
        if (nv > 0) virt_update();
        if (nf > 0) {
            find_fluid_pair();
            fluid_update();
        }
        if (ns > 0)
            for (int s = 0; s < p.solid_sub_step; ++s) {
                solid_deformation();
                solid_force();
                solid_update();
            }
        if (nf > 0) {
            R ms = get_max_speed();
            last_max_speed = (float)ms;
            for (int s = 0; s < p.shift_per_step; ++s) {
                correction_calculate();
                correction_update(ms);
            }
        }
    }

    int step(int n) override {
        for (int s = 0; s < n; ++s) {
            if (err) return err;
            one_step();
        }
        return err;
    }

    int download(uint32_t mask, sphnj_host_state &s) override {
        if (mask & SPHNJ_F_FLUID_KINEMATICS)
            for (int i = 0; i < nf; ++i) {
                if (s.fluid_position) { s.fluid_position[2 * i] = (float)f_pos[i].x; s.fluid_position[2 * i + 1] = (float)f_pos[i].y; }
                if (s.fluid_velocity) { s.fluid_velocity[2 * i] = (float)f_vel[i].x; s.fluid_velocity[2 * i + 1] = (float)f_vel[i].y; }
            }
        if (mask & SPHNJ_F_FLUID_THERMO)
            for (int i = 0; i < nf; ++i) {
                if (s.fluid_density) s.fluid_density[i] = (float)f_rho[i];
                if (s.fluid_pressure) s.fluid_pressure[i] = (float)f_p[i];
                if (s.fluid_phase) s.fluid_phase[i] = f_phase[i];
            }
        if (mask & SPHNJ_F_FLUID_FLAGS)
            for (int i = 0; i < nf; ++i) {
                if (s.fluid_boundary_type) s.fluid_boundary_type[i] = f_fbt[i];
                if (s.fluid_has_near_particle) s.fluid_has_near_particle[i] = f_near[i];
            }
        if (mask & SPHNJ_F_FLUID_DERIVED)
            for (int i = 0; i < nf; ++i) {
                if (s.fluid_du_dx) {
                    s.fluid_du_dx[4 * i] = (float)f_dudx[i].m00; s.fluid_du_dx[4 * i + 1] = (float)f_dudx[i].m10;
                    s.fluid_du_dx[4 * i + 2] = (float)f_dudx[i].m01; s.fluid_du_dx[4 * i + 3] = (float)f_dudx[i].m11;
                }
                if (s.fluid_gradient) { s.fluid_gradient[2 * i] = (float)f_grad[i].x; s.fluid_gradient[2 * i + 1] = (float)f_grad[i].y; }
                if (s.fluid_du_dt) { s.fluid_du_dt[2 * i] = (float)f_dudt[i].x; s.fluid_du_dt[2 * i + 1] = (float)f_dudt[i].y; }
                if (s.fluid_color) s.fluid_color[i] = (float)f_color[i];
                if (s.fluid_drho_dt) s.fluid_drho_dt[i] = (float)f_drho[i];
            }
        if (mask & SPHNJ_F_SOLID_KINEMATICS)
            for (int i = 0; i < ns; ++i) {
                if (s.solid_position) { s.solid_position[2 * i] = s_pos[i].x; s.solid_position[2 * i + 1] = s_pos[i].y; }
                if (s.solid_reference_position) { s.solid_reference_position[2 * i] = s_ref[i].x; s.solid_reference_position[2 * i + 1] = s_ref[i].y; }
                if (s.solid_velocity) { s.solid_velocity[2 * i] = s_vel[i].x; s.solid_velocity[2 * i + 1] = s_vel[i].y; }
            }
        if (mask & SPHNJ_F_SOLID_MATERIAL)
            for (int i = 0; i < ns; ++i) {
                if (s.solid_boundary_type) s.solid_boundary_type[i] = s_bt[i];
                if (s.solid_material_type) s.solid_material_type[i] = s_mat[i];
                if (s.solid_max_strain) {
                    s.solid_max_strain[4 * i] = s_maxstrain[i].m00; s.solid_max_strain[4 * i + 1] = s_maxstrain[i].m10;
                    s.solid_max_strain[4 * i + 2] = s_maxstrain[i].m01; s.solid_max_strain[4 * i + 3] = s_maxstrain[i].m11;
                }
            }
        if (mask & SPHNJ_F_SOLID_DERIVED)
            for (int i = 0; i < ns; ++i) {
                if (s.solid_pressure) s.solid_pressure[i] = (float)s_p[i];
                auto put4 = [&](double *dst, const MD &m) {
                    if (!dst) return;
                    dst[4 * i] = m.m00; dst[4 * i + 1] = m.m10; dst[4 * i + 2] = m.m01; dst[4 * i + 3] = m.m11;
                };
                put4(s.solid_deformation, s_F[i]);
                put4(s.solid_stress_1st_piola, s_P[i]);
                put4(s.solid_correction, s_L[i]);
                if (s.solid_du_dt) { s.solid_du_dt[2 * i] = s_dudt[i].x; s.solid_du_dt[2 * i + 1] = s_dudt[i].y; }
                if (s.solid_normal) { s.solid_normal[2 * i] = (float)s_normal[i].x; s.solid_normal[2 * i + 1] = (float)s_normal[i].y; }
                if (s.solid_couple_dudt) { s.solid_couple_dudt[2 * i] = (float)s_couple[i].x; s.solid_couple_dudt[2 * i + 1] = (float)s_couple[i].y; }
            }
        if (mask & SPHNJ_F_VIRT)
            for (int i = 0; i < nv; ++i) {
                if (s.virt_position) { s.virt_position[2 * i] = (float)v_pos[i].x; s.virt_position[2 * i + 1] = (float)v_pos[i].y; }
                if (s.virt_normal) { s.virt_normal[2 * i] = (float)v_normal[i].x; s.virt_normal[2 * i + 1] = (float)v_normal[i].y; }
                if (s.virt_velocity) { s.virt_velocity[2 * i] = (float)v_vel[i].x; s.virt_velocity[2 * i + 1] = (float)v_vel[i].y; }
                if (s.virt_pressure) s.virt_pressure[i] = (float)v_p[i];
                if (s.virt_density) s.virt_density[i] = (float)v_rho[i];
                if (s.virt_phase) s.virt_phase[i] = v_phase[i];
                if (s.virt_boundary_type) s.virt_boundary_type[i] = v_bt[i];
            }
        if (mask & SPHNJ_F_CELL_IDS) {
            if (s.fluid_cell_id) for (int i = 0; i < nf; ++i) s.fluid_cell_id[i] = f_cell[i];
            if (s.solid_cell_id) for (int i = 0; i < ns; ++i) s.solid_cell_id[i] = s_cell[i];
            if (s.virt_cell_id) for (int i = 0; i < nv; ++i) s.virt_cell_id[i] = v_cell[i];
        }
        return SPHNJ_OK;
    }

    // Cell lists in canonical CSR form: start = exclusive prefix sum of the
    // per-cell counts in cell order, list = concatenation.
    int cells(int type, int32_t *start, int32_t *count, int32_t *list, int32_t *n_listed) override {
        int acc = 0;
        for (int c = 0; c < C; ++c) {
            const Cell &cl = cells_[c];
            int n = type == 0 ? cl.fluid_num : type == 1 ? cl.solid_num : cl.virt_num;
            int off = type == 0 ? 0 : type == 1 ? cl.fluid_num : cl.fluid_num + cl.solid_num;
            if (start) start[c] = acc;
            if (count) count[c] = n;
            if (list)
                for (int q = 0; q < n && off + q < CELL_SIZE; ++q) list[acc + q] = cl.particle_list[off + q];
            acc += n;
        }
        if (n_listed) *n_listed = acc;
        return SPHNJ_OK;
    }
    float max_speed() const override { return last_max_speed; }
    int get_step() const override { return step_i; }
    int error() const override { return err; }

    // Current lists from per-cell counts + concatenated lists (fluid ||
    // solid || virtual inside each Cell, as updateCell* lays them out).
    int set_cells(const int32_t *cnt[3], const int32_t *lst[3]) override {
        long off[3] = {0, 0, 0};
        for (int c = 0; c < C; ++c) {
            Cell &cl = cells_[c];
            int n[3];
            for (int k = 0; k < 3; ++k) n[k] = cnt[k] ? cnt[k][c] : 0;
            cl.fluid_num = n[0];
            cl.solid_num = n[1];
            cl.virt_num = n[2];
            int q = 0;
            for (int k = 0; k < 3; ++k)
                for (int t = 0; t < n[k]; ++t) {
                    if (q < CELL_SIZE) cl.particle_list[q] = lst[k][off[k] + t];
                    else err = SPHNJ_ERR_CELL_OVERFLOW;
                    ++q;
                }
            for (int k = 0; k < 3; ++k) off[k] += n[k];
        }
        return err;
    }
    void set_step(int s) override { step_i = s; }
};

}  // namespace oracle

struct oracle_ctx {
    oracle::Base *impl;
};

namespace oracle {

// key -> value of a flat ini text: '#' starts a comment, '[section]' lines
// carry no keys, a later key replaces an earlier one (Config, config.cpp:59-129
// and config.h:122-159, for the files this project writes).
struct Ini {
    std::vector<std::pair<std::string, std::string>> kv;
    explicit Ini(const char *text) {
        std::string all(text ? text : ""), line;
        size_t a = 0;
        while (a <= all.size()) {
            size_t b = all.find('\n', a);
            if (b == std::string::npos) b = all.size();
            line = all.substr(a, b - a);
            a = b + 1;
            const size_t hash = line.find('#');
            if (hash != std::string::npos) line.resize(hash);
            const size_t eq = line.find('=');
            if (eq == std::string::npos || line.find('[') != std::string::npos) continue;
            auto trim = [](std::string t) {
                const size_t f = t.find_first_not_of(" \t\r"), l = t.find_last_not_of(" \t\r");
                return f == std::string::npos ? std::string() : t.substr(f, l - f + 1);
            };
            const std::string k = trim(line.substr(0, eq)), v = trim(line.substr(eq + 1));
            if (!k.empty()) kv.emplace_back(k, v);
        }
    }
    const std::string *find(const char *key) const {
        for (auto it = kv.rbegin(); it != kv.rend(); ++it)
            if (it->first == key) return &it->second;
        return nullptr;
    }
    float f(const char *key, float dflt) const {
        const std::string *v = find(key);
        return v ? std::strtof(v->c_str(), nullptr) : dflt;
    }
    double d(const char *key, double dflt) const {
        const std::string *v = find(key);
        return v ? std::strtod(v->c_str(), nullptr) : dflt;
    }
    int i(const char *key, int dflt) const {
        const std::string *v = find(key);
        return v ? (int)std::strtol(v->c_str(), nullptr, 10) : dflt;
    }
    bool b(const char *key, bool dflt) const {
        const std::string *v = find(key);
        if (!v) return dflt;
        return *v == "true" || *v == "1" || *v == "yes" || *v == "on" || *v == "True" || *v == "TRUE";
    }
};

// Parameter::readParameter + Parameter::initiate in the reference's float
// arithmetic: the ini reads with their defaults (physics.cpp:12-17,
// properties.cpp:37-49,120-149, domain.cpp:10-18, sim_time.cpp:10-16,
// kernel.cpp:11-14) and the derived constants (properties.cpp:53-89,
// kernel.cpp:25-41 with the truncated-Gaussian constants of global.h:11-13,
// domain.cpp:37-49).
static int params_from_ini(const char *text, const int counts[4], sphnj_params *p) {
    const Ini c(text);
    std::memset(p, 0, sizeof *p);
    p->gravity[0] = 0.0f;
    p->gravity[1] = -c.f("gravity", 9.81f);
    p->transient_type = c.b("is_steady", false) ? SPHNJ_STEADY : SPHNJ_TRANSIENT;
    p->fluid_number[0] = counts[0];
    p->fluid_number[1] = counts[1];
    p->fluid_number_total = counts[0] + counts[1];
    p->solid_number = counts[2];
    p->virt_number = counts[3];
    p->particle_shift_coef = c.f("particle_shift_coef", 0.4f);
    p->is_fluid_viscid = c.b("is_viscid", false) ? 1 : 0;
    p->min_pressure = c.f("min_pressure", -1.013e5f);
    const char *phase[2] = {"liquid", "gas"};
    const float cs0[2] = {1500.0f, 340.0f}, rho0[2] = {1000.0f, 1.29f}, g0[2] = {7.0f, 1.4f},
                mu0[2] = {1.01e-3f, 17.9e-6f};
    for (int k = 0; k < 2; ++k) {
        const std::string pre(phase[k]);
        p->sound_speed[k] = c.f((pre + "_sound_speed").c_str(), cs0[k]);
        p->reference_density[k] = c.f((pre + "_density").c_str(), rho0[k]);
        p->gamma[k] = c.f((pre + "_gamma").c_str(), g0[k]);
        p->viscosity[k] = c.f((pre + "_viscosity").c_str(), mu0[k]);
        // FluidProperties::initiate
        p->coefficient_p2rho[k] = p->gamma[k] * powf(p->sound_speed[k], -2.0f) / p->reference_density[k];
        p->coefficient_rho2p[k] = 1.0f / p->coefficient_p2rho[k];
        p->gamma_inv[k] = 1.0f / p->gamma[k];
        p->reference_density_inverse[k] = 1.0f / p->reference_density[k];
        p->min_density[k] = (1.0f - 0.4f) * p->reference_density[k];
    }
    p->solid_reference_density = c.f("solid_density", 2700.0f);
    p->youngs_modulus = c.f("youngs_modulus", 67.5e9f);
    p->poisson_ratio = c.f("poisson_ratio", 0.34f);
    p->artificial_viscosity[0] = c.f("arti_vis_alpha", 2.5f);
    p->artificial_viscosity[1] = c.f("arti_vis_beta", 2.5f);
    p->fixed_speed[0] = c.d("solid_fixed_speed_x", 0.0);
    p->fixed_speed[1] = c.d("solid_fixed_speed_y", 0.0);
    p->constitution_type = c.b("is_2D_strain", false) ? SPHNJ_STRAIN_2D : SPHNJ_STRESS_2D;
    p->plastic_type = c.b("is_plastic", false) ? SPHNJ_PLASTIC : SPHNJ_HYPER_ELASTIC;
    p->auxetic_density = c.f("auxetic_density", 636.0f);
    p->auxetic_modulus = c.f("auxetic_modulus", 0.0f);
    p->auxetic_poisson_ratio = c.f("auxetic_poisson_ratio", -0.2f);
    p->yield_strain = c.f("yield_strain", 0.0f);
    p->yield_stress = c.f("yield_stress", 2.0e7f);
    p->harden_strain = c.f("harden_strain", 0.5f);
    p->harden_coef = c.f("harden_coef", 100.0f);
    // one of the auxetic modulus and the yield strain follows from the
    // other and the yield stress (properties.cpp:150-158)
    if (p->auxetic_modulus == 0.0f && p->yield_strain == 0.0f) return SPHNJ_ERR_CONFIG;
    if (p->yield_strain != 0.0f) p->auxetic_modulus = p->yield_stress / p->yield_strain;
    else p->yield_strain = p->yield_stress / p->auxetic_modulus;
    // SolidProperties::initiate
    const float E = p->youngs_modulus, nu = p->poisson_ratio, aE = p->auxetic_modulus, anu = p->auxetic_poisson_ratio;
    const bool strain = p->constitution_type == SPHNJ_STRAIN_2D;
    p->lambda = E * nu / (strain ? 1.0f - 2.0f * nu : 1.0f - nu) / (1.0f + nu);
    p->nu = E / (1.0f + nu) / 2.0f;
    p->auxetic_lambda = aE * anu / (strain ? 1.0f - 2.0f * anu : 1.0f - anu) / (1.0f + anu);
    p->auxetic_nu = aE / (1.0f + anu) / 2.0f;
    p->bulk_modulus = E / (3.0f * (1.0f - 2.0f * nu));
    p->solid_sound_speed = sqrtf(p->bulk_modulus / p->solid_reference_density);
    // Domain
    p->cell_xmin[0] = c.f("cell_xmin", 0.0f);
    p->cell_xmin[1] = c.f("cell_ymin", 0.0f);
    p->cell_xmax[0] = c.f("cell_xmax", 0.0f);
    p->cell_xmax[1] = c.f("cell_ymax", 0.0f);
    p->domain_xmin[0] = c.f("domain_xmin", 0.0f);
    p->domain_xmin[1] = c.f("domain_ymin", 0.0f);
    p->domain_xmax[0] = c.f("domain_xmax", 0.0f);
    p->domain_xmax[1] = c.f("domain_ymax", 0.0f);
    // SimTime
    p->dt = c.f("dt", 0.0f);
    p->istart = c.i("istart", 0);
    p->iend = c.i("iend", 0);
    p->solid_sub_step = c.i("solid_sub_step", 1);
    p->result_interval = c.i("result_interval", 1);
    p->sort_every_step = c.i("sort_every_step", 1);
    p->shift_per_step = c.i("shift_per_step", 1);
    // Kernel
    p->smoothing_length = c.f("smoothing_length", 0.0f);
    p->particle_diameter = c.f("particle_diameter", 0.0f);
    p->impact_length_hsml_ratio = c.f("impact_length_hsml_ratio", 3.0f);
    p->thread_num = c.i("thread_num", 32);
    const float h = p->smoothing_length, dd = p->particle_diameter, R = p->impact_length_hsml_ratio;
    if (h <= 0.0f || dd <= 0.0f) return SPHNJ_ERR_CONFIG;
    p->particle_volume = powf(dd, 3.0f);
    p->diameter_square = powf(dd, 2.0f);
    p->smoothing_length_square = powf(h, 2.0f);
    p->smoothing_length_inverse = 1.0f / h;
    p->smoothing_length_inverse_square = powf(p->smoothing_length_inverse, 2.0f);
    p->impact_distance_square = powf(R, 2.0f) * powf(h, 2.0f);
    const float tg2 = 5.551921f;  // global.h:12
    p->kernel_coefficient_1 = expf(-powf(R, 2.0f));
    p->kernel_coefficient_2 = 1.0f / tg2 * powf(h / dd, -3.0f);
    p->kernel_differential = 2.0f / tg2 * powf(h / dd, -3.0f) * powf(h, -2.0f);
    p->coefficient_3d_to_2d = 2.120729f;  // global.h:13
    for (int k = 0; k < 2; ++k) {
        const float span = p->cell_xmax[k] - p->cell_xmin[k];
        if (span == 0.0f) return SPHNJ_ERR_CONFIG;
        p->cell_number[k] = (int)(span / (R * h));
        p->interval[k] = span / (float)p->cell_number[k];
        p->interval_inv[k] = 1.0f / p->interval[k];
    }
    p->cell_number_total = p->cell_number[0] * p->cell_number[1];
    return SPHNJ_OK;
}

}  // namespace oracle

extern "C" {

// precision: 0 = reference precision (fluid FP32, solid FP64), 1 = FP64.
// threads: OpenMP threads (<= 0: library default).
int oracle_create(const sphnj_params *p, int precision, int threads, oracle_ctx **out) {
    if (!p || !out) return SPHNJ_ERR_ARG;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    oracle_ctx *c = new oracle_ctx;
    if (precision == 1) c->impl = new oracle::Sim<double>(*p);
    else c->impl = new oracle::Sim<float>(*p);
    *out = c;
    return SPHNJ_OK;
}
int oracle_upload(oracle_ctx *c, const sphnj_host_state *s) { return c && s ? c->impl->upload(*s) : SPHNJ_ERR_ARG; }
int oracle_step(oracle_ctx *c, int n) { return c ? c->impl->step(n) : SPHNJ_ERR_ARG; }
int oracle_download(oracle_ctx *c, uint32_t mask, sphnj_host_state *s) {
    return c && s ? c->impl->download(mask, *s) : SPHNJ_ERR_ARG;
}
int oracle_debug_cells(oracle_ctx *c, int type, int32_t *start, int32_t *count, int32_t *list, int32_t *n_listed) {
    return c ? c->impl->cells(type, start, count, list, n_listed) : SPHNJ_ERR_ARG;
}
int oracle_debug_max_speed(oracle_ctx *c, float *ms) {
    if (!c || !ms) return SPHNJ_ERR_ARG;
    *ms = c->impl->max_speed();
    return SPHNJ_OK;
}
int oracle_get_step(oracle_ctx *c, int *st) {
    if (!c || !st) return SPHNJ_ERR_ARG;
    *st = c->impl->get_step();
    return SPHNJ_OK;
}
int oracle_error(oracle_ctx *c) { return c ? c->impl->error() : SPHNJ_ERR_ARG; }
int oracle_debug_set_cells(oracle_ctx *c, const int32_t *cf, const int32_t *lf, const int32_t *cs,
                           const int32_t *ls, const int32_t *cv, const int32_t *lv) {
    if (!c) return SPHNJ_ERR_ARG;
    const int32_t *cnt[3] = {cf, cs, cv}, *lst[3] = {lf, ls, lv};
    return c->impl->set_cells(cnt, lst);
}
int oracle_debug_set_step(oracle_ctx *c, int s) {
    if (!c) return SPHNJ_ERR_ARG;
    c->impl->set_step(s);
    return SPHNJ_OK;
}
// Parameters of a case from its input.ini text and its particle counts
// (n_liquid, n_gas, n_solid, n_virt), derived by the oracle itself.
int oracle_params_from_ini(const char *ini_text, const int32_t *counts, sphnj_params *out) {
    if (!ini_text || !counts || !out) return SPHNJ_ERR_ARG;
    const int c[4] = {counts[0], counts[1], counts[2], counts[3]};
    return oracle::params_from_ini(ini_text, c, out);
}
int oracle_set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
    return omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}
int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void oracle_destroy(oracle_ctx *c) {
    if (!c) return;
    delete c->impl;
    delete c;
}

}  // extern "C"
