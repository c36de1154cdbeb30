// Harness around the SPHNJ reference's own CUDA build - test infrastructure
// (it generates the golden fixtures and times the reference on the GPU).
//
// It links the reference's src/*.cu and src/*.cpp (everything except
// main.cu) and drives the reference's own stage functions in the order of
// DeviceCalculation::calculation (calculation.cu:28-43), skipping only the
// output calls (Output::outputData / outputGlobalData only read state).
// After chosen steps it dumps the reference's device state - every
// per-particle array, the Cell lists and the derived Parameter values - in a
// small binary format read by tests/golden/make_fixtures.py.
//
// usage (run directory prepared by oracle/ref/build_ref.py):
//   harness dump  <nsteps> <step,step,...> <out_prefix> [diag_every]
//   harness time  <warmup> <steps>
//   harness run   <global,global,...>
// `run` is DeviceCalculation::calculation (calculation.cu:20-48) with its
// outputs: per step Output::outputData, then the named global writers of
// output.cu ("default" = Output::outputGlobalData, or any of edge,
// total_force, wedge_disp, middle_position, end_position, tank_beam_end,
// total_energy, crush_force, von_mises_stress, mean_pressure), then the
// stages; a final outputData after the loop.  The reference's Windows paths
// ("..\\..\\out\\...") become file names containing backslashes in the run
// directory.
#include "calculation.cuh"
#include "function.cuh"
#include "output.cuh"
#include "memory_copy.cuh"
#include "sim.cuh"

#include "thrust/host_vector.h"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include <windows.h>

namespace {

struct Writer {
    FILE *f;
    int n = 0;
    std::vector<char> body;
    template <class T> void rec(const char *name, const char *dt, const T *data, int64_t count) {
        char nm[48] = {0}, ty[8] = {0};
        std::strncpy(nm, name, 47);
        std::strncpy(ty, dt, 7);
        body.insert(body.end(), nm, nm + 48);
        body.insert(body.end(), ty, ty + 8);
        const char *c = reinterpret_cast<const char *>(&count);
        body.insert(body.end(), c, c + 8);
        const char *d = reinterpret_cast<const char *>(data);
        body.insert(body.end(), d, d + count * (int64_t)sizeof(T));
        ++n;
    }
    void close(int step) {
        std::fwrite("SPHREF01", 1, 8, f);
        int32_t h[2] = {step, n};
        std::fwrite(h, 4, 2, f);
        std::fwrite(body.data(), 1, body.size(), f);
        std::fclose(f);
    }
};

template <class E> std::vector<float> flat_f(const thrust::device_vector<E> &v, int w) {
    thrust::host_vector<E> h = v;
    std::vector<float> o(h.size() * w);
    for (size_t i = 0; i < h.size(); ++i)
        for (int k = 0; k < w; ++k) o[i * w + k] = h[i].v[k];
    return o;
}
template <class E> std::vector<double> flat_d(const thrust::device_vector<E> &v, int w) {
    thrust::host_vector<E> h = v;
    std::vector<double> o(h.size() * w);
    for (size_t i = 0; i < h.size(); ++i)
        for (int k = 0; k < w; ++k) o[i * w + k] = h[i].v[k];
    return o;
}
template <class T> std::vector<int32_t> ints(const thrust::device_vector<T> &v) {
    thrust::host_vector<T> h = v;
    std::vector<int32_t> o(h.size());
    for (size_t i = 0; i < h.size(); ++i) o[i] = (int32_t)h[i];
    return o;
}
template <class T> std::vector<T> plain(const thrust::device_vector<T> &v) {
    thrust::host_vector<T> h = v;
    return std::vector<T>(h.begin(), h.end());
}

void dump(Sim *sim, int step, const std::string &prefix) {
    char path[512];
    std::snprintf(path, sizeof path, "%s_%06d.bin", prefix.c_str(), step);
    Writer w{std::fopen(path, "wb")};
    if (!w.f) {
        std::perror(path);
        return;
    }
    Parameter &P = Sim::parameter;
    // derived parameters
    float pf[] = {P.kernel.smoothing_length_square, P.kernel.smoothing_length_inverse_square,
                  P.kernel.impact_distance_square, P.kernel.kernel_coefficient_1, P.kernel.kernel_coefficient_2,
                  P.kernel.kernel_differential, P.kernel.coefficient_3d_to_2d, P.domain.interval[0],
                  P.domain.interval[1], P.domain.interval_inv[0], P.domain.interval_inv[1],
                  P.fluid.coefficient_p2rho[0], P.fluid.coefficient_p2rho[1], P.fluid.coefficient_rho2p[0],
                  P.fluid.coefficient_rho2p[1], P.fluid.gamma_inv[0], P.fluid.gamma_inv[1], P.fluid.min_density[0],
                  P.fluid.min_density[1], P.solid.lambda, P.solid.nu, P.solid.bulk_modulus, P.solid.sound_speed,
                  P.time.dt, P.physics.gravity[1], P.fluid.reference_density_inverse[0],
                  P.fluid.reference_density_inverse[1]};
    w.rec("param_f", "f4", pf, (int64_t)(sizeof pf / sizeof pf[0]));
    int32_t pi[] = {P.domain.cell_number[0], P.domain.cell_number[1], P.domain.cell_number_total,
                    P.fluid.number_total, P.solid.number, P.virt.number, P.time.i};
    w.rec("param_i", "i4", pi, (int64_t)(sizeof pi / sizeof pi[0]));
    if (P.fluid.number_total > 0) {
        Fluid_List &F = sim->fluid_list;
        auto a = flat_f(F.position, 2); w.rec("fluid_position", "f4", a.data(), a.size());
        a = flat_f(F.velocity, 2); w.rec("fluid_velocity", "f4", a.data(), a.size());
        auto s = plain(F.density); w.rec("fluid_density", "f4", s.data(), s.size());
        s = plain(F.pressure); w.rec("fluid_pressure", "f4", s.data(), s.size());
        auto ii = ints(F.phase_type); w.rec("fluid_phase", "i4", ii.data(), ii.size());
        ii = ints(F.fluid_boundary_type); w.rec("fluid_boundary_type", "i4", ii.data(), ii.size());
        ii = ints(F.has_near_particle); w.rec("fluid_has_near_particle", "i4", ii.data(), ii.size());
        ii = ints(F.cell_id); w.rec("fluid_cell_id", "i4", ii.data(), ii.size());
        a = flat_f(F.du_dx, 4); w.rec("fluid_du_dx", "f4", a.data(), a.size());
        a = flat_f(F.gradient, 2); w.rec("fluid_gradient", "f4", a.data(), a.size());
        a = flat_f(F.du_dt, 2); w.rec("fluid_du_dt", "f4", a.data(), a.size());
        s = plain(F.color); w.rec("fluid_color", "f4", s.data(), s.size());
        s = plain(F.drho_dt); w.rec("fluid_drho_dt", "f4", s.data(), s.size());
    }
    if (P.solid.number > 0) {
        Solid_List &S = sim->solid_list;
        auto d = flat_d(S.position, 2); w.rec("solid_position", "f8", d.data(), d.size());
        d = flat_d(S.reference_position, 2); w.rec("solid_reference_position", "f8", d.data(), d.size());
        d = flat_d(S.velocity, 2); w.rec("solid_velocity", "f8", d.data(), d.size());
        auto ii = ints(S.boundary_type); w.rec("solid_boundary_type", "i4", ii.data(), ii.size());
        ii = ints(S.material_type); w.rec("solid_material_type", "i4", ii.data(), ii.size());
        ii = ints(S.cell_id); w.rec("solid_cell_id", "i4", ii.data(), ii.size());
        d = flat_d(S.max_strain, 4); w.rec("solid_max_strain", "f8", d.data(), d.size());
        auto s = plain(S.pressure); w.rec("solid_pressure", "f4", s.data(), s.size());
        d = flat_d(S.deformation, 4); w.rec("solid_deformation", "f8", d.data(), d.size());
        d = flat_d(S.stress_1st_piola, 4); w.rec("solid_stress_1st_piola", "f8", d.data(), d.size());
        d = flat_d(S.correction, 4); w.rec("solid_correction", "f8", d.data(), d.size());
        d = flat_d(S.du_dt, 2); w.rec("solid_du_dt", "f8", d.data(), d.size());
        auto a = flat_f(S.normal, 2); w.rec("solid_normal", "f4", a.data(), a.size());
        a = flat_f(S.couple_dudt, 2); w.rec("solid_couple_dudt", "f4", a.data(), a.size());
    }
    if (P.virt.number > 0) {
        Virtual_List &V = sim->virt_list;
        auto a = flat_f(V.position, 2); w.rec("virt_position", "f4", a.data(), a.size());
        a = flat_f(V.normal, 2); w.rec("virt_normal", "f4", a.data(), a.size());
        a = flat_f(V.velocity, 2); w.rec("virt_velocity", "f4", a.data(), a.size());
        auto s = plain(V.pressure); w.rec("virt_pressure", "f4", s.data(), s.size());
        s = plain(V.density); w.rec("virt_density", "f4", s.data(), s.size());
        auto ii = ints(V.phase_type); w.rec("virt_phase", "i4", ii.data(), ii.size());
        ii = ints(V.boundary_type); w.rec("virt_boundary_type", "i4", ii.data(), ii.size());
        ii = ints(V.cell_id); w.rec("virt_cell_id", "i4", ii.data(), ii.size());
    }
    // cell lists: per cell the three counts, then the concatenated lists
    thrust::host_vector<Cell> cells = sim->cell_list;
    const int C = (int)cells.size();
    std::vector<int32_t> cnt(3 * (size_t)C), lf, ls, lv;
    for (int c = 0; c < C; ++c) {
        const Cell &x = cells[c];
        cnt[3 * c] = x.fluid_num;
        cnt[3 * c + 1] = x.solid_num;
        cnt[3 * c + 2] = x.virt_num;
        int k = 0;
        for (int q = 0; q < x.fluid_num && k < CELL_SIZE; ++q) lf.push_back(x.particle_list[k++]);
        for (int q = 0; q < x.solid_num && k < CELL_SIZE; ++q) ls.push_back(x.particle_list[k++]);
        for (int q = 0; q < x.virt_num && k < CELL_SIZE; ++q) lv.push_back(x.particle_list[k++]);
    }
    w.rec("cell_counts", "i4", cnt.data(), cnt.size());
    w.rec("cell_list_fluid", "i4", lf.data(), lf.size());
    w.rec("cell_list_solid", "i4", ls.data(), ls.size());
    w.rec("cell_list_virt", "i4", lv.data(), lv.size());
    w.close(step);
}

// Global diagnostics, in double from the device state (definitions shared
// with sphnj_gb300.diagnostics):
//   front   max x over liquid particles + d/2          (outputEdge, output.cu:339-352)
//   mom     sum m v,  m = rho0[phase] d^2 (constant particle mass)
//   ek      sum m |v|^2 / 2 over fluid
//   rho_sum sum rho d^2
//   tip     position - reference position of the solid particle with the
//           largest reference x (ties: closest to the mean reference y)
//   eks     sum rho_s d^2 |v|^2 / 2 over solid
//   eps     sum (lambda/2 tr(E)^2 + mu E:E) d^2, E = (F^T F - I)/2
//           (outputTotalEnergy, output.cu:426-455)
void diag_line(Sim *sim, int step, FILE *f) {
    Parameter &P = Sim::parameter;
    const double d2 = (double)P.kernel.particle_diameter * P.kernel.particle_diameter;
    double front = -1e300, mx = 0, my = 0, ek = 0, rs = 0;
    if (P.fluid.number_total > 0) {
        thrust::host_vector<Eigen::Vector2f> x = sim->fluid_list.position, v = sim->fluid_list.velocity;
        thrust::host_vector<float> rho = sim->fluid_list.density;
        thrust::host_vector<PhaseType> ph = sim->fluid_list.phase_type;
        for (size_t i = 0; i < x.size(); ++i) {
            double m = (double)P.fluid.reference_density[ph[i]] * d2;
            if (ph[i] == LIQUID && x[i](0) > front) front = x[i](0);
            mx += m * v[i](0);
            my += m * v[i](1);
            ek += 0.5 * m * ((double)v[i](0) * v[i](0) + (double)v[i](1) * v[i](1));
            rs += (double)rho[i] * d2;
        }
        front += 0.5 * P.kernel.particle_diameter;
    }
    double tx = 0, ty = 0, eks = 0, eps = 0;
    if (P.solid.number > 0) {
        thrust::host_vector<Eigen::Vector2d> x = sim->solid_list.position, r = sim->solid_list.reference_position,
                                             v = sim->solid_list.velocity;
        thrust::host_vector<Eigen::Matrix2d> F = sim->solid_list.deformation;
        double ymean = 0;
        for (size_t i = 0; i < r.size(); ++i) ymean += r[i](1);
        ymean /= (double)r.size();
        size_t best = 0;
        for (size_t i = 1; i < r.size(); ++i) {
            if (r[i](0) > r[best](0) + 1e-12 ||
                (std::fabs(r[i](0) - r[best](0)) <= 1e-12 && std::fabs(r[i](1) - ymean) < std::fabs(r[best](1) - ymean)))
                best = i;
        }
        tx = x[best](0) - r[best](0);
        ty = x[best](1) - r[best](1);
        const double rho = P.solid.reference_density, lam = P.solid.lambda, mu = P.solid.nu;
        for (size_t i = 0; i < x.size(); ++i) {
            eks += 0.5 * rho * d2 * (v[i](0) * v[i](0) + v[i](1) * v[i](1));
            const Eigen::Matrix2d &Fi = F[i];
            double e00 = 0.5 * (Fi(0, 0) * Fi(0, 0) + Fi(1, 0) * Fi(1, 0) - 1.0);
            double e11 = 0.5 * (Fi(0, 1) * Fi(0, 1) + Fi(1, 1) * Fi(1, 1) - 1.0);
            double e01 = 0.5 * (Fi(0, 0) * Fi(0, 1) + Fi(1, 0) * Fi(1, 1));
            double tr = e00 + e11;
            eps += (0.5 * lam * tr * tr + mu * (e00 * e00 + e11 * e11 + 2.0 * e01 * e01)) * d2;
        }
    }
    std::fprintf(f, "%d %.12g %.12g %.12g %.12g %.12g %.12g %.12g %.12g %.12g\n", step, front, mx, my, ek, rs, tx, ty,
                 eks, eps);
}

// max |v| exactly as getMaxSpeed (fluid.cu:429-440)
float max_speed(Sim *sim) {
    thrust::host_vector<Eigen::Vector2f> v = sim->fluid_list.velocity;
    float m = 0.0f;
    for (auto fp : v)
        if (fp.norm() > m) m = fp.norm();
    float mc = std::min(Sim::parameter.fluid.sound_speed[0], Sim::parameter.fluid.sound_speed[1]);
    return std::min(m, 0.1f * mc);
}

void one_step(Sim *sim, float *ms) {
    SimTime *time = Sim::parameter.getTime();
    time->addStep();
    DeviceCalculation::particleCellUpdate();
    DeviceCalculation::sortParticle(sim);
    DeviceCalculation::fillCell();
    DeviceCalculation::coupleCalculation();
    DeviceCalculation::virtUpdate();
    DeviceCalculation::fluidCalculation();
    DeviceCalculation::solidCalculation(sim);
    if (ms && Sim::parameter.hasFluid()) *ms = max_speed(sim);
    DeviceCalculation::fluidCorrection(sim);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: harness dump|time ...\n");
        return 2;
    }
    std::string mode = argv[1];
    try {
        Sim::parameter.initiate();
        Sim *sim = new Sim;
        sim->initiate();
        Sim::data_pointer.initiate(sim->fluid_list, sim->solid_list, sim->virt_list, sim->cell_list);
        MemoryCopy::copyConstant();
        DeviceCalculation::virtNormalCalculation();
        if (mode == "dump") {
            int nsteps = std::atoi(argv[2]);
            std::set<int> steps;
            std::stringstream ss(argv[3]);
            std::string tok;
            while (std::getline(ss, tok, ','))
                if (!tok.empty()) steps.insert(std::atoi(tok.c_str()));
            std::string prefix = argv[4];
            const int diag_every = argc > 5 ? std::atoi(argv[5]) : 0;
            FILE *ms_log = std::fopen((prefix + "_maxspeed.txt").c_str(), "w");
            FILE *dg = diag_every > 0 ? std::fopen((prefix + "_diag.txt").c_str(), "w") : nullptr;
            if (steps.count(0)) dump(sim, 0, prefix);
            if (dg) diag_line(sim, 0, dg);
            for (int s = 1; s <= nsteps; ++s) {
                float ms = 0.0f;
                one_step(sim, &ms);
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) {
                    std::fprintf(stderr, "CUDA error at step %d: %s\n", s, cudaGetErrorString(e));
                    return 3;
                }
                if (ms_log && s <= 1000) std::fprintf(ms_log, "%d %.9g\n", s, ms);
                if (steps.count(s)) dump(sim, s, prefix);
                if (dg && s % diag_every == 0) diag_line(sim, s, dg);
            }
            if (ms_log) std::fclose(ms_log);
            if (dg) std::fclose(dg);
        } else if (mode == "run") {
            std::vector<std::string> globals;
            std::stringstream ss(argc > 2 ? argv[2] : "default");
            std::string tok;
            while (std::getline(ss, tok, ','))
                if (!tok.empty()) globals.push_back(tok);
            const std::string gpath = "..\\..\\out\\global";
            SimTime *time = Sim::parameter.getTime();
            while (time->addStep()) {
                Output::outputData(sim);
                CreateDirectory(gpath.c_str(), NULL);
                for (const std::string &g : globals) {
                    if (g == "default") Output::outputGlobalData(sim);
                    else if (g == "edge") Output::outputEdge(sim, gpath);
                    else if (g == "total_force") Output::outputTotalForce(sim, gpath);
                    else if (g == "wedge_disp") Output::outputWedgeDisp(sim, gpath);
                    else if (g == "middle_position") Output::outputMiddlePosition(sim, gpath);
                    else if (g == "end_position") Output::outputEndPosition(sim, gpath);
                    else if (g == "tank_beam_end") Output::outputTankBeamEnd(sim, gpath);
                    else if (g == "total_energy") Output::outputTotalEnergy(sim, gpath);
                    else if (g == "crush_force") Output::outputCrushForce(sim, gpath);
                    else if (g == "von_mises_stress") Output::outputVonMisesStress(sim, gpath);
                    else if (g == "mean_pressure") Output::outputMeanPressure(sim, gpath);
                    else {
                        std::fprintf(stderr, "unknown global writer %s\n", g.c_str());
                        return 2;
                    }
                }
                DeviceCalculation::particleCellUpdate();
                DeviceCalculation::sortParticle(sim);
                DeviceCalculation::fillCell();
                DeviceCalculation::coupleCalculation();
                DeviceCalculation::virtUpdate();
                DeviceCalculation::fluidCalculation();
                DeviceCalculation::solidCalculation(sim);
                DeviceCalculation::fluidCorrection(sim);
            }
            Output::outputData(sim);
        } else if (mode == "time") {
            int warm = std::atoi(argv[2]), steps = std::atoi(argv[3]);
            for (int s = 0; s < warm; ++s) one_step(sim, nullptr);
            cudaDeviceSynchronize();
            auto t0 = std::chrono::steady_clock::now();
            for (int s = 0; s < steps; ++s) one_step(sim, nullptr);
            cudaDeviceSynchronize();
            auto t1 = std::chrono::steady_clock::now();
            double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
            std::printf("{\"steps\": %d, \"ms_total\": %.3f, \"ms_per_step\": %.6f, \"n_fluid\": %d, \"n_solid\": %d, "
                        "\"n_virt\": %d}\n",
                        steps, ms, ms / steps, Sim::parameter.fluid.number_total, Sim::parameter.solid.number,
                        Sim::parameter.virt.number);
        }
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            std::fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(e));
            return 3;
        }
        delete sim;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
