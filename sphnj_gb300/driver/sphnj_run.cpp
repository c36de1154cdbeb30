// sphnj_run: host driver for SPHNJ case directories on libsphnj.
//
// Drop-in for the reference's executable (main.cu:14-35 with the loop of
// calculation.cu:20-48): it reads CASE/config/input.ini and CASE/data/*.dat
// through the C ABI, runs steps istart+1 .. iend, and writes the reference's
// outputs into OUT (default CASE/out):
//   OUT/{fluid,solid,virtual}/<field>-<file_step>.vtk  every result_interval
//       steps, before the step's stages, as Output::outputData
//       (output.cu:7-281), fields and quirks included: fluid_density holds the
//       boundary type (-1 for gas), solid_velocity holds P(1,1) and the two
//       principal max strains, virt_pressure holds the phase;
//   OUT/global/*.dat  one line every --global-every steps (1 = every step, as
//       the reference), from sphnj_diagnostics (FP64 device reductions);
//   OUT/global/probe-<id>.dat  "x y vx vy p rho" per --probe point.
// VTK files are formatted on a background thread from a host copy of the
// state while the GPU continues stepping.  Numbers are written with the C++
// stream defaults (6 significant digits), as the reference writes them.
#include "sphnj.h"

#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace fs = std::filesystem;

namespace {

const char *kUsage =
    "usage: sphnj_run CASE_DIR [options]\n"
    "  --out DIR             output directory (default CASE_DIR/out)\n"
    "  --form plain|mixed    reference precision (default) or the mixed-precision form\n"
    "  --iend N              last step (default: the ini's iend)\n"
    "  --result-interval N   VTK output interval (default: the ini's result_interval)\n"
    "  --no-vtk              no VTK output\n"
    "  --global-every N      global data every N steps (default 1; 0 = none)\n"
    "  --global LIST         comma-separated global writers of output.cu: total_force,\n"
    "                        wedge_disp, von_mises_stress, mean_pressure (the four that\n"
    "                        Output::outputGlobalData calls: 'default'), edge (frontier.dat\n"
    "                        and height.dat), frontier, total_energy, end_position,\n"
    "                        middle_position, tank_beam_end, crush_force, and tip_disp\n"
    "                        (default: default)\n"
    "  --probe X,Y           a probe point (repeatable), written to global/probe-<id>.dat\n"
    "  --restart FILE        start from a checkpoint instead of the .dat files\n"
    "  --checkpoint-every N  write OUT/checkpoint-<step>.bin every N steps\n"
    "  --autotune STEPS      tune the sweep launch shape on the first STEPS steps' state\n"
    "  --quiet               no progress lines\n";

struct Args {
    std::string case_dir, out_dir, restart;
    int form = SPHNJ_FORM_PLAIN;
    long iend = -1, result_interval = -1, global_every = 1, checkpoint_every = 0, autotune = 0;
    bool vtk = true, quiet = false;
    std::vector<std::string> global = {"total_force", "wedge_disp", "von_mises_stress", "mean_pressure"};
    std::vector<std::pair<float, float>> probes;
};

[[noreturn]] void die(const std::string &m, int code = 1) {
    std::cerr << "sphnj_run: " << m << std::endl;
    std::exit(code);
}

long to_long(const char *s, const char *what) {
    char *end = nullptr;
    errno = 0;
    const long v = std::strtol(s, &end, 10);
    if (errno || !end || *end) die(std::string("bad ") + what + ": " + s, 2);
    return v;
}

Args parse(int argc, char **argv) {
    Args a;
    for (int k = 1; k < argc; ++k) {
        const std::string s = argv[k];
        auto next = [&](const char *what) -> const char * {
            if (k + 1 >= argc) die(std::string("missing value for ") + what, 2);
            return argv[++k];
        };
        if (s == "-h" || s == "--help") {
            std::cout << kUsage;
            std::exit(0);
        } else if (s == "--out") a.out_dir = next("--out");
        else if (s == "--form") {
            const std::string f = next("--form");
            if (f == "plain") a.form = SPHNJ_FORM_PLAIN;
            else if (f == "mixed") a.form = SPHNJ_FORM_MIXED;
            else die("--form must be plain or mixed", 2);
        } else if (s == "--iend") a.iend = to_long(next("--iend"), "--iend");
        else if (s == "--result-interval") a.result_interval = to_long(next(s.c_str()), "--result-interval");
        else if (s == "--no-vtk") a.vtk = false;
        else if (s == "--global-every") a.global_every = to_long(next(s.c_str()), "--global-every");
        else if (s == "--global") {
            a.global.clear();
            std::stringstream ss(next("--global"));
            std::string item;
            while (std::getline(ss, item, ',')) {
                if (item == "default")  // Output::outputGlobalData, output.cu:562-582
                    a.global.insert(a.global.end(), {"total_force", "wedge_disp", "von_mises_stress", "mean_pressure"});
                else if (item == "edge")  // outputEdge writes both files, output.cu:339-369
                    a.global.insert(a.global.end(), {"frontier", "height"});
                else if (!item.empty())
                    a.global.push_back(item);
            }
        } else if (s == "--probe") {
            float x, y;
            if (std::sscanf(next("--probe"), "%f,%f", &x, &y) != 2) die("--probe wants X,Y", 2);
            a.probes.emplace_back(x, y);
        } else if (s == "--restart") a.restart = next("--restart");
        else if (s == "--checkpoint-every") a.checkpoint_every = to_long(next(s.c_str()), "--checkpoint-every");
        else if (s == "--autotune") a.autotune = to_long(next("--autotune"), "--autotune");
        else if (s == "--quiet") a.quiet = true;
        else if (!s.empty() && s[0] == '-') die("unknown option " + s + "\n" + kUsage, 2);
        else if (a.case_dir.empty()) a.case_dir = s;
        else die("more than one case directory", 2);
    }
    if (a.case_dir.empty()) die(std::string("no case directory\n") + kUsage, 2);
    if (a.out_dir.empty()) a.out_dir = (fs::path(a.case_dir) / "out").string();
    static const char *known[] = {"total_force",     "wedge_disp",    "von_mises_stress", "mean_pressure",
                                  "frontier",        "height",        "total_energy",     "end_position",
                                  "middle_position", "tank_beam_end", "crush_force",      "tip_disp"};
    for (const auto &g : a.global) {
        bool ok = false;
        for (const char *k : known) ok = ok || g == k;
        if (!ok) die("unknown global output " + g, 2);
    }
    return a;
}

// Host copy of the state (sphnj_host_state over owned vectors).
struct HostState {
    std::vector<float> fpos, fvel, frho, fp, fdudx, fgrad, fdudt, fcolor, fdrho;
    std::vector<int32_t> fphase, fbt, fnear, fcell, scell, vcell;
    std::vector<double> spos, sref, svel, sdudt, sF, sP, sL, sms;
    std::vector<float> sp, snormal, scouple, vpos, vnormal, vvel, vp, vrho;
    std::vector<int32_t> sbt, smat, vphase, vbt;
    sphnj_host_state s{};
    explicit HostState(const sphnj_params &p) {
        const size_t nf = p.fluid_number_total, ns = p.solid_number, nv = p.virt_number;
        fpos.resize(2 * nf); fvel.resize(2 * nf); frho.resize(nf); fp.resize(nf); fdudx.resize(4 * nf);
        fgrad.resize(2 * nf); fdudt.resize(2 * nf); fcolor.resize(nf); fdrho.resize(nf);
        fphase.resize(nf); fbt.resize(nf); fnear.resize(nf); fcell.resize(nf);
        spos.resize(2 * ns); sref.resize(2 * ns); svel.resize(2 * ns); sdudt.resize(2 * ns);
        sF.resize(4 * ns); sP.resize(4 * ns); sL.resize(4 * ns); sms.resize(4 * ns);
        sp.resize(ns); snormal.resize(2 * ns); scouple.resize(2 * ns); sbt.resize(ns); smat.resize(ns);
        scell.resize(ns);
        vpos.resize(2 * nv); vnormal.resize(2 * nv); vvel.resize(2 * nv); vp.resize(nv); vrho.resize(nv);
        vphase.resize(nv); vbt.resize(nv); vcell.resize(nv);
        auto P = [](auto &v) { return v.empty() ? nullptr : v.data(); };
        s.fluid_position = P(fpos); s.fluid_velocity = P(fvel); s.fluid_density = P(frho);
        s.fluid_pressure = P(fp); s.fluid_phase = P(fphase); s.fluid_boundary_type = P(fbt);
        s.fluid_has_near_particle = P(fnear); s.fluid_du_dx = P(fdudx); s.fluid_gradient = P(fgrad);
        s.fluid_du_dt = P(fdudt); s.fluid_color = P(fcolor); s.fluid_drho_dt = P(fdrho);
        s.solid_position = P(spos); s.solid_reference_position = P(sref); s.solid_velocity = P(svel);
        s.solid_boundary_type = P(sbt); s.solid_material_type = P(smat); s.solid_max_strain = P(sms);
        s.solid_pressure = P(sp); s.solid_deformation = P(sF); s.solid_stress_1st_piola = P(sP);
        s.solid_correction = P(sL); s.solid_du_dt = P(sdudt); s.solid_normal = P(snormal);
        s.solid_couple_dudt = P(scouple);
        s.virt_position = P(vpos); s.virt_normal = P(vnormal); s.virt_velocity = P(vvel);
        s.virt_pressure = P(vp); s.virt_density = P(vrho); s.virt_phase = P(vphase); s.virt_boundary_type = P(vbt);
        s.fluid_cell_id = P(fcell); s.solid_cell_id = P(scell); s.virt_cell_id = P(vcell);
    }
};

// ---- VTK writers (output.cu:7-247) --------------------------------------------
template <class T> void points(std::ostream &o, const std::vector<T> &xy, size_t n) {
    o << "POINTS " << n << " float" << std::endl;
    for (size_t i = 0; i < n; ++i) o << xy[2 * i] << " " << xy[2 * i + 1] << " 0.0\n";
    o << "POINT_DATA " << n << std::endl;
}

void header(std::ostream &o, const char *title) {
    o << "# vtk DataFile Version 2.0" << std::endl << title << std::endl << "ASCII" << std::endl
      << "DATASET POLYDATA" << std::endl;
}

std::ofstream open_vtk(const fs::path &dir, const char *field, long file_step) {
    std::ofstream o(dir / (std::string(field) + "-" + std::to_string(file_step) + ".vtk"));
    if (!o) die("cannot write " + (dir / field).string());
    return o;
}

void write_vtk(const HostState &h, const sphnj_params &p, const fs::path &out, long file_step) {
    const size_t nf = p.fluid_number_total, ns = p.solid_number, nv = p.virt_number;
    if (nf) {  // Output::outputData, output.cu:256-263
        const fs::path dir = out / "fluid";
        {
            auto o = open_vtk(dir, "fluid_velocity", file_step);
            header(o, "Velocity vector file");
            points(o, h.fpos, nf);
            o << "VECTORS velocity float " << std::endl;
            for (size_t i = 0; i < nf; ++i) o << h.fvel[2 * i] << " " << h.fvel[2 * i + 1] << " 0.0\n";
        }
        {
            auto o = open_vtk(dir, "fluid_density", file_step);
            header(o, "scalar file");
            points(o, h.fpos, nf);
            o << "SCALARS density float 1" << std::endl << "LOOKUP_TABLE default" << std::endl;
            for (size_t i = 0; i < nf; ++i) {  // output.cu:54-62: the boundary type, -1 for gas
                if (h.fphase[i] == SPHNJ_LIQUID) o << h.fbt[i] << "\n";
                else o << -1 << "\n";
            }
        }
        {
            auto o = open_vtk(dir, "fluid_pressure", file_step);
            header(o, "scalar file");
            points(o, h.fpos, nf);
            o << "SCALARS pressure float 1" << std::endl << "LOOKUP_TABLE default" << std::endl;
            for (size_t i = 0; i < nf; ++i) o << h.fp[i] << "\n";
        }
    }
    if (ns) {  // output.cu:264-272
        const fs::path dir = out / "solid";
        {
            auto o = open_vtk(dir, "solid_velocity", file_step);
            header(o, "Velocity vector file");
            points(o, h.spos, ns);
            o << "VECTORS velocity float " << std::endl;
            for (size_t i = 0; i < ns; ++i)  // output.cu:112-113: P(1,1), max strain (0,0) and (1,1)
                o << (float)h.sP[4 * i + 3] << " " << (float)h.sms[4 * i] << " " << (float)h.sms[4 * i + 3] << "\n";
        }
        {
            auto o = open_vtk(dir, "solid_pressure", file_step);
            header(o, "scalar file");
            points(o, h.spos, ns);
            o << "SCALARS pressure float 1" << std::endl << "LOOKUP_TABLE default" << std::endl;
            for (size_t i = 0; i < ns; ++i) o << h.sp[i] << "\n";
        }
        {
            auto o = open_vtk(dir, "solid_density", file_step);
            header(o, "scalar file");
            points(o, h.spos, ns);
            o << "SCALARS density float 1" << std::endl << "LOOKUP_TABLE default" << std::endl;
            for (size_t i = 0; i < ns; ++i)
                o << (h.smat[i] == SPHNJ_LINEAR_ELASTIC ? p.solid_reference_density : p.auxetic_density) << "\n";
        }
        {
            auto o = open_vtk(dir, "solid_stress", file_step);
            header(o, "Velocity vector file");
            points(o, h.spos, ns);
            o << "VECTORS stress float " << std::endl;
            for (size_t i = 0; i < ns; ++i) {
                if (h.smat[i] == SPHNJ_LINEAR_ELASTIC) o << "0.0 0.0 0.0\n";
                else o << (float)h.sP[4 * i] << " " << (float)h.sP[4 * i + 3] << " " << (float)h.sP[4 * i + 2] << "\n";
            }
        }
    }
    if (nv) {  // output.cu:273-280
        const fs::path dir = out / "virtual";
        {
            auto o = open_vtk(dir, "virt_normal", file_step);
            header(o, "Velocity vector file");
            points(o, h.vpos, nv);
            o << "VECTORS normal float " << std::endl;
            for (size_t i = 0; i < nv; ++i) o << h.vnormal[2 * i] << " " << h.vnormal[2 * i + 1] << " 0.0\n";
        }
        {
            auto o = open_vtk(dir, "virt_pressure", file_step);
            header(o, "scalar file");
            points(o, h.vpos, nv);
            o << "SCALARS pressure float 1" << std::endl << "LOOKUP_TABLE default" << std::endl;
            for (size_t i = 0; i < nv; ++i) o << h.vphase[i] << "\n";  // output.cu:244: the phase
        }
    }
}

}  // namespace

namespace {

// Appends one line to OUT/global/<name>.dat (output.cu:283-560 open each
// file in append mode per line).
void append(const fs::path &dir, const std::string &name, const std::string &line) {
    std::ofstream o(dir / (name + ".dat"), std::ios::app);
    if (!o) die("cannot write " + (dir / name).string());
    o << line << std::endl;
}

std::string fmt(std::initializer_list<double> v, bool as_float) {
    std::ostringstream s;
    bool first = true;
    for (double x : v) {
        if (!first) s << " ";
        first = false;
        if (as_float) s << (float)x;
        else s << x;
    }
    return s.str();
}

// The writers of output.cu that follow one particle of a hard-coded case
// geometry (the wedge, a beam's end or middle, the tank beam's end) or sum
// over a band of particles read the state on the host, as the reference
// does: the solid positions and coupling forces, or the fluid positions, are
// copied for them.
bool host_writer(const std::string &name) {
    return name == "wedge_disp" || name == "middle_position" || name == "end_position" ||
           name == "tank_beam_end" || name == "crush_force" || name == "height";
}

// Index of the solid particle whose reference position lies within half a
// particle spacing of (x, y): the first one (the loops that `break`) or the
// last one (outputWedgeDisp has no break); -1 if none.
long solid_at(const HostState &h, size_t ns, double x, double y, float dx, bool last) {
    long found = -1;
    for (size_t i = 0; i < ns; ++i) {
        const double ex = h.sref[2 * i] - x, ey = h.sref[2 * i + 1] - y;
        if (std::sqrt(ex * ex + ey * ey) < 0.5 * dx) {
            found = (long)i;
            if (!last) break;
        }
    }
    return found;
}

// Where no particle sits at the writer's point the reference leaves its
// position vector uninitialised; its build prints zeros there (the vector
// as zero, then the writer's offsets added), and so does this driver.

void write_host_global(sphnj_ctx *ctx, const std::string &name, const sphnj_params &p, const fs::path &gdir,
                       HostState &h, uint32_t &have) {
    const bool fluid = name == "height";
    const uint32_t mask = fluid ? (SPHNJ_F_FLUID_KINEMATICS | SPHNJ_F_FLUID_THERMO)
                                : (SPHNJ_F_SOLID_KINEMATICS | SPHNJ_F_SOLID_DERIVED);
    if ((have & mask) != mask && (fluid ? p.fluid_number_total : p.solid_number) > 0) {
        if (sphnj_download(ctx, mask, &h.s)) die(sphnj_last_error(ctx), 3);
        have |= mask;
    }
    const size_t ns = p.solid_number, nf = p.fluid_number_total;
    const float dx = p.particle_diameter;
    int step = 0;
    sphnj_get_step(ctx, &step);
    if (name == "wedge_disp") {  // outputWedgeDisp, output.cu:307-337
        // SimTime's current_time - dt at this output (output before step + 1)
        const float t = (float)(step + 1) * p.dt - p.dt;
        const double middle = 1.5, half_L = 0.6, shift = 2.02;
        const double left_mid_x = middle - 0.5 * half_L;
        const double tan_10 = std::tan(10.0 * 3.141593f / 180.0);  // PI of global.h:4
        const double left_mid_y = -tan_10 * (left_mid_x - middle) + shift;
        const long k = solid_at(h, ns, left_mid_x - 0.5 * dx, left_mid_y + 0.5 * dx, dx, true);
        const double down = -30.0 * t;
        append(gdir, name, k < 0 ? fmt({0.0, 0.0}, false)
                                 : fmt({h.spos[2 * k] - h.sref[2 * k], h.spos[2 * k + 1] - h.sref[2 * k + 1] - down},
                                       false));
    } else if (name == "middle_position") {  // outputMiddlePosition, output.cu:371-397
        const float thick = 0.05f;
        const long k = solid_at(h, ns, 0.5 * ((double)p.domain_xmax[0] + p.domain_xmin[0]) - 0.5 * dx,
                                -thick + 0.5 * dx, dx, false);
        append(gdir, name, fmt({(k < 0 ? 0.0 : h.spos[2 * k]) + 0.5 * dx,
                                (k < 0 ? 0.0 : h.spos[2 * k + 1]) + (thick - 0.5 * dx)}, false));
    } else if (name == "end_position") {  // outputEndPosition, output.cu:399-424
        const long k = solid_at(h, ns, (double)p.domain_xmax[0] - 0.5 * dx,
                                0.5 * ((double)p.domain_xmin[1] + p.domain_xmax[1]) - 0.5 * dx, dx, false);
        append(gdir, name, fmt({(k < 0 ? 0.0 : h.spos[2 * k]) + 0.5 * dx, (k < 0 ? 0.0 : h.spos[2 * k + 1]) + 0.5 * dx},
                               false));
    } else if (name == "tank_beam_end") {  // outputTankBeamEnd, output.cu:457-478
        const double thick = 0.005, px = -0.5 * thick + 0.5 * dx, py = 0.5 * dx;
        const long k = solid_at(h, ns, px, py, dx, false);
        append(gdir, name, k < 0 ? fmt({0.0, 0.0}, false) : fmt({h.spos[2 * k] - px, h.spos[2 * k + 1] - py}, false));
    } else if (name == "crush_force") {  // outputCrushForce, output.cu:480-502
        const float rho = p.auxetic_density, dv = p.diameter_square;
        float force = 0.0f;
        for (size_t i = 0; i < ns; ++i)
            if (h.sref[2 * i + 1] < dx && h.sref[2 * i + 1] > 0.0) force += h.scouple[2 * i + 1] * rho * dv;
        append(gdir, name, fmt({force / 16.2e-3}, false));
    } else if (name == "height") {  // outputEdge's height.dat, output.cu:354-368
        float h0 = -0.5f * dx, h1 = -0.5f * dx;
        const float x0 = 5.366f - 0.825f, x1 = 5.366f - 1.653f;
        for (size_t i = 0; i < nf; ++i) {
            if (h.fphase[i] != SPHNJ_LIQUID) continue;
            const float x = h.fpos[2 * i], y = h.fpos[2 * i + 1];
            if (y > h0 && x < x0 + 0.5f * dx && x > x0 - 0.5f * dx) h0 = y;
            if (y > h1 && x < x1 + 0.5f * dx && x > x1 - 0.5f * dx) h1 = y;
        }
        append(gdir, name, fmt({h0 + dx * 0.5f, h1 + dx * 0.5f}, true));
    }
}

// Output::outputGlobalData and Probe::outputData for the current state, in
// the order the writers are named.
void write_global(sphnj_ctx *ctx, const Args &a, const sphnj_params &p, const fs::path &gdir, HostState &h) {
    sphnj_diag g{};
    int rc = sphnj_diagnostics(ctx, &g);
    if (rc) die(std::string("diagnostics: ") + sphnj_last_error(ctx), 3);
    uint32_t have = 0;  // fields copied to h for this output
    for (const auto &name : a.global) {
        if (host_writer(name)) {
            write_host_global(ctx, name, p, gdir, h, have);
            continue;
        }

        if (name == "total_force") append(gdir, name, fmt({g.total_force[0], g.total_force[1]}, true));
        else if (name == "von_mises_stress")
            append(gdir, name, fmt({g.von_mises[0], g.von_mises[1], std::max(g.von_mises[0], g.von_mises[1])}, false));
        else if (name == "mean_pressure")
            append(gdir, name, p.solid_number ? fmt({g.mean_pressure}, true) : std::string("nan"));
        else if (name == "frontier")  // outputEdge: max liquid x (from 0) + d/2
            append(gdir, name, fmt({std::max(g.front, 0.5 * (double)p.particle_diameter)}, true));
        else if (name == "total_energy") append(gdir, name, fmt({g.solid_strain, g.solid_kinetic}, false));
        else if (name == "tip_disp") append(gdir, name, fmt({g.tip_disp[0], g.tip_disp[1]}, false));
    }
    if (!a.probes.empty()) {
        std::vector<float> xy, out(4 * a.probes.size());
        for (const auto &q : a.probes) {
            xy.push_back(q.first);
            xy.push_back(q.second);
        }
        rc = sphnj_probe(ctx, (int)a.probes.size(), xy.data(), out.data());
        if (rc) die(std::string("probe: ") + sphnj_last_error(ctx), 3);
        for (size_t k = 0; k < a.probes.size(); ++k)  // probe.cu:127
            append(gdir, "probe-" + std::to_string(k),
                   fmt({a.probes[k].first, a.probes[k].second, out[4 * k], out[4 * k + 1], out[4 * k + 2],
                        out[4 * k + 3]}, true));
    }
}

// At most one VTK job in flight, on its own thread, from its own host copy.
class Writer {
  public:
    void submit(std::function<void()> job) {
        wait();
        t_ = std::thread(std::move(job));
    }
    void wait() {
        if (t_.joinable()) t_.join();
    }
    ~Writer() { wait(); }

  private:
    std::thread t_;
};

}  // namespace

int main(int argc, char **argv) {
    const Args a = parse(argc, argv);
    const fs::path cdir(a.case_dir), ddir = fs::path(a.case_dir) / "data", out(a.out_dir);
    // Parameter::initiate (parameter.h:28-33): counts, ini keys, derived constants
    sphnj_params p{};
    int rc = sphnj_params_read_ini((cdir / "config" / "input.ini").string().c_str(), &p);
    if (rc == SPHNJ_ERR_CONFIG) die("config/input.ini: a required key is missing or invalid", 1);
    if (rc) die("cannot read " + (cdir / "config" / "input.ini").string(), 1);
    if ((rc = sphnj_params_read_counts(ddir.string().c_str(), &p))) die("cannot read the particle counts", 1);
    if (a.iend >= 0) p.iend = (int)a.iend;
    if (a.result_interval > 0) p.result_interval = (int)a.result_interval;
    if ((rc = sphnj_params_derive(&p))) die("bad parameters", 1);

    sphnj_ctx *ctx = nullptr;
    if ((rc = sphnj_create(&p, a.form, &ctx))) die("sphnj_create failed (status " + std::to_string(rc) + ")", 3);
    std::unique_ptr<sphnj_ctx, void (*)(sphnj_ctx *)> guard(ctx, sphnj_destroy);
    if (!a.restart.empty()) {
        if ((rc = sphnj_checkpoint_read(ctx, a.restart.c_str()))) die(sphnj_last_error(ctx), 3);
    } else {
        HostState in(p);  // Sim::initiate, sim.cu:40-60
        if ((rc = sphnj_read_particles(ddir.string().c_str(), &p, &in.s))) die("cannot read the particle files", 1);
        sphnj_host_state s{};
        s.fluid_position = in.s.fluid_position; s.fluid_velocity = in.s.fluid_velocity;
        s.fluid_density = in.s.fluid_density; s.fluid_pressure = in.s.fluid_pressure;
        s.fluid_phase = in.s.fluid_phase;
        s.solid_position = in.s.solid_position; s.solid_velocity = in.s.solid_velocity;
        s.solid_reference_position = in.s.solid_reference_position;
        s.solid_material_type = in.s.solid_material_type; s.solid_boundary_type = in.s.solid_boundary_type;
        s.virt_position = in.s.virt_position; s.virt_boundary_type = in.s.virt_boundary_type;
        if ((rc = sphnj_upload(ctx, &s))) die(sphnj_last_error(ctx), 3);
    }
    if (a.autotune > 0) {
        sphnj_tuning t{};
        if ((rc = sphnj_autotune(ctx, (int)a.autotune, &t))) die(sphnj_last_error(ctx), 3);
        if (!a.quiet)
            std::cout << "autotune: " << (t.tiled ? "tiles of " + std::to_string(t.tile_h) + " cells" : "per particle")
                      << (t.tiled ? (t.lists ? ", stored lists" : ", stencil walk") : "") << ", " << t.ms_per_step
                      << " ms/step" << std::endl;
    }
    const fs::path gdir = out / "global";
    for (const char *sub : {"fluid", "solid", "virtual", "global"}) fs::create_directories(out / sub);

    const long ri = p.result_interval > 0 ? p.result_interval : 1;
    HostState bufs[2] = {HostState(p), HostState(p)};
    HostState gbuf(p);  // host copy for the writers that read particles
    int cur = 0;
    Writer writer;
    const uint32_t vtk_mask = SPHNJ_F_FLUID_KINEMATICS | SPHNJ_F_FLUID_THERMO | SPHNJ_F_FLUID_FLAGS |
                              SPHNJ_F_SOLID_KINEMATICS | SPHNJ_F_SOLID_MATERIAL | SPHNJ_F_SOLID_DERIVED | SPHNJ_F_VIRT;
    auto output_vtk = [&](long file_step) {
        HostState &h = bufs[cur];
        writer.wait();  // the other buffer's job may still run; this one is free after the wait
        if (sphnj_download(ctx, vtk_mask, &h.s)) die(sphnj_last_error(ctx), 3);
        writer.submit([&h, &p, out, file_step] { write_vtk(h, p, out, file_step); });
        cur ^= 1;
    };

    int step = 0;
    sphnj_get_step(ctx, &step);
    const auto t0 = std::chrono::steady_clock::now();
    long i = step;
    while (true) {
        // SimTime::addStep (sim_time.cpp:34-40); the outputs come before the
        // step's stages, from the state after step i - 1 (calculation.cu:30-34)
        const long next = i + 1;
        if (next > p.iend) break;
        if (a.vtk && (next - 1) % ri == 0) {
            if (!a.quiet)
                std::cout << "Outputing Data...\n--step=" << next - 1 << " file_step=" << next / ri << "--" << std::endl;
            output_vtk(next / ri);
        }
        if (a.global_every > 0 && (next - 1) % a.global_every == 0) write_global(ctx, a, p, gdir, gbuf);
        // run to the next event in one call
        long run = p.iend - i;
        auto until = [&](long every) {
            if (every <= 0) return;
            const long k = ((next - 1) / every + 1) * every + 1;  // next step j > next with (j - 1) % every == 0
            run = std::min(run, k - 1 - i);
        };
        if (a.vtk) until(ri);
        until(a.global_every);
        until(a.checkpoint_every);
        run = std::max(run, 1L);
        if ((rc = sphnj_step(ctx, (int)run))) die(sphnj_last_error(ctx), 3);
        i += run;
        if (a.checkpoint_every > 0 && i % a.checkpoint_every == 0) {
            if ((rc = sphnj_synchronize(ctx))) die(sphnj_last_error(ctx), 4);
            if ((rc = sphnj_checkpoint_write(ctx, (out / ("checkpoint-" + std::to_string(i) + ".bin")).string().c_str())))
                die(sphnj_last_error(ctx), 3);
        }
    }
    if ((rc = sphnj_synchronize(ctx))) die(sphnj_last_error(ctx), 4);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    std::printf("total time=%dms\n", (int)ms);
    // the final Output::outputData after the loop (calculation.cu:46), at i = iend + 1
    if (a.vtk && (p.iend % ri) == 0) output_vtk((p.iend + 1) / ri);
    writer.wait();
    return 0;
}
