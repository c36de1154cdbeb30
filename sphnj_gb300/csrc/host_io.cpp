// Host-side parameter and case I/O of libsphnj (no device code).
//
// Restates the reference's host configuration surface so that an existing
// SPHNJ case directory (config/input.ini + data/*.dat) drives this library
// unchanged:
//   - flat ini reader            config.cpp:59-129, config.h:112-159
//   - per-group readParameter    physics.cpp:12-17, properties.cpp:37-49,
//                                properties.cpp:120-162, domain.cpp:10-33,
//                                sim_time.cpp:10-25, kernel.cpp:11-22
//   - derived constants          kernel.cpp:25-41, properties.cpp:53-89,
//                                domain.cpp:37-49
//   - .dat particle files        properties.cpp:7-33,91-116,164-189,
//                                host_data.cuh:24-115
// Floating-point derivations use float arithmetic with powf where the
// reference calls pow() on float arguments (MSVC resolves those to the float
// overload), so the derived constants match the reference's to the bit.
#include "../../include/sphnj.h"

#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

namespace {

// ---- flat ini (Config) --------------------------------------------------
void trim(std::string &s) {
    static const char ws[] = " \n\t\v\r\f";
    s.erase(0, s.find_first_not_of(ws));
    s.erase(s.find_last_not_of(ws) + 1U);
}

// Same control flow as Config's operator>> (config.cpp:59-129): a value may
// continue over following lines that hold no '=' (comment-only lines add
// nothing); a blank line or a line with '=' ends it; the last occurrence of
// a key wins.
bool parse_ini(const std::string &path, std::map<std::string, std::string> &kv) {
    std::ifstream is(path.c_str());
    if (!is) return false;
    const std::string delim = "=", comm = "#";
    std::string nextline;
    while (is || nextline.length() > 0) {
        std::string line;
        if (nextline.length() > 0) {
            line = nextline;
            nextline = "";
        } else {
            std::getline(is, line);
        }
        line = line.substr(0, line.find(comm));
        std::string::size_type dp = line.find(delim);
        if (dp < std::string::npos) {
            std::string key = line.substr(0, dp);
            line.replace(0, dp + delim.length(), "");
            bool terminate = false;
            while (!terminate && is) {
                std::getline(is, nextline);
                terminate = true;
                std::string nl = nextline;
                trim(nl);
                if (nl == "") continue;
                nextline = nextline.substr(0, nextline.find(comm));
                if (nextline.find(delim) != std::string::npos) continue;
                nl = nextline;
                trim(nl);
                if (nl != "") line += "\n";
                line += nextline;
                terminate = false;
            }
            trim(key);
            trim(line);
            kv[key] = line;
        }
    }
    return true;
}

template <class T> T as_value(const std::string &s) {
    T t{};
    std::istringstream ist(s);
    ist >> t;  // on failure t becomes 0, as in Config::string_as_T
    return t;
}
template <> bool as_value<bool>(const std::string &s) {
    std::string up = s;
    for (auto &c : up) c = (char)std::toupper((unsigned char)c);
    return !(up == "FALSE" || up == "F" || up == "NO" || up == "N" || up == "0" || up == "NONE");
}

struct Ini {
    std::map<std::string, std::string> kv;
    template <class T> T get(const char *key, T def) const {
        auto it = kv.find(key);
        return it == kv.end() ? def : as_value<T>(it->second);
    }
};

bool read_header_and_count(const std::string &file, int *numbers, int n_numbers, long *lines) {
    std::ifstream in(file.c_str());
    if (!in.is_open()) return false;
    std::string str;
    std::getline(in, str);
    std::istringstream h(str);
    for (int k = 0; k < n_numbers; ++k) {
        numbers[k] = 0;
        h >> numbers[k];
    }
    long c = 0;
    while (std::getline(in, str)) ++c;
    *lines = c;
    return true;
}

std::string join(const char *dir, const char *name) {
    std::string d(dir ? dir : ".");
    if (!d.empty() && d.back() != '/') d += "/";
    return d + name;
}

}  // namespace

extern "C" int sphnj_params_read_ini(const char *ini_path, sphnj_params *p) {
    if (!ini_path || !p) return SPHNJ_ERR_ARG;
    Ini ini;
    if (!parse_ini(ini_path, ini.kv)) return SPHNJ_ERR_IO;
    bool err = false;

    // physics.cpp:12-17
    float g = ini.get<float>("gravity", 9.81f);
    p->gravity[0] = 0.0f;
    p->gravity[1] = -g;
    p->transient_type = ini.get<bool>("is_steady", false) ? SPHNJ_STEADY : SPHNJ_TRANSIENT;

    // properties.cpp:37-49
    p->particle_shift_coef = ini.get<float>("particle_shift_coef", 0.4f);
    p->is_fluid_viscid = ini.get<bool>("is_viscid", false) ? 1 : 0;
    p->min_pressure = ini.get<float>("min_pressure", -1.013e5f);
    p->sound_speed[0] = ini.get<float>("liquid_sound_speed", 1500.0f);
    p->reference_density[0] = ini.get<float>("liquid_density", 1000.0f);
    p->gamma[0] = ini.get<float>("liquid_gamma", 7.0f);
    p->viscosity[0] = ini.get<float>("liquid_viscosity", 1.01e-3f);
    p->sound_speed[1] = ini.get<float>("gas_sound_speed", 340.0f);
    p->reference_density[1] = ini.get<float>("gas_density", 1.29f);
    p->gamma[1] = ini.get<float>("gas_gamma", 1.4f);
    p->viscosity[1] = ini.get<float>("gas_viscosity", 17.9e-6f);

    // properties.cpp:120-162
    p->solid_reference_density = ini.get<float>("solid_density", 2700.0f);
    p->youngs_modulus = ini.get<float>("youngs_modulus", 67.5e9f);
    p->poisson_ratio = ini.get<float>("poisson_ratio", 0.34f);
    p->artificial_viscosity[0] = ini.get<float>("arti_vis_alpha", 2.5f);
    p->artificial_viscosity[1] = ini.get<float>("arti_vis_beta", 2.5f);
    p->fixed_speed[0] = ini.get<double>("solid_fixed_speed_x", 0.0);
    p->fixed_speed[1] = ini.get<double>("solid_fixed_speed_y", 0.0);
    p->constitution_type = ini.get<bool>("is_2D_strain", false) ? SPHNJ_STRAIN_2D : SPHNJ_STRESS_2D;
    p->plastic_type = ini.get<bool>("is_plastic", false) ? SPHNJ_PLASTIC : SPHNJ_HYPER_ELASTIC;
    p->auxetic_density = ini.get<float>("auxetic_density", 636.0f);
    p->auxetic_modulus = ini.get<float>("auxetic_modulus", 0.0f);
    p->auxetic_poisson_ratio = ini.get<float>("auxetic_poisson_ratio", -0.2f);
    p->yield_strain = ini.get<float>("yield_strain", 0.0f);
    p->yield_stress = ini.get<float>("yield_stress", 2.0e7f);
    p->harden_strain = ini.get<float>("harden_strain", 0.5f);
    p->harden_coef = ini.get<float>("harden_coef", 100.0f);
    if (p->auxetic_modulus == 0.0f && p->yield_strain == 0.0f) {
        err = true;
    } else if (p->yield_strain != 0.0f) {
        p->auxetic_modulus = p->yield_stress / p->yield_strain;
    } else {
        p->yield_strain = p->yield_stress / p->auxetic_modulus;
    }

    // domain.cpp:10-33
    p->cell_xmin[0] = ini.get<float>("cell_xmin", 0.0f);
    p->cell_xmin[1] = ini.get<float>("cell_ymin", 0.0f);
    p->cell_xmax[0] = ini.get<float>("cell_xmax", 0.0f);
    p->cell_xmax[1] = ini.get<float>("cell_ymax", 0.0f);
    p->domain_xmin[0] = ini.get<float>("domain_xmin", 0.0f);
    p->domain_xmin[1] = ini.get<float>("domain_ymin", 0.0f);
    p->domain_xmax[0] = ini.get<float>("domain_xmax", 0.0f);
    p->domain_xmax[1] = ini.get<float>("domain_ymax", 0.0f);
    if (p->cell_xmax[0] - p->cell_xmin[0] == 0.0f || p->cell_xmax[1] - p->cell_xmin[1] == 0.0f) err = true;
    if (p->domain_xmax[0] - p->domain_xmin[0] == 0.0f || p->domain_xmax[1] - p->domain_xmin[1] == 0.0f) err = true;

    // sim_time.cpp:10-25
    p->dt = ini.get<float>("dt", 0.0f);
    p->istart = ini.get<int>("istart", 0);
    p->iend = ini.get<int>("iend", 0);
    p->solid_sub_step = ini.get<int>("solid_sub_step", 1);
    p->result_interval = ini.get<int>("result_interval", 1);
    p->sort_every_step = ini.get<int>("sort_every_step", 1);
    p->shift_per_step = ini.get<int>("shift_per_step", 1);
    if (p->dt == 0.0f || p->istart - p->iend == 0) err = true;

    // kernel.cpp:11-22
    p->smoothing_length = ini.get<float>("smoothing_length", 0.0f);
    p->particle_diameter = ini.get<float>("particle_diameter", 0.0f);
    p->impact_length_hsml_ratio = ini.get<float>("impact_length_hsml_ratio", 3.0f);
    p->thread_num = ini.get<int>("thread_num", 32);
    if (p->smoothing_length == 0.0f || p->particle_diameter == 0.0f) err = true;

    return err ? SPHNJ_ERR_CONFIG : SPHNJ_OK;
}

extern "C" int sphnj_params_read_counts(const char *data_dir, sphnj_params *p) {
    if (!p) return SPHNJ_ERR_ARG;
    int rc = SPHNJ_OK;
    long lines = 0;
    int nf[2] = {0, 0};
    if (!read_header_and_count(join(data_dir, "fluid_particle.dat"), nf, 2, &lines)) {
        rc = SPHNJ_ERR_IO;
    } else {
        p->fluid_number[0] = nf[0];
        p->fluid_number[1] = nf[1];
        p->fluid_number_total = nf[0] + nf[1];
        if (p->fluid_number_total != 0 && lines != p->fluid_number_total) rc = SPHNJ_ERR_COUNT;
    }
    int ns = 0;
    if (!read_header_and_count(join(data_dir, "solid_particle.dat"), &ns, 1, &lines)) {
        rc = rc ? rc : SPHNJ_ERR_IO;
    } else {
        p->solid_number = ns;
        if (ns != 0 && lines != ns) rc = rc ? rc : SPHNJ_ERR_COUNT;
    }
    int nv = 0;
    if (!read_header_and_count(join(data_dir, "virt_particle.dat"), &nv, 1, &lines)) {
        rc = rc ? rc : SPHNJ_ERR_IO;
    } else {
        p->virt_number = nv;
        if (nv != 0 && lines != nv) rc = rc ? rc : SPHNJ_ERR_COUNT;
    }
    return rc;
}

extern "C" int sphnj_params_derive(sphnj_params *p) {
    if (!p) return SPHNJ_ERR_ARG;
    // FluidProperties::initiate, properties.cpp:53-67
    const float variation_percent = 0.4f;
    for (int i = 0; i < 2; ++i) {
        p->coefficient_p2rho[i] = p->gamma[i] * powf(p->sound_speed[i], -2.0f) / p->reference_density[i];
        p->coefficient_rho2p[i] = 1.0f / p->coefficient_p2rho[i];
        p->gamma_inv[i] = 1.0f / p->gamma[i];
        p->reference_density_inverse[i] = 1.0f / p->reference_density[i];
        p->min_density[i] = (1.0f - variation_percent) * p->reference_density[i];
    }
    // SolidProperties::initiate, properties.cpp:69-89
    const float E = p->youngs_modulus, v = p->poisson_ratio;
    const float aE = p->auxetic_modulus, av = p->auxetic_poisson_ratio;
    if (p->constitution_type == SPHNJ_STRAIN_2D) {
        p->lambda = E * v / (1.0f - 2.0f * v) / (1.0f + v);
        p->nu = E / (1.0f + v) / 2.0f;
        p->auxetic_lambda = aE * av / (1.0f - 2.0f * av) / (1.0f + av);
        p->auxetic_nu = aE / (1.0f + av) / 2.0f;
    } else {
        p->lambda = E * v / (1.0f - v) / (1.0f + v);
        p->nu = E / (1.0f + v) / 2.0f;
        p->auxetic_lambda = aE * av / (1.0f - av) / (1.0f + av);
        p->auxetic_nu = aE / (1.0f + av) / 2.0f;
    }
    p->bulk_modulus = E / (3.0f * (1.0f - 2.0f * v));
    p->solid_sound_speed = sqrtf(p->bulk_modulus / p->solid_reference_density);
    // Kernel::initiate, kernel.cpp:25-41 (truncated Gaussian, global.h:11-13)
    const float h = p->smoothing_length, d = p->particle_diameter, R = p->impact_length_hsml_ratio;
    p->particle_volume = powf(d, 3.0f);
    p->diameter_square = powf(d, 2.0f);
    p->smoothing_length_square = powf(h, 2.0f);
    p->smoothing_length_inverse = 1.0f / h;
    p->smoothing_length_inverse_square = powf(p->smoothing_length_inverse, 2.0f);
    p->impact_distance_square = powf(R, 2.0f) * powf(h, 2.0f);
    const float hd = h / d;
    const float tg_coef_2 = 5.551921f;
    p->kernel_coefficient_1 = expf(-powf(R, 2.0f));
    p->kernel_coefficient_2 = 1.0f / tg_coef_2 * powf(hd, -3.0f);
    p->kernel_differential = 2.0f / tg_coef_2 * powf(hd, -3.0f) * powf(h, -2.0f);
    p->coefficient_3d_to_2d = 2.120729f;
    // Domain::initiate(Kernel), domain.cpp:37-49
    const float cell_size_max = R * h;
    for (int i = 0; i < 2; ++i) {
        p->cell_number[i] = (int)((p->cell_xmax[i] - p->cell_xmin[i]) / cell_size_max);
        p->interval[i] = (p->cell_xmax[i] - p->cell_xmin[i]) / (float)p->cell_number[i];
        p->interval_inv[i] = 1.0f / p->interval[i];
    }
    p->cell_number_total = p->cell_number[0] * p->cell_number[1];
    if (p->cell_number[0] < 3 || p->cell_number[1] < 3) return SPHNJ_ERR_CONFIG;
    return SPHNJ_OK;
}

extern "C" int sphnj_read_particles(const char *data_dir, const sphnj_params *p, sphnj_host_state *s) {
    if (!p || !s) return SPHNJ_ERR_ARG;
    std::string str;
    if (p->fluid_number_total > 0) {
        std::ifstream in(join(data_dir, "fluid_particle.dat").c_str());
        if (!in.is_open()) return SPHNJ_ERR_IO;
        std::getline(in, str);
        long k = 0;
        while (std::getline(in, str)) {
            if (k >= p->fluid_number_total) return SPHNJ_ERR_COUNT;
            std::istringstream ss(str);
            float x = 0, y = 0, vx = 0, vy = 0, rho = 0, pr = 0;
            int phase = 0;
            ss >> x >> y >> vx >> vy >> rho >> pr >> phase;
            if (s->fluid_position) { s->fluid_position[2 * k] = x; s->fluid_position[2 * k + 1] = y; }
            if (s->fluid_velocity) { s->fluid_velocity[2 * k] = vx; s->fluid_velocity[2 * k + 1] = vy; }
            if (s->fluid_density) s->fluid_density[k] = rho;
            if (s->fluid_pressure) s->fluid_pressure[k] = pr;
            if (s->fluid_phase) s->fluid_phase[k] = phase;
            ++k;
        }
        if (k != p->fluid_number_total) return SPHNJ_ERR_COUNT;
    }
    if (p->solid_number > 0) {
        std::ifstream in(join(data_dir, "solid_particle.dat").c_str());
        if (!in.is_open()) return SPHNJ_ERR_IO;
        std::getline(in, str);
        long k = 0;
        while (std::getline(in, str)) {
            if (k >= p->solid_number) return SPHNJ_ERR_COUNT;
            std::istringstream ss(str);
            double x = 0, y = 0, vx = 0, vy = 0, rx = 0, ry = 0;
            int material = 0, boundary = 0;
            ss >> x >> y >> vx >> vy >> rx >> ry >> material >> boundary;
            if (s->solid_position) { s->solid_position[2 * k] = x; s->solid_position[2 * k + 1] = y; }
            if (s->solid_velocity) { s->solid_velocity[2 * k] = vx; s->solid_velocity[2 * k + 1] = vy; }
            if (s->solid_reference_position) {
                s->solid_reference_position[2 * k] = rx;
                s->solid_reference_position[2 * k + 1] = ry;
            }
            if (s->solid_material_type) s->solid_material_type[k] = material;
            if (s->solid_boundary_type) s->solid_boundary_type[k] = boundary;
            ++k;
        }
        if (k != p->solid_number) return SPHNJ_ERR_COUNT;
    }
    if (p->virt_number > 0) {
        std::ifstream in(join(data_dir, "virt_particle.dat").c_str());
        if (!in.is_open()) return SPHNJ_ERR_IO;
        std::getline(in, str);
        long k = 0;
        while (std::getline(in, str)) {
            if (k >= p->virt_number) return SPHNJ_ERR_COUNT;
            std::istringstream ss(str);
            float x = 0, y = 0;
            int boundary = 0;
            ss >> x >> y >> boundary;
            if (s->virt_position) { s->virt_position[2 * k] = x; s->virt_position[2 * k + 1] = y; }
            if (s->virt_boundary_type) s->virt_boundary_type[k] = boundary;
            ++k;
        }
        if (k != p->virt_number) return SPHNJ_ERR_COUNT;
    }
    return SPHNJ_OK;
}

extern "C" int sphnj_abi_sizeof(int which) {
    if (which == 0) return (int)sizeof(sphnj_params);
    if (which == 1) return (int)sizeof(sphnj_host_state);
    if (which == 2) return (int)sizeof(sphnj_diag);
    if (which == 3) return (int)sizeof(sphnj_tuning);
    return -1;
}
