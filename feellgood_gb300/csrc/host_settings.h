// Settings of a simulation (host side): YAML-subset tree and the reference's schema.
#pragma once

#include <iostream>
#include <memory>
#include <stdexcept>
#include <cmath>
#include <string>
#include <utility>
#include <vector>

namespace fgh {

struct YamlError : std::runtime_error {
    explicit YamlError(const std::string &m) : std::runtime_error("YAML: " + m) {}
};
struct SettingsError : std::runtime_error {
    explicit SettingsError(const std::string &m) : std::runtime_error("CONFIGURATION ERROR: " + m) {}
};

struct YNode {
    enum Kind { NUL, SCALAR, SEQ, MAP } kind = NUL;
    std::string scalar;
    bool quoted = false;
    std::vector<std::shared_ptr<YNode>> seq;
    std::vector<std::pair<std::string, std::shared_ptr<YNode>>> map;
    std::shared_ptr<YNode> get(const std::string &k) const;
};

std::shared_ptr<YNode> yaml_parse(const std::string &text);

// Tetra::prm / Triangle::prm subsets with the defaults of src/default-settings.yml.
struct VolRegion {
    std::string name;
    double Ae = 1e-11, Ms = 795774.7, K = 0.0, uk[3] = {0, 0, 1}, K3 = 0.0;
    double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0}, ez[3] = {0, 0, 1}, alpha = 0.5;
    double sigma = 0.0, dens_state = 0.0, P = 0.0, lsd = 0.0, lsf = 0.0;  // spin accumulation
};
struct SurfRegion {
    std::string name;
    bool suppress_charges = false;
    double Ks = 0.0, uk[3] = {0, 0, 1};
    // boundary conditions of the electrostatic and spin-diffusion problems (NaN: not given)
    double jn = std::nan(""), V = std::nan(""), uP[3] = {0, 0, 1};
    double s[3] = {std::nan(""), std::nan(""), std::nan("")};
};

struct Settings {
    Settings();
    std::string out_dir = ".", sim_name, mesh_file, restore_file;
    double evol_time_step = 5e-13, final_time = 1e-10;
    std::vector<std::string> evol_columns;
    int save_period = 100;
    std::vector<std::pair<std::string, std::string>> metadata;
    double length_unit = 1e-9;
    VolRegion vol_default;
    SurfRegion surf_default;
    std::vector<VolRegion> vol;
    std::vector<SurfRegion> surf;
    bool init_from_file = false;
    double m0[3] = {0, 0, 1};
    double initial_time = std::nan("");
    double Bext[3] = {0, 0, 0};  // tesla; H = B / mu0
    int max_iter = 700;
    double tol = 1e-6;
    double dumax = 0.02, dt_min = 1e-16, dt_max = 5e-13;
    int precision = 7;  // significant digits of .sol files
    // options of this build, read from an optional "gpu:" section
    int gpu_precision = 0, gpu_demag = 0;
    bool gpu_learned = false, one_gauss_point = false;
    bool spin_acc = false, V_file = false;  // spin_accumulation.enable, .V_file
    bool recenter = false;                  // recentering.enable
    int recenter_dir = 2;                   // recentering.direction X/Y/Z -> 0/1/2
    double recenter_threshold = 0.1;
    int checkpoint_every = 0;    // write <out_dir>/<sim_name>.ckpt after every n-th output row
    int solver_lpr = 0, solver_blocks = 0, fmm_depth = 0;  // fixed solver / FMM choices (0: timed)
    int solver_threads = 0;                                 // threads per solver block (0: 256)
    std::string resume_file;     // continue the run of this checkpoint
    void finish();
};

Settings read_settings_text(const std::string &text);
Settings read_settings_file(const std::string &path);

}  // namespace fgh
