// Time-integration driver around the GPU step: what FeeLLGood's main() and
// Fem::time_integration do (src/main.cpp:204-286, src/time_integration.cpp:11-254),
// with every per-step computation on the GPU through the C ABI.
//   settings -> mesh set-up -> context -> initial state (constant vector or .sol file,
//   mesh::readSol src/read.cpp:199-249) -> compute_all -> visible steps, each a loop of
//   attempted steps with TimeStepper, dt halving on solver failure and the max(du)
//   rejection -> .evol rows (Fem::saver, src/save.cpp:13-162) and .sol snapshots
//   (mesh::savesol, src/save.cpp:164-186; metadata src/settings.cpp:272-313).
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "fg_host.h"
#include "host_settings.h"

namespace {

constexpr double MU0 = 1.25663706127e-6;
thread_local std::string g_run_error;
std::atomic<int> g_stop{0};

struct Stepper {  // TimeStepper (src/time_integration.cpp:11-38)
    double hard_min, hard_max, soft_max;
    void set_soft_limit(double m) { soft_max = std::min(soft_max, m); }
    double operator()(double stride) {
        double step = std::min(stride, soft_max);
        if (step > stride - 2 * hard_min && step < stride) step = stride - 2 * hard_min;
        soft_max = std::max(soft_max, std::min(step * 1.1, hard_max));
        return step;
    }
};

double prefactor_of(double dt, double dtmax) {  // timing::set_dt (src/time_integration.h:37-42)
    const double tt = dt / (100.0 * dtmax);
    return 1.0 + tt * std::fabs(std::log(tt));
}

std::string now_string() {
    char buf[64];
    std::time_t t = std::time(nullptr);
    std::strftime(buf, sizeof(buf), "%a %b %e %H:%M:%S %Y", std::localtime(&t));
    return buf;
}

std::string common_metadata(const fgh::Settings &S, const std::string &settings_name) {
    std::ostringstream ss;
    ss << "## feeLLGood version: fggpu GB300 build\n";
    char host[256] = {0};
    if (gethostname(host, sizeof(host) - 1) == 0) ss << "## hostname: " << host << "\n";
    ss << "## real-world time: " << now_string() << "\n";
    ss << "## settings file: " << settings_name << "\n";
    for (auto &kv : S.metadata) ss << "## " << kv.first << ": " << kv.second << "\n";
    return ss.str();
}

struct Run {
    fgh::Settings S;
    std::string settings_name;
    fg_mesh_data *md = nullptr;
    fg_ctx *ctx = nullptr;
    std::vector<unsigned char> mag;
    std::vector<double> u, v, phi, phiv;
    double E[4] = {0, 0, 0, 0};
    double vmax = 0, t = 0, dt = 0;
    long long nsteps = 0;
    long long rng_draws = 0;  // basis angles drawn since fg_rng_seed (for checkpoints)
    std::vector<std::pair<int, int>> edges;
    ~Run() {
        if (ctx) fg_destroy(ctx);
        if (md) fg_mesh_free(md);
    }
};

int fail(int code, const std::string &msg) {
    g_run_error = msg;
    return code;
}

int read_sol(Run &R, const std::string &file, double *t_out) {
    std::ifstream in(file);
    if (!in) return fail(FG_EIO, "cannot open file " + file);
    std::string line;
    bool has_t = false;
    double t = 0;
    std::streampos data_start = in.tellg();
    while (in.peek() == '#' || in.peek() == '\n') {
        std::getline(in, line);
        const size_t p = line.find("## time:");
        if (p != std::string::npos) {
            t = std::stod(line.substr(p + 8));
            has_t = true;
        }
        data_start = in.tellg();
    }
    if (!has_t) return fail(FG_EIO, "error: no ## time: tag in input .sol file " + file);
    const int nn = R.md->n_nodes;
    for (int i = 0; i < nn; i++) {
        long idx;
        double mx, my, mz, ph;
        if (!(in >> idx >> mx >> my >> mz >> ph)) return fail(FG_EIO, "truncated .sol file " + file);
        if (idx != i) return fail(FG_EIO, "error: mesh node index mismatch between mesh and input .sol file");
        const int k = R.md->node_index[i];
        R.u[3 * k] = mx; R.u[3 * k + 1] = my; R.u[3 * k + 2] = mz;
        R.phi[k] = ph;
    }
    *t_out = t;
    return FG_OK;
}

int write_sol(Run &R, const std::string &file, double t) {
    std::FILE *f = std::fopen(file.c_str(), "w");
    if (!f) return fail(FG_EIO, "cannot open file " + file);
    std::string meta = common_metadata(R.S, R.settings_name);
    std::fprintf(f, "%s", meta.c_str());
    const bool spin = R.S.spin_acc;
    std::fprintf(f, "## time: %e\n## columns: idx\tmx\tmy\tmz\tphi%s\n", t, spin ? "\tsx\tsy\tsz" : "");
    const int p = R.S.precision;
    const int nn = R.md->n_nodes;
    std::vector<double> s;
    if (spin) {  // mesh::savesol with the spin accumulation (src/save.cpp:164-186)
        s.assign(3 * (size_t)nn, 0.0);
        if (fg_get_spin(R.ctx, s.data()) != FG_OK) {
            std::fclose(f);
            return fail(FG_EIO, "cannot read the spin accumulation");
        }
    }
    for (int i = 0; i < nn; i++) {
        const int k = R.md->node_index[i];
        if (R.mag[k])
            std::fprintf(f, "%d\t%.*e\t%.*e\t%.*e\t%.*e", i, p, R.u[3 * k], p, R.u[3 * k + 1], p, R.u[3 * k + 2], p,
                         R.phi[k]);
        else
            std::fprintf(f, "%d\tnan\tnan\tnan\t%.*e", i, p, R.phi[k]);
        if (spin) std::fprintf(f, "\t%.*e\t%.*e\t%.*e", p, s[3 * k], p, s[3 * k + 1], p, s[3 * k + 2]);
        std::fputc('\n', f);
    }
    std::fclose(f);
    return FG_OK;
}

double max_angle(Run &R) {  // mesh::max_angle (src/mesh.h:295-306) on the NEXT state
    double mn = 1.0;
    for (auto &e : R.edges) {
        const double *a = &R.u[3 * e.first], *b = &R.u[3 * e.second];
        mn = std::min(mn, a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
    }
    return std::acos(mn);
}

int evol_row(Run &R, std::FILE *f, int nt, const double H[3]) {
    double avg_u[3] = {0, 0, 0}, avg_v[3] = {0, 0, 0};
    bool need_u = false, need_v = false, need_state = false;
    for (auto &c : R.S.evol_columns) {
        if (c == "<Mx>" || c == "<My>" || c == "<Mz>") need_u = true;
        if (c == "<dMx/dt>" || c == "<dMy/dt>" || c == "<dMz/dt>") need_v = true;
        if (c == "max_angle") need_state = true;
    }
    if (need_u && fg_average(R.ctx, 0, avg_u) != FG_OK) return fail(FG_ECUDA, fg_last_error(R.ctx));
    if (need_v && fg_average(R.ctx, 1, avg_v) != FG_OK) return fail(FG_ECUDA, fg_last_error(R.ctx));
    if (need_state && fg_get_state(R.ctx, 1, R.u.data(), nullptr, nullptr, nullptr) != FG_OK)
        return fail(FG_ECUDA, fg_last_error(R.ctx));
    const size_t nc = R.S.evol_columns.size();
    for (size_t k = 0; k < nc; k++) {
        const std::string &c = R.S.evol_columns[k];
        double val;
        if (c == "iter") { std::fprintf(f, "%d", nt); goto sep; }
        else if (c == "t") val = R.t;
        else if (c == "dt") val = R.dt;
        else if (c == "max_dm") val = R.vmax * R.dt;
        else if (c == "max_angle") val = max_angle(R);
        else if (c == "<Mx>") val = avg_u[0];
        else if (c == "<My>") val = avg_u[1];
        else if (c == "<Mz>") val = avg_u[2];
        else if (c == "<dMx/dt>") val = avg_v[0];
        else if (c == "<dMy/dt>") val = avg_v[1];
        else if (c == "<dMz/dt>") val = avg_v[2];
        else if (c == "E_ex") val = R.E[0];
        else if (c == "E_aniso") val = R.E[1];
        else if (c == "E_demag") val = R.E[2];
        else if (c == "E_zeeman") val = R.E[3];
        else if (c == "E_tot") val = R.E[0] + R.E[1] + R.E[2] + R.E[3];
        else if (c == "Hx") val = H[0];
        else if (c == "Hy") val = H[1];
        else if (c == "Hz") val = H[2];
        else return fail(FG_EINVAL, "Error: invalid column name '" + c + "'");
        std::fprintf(f, "%.16g", val);
    sep:
        std::fputc(k + 1 == nc ? '\n' : '\t', f);
    }
    std::fflush(f);
    return FG_OK;
}

int run_impl(Run &R, const char *settings_path, unsigned int seed, int verbose, fg_run_report *rep) {
    try {
        R.S = fgh::read_settings_file(settings_path);
    } catch (const std::exception &e) {
        return fail(FG_EINVAL, e.what());
    }
    fgh::Settings &S = R.S;
    R.settings_name = std::string(settings_path) == "-" ? "standard input" : settings_path;
    // mesh (mesh::mesh construction)
    std::vector<const char *> vn, sn;
    std::vector<double> ms;
    for (auto &r : S.vol) { vn.push_back(r.name.c_str()); ms.push_back(r.Ms); }
    for (auto &r : S.surf) sn.push_back(r.name.c_str());
    int s = fg_mesh_load_msh(S.mesh_file.c_str(), S.length_unit, (int)vn.size(), vn.data(), ms.data(), (int)sn.size(),
                             sn.data(), &R.md);
    if (s != FG_OK) return fail(s, fg_mesh_last_error());
    // region tables: index 0 is the __default__ region, created surface regions copy it
    std::vector<fg_region> regs(1 + S.vol.size());
    auto set_vol = [](fg_region &g, const fgh::VolRegion &r) {
        g.Ae = r.Ae; g.Ms = r.Ms; g.K = r.K; g.K3 = r.K3; g.alpha = r.alpha;
        g.sigma = r.sigma; g.dens_state = r.dens_state; g.P = r.P; g.lsd = r.lsd; g.lsf = r.lsf;
        for (int k = 0; k < 3; k++) { g.uk[k] = r.uk[k]; g.ex[k] = r.ex[k]; g.ey[k] = r.ey[k]; g.ez[k] = r.ez[k]; }
    };
    set_vol(regs[0], S.vol_default);
    for (size_t k = 0; k < S.vol.size(); k++) set_vol(regs[k + 1], S.vol[k]);
    std::vector<fg_tri_region> tregs(std::max(1, R.md->n_surf_regions));
    auto set_surf = [](fg_tri_region &g, const fgh::SurfRegion &r) {
        g.Ks = r.Ks; g.suppress_charges = r.suppress_charges ? 1 : 0;
        g.jn = r.jn; g.V = r.V;
        for (int k = 0; k < 3; k++) { g.uk[k] = r.uk[k]; g.uP[k] = r.uP[k]; g.s[k] = r.s[k]; }
    };
    for (int k = 0; k < R.md->n_surf_regions; k++) {
        if (k >= 1 && k <= (int)S.surf.size()) set_surf(tregs[k], S.surf[k - 1]);
        else set_surf(tregs[k], S.surf_default);
    }
    // resume: the checkpoint fixes the solver's and the FMM's choices of the original run, so
    // that the continuation repeats it bit for bit
    fg_checkpoint_shape ck{};
    fg_checkpoint_meta cm{};
    const bool resume = !S.resume_file.empty();
    if (resume && fg_checkpoint_peek(S.resume_file.c_str(), &ck, &cm) != FG_OK)
        return fail(FG_EIO, "cannot read checkpoint " + S.resume_file);
    fg_opts o;
    fg_opts_default(&o);
    o.solver_lpr = S.solver_lpr;
    o.solver_blocks = S.solver_blocks;
    o.solver_threads = S.solver_threads;
    if (S.fmm_depth > 0) o.fmm_leaf = -S.fmm_depth;
    if (resume) {
        o.solver_lpr = ck.solver_lpr;
        o.solver_blocks = ck.solver_blocks;
        o.solver_threads = ck.solver_threads;
        if (ck.fmm_depth > 0) o.fmm_leaf = -ck.fmm_depth;
    }
    o.tol = S.tol;
    o.max_iter = S.max_iter;
    o.precision = S.gpu_precision;
    o.learned_guess = S.gpu_learned ? 1 : 0;
    o.demag = S.gpu_demag;
    o.one_gauss_point = S.one_gauss_point ? 1 : 0;
    o.spin_acc = S.spin_acc ? 1 : 0;
    o.verbose = verbose;
    fg_mesh m;
    fg_mesh_view(R.md, &m);
    s = fg_create(&m, regs.data(), (int)regs.size(), tregs.data(), R.md->n_surf_regions, &o, &R.ctx);
    if (s != FG_OK) return fail(s, fg_last_error(nullptr));
    const int nn = R.md->n_nodes;
    if (S.spin_acc && S.V_file) {  // electrostatSolver::save (src/electrostatSolver.cpp:133-152)
        std::vector<double> V(nn);
        if (fg_spin_info(R.ctx, nullptr, nullptr, V.data(), nullptr, nullptr) != FG_OK)
            return fail(FG_EINVAL, "no potential");
        const std::string vf = S.out_dir + "/" + S.sim_name + "_V.sol";
        std::FILE *f = std::fopen(vf.c_str(), "w");
        if (!f) return fail(FG_EIO, "cannot open file " + vf);
        std::fprintf(f, "## real-world time: %s\n## columns: index\tV\n", now_string().c_str());
        for (int i = 0; i < nn; i++) std::fprintf(f, "%d\t%.8e\n", i, V[R.md->node_index[i]]);
        std::fclose(f);
    }
    R.mag.assign(nn, 0);
    for (int t = 0; t < R.md->n_tets; t++)
        if (regs[R.md->tet_region[t]].Ms > 0)
            for (int i = 0; i < 4; i++) R.mag[R.md->tet4[4 * t + i]] = 1;
    for (int t = 0; t < R.md->n_tets; t++)
        for (int i = 0; i < 3; i++)
            for (int j = i + 1; j < 4; j++) {
                const int a = R.md->tet4[4 * t + i], b = R.md->tet4[4 * t + j];
                R.edges.push_back({std::min(a, b), std::max(a, b)});
            }
    std::sort(R.edges.begin(), R.edges.end());
    R.edges.erase(std::unique(R.edges.begin(), R.edges.end()), R.edges.end());
    R.u.assign(3 * (size_t)nn, 0.0);
    R.v.assign(3 * (size_t)nn, 0.0);
    R.phi.assign(nn, 0.0);
    R.phiv.assign(nn, 0.0);
    double t0 = 0.0;
    const double H[3] = {S.Bext[0] / MU0, S.Bext[1] / MU0, S.Bext[2] / MU0};
    if (resume) {
        // full-precision state of the checkpoint; its energies stand for the initial compute_all
        s = fg_checkpoint_load(R.ctx, S.resume_file.c_str(), &cm);
        if (s != FG_OK) return fail(s, fg_last_error(R.ctx));
        t0 = cm.t0;
        for (int k = 0; k < 4; k++) R.E[k] = cm.E[k];
        seed = cm.rng_seed;
        fg_rng_seed(seed);
        for (long long k = 0; k < cm.rng_draws; k++) fg_rng_angle();
        R.rng_draws = cm.rng_draws;
    } else {
        if (S.init_from_file) {
            s = read_sol(R, S.restore_file, &t0);
            if (s != FG_OK) return s;
        } else {
            for (int i = 0; i < nn; i++)
                if (R.mag[i])
                    for (int k = 0; k < 3; k++) R.u[3 * i + k] = S.m0[k];
        }
        if (!std::isnan(S.initial_time)) t0 = S.initial_time;
        // the potentials of the initial state are not known: the first compute_all evaluates them
        s = fg_set_state(R.ctx, R.u.data(), R.v.data(), nullptr, nullptr);
        if (s != FG_OK) return fail(s, fg_last_error(R.ctx));
        // main(): srand(seed); the LinAlgebra constructor draws one basis angle
        fg_rng_seed(seed);
        fg_rng_angle();
        R.rng_draws = 1;
        s = fg_compute_all(R.ctx, H, R.E);
        if (s != FG_OK) return fail(s, fg_last_error(R.ctx));
    }
    const std::string base = S.out_dir + "/" + S.sim_name;
    // a resumed run appends its rows to the .evol of the original run
    std::FILE *fe = std::fopen((base + ".evol").c_str(), resume ? "a" : "w");
    if (!fe) return fail(FG_EIO, "cannot open file " + base + ".evol");
    if (!resume) {
        std::string meta = common_metadata(S, R.settings_name);
        std::fprintf(fe, "%s## columns:", meta.c_str());
        for (size_t k = 0; k < S.evol_columns.size(); k++)
            std::fprintf(fe, "%c%s", k ? '\t' : ' ', S.evol_columns[k].c_str());
        std::fputc('\n', fe);
    }
    R.t = t0;
    R.dt = std::sqrt(S.dt_min * S.dt_max);
    Stepper st{S.dt_min, S.dt_max * (1 + FLT_EPSILON), R.dt};
    const int step_count = (int)std::lround((S.final_time - t0) / S.evol_time_step);
    int status = FG_OK, nt_output = 0;
    if (resume) {
        R.t = cm.t;
        R.dt = cm.dt;
        st.soft_max = cm.dt_soft_max;
        R.nsteps = cm.steps;
        nt_output = (int)cm.output_index;
    }
    const auto wall0 = std::chrono::steady_clock::now();
    for (int step_nb = nt_output; step_nb <= step_count && status == FG_OK; step_nb++) {
        const double target = t0 + step_nb * S.evol_time_step;
        while (R.t < target) {
            if (g_stop.load()) {
                fg_get_state(R.ctx, 1, R.u.data(), nullptr, R.phi.data(), nullptr);
                if (S.save_period > 0) write_sol(R, base + "_at_exit.sol", R.t);
                status = FG_EINVAL;
                g_run_error = "interrupted";
                break;
            }
            R.dt = st(target - R.t);
            const bool last = (R.dt == target - R.t);
            if (R.dt < S.dt_min) {
                status = FG_SOLVER_CANNOT_CONVERGE;
                g_run_error = "**ABORTED**: dt < DTMIN";
                break;
            }
            fg_step_report rp;
            R.rng_draws++;
            s = fg_step(R.ctx, R.dt, prefactor_of(R.dt, S.dt_max), H, fg_rng_angle(), &rp);
            if (s != FG_OK && s != FG_SOLVER_ITER_OVERFLOW && s != FG_SOLVER_CANNOT_CONVERGE) {
                status = s;
                g_run_error = fg_last_error(R.ctx);
                break;
            }
            if (s != FG_OK) {  // dt halving retry (src/time_integration.cpp:207-214)
                st.set_soft_limit(R.dt / 2);
                if (verbose) std::fprintf(stderr, "solver failed (%s), retrying with dt/2\n", fg_strerror(s));
                continue;
            }
            R.vmax = rp.vmax;
            const double dumax = R.dt * R.vmax;
            st.set_soft_limit((S.dumax / R.vmax) * 0.95);
            if (dumax > S.dumax) continue;
            s = fg_compute_all(R.ctx, H, R.E);
            if (s != FG_OK) {
                status = s;
                g_run_error = fg_last_error(R.ctx);
                break;
            }
            R.nsteps++;
            R.t = last ? target : R.t + R.dt;
            if (S.recenter) {  // src/time_integration.cpp:241
                int shifted = 0;
                s = fg_recenter(R.ctx, S.recenter_dir, S.recenter_threshold, &shifted);
                if (s != FG_OK) {
                    status = s;
                    g_run_error = std::string("Error No Domain Wall: ") + fg_last_error(R.ctx);
                    break;
                }
            }
        }
        if (status != FG_OK) break;
        s = evol_row(R, fe, nt_output, H);
        if (s != FG_OK) { status = s; break; }
        if (S.save_period && (nt_output % S.save_period) == 0) {
            fg_get_state(R.ctx, 1, R.u.data(), nullptr, R.phi.data(), nullptr);
            s = write_sol(R, base + "_iter" + std::to_string(nt_output) + ".sol", R.t);
            if (s != FG_OK) { status = s; break; }
        }
        nt_output++;
        if (S.checkpoint_every > 0 && nt_output % S.checkpoint_every == 0) {
            fg_checkpoint_meta m{};
            m.t0 = t0;
            m.t = R.t;
            m.dt = R.dt;
            m.dt_soft_max = st.soft_max;
            m.steps = R.nsteps;
            m.output_index = nt_output;
            m.rng_seed = seed;
            m.rng_draws = R.rng_draws;
            for (int k = 0; k < 4; k++) m.E[k] = R.E[k];
            s = fg_checkpoint_save(R.ctx, (base + ".ckpt").c_str(), &m);
            if (s != FG_OK) {
                status = s;
                g_run_error = fg_last_error(R.ctx);
                break;
            }
        }
    }
    std::fclose(fe);
    if (rep) {
        rep->status = status;
        rep->steps = R.nsteps;
        rep->t = R.t;
        rep->wall_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
        for (int k = 0; k < 4; k++) rep->E[k] = R.E[k];
    }
    return status;
}

}  // namespace

extern "C" {

const char *fg_run_last_error(void) { return g_run_error.c_str(); }

void fg_run_request_stop(void) { g_stop.store(1); }

int fg_run(const char *settings_path, unsigned int seed, int verbose, fg_run_report *report) {
    if (!settings_path) return FG_EINVAL;
    g_stop.store(0);
    g_run_error.clear();
    try {
        Run R;
        return run_impl(R, settings_path, seed, verbose, report);
    } catch (const std::exception &e) {
        g_run_error = e.what();
        return FG_EINVAL;
    } catch (...) {
        g_run_error = "unexpected exception";
        return FG_EINVAL;
    }
}

// Parsed settings as a short JSON text (no GPU work), for checks of the settings reader.
int fg_settings_dump(const char *settings_path, char *out, int len) {
    if (!settings_path || !out || len <= 0) return FG_EINVAL;
    try {
        fgh::Settings S = fgh::read_settings_file(settings_path);
        std::ostringstream j;
        j.precision(17);
        j << "{\"mesh\": \"" << S.mesh_file << "\", \"length_unit\": " << S.length_unit << ", \"sim_name\": \""
          << S.sim_name << "\", \"final_time\": " << S.final_time << ", \"evol_time_step\": " << S.evol_time_step
          << ", \"save_period\": " << S.save_period << ", \"tol\": " << S.tol << ", \"max_iter\": " << S.max_iter
          << ", \"dumax\": " << S.dumax << ", \"dt_min\": " << S.dt_min << ", \"dt_max\": " << S.dt_max
          << ", \"Bext\": [" << S.Bext[0] << ", " << S.Bext[1] << ", " << S.Bext[2] << "], \"m0\": [" << S.m0[0]
          << ", " << S.m0[1] << ", " << S.m0[2] << "], \"init_from_file\": " << (S.init_from_file ? "true" : "false")
          << ", \"restore_file\": \"" << S.restore_file << "\", \"evol_columns\": [";
        for (size_t k = 0; k < S.evol_columns.size(); k++) j << (k ? ", " : "") << "\"" << S.evol_columns[k] << "\"";
        j << "], \"volume_regions\": [";
        for (size_t k = 0; k < S.vol.size(); k++) {
            const auto &r = S.vol[k];
            j << (k ? ", " : "") << "{\"name\": \"" << r.name << "\", \"Ae\": " << r.Ae << ", \"Ms\": " << r.Ms
              << ", \"K\": " << r.K << ", \"uk\": [" << r.uk[0] << ", " << r.uk[1] << ", " << r.uk[2]
              << "], \"alpha\": " << r.alpha << "}";
        }
        j << "], \"surface_regions\": [";
        for (size_t k = 0; k < S.surf.size(); k++)
            j << (k ? ", " : "") << "{\"name\": \"" << S.surf[k].name << "\", \"Ks\": " << S.surf[k].Ks
              << ", \"suppress_charges\": " << (S.surf[k].suppress_charges ? "true" : "false") << "}";
        auto num = [&](double x) {  // NaN (not given) as null
            if (std::isnan(x)) j << "null";
            else j << x;
        };
        j << "], \"spin_accumulation\": {\"enable\": " << (S.spin_acc ? "true" : "false")
          << ", \"V_file\": " << (S.V_file ? "true" : "false") << ", \"volume\": [";
        for (size_t k = 0; k < S.vol.size(); k++) {
            const auto &r = S.vol[k];
            j << (k ? ", " : "") << "{\"name\": \"" << r.name << "\", \"sigma\": " << r.sigma
              << ", \"dens_state\": " << r.dens_state << ", \"P\": " << r.P << ", \"l_sd\": " << r.lsd
              << ", \"l_sf\": " << r.lsf << "}";
        }
        j << "], \"surface\": [";
        for (size_t k = 0; k < S.surf.size(); k++) {
            const auto &r = S.surf[k];
            j << (k ? ", " : "") << "{\"name\": \"" << r.name << "\", \"jn\": ";
            num(r.jn);
            j << ", \"V\": ";
            num(r.V);
            j << ", \"uP\": [" << r.uP[0] << ", " << r.uP[1] << ", " << r.uP[2] << "], \"s\": [";
            num(r.s[0]); j << ", "; num(r.s[1]); j << ", "; num(r.s[2]);
            j << "]}";
        }
        j << "]}, \"recentering\": {\"enable\": " << (S.recenter ? "true" : "false") << ", \"direction\": "
          << S.recenter_dir << ", \"threshold\": " << S.recenter_threshold << "}}";
        const std::string s = j.str();
        if ((int)s.size() + 1 > len) return FG_EINVAL;
        std::memcpy(out, s.c_str(), s.size() + 1);
        return FG_OK;
    } catch (const std::exception &e) {
        g_run_error = e.what();
        return FG_EINVAL;
    }
}

}  // extern "C"
