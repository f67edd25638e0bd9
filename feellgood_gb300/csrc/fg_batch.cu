// Batches of independent samples: many meshes packed into one context and stepped
// together. The reference runs one mesh per process (src/time_integration.cpp:193-231 is
// its per-step sequence); here sample g owns a contiguous range of nodes, magnetic tets,
// magnetic triangles and Gauss-point sources, so
//   - the element and node kernels read the sample's dt, field and basis angle (SegPar),
//   - the per-step system is block diagonal and the persistent solver gives every sample
//     its own range of blocks, Krylov scalars and stopping test (k_mixed, nseg > 1),
//   - the demag field is a forest FMM with one octree per sample (fg_fmm.cu),
//   - energies are reduced per sample over blocks aligned to the samples.
// The solver is the FP32 body with FP64 refinement (k_mixed, nseg > 1) or, with precision
// FG_PREC_FP64, the plain FP64 BiCGSTAB (k_bicg64_seg), per sample exactly the iteration of
// a single context. With the learned guess (FP32 + refinement) one network serves all
// samples: fg_batch_step trains it on the batch's solutions as fg_step does, the solver
// forms and judges its candidate per sample, and fg_batch_run replays its inference with
// the network frozen.
// fg_batch_run uploads a whole schedule of per-step parameters once and replays the step
// (parameter select, elements, nodes, solve, two demag evaluations, evolution, step
// counter) as one CUDA graph, so a run needs no host round trip between steps.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <queue>
#include <string>
#include <vector>

#include "fg_internal.h"

namespace fg {


#define BCK(call)                                                                     \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            c.err = std::string(#call) + ": " + cudaGetErrorString(e_);               \
            return FG_ECUDA;                                                          \
        }                                                                             \
    } while (0)

template <typename T>
static cudaError_t balloc(T **p, size_t n) {
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T));
}
template <typename T>
static cudaError_t bupload(T **p, const std::vector<T> &h) {
    cudaError_t e = balloc(p, h.size());
    if (e != cudaSuccess) return e;
    if (!h.empty()) e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

// Offsets of a sample-sorted id list (ids must be non-decreasing).
static bool offsets_of(const std::vector<int> &ids, int nseg, std::vector<int> &off) {
    off.assign(nseg + 1, 0);
    for (size_t k = 0; k < ids.size(); k++) {
        if (ids[k] < 0 || ids[k] >= nseg || (k > 0 && ids[k] < ids[k - 1])) return false;
        off[ids[k] + 1]++;
    }
    for (int g = 0; g < nseg; g++) off[g + 1] += off[g];
    return true;
}

int batch_setup(Ctx &c, const std::vector<int4> &htet, const std::vector<int4> &htri) {
    const int ns = c.nseg;
    const std::vector<int> &nseg_of = c.h_node_seg;
    if ((int)nseg_of.size() != c.nn || ns < 1) {
        c.err = "batch: node sample ids missing";
        return FG_EINVAL;
    }
    if (!offsets_of(nseg_of, ns, c.h_seg_node)) {
        c.err = "batch: nodes are not grouped by sample";
        return FG_EINVAL;
    }
    std::vector<int> tseg(htet.size()), fseg(htri.size());
    for (size_t k = 0; k < htet.size(); k++) {
        const int4 I = htet[k];
        const int g = nseg_of[I.x];
        if (nseg_of[I.y] != g || nseg_of[I.z] != g || nseg_of[I.w] != g) {
            c.err = "batch: a tetrahedron spans two samples";
            return FG_EMESH;
        }
        tseg[k] = g;
    }
    for (size_t f = 0; f < htri.size(); f++) {
        const int4 I = htri[f];
        const int g = nseg_of[I.x];
        if (nseg_of[I.y] != g || nseg_of[I.z] != g) {
            c.err = "batch: a triangle spans two samples";
            return FG_EMESH;
        }
        fseg[f] = g;
    }
    if (!offsets_of(tseg, ns, c.h_seg_tet) || !offsets_of(fseg, ns, c.h_seg_tri)) {
        c.err = "batch: elements are not grouped by sample";
        return FG_EINVAL;
    }
    // sample of every Gauss-point source (magnetic tets, then magnetic triangles)
    c.h_src_seg.resize(c.nsrc);
    for (size_t k = 0; k < tseg.size(); k++)
        for (int g = 0; g < c.npi_t; g++) c.h_src_seg[k * c.npi_t + g] = tseg[k];
    for (size_t f = 0; f < fseg.size(); f++)
        for (int g = 0; g < c.npi_f; g++) c.h_src_seg[tseg.size() * c.npi_t + f * c.npi_f + g] = fseg[f];
    BCK(bupload(&c.tet_seg, tseg));
    BCK(bupload(&c.node_seg, c.h_node_seg));
    BCK(bupload(&c.d_seg_node, c.h_seg_node));

    // persistent-solver blocks: at least one per sample, the rest spread so that the rows
    // per block are as even as possible (largest rows-per-block first)
    const bool fp64 = c.opts.precision == FG_PREC_FP64;
    const int gmax = fp64 ? bicg_seg_max_blocks(c) : mixed_max_blocks(c);
    if (ns > gmax) {
        c.err = "batch: " + std::to_string(ns) + " samples exceed the " + std::to_string(gmax) +
                " co-resident blocks of one persistent launch";
        return FG_EINVAL;
    }
    std::vector<int> need(ns), nb(ns, 1);
    long total_need = 0;
    for (int g = 0; g < ns; g++) {
        const int rows = c.h_seg_node[g + 1] - c.h_seg_node[g];
        need[g] = std::max(1, (rows + 255) / 256);
        total_need += need[g];
    }
    const int T = (int)std::min<long>(gmax, total_need);
    {
        auto load = [&](int g) { return (double)(c.h_seg_node[g + 1] - c.h_seg_node[g]) / nb[g]; };
        std::priority_queue<std::pair<double, int>> q;
        for (int g = 0; g < ns; g++)
            if (nb[g] < need[g]) q.push({load(g), g});
        int used = ns;
        while (used < T && !q.empty()) {
            const int g = q.top().second;
            q.pop();
            nb[g]++;
            used++;
            if (nb[g] < need[g]) q.push({load(g), g});
        }
    }
    c.h_seg_blk.assign(ns + 1, 0);
    for (int g = 0; g < ns; g++) c.h_seg_blk[g + 1] = c.h_seg_blk[g] + nb[g];
    c.seg_grid = c.h_seg_blk[ns];
    BCK(bupload(&c.d_seg_blk, c.h_seg_blk));
    if (fp64) c.lpr = 1;  // one thread per row: no solver variant to choose
    if (c.partial_len < 8 * c.seg_grid) {
        cudaFree(c.partial);
        c.partial = nullptr;
        c.partial_len = 8 * c.seg_grid;
        BCK(balloc(&c.partial, c.partial_len));
    }
    // per-sample results, parameters and run accumulators
    cudaFree(c.dres);
    c.dres = nullptr;
    cudaFreeHost(c.hres);
    c.hres = nullptr;
    BCK(balloc(&c.dres, ns));
    BCK(cudaMallocHost((void **)&c.hres, sizeof(SolveResult) * ns));
    BCK(balloc(&c.seg_par, ns));
    BCK(cudaMallocHost((void **)&c.hseg_par, sizeof(SegPar) * ns));
    BCK(cudaMemset(c.seg_par, 0, sizeof(SegPar) * ns));
    BCK(balloc(&c.step_ctr, 1));
    BCK(cudaMemset(c.step_ctr, 0, sizeof(int)));
    BCK(balloc(&c.seg_acc, ns));
    BCK(cudaMallocHost((void **)&c.hseg_acc, sizeof(SegAcc) * ns));
    // energy blocks: each covers a slice of one sample's tets and triangles
    std::vector<int4> rng;
    std::vector<int> eseg, seg_eblk(ns + 1, 0);
    for (int g = 0; g < ns; g++) {
        const int t0 = c.h_seg_tet[g], nt = c.h_seg_tet[g + 1] - t0;
        const int f0 = c.h_seg_tri[g], nf = c.h_seg_tri[g + 1] - f0;
        const int k = std::max(1, (std::max(nt, nf) + 1023) / 1024);
        for (int j = 0; j < k; j++) {
            rng.push_back(make_int4(t0 + (int)((long)nt * j / k), t0 + (int)((long)nt * (j + 1) / k),
                                    f0 + (int)((long)nf * j / k), f0 + (int)((long)nf * (j + 1) / k)));
            eseg.push_back(g);
        }
        seg_eblk[g + 1] = (int)rng.size();
    }
    c.eblk_n = (int)rng.size();
    BCK(bupload(&c.eblk_rng, rng));
    BCK(bupload(&c.eblk_seg, eseg));
    BCK(bupload(&c.d_seg_eblk, seg_eblk));
    BCK(balloc(&c.seg_epart, 7 * (size_t)c.eblk_n));
    BCK(balloc(&c.seg_energy, 7 * (size_t)ns));
    BCK(cudaMallocHost((void **)&c.hseg_energy, 7 * sizeof(double) * ns));
    BCK(balloc(&c.seg_H, 3 * (size_t)ns));
    BCK(cudaMallocHost((void **)&c.hseg_H, 3 * sizeof(double) * ns));
    if (c.opts.verbose)
        fprintf(stderr, "batch: %d samples, %d solver blocks, %d energy blocks\n", ns, c.seg_grid, c.eblk_n);
    return FG_OK;
}

void batch_free(Ctx &c) {
    if (c.graph) cudaGraphExecDestroy(c.graph);
    c.graph = nullptr;
    void *d[] = {c.tet_seg, c.node_seg, c.d_seg_node, c.d_seg_blk, c.seg_par, c.seg_sched, c.step_ctr, c.seg_acc,
                 c.eblk_rng, c.eblk_seg, c.d_seg_eblk, c.seg_H, c.seg_epart, c.seg_energy};
    for (void *p : d)
        if (p) cudaFree(p);
    void *hp[] = {c.hseg_par, c.hseg_acc, c.hseg_H, c.hseg_energy};
    for (void *p : hp)
        if (p) cudaFreeHost(p);
}

static void fill_par(SegPar &P, const fg_sample_step &s) {
    P.dt = s.dt;
    P.prefactor = s.prefactor;
    for (int k = 0; k < 3; k++) P.H[k] = s.Hext[k];
    P.cr = std::cos(s.basis_angle);
    P.sr = std::sin(s.basis_angle);
    P.c0 = s.prefactor * FG_THETA * s.dt * FG_GAMMA0;
    auto pair = [](double x) {
        const float h = (float)x;
        return make_float2(h, (float)(x - (double)h));
    };
    for (int k = 0; k < 3; k++) P.H_ds[k] = pair(s.Hext[k]);
    P.rdt_ds = pair(FG_GAMMA0 * s.dt);
    P.kv_ds = pair(FG_THETA * s.dt);
}


// The per-step solve of every sample: FP64 BiCGSTAB, or the FP32 body with FP64 refinement.
static cudaError_t batch_solve(Ctx &c) {
    if (c.opts.precision == FG_PREC_FP64) return launch_bicg64(c, 1.0, 1.0);
    return launch_mixed(c, 1.0, 1.0);
}

// Demag of m (and of v beside it, one FMM evaluation of both charge sets).
static cudaError_t batch_demag_all(Ctx &c) {
    const int nq = c.opts.first_order ? 1 : 2;
    cudaError_t e = nq == 2 ? launch_charges_pair(c, c.u[1], c.v[1]) : launch_charges(c, c.u[1], 0);
    if (e == cudaSuccess) e = fmm_eval(c, nq);
    if (e == cudaSuccess) e = launch_phi_final(c, c.phi[1], 0);
    if (e == cudaSuccess && nq == 2) e = launch_phi_final(c, c.phiv[1], 1);
    return e;
}

static int demag_launches(const Ctx &c) {
    const int nq = c.opts.first_order ? 1 : 2;
    return 1 + nq + fmm_launches_per_eval(c, nq);
}

// Whether a step uses the learned guess (after its training solves; the network of a batch is
// trained by fg_batch_step and frozen inside fg_batch_run).
static bool batch_use_mlp(const Ctx &c) { return c.mlp && mlp_steps(c) >= c.opts.mlp_train_steps; }

// Stream-ordered body of one step of a run (the graph is a capture of exactly this).
static cudaError_t run_body(Ctx &c) {
    const double H0[3] = {0, 0, 0};
    const bool use = batch_use_mlp(c);
    cudaError_t e;
    if ((e = launch_select_params(c)) != cudaSuccess) return e;
    if ((e = launch_tet(c, 1.0, H0)) != cudaSuccess) return e;
    if (use) c.node_feat = mlp_node_features(c);
    e = launch_node(c, 0.0);
    c.node_feat.feat = nullptr;
    if (e != cudaSuccess) return e;
    if (use && (e = mlp_before_solve(c, 0.0, true, false)) != cudaSuccess) return e;
    e = batch_solve(c);
    c.cand_x = c.cand_W = nullptr;  // a candidate is judged by one solve only
    c.cand_o = nullptr;
    if (e != cudaSuccess) return e;
    if ((e = batch_demag_all(c)) != cudaSuccess) return e;
    if (use && (e = mlp_before_evolution(c)) != cudaSuccess) return e;
    const size_t n3 = 3 * sizeof(double) * c.nn, n1 = sizeof(double) * c.nn;
    if ((e = cudaMemcpyAsync(c.u[0], c.u[1], n3, cudaMemcpyDeviceToDevice, c.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.v[0], c.v[1], n3, cudaMemcpyDeviceToDevice, c.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.phi[0], c.phi[1], n1, cudaMemcpyDeviceToDevice, c.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c.phiv[0], c.phiv[1], n1, cudaMemcpyDeviceToDevice, c.stream)) != cudaSuccess)
        return e;
    return launch_advance(c);
}

static int body_launches(const Ctx &c) {
    return 5 + demag_launches(c) + (batch_use_mlp(c) ? 1 : 0);
}

static void try_capture(Ctx &c) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t eb = run_body(c);
        cudaError_t ee = cudaStreamEndCapture(c.stream, &g);
        if (eb == cudaSuccess && ee == cudaSuccess && g) e = cudaGraphInstantiate(&c.graph, g, 0);
        else e = (eb != cudaSuccess) ? eb : (ee != cudaSuccess ? ee : cudaErrorUnknown);
        if (g) cudaGraphDestroy(g);
    }
    c.graph_mlp = batch_use_mlp(c);
    if (e != cudaSuccess || !c.graph) {
        if (c.graph) cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
        c.graph_state = -1;
        cudaGetLastError();
        if (c.opts.verbose) fprintf(stderr, "batch: step graph not captured (%s)\n", cudaGetErrorString(e));
    } else {
        c.graph_state = 1;
    }
}

static int status_of(const SolveResult &r) {
    if (r.timeout) return FG_ETIMEDOUT;
    if (r.status == 1) return FG_SOLVER_ITER_OVERFLOW;
    if (r.status == 2 || r.fail) return FG_SOLVER_CANNOT_CONVERGE;
    return FG_OK;
}

// severity order for the combined return value
static int worse(int a, int b) {
    auto rank = [](int s) { return s == FG_ETIMEDOUT ? 3 : s == FG_SOLVER_CANNOT_CONVERGE ? 2 : s == FG_SOLVER_ITER_OVERFLOW ? 1 : 0; };
    return rank(b) > rank(a) ? b : a;
}

}  // namespace fg

using namespace fg;

#define CK(call) BCK(call)

extern "C" {

int fg_batch_info(const fg_ctx *h, int *n_samples, int *node_offsets) {
    if (!h) return FG_EINVAL;
    const Ctx &c = h->c;
    if (n_samples) *n_samples = c.batch ? c.nseg : 1;
    if (node_offsets) {
        if (c.batch) std::copy(c.h_seg_node.begin(), c.h_seg_node.end(), node_offsets);
        else { node_offsets[0] = 0; node_offsets[1] = c.nn; }
    }
    return FG_OK;
}

int fg_batch_step(fg_ctx *h, const fg_sample_step *steps, fg_step_report *reps) {
    if (!h || !steps) return FG_EINVAL;
    Ctx &c = h->c;
    if (!c.batch) {
        c.err = "fg_batch_step: not a batch context";
        return FG_EINVAL;
    }
    const int ns = c.nseg;
    for (int g = 0; g < ns; g++)
        if (!(steps[g].dt > 0)) {
            c.err = "fg_batch_step: dt of sample " + std::to_string(g) + " is not positive";
            return FG_EINVAL;
        }
    for (int g = 0; g < ns; g++) fill_par(c.hseg_par[g], steps[g]);
    const double H0[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(c.seg_par, c.hseg_par, sizeof(SegPar) * ns, cudaMemcpyHostToDevice, c.stream));
    if (c.lpr == 0) {
        CK(launch_tet(c, 1.0, H0));
        CK(mixed_autotune(c, 1.0, 1.0, 0.0));
    }
    CK(cudaEventRecord(c.ev[0], c.stream));
    c.step_open = true;
    // the learned guess as in fg_step: one network for all samples, trained on the batch's
    // solutions, its candidate judged per sample inside the solver
    const bool use_mlp = batch_use_mlp(c);
    const int train_every = std::max(1, c.opts.mlp_train_every);
    const bool will_train = c.mlp && (!use_mlp || h->solves_since_train + 1 >= train_every);
    CK(launch_tet(c, 1.0, H0));
    if (c.mlp && (use_mlp || will_train)) c.node_feat = mlp_node_features(c);
    const cudaError_t en = launch_node(c, 0.0);
    c.node_feat.feat = nullptr;
    CK(en);
    c.launches += 2;
    if (c.mlp) CK(mlp_before_solve(c, 0.0, use_mlp, will_train));
    CK(cudaEventRecord(c.ev[1], c.stream));
    c.acc_active = nullptr;
    {
        const cudaError_t e = batch_solve(c);
        c.cand_x = c.cand_W = nullptr;
        c.cand_o = nullptr;
        CK(e);
    }
    CK(cudaEventRecord(c.ev[2], c.stream));
    c.launches += 1;
    CK(cudaMemcpyAsync(c.hres, c.dres, sizeof(SolveResult) * ns, cudaMemcpyDeviceToHost, c.stream));
    if (c.mlp) CK(mlp_before_sync(c));
    CK(cudaStreamSynchronize(c.stream));
    cudaEventElapsedTime(&c.ms[0], c.ev[0], c.ev[1]);
    cudaEventElapsedTime(&c.ms[1], c.ev[1], c.ev[2]);
    int worst = FG_OK;
    for (int g = 0; g < ns; g++) {
        const SolveResult &r = c.hres[g];
        const int st = status_of(r);
        worst = worse(worst, st);
        if (reps) {
            fg_step_report &p = reps[g];
            std::memset(&p, 0, sizeof(p));
            p.status = st;
            p.iters = r.nit;
            p.refinements = r.nref;
            p.vmax = FG_GAMMA0 * std::sqrt(r.v2max);
            p.res = r.res;
            p.rhsn = r.rhsn;
            p.res0 = r.res0;
            p.res0_fallback = r.res0;
            if (use_mlp) {
                double r0m = 0.0, r0p = 0.0;
                mlp_sample_flags(c, g, &p.guess_accepted, &r0m, &r0p);
                p.res0_fallback = r0p;
            }
        }
    }
    if (c.mlp) {
        double r0m = 0.0, r0p = 0.0;
        mlp_after_sync(c, nullptr, &r0m, &r0p, nullptr);  // the training loss and the timeout flag
        if (mlp_take_timeout(c)) {
            worst = FG_ETIMEDOUT;
            c.err = "learned guess: a tensor-core pipeline wait timed out";
            return worst;
        }
        // train on this step's solutions of every sample (asynchronous)
        if (worst == FG_OK) {
            ++h->solves_since_train;
            if (will_train) {
                h->solves_since_train = 0;
                CK(mlp_train(c));
            }
        }
    }
    if (worst == FG_ETIMEDOUT) c.err = "persistent solver: grid barrier timed out";
    return worst;
}

int fg_batch_compute_all(fg_ctx *h, const double *Hext, double *energies) {
    if (!h) return FG_EINVAL;
    Ctx &c = h->c;
    if (!c.batch) {
        c.err = "fg_batch_compute_all: not a batch context";
        return FG_EINVAL;
    }
    const int ns = c.nseg;
    CK(cudaEventRecord(c.ev[3], c.stream));
    CK(batch_demag_all(c));
    c.launches += demag_launches(c);
    CK(cudaEventRecord(c.ev[4], c.stream));
    if (energies) {
        for (int k = 0; k < 3 * ns; k++) c.hseg_H[k] = Hext ? Hext[k] : 0.0;
        CK(cudaMemcpyAsync(c.seg_H, c.hseg_H, 3 * sizeof(double) * ns, cudaMemcpyHostToDevice, c.stream));
        CK(launch_energy_seg(c));
        c.launches += 2;
        CK(cudaMemcpyAsync(c.hseg_energy, c.seg_energy, 7 * sizeof(double) * ns, cudaMemcpyDeviceToHost, c.stream));
    }
    const size_t n3 = 3 * sizeof(double) * c.nn, n1 = sizeof(double) * c.nn;
    if (c.mlp) CK(mlp_before_evolution(c));  // v_prev2 of the learned guess's extrapolation
    CK(cudaMemcpyAsync(c.u[0], c.u[1], n3, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.v[0], c.v[1], n3, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.phi[0], c.phi[1], n1, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.phiv[0], c.phiv[1], n1, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaEventRecord(c.ev[5], c.stream));
    if (int *fl = fmm_error_flag(c)) CK(cudaMemcpyAsync(c.hflag, fl, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (*c.hflag) {
        c.err = "fmm: a tensor-core pipeline wait timed out";
        *c.hflag = 0;
        cudaMemsetAsync(fmm_error_flag(c), 0, sizeof(int), c.stream);
        return FG_ETIMEDOUT;
    }
    cudaEventElapsedTime(&c.ms[2], c.ev[3], c.ev[4]);
    cudaEventElapsedTime(&c.ms[3], c.ev[4], c.ev[5]);
    c.ms[4] = c.ms[2] + c.ms[3];
    if (c.step_open) cudaEventElapsedTime(&c.ms[4], c.ev[0], c.ev[5]);
    c.step_open = false;
    if (energies)
        for (int g = 0; g < ns; g++)
            for (int k = 0; k < 4; k++) energies[4 * g + k] = c.hseg_energy[7 * g + k];
    return FG_OK;
}

int fg_batch_run(fg_ctx *h, int n_steps, const fg_sample_step *steps, fg_batch_report *reps) {
    if (!h || !steps || n_steps <= 0) return FG_EINVAL;
    Ctx &c = h->c;
    if (!c.batch) {
        c.err = "fg_batch_run: not a batch context";
        return FG_EINVAL;
    }
    const int ns = c.nseg;
    const size_t need = (size_t)n_steps * ns;
    std::vector<SegPar> sched(need);
    for (size_t k = 0; k < need; k++) {
        if (!(steps[k].dt > 0)) {
            c.err = "fg_batch_run: a dt is not positive";
            return FG_EINVAL;
        }
        fill_par(sched[k], steps[k]);
    }
    if ((long long)need > c.seg_sched_len) {
        // the graph reads the schedule through a fixed pointer: re-capture after growing it
        if (c.graph) cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
        c.graph_state = 0;
        if (c.seg_sched) cudaFree(c.seg_sched);
        c.seg_sched = nullptr;
        CK(balloc(&c.seg_sched, need));
        c.seg_sched_len = (long long)need;
    }
    CK(cudaMemcpyAsync(c.seg_sched, sched.data(), need * sizeof(SegPar), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemsetAsync(c.step_ctr, 0, sizeof(int), c.stream));
    CK(cudaMemsetAsync(c.seg_acc, 0, sizeof(SegAcc) * ns, c.stream));
    CK(cudaStreamSynchronize(c.stream));  // the host schedule buffer is released below
    if (c.lpr == 0) {  // choose the solver variant on the run's first step, before the capture
        const double H0[3] = {0, 0, 0};
        c.acc_active = nullptr;
        CK(cudaMemcpyAsync(c.seg_par, c.seg_sched, sizeof(SegPar) * ns, cudaMemcpyDeviceToDevice, c.stream));
        CK(launch_tet(c, 1.0, H0));
        CK(mixed_autotune(c, 1.0, 1.0, 0.0));
    }
    c.acc_active = c.seg_acc;
    if (c.graph_state == 1 && c.graph_mlp != batch_use_mlp(c)) {  // the network became usable: recapture
        cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
        c.graph_state = 0;
    }
    if (c.graph_state == 0) try_capture(c);
    CK(cudaEventRecord(c.ev[6], c.stream));
    for (int k = 0; k < n_steps; k++) {
        if (c.graph_state == 1) CK(cudaGraphLaunch(c.graph, c.stream));
        else CK(run_body(c));
    }
    CK(cudaEventRecord(c.ev[7], c.stream));
    c.launches += (long long)n_steps * body_launches(c);
    c.run_graph = (c.graph_state == 1);
    CK(cudaMemcpyAsync(c.hseg_acc, c.seg_acc, sizeof(SegAcc) * ns, cudaMemcpyDeviceToHost, c.stream));
    if (int *fl = fmm_error_flag(c)) CK(cudaMemcpyAsync(c.hflag, fl, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (*c.hflag) {
        c.err = "fmm: a tensor-core pipeline wait timed out";
        *c.hflag = 0;
        cudaMemsetAsync(fmm_error_flag(c), 0, sizeof(int), c.stream);
        c.acc_active = nullptr;
        return FG_ETIMEDOUT;
    }
    c.acc_active = nullptr;
    cudaEventElapsedTime(&c.run_ms, c.ev[6], c.ev[7]);
    int worst = FG_OK;
    for (int g = 0; g < ns; g++) {
        const SegAcc &A = c.hseg_acc[g];
        const int st = A.worst == 3 ? FG_ETIMEDOUT
                       : A.worst == 2 ? FG_SOLVER_CANNOT_CONVERGE
                       : A.worst == 1 ? FG_SOLVER_ITER_OVERFLOW : FG_OK;
        worst = worse(worst, st);
        if (reps) {
            fg_batch_report &r = reps[g];
            r.fails = A.fails;
            r.first_fail = A.fails ? A.first_fail : -1;
            r.iters_max = A.nit_max;
            r.refinements_max = A.nref_max;
            r.iters = A.nit_sum;
            r.refinements = A.nref_sum;
            r.vmax = FG_GAMMA0 * std::sqrt(A.v2max);
        }
    }
    if (worst == FG_ETIMEDOUT) c.err = "persistent solver: grid barrier timed out";
    return worst;
}

int fg_batch_run_info(const fg_ctx *h, int *graph_used, double *device_ms) {
    if (!h) return FG_EINVAL;
    if (graph_used) *graph_used = h->c.run_graph ? 1 : 0;
    if (device_ms) *device_ms = h->c.run_ms;
    return FG_OK;
}

}  // extern "C"
