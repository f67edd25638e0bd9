/* fggpu.h — C ABI of the GB300 implementation of FeeLLGood's per-time-step LLG update.
 *
 * One context owns all device memory of one mesh (or of a batch of independent meshes)
 * on one GPU and one CUDA stream. All arrays crossing this ABI are HOST arrays in the
 * caller's node numbering; indices are 0-based. No call exits the process and no C++
 * exception crosses the ABI: every entry point returns an FG_* status code.
 *
 * Reference interfaces replaced (paths in the FeeLLGood source tree):
 *   fg_create        Fem/mesh/LinAlgebra/scal_fmm::fmm construction: src/fem.h:46-121,
 *                    src/linear_algebra.h:40-65 (CSR shape, Dirichlet list),
 *                    src/fmm_demag.h:64-90 (octree insertion, done once)
 *   fg_set_state     mesh::init_distrib / mesh::readSol: src/mesh.h:221-277, src/read.cpp:199-249
 *   fg_step          LinAlgebra::base_projection + prepareElements + solve (+ updateNode):
 *                    src/time_integration.cpp:193-205, src/linear_algebra.cpp:3-53,
 *                    src/solver.cpp:6-89
 *   fg_compute_all   Fem::compute_all (demag of m and of v, energy, evolution): src/fem.h:203-224
 *   fg_get_state     the node data read by mesh::savesol / Fem::saver: src/save.cpp:164-186
 *   fg_demag         scal_fmm::fmm::demag for one field: src/fmm_demag.h:184-224
 *   fg_energy        Fem::energy: src/energy.cpp:5-68
 *   fg_batch_*       no counterpart: the reference runs one mesh per process. A batch is
 *                    many independent meshes stepped together, each sample following the
 *                    per-step sequence above (src/time_integration.cpp:193-231) on its own.
 */
#ifndef FGGPU_H
#define FGGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; 1 and 2 keep the meaning of algebra::algoStatus (src/algebra/iter.h:24-30) */
#define FG_OK 0
#define FG_SOLVER_ITER_OVERFLOW 1
#define FG_SOLVER_CANNOT_CONVERGE 2
#define FG_ETIMEDOUT 3 /* a bounded device-side wait gave up; the context stays usable */
#define FG_EINVAL 4
#define FG_ECUDA 5
#define FG_ENOMEM 6
#define FG_EMESH 7
#define FG_EIO 8

/* precision of the per-step solve */
#define FG_PREC_FP64 0        /* plain path: every stage in FP64, as the reference */
#define FG_PREC_FP32_REFINE 1 /* FP32 Krylov body and FP32 FMM, FP64 refinement residual */

/* demagnetising-potential evaluator */
#define FG_DEMAG_AUTO 0
#define FG_DEMAG_DIRECT 1 /* exact tiled direct sum */
#define FG_DEMAG_FMM 2    /* fast multipole method on a uniform octree */

typedef struct fg_ctx fg_ctx;

/* A set-up mesh: tetrahedra oriented (positive Jacobian, Tet::orientate), boundary and
 * interface triangles present with their signed dMs (mesh::controlTriangles). xyz in m. */
typedef struct {
    int n_nodes, n_tets, n_tris;
    const double *xyz;         /* n_nodes*3 */
    const int32_t *tet4;       /* n_tets*4 */
    const int32_t *tet_region; /* n_tets, index into the region table */
    const int32_t *tri3;       /* n_tris*3 */
    const int32_t *tri_region; /* n_tris, index into the triangle region table */
    const double *tri_dMs;     /* n_tris */
} fg_mesh;

/* Tetra::prm subset (src/tetra.h:86-112); Ms <= 0 marks a non-magnetic region. The last
 * five are the spin-accumulation parameters (used only with fg_opts.spin_acc): conductivity
 * sigma, density of states N0 (dens_state), polarization rate P, s-d and spin-flip lengths. */
typedef struct {
    double Ae, Ms, K, uk[3], K3, ex[3], ey[3], ez[3], alpha;
    double sigma, dens_state, P, lsd, lsf;
} fg_region;

/* Triangle::prm subset (src/triangle.h:69-101). jn, V and s are NaN where not given (the
 * boundary conditions of the electrostatic and spin-diffusion problems, fg_opts.spin_acc). */
typedef struct {
    double Ks, uk[3];
    int suppress_charges;
    double jn, V, uP[3], s[3];
} fg_tri_region;

typedef struct {
    double tol;           /* BiCG relative tolerance (finite_element_solver.tolerance) */
    int max_iter;         /* finite_element_solver.max(iter) */
    int precision;        /* FG_PREC_* */
    int learned_guess;    /* 1: online-trained per-node MLP proposes the initial guess */
    int demag;            /* FG_DEMAG_* */
    int fmm_order;        /* expansion order P of the FMM (0: default) */
    int fmm_leaf;         /* target number of sources per leaf (0: autotuned; -L: octree depth L) */
    int one_gauss_point;  /* 1: single Gauss point rules (reference ONE_GAUSS_POINT build) */
    int first_order;      /* 1: skip the demag of v (reference FIRST_ORDER build) */
    int refine_max;       /* FP64 refinement sweeps in FG_PREC_FP32_REFINE */
    double inner_tol;     /* floor of the relative target of each FP32 inner solve (1e-5) */
    int verbose;
    int profile;          /* 1: record device events around every FMM stage (fg_fmm_timings) */
    int mlp_train_steps;  /* learned guess: solves that only train before the guess is proposed */
    int mlp_batch;        /* learned guess: nodes per training minibatch */
    double mlp_lr;        /* learned guess: Adam learning rate */
    int fmm_tensor;       /* FP32 FMM: 1 (default) translations on the tensor cores (3 x TF32 MMAs),
                             0 on the CUDA cores */
    int mlp_train_every;  /* learned guess: after the first mlp_train_steps solves, train on every
                             n-th successful solve only (1, the default: on every one) */
    int fmm_native_fp64;  /* FP64 FMM: 0 (default) P2M, near field and translations in
                             double-single arithmetic on the FP32 pipes (relative error
                             ~1e-13); 1 all three on the FP64 pipe */
    int solver_lpr;       /* FP32 + refinement solver: lanes sharing one row of the operator
                             (1 thread per row, 4, 8); 0 (default): the fastest, timed on the
                             first step */
    int solver_blocks;    /* FP32 + refinement solver with solver_lpr set: persistent blocks
                             (0: all co-resident blocks). Fixing both, solver_threads (and
                             fmm_leaf = -depth) makes runs repeat bit for bit: the timed
                             choices decide the order of the solver's reductions */
    int spin_acc;         /* 1: spin accumulation coupling (spin_accumulation.enable): the
                             electrostatic potential is solved once, the spin accumulation s
                             in every fg_compute_all, and its field Hst enters the next
                             step's element integrals */
    double spin_tol;      /* relative tolerance of the spin and potential solves (1e-8) */
    int spin_max_iter;    /* their iteration limit (1000) */
    int demag_increment;  /* FP32 + refinement with the FMM (single contexts): 1 (default) every
                             fg_compute_all forms the potentials of NEXT as those of CURRENT plus
                             the FP32 FMM of the change of the field (the potential is linear in
                             the field), accumulated in FP64, so the FP32 FMM's rounding acts
                             on the step's change only; where CURRENT has no valid potentials
                             (after fg_create, fg_set_state without them, fg_recenter) the
                             potentials are evaluated in full by the FP64 FMM. 0: a full FP32
                             FMM evaluation in every fg_compute_all; 2: a full FP64 FMM
                             evaluation in every fg_compute_all (accuracy studies) */
    int fmm_overlap;      /* FMM: 1 the near field runs on a second stream of lower priority
                             concurrently with M2L and L2L, then the local expansions are
                             added (the same arithmetic, results bit-identical); 0 (default):
                             one stream (on GB300 the near field's blocks crowd out the short
                             translation launches: the film's step is 0.1 ms slower overlapped) */
    int fmm_tree_host;    /* FMM octree build: 0 (default) Morton keys and their radix sort on the
                             device; 1 keys and a comparison sort on the host (the same tree) */
    int solver_threads;   /* FP32 + refinement solver with solver_lpr set: threads per persistent
                             block, 256 or 512 (one block per SM: twice the warps to hide the
                             operator's gathers, the same number of grid-barrier participants);
                             0: 256 */
} fg_opts;

typedef struct {
    int status;         /* FG_OK, FG_SOLVER_ITER_OVERFLOW, FG_SOLVER_CANNOT_CONVERGE, FG_ETIMEDOUT */
    int iters;          /* BiCG iterations (sum of inner iterations when refining) */
    int refinements;    /* FP64 refinement sweeps */
    int guess_accepted; /* 1 if the learned guess was used */
    double vmax;        /* gamma0 * max sqrt(vp^2 + vq^2), src/solver.cpp:74-88 */
    double res;         /* final residual norm (absolute) */
    double rhsn;        /* masked RHS norm */
    double res0;        /* initial residual norm of the guess used */
    double res0_fallback; /* initial residual norm of the previous-step guess */
} fg_step_report;

void fg_opts_default(fg_opts *opts);
const char *fg_strerror(int status);
/* Last error message of a context (or of the last failed fg_create when ctx is NULL). */
const char *fg_last_error(const fg_ctx *ctx);

int fg_create(const fg_mesh *mesh, const fg_region *regions, int n_regions, const fg_tri_region *tri_regions,
              int n_tri_regions, const fg_opts *opts, fg_ctx **out);
void fg_destroy(fg_ctx *ctx);

/* Sets CURRENT and NEXT node data. v, phi, phiv may be NULL (zero). phi and phiv, when
 * given, are taken as the demag potentials of u and v (fg_opts.demag_increment continues
 * from them); pass NULL where they are not (the next fg_compute_all then evaluates them). */
int fg_set_state(fg_ctx *ctx, const double *u, const double *v, const double *phi, const double *phiv);

/* One attempt of a time step: tangent basis rotated by basis_angle (radians), element
 * integrals, solve, and on success the node update into NEXT. Does not commit NEXT. */
int fg_step(fg_ctx *ctx, double dt, double prefactor, const double Hext[3], double basis_angle,
            fg_step_report *report);

/* demag(u_NEXT) -> phi, demag(v_NEXT) -> phiv, energies of NEXT, then CURRENT <- NEXT.
 * energies: exchange, anisotropy, demag, zeeman (src/fem.h:27-36). May be NULL. */
int fg_compute_all(fg_ctx *ctx, const double Hext[3], double energies[4]);

/* which: 0 = CURRENT, 1 = NEXT. Any output may be NULL. */
int fg_get_state(const fg_ctx *ctx, int which, double *u, double *v, double *phi, double *phiv);

/* Page-locked host memory for the state buffers of fg_set_state / fg_get_state: transfers
 * from and to it run at the host link's full speed, pageable buffers are staged by the
 * driver. No counterpart in the reference (its state never leaves the host). */
int fg_host_alloc(size_t bytes, void **ptr);
int fg_host_free(void *ptr);

/* Demag potential of the NEXT field (which: 0 = u, 1 = v) into out[n_nodes], without
 * touching the state. */
int fg_demag(fg_ctx *ctx, int which, double *out);

/* Energies of the NEXT state for a constant applied field. */
int fg_energy(fg_ctx *ctx, const double Hext[3], double energies[4]);

/* fg_energy for callers that cannot allocate device memory when they call (a framework
 * that owns all device memory after start-up, or code that must not trigger the device
 * synchronisation an allocation may cause). No counterpart in the reference. Allocates
 * nothing: the reduction's partial sums go to a static device array of 8192 doubles shared
 * by all calls in the process; a context needing more returns FG_EINVAL. The first call on
 * a device looks that array up (make it before any stream capture); calls whose GPU work
 * overlaps race on the array. Same results as fg_energy. */
int fg_energy_noalloc(fg_ctx *ctx, const double Hext[3], double energies[4]);

/* Space-dependent applied field, the reference's R4toR3 field type B(x, t) = A(t) f(x)
 * (src/settings.h:33-43; mesh::setExtSpaceField src/mesh.cpp:377-389 evaluates f at the
 * Gauss points of the magnetic tets, LinAlgebra::prepareElements src/linear_algebra.cpp:54-81
 * and Tet::zeemanEnergy src/tetra.cpp:381-390 use A(t) f). The caller evaluates f (A/m)
 * itself:
 *   fg_gauss_points: *n_points = magnetic tets x Gauss points; pts (may be NULL) gets their
 *     coordinates [n_mag_tets][npi][3], magnetic tets in mesh order (the order of magTet);
 *   fg_set_space_field: field [n_mag_tets][npi][3] at those points, copied to the device
 *     (NULL removes it);
 *   fg_set_field_amplitude: A of the next fg_step / fg_compute_all calls (default 1).
 * With a space field set, the applied field at Gauss point g is Hext + A f(g), Hext being the
 * uniform field those calls take (pass zeros for a pure R4toR3 run). Not for batches. */
int fg_gauss_points(const fg_ctx *ctx, int *n_points, double *pts);

/* Spin accumulation (fg_opts.spin_acc): the last spin solve's status (FG_OK when converged;
 * on failure s is zero, as spinAcc::compute leaves it), iterations and device time in ms,
 * the electrostatic potential V[n_nodes] (host copy) and its CG iterations (any pointer may
 * be NULL); fg_get_spin copies s [n_nodes][3] (the field of the next step's Hst). */
int fg_spin_info(const fg_ctx *ctx, int *status, int *iters, double *V, int *v_iters, double *ms);
int fg_get_spin(const fg_ctx *ctx, double *s);
int fg_set_space_field(fg_ctx *ctx, const double *field);
int fg_set_field_amplitude(fg_ctx *ctx, double amplitude);

/* Recentering drift of the element integrals (Tet::add_drift_BE, src/tetra.cpp:150-169,
 * applied at :277-288): direction 0/1/2 (x/y/z, the recentering direction; -1 none) and the
 * drift speed in m/s (LinAlgebra::set_DW_vz, src/linear_algebra.h:97-98). With a speed other
 * than 0, BE_i of every magnetic tet gains vdrift sum_g w_g a_i(g) (alpha dU + U x dU +
 * s_dt (alpha dV + U x dV + V x dU)), dU and dV the derivatives of u and v along the
 * direction. Not for batches. */
int fg_set_drift(fg_ctx *ctx, int direction, double vdrift);

/* Full-precision checkpoint of a context (no reference counterpart: the reference's .sol
 * keeps u and phi to 7 digits and loses v and phiv, src/save.cpp:164-186). The file holds the
 * CURRENT state (u, v, phi, phiv in FP64), the caller's run metadata below, and the choices
 * that fix the order of the solver's and the FMM's arithmetic (solver lanes per row and
 * blocks and threads, FMM depth), so that a run resumed from it with those choices
 * (fg_opts.solver_lpr, solver_blocks, solver_threads, fmm_leaf = -depth) repeats the
 * uninterrupted run bit for bit (the learned
 * guess's network is not saved: with it the resumed run agrees to the solver tolerance).
 * Binary, little-endian, with an FNV-1a checksum; fg_checkpoint_peek reads the header
 * without a context. Call fg_checkpoint_save after fg_compute_all. */
typedef struct {
    double t0;                 /* start time of the run */
    double t, dt, dt_soft_max; /* time, last dt, the step controller's soft limit */
    long long steps;           /* accepted steps */
    long long output_index;    /* next output row */
    unsigned int rng_seed;     /* fg_rng_seed of the run */
    long long rng_draws;       /* fg_rng_angle draws since then */
    double E[4];               /* energies of the state */
} fg_checkpoint_meta;
typedef struct {
    int n_nodes, n_mag_tets, precision;
    int solver_lpr, solver_blocks, fmm_depth; /* 0 where not used */
    int solver_threads;                       /* 0 where not used (and in version-1 files) */
} fg_checkpoint_shape;
int fg_checkpoint_save(fg_ctx *ctx, const char *path, const fg_checkpoint_meta *meta);
int fg_checkpoint_peek(const char *path, fg_checkpoint_shape *shape, fg_checkpoint_meta *meta);
int fg_checkpoint_load(fg_ctx *ctx, const char *path, fg_checkpoint_meta *meta);

/* Recentering (Fem::recenter, src/recentering.cpp:47-131; call after fg_compute_all): when
 * |<u_dir>| (NEXT, magnetic volume) reaches threshold, translates the magnetisation pattern by
 * D = <u_dir> (l_dir / 2) u_dir(left end) along direction (0 x, 1 y, 2 z; l = the mesh's
 * bounding box): CURRENT u of every node becomes NEXT u of the node nearest to its shifted
 * position (clamped to the box as the reference does) and NEXT v becomes zero. *shifted tells
 * whether it moved. FG_EINVAL when both ends have the same sign along the direction (the
 * reference's "No Domain Wall" exit). The nearest node is exact, equal distances going to
 * the lower node index (the reference's kd-tree may pick another of equally near nodes). */
int fg_recenter(fg_ctx *ctx, int direction, double threshold, int *shifted);

/* <u_d> (which 0) or <v_d> (which 1) of NEXT over the magnetic volume, src/mesh.cpp:89-106. */
int fg_average(fg_ctx *ctx, int which, double avg[3]);

/* Inspection of the assembled system of the last fg_step, for parity tests:
 * rhs[2n] and the basis ep/eq[3n]; y = K x for a host x[2n]. */
int fg_debug_system(fg_ctx *ctx, double *rhs, double *ep, double *eq);
int fg_debug_apply(fg_ctx *ctx, const double *x, double *y);

/* Device time of the last fg_step / fg_compute_all phases, in ms:
 * [0] elements, [1] solve, [2] demag, [3] energy+evolution, [4] the whole step on the
 * stream's timeline from fg_step's start to fg_compute_all's end (adds the learned guess's
 * training kernels and any host gap between the two calls). */
int fg_timings(const fg_ctx *ctx, double ms[5]);

/* Counters: [0] kernels launched by the context so far, [1] FMM tree depth (0 without FMM),
 * [2] M2L (cell, cell) pairs, [3] P2P (target, source) pairs per evaluation. */
int fg_counters(const fg_ctx *ctx, long long out[4]);

/* Failure-path check (no reference counterpart): runs a device wait that nothing ends —
 * which 0: the persistent solvers' grid barrier with one block that never arrives (about
 * 2 s); 1: an mbarrier wait of the tensor-core pipeline with no arrival (about 1 s) — and
 * returns FG_ETIMEDOUT when the bounded wait expired as designed. The context stays usable. */
int fg_debug_wait_timeout(fg_ctx *ctx, int which);

/* Lanes per row the FP32 + refinement solver uses (1, 4 or 8; 0 before the first step when
 * it is chosen by timing) and its number of blocks (either may be NULL). */
int fg_solver_info(const fg_ctx *ctx, int *lanes_per_row, int *blocks);

/* Learned guess: training steps done and the last minibatch MSE (scaled units). */
int fg_mlp_info(const fg_ctx *ctx, long long *train_steps, double *last_loss);

/* Learned guess, for gradient checks: runs the training forward/backward kernels on
 * nsamples (a multiple of 128) caller-given feature rows (12 floats) and targets (3 floats);
 * returns the weights used (BF16 values as float), the summed loss gradient and the mean
 * squared loss. Parameter layout: W1[64][12], b1[64], W2[64][64], b2[64], W3[3][64], b3[3]. */
int fg_mlp_debug_grad(fg_ctx *ctx, int nsamples, const float *feat, const float *target, float *weights,
                      float *grad, float *loss);
int fg_mlp_nparam(void);
/* Learned guess, for forward checks: the inference kernel (tensor-core BF16 GEMMs with FP32
 * accumulation) on n caller-given feature rows (12 floats each) with the context's current
 * weights; out[n][3] gets the network's outputs (before the step's scale). */
int fg_mlp_debug_infer(fg_ctx *ctx, int n, const float *feat, float *out);

/* ---- batches of independent samples ----------------------------------------------
 * n_samples meshes (all sharing the region tables) packed into one context: their node
 * arrays are concatenated in sample order (fg_set_state / fg_get_state / fg_demag use
 * that order; fg_batch_info gives the offsets), the per-step system is block diagonal
 * and one persistent launch solves every block with its own Krylov scalars and its own
 * stopping test, so each sample follows the iteration it would follow alone. The demag
 * field is a forest FMM (one octree per sample): samples do not interact. A batch needs
 * opts.precision = FG_PREC_FP32_REFINE and no learned guess. fg_step does not apply to a
 * batch context; fg_compute_all and fg_energy sum over all samples with one field. */

/* Per-sample parameters of one step (the arguments of fg_step). */
typedef struct {
    double dt, prefactor, Hext[3], basis_angle;
} fg_sample_step;

/* Per-sample summary of fg_batch_run. */
typedef struct {
    int fails;           /* steps whose solve failed (the sample kept its state on those) */
    int first_fail;      /* index of the first failed step, if any */
    int iters_max;       /* largest per-step iteration count */
    int refinements_max;
    long long iters;     /* summed over the run */
    long long refinements;
    double vmax;         /* largest per-step vmax */
} fg_batch_report;

int fg_batch_create(const fg_mesh *meshes, int n_samples, const fg_region *regions, int n_regions,
                    const fg_tri_region *tri_regions, int n_tri_regions, const fg_opts *opts, fg_ctx **out);
/* n_samples and, if node_offsets is not NULL, the n_samples + 1 node offsets. */
int fg_batch_info(const fg_ctx *ctx, int *n_samples, int *node_offsets);
/* fg_step for every sample at once: steps[n_samples] in, reports[n_samples] out (may be
 * NULL). Returns FG_OK when every sample succeeded, else the worst sample status. */
int fg_batch_step(fg_ctx *ctx, const fg_sample_step *steps, fg_step_report *reports);
/* fg_compute_all for every sample; Hext[3*n_samples] (NULL: zero field) is used for the
 * per-sample energies[4*n_samples] (may be NULL: energies skipped). */
int fg_batch_compute_all(fg_ctx *ctx, const double *Hext, double *energies);
/* n_steps of fg_batch_step + fg_batch_compute_all with no host round trip in between:
 * steps[n_steps * n_samples] (step-major) are uploaded once and the whole step is
 * replayed as one CUDA graph (or launched stream-ordered where the graph cannot be
 * captured). reports[n_samples] may be NULL. Returns FG_OK or the worst status seen. */
int fg_batch_run(fg_ctx *ctx, int n_steps, const fg_sample_step *steps, fg_batch_report *reports);
/* Of the last fg_batch_run: graph_used 1 if it replayed a CUDA graph (0: stream-ordered
 * launches) and its device time in ms (CUDA events around the steps). Either may be NULL. */
int fg_batch_run_info(const fg_ctx *ctx, int *graph_used, double *device_ms);

/* Precision check of the tensor-core FMM translation (no reference counterpart): runs the
 * kernel once on host data, out[c*100 + i] = sum_code sum_j ops[code][i][j] in[tab[c][code]][j]
 * (tab entries -1 = no input; 100 coefficients per expansion), with the product terms of
 * the TF32 hi/lo split selected by terms (bit 0 hi*hi, bit 1 hi*lo, bit 2 lo*hi; 7 is what
 * the FMM uses). Allocates and frees its own device buffers. */
int fg_debug_translate_tc(int n_in, int n_out, int ncode, const float *ops, const int *tab, const float *in,
                          float *out, int terms);

/* Launch resources of the tensor-core translation kernel as the CUDA runtime sees them:
 * attrs[0] registers per thread, [1] max threads per block, [2] static shared bytes,
 * [3] max dynamic shared bytes (attribute), [4] local bytes per thread, [5] dynamic shared
 * bytes a launch asks for, [6] threads per block of a launch, [7] resident blocks per SM
 * for that launch (0: it cannot launch). */
int fg_debug_tc_resources(int attrs[8]);

/* Measured compute roofs of the current device (no reference counterpart), for the rooflines
 * of the compute-bound kernels: throughput microbenchmarks of a few ms each, counted per SM
 * and per clock cycle (clock64 over each run, so the figures hold at any clock):
 *   out[0] FP32 fused multiply-add lane operations (fma.rn.f32)
 *   out[1] the same through packed pairs (fma.rn.f32x2, two lane operations an instruction)
 *   out[2] SFU reciprocal square roots (rsqrt.approx.ftz.f32)
 *   out[3] tensor flops of tcgen05.mma kind::tf32, M = 128, N = 128, K = 8 (the FMM
 *          translations' shape), out[4] the same with N = 256
 *   out[5] the SM clock in MHz during the FP32 run (cycles over its event time)
 *   out[6] the number of SMs
 * Allocates and frees its own device buffers and stream. */
int fg_measure_peaks(double out[7]);

/* Device ms of the FMM stages when opts.profile is set, averaged over the evaluations
 * since the previous call (CUDA events around each stage, recorded without any extra
 * synchronisation): [0] P2M, [1] M2M, [2] M2L, [3] L2L, [4] L2P + P2P (with
 * fg_opts.fmm_overlap: the near-field kernel on its own stream, concurrent with [0]-[3]). */
int fg_fmm_timings(const fg_ctx *ctx, double ms[5]);

/* FMM set-up of fg_create / fg_batch_create: out[0] wall ms of the whole set-up (octree
 * builds for every depth the autotune tries, table uploads, the autotune's evaluations),
 * out[1] wall ms of the octree builds alone, out[2] device ms of the Morton-key and
 * radix-sort kernels (0 with fg_opts.fmm_tree_host), out[3] octree depth, out[4] trees. */
int fg_fmm_tree_info(const fg_ctx *ctx, double out[5]);

/* ---- host-side mesh set-up (no GPU work) ----------------------------------------
 * A set-up mesh owned by the library: the fg_mesh fields plus region names (index 0 is
 * "__default__", as in the reference's Settings) and node_index[file node] = internal
 * node (mesh::sortNodes). Free with fg_mesh_free.
 *   fg_mesh_load_msh  mesh::mesh(Settings&) construction: src/mesh.h:38-135, src/read.cpp:12-197,
 *                     src/mesh.cpp:121-367 (gmsh 2.2/4.1 ASCII, orientation, controlTriangles, sortNodes)
 *   fg_mesh_cuboid    python-modules/meshMaker.py:440-483 (Cuboid, 6 tetrahedra per cell) followed
 *                     by the same set-up, one volume region "volume" of saturation Ms */
typedef struct {
    int n_nodes, n_tets, n_tris;
    double *xyz;
    int32_t *tet4, *tet_region, *tri3, *tri_region;
    double *tri_dMs;
    int32_t *node_index;
    int n_vol_regions, n_surf_regions;
    char **vol_names, **surf_names;
} fg_mesh_data;

int fg_mesh_load_msh(const char *path, double length_unit, int n_vol, const char *const *vol_names,
                     const double *vol_Ms, int n_surf, const char *const *surf_names, fg_mesh_data **out);
int fg_mesh_cuboid(int nx, int ny, int nz, double lx, double ly, double lz, double length_unit, double Ms,
                   fg_mesh_data **out);
int fg_mesh_view(const fg_mesh_data *data, fg_mesh *mesh);
void fg_mesh_free(fg_mesh_data *data);
const char *fg_mesh_last_error(void);

/* Basis-angle stream of LinAlgebra::base_projection (src/linear_algebra.cpp:3-11):
 * fg_rng_seed = srand(seed) (src/main.cpp:211); each fg_rng_angle() = M_2_PI * U(0,1) from
 * std::mt19937(rand()). */
void fg_rng_seed(unsigned int seed);
double fg_rng_angle(void);

/* ---- whole simulations from a settings file (host driver around the GPU step) -----
 * fg_run reproduces `feellgood [--seed seed] settings.yml` (src/main.cpp:204-286 and
 * Fem::time_integration, src/time_integration.cpp:136-254): the same YAML/JSON settings
 * keys (numbers only where the reference accepts expressions), the gmsh mesh, the
 * TimeStepper with dt halving and max(du) rejection, <basename>.evol and
 * <basename>_iter<N>.sol outputs in the reference's formats, "-" reads stdin.
 * An optional "gpu:" section selects precision (fp64 | fp32_refine), learned_guess,
 * demag (auto | direct | fmm) and one_gauss_point. */
typedef struct {
    int status;
    long long steps; /* accepted time steps */
    double t;        /* final time */
    double wall_s;   /* wall time of the time loop */
    double E[4];     /* last energies */
} fg_run_report;

int fg_run(const char *settings_path, unsigned int seed, int verbose, fg_run_report *report);
const char *fg_run_last_error(void);
/* Ask a running fg_run to stop after the current step, saving <basename>_at_exit.sol
 * (the reference's SIGINT/SIGTERM behaviour, src/time_integration.cpp:101-134). */
void fg_run_request_stop(void);
/* Parsed settings as JSON (no GPU work). */
int fg_settings_dump(const char *settings_path, char *out, int len);

#ifdef __cplusplus
}
#endif
#endif /* FGGPU_H */
