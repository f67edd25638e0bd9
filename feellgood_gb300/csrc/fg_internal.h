// Internal declarations shared by the host orchestration (fg_api.cu) and the device
// kernels (fg_kernels.cu, fg_fmm.cu, fg_mlp.cu) of the fggpu library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fggpu.h"

// Physical constants of the reference (src/config.h.in:31-32, :59).
#define FG_MU0 1.25663706127e-6
#define FG_GAMMA0 (1.76085962784e11 * FG_MU0)
#define FG_THETA 0.5

namespace fg {

// Per-region material constants, precomputed once (Tetra::prm, src/tetra.h:86-112).
struct DevRegion {
    double A, Ms, alpha, Abis, K, Kbis, K3, K3bis;
    double uk[3], ex[3], ey[3], ez[3];
    double hst;  // spin accumulation: Hst = hst * s at the Gauss points (0 without the coupling)
    float2 Abis_ds, alpha_ds;  // double-single copies for the double-single element kernel
    float2 A_ds, edm_ds, ez_ds;  // double-single A, -mu0 Ms / 2 and -mu0 Ms for the energies
    float2 hst_ds;               // double-single hst
};

// The double-single element slots are scaled by 2^DS_SLOT_SCALE (the Jacobian is scaled on
// the host) so that their low words stay normal FP32 numbers.
constexpr int DS_SLOT_SCALE = 70;
constexpr double DS_SLOT_INV = 0x1p-70;  // 2^-DS_SLOT_SCALE: the scale undone by an exact product
static_assert(DS_SLOT_SCALE == 70 && DS_SLOT_INV * 0x1p70 == 1.0, "DS_SLOT_INV is 2^-DS_SLOT_SCALE");

// Gauss rules of the tets (5 points, or 1) and triangles (4 points, or 1): shape functions
// a_i(g) and weights per unit Jacobian (src/tetra.h:27-81, src/triangle.h:43-66).
struct Rules {
    int npi_t, npi_f;
    double ta[4][5], tp[5], fa[3][4], fp[4];
};
Rules make_rules(bool one_point);

// Per-magnetic-triangle constants for charges, self-corrections and energies.
struct DevTri {
    double n[3];
    double dMs;
    double w[4];     // Gauss weights 2*surf*pds
    double beta[9];  // corr_i += dMs * sum_k beta[3i+k] * (m_k . n): correctionCharges + potential
    double Ks;       // surface anisotropy constant
    double uk[3];
};

// Result of one solve, written by the persistent BiCG kernel.
struct SolveResult {
    int status;     // -1 undefined, 0 converged, 1 overflow, 2 cannot converge
    int nit;
    int fail;       // solve() returned true
    int timeout;
    double res, rhsn, v2max, res0;
    int nref;
    int pad;
};

// The learned guess's per-node features, formed by the node kernel when feat is set:
// row i = m_i, H_eff,i * inv_ms, v_prev,i * inv_v0 (features 0..8; the mean of m over i's
// neighbours, 9..11, is added from these rows by the inference or by k_feat_ring).
struct NodeFeat {
    float *feat;  // [nn][12] or nullptr
    double inv_ms, inv_v0;
};

// Per-sample parameters of one step of a batch of independent samples (device copy).
struct SegPar {
    double dt, prefactor;
    double H[3];    // applied field, A/m
    double cr, sr;  // cos / sin of the basis rotation angle of Node::setBasis
    double c0;      // prefactor * theta * dt * gamma0
    // double-single pairs for the double-single element kernel, formed on the host: H,
    // gamma0 dt and theta dt
    float2 H_ds[3], rdt_ds, kv_ds;
};

// Per-sample results accumulated over a multi-step batch run.
struct SegAcc {
    int fails;       // failed solves
    int first_fail;  // step index of the first failure (valid if fails > 0)
    int nit_max;
    int nref_max;
    int worst;       // worst step status: 0 ok, 1 iteration overflow, 2 cannot converge, 3 timed out
    int pad;
    long long nit_sum, nref_sum;
    double v2max;    // max over steps of max |v|^2 / gamma0^2 (bit pattern compared as unsigned)
};

// Grid-wide barrier state of the persistent kernels (bounded wait, no hang).
struct GridBar {
    unsigned int count;
    unsigned int gen;
    int err;
    int pad;
};

// Arguments of the FP64 BiCGSTAB persistent kernel (bicg_dir, src/algebra/bicg.h:163-234).
struct BicgArgs {
    int nn;
    const int *Sptr, *Scol;
    const double *Sval, *A, *Dl, *ep, *eq;
    const unsigned char *mag;
    double c0;
    const double *b;
    double *x, *r, *rt, *p, *v, *s, *t, *phat, *shat, *Minv, *W;
    double *partial;
    GridBar *bar;
    SolveResult *res;
    double tol;
    int maxiter;
    // fused node update (Node::make_evol, src/node.h:116-122)
    double dt;
    const double *u0;
    double *u1, *v1;
    // batch of independent samples (k_bicg64_seg): sample g owns nodes
    // [seg_node[g], seg_node[g+1]) and blocks [seg_blk[g], seg_blk[g+1]), its own dt and c0
    int nseg;
    const int *seg_node, *seg_blk;
    const SegPar *seg;
    SegAcc *acc;          // per-sample accumulation over a run (nullable)
    const int *step_ctr;  // step index of the run (with acc)
};

// Arguments of the FP32 inner Krylov solve with FP64 iterative refinement.
struct MixedArgs {
    int nn;
    const int *Sptr, *Scol;
    const double *Sval, *A, *Dl, *ep, *eq;  // FP64 operator (refinement residual)
    const float *Sval32, *A32;              // static FP32 copies (A32 = A * scale)
    float *ep32, *eq32, *Dl32, *Minv32;     // per-step FP32 copies, written in phase 0
    const unsigned char *mag;
    double c0;
    const double *b;
    double *x, *r64, *W64;
    float *r, *rt, *p, *v, *s, *t, *phat, *shat, *d, *W32;
    double *partial;
    GridBar *bar;
    SolveResult *res;
    double tol, inner_tol;
    int maxiter, refine_max;
    double dt;
    const double *u0;
    double *u1, *v1;
    double scale;  // 1/mean(A): the FP32 system is scale*K, entries O(1)
    // batch of independent samples: sample g owns nodes [seg_node[g], seg_node[g+1]) and
    // blocks [seg_blk[g], seg_blk[g+1]); each sample runs its own Krylov scalars and stops
    // on its own residual (nseg == 1: one system over all nodes and blocks)
    int nseg;
    const int *seg_node, *seg_blk;
    const SegPar *seg;    // per-sample dt and c0 (nullptr: the scalars above)
    SegAcc *acc;          // per-sample accumulation over a run (nullable)
    const int *step_ctr;  // step index of the run (with acc)
    // learned initial guess (single system): a candidate x and its tangent vectors beside
    // the fallback in x; the first refinement residual is formed for both and the smaller
    // one wins (cand_flag 1: the candidate), cand_res2 = {|r_cand|^2, |r_fallback|^2}
    double *cand_x, *cand_W;
    double *cand_r;       // the candidate's residual [2 nn]
    int *cand_flag;
    double *cand_res2;
    // with cand_o set, phase 0 forms the candidate itself (into cand_x / cand_W) from the
    // network's outputs cand_o [nn][3]: their mean over the node and its magnetic neighbours
    // times cand_scale, added to the extrapolation 2 v_prev - cand_vprev2 (v_prev = u0's v,
    // cand_vprev), projected on the new basis
    const float *cand_o;
    const double *cand_vprev, *cand_vprev2, *cand_scale;
};

struct Ctx {
    int device = 0, nsm = 0;
    cudaStream_t stream = nullptr;   // every launch of the context (highest priority)
    cudaStream_t stream2 = nullptr;  // the FMM near field beside the far field (lowest priority)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    fg_opts opts{};
    std::string err;

    int nn = 0;        // nodes
    int nmt = 0;       // magnetic tetrahedra
    int nft = 0;       // magnetic (charge-carrying) triangles
    int npi_t = 5, npi_f = 4;
    int nsrc = 0;      // Gauss-point sources
    int n_tets_total = 0;
    double total_mag_vol = 0;
    double mean_A = 0;
    bool aniso = false;  // some magnetic region has K != 0 or K3 != 0
    double ms_ref = 1.0; // largest Ms of the magnetic regions (feature scale of the learned guess)

    std::vector<unsigned char> h_mag;
    std::vector<double> h_xyz;

    // device: static mesh data
    double *xyz = nullptr;
    int4 *tet = nullptr;        // magnetic tets
    double *da = nullptr;       // 12 x nmt (structure of arrays)
    double *detJ = nullptr;     // nmt
    int *treg = nullptr;        // nmt
    DevRegion *regs = nullptr;
    int nreg = 0;
    unsigned char *mag = nullptr;
    int *inc_ptr = nullptr, *inc = nullptr;      // node -> tet slots
    int *Sptr = nullptr, *Scol = nullptr;         // static stiffness pattern (with diagonal)
    double *Sval = nullptr;
    float *Sval32 = nullptr;
    int nnzS = 0;
    double *A = nullptr;        // lumped mass per node
    double *Ainv = nullptr;     // 1 / A on the magnetic nodes, 0 elsewhere
    float *A32 = nullptr;
    int4 *tri = nullptr;        // magnetic triangles: 3 nodes + index
    DevTri *tri_c = nullptr;
    int *tinc_ptr = nullptr, *tinc = nullptr;    // node -> tri-vertex slots
    double *src_xyz = nullptr;  // nsrc x 3, magTet*npi then magTri*npi_f
    int *mag_nodes = nullptr;   // list of magnetic nodes
    int n_mag_nodes = 0;

    // device: state (interleaved xyz per node)
    double *u[2] = {nullptr, nullptr}, *v[2] = {nullptr, nullptr};
    double *phi[2] = {nullptr, nullptr}, *phiv[2] = {nullptr, nullptr};
    double *ep = nullptr, *eq = nullptr;
    float *ep32 = nullptr, *eq32 = nullptr, *Dl32 = nullptr;

    // device: per step
    double4 *slot = nullptr;    // 4 x nmt: (lumped alpha, BE)
    double *Dl = nullptr;       // nn
    double *rhs = nullptr, *x = nullptr;  // 2 nn
    double *bv = nullptr;       // 10 x 2nn FP64 BiCG vectors
    double *W = nullptr;        // 3 nn
    float *fv = nullptr;        // FP32 vectors
    double *partial = nullptr;  // reductions
    int partial_len = 0;
    GridBar *bar = nullptr;
    SolveResult *dres = nullptr;
    SolveResult *hres = nullptr;  // pinned
    int *hflag = nullptr;         // pinned copy of the FMM error flag

    // device: demag
    std::vector<double> h_src_xyz;  // source points (original order), host copy for the FMM tree
    int nseg = 1;                   // independent samples packed in this context
    // FMM set-up in fg_create: wall time of the whole set-up (tree builds, table uploads, the
    // depth autotune's evaluations), of the tree builds alone, and device time of the Morton
    // key and radix-sort kernels
    double fmm_setup_ms = 0.0, tree_wall_ms = 0.0, tree_sort_ms = 0.0;
    std::vector<int> h_src_seg, h_node_seg;  // sample of every source / node (empty: one sample)
    int *src_dst = nullptr;      // original source index -> storage position (FMM order)
    void *fmm = nullptr;         // FMM tree and buffers (fg_fmm.cu)
    double *src_q = nullptr;
    double *src_q2 = nullptr;    // charges of v (demag of m and v evaluated together), or nullptr
    double *tri_slot = nullptr;  // 3 x nft corrections
    double *tri_slot2 = nullptr; // 3 x nft corrections of src_q2
    double *tri_be = nullptr;    // 9 x nft surface-anisotropy BE per (triangle, vertex), or nullptr (all Ks = 0)
    // space-dependent applied field (the reference's R4toR3 field type): H(g) = Hext + amp F(g)
    // at every Gauss point g of every magnetic tet; F is [nmt][npi_t][3] or nullptr
    double *hsp = nullptr;
    double field_amp = 1.0;
    // recentering drift of the element integrals (fg_set_drift): direction 0/1/2 or -1, speed
    int drift_dir = -1;
    double drift_v = 0.0;
    // spin accumulation (fg_spin.cu): solver state and the last solution s [3 nn]
    void *spin = nullptr;
    double *spin_s = nullptr;
    bool spin_timed = false;  // ev[6] / ev[7] bracket the last spin solve
    void *recenter = nullptr;  // nearest-node grid for recentering (fg_recenter.cu), built on first use
    // double-single element integrals (fg_elem_ds.cu): da [12][nmt], detJ * 2^DS_SLOT_SCALE,
    // per-step double-single copies of u, phi, phiv of CURRENT
    bool elem_ds = false;
    float2 *da_ds = nullptr, *J_ds = nullptr, *state_ds = nullptr;
    float4 *tri_ds = nullptr;  // energies: per triangle normal and 0.5 mu0 dMs w_g as double-single pairs
    double *pot = nullptr;       // nn
    double *pot2 = nullptr;      // nn, potential of src_q2
    // incremental demag of the FP32 + refinement path (fg_opts.demag_increment): NEXT's
    // potentials = CURRENT's + the potentials of NEXT - CURRENT (the potential is linear in
    // the field), the FP32 FMM acting on the change only, the sum kept in FP64
    bool dinc = false;
    bool dinc_valid[2] = {false, false};  // phi / phiv of CURRENT are the potentials of u / v
    float *dstate32 = nullptr;           // NEXT - CURRENT in FP32: u [3 nn], then v [3 nn]
    float *da32 = nullptr, *cq32 = nullptr;  // FP32 da [12][nmt] and -Ms detJ [nmt] (incremental demag)
    float *src_qf = nullptr, *src_q2f = nullptr;  // FP32 charges of the change (FMM leaf order)
    float4 *tri32 = nullptr;  // per triangle n, dMs w_g, dMs beta in FP32 (charges of the change)
    bool charges32 = false;              // the FMM evaluation reads src_qf / src_q2f
    void *fmm64 = nullptr;               // FP64 tree at the FP32 tree's depth, built on first use
    double *epart = nullptr;     // energy partials
    double *hepart = nullptr;    // pinned
    int epart_blocks = 0;

    // persistent-kernel launch shapes
    int bicg_grid = 0, bicg_block = 256;
    int mixed_grid = 0;
    int mixed_threads = 256;  // threads per block of the single-system solver (256 or 512)
    int lpr = 0;  // lanes per row of the mixed solver's operator applications (0: not chosen yet)

    // timings
    cudaEvent_t ev[8];
    float ms[5] = {0, 0, 0, 0, 0};
    bool step_open = false;  // ev[0] recorded by a step not yet closed by compute_all
    long long launches = 0;  // kernels launched by this context
    void *mlp = nullptr;     // learned initial guess (fg_mlp.cu)
    // a candidate guess for the next FP32 + refinement solve to judge (set by the learned guess)
    double *cand_x = nullptr, *cand_W = nullptr;
    double *cand_r = nullptr, *cand_res2 = nullptr;
    int *cand_flag = nullptr;
    const float *cand_o = nullptr;  // the solver forms the candidate from these network outputs
    const double *cand_vprev = nullptr, *cand_vprev2 = nullptr, *cand_scale = nullptr;
    NodeFeat node_feat{nullptr, 0.0, 0.0};  // features the next node kernel forms

    // batch of independent samples packed as one block-diagonal system (fg_batch_*)
    bool batch = false;
    std::vector<int> h_seg_node, h_seg_tet, h_seg_tri;  // nseg+1 offsets (nodes, magnetic tets / tris)
    std::vector<int> h_seg_blk;                         // nseg+1 block offsets of the persistent solver
    int seg_grid = 0;                                   // blocks of the segmented persistent solver
    int *tet_seg = nullptr, *node_seg = nullptr;        // sample of every magnetic tet / node
    int *d_seg_node = nullptr, *d_seg_blk = nullptr;
    SegPar *seg_par = nullptr;                          // current step's per-sample parameters
    SegPar *hseg_par = nullptr;                         // pinned staging
    SegPar *seg_sched = nullptr;                        // schedule of a multi-step run
    long long seg_sched_len = 0;
    int *step_ctr = nullptr;
    SegAcc *seg_acc = nullptr, *hseg_acc = nullptr;
    SegAcc *acc_active = nullptr;                       // set while a run is launched
    int4 *eblk_rng = nullptr;                           // energy blocks: tet and tri ranges
    int *eblk_seg = nullptr, *d_seg_eblk = nullptr;
    int eblk_n = 0;
    double *seg_H = nullptr, *hseg_H = nullptr;         // per-sample field of the energy
    double *seg_epart = nullptr, *seg_energy = nullptr, *hseg_energy = nullptr;
    cudaGraphExec_t graph = nullptr;                    // captured step + compute_all of a run
    int graph_state = 0;                                // 0 not tried, 1 captured, -1 capture refused
    bool run_graph = false;                             // the last run replayed the graph
    bool graph_mlp = false;                             // the captured step runs the learned guess's inference
    float run_ms = 0.f;                                 // device time of the last run
};

// kernels (fg_kernels.cu)
cudaError_t launch_tet(Ctx &c, double dt, const double Hext[3]);
cudaError_t launch_node(Ctx &c, double angle);
cudaError_t launch_bicg64(Ctx &c, double dt, double prefactor);
cudaError_t launch_mixed(Ctx &c, double dt, double prefactor);
cudaError_t launch_apply(Ctx &c, double c0, const double *x, double *y);
// set 0: charges into src_q / tri_slot, potential from pot; set 1: src_q2 / tri_slot2 / pot2
cudaError_t launch_charges(Ctx &c, const double *m, int set = 0);
cudaError_t launch_charges_pair(Ctx &c, const double *m, const double *v);  // sets 0 and 1 in one pass
cudaError_t launch_p2p_direct(Ctx &c);
// phi_out = base + (pot + corr) / (4 pi) (base nullptr: no base)
cudaError_t launch_phi_final(Ctx &c, double *phi_out, int set = 0, const double *base = nullptr);
cudaError_t launch_state_diff(Ctx &c);  // dstate32 = NEXT - CURRENT for u and v (FP32)
cudaError_t launch_charges32(Ctx &c, int nq);  // FP32 charges of dstate32 (incremental demag)
cudaError_t launch_energy(Ctx &c, const double Hext[3]);
cudaError_t launch_energy_into(Ctx &c, const double Hext[3], double *partial);
int bicg_grid_size(Ctx &c, bool mixed);
cudaError_t morton_sort(Ctx &c, int n, int L, int nseg, const double *xyz, const int *seg,
                        const std::vector<double4> &roots, const unsigned char *keep, std::vector<uint64_t> &keys,
                        std::vector<int> &idx, double *dev_ms);
int bicg_seg_max_blocks(Ctx &c);  // co-resident blocks of the batched FP64 solver
int mixed_grid_size(Ctx &c);
int mixed_max_blocks(Ctx &c);
// Chooses the lanes per row of the mixed solver (opts.solver_lpr, or the fastest of 1, 4, 8
// timed on the current step's system) and, for a single system, its grid size (all
// co-resident blocks, 2 or 1 per SM); the node kernel is rerun before each timing.
cudaError_t mixed_autotune(Ctx &c, double dt, double prefactor, double angle);
// failure-path probes: a bounded device wait that nothing ends (*out / *err set on expiry)
cudaError_t launch_barrier_timeout_probe(Ctx &c, int *out);
cudaError_t launch_mbar_timeout_probe(cudaStream_t st, int *err);
// throughput probe of tcgen05.mma kind::tf32 (M = 128, N = n, K = 8), one CTA per SM
cudaError_t launch_peak_mma_tf32(cudaStream_t st, int grid, int n, int iters, long long *cyc, int *err);
int fmm_info(const Ctx &c, int *L, int *nleaf, double *n_m2l, double *n_p2p);
int *fmm_error_flag(const Ctx &c);
cudaError_t fmm_eval(Ctx &c, int nq = 1);  // nq 2: c.src_q2 -> c.pot2 beside c.src_q -> c.pot
// The same evaluation with an FP64 tree of the FP32 tree's depth (built on first use; the
// FP32 tree itself when the context is FP64); FG_* status
int fmm_eval_fp64(Ctx &c, int nq);
void fmm64_free(Ctx &c);
int fmm_launches_per_eval(const Ctx &c, int nq = 1);  // kernels one FMM evaluation launches  // device int: FG_ETIMEDOUT after an expired wait (or nullptr)
// tensor-core translations (fg_fmm_tc.cu)
int translate_tc_smem();
int translate_tc_tile();  // output cells per tile of the tensor-core translations
cudaError_t translate_tc_setup();
// out (+)= sum_code Op[code] in[tab[cell][code]] over n_out cells from out0 (FP32 path)
struct TcArgs {
    int n_out, out0, ncode;
    const int *tab;                 // [cell][ncode] input cell or -1
    const unsigned char *op_img;    // translate_tc_images of the operators
    const float *in_hi, *in_lo;     // inputs split hi = tf32(x), lo = x - hi
    float *out, *out_hi, *out_lo;   // outputs and their split
    int accumulate;                 // 1: out += result
    const int *tile_code;           // codes that reach each tile of 64 cells, tile after tile
    const int4 *units;              // per CTA: tile, first and end index into tile_code, scratch slot
    int nunits;                     //   (slot -1: the tile's only unit, which writes the output)
    float *scratch;                 // [slot][64][100] partial results of tiles split over units
    const int4 *comb;               // per split tile: tile, first slot, number of slots
    int ncomb;
    int *err;                       // FG_ETIMEDOUT after an expired wait
    int terms;                      // product terms of the split (7 in production)
    int nset;                       // sets of expansions (at most 2, columns of one MMA; 0 or 1: one)
    size_t set_io, set_scratch;     // floats between sets in in/out arrays and in scratch
};
cudaError_t launch_translate_tc(cudaStream_t st, const TcArgs &a);
std::vector<float> translate_tc_images(const std::vector<double> &ops, int ncode);
// Work units of one translation launch: the codes reaching each tile of 64 output cells,
// split into units of at most max_codes codes (appended to codes/units/comb; nslot grows).
void translate_tc_units(int n_out, int ncode, const int *tab, int out0, int max_codes, std::vector<int> &codes,
                        std::vector<int4> &units, std::vector<int4> &comb, int &nslot);
int fmm_stage_ms(const Ctx &c, double ms[5]);
int mlp_create(Ctx &c);
void mlp_free(Ctx &c);
cudaError_t mlp_before_solve(Ctx &c, double c0, bool use, bool train);
cudaError_t mlp_train(Ctx &c);
void mlp_sample_flags(const Ctx &c, int g, int *accepted, double *res0_mlp, double *res0_prev);
cudaError_t mlp_before_sync(Ctx &c);
void mlp_after_sync(Ctx &c, int *accepted, double *res0_mlp, double *res0_prev, double *loss);
long long mlp_steps(const Ctx &c);
cudaError_t mlp_before_evolution(Ctx &c);
double mlp_loss(const Ctx &c);
int mlp_debug_grad(Ctx &c, int nsamples, const float *hx, const float *hy, float *w_out, float *g_out, float *loss);
int mlp_nparam();
int mlp_debug_infer(Ctx &c, int n, const float *hx, float *hy);
bool mlp_take_timeout(Ctx &c);  // a tensor-core wait of the learned guess expired (then cleared)
NodeFeat mlp_node_features(Ctx &c);  // where the node kernel writes the learned guess's features
int batch_setup(Ctx &c, const std::vector<int4> &htet, const std::vector<int4> &htri);
void batch_free(Ctx &c);
int spin_setup(Ctx &c, const fg_mesh *m, const fg_region *regs, int nreg, const fg_tri_region *tregs, int ntreg,
               std::vector<DevRegion> &hreg);
void spin_free(Ctx &c);
cudaError_t launch_spin(Ctx &c);
int spin_info(const Ctx &c, int *status, int *iters, double *V, int *v_iters);
int recenter_apply(Ctx &c, int dir, double threshold, double avg_dir, int *shifted);
int elem_ds_setup(Ctx &c, const std::vector<double> &da, const std::vector<double> &detJ);
void upload_rules_ds(const double ta[4][5], const double tp[5]);
cudaError_t launch_tet_ds(Ctx &c, double dt, const double H[3]);
cudaError_t launch_state_ds(Ctx &c, const double *u, const double *phi, const double *phiv);
inline bool drift_on(const Ctx &c) { return c.drift_dir >= 0 && c.drift_v != 0.0; }
inline bool use_elem_ds(const Ctx &c) { return c.elem_ds && !c.hsp && !drift_on(c); }
void recenter_free(Ctx &c);
cudaError_t launch_select_params(Ctx &c);
cudaError_t launch_advance(Ctx &c);
cudaError_t launch_energy_seg(Ctx &c);

}  // namespace fg

// The opaque handle of the C ABI.
struct fg_ctx {
    fg::Ctx c;
    double last_c0 = 0.0;
    int solves_since_train = 0;  // learned guess: successful solves since the last training step
};
