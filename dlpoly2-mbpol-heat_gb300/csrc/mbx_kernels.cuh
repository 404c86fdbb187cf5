// Internal declarations shared by the MB-pol CUDA translation units.
#pragma once

#include "mbx_common.cuh"
#include "mbx_spme.cuh"

#include <functional>
#include <vector>

namespace mbx {

// Accumulator slots of the per-evaluation scalar buffer (double, device).
enum Slot {
    S_E2 = 0,       // 2B energy (internal units)
    S_E3 = 1,       // 3B energy
    S_VIR = 2,      // virial sum w.g (internal units)
    S_STRESS = 3,   // 9 stress components (3..11)
    S_JPOT = 12,    // 3 heat-current jpot components (12..14)
    S_JKIN = 15,    // 3 heat-current jkin components (15..17)
    S_NSLOTS = 18
};

// Device inputs/outputs of one MB-pol evaluation.
struct MbpolArgs {
    int nw;
    Cell cell;
    const int* list;                 // listttm2, 1-based, 3*nw
    const double *x, *y, *z;         // raw positions (heat current uses these)
    const double *vx, *vy, *vz;      // velocities or null
    const double* mono;              // imaged monomers, 9 per water
    double *fx, *fy, *fz;            // forces, accumulated
    double* ae;                      // per-atom energy, accumulated (may be null)
    double* acc;                     // S_NSLOTS scalars, accumulated
    // several boxes in one launch (null for one box): cell of box b, box of water i,
    // and per-box accumulators acc_box[b * S_NSLOTS + slot]
    const Cell* cells = nullptr;
    const int* wbox = nullptr;
    double* acc_box = nullptr;
};

// Mixed-precision pass: FP32 kernels hand ill-conditioned clusters (a shifted
// variable further than limit2/limit3 from its centre) to an FP64 kernel through
// these device lists; count[0] dimers, count[1] trimers (zeroed by the caller).
struct MixedPass {
    int2* hard2;
    int4* hard3;
    int* count;
    float limit2, limit3;
};

// Fused cluster kernels (mbx_mbpol.cu).  precision: 0 FP64, 1 mixed.
cudaError_t launch_2b(const MbpolArgs& a, const int2* pairs, int npairs, int precision, const MixedPass& mp,
                      cudaStream_t s);
cudaError_t launch_3b(const MbpolArgs& a, const int4* trip, int ntrip, int precision, const MixedPass& mp,
                      cudaStream_t s);
// The same with the cluster count on the device (`n_dev`) and the grid sized for `cap`
// clusters: no host synchronisation between list building and evaluation.
cudaError_t launch_2b_dev(const MbpolArgs& a, const int2* pairs, long cap, const int* n_dev, int precision,
                          const MixedPass& mp, cudaStream_t s);
cudaError_t launch_3b_dev(const MbpolArgs& a, const int4* trip, long cap, const int* n_dev, int precision,
                          const MixedPass& mp, cudaStream_t s);
// Both bodies of the mixed method in one persistent launch of `nsm` blocks (one per
// SM): the dimers and trimers are claimed in chunks through ctr[2] (device ints, zeroed
// here).  Counts are n2/n3, or read from n2_dev/n3_dev when those are not null.
// Applies to the default mixed split only (fused_applies); otherwise launch_2b/3b.
// With `partial` (dimer_parts() * 32 doubles per dimer) and `done` (one int per dimer),
// both for part_cap dimers (done is zeroed here), every FP64 dimer is split into
// dimer_parts() tasks, one polynomial chunk each, so the FP64 work is claimed in finer
// pieces; with more dimers than part_cap, or null buffers, one task per dimer.
bool fused_applies(int precision, const MixedPass& mp);
int dimer_parts();
cudaError_t launch_23(const MbpolArgs& a, const int2* pairs, int n2, const int* n2_dev, const int4* trip, int n3,
                      const int* n3_dev, int precision, int* ctr, int nsm, cudaStream_t s,
                      double* partial = nullptr, int* done = nullptr, long part_cap = 0, int dimer_warps = 0,
                      bool shared_sm = false);
// Isolated polynomial + model evaluation for explicit clusters (the per-call ABI).
cudaError_t launch_2b_direct(int n, const double* w1, const double* w2, double* E, double* g1, double* g2,
                             int precision, cudaStream_t s);
cudaError_t launch_3b_direct(int n, const double* w1, const double* w2, const double* w3, double* E,
                             double* g1, double* g2, double* g3, int precision, cudaStream_t s);
// The force matrices of the per-cluster C entry points (FP64): 108 doubles per dimer, 243
// per trimer, entries written as the reference writes them (the rest left as they are).
cudaError_t launch_2b_fm(int n, const double* w1, const double* w2, double* fm, cudaStream_t s);
cudaError_t launch_3b_fm(int n, const double* w1, const double* w2, const double* w3, double* fm, cudaStream_t s);
// Path-integral bead coupling (mbx_pimd.cu): the normal-mode matrices of
// SOURCE/centroid_matrix.f (nmode_to_cart[bead][mode], cart_to_nmode[mode][bead], lambda),
// the transform out = A in over P beads of m values, and the spring forces of
// SOURCE/centroid_spring_force.f (acc[0] += sum m |d2|^2, acc[1] += sum -d1 . f).
void pimd_matrices(int P, bool langevin, std::vector<double>& n2c, std::vector<double>& c2n,
                   std::vector<double>& lam);
int pimd_max_beads();
cudaError_t launch_pimd_transform(int P, long m, const double* A, const double* in, double* out, cudaStream_t s);
cudaError_t launch_pimd_springs(int P, int n, const double* c2n0, const double* x, const double* y, const double* z,
                                double* fx, double* fy, double* fz, const double* mass, double coeff, double fac1,
                                double fac3, double* acc, cudaStream_t s);
// jkin = sum_i (K_i + U_i) v_i over the water atoms (SOURCE/heatcurrent.f90:713-716).
cudaError_t launch_jkin(int nwat_atoms, const double* vx, const double* vy, const double* vz,
                        const double* mass, const double* ae, double* acc, cudaStream_t s);

// 1-body PS PES over H-O-H angles (mbx_pes.cu); acc14 = {E, virial, stress[9], jpot[3]}.
cudaError_t launch_ps_pes(int nang, const int* listang, const Cell& cl, const double* x, const double* y,
                          const double* z, double* fx, double* fy, double* fz, double* ae, const double* vx,
                          const double* vy, const double* vz, double* acc14, cudaStream_t s);

// The same over the waters of many boxes: angle t belongs to box abox[t], with cell
// cells[box] and accumulators acc14_box[14 * box ..]; nothing is done when *skip != 0.
cudaError_t launch_ps_pes_boxes(int nang, const int* listang, const Cell* cells, const int* abox, const double* x,
                                const double* y, const double* z, double* fx, double* fy, double* fz, double* ae,
                                const double* vx, const double* vy, const double* vz, double* acc14_box,
                                const int* skip, cudaStream_t s);

// M sites written into x/y/z at index listttm2[3nw-1] + i (0-based) and DMS charges
// into chge (H1, H2, M) and dp[6*nw] (mbx_pes.cu); chge/dp may be null.
cudaError_t launch_msites_dms(int nw, const int* list, const Cell& cl, double* x, double* y, double* z, double gamma,
                              double* chge, double* dp, cudaStream_t s);

// Dimer list from the per-water partner lists: pairs[off2[i] + q] = (i, l2[i*cap2 + q]).
void launch_pairs_compact(int nw, int cap2, const int* n2, const int* off2, const int* l2, int2* pairs,
                          cudaStream_t s);

__global__ void k_list_totals(int nw, const int* n2, const int* off2, const int* tcnt, const int* toff,
                              const int* flag, int* totals);

// Cell-list builder of the dimer and trimer lists (mbx_lists.cu).
struct ListBuilder {
    int cap2 = 64;      // dimer partners j > i per water
    int cap3 = 48;      // 3B neighbours per water
    int cap2_alloc = 0, cap3_alloc = 0;
    int nw_cap = 0, ncell_cap = 0;
    unsigned *key = nullptr, *skey = nullptr;
    int *idx = nullptr, *sidx = nullptr, *cstart = nullptr, *cend = nullptr;
    int *n2 = nullptr, *l2 = nullptr, *off2 = nullptr, *n3 = nullptr, *l3 = nullptr;
    int *tcnt = nullptr, *toff = nullptr, *flag = nullptr;
    float4* of = nullptr;   // FP32 copies of the imaged O positions (list pre-tests)
    void *scan_tmp = nullptr, *sort_tmp = nullptr;
    size_t scan_bytes = 0, sort_bytes = 0;
    int3 nc_last = {1, 1, 1};
    int all_pairs_last = 1;
    long launches_last = 0;  // kernels launched by the last phase1 + phase2 (CUB included)
    // external = true: the buffers above were set by the caller (fixed capacities, no
    // allocation, no cell sort: candidates are all waters); reserve() only checks sizes
    bool external = false;

    ~ListBuilder();
    void release();
    cudaError_t reserve(int nw, int ncell);
    // totals_dev[0] = #pairs, [1] = #trimers, [2] = overflow flag
    cudaError_t phase1(int nw, const int* list, const double* x, const double* y, const double* z, const Cell& cl,
                       double* mono, int* totals_dev, cudaStream_t s);
    cudaError_t phase2(int nw, const Cell& cl, const double* mono, int2* pairs, int4* trip, cudaStream_t s);
};

// Short-range dispersion, DL_POLY vdw type 12 (mbx_disp.cu): tables, Verlet list with
// skin, forces.  Types are 1-based (0: none), prm holds {C6, a6, C8, a8} per pair type
// (pair i >= j at i(i-1)/2 + j - 1); atoms of the same molecule do not interact.
struct DispState {
    int ntypes = 0, mxgrid = 0;
    double rcut = 0.0, delr = 0.0;
    std::vector<double> prm;
    double *vvv = nullptr, *ggg = nullptr;       // tables [pair][mxgrid]
    float *vvv32 = nullptr, *ggg32 = nullptr;    // their FP32 copies (one allocation at vvv32)
    float4* vf = nullptr;                        // FP32 velocities of the mixed form
    int vf_cap = 0;
    unsigned vdw_types = 0;
    unsigned long long vdw_pairs[3] = {0, 0, 0};
    int cap = 512, cap_alloc = 0;                // list partners j > i per atom
    int *nn = nullptr, *nbr = nullptr, *flag = nullptr;
    double* xref = nullptr;                      // positions at the last build (x, y, z blocks)
    unsigned *key = nullptr, *skey = nullptr;
    int *idx = nullptr, *sidx = nullptr, *cstart = nullptr, *cend = nullptr;
    void* sort_tmp = nullptr;
    size_t sort_bytes = 0;
    int natms_cap = 0, ncell_cap = 0;
    bool valid = false;                          // the list matches the inputs below
    int natms_last = 0, imcon_last = 0;
    const int *ltype_last = nullptr, *mol_last = nullptr;
    double cell_last[9] = {0};
    long builds = 0, launches = 0;

    ~DispState();
    void release();
    cudaError_t setup(int ntypes, const double* prm, double rcut, double delr, int mxgrid);
    cudaError_t forces(const Cell& cl, int natms, const int* ltype, const int* mol, const double* x,
                       const double* y, const double* z, double* fx, double* fy, double* fz, const double* vx,
                       const double* vy, const double* vz, double* ae, double* out14, int* flag_host,
                       cudaStream_t s, bool* rebuilt, bool fp32 = false);   // fp32: the mixed form
};
// TTM4-F polarizable electrostatics of MB-pol water (mbx_polar.cu): the reference's polar
// Ewald branch (rfield, ewald1p, iter, coulomb_polar, ewald2p, ewald3p, qdforce) with its
// heat-current terms, on 4 * nw sites in the standard layout.
struct PolarState {
    int cap = 512, cap_alloc = 0;          // list partners per site
    int n_cap = 0, nw_cap = 0, k_cap = 0;
    size_t eik_cap = 0;
    int mxegrd = 0;
    double drewd = 0.0, tab_alpha = -1.0, tab_rcut = -1.0;
    double4* ercp = nullptr;               // erfcgenp table, rows 0..mxegrd
    float4* ercp32 = nullptr;              // its screened functions C_n in FP32 (mixed-path ewald2p)
    bool ewald2p_fp64 = false;             // mixed path: keep ewald2p's pair terms in FP64
    // mixed path: the final pass (forces, energies, virial, heat current of the converged
    // dipoles) in FP64 as in the FP64 method; the solve stays mixed
    bool final_fp64 = false;
    // Verlet skin of the site pair list (0: the list is rebuilt at every call): the pairs
    // within rcut + list_skin, kept until a site moved more than list_skin / 2
    double list_skin = 1.0;
    int *nn_s = nullptr, *nbr_s = nullptr, *npol_s = nullptr;
    int2* nup_s = nullptr;
    int cap_s = 768, cap_s_alloc = 0, ns_cap = 0;
    double* xref = nullptr;                // positions at the skin list's build (x, y, z blocks)
    bool skin_ok = false;
    int skin_n = 0, skin_imcon = 0;
    double skin_rcut = 0.0, skin_delr = 0.0, skin_cell[9] = {};
    long list_builds = 0;
    int last_n = 0;                        // sites of the last call (the pair list's rows)
    int *nn = nullptr, *nbr = nullptr, *flag = nullptr;
    int* npol = nullptr;                   // per row: the polarizable partners, first in the row
    int2* nup = nullptr;                   // per row: partners j > i heading each group (pol, other)
    float4* xf = nullptr;
    double* tens = nullptr;                // dipole tensors of the list pairs (6 blocks)
    double* intra = nullptr;               // intramolecular O/H dipole tensors (18 per water)
    double* fld = nullptr;                 // efk, efc, emu, efm (3 blocks of n each)
    double *vesp = nullptr, *ae = nullptr;
    double* polr6 = nullptr;               // polr^(1/6) per site
    // cell list of the pair-list build: sort keys and indices, radix-sort scratch, bounds
    unsigned *ckey = nullptr, *cskey = nullptr;
    int *cidx = nullptr, *csidx = nullptr, *cstart = nullptr, *cend = nullptr;
    void* csort = nullptr;
    size_t csort_bytes = 0;
    int cell_n_cap = 0, ncell_cap = 0;
    double2* eik = nullptr;                // exp(ik.r) [k][site]
    double2* fac = nullptr;                // per-site phase factors per axis and index
    size_t fac_cap = 0;
    double4* md = nullptr;                 // dipoles of the polarizable sites
    double* vh = nullptr;                  // per-site products of the ew1p heat sums (12 per site)
    double* kco = nullptr;                 // per-k coefficients of the gathers
    // mixed precision: FP32 tensors, axis factors and correction solve
    float* tens32 = nullptr;
    float2* fac32 = nullptr;               // FP32 copy of fac (the FP32 k-space passes form their phases)
    int4* ktile = nullptr;                 // per 256 k vectors: first (l, m) column, columns
    int4* kaux = nullptr;                  // per k: column in its tile, next column, column, z offset
    int* kcol = nullptr;                   // per (l, m) column: l << 16 | y row
    int2* colk = nullptr;                  // per (l, m) column: first k vector, count
    std::vector<int2> hcolk;
    std::vector<int4> hktile, hkaux;
    std::vector<int> hkcol;
    int ktile_cap = 0;
    float* kco32 = nullptr;
    float4 *r32 = nullptr, *d32 = nullptr, *cg_x = nullptr, *cg_r = nullptr, *cg_q = nullptr;
    float4* vh32 = nullptr;                // FP32 heat weights of the final pass (3 per site)
    float4* cg_z = nullptr;                // preconditioned residual of the correction solve
    int precond_sweeps = 0;                // Jacobi sweeps of the CG preconditioner (odd; 1: diagonal
                                           // only; 0: 1 with SPME, 3 with the Ewald sum)
    bool precond_block = true;             // the per-water block-Jacobi preconditioner instead
    float* binv = nullptr;                 // its 9x9 inverses (81 floats per water)
    int binv_cap = 0;
    float* e32 = nullptr;
    int cap32 = 0, n32 = 0, k32 = 0;
    size_t fac32_cap = 0;
    long inner_sweeps = 0;                 // FP32 conjugate-gradient iterations of the last call
    int cg_hint = 8;                       // sweeps the last correction solve took (first batch size)
    double* kpart = nullptr;               // per-chunk partial sums of the k-space gathers
    size_t part_cap = 0;
    int nsm = 152;                         // SMs of the device (grid sizing)
    bool profiling = false;                // record the phase times below
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    float phase_ms[4] = {0, 0, 0, 0};      // setup (lists, static fields, phases), dipole solve,
                                           // final structure factors, rest of the final pass
    long K_last = 0;                       // k vectors of the last call
    static constexpr int kKfEvents = 16;
    cudaEvent_t kfev[kKfEvents][2] = {};   // profiling: around the FP64 field gathers (k_pol_kfield)
    float kf_ms = 0.f;                     // their device time, algorithmic flops and launches
    double kf_flops = 0.0;
    long kf_launches = 0;
    double4* kv = nullptr;                 // kx, ky, kz, akk
    double2* kx2 = nullptr;                // rksq, akv2
    int4* lmn = nullptr;
    double *sf = nullptr, *kterm = nullptr, *acc = nullptr, *acc_h = nullptr;
    std::vector<double4> hk;
    std::vector<double2> hk2;
    std::vector<int4> hlmn;
    bool converged = false;
    int iterations = 0;
    long launches = 0;
    // k space: the explicit Ewald sum of the reference (spme_order 0), or SPME of order
    // spme_order on spme_grid (or, with spme_grid[0] == 0, the smallest even 2-3-5 grid
    // with spacing <= spme_spacing along each cell width)
    int spme_order = 0;
    int spme_grid[3] = {0, 0, 0};
    double spme_spacing = 0.8;
    int spme_K_last[3] = {0, 0, 0};
    SpmeState spme;
    float spme_ms = 0.f;                   // profiling: device time of the SPME passes of the last call
    long spme_calls = 0;
    cudaEvent_t spev[2] = {nullptr, nullptr};
    // ASPC (Kolafa's always stable predictor-corrector; SOURCE/aspc.f90 and forces.f:334-366):
    // order aspc_k (2 or 4; 0: off); each call is one MD step (aspc_step, the reference's
    // nstep_for_guess); after aspc_niter steps the dipoles start from the prediction over
    // the last k+2 steps, and one corrector iteration replaces the converged solve
    int aspc_k = 0, aspc_niter = 0, aspc_step = 0;
    int aspc_n = 0, aspc_head = 0;         // sites of the history; its newest slot
    double* aspc_hist = nullptr;           // k+2 slots of 3 x aspc_n dipoles (x, y, z blocks)
    cudaError_t aspc_reset(int k, int niter);   // aspc_init: history zeroed, step count 0
    void aspc_restart();                         // nstep_for_guess = 0 (an image change)
    // Not the reference's: the initial guess of the converged solve extrapolated from the last
    // guess_order+1 steps' dipoles (0: off), the same history; the solve still iterates to toler
    int guess_order = 0;
    cudaError_t guess_reset(int order);   // history cleared, step count 0, ASPC off
    int aspc_slots() const { return aspc_k ? aspc_k + 2 : guess_order + 1; }
    cudaError_t aspc_predict(int n, double* mx, double* my, double* mz, cudaStream_t s);
    cudaError_t aspc_push(int n, const double* mx, const double* my, const double* mz, cudaStream_t s);

    ~PolarState();
    void release();
    // device bytes held by the large buffers (phase tables, pair tensors)
    size_t held_bytes() const {
        return eik_cap * sizeof(double2) + fac32_cap * sizeof(float2) + fac_cap * sizeof(double2) +
               (size_t)n_cap * cap_alloc * (6 * sizeof(double) + sizeof(int)) + (size_t)n32 * cap32 * 6 * sizeof(float) +
               part_cap * sizeof(double);
    }
    cudaError_t table(double alpha, double rcut, cudaStream_t s);
    cudaError_t reserve(int nw, int K, size_t nfac);
    cudaError_t reserve_mixed(int n, int K, size_t nfac);
    cudaError_t reserve_part(size_t ndouble);
    cudaError_t reserve_skin(int n);
    cudaError_t reserve_cells(int n, int ncell);
    // One evaluation on device arrays (precision MBX_FP64 or MBX_MIXED: the dipole
    // equations solved by FP32 corrections under FP64 refinement).  prm[15] as
    // mbx_polar_forces; forces, per-site
    // energies (ae_out, may be null), jpot and jkin are ACCUMULATED; the dipoles are
    // updated in place; out16 as mbx_polar_forces.  `converged` tells whether the dipole
    // iteration reached toler within maxit iterations.
    // Optional hooks of the mixed solve, for work the caller runs beside it: fork_hook is
    // called once, when the first FP32 CG solve is about to be enqueued (or before the final
    // pass if none is), join_hook before the final pass (the caller's work must be done
    // before it: both add to the force arrays).
    std::function<cudaError_t()> fork_hook, join_hook;
    cudaError_t run(int precision, const Cell& cl, const double* prm, int nw, const double* x, const double* y,
                    const double* z,
                    const double* q, const double* dp, const double* polr, const double* polr2, double* mx,
                    double* my, double* mz, double* fx, double* fy, double* fz, double* ae_out, const double* vx,
                    const double* vy, const double* vz, double* out16, double* jpot, double* jkin, cudaStream_t s);
};

// M-site force redistribution onto O, H1, H2 (standard layout, device arrays).
cudaError_t launch_msite_redistribute(int nw, double gamma, double* fx, double* fy, double* fz, cudaStream_t s);
// y += x on the device
cudaError_t launch_add(int n, const double* x, double* y, cudaStream_t s);

// lrcorrect for vdw type 12 (host): elrc and virlrc for numtyp[t] atoms of type t + 1.
void disp_lrc(int ntypes, const double* prm, const int* numtyp, double rcut, double volm, double* elrc,
              double* virlrc);

// Many independent water boxes evaluated by one set of launches (mbx_multi.cu).
// Box b holds nw_b waters in the standard layout (3*nw_b water atoms, O H1 H2, then
// nw_b M sites) at atom offset 4 * sum_{b'<b} nw_b'.  Every size is fixed by setup(),
// list lengths stay on the device, so enqueue() issues no host synchronisation and can
// be captured as a CUDA graph.
struct MultiBoxes {
    int cap2 = 64, cap3 = 48;     // partners / 3B neighbours per water
    int trip_per_water = 160;     // trimer capacity per water (a 4096-water liquid box has ~98)
    int nbox = 0, nw = 0, natms = 0;
    std::vector<int> nw_of_box;
    int *list = nullptr, *listang = nullptr, *wbox = nullptr, *abox = nullptr;
    unsigned char* is_water = nullptr;
    Cell* cells = nullptr;
    int *bstart = nullptr, *bcount = nullptr;
    double* mono = nullptr;
    float4* of = nullptr;          // FP32 copies of the imaged O positions (list pre-tests)
    int *n2 = nullptr, *l2 = nullptr, *off2 = nullptr, *n3 = nullptr, *l3 = nullptr, *tcnt = nullptr,
        *toff = nullptr;
    int2* pairs = nullptr;
    int4* trip = nullptr;
    long pair_cap = 0, trip_cap = 0;
    int2* hard2 = nullptr;         // mixed-path hand-off lists (allocated when a limit asks)
    int4* hard3 = nullptr;
    int* hard_count = nullptr;
    void* scan_tmp = nullptr;
    size_t scan_bytes = 0;
    double* acc_box = nullptr;     // S_NSLOTS per box
    double* pes_box = nullptr;     // 14 per box (1-body term)
    double* ae_scratch = nullptr;  // per-atom energy for the heat current when the caller passes none
    int* totals = nullptr;         // [0] dimers, [1] trimers
    int* flag = nullptr;           // bit 0: neighbour capacity, bit 1: trimer capacity
    long launches = 0;             // kernels issued by one enqueue (CUB included)
    long gen = 0;                  // bumped whenever setup() (re)allocates

    ~MultiBoxes();
    void release();
    // (re)allocate for this box layout; a no-op when the layout is unchanged
    cudaError_t setup(int nbox, const int* nw_box, bool need_hard, cudaStream_t s);
    int* ctr = nullptr;            // work counters of the persistent 2B+3B kernel
    double* partial = nullptr;     // split FP64 dimers: per-chunk [E, dE/dx] (launch_23)
    int* done = nullptr;
    long part_cap = 0;
    int nsm = 0;
    cudaError_t enqueue(int precision, const MixedPass& limits, bool fused, const double* x, const double* y,
                        const double* z,
                        double* fx, double* fy, double* fz, const double* vx, const double* vy, const double* vz,
                        const double* mass, double* ae, cudaStream_t s);
};

}  // namespace mbx

// The context's last error text (host code outside mbx_capi.cu: the i-PI driver).
struct mbx_context;
void mbx_set_error_text(mbx_context* ctx, const char* msg);
