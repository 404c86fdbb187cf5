/*
 * libmbx -- GB300-native MB-pol force and heat-current path.
 *
 * C ABI: plain pointers and sizes, no C++ types, no exceptions across the
 * boundary.  Every entry point returns an int status (MBX_OK = 0) unless it is a
 * drop-in for a reference symbol whose signature returns void.
 *
 * Units and layouts follow the reference DL_POLY 2 fork: Angstrom, DL_POLY
 * internal energy units (10 J/mol; 418.4 per kcal/mol), per-atom arrays in
 * structure-of-arrays form (xxx, yyy, zzz), water atoms 1..3*nw in (O, H1, H2)
 * triples located through the 1-based `listttm2` array, M sites after them.
 *
 * Precision modes: MBX_FP64 reproduces the reference's FP64 arithmetic;
 * MBX_MIXED evaluates each dimer/trimer in FP32 and accumulates forces,
 * energies, virial, stress and heat current in FP64.
 */
#ifndef MBX_H
#define MBX_H

#ifdef __cplusplus
extern "C" {
#endif

#define MBX_FP64 0
#define MBX_MIXED 1

#define MBX_OK 0
#define MBX_ERR_ARG 1           /* invalid argument (null pointer, bad size, bad imcon) */
#define MBX_ERR_CUDA 2          /* a CUDA call failed; see mbx_error() */
#define MBX_ERR_CAPACITY 3      /* a list outgrew the largest capacity the context allows */
#define MBX_ERR_NO_DEVICE 4     /* no CUDA device, or the device is not an sm_103 part */
#define MBX_ERR_CONVERGE 5      /* the induced dipoles did not converge within maxit iterations */

/* Scalar outputs of one evaluation (indices into the `scalars` array). */
#define MBX_S_ENG2 0            /* MB-pol 2B energy (internal units) */
#define MBX_S_ENG3 1            /* MB-pol 3B energy */
#define MBX_S_VIR 2             /* virial: sum over clusters of w . dE/dw */
#define MBX_S_STRESS 3          /* 9 stress components, DL_POLY order (3..11) */
#define MBX_S_JPOT 12           /* heat current, potential part jpot (12..14) */
#define MBX_S_JKIN 15           /* heat current, kinetic+energy part jkin (15..17) */
#define MBX_NSCALARS 18

typedef struct mbx_context mbx_context;

/* Create a context on CUDA device `device` (its own stream and buffers). */
int mbx_create(mbx_context** ctx, int device);
void mbx_destroy(mbx_context* ctx);
/* Last error message of the context (never NULL). */
const char* mbx_error(const mbx_context* ctx);
/* Use the caller's CUDA stream (a cudaStream_t passed as void*; NULL = the context's own). */
int mbx_set_stream(mbx_context* ctx, void* stream);

/* Time each phase of later evaluations with CUDA events on the context's stream. */
int mbx_set_profiling(mbx_context* ctx, int on);
/* Phase times of the last evaluation in ms: [0] lists, [1] 2B kernels (the fused 2B+3B
 * kernel when it runs), [2] 3B kernels (0 when fused), [3] heat-current jkin (or -1 when
 * profiling is off); counts[5]: [0] dimers, [1] trimers,
 * [2] kernel launches issued, [3]/[4] dimers/trimers the mixed path handed to FP64.
 * Either pointer may be NULL. */
int mbx_last_timings(mbx_context* ctx, double* ms, long* counts);

/* Mixed path: a dimer (trimer) is evaluated in FP32 only while every polynomial
 * variable is within limit2b (limit3b) of its shift centre; the others go to the
 * FP64 kernels in the same call.  0 sends every cluster of that body to FP64; a
 * limit >= 3.4e38 keeps every cluster in FP32.  Defaults: 0 (2B in FP64) and
 * 3.4e38 (3B in FP32). */
int mbx_set_mixed_limits(mbx_context* ctx, double limit2b, double limit3b);

/* Mixed method: evaluate the 2B and 3B terms in one persistent launch (1, default) or
 * in separate kernels (0).  Fused, each SM runs FP64 dimer warps and FP32 trimer warps
 * side by side, so the two bodies overlap on their own pipes.  It applies to the
 * default mixed split; hand-off limits and MBX_FP64 use the separate kernels.  The two
 * forms agree to FP32 rounding (the compiler may contract the FP32 model code
 * differently in the two kernels). */
int mbx_set_fused(mbx_context* ctx, int on);

/* The fused launch's split of each 384-thread block: dimer_warps of its 12 warps start on the
 * FP64 dimers, the rest on the FP32 trimers (either queue's warps take the other's work when
 * theirs runs dry).  0 = the default (4, one per SM sub-partition); 1..11 otherwise.  A
 * tuning knob: the split changes timings, and results only in the order of FP64 atomics. */
int mbx_set_fused_split(mbx_context* ctx, int dimer_warps);

/* mbx_water_step / mbx_water_step_device, mixed precision: run the MB-pol 2B/3B terms (they
 * need the positions only) on a second stream of the context while the electrostatics solve
 * its dipoles (on = 1), in an 8-warp form of the fused kernel (dimer_warps of them on the
 * dimers; 0 = 4) that leaves room on every SM for the FP32 CG kernels; the final pass of the
 * electrostatics starts after it.  Results equal the sequential form's up to the order of
 * FP64 atomic additions.  Default off. */
int mbx_set_overlap(mbx_context* ctx, int on, int dimer_warps);

/* mbx_water_step / mbx_water_step_device: run the 1-body and dispersion terms (positions
 * only) on a third stream of the context beside the electrostatics' setup and solve (on = 1);
 * the electrostatics' final pass, whose kernels add to the same force arrays, starts after
 * them.  Results equal the sequential form's up to the order of FP64 atomic additions.
 * Default off. */
int mbx_set_overlap_terms(mbx_context* ctx, int on);

/* Mixed method (mbx_polar_forces, mbx_water_step, mbx_water_step_multi): evaluate the
 * electrostatics' final pass -- forces, energies, virial, stress and heat current of the
 * converged dipoles -- in FP64 as the FP64 method does (on = 1), instead of its FP32 pair
 * forces, FP32 k-space heat sums and FP32 SPME heat grids.  The dipole solve stays mixed.
 * Default off. */
int mbx_set_final_fp64(mbx_context* ctx, int on);

/*
 * MB-pol 2B + 3B forces with the heat-current bookkeeping.
 * Replaces mbpol_forces (SOURCE/mbpol.f90:98-449, called from SOURCE/dlpoly_cmd.f:2504)
 * together with the HEAT_CURRENT hooks of do_dimer / do_trimer
 * (SOURCE/mbpol.f90:515-556, :897-952) and compute_heat_flux2's jkin/jpot sums
 * (SOURCE/heatcurrent.f90:703-728) for the MB-pol terms.
 *
 * HOST arrays (copied to and from the device inside the call):
 *   imcon, cell[9]          DL_POLY boundary key (1 cubic, 2 orthorhombic, 3 parallelepiped)
 *   nttm2, listttm2[nttm2]  water atoms (nttm2 = 3*nw), 1-based indices, O first
 *   natms                   length of every per-atom array
 *   xxx,yyy,zzz             positions
 *   fxx,fyy,fzz             forces, ACCUMULATED (like mbpol_forces)
 *   engsrp, virsrp          ACCUMULATED with eng2+eng3 and the virial
 *   stress[9]               ACCUMULATED
 *   vxx,vyy,vzz,weight      velocities and masses for the heat current, or all NULL
 *   atomic_energy           per-atom MB-pol energy, ACCUMULATED, or NULL
 *   scalars[MBX_NSCALARS]   this call's totals (see MBX_S_*), or NULL
 */
int mbx_mbpol_forces(mbx_context* ctx, int precision, int imcon, const double* cell, int nttm2,
                     const int* listttm2, int natms, const double* xxx, const double* yyy, const double* zzz,
                     double* fxx, double* fyy, double* fzz, double* engsrp, double* virsrp, double* stress,
                     const double* vxx, const double* vyy, const double* vzz, const double* weight,
                     double* atomic_energy, double* scalars);

/*
 * The same evaluation on DEVICE-resident arrays (no host copies of per-atom data;
 * the call returns after the scalars are on the host).  listttm2 is a device array.
 * fxx.. and atomic_energy are ACCUMULATED on the device.
 */
int mbx_mbpol_forces_device(mbx_context* ctx, int precision, int imcon, const double* cell, int nttm2,
                            const int* listttm2, int natms, const double* xxx, const double* yyy,
                            const double* zzz, double* fxx, double* fyy, double* fzz, const double* vxx,
                            const double* vyy, const double* vzz, const double* weight, double* atomic_energy,
                            double* scalars);

/*
 * The same evaluation for callers that cannot allocate device memory at the point of
 * the call: hosts whose device memory belongs to another allocator or pool, and MD
 * drivers that forbid allocation after start-up.  It needs no context and calls no
 * cudaMalloc/cudaFree: every intermediate lives in one fixed-size static device array
 * (~2.7 MB per GPU, held until the process exits).  The call synchronises `stream`
 * twice (after the list totals, and at the end for the scalars).
 * This entry point has no counterpart in the reference.
 *   - limits: at most 512 waters (nttm2 <= 1536), 64 dimer partners and 48 3B
 *     neighbours per water, 131072 trimers; larger systems return MBX_ERR_ARG or
 *     MBX_ERR_CAPACITY (with a message on stderr) and compute nothing;
 *   - arguments as mbx_mbpol_forces_device (device arrays, forces and atomic_energy
 *     ACCUMULATED), `scalars` is a host array or NULL, `stream` a cudaStream_t or NULL;
 *   - mixed precision uses the default split (2B FP64, 3B FP32);
 *   - the first call on a device looks up the array's device address and caches it for
 *     the process: do not call it across a cudaDeviceReset; every call shares the one
 *     array, so calls that overlap on the GPU (other streams, other host threads) race
 *     and must be serialised.
 */
int mbx_mbpol_forces_noalloc(int precision, int imcon, const double* cell, int nttm2, const int* listttm2,
                             int natms, const double* xxx, const double* yyy, const double* zzz, double* fxx,
                             double* fyy, double* fzz, const double* vxx, const double* vyy, const double* vzz,
                             const double* weight, double* atomic_energy, double* scalars, void* stream);

/*
 * 1-body MB-pol monomer term: the Partridge-Schwenke water PES with the angfrc
 * bookkeeping.  Replaces angfrc for angle type 9 (SOURCE/angfrc.f:150-545, calling
 * ps_type_couple, SOURCE/ps_type_couple.f90:15-274) with its HEAT_CURRENT hooks.
 *   nang, listang[3*nang]  H-O-H angles as (ia, ib, ic), 1-based, ib the central O
 *                          (listang(:,2:4) of the reference)
 *   fxx..                  ACCUMULATED; engang, virang, stress[9] ACCUMULATED
 *   vxx..                  velocities or NULL; jpot[3] ACCUMULATED (the force-matrix
 *                          entries (ia,ib),(ib,ia),(ic,ib),(ib,ic) contracted)
 *   atomic_energy          ACCUMULATED with pterm/3 per atom, or NULL
 * Host arrays; the _device variant takes device arrays and returns
 * out[14] = {engang, virang, stress[9], jpot[3]} on the host.
 */
int mbx_ps_pes_forces(mbx_context* ctx, int imcon, const double* cell, int nang, const int* listang, int natms,
                      const double* xxx, const double* yyy, const double* zzz, double* fxx, double* fyy,
                      double* fzz, double* engang, double* virang, double* stress, const double* vxx,
                      const double* vyy, const double* vzz, double* atomic_energy, double* jpot);
int mbx_ps_pes_forces_device(mbx_context* ctx, int imcon, const double* cell, int nang, const int* listang,
                             int natms, const double* xxx, const double* yyy, const double* zzz, double* fxx,
                             double* fyy, double* fzz, const double* vxx, const double* vyy, const double* vzz,
                             double* atomic_energy, double* out);

/*
 * M sites and Partridge-Schwenke dipole-moment-surface charges with MB-pol's settings
 * (ldms, new charge assignment, gamma = 0.426706882).  Replaces the M-site placement of
 * SOURCE/dlpoly_cmd.f:2041-2057 and qdetermine (SOURCE/qdetermine.f90:15-321).
 *   xxx,yyy,zzz      M-site positions WRITTEN at 1-based index listttm2[nttm2-1] + i
 *                    for water i = 1..nw (H and O read)
 *   chge             q_H1, q_H2, q_M WRITTEN (other entries untouched), or NULL
 *   dqdr[6*nw]       per water {dp1dr1, dp1dr2, dp2dr1, dp2dr2, dp1dcos, dp2dcos} (the
 *                    arrays qdforce contracts), or NULL
 * mbx_msites_dms takes host arrays; the _device variant device arrays.
 */
int mbx_msites_dms(mbx_context* ctx, int imcon, const double* cell, int nttm2, const int* listttm2, int natms,
                   double gamma, double* xxx, double* yyy, double* zzz, double* chge, double* dqdr);
int mbx_msites_dms_device(mbx_context* ctx, int imcon, const double* cell, int nttm2, const int* listttm2,
                          int natms, double gamma, double* xxx, double* yyy, double* zzz, double* chge,
                          double* dqdr);

/*
 * TTM4-F polarizable electrostatics of MB-pol water: the polar Ewald branch of the
 * reference's forces (SOURCE/forces.f:271-366 and :518-805) with the vmbpol settings
 * (SOURCE/simdef_cmd.f:1040-1060) -- rfield (SOURCE/rfield.f), ewald1p (SOURCE/ewald1p.f),
 * iter (SOURCE/iter.f), coulomb_polar (SOURCE/coulomb_polar.f), ewald2p (SOURCE/ewald2p.f),
 * ewald3p (SOURCE/ewald3p.f), qdforce (SOURCE/qdforce.f90) -- and their HEAT_CURRENT terms.
 * Replaces that branch of `forces` for a water-only system; ewald4p has no pairs there.
 *   precision MBX_FP64: the reference's SOR iteration (iter) in FP64.  MBX_MIXED: the same
 *             fixed point by FP64 iterative refinement -- the FP64 residual of the dipole
 *             equations, an FP32 conjugate-gradient solve of the correction (FP32 dipole
 *             tensors and exp(ik.r) table), repeated until (1 - sor_omega) * rms(residual) <= toler,
 *             then the reference's FP64 SOR step; everything after the dipoles in FP64.
 *   prm[15]   {alpha, rcut, epsq, toler (e*Angstrom, the CONTROL `iter` value / 4.803239),
 *              sor_omega, athole, athole12, athole13, ascc, ascd, gamma, kmax1, kmax2,
 *              kmax3, maxit}
 *   sites     4*nw in the standard layout: water w has O, H1, H2 at 3w..3w+2 and its M site
 *             at 3nw+w (0-based), M sites placed (mbx_msites_dms)
 *   chge      DMS charges, dqdr[6*nw] from mbx_msites_dms; polr (Thole widths) and polr2
 *             (polarizabilities, 0 = no dipole) per site, the FIELD `polar`/`polar2` values
 *   dip*      in: starting dipoles (0 on non-polarizable sites), out: converged dipoles
 *   f*        ACCUMULATED site forces; M-site forces are not redistributed (see
 *             mbx_msite_redistribute)
 *   out16     {engcpe, vircpe, stress[9], iterations, rms dipole change, polarization energy
 *              (coulomb_polar), k-space energy (with the self term), real-space energy}
 *             written; stress is this term's contribution
 *   atomic_energy  per-site electrostatic energy ACCUMULATED (update_energy_ew1p/ew2p/ew3p
 *             and _polar), not redistributed; may be NULL
 *   v*        velocities of the 3*nw water atoms, or NULL; then jpot[3] is ACCUMULATED with
 *             the electrostatic force-matrix and ew1p-stress terms of compute_heat_flux2
 *             after the M-site redistribution, and jkin[3] with the redistributed per-site
 *             energies times the velocities
 * Returns MBX_ERR_CONVERGE (results of the last iteration written) when the dipoles did
 * not reach toler within maxit iterations (the reference stops at 22581).
 */
int mbx_polar_forces(mbx_context* ctx, int precision, const double* prm, int imcon, const double* cell, int nw,
                     const double* xxx, const double* yyy, const double* zzz, const double* chge, const double* dqdr,
                     const double* polr, const double* polr2, double* dipx, double* dipy, double* dipz, double* fxx,
                     double* fyy, double* fzz, double* out16, double* atomic_energy, const double* vxx,
                     const double* vyy, const double* vzz, double* jpot, double* jkin);
int mbx_polar_forces_device(mbx_context* ctx, int precision, const double* prm, int imcon, const double* cell, int nw,
                            const double* xxx, const double* yyy, const double* zzz, const double* chge,
                            const double* dqdr, const double* polr, const double* polr2, double* dipx, double* dipy,
                            double* dipz, double* fxx, double* fyy, double* fzz, double* out16,
                            double* atomic_energy, const double* vxx, const double* vyy, const double* vzz,
                            double* jpot, double* jkin);
/* Dipole iterations of the last mbx_polar_forces call (MBX_MIXED: FP64 field evaluations),
 * and the FP32 conjugate-gradient iterations of the last MBX_MIXED call. */
int mbx_polar_iterations(const mbx_context* ctx);
long mbx_polar_inner_sweeps(const mbx_context* ctx);
/* With mbx_set_profiling on: the last electrostatics call's phase times in ms[4] (lists,
 * static fields and exp(ik.r) table; dipole solve; final structure factors with the heat
 * sums; rest of the final pass) and its number of k vectors. */
int mbx_polar_timings(const mbx_context* ctx, float* ms4, long* kvectors);
/* With mbx_set_profiling on: the FP64 k-space field gathers of the last call (the
 * iteration's largest FP64 kernel): device ms, algorithmic flops (9 per k vector and site,
 * 18 in the first evaluation, which adds the static charge field) and launches timed. */
int mbx_polar_field_timing(const mbx_context* ctx, double* ms, double* flops, long* launches);
/* Frees the electrostatics' device buffers (phase tables, pair tensors) of a context when
 * they hold more than keep_bytes; returns the bytes freed (0: kept).  The next call
 * allocates them again. */
double mbx_trim(mbx_context* ctx, double keep_bytes);
/*
 * k space of the electrostatics: the reference's explicit Ewald sum (order 0, the default;
 * kmax from prm[11..13]) or smooth particle-mesh Ewald (order 4..8) for later
 * mbx_polar_forces / mbx_water_step calls of the context (and its worker lanes).  SPME
 * spreads charges and induced dipoles (mu . grad of the B-splines) on a K1 x K2 x K3 grid:
 * grid[3] (even, no prime factor above 5), or grid NULL / grid[0] == 0 for the smallest
 * such grid whose spacing along each cell width is <= `spacing` Angstrom.  The charge part
 * follows the reference's ewald_spme (SOURCE/ewald_spme.f:1-362, SOURCE/bspgen.f,
 * SOURCE/bspcoe.f, SOURCE/spme_for.f: fractional coordinates shifted by half a cell, the
 * Euler-spline moduli, the spherical k cut at 1.05 x half the grid, the mean k-space force
 * removed); the reference evaluates induced dipoles with the explicit Ewald sum only
 * (SOURCE/ewald1p.f), so the dipole part has no counterpart there.  alpha and rcut still
 * come from prm; the real-space terms are unchanged.  mbx_spme_last_grid gives the grid
 * of the last electrostatics call (zeros with the Ewald sum).
 */
int mbx_set_spme(mbx_context* ctx, int order, double spacing, const int* grid);
/*
 * The electrostatics' site pair list as the reference's Verlet list (SOURCE/parlst.f with
 * the rebuild test of SOURCE/centroid_vertest.f:53-88): the pairs within rcut + delr are kept
 * between calls of the context and rebuilt once a site has moved more than delr / 2 since
 * the build (or the cell, rcut or size changed); every call filters the pairs within rcut
 * from them with the reference's cut test, so results do not depend on delr.  delr 0
 * rebuilds the list at every call; the default is 1 Angstrom.  mbx_polar_list_builds
 * counts the builds; mbx_polar_last_pairs gives the last call's pairs within rcut (i < j,
 * 0-based sites), up to cap of them in pairs[2 * cap], their count in *npairs.
 */
int mbx_set_polar_skin(mbx_context* ctx, double delr);
long mbx_polar_list_builds(const mbx_context* ctx);
int mbx_polar_last_pairs(mbx_context* ctx, int* pairs, long cap, long* npairs);
int mbx_spme_last_grid(const mbx_context* ctx, int* grid);
/* The grid mbx_set_spme picks for a cell at a spacing (grid[3] written). */
int mbx_spme_grid_for_cell(const double* cell, double spacing, int* grid);
/*
 * SPME k space of point charges and point dipoles, one call on host arrays (the
 * reference's ewald_spme for the charges, SOURCE/ewald_spme.f:1-362, with the dipole
 * extension above):
 *   prm[2] = {alpha, epsq}; order 4..8; grid[3] as mbx_set_spme; imcon, cell[9]
 *   n sites: xxx, yyy, zzz, chge; dip (3 blocks of n: x, y, z) or NULL
 *   vel (3 blocks of n) or NULL: the velocity each site's heat terms are carried with
 *   forces[3n]  WRITTEN: -dE/dr of the k-space energy, the mean over the sites removed
 *   field[3n]   WRITTEN or NULL: the k-space field -dE/dmu (no self term)
 *   pot[n]      WRITTEN or NULL: dE/dq
 *   out[14]     WRITTEN: {E of the charges alone, E of charges and dipoles, stress[9] (with
 *               the dipoles' strain term), jpot[3] (ewald1p's HEAT_CURRENT per-atom stress
 *               contracted with vel, SOURCE/ewald1p.f:575-690; 0 without vel)}
 * E excludes the self terms; units as mbx_polar_forces.
 */
int mbx_spme_kspace(mbx_context* ctx, const double* prm, int order, const int* grid, int imcon, const double* cell,
                    int n, const double* xxx, const double* yyy, const double* zzz, const double* chge,
                    const double* dip, const double* vel, double* forces, double* field, double* pot, double* out);
/*
 * The hand-written 3D FFT of the SPME path on `count` complex grids (host array, interleaved
 * re/im, x fastest, n1 x n2 x n3 each, sizes 4..1024 with no prime factor above 5), in
 * place and unnormalised: sign +1 sums data * exp(+2 pi i m.g / n), sign -1 with the
 * opposite exponent.  The counterpart of the reference's dlpfft3 (SOURCE/dlpfft3.f:1-401).
 */
int mbx_fft3d(mbx_context* ctx, int n1, int n2, int n3, int count, int sign, double* data);
/* M-site force redistribution of the reference's MD step (SOURCE/dlpoly_cmd.f:2585-2601):
 * F_O += (1 - gamma) F_M, F_H1 += F_M gamma / 2, F_H2 += F_M gamma / 2 (standard layout,
 * host arrays of 4*nw sites; the M-site entries are left as they are). */
int mbx_msite_redistribute(int nw, double gamma, double* fxx, double* fyy, double* fzz);

/*
 * The whole force evaluation of one MD step of MB-pol water, as the reference's MD loop
 * runs it (SOURCE/dlpoly_cmd.f:2041-2057 M sites, qdetermine, forces with the polar Ewald
 * branch and srfrce2, angfrc keya 9, mbpol_forces at :2504, the M-site redistribution at
 * :2585-2606, and their HEAT_CURRENT terms), in one host call.  Standard layout only:
 * natms = 4*nw, water w has O, H1, H2 at 3w..3w+2 and its M site at 3nw+w; the 1-body
 * term runs over the (H1, O, H2) angle of every water.
 *   precision   MBX_FP64 or MBX_MIXED (applies to the MB-pol polynomials and the dipole solve)
 *   polar_prm, polr, polr2   as mbx_polar_forces (gamma is polar_prm[10])
 *   ltype, molecule          per-atom dispersion types and molecules (1-based types, 0 none)
 *                            as mbx_disp_forces, after mbx_disp_setup; NULL: no dispersion
 *   xxx..       water atom positions in; the M-site positions are written (natms entries)
 *   dip*        in: starting dipoles (the previous step's, or 0), out: converged dipoles
 *   f*          ACCUMULATED; M-site forces redistributed onto O, H1, H2 (the M entries keep
 *               their value, as the reference leaves them)
 *   v*, weight  velocities and masses (NULL: no heat current)
 *   atomic_energy  per-site energy of every term ACCUMULATED (not redistributed), or NULL
 *   chge        site charges written, or NULL
 *   scalars[MBX_NSTEPSCALARS]  written: the mbx_water_forces block (MB-pol, 1-body,
 *               dispersion), then mbx_polar_forces' out16, then the electrostatic jpot[3]
 *               and jkin[3].  The total heat current is the sum of the jpot and jkin
 *               entries of all blocks.
 * Returns MBX_ERR_CONVERGE (everything written) when the dipoles did not converge.
 */
#define MBX_NSTEPSCALARS (MBX_NWATERSCALARS + 22)
int mbx_water_step(mbx_context* ctx, int precision, int imcon, const double* cell, int nw, int natms,
                   const double* polar_prm, const double* polr, const double* polr2, const int* ltype,
                   const int* molecule, double* xxx, double* yyy, double* zzz, double* dipx, double* dipy,
                   double* dipz, double* fxx, double* fyy, double* fzz, const double* vxx, const double* vyy,
                   const double* vzz, const double* weight, double* atomic_energy, double* chge, double* scalars);
/* The same on device arrays (ltype/molecule, polr/polr2 and every per-site array device
 * pointers; chge is required, it is the charge workspace); scalars is a host array. */
int mbx_water_step_device(mbx_context* ctx, int precision, int imcon, const double* cell, int nw, int natms,
                          const double* polar_prm, const double* polr, const double* polr2, const int* ltype,
                          const int* molecule, double* xxx, double* yyy, double* zzz, double* dipx, double* dipy,
                          double* dipz, double* fxx, double* fyy, double* fzz, const double* vxx, const double* vyy,
                          const double* vzz, const double* weight, double* atomic_energy, double* chge,
                          double* scalars);

/*
 * Whole force evaluations (as mbx_water_step) of many independent boxes in one host call:
 * path-integral beads, or separate simulations of any sizes.  The boxes run concurrently
 * on the context's worker lanes (mbx_set_lanes, default 8): each lane is a child context
 * with its own CUDA stream and device buffers, kept between calls, and one host thread
 * for the call; boxes are handed out largest first.  Box b's results are those of
 * mbx_water_step on its slice.  The reference gives each bead its own MPI group
 * (SOURCE/multibead.f90:75-84), which runs one force evaluation per step
 * (SOURCE/dlpoly_cmd.f:2287, :2504).
 *   nbox; imcon[nbox], cell[9*nbox], nw[nbox]; box b has 4*nw[b] sites (standard layout)
 *        stored from offset sum_{c<b} 4*nw[c] in every per-site array below
 *   polar_prm[15*nbox]  per box (kmax follows the box size)
 *   polr, polr2, ltype, molecule, xxx.., dip*, f*, v*, weight, atomic_energy, chge
 *        as mbx_water_step, concatenated over the boxes (ltype/molecule NULL: no
 *        dispersion; its setup is the one of mbx_disp_setup on this context)
 *   scalars[MBX_NSTEPSCALARS*nbox]  per box; status[nbox] per box, or NULL
 * Returns the first failing box's error, else MBX_ERR_CONVERGE when a box's dipoles did
 * not converge (everything written), else MBX_OK.
 */
int mbx_set_lanes(mbx_context* ctx, int lanes);
/* MBX_MIXED dipole solve, with the block preconditioner off (mbx_set_precond_block): Jacobi
 * sweeps of the conjugate-gradient preconditioner on the real-space part of the dipole
 * equations, odd 1..9 (1: the diagonal alone), or 0 (the default): 1 with SPME, whose k
 * space makes a CG sweep cheap beside two more real-space sweeps, 3 with the Ewald sum.
 * An odd count keeps the preconditioner positive definite; a breakdown or an outer step
 * that does not halve the residual falls back to the diagonal.  Changes the iteration
 * count, not the converged dipoles beyond the dipole tolerance. */
int mbx_set_precond_sweeps(mbx_context* ctx, int sweeps);
/* MBX_MIXED dipole solve: with on != 0 (the default) the conjugate-gradient preconditioner
 * is the inverse of each water's 9x9 block of the system (the polarizabilities, the self
 * term and the three intramolecular dipole tensors; Cholesky per water once per call)
 * instead of the sweeps of mbx_set_precond_sweeps, which apply with on == 0.  A water whose
 * block is not positive definite keeps the diagonal; a breakdown or an outer step that does
 * not halve the residual falls back to the diagonal.  Changes the iteration count, not the
 * converged dipoles beyond the dipole tolerance. */
int mbx_set_precond_block(mbx_context* ctx, int on);
/* ASPC dipole prediction, the CONTROL keywords `aspc` and `aspc_k` (replaces aspc_init,
 * aspc_predict and aspc_set of SOURCE/aspc.f90:45-251 with the ASPC branch of the dipole
 * loop, SOURCE/forces.f:334-366, as SOURCE/dlpoly_cmd.f:2273-2320 drives them).
 *   k           2 or 4 turns it on; 0 (the default) turns it off: each call's dipoles then
 *               start from the caller's, as set_guess_dipole(1, ...) leaves them
 *   iter_nstep  aspc_iter_nstep: k+2 when the deck sets `aspc_k`, 6 for `aspc`
 * Each later mbx_polar_forces / mbx_water_step(_device) call on this context is one MD
 * step.  Steps 1..iter_nstep iterate to toler (SOR weight 0.3 for steps 1..4, then
 * polar_prm[4]).  Every later step starts from sum_j B_j mu(t - j) over the last k+2
 * steps' dipoles (Kolafa's coefficients) and makes ONE SOR iteration with polar_prm[4]
 * (4/7 or 6/11 when the deck sets `aspc_k`): its dipoles are not converged, as in the
 * reference.  The history is kept per context on the device.  Calling this again clears the
 * history and the step count (aspc_init), as does a change of the site count.  The worker
 * lanes of mbx_water_step_multi do not predict. */
int mbx_set_aspc(mbx_context* ctx, int k, int iter_nstep);
/* nstep_for_guess = 0 (SOURCE/dlpoly_cmd.f:1765-1768, an i-PI image change): the next call
 * is ASPC step 1 again; the history is kept, as the reference keeps it.  mbx_ipi_run does
 * this when the replica changes. */
int mbx_aspc_restart(mbx_context* ctx);
/* Not a reference option: the initial guess of each converged dipole solve (ASPC off) is
 * the polynomial of degree `order` (1..3; 0 off, the default) through the last order+1
 * calls' converged dipoles, extrapolated one step, for sites whose input dipoles are the
 * last call's output (the caller carried them over); other sites start from the caller's.
 * The solve still iterates to toler: results stay within the dipole tolerance of a
 * warm-started solve; the number of iterations changes.  The history is the ASPC one (per
 * context; this call clears it and turns ASPC off; mbx_set_aspc turns the guess off). */
int mbx_set_dipole_guess(mbx_context* ctx, int order);
/* The ASPC step count of the context (nstep_for_guess); -1 without a context. */
int mbx_aspc_step(mbx_context* ctx);
int mbx_water_step_multi(mbx_context* ctx, int precision, int nbox, const int* imcon, const double* cell,
                         const int* nw, const double* polar_prm, const double* polr, const double* polr2,
                         const int* ltype, const int* molecule, double* xxx, double* yyy, double* zzz, double* dipx,
                         double* dipy, double* dipz, double* fxx, double* fyy, double* fzz, const double* vxx,
                         const double* vyy, const double* vzz, const double* weight, double* atomic_energy,
                         double* chge, double* scalars, int* status);

/*
 * The Ewald and dipole settings the server uses for a cell (cell[9], Angstrom): rcut =
 * min(9, 0.49 x the narrowest width), alpha = 2.7 / rcut, kmax per axis scaled from the
 * 256-water box's alpha 0.3 / kmax 8, the vmbpol Thole and smearing constants, toler
 * 1e-8 D, SOR weight 0.3, maxit 22581; written to prm[15] in mbx_polar_forces' layout.
 */
void mbx_polar_params_for_cell(const double* cell, double* prm);

/*
 * i-PI driver mode: the reference's IPI_INIT / IPI_STEP (SOURCE/ipi.f90:33-198) with its
 * socket wrapper (SOURCE/sockets.c).  The client connects to an i-PI server at `address`:
 * "inet:host:port", "unix:name:port" (the socket /tmp/ipi_<name>), or "host:port".  It
 * answers STATUS (HAVEDATA / READY / NEEDINIT), INIT (replica index and parameter string),
 * POSDATA (cell, inverse, atoms, positions in bohr: the configuration is evaluated) and
 * GETFORCE (FORCEREADY, energy, atoms, forces, virial in atomic units, then the water
 * dipoles as text), until EXIT or max_steps force replies (0: no limit).  Unit factors are
 * the reference's single-precision constants (SOURCE/ipi.f90:72-77); the cell and the
 * virial are transposed as there.
 *   mbx_ipi_run           evaluates each configuration of nat = 3 nw atoms (O, H, H per
 *                         water) with mbx_water_step on ctx: polar_prm[15], or NULL for
 *                         mbx_polar_params_for_cell of each cell; dispersion != 0 uses the
 *                         mbx_disp_setup of ctx with types 1 (O), 2 (H), 3 (M).  Each
 *                         replica's dipoles are the warm start of its next configuration.
 *                         The energy sent is the sum of the evaluated terms (the dispersion
 *                         long-range correction, a constant of the volume, is not included).
 *   mbx_ipi_run_callback  the protocol with a caller's force function: it gets the replica,
 *                         atoms, cell[9] and interleaved positions in Angstrom and returns
 *                         the energy, interleaved forces and stress[9] in DL_POLY units
 *                         (10 J/mol, Angstrom) and 3 values per water for the dipole text;
 *                         it returns MBX_OK (or MBX_ERR_CONVERGE) to continue.  err[errlen]
 *                         receives the reason of a failure.
 * Both return MBX_OK after EXIT or max_steps, else the failure's status.
 */
typedef int (*mbx_ipi_force_fn)(void* user, int replica, int natoms, const double* cell, const double* xyz,
                                double* energy, double* forces, double* stress, double* moldip);
int mbx_ipi_run_callback(const char* address, mbx_ipi_force_fn fn, void* user, long max_steps, long* steps_done,
                         char* err, int errlen);
int mbx_ipi_run(mbx_context* ctx, const char* address, int precision, const double* polar_prm, int dispersion,
                long max_steps, long* steps_done);

/*
 * Path-integral bead coupling of the reference's PIMD/CMD mode on the device, for callers
 * that evaluate the beads' physical forces with mbx_water_step_multi (one box per bead) and
 * propagate them: the normal-mode transformation (transformation_matrix and the
 * cart <-> normal-mode transforms, SOURCE/centroid_matrix.f:3-270) and the ring-polymer
 * spring forces (SOURCE/centroid_spring_force.f:1-157).  nbead even, 2..256; the beads are
 * a leading array axis (value j of bead b at b * n + j), not MPI ring ranks.
 *   mbx_pimd_matrices          host only: nmode_to_cart[bead * P + mode],
 *                              cart_to_nmode[mode * P + bead], lambda[P] (any may be NULL)
 *   mbx_pimd_transform_device  out[p * nvals + j] = sum_b A[p][b] in[b * nvals + j] with A
 *                              cart_to_nmode (to_modes != 0) or nmode_to_cart; device arrays
 *   mbx_pimd_spring_forces_device  natms atoms per bead (x, y, z, f device arrays of
 *                              nbead * natms, mass[natms] device, the physical masses);
 *                              the spring forces coeff m (2 r_k - r_{k-1} - r_{k+1}) x
 *                              force_scale (0 with langevin and add_spring_to_forces 0)
 *                              SUBTRACTED from f, coeff = nbead / (hbar beta)^2;
 *                              energies[2] (host) = {the spring energy
 *                              0.5 coeff sum m |r_k - r_{k-1}|^2, the centroid-virial term
 *                              0.5 sum -(r_k - c) . f_k / force_scale with the incoming
 *                              forces}; c the centroid, the first normal mode as a position.
 */
int mbx_pimd_matrices(int nbead, int langevin, double* nmode_to_cart, double* cart_to_nmode, double* lambda);
int mbx_pimd_transform_device(mbx_context* ctx, int nbead, int langevin, int to_modes, long nvals, const double* in,
                              double* out);
int mbx_pimd_spring_forces_device(mbx_context* ctx, int nbead, int langevin, int add_spring_to_forces, double hbar,
                                  double beta, double force_scale, int natms, const double* xxx, const double* yyy,
                                  const double* zzz, double* fxx, double* fyy, double* fzz, const double* mass,
                                  double* energies);

/*
 * Continuous-batching force server.  `slots` worker slots, each with its own context and
 * CUDA stream on `device`, evaluate independent water boxes concurrently; a FIFO queue
 * admits the next request as soon as a slot is free and its estimated device-memory
 * footprint fits `budget_bytes` (a request larger than the budget runs alone).  Every
 * request runs the 1-body term and the MB-pol 2B/3B terms with the heat current
 * (standard layout: waters 1..3*nw as O,H1,H2, M sites after them, natms >= 4*nw).
 * No counterpart in the reference (its i-PI client serves one request at a time,
 * SOURCE/ipi.f90:33-198).
 *   mbx_server_submit  copies the host inputs and returns a request id > 0, or -status
 *   mbx_server_wait    blocks until the request is done, copies forces (natms each),
 *                      per-atom energies, scalars[MBX_NSCALARS + 14] (the MB-pol block,
 *                      then engang, virang, stress[9], jpot[3] of the 1-body term) and
 *                      times[3] = {queueing, on a slot, total latency} in seconds; any
 *                      output pointer may be NULL.  Returns the request's status.
 */
typedef struct mbx_server mbx_server;
int mbx_server_create(mbx_server** server, int device, int slots, double budget_bytes);
void mbx_server_destroy(mbx_server* server);
long mbx_server_submit(mbx_server* server, int precision, int imcon, const double* cell, int nw, int natms,
                       const double* xxx, const double* yyy, const double* zzz, const double* vxx, const double* vyy,
                       const double* vzz, const double* weight);
int mbx_server_wait(mbx_server* server, long id, double* fxx, double* fyy, double* fzz, double* atomic_energy,
                    double* scalars, double* times);
/*
 * The whole force evaluation per request (mbx_water_step: M sites, DMS charges, TTM4-F
 * electrostatics, 1-body, 2B, 3B, M-site redistribution, heat current); natms = 4*nw in
 * the standard layout.  The Ewald settings follow the cell: rcut = min(9, 0.49 x the
 * narrowest width), alpha = 2.7 / rcut, kmax per axis keeping 2 pi kmax / (alpha L) of
 * the 256-water box (kmax 8 at alpha 0.3, L 19.73); the vmbpol Thole settings, MB-pol's
 * polarizabilities, dipoles to 1e-8 D.  The induced dipoles start from the last converged
 * ones of the same `client` (zero for its first request or after a size change); a
 * client's requests run one at a time in submission order.  Admission counts the
 * electrostatics' phase tables and pair tensors in the footprint.
 *   mbx_server_wait_step  as mbx_server_wait, plus the converged dipoles (3 * natms, x
 *                         block then y then z) and scalars[MBX_NSTEPSCALARS].
 */
long mbx_server_submit_step(mbx_server* server, int precision, long client, int imcon, const double* cell, int nw,
                            const double* xxx, const double* yyy, const double* zzz, const double* vxx,
                            const double* vyy, const double* vzz, const double* weight);
int mbx_server_wait_step(mbx_server* server, long id, double* fxx, double* fyy, double* fzz, double* atomic_energy,
                         double* dipoles, double* scalars, double* times);
const char* mbx_server_error(const mbx_server* server);
/* k space of later step requests: SPME of `order` (4..8) on the grid of `spacing` per cell
 * (as mbx_set_spme with grid NULL), or order 0 for the explicit Ewald sum (the default).
 * With SPME the admission footprint holds the grids instead of the exp(ik.r) tables. */
int mbx_server_set_spme(mbx_server* server, int order, double spacing);

/*
 * Many independent water boxes (path-integral beads, separate simulations) in ONE
 * evaluation: the 1-body term and the MB-pol 2B/3B terms with the heat current of every
 * box, with one set of kernel launches over all boxes and per-box scalars.  Replaces the
 * reference's bead parallelism, where MPI ranks are split into one group per bead
 * (SOURCE/multibead.f90:25-80) and every group runs the force routines on its own
 * replica (SOURCE/dlpoly_cmd.f:483-511); a single call over all beads has no
 * counterpart there.
 *   nbox, nw_box[nbox]      waters per box; box b occupies atoms [4*W_b, 4*W_b + 4*nw_b)
 *                           with W_b = sum of nw_box[b'] for b' < b: 3*nw_b water atoms
 *                           (O, H1, H2) then nw_b M sites (not read), natms = 4 * sum nw_box
 *   imcon, cells[9*nbox]    boundary key for all boxes and each box's cell (host array)
 *   xxx.. fxx.. vxx.. weight, atomic_energy   per-atom arrays of length natms; forces and
 *                           energies ACCUMULATED; velocities+weight NULL for no heat current
 *   scalars[nbox * MBX_NBOXSCALARS] (host, or NULL): per box the MB-pol block
 *                           (MBX_S_*), then engang, virang, stress[9], jpot[3] of the
 *                           1-body term (as mbx_ps_pes_forces)
 * Dimer and trimer candidates are the waters of the same box (O(nw_b^2) tests per box,
 * meant for boxes of up to a few thousand waters), with the reference's O-O criteria.
 * The lists stay on the device: the step is enqueued without host synchronisation and,
 * with graphs on (mbx_set_graphs, default on), captured once as a CUDA graph and
 * replayed while the arrays, box layout, precision and limits are unchanged.  The call
 * returns after the step and the per-box scalars are done.  Mixed precision follows
 * mbx_set_mixed_limits.  mbx_last_timings: ms[0] the whole step, counts as usual.
 *   mbx_mbpol_multi_device  all per-atom arrays on the device
 *   mbx_mbpol_multi         host arrays, copied in and out inside the call
 */
#define MBX_NBOXSCALARS (MBX_NSCALARS + 14)
int mbx_mbpol_multi_device(mbx_context* ctx, int precision, int imcon, int nbox, const int* nw_box,
                           const double* cells, const double* xxx, const double* yyy, const double* zzz,
                           double* fxx, double* fyy, double* fzz, const double* vxx, const double* vyy,
                           const double* vzz, const double* weight, double* atomic_energy, double* scalars);
int mbx_mbpol_multi(mbx_context* ctx, int precision, int imcon, int nbox, const int* nw_box, const double* cells,
                    const double* xxx, const double* yyy, const double* zzz, double* fxx, double* fyy, double* fzz,
                    const double* vxx, const double* vyy, const double* vzz, const double* weight,
                    double* atomic_energy, double* scalars);
/* Capture and replay the multi-box step as a CUDA graph (1, default) or launch it
 * directly (0); mbx_graph_launches counts the graph replays of the context. */
int mbx_set_graphs(mbx_context* ctx, int on);
long mbx_graph_launches(const mbx_context* ctx);

/*
 * The water force field of one MD step in one call: the 1-body term (as
 * mbx_ps_pes_forces), the dispersion term when ltype and molecule are given (as
 * mbx_disp_forces, after mbx_disp_setup), then the MB-pol 2B/3B terms (as
 * mbx_mbpol_forces), with the heat current.  Replaces the angfrc (keya 9), srfrce2 and
 * mbpol_forces calls of one force evaluation (SOURCE/dlpoly_cmd.f:2430, SOURCE/forces.f:552,
 * SOURCE/dlpoly_cmd.f:2504); every input is copied to the device once and the forces and
 * per-atom energies come back once.  Host arrays; forces and atomic_energy ACCUMULATED.
 * jkin (scalars[MBX_S_JKIN..]) uses the per-atom energies of every term in the call.
 *   scalars[MBX_NWATERSCALARS] (or NULL): the MB-pol block (MBX_S_*), then engang,
 *   virang, stress[9], jpot[3] of the 1-body term, then engsrp, virsrp, stress[9],
 *   jpot[3] of the dispersion term (zeros without it).
 */
#define MBX_NWATERSCALARS (MBX_NSCALARS + 28)
int mbx_water_forces(mbx_context* ctx, int precision, int imcon, const double* cell, int nttm2, const int* listttm2,
                     int nang, const int* listang, const int* ltype, const int* molecule, int natms,
                     const double* xxx, const double* yyy, const double* zzz, double* fxx, double* fyy, double* fzz,
                     const double* vxx, const double* vyy, const double* vzz, const double* weight,
                     double* atomic_energy, double* scalars);

/*
 * Short-range dispersion: DL_POLY van der Waals type 12, Tang-Toennies damped
 * -C6 f6(a6 r)/r^6 - C8 f8(a8 r)/r^8.  Replaces forgen's type-12 tables
 * (SOURCE/forgen.f:97, :262-270, :337-357), the Verlet list of parlst with the
 * intramolecular exclusions (SOURCE/parlst.f, SOURCE/exclude_ttm.f) and srfrce2
 * (SOURCE/srfrce2.f:80-270) with its HEAT_CURRENT hooks (update_energy_srf,
 * update_forces), and lrcorrect for type 12 (SOURCE/lrcorrect.f:112-223).
 *   mbx_disp_setup   ntypes atom types (1-based, <= 15); prm[4 * ntypes(ntypes+1)/2] =
 *                    {C6, a6, C8, a8} per pair type, pair (i >= j) at index
 *                    i(i-1)/2 + j - 1 (lstvdw order), internal energy units and Angstrom;
 *                    a pair type whose parameters are all 0 does not interact; rcut and
 *                    the Verlet skin delr in Angstrom; mxgrid table points, 0 = the
 *                    reference's default max(1000, rcut / 1e-4 + 4).  The reference reads
 *                    these parameters from its FIELD file.
 *   mbx_disp_forces  ltype[natms] (0 = no dispersion, e.g. M sites), molecule[natms]
 *                    (atoms of one molecule do not interact); forces, engsrp, virsrp,
 *                    stress ACCUMULATED; per-atom energies get half of each pair energy;
 *                    velocities (or NULL) give jpot[3] ACCUMULATED.  Host arrays.
 *   _device          device arrays; out[14] = {engsrp, virsrp, stress[9], jpot[3]} on
 *                    the host.  The Verlet list (pairs within rcut + delr) is kept between
 *                    calls and rebuilt when an atom has moved more than delr / 2, or natms,
 *                    the cell or the ltype/molecule arrays change (mbx_disp_setup also
 *                    drops it); mbx_disp_list_builds counts the builds.
 *   mbx_disp_lrc     elrc and virlrc for numtyp[t] atoms of type t + 1 in volume volm
 *                    (host only, no GPU), with the reference's factorial in
 *                    tang_toennies_lr (it multiplies by its argument at every step).
 */
int mbx_disp_setup(mbx_context* ctx, int ntypes, const double* prm, double rcut, double delr, int mxgrid);
int mbx_disp_forces(mbx_context* ctx, int imcon, const double* cell, int natms, const int* ltype, const int* molecule,
                    const double* xxx, const double* yyy, const double* zzz, double* fxx, double* fyy, double* fzz,
                    double* engsrp, double* virsrp, double* stress, const double* vxx, const double* vyy,
                    const double* vzz, double* atomic_energy, double* jpot);
int mbx_disp_forces_device(mbx_context* ctx, int imcon, const double* cell, int natms, const int* ltype,
                           const int* molecule, const double* xxx, const double* yyy, const double* zzz, double* fxx,
                           double* fyy, double* fzz, const double* vxx, const double* vyy, const double* vzz,
                           double* atomic_energy, double* out);
int mbx_disp_lrc(int ntypes, const double* prm, const int* numtyp, double rcut, double volm, double* elrc,
                 double* virlrc);
long mbx_disp_list_builds(const mbx_context* ctx);

/* Dimer and trimer lists of the last evaluation (0-based water indices, i<j<k), as
 * index sets; the host arrays receive up to cap entries; counts are always written. */
int mbx_last_lists(mbx_context* ctx, int* pairs, long cap_pairs, long* npairs, int* trimers, long cap_trimers,
                   long* ntrimers);

/*
 * Batched model evaluation for explicit clusters (host arrays, 9 doubles per monomer,
 * O H1 H2, already imaged; kcal/mol and Angstrom like the reference's C++).
 * mbx_2b_poly_batch ASSIGNS g1/g2; mbx_3b_poly_batch ACCUMULATES into g1..g3, as
 * x2b_v6x_p / x3b_v2x_p do (SOURCE/mbpol-2b-poly.cpp:609-612, SOURCE/mbpol-3b-poly.cpp:39-42).
 */
int mbx_2b_poly_batch(mbx_context* ctx, int precision, long n, const double* w1, const double* w2, double* E,
                      double* g1, double* g2);
int mbx_3b_poly_batch(mbx_context* ctx, int precision, long n, const double* w1, const double* w2,
                      const double* w3, double* E, double* g1, double* g2, double* g3);

/*
 * Drop-ins for the reference's per-cluster C entry points, same signatures and
 * meaning (SOURCE/mbpol-2b-poly.cpp:1884-1904, SOURCE/mbpol-3b-poly.cpp:1522-1542).
 * They run one FP64 evaluation on the current CUDA device through a process-wide
 * context.  A non-NULL `force_matrix` receives the reference's pairwise split of the
 * gradient (read by its HEAT_STRESS build, SOURCE/mbpol.f90:564-566, :951-953), as
 * mbx_2b_force_matrix_batch / mbx_3b_force_matrix_batch below write it.
 * On a CUDA error they print a message and abort (the reference has no error path).
 */
/*
 * The force matrices of many clusters (host arrays, FP64), as the reference's C models
 * write them (SOURCE/mbpol-2b-poly.cpp:449-653, SOURCE/mbpol-3b-poly.cpp:208-312): entry
 * (i, j, c) of the cluster's sites (O, H1, H2 per monomer) is component c of the gradient
 * of the polynomial variable linking sites i and j, with the sign of r_i - r_j.
 *   2B: fm[108 n], 6 x 6 x 3 per dimer; the X sites' rows are redistributed onto their
 *       monomer's atoms through the X-site geometry and their columns onto the other
 *       monomer's O; times the switch, its gradient added to the O-O entries.  Diagonal
 *       entries are written 0 (the reference copies them from an uninitialised array;
 *       its reader skips them).  Dimers beyond the 6.5 A cutoff are left untouched.
 *   3B: fm[243 n], 9 x 9 x 3 per trimer; every off-diagonal entry written (the switching
 *       product included), the switch gradients added to the O-O entries, the diagonal
 *       left untouched.
 */
int mbx_2b_force_matrix_batch(mbx_context* ctx, long n, const double* w1, const double* w2, double* fm);
int mbx_3b_force_matrix_batch(mbx_context* ctx, long n, const double* w1, const double* w2, const double* w3,
                              double* fm);
void mbpol_2b_poly_(const double* w1, const double* w2, double* E, double* g1, double* g2, double* force_matrix);
void mbpol_3b_poly_(const double* w1, const double* w2, const double* w3, double* E, double* g1, double* g2,
                    double* g3, double* force_matrix);
void mbpol_2b_cutoff_(double* r);
void mbpol_3b_cutoff_(double* r);

#ifdef __cplusplus
}
#endif
#endif /* MBX_H */
