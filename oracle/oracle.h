/*
 * CPU oracle for the MB-pol force + heat-current path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The product
 * (libmbx.so) never links, loads or calls it.
 *
 * It restates, in plain C++, the reference DL_POLY 2 fork's Fortran driver
 * (SOURCE/mbpol.f90) and its 2B/3B model wrappers (SOURCE/mbpol-2b-poly.cpp,
 * SOURCE/mbpol-3b-poly.cpp) operation by operation.  The two polynomials are
 * evaluated from the monomial tables extracted from the reference's generated
 * evaluators; the tables and the whole 2B/3B model are pinned against the
 * reference's own C++ compiled from its sources (golden vectors in tests/golden/).
 *
 * Units follow the reference: Angstrom, kcal/mol inside the models, DL_POLY
 * internal energy units (10 J/mol, engunit = 418.4 per kcal/mol) in the driver.
 */
#ifndef MBX_ORACLE_H
#define MBX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Load the monomial tables (text files written by extract_poly_tables.py). 0 = ok. */
int orc_load_tables(const char* poly2b_path, const char* poly3b_path);

/* Polynomial value and gradient, table-driven (SOURCE/poly-2b-v6x.cpp:5, poly-3b-v2x.cpp:5). */
double orc_poly2b(const double x[31], double g[31]);
double orc_poly3b(const double x[36], double g[36]);
/* Same polynomials summed monomial by monomial (slow, independent cross-check). */
double orc_poly2b_naive(const double x[31], double g[31]);
double orc_poly3b_naive(const double x[36], double g[36]);

/* x2b_v6x_p::operator() (SOURCE/mbpol-2b-poly.cpp:358-682).  g1/g2 are ASSIGNED.
 * Returns E in kcal/mol. */
double orc_2b(const double w1[9], const double w2[9], double g1[9], double g2[9]);
/* x3b_v2x_p::operator() (SOURCE/mbpol-3b-poly.cpp:148-312).  g1..g3 are ACCUMULATED. */
double orc_3b(const double w1[9], const double w2[9], const double w3[9],
              double g1[9], double g2[9], double g3[9]);

/* 2B variables (31) and 3B variables (36) exactly as the models build them. */
void orc_2b_vars(const double w1[9], const double w2[9], double v[31]);
void orc_3b_vars(const double w1[9], const double w2[9], const double w3[9], double v[36]);

/*
 * mbpol_forces (SOURCE/mbpol.f90:98-449) with the HEAT_CURRENT bookkeeping of
 * do_dimer/do_trimer (SOURCE/mbpol.f90:453-1271) for one replica (bead_size 1).
 *
 *   imcon, cell[9]        DL_POLY boundary key (1,2,3) and cell vectors
 *   nw                    number of waters; listttm2[3*nw] 1-based atom indices
 *   x,y,z[natms]          positions; f{x,y,z}[natms] are ACCUMULATED (-gradient)
 *   eng, vir, stress[9]   ACCUMULATED like engsrp, virsrp, stress
 *   atomic_energy[natms]  ACCUMULATED per-atom MB-pol energy (1/6 per dimer atom,
 *                         1/9 per trimer atom); may be NULL
 *   vx,vy,vz              velocities (may be NULL: no heat current)
 *   jpot[3]               ACCUMULATED potential heat-current term of the MB-pol
 *                         force-matrix entries (raw, un-imaged coordinates)
 *   dense                 1: build the reference's dense N x N force matrix and
 *                         contract it like compute_heat_flux2 (SOURCE/heatcurrent.f90:703-728);
 *                         0: the exact per-interaction contraction (no N^2 memory)
 *   pairs_out/trip_out    optional outputs of the dimer / trimer index lists
 *                         (0-based water indices i<j<k, in loop order); counts in
 *                         *npairs, *ntrip (capacity cap_pairs/cap_trip)
 *   nthreads              >1 runs the 2B and 3B sums on OpenMP threads (the lists
 *                         and the in-place re-imaging are then done per thread on
 *                         private copies; the results differ only by rounding)
 * Returns 0, or 1 if a list capacity was too small.
 */
int orc_mbpol_forces(int imcon, const double* cell, int nw, const int* listttm2,
                     const double* x, const double* y, const double* z,
                     double* fx, double* fy, double* fz,
                     double* eng2, double* eng3, double* vir, double* stress,
                     double* atomic_energy,
                     const double* vx, const double* vy, const double* vz,
                     double* jpot, int dense, int natms,
                     int* pairs_out, long cap_pairs, long* npairs,
                     int* trip_out, long cap_trip, long* ntrip, int nthreads);

/* Time-boxed sample of the 3B sum over an explicit trimer list: evaluates the
 * trimers [0, n) of `trip` (0-based waters) with do_trimer semantics and returns
 * their energy (internal units).  Used for the CPU baseline timing only. */
double orc_trimer_sample(int imcon, const double* cell, int nw, const double* monomers,
                         const int* trip, long n, int nthreads);
double orc_dimer_sample(int imcon, const double* cell, int nw, const double* monomers,
                        const int* pairs, long n, int nthreads);

/* CPU baseline: ranks [rank_begin, rank_end) of a bead_size = `size` split of the
 * reference's pair/triple loops, one OpenMP thread per rank; returns their energy. */
double orc_mbpol_ranks(int imcon, const double* cell, int nw, const int* listttm2, const double* x,
                       const double* y, const double* z, int natms, int rank_begin, int rank_end, int size,
                       int nthreads);

/* 1-body Partridge-Schwenke PES (SOURCE/ps_type_couple.f90, SOURCE/angfrc.f keya 9).
 * orc_pes_load reads tables/ps_pes.tbl and applies init_ps_type_pes. */
int orc_pes_load(const char* path);
void orc_ps_couple(double roh1, double xoh1, double yoh1, double zoh1, double roh2, double xoh2, double yoh2,
                   double zoh2, double theta, double* pterm, double* fdum, double* vterm);
int orc_angfrc_ps(int imcon, const double* cell, int nang, const int* listang, const double* x, const double* y,
                  const double* z, double* fx, double* fy, double* fz, double* engang, double* virang,
                  double* stress, double* atomic_energy, const double* vx, const double* vy, const double* vz,
                  double* jpot);

/* M sites (SOURCE/dlpoly_cmd.f:2041-2057) and DMS charges (SOURCE/qdetermine.f90, MB-pol
 * settings).  M site of water i is atom listttm2[3nw-1] + i (1-based). */
int orc_dms_load(const char* path);
void orc_msites(int imcon, const double* cell, int nw, const int* listttm2, double* x, double* y, double* z,
                double gamma);
double orc_qdetermine(int imcon, const double* cell, int nw, const int* listttm2, const double* x, const double* y,
                      const double* z, double gamma, double* chge, double* dp);

/* image_monomers (SOURCE/mbpol.f90:1275-1301): H atoms next to their O. */
void orc_image_monomers(int imcon, const double* cell, int nw, double* xyz);

/* Short-range dispersion, DL_POLY vdw type 12 (Tang-Toennies damped C6/C8):
 * SOURCE/tang-toennies.f90, SOURCE/forgen.f (tables), SOURCE/srfrce2.f (forces),
 * SOURCE/lrcorrect.f (long-range correction).  Types are 1-based (0: none); prm holds
 * {C6, a6, C8, a8} per pair type, pair (i >= j) at index i(i-1)/2 + j - 1.  Pairs of the
 * same molecule are excluded.  All outputs ACCUMULATED; returns the pair count. */
double orc_tang_toennies(int n, double x);
double orc_tang_toennies_lr(int n, double x);
void orc_disp_tables(int npair, const double* prm, int mxgrid, double dlrpot, double* vvv, double* ggg);
long orc_dispersion(int imcon, const double* cell, int natms, const int* ltype, const int* mol, int ntypes,
                    const double* prm, double rcut, int mxgrid, const double* x, const double* y, const double* z,
                    double* fx, double* fy, double* fz, double* eng, double* vir, double* stress,
                    double* atomic_energy, const double* vx, const double* vy, const double* vz, double* jpot);
void orc_disp_lrc(int ntypes, const double* prm, const int* numtyp, double rcut, double volm, double* elrc,
                  double* virlrc);

/* TTM4-F polarizable electrostatics of MB-pol water (SOURCE/forces.f polar Ewald branch:
 * rfield, ewald1p, iter, coulomb_polar, ewald2p, ewald3p, qdforce) with the heat-current
 * bookkeeping and the M-site redistribution of compute_heat_flux2.  Standard layout, 4*nw
 * sites (water w: O, H1, H2 at 3w..3w+2, M at 3nw + w).
 *   prm[15]   {alpha, rcut, epsq, toler (e A), sor_omega, athole, athole12, athole13, ascc,
 *              ascd, gamma, kmax1, kmax2, kmax3, maxit}
 *   chge, dp  DMS charges and dp[6*nw] from orc_qdetermine; polr (Thole widths), polr2
 *             (polarizabilities) per site
 *   dip*      in: starting dipoles, out: converged dipoles
 *   f*        ACCUMULATED site forces (M sites not redistributed)
 *   out[16]   {engcpe, vircpe, stress[9], iterations, deltadip, eng_polar, eng_kspace,
 *              eng_realspace}
 *   atomic_energy (per site, not redistributed), jpot[3], jkin[3] (the redistributed
 *   electrostatic per-atom energies times the velocities) ACCUMULATED; jpot/jkin need v*.
 *   dense     1: contract a dense N x N force matrix as compute_heat_flux2 does; 0: entry by
 *             entry (same value in exact arithmetic).
 * Returns 0, or 1 when the dipoles did not converge within maxit iterations. */
int orc_polar(const double* prm, int imcon, const double* cell, int nw, const double* x, const double* y,
              const double* z, const double* chge, const double* dp, const double* polr, const double* polr2,
              double* dipx, double* dipy, double* dipz, double* fx, double* fy, double* fz, double* out,
              double* atomic_energy, const double* vx, const double* vy, const double* vz, double* jpot,
              double* jkin, int dense);
double orc_erfcc(double x);
double orc_gammq(double a, double x);
double orc_gammln(double x);

#ifdef __cplusplus
}
#endif
#endif
