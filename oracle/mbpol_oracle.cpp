// Oracle restatement of the MB-pol 2B/3B models and of the mbpol_forces driver
// with its heat-current bookkeeping.  TEST INFRASTRUCTURE ONLY (see oracle.h).
// The 2B/3B models are pinned against the reference's own C++ (golden vectors); the
// mbpol_forces driver is restated from Fortran that cannot be compiled in this image
// (parity unpinned for the driver: checked by finite differences, the dense
// force-matrix heat form and bit-exact list sets).
//
// Floating-point expressions keep the reference's association order so that the
// oracle agrees with the reference to rounding; the file is compiled with
// -ffp-contract=off (no fused multiply-add), like the reference on x86-64.
#include "oracle.h"

#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kEngUnit = 418.4;  // SOURCE/mbpol.f90:37

// ---------------------------------------------------------------------------
// 2B model constants, x2b_v6x_p::x2b_v6x_p (SOURCE/mbpol-2b-poly.cpp:1846-1866)
const double k_HH_intra = -6.480884773303821e-01;
const double k_OH_intra = 1.674518993682975e+00;
const double k_HH_coul = 1.148231864355956e+00;
const double k_OH_coul = 1.205989761123099e+00;
const double k_OO_coul = 1.395357065790959e+00;
const double k_XH_main = 7.347036852042255e-01;
const double k_XO_main = 7.998249864422826e-01;
const double k_XX_main = 7.960663960630585e-01;
const double in_plane_gamma = -9.721486914088159e-02;
const double out_of_plane_gamma = 9.859272078406150e-02;
const double r2i = 4.5, r2f = 6.5;

// Site offsets in the 30-double 2B coordinate block (SOURCE/mbpol-2b-poly.cpp:374-386).
enum { Oa = 0, Ha1 = 3, Ha2 = 6, Ob = 9, Hb1 = 12, Hb2 = 15, Xa1 = 18, Xa2 = 21, Xb1 = 24, Xb2 = 27 };

struct Var2B { int coul; double r0, k; int s1, s2; };
// The 31 variables of SOURCE/mbpol-2b-poly.cpp:415-445 (exp: 0, exp/r: 1).
const Var2B kVars2B[31] = {
    {0, 1.0, k_HH_intra, Ha1, Ha2}, {0, 1.0, k_HH_intra, Hb1, Hb2},
    {0, 1.0, k_OH_intra, Oa, Ha1},  {0, 1.0, k_OH_intra, Oa, Ha2},
    {0, 1.0, k_OH_intra, Ob, Hb1},  {0, 1.0, k_OH_intra, Ob, Hb2},
    {1, 4.0, k_HH_coul, Ha1, Hb1},  {1, 4.0, k_HH_coul, Ha1, Hb2},
    {1, 4.0, k_HH_coul, Ha2, Hb1},  {1, 4.0, k_HH_coul, Ha2, Hb2},
    {1, 4.0, k_OH_coul, Oa, Hb1},   {1, 4.0, k_OH_coul, Oa, Hb2},
    {1, 4.0, k_OH_coul, Ob, Ha1},   {1, 4.0, k_OH_coul, Ob, Ha2},
    {1, 4.0, k_OO_coul, Oa, Ob},
    {0, 4.0, k_XH_main, Xa1, Hb1},  {0, 4.0, k_XH_main, Xa1, Hb2},
    {0, 4.0, k_XH_main, Xa2, Hb1},  {0, 4.0, k_XH_main, Xa2, Hb2},
    {0, 4.0, k_XH_main, Xb1, Ha1},  {0, 4.0, k_XH_main, Xb1, Ha2},
    {0, 4.0, k_XH_main, Xb2, Ha1},  {0, 4.0, k_XH_main, Xb2, Ha2},
    {0, 4.0, k_XO_main, Oa, Xb1},   {0, 4.0, k_XO_main, Oa, Xb2},
    {0, 4.0, k_XO_main, Ob, Xa1},   {0, 4.0, k_XO_main, Ob, Xa2},
    {0, 4.0, k_XX_main, Xa1, Xb1},  {0, 4.0, k_XX_main, Xa1, Xb2},
    {0, 4.0, k_XX_main, Xa2, Xb1},  {0, 4.0, k_XX_main, Xa2, Xb2},
};

// variable::v_exp / v_coul (SOURCE/mbpol-2b-poly.cpp:27-68): value, and the
// gradient direction d(value)/d(p1 - p2) in gv.
double var2b(const Var2B& v, const double* xc, double gv[3]) {
    gv[0] = xc[v.s1 + 0] - xc[v.s2 + 0];
    gv[1] = xc[v.s1 + 1] - xc[v.s2 + 1];
    gv[2] = xc[v.s1 + 2] - xc[v.s2 + 2];
    const double rsq = gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2];
    const double r = std::sqrt(rsq);
    const double e = std::exp(v.k * (v.r0 - r));
    double val, gg;
    if (!v.coul) {
        val = e;
        gg = -v.k * e / r;
    } else {
        const double rinv = 1.0 / r;
        val = e * rinv;
        gg = -(v.k + rinv) * val * rinv;
    }
    gv[0] *= gg;
    gv[1] *= gg;
    gv[2] *= gg;
    return val;
}

// monomer::setup (SOURCE/mbpol-2b-poly.cpp:118-140): the two X sites.
void xsites(const double* ohh, double oh1[3], double oh2[3], double* x1, double* x2) {
    for (int i = 0; i < 3; ++i) {
        oh1[i] = ohh[i + 3] - ohh[i];
        oh2[i] = ohh[i + 6] - ohh[i];
    }
    const double v[3] = {oh1[1] * oh2[2] - oh1[2] * oh2[1],
                         oh1[2] * oh2[0] - oh1[0] * oh2[2],
                         oh1[0] * oh2[1] - oh1[1] * oh2[0]};
    for (int i = 0; i < 3; ++i) {
        const double in_plane = ohh[i] + 0.5 * in_plane_gamma * (oh1[i] + oh2[i]);
        const double out_of_plane = out_of_plane_gamma * v[i];
        x1[i] = in_plane + out_of_plane;
        x2[i] = in_plane - out_of_plane;
    }
}

// monomer::grads (SOURCE/mbpol-2b-poly.cpp:144-177): X-site gradients onto O, H1, H2.
void xsite_grads(const double oh1[3], const double oh2[3], const double* g1, const double* g2,
                 double* grd) {
    const double gm[3] = {g1[0] - g2[0], g1[1] - g2[1], g1[2] - g2[2]};
    const double t1[3] = {oh2[1] * gm[2] - oh2[2] * gm[1], oh2[2] * gm[0] - oh2[0] * gm[2],
                          oh2[0] * gm[1] - oh2[1] * gm[0]};
    const double t2[3] = {oh1[1] * gm[2] - oh1[2] * gm[1], oh1[2] * gm[0] - oh1[0] * gm[2],
                          oh1[0] * gm[1] - oh1[1] * gm[0]};
    for (int i = 0; i < 3; ++i) {
        const double gsum = g1[i] + g2[i];
        const double in_plane = 0.5 * in_plane_gamma * gsum;
        const double gh1 = in_plane + out_of_plane_gamma * t1[i];
        const double gh2 = in_plane - out_of_plane_gamma * t2[i];
        grd[i + 0] += gsum - (gh1 + gh2);
        grd[i + 3] += gh1;
        grd[i + 6] += gh2;
    }
}

// f_switch with bounds ri, rf (SOURCE/mbpol-2b-poly.cpp:340-354, mbpol-3b-poly.cpp:130-144).
double f_switch(double r, double ri, double rf, double& g) {
    if (r > rf) {
        g = 0.0;
        return 0.0;
    } else if (r > ri) {
        const double t1 = M_PI / (rf - ri);
        const double x = (r - ri) * t1;
        g = -std::sin(x) * t1 / 2.0;
        return (1.0 + std::cos(x)) / 2.0;
    }
    g = 0.0;
    return 1.0;
}

void build_2b_coords(const double* w1, const double* w2, double* xc, double oha[2][3], double ohb[2][3]) {
    std::memcpy(xc, w1, 9 * sizeof(double));
    std::memcpy(xc + 9, w2, 9 * sizeof(double));
    xsites(xc + Oa, oha[0], oha[1], xc + Xa1, xc + Xa2);
    xsites(xc + Ob, ohb[0], ohb[1], xc + Xb1, xc + Xb2);
}

// ---------------------------------------------------------------------------
// 3B model constants, x3b_v2x_p::x3b_v2x_p (SOURCE/mbpol-3b-poly.cpp:1486-1506)
const double r3i = 0.0, r3f = 4.5;
const double kHH_intra = -2.254303257872797e+00;
const double kOH_intra = -2.564771901404151e-01;
const double kHH = 4.247920544074333e-01;
const double kOH = 8.128985941165371e-01;
const double kOO = 3.749457984616480e-02;
const double dHH_intra = 1.690594510379166e+00;
const double dOH_intra = -2.999999868517452e+00;
const double dHH = 3.499031358429095e+00;
const double dOH = 4.854042963514281e+00;
const double dOO = 4.816312044947604e-08;

struct Var3B { double k, r0; int a1, a2; };  // atom offsets in the 27-double trimer block
enum { tOa = 0, tHa1 = 3, tHa2 = 6, tOb = 9, tHb1 = 12, tHb2 = 15, tOc = 18, tHc1 = 21, tHc2 = 24 };
// The 36 variables of SOURCE/mbpol-3b-poly.cpp:170-206.
const Var3B kVars3B[36] = {
    {kHH_intra, dHH_intra, tHa1, tHa2}, {kHH_intra, dHH_intra, tHb1, tHb2},
    {kHH_intra, dHH_intra, tHc1, tHc2}, {kOH_intra, dOH_intra, tOa, tHa1},
    {kOH_intra, dOH_intra, tOa, tHa2},  {kOH_intra, dOH_intra, tOb, tHb1},
    {kOH_intra, dOH_intra, tOb, tHb2},  {kOH_intra, dOH_intra, tOc, tHc1},
    {kOH_intra, dOH_intra, tOc, tHc2},
    {kHH, dHH, tHa1, tHb1}, {kHH, dHH, tHa1, tHb2}, {kHH, dHH, tHa1, tHc1}, {kHH, dHH, tHa1, tHc2},
    {kHH, dHH, tHa2, tHb1}, {kHH, dHH, tHa2, tHb2}, {kHH, dHH, tHa2, tHc1}, {kHH, dHH, tHa2, tHc2},
    {kHH, dHH, tHb1, tHc1}, {kHH, dHH, tHb1, tHc2}, {kHH, dHH, tHb2, tHc1}, {kHH, dHH, tHb2, tHc2},
    {kOH, dOH, tOa, tHb1},  {kOH, dOH, tOa, tHb2},  {kOH, dOH, tOa, tHc1},  {kOH, dOH, tOa, tHc2},
    {kOH, dOH, tOb, tHa1},  {kOH, dOH, tOb, tHa2},  {kOH, dOH, tOb, tHc1},  {kOH, dOH, tOb, tHc2},
    {kOH, dOH, tOc, tHa1},  {kOH, dOH, tOc, tHa2},  {kOH, dOH, tOc, tHb1},  {kOH, dOH, tOc, tHb2},
    {kOO, dOO, tOa, tOb},   {kOO, dOO, tOa, tOc},   {kOO, dOO, tOb, tOc},
};

// v_intra / v_main (SOURCE/mbpol-3b-poly.cpp:12-62): exp(-k (d - r0)).
double var3b(const Var3B& v, const double* t) {
    const double dx[3] = {t[v.a1] - t[v.a2], t[v.a1 + 1] - t[v.a2 + 1], t[v.a1 + 2] - t[v.a2 + 2]};
    const double dsq = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    const double d = std::sqrt(dsq);
    return std::exp(-v.k * (d - v.r0));
}

// g_intra / g_main (SOURCE/mbpol-3b-poly.cpp:26-47, 66-87) without the force_matrix part.
void gvar3b(const Var3B& v, double g, const double* t, double* gt) {
    const double dx[3] = {t[v.a1] - t[v.a2], t[v.a1 + 1] - t[v.a2 + 1], t[v.a1 + 2] - t[v.a2 + 2]};
    const double dsq = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    const double d = std::sqrt(dsq);
    const double gg = -v.k * g * std::exp(-v.k * (d - v.r0)) / d;
    for (int i = 0; i < 3; ++i) {
        gt[v.a1 + i] += gg * dx[i];
        gt[v.a2 + i] -= gg * dx[i];
    }
}

// ---------------------------------------------------------------------------
// image_vectors (SOURCE/mbpol.f90:1305-1361); nint = round half away from zero.
void invert3(const double* a, double* b) {  // SOURCE/invert.f
    b[0] = a[4] * a[8] - a[5] * a[7];
    b[1] = a[2] * a[7] - a[1] * a[8];
    b[2] = a[1] * a[5] - a[2] * a[4];
    b[3] = a[5] * a[6] - a[3] * a[8];
    b[4] = a[0] * a[8] - a[2] * a[6];
    b[5] = a[2] * a[3] - a[0] * a[5];
    b[6] = a[3] * a[7] - a[4] * a[6];
    b[7] = a[1] * a[6] - a[0] * a[7];
    b[8] = a[0] * a[4] - a[1] * a[3];
    const double d = a[0] * b[0] + a[3] * b[1] + a[6] * b[2];
    double r = 0.0;
    if (std::fabs(d) > 0.0) r = 1.0 / d;
    for (int i = 0; i < 9; ++i) b[i] = r * b[i];
}

void image_vectors(int imcon, const double* cell, int n, double* dx) {
    if (imcon == 1) {
        const double a1 = 1.0 / cell[0];
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) dx[3 * i + k] = dx[3 * i + k] - cell[0] * std::round(dx[3 * i + k] * a1);
    } else if (imcon == 2) {
        const double a1 = 1.0 / cell[0], b1 = 1.0 / cell[4], c1 = 1.0 / cell[8];
        for (int i = 0; i < n; ++i) {
            dx[3 * i + 0] = dx[3 * i + 0] - cell[0] * std::round(dx[3 * i + 0] * a1);
            dx[3 * i + 1] = dx[3 * i + 1] - cell[4] * std::round(dx[3 * i + 1] * b1);
            dx[3 * i + 2] = dx[3 * i + 2] - cell[8] * std::round(dx[3 * i + 2] * c1);
        }
    } else {
        double rc[9];
        invert3(cell, rc);
        for (int i = 0; i < n; ++i) {
            double* d = dx + 3 * i;
            const double ssx = (rc[0] * d[0] + rc[3] * d[1] + rc[6] * d[2]);
            const double ssy = (rc[1] * d[0] + rc[4] * d[1] + rc[7] * d[2]);
            const double ssz = (rc[2] * d[0] + rc[5] * d[1] + rc[8] * d[2]);
            const double xss = ssx - std::round(ssx);
            const double yss = ssy - std::round(ssy);
            const double zss = ssz - std::round(ssz);
            d[0] = (cell[0] * xss + cell[3] * yss + cell[6] * zss);
            d[1] = (cell[1] * xss + cell[4] * yss + cell[7] * zss);
            d[2] = (cell[2] * xss + cell[5] * yss + cell[8] * zss);
        }
    }
}

struct HeatAcc {
    // per-rank private accumulators of the driver
    std::vector<double> f, ae, fm;  // forces (3N), atomic energies (N), dense force matrix (N*N*3)
    double eng2 = 0, eng3 = 0, vir = 0, stress[9] = {0};
    double jpot[3] = {0};
};

struct DriverIn {
    int imcon; const double* cell; int nw; const int* list;
    const double *x, *y, *z, *vx, *vy, *vz;
    int natms; int dense;
};

// Per-interaction heat term: sum_i (F_i . v_i)(n r_i - sum_j r_j), F_i = -(g_i/n) engunit,
// which is what compute_heat_flux2 (SOURCE/heatcurrent.f90:703-728) extracts from the
// force-matrix rows F(i, j) = -(1/n) g_i engunit written for every j of the cluster
// (SOURCE/mbpol.f90:533-556, :920-952).  Raw coordinates, as in the reference.
void heat_cluster(const DriverIn& in, HeatAcc& acc, int n, const int* idx, const double* const* g,
                  double inv_n) {
    if (!in.vx) return;
    double rsum[3] = {0, 0, 0};
    for (int a = 0; a < n; ++a) {
        rsum[0] += in.x[idx[a]];
        rsum[1] += in.y[idx[a]];
        rsum[2] += in.z[idx[a]];
    }
    for (int a = 0; a < n; ++a) {
        const int i = idx[a];
        const double f0 = -(inv_n * g[a][0]) * kEngUnit;
        const double f1 = -(inv_n * g[a][1]) * kEngUnit;
        const double f2 = -(inv_n * g[a][2]) * kEngUnit;
        if (in.dense) {
            const size_t N = (size_t)in.natms;
            for (int b = 0; b < n; ++b) {
                const size_t j = (size_t)idx[b];
                acc.fm[((size_t)i * N + j) * 3 + 0] += f0;
                acc.fm[((size_t)i * N + j) * 3 + 1] += f1;
                acc.fm[((size_t)i * N + j) * 3 + 2] += f2;
            }
        } else {
            const double fv = f0 * in.vx[i] + f1 * in.vy[i] + f2 * in.vz[i];
            acc.jpot[0] += fv * (n * in.x[i] - rsum[0]);
            acc.jpot[1] += fv * (n * in.y[i] - rsum[1]);
            acc.jpot[2] += fv * (n * in.z[i] - rsum[2]);
        }
    }
}

// do_dimer (SOURCE/mbpol.f90:453-790).  w1 is re-imaged in place next to w2.
bool do_dimer(const DriverIn& in, double* w1, const double* w2, int o1, int o2, HeatAcc& acc) {
    double r12[3] = {w1[0] - w2[0], w1[1] - w2[1], w1[2] - w2[2]};
    image_vectors(in.imcon, in.cell, 1, r12);
    if ((r12[0] * r12[0] + r12[1] * r12[1] + r12[2] * r12[2]) > r2f * r2f) return false;
    for (int k = 0; k < 3; ++k) {
        w1[3 + k] = (w1[3 + k] - w1[k]) + (w2[k] + r12[k]);
        w1[6 + k] = (w1[6 + k] - w1[k]) + (w2[k] + r12[k]);
        w1[k] = w2[k] + r12[k];
    }
    double g1[9], g2[9];
    const double e2 = orc_2b(w1, w2, g1, g2);
    acc.eng2 += e2 * kEngUnit;
    const int idx[6] = {o1, o1 + 1, o1 + 2, o2, o2 + 1, o2 + 2};
    for (int a = 0; a < 6; ++a) acc.ae[idx[a]] += (1.0 / 6.0) * e2 * kEngUnit;
    const double* gp[6] = {g1, g1 + 3, g1 + 6, g2, g2 + 3, g2 + 6};
    heat_cluster(in, acc, 6, idx, gp, 1.0 / 6.0);
    for (int k = 0; k < 9; ++k) {
        g1[k] = g1[k] * kEngUnit;
        acc.vir = acc.vir + w1[k] * g1[k];
        g2[k] = g2[k] * kEngUnit;
        acc.vir = acc.vir + w2[k] * g2[k];
    }
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            acc.f[3 * (o1 + a) + c] -= g1[3 * a + c];
            acc.f[3 * (o2 + a) + c] -= g2[3 * a + c];
        }
    const double* ws[2] = {w1, w2};
    const double* gs[2] = {g1, g2};
    // strs(1..9) (SOURCE/mbpol.f90:609-667), symmetric pairs copied, then negated
    double s[9];
    const int rr[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    double sv[6];
    for (int q = 0; q < 6; ++q) {
        double t = 0.0;
        bool first = true;
        for (int m = 0; m < 2; ++m)
            for (int a = 0; a < 3; ++a) {
                const double p = ws[m][3 * a + rr[q][0]] * gs[m][3 * a + rr[q][1]];
                t = first ? p : t + p;
                first = false;
            }
        sv[q] = t;
    }
    s[0] = sv[0]; s[1] = sv[1]; s[2] = sv[2]; s[3] = sv[1]; s[4] = sv[3];
    s[5] = sv[4]; s[6] = sv[2]; s[7] = sv[4]; s[8] = sv[5];
    for (int q = 0; q < 9; ++q) acc.stress[q] += -s[q];
    return true;
}

// do_trimer (SOURCE/mbpol.f90:795-1271).  w1 and w3 are re-imaged in place around w2.
bool do_trimer(const DriverIn& in, double* w1, const double* w2, double* w3, int o1, int o2, int o3,
               HeatAcc& acc) {
    double rab[9];
    for (int k = 0; k < 3; ++k) {
        rab[k + 0] = w1[k] - w2[k];
        rab[k + 3] = w2[k] - w3[k];
        rab[k + 6] = w1[k] - w3[k];
    }
    image_vectors(in.imcon, in.cell, 3, rab);
    double r12 = 0.0, r23 = 0.0, r13 = 0.0;
    for (int k = 0; k < 3; ++k) {
        r12 = r12 + rab[k] * rab[k];
        r23 = r23 + rab[k + 3] * rab[k + 3];
        r13 = r13 + rab[k + 6] * rab[k + 6];
    }
    r12 = std::sqrt(r12);
    r23 = std::sqrt(r23);
    r13 = std::sqrt(r13);
    const bool big1 = r12 > r3f || r13 > r3f;
    const bool big2 = r12 > r3f || r23 > r3f;
    const bool big3 = r13 > r3f || r23 > r3f;
    if (big1 && big2 && big3) return false;
    for (int k = 0; k < 3; ++k) {
        w1[3 + k] = (w1[3 + k] - w1[k]) + (w2[k] + rab[k]);
        w1[6 + k] = (w1[6 + k] - w1[k]) + (w2[k] + rab[k]);
        w1[k] = w2[k] + rab[k];
        w3[3 + k] = (w3[3 + k] - w3[k]) + (w2[k] - rab[k + 3]);
        w3[6 + k] = (w3[6 + k] - w3[k]) + (w2[k] - rab[k + 3]);
        w3[k] = w2[k] - rab[k + 3];
    }
    double g1[9] = {0}, g2[9] = {0}, g3[9] = {0};
    const double e3 = orc_3b(w1, w2, w3, g1, g2, g3);
    acc.eng3 += e3 * kEngUnit;
    const int idx[9] = {o1, o1 + 1, o1 + 2, o2, o2 + 1, o2 + 2, o3, o3 + 1, o3 + 2};
    for (int a = 0; a < 9; ++a) acc.ae[idx[a]] += (1.0 / 9.0) * e3 * kEngUnit;
    const double* gp[9] = {g1, g1 + 3, g1 + 6, g2, g2 + 3, g2 + 6, g3, g3 + 3, g3 + 6};
    heat_cluster(in, acc, 9, idx, gp, 1.0 / 9.0);
    for (int k = 0; k < 9; ++k) {
        g1[k] = g1[k] * kEngUnit;
        acc.vir = acc.vir + w1[k] * g1[k];
        g2[k] = g2[k] * kEngUnit;
        acc.vir = acc.vir + w2[k] * g2[k];
        g3[k] = g3[k] * kEngUnit;
        acc.vir = acc.vir + w3[k] * g3[k];
    }
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            acc.f[3 * (o1 + a) + c] -= g1[3 * a + c];
            acc.f[3 * (o2 + a) + c] -= g2[3 * a + c];
            acc.f[3 * (o3 + a) + c] -= g3[3 * a + c];
        }
    const double* ws[3] = {w1, w2, w3};
    const double* gs[3] = {g1, g2, g3};
    const int rr[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    double sv[6];
    for (int q = 0; q < 6; ++q) {
        double t = 0.0;
        bool first = true;
        for (int m = 0; m < 3; ++m)
            for (int a = 0; a < 3; ++a) {
                const double p = ws[m][3 * a + rr[q][0]] * gs[m][3 * a + rr[q][1]];
                t = first ? p : t + p;
                first = false;
            }
        sv[q] = t;
    }
    const double s[9] = {sv[0], sv[1], sv[2], sv[1], sv[3], sv[4], sv[2], sv[4], sv[5]};
    for (int q = 0; q < 9; ++q) acc.stress[q] += -s[q];
    return true;
}

// One rank of mbpol_forces (SOURCE/mbpol.f90:98-449) with bead_rank/bead_size striding.
int run_rank(const DriverIn& in, int rank, int size, HeatAcc& acc, int* pairs_out, long cap_pairs,
             long* npairs, int* trip_out, long cap_trip, long* ntrip) {
    const int nw = in.nw;
    std::vector<double> mono(9 * (size_t)nw);
    for (int t = 0; t < 3 * nw; ++t) {
        const int i = in.list[t] - 1;
        mono[3 * t + 0] = in.x[i];
        mono[3 * t + 1] = in.y[i];
        mono[3 * t + 2] = in.z[i];
    }
    orc_image_monomers(in.imcon, in.cell, nw, mono.data());
    int rc = 0;
    long np = 0, nt = 0;
    // pairs
    {
        const long long nw2 = ((long long)nw * (nw - 1)) / 2;
        long long i = 1, j = 2 + rank;
        for (long long t = rank; t <= nw2 - 1; t += size) {
            const int o1 = in.list[3 * i - 3] - 1, o2 = in.list[3 * j - 3] - 1;
            if (do_dimer(in, &mono[9 * (i - 1)], &mono[9 * (j - 1)], o1, o2, acc)) {
                if (pairs_out) {
                    if (np < cap_pairs) {
                        pairs_out[2 * np] = (int)(i - 1);
                        pairs_out[2 * np + 1] = (int)(j - 1);
                    } else {
                        rc = 1;
                    }
                }
                ++np;
            }
            // The advance after the last pair is dead; in the reference the while loop
            // then runs until its 32-bit integers wrap, so it is skipped here.
            if (t + size > nw2 - 1) break;
            j = j + size;
            if (j > nw) {
                while (j > nw) {
                    i = i + 1;
                    j = i + j - nw;
                }
            }
        }
    }
    // triples
    {
        const long long nw3 = ((long long)nw * (nw - 1) * (nw - 2)) / 6;
        long long i = 1, j = 2, k = 3 + rank;
        for (long long t = rank; t <= nw3 - 1; t += size) {
            const int o1 = in.list[3 * i - 3] - 1, o2 = in.list[3 * j - 3] - 1, o3 = in.list[3 * k - 3] - 1;
            if (do_trimer(in, &mono[9 * (i - 1)], &mono[9 * (j - 1)], &mono[9 * (k - 1)], o1, o2, o3, acc)) {
                if (trip_out) {
                    if (nt < cap_trip) {
                        trip_out[3 * nt] = (int)(i - 1);
                        trip_out[3 * nt + 1] = (int)(j - 1);
                        trip_out[3 * nt + 2] = (int)(k - 1);
                    } else {
                        rc = 1;
                    }
                }
                ++nt;
            }
            if (t + size > nw3 - 1) break;  // dead advance after the last triple
            k = k + size;
            if (k > nw) {
                while (k > nw) {
                    j = j + 1;
                    if ((j + 1) > nw) {
                        i = i + 1;
                        j = i + 1;
                    }
                    k = j + (k - nw);
                }
            }
        }
    }
    if (npairs) *npairs = np;
    if (ntrip) *ntrip = nt;
    return rc;
}

}  // namespace

// ===========================================================================
extern "C" void orc_2b_vars(const double* w1, const double* w2, double* v) {
    double xc[30], oha[2][3], ohb[2][3], gv[3];
    build_2b_coords(w1, w2, xc, oha, ohb);
    for (int i = 0; i < 31; ++i) v[i] = var2b(kVars2B[i], xc, gv);
}

extern "C" double orc_2b(const double* w1, const double* w2, double* g1, double* g2) {
    const double dOO[3] = {w1[0] - w2[0], w1[1] - w2[1], w1[2] - w2[2]};
    const double rOOsq = dOO[0] * dOO[0] + dOO[1] * dOO[1] + dOO[2] * dOO[2];
    const double rOO = std::sqrt(rOOsq);
    if (rOO > r2f) {
        // the reference returns 0 here and leaves g1/g2 untouched; the oracle zeroes them
        for (int i = 0; i < 9; ++i) g1[i] = g2[i] = 0.0;
        return 0.0;
    }
    double xc[30], oha[2][3], ohb[2][3];
    build_2b_coords(w1, w2, xc, oha, ohb);
    double v[31], gv[31][3];
    for (int i = 0; i < 31; ++i) v[i] = var2b(kVars2B[i], xc, gv[i]);
    double g[31];
    const double E_poly = orc_poly2b(v, g);
    double xgrd[30] = {0};
    for (int i = 0; i < 31; ++i) {
        const Var2B& d = kVars2B[i];
        for (int c = 0; c < 3; ++c) {
            const double t = g[i] * gv[i][c];
            xgrd[d.s1 + c] += t;
            xgrd[d.s2 + c] -= t;
        }
    }
    xsite_grads(oha[0], oha[1], xgrd + Xa1, xgrd + Xa2, xgrd + Oa);
    xsite_grads(ohb[0], ohb[1], xgrd + Xb1, xgrd + Xb2, xgrd + Ob);
    double gsw;
    const double sw = f_switch(rOO, r2i, r2f, gsw);
    for (int i = 0; i < 9; ++i) {
        g1[i] = sw * xgrd[i];
        g2[i] = sw * xgrd[i + 9];
    }
    gsw *= E_poly / rOO;
    for (int i = 0; i < 3; ++i) {
        const double d = gsw * dOO[i];
        g1[i] += d;
        g2[i] -= d;
    }
    return sw * E_poly;
}

extern "C" void orc_3b_vars(const double* w1, const double* w2, const double* w3, double* v) {
    double t[27];
    std::memcpy(t, w1, 9 * sizeof(double));
    std::memcpy(t + 9, w2, 9 * sizeof(double));
    std::memcpy(t + 18, w3, 9 * sizeof(double));
    for (int i = 0; i < 36; ++i) v[i] = var3b(kVars3B[i], t);
}

extern "C" double orc_3b(const double* w1, const double* w2, const double* w3, double* g1, double* g2,
                         double* g3) {
    double t[27];
    std::memcpy(t, w1, 9 * sizeof(double));
    std::memcpy(t + 9, w2, 9 * sizeof(double));
    std::memcpy(t + 18, w3, 9 * sizeof(double));
    double x[36];
    for (int i = 0; i < 36; ++i) x[i] = var3b(kVars3B[i], t);
    double g[36];
    double retval = orc_poly3b(x, g);
    double rab[3], rac[3], rbc[3];
    double drab = 0, drac = 0, drbc = 0;
    for (int n = 0; n < 3; ++n) {
        rab[n] = w1[n] - w2[n];
        drab += rab[n] * rab[n];
        rac[n] = w1[n] - w3[n];
        drac += rac[n] * rac[n];
        rbc[n] = w2[n] - w3[n];
        drbc += rbc[n] * rbc[n];
    }
    drab = std::sqrt(drab);
    drac = std::sqrt(drac);
    drbc = std::sqrt(drbc);
    double gab, gac, gbc;
    const double sab = f_switch(drab, r3i, r3f, gab);
    const double sac = f_switch(drac, r3i, r3f, gac);
    const double sbc = f_switch(drbc, r3i, r3f, gbc);
    const double s = sab * sac + sab * sbc + sac * sbc;
    for (int n = 0; n < 36; ++n) g[n] *= s;
    double gt[27];
    for (int i = 0; i < 9; ++i) {
        gt[i] = g1[i];
        gt[9 + i] = g2[i];
        gt[18 + i] = g3[i];
    }
    for (int i = 0; i < 36; ++i) gvar3b(kVars3B[i], g[i], t, gt);
    gab *= (sac + sbc) * retval / drab;
    gac *= (sab + sbc) * retval / drac;
    gbc *= (sab + sac) * retval / drbc;
    retval *= s;
    for (int n = 0; n < 3; ++n) {
        gt[n] += gab * rab[n] + gac * rac[n];
        gt[9 + n] += gbc * rbc[n] - gab * rab[n];
        gt[18 + n] -= gac * rac[n] + gbc * rbc[n];
    }
    for (int i = 0; i < 9; ++i) {
        g1[i] = gt[i];
        g2[i] = gt[9 + i];
        g3[i] = gt[18 + i];
    }
    return retval;
}

// image_vectors for the other restatements in this library (images.f's imcon 1-3)
extern "C" void orc_image_vectors(int imcon, const double* cell, int n, double* dx) {
    image_vectors(imcon, cell, n, dx);
}

extern "C" void orc_image_monomers(int imcon, const double* cell, int nw, double* xyz) {
    for (int i = 0; i < nw; ++i) {
        double* w = xyz + 9 * (size_t)i;
        double oh[6];
        for (int k = 0; k < 3; ++k) {
            oh[k] = w[3 + k] - w[k];
            oh[k + 3] = w[6 + k] - w[k];
        }
        image_vectors(imcon, cell, 2, oh);
        for (int k = 0; k < 3; ++k) {
            w[3 + k] = w[k] + oh[k];
            w[6 + k] = w[k] + oh[k + 3];
        }
    }
}

extern "C" int orc_mbpol_forces(int imcon, const double* cell, int nw, const int* listttm2,
                                const double* x, const double* y, const double* z, double* fx, double* fy,
                                double* fz, double* eng2, double* eng3, double* vir, double* stress,
                                double* atomic_energy, const double* vx, const double* vy, const double* vz,
                                double* jpot, int dense, int natms, int* pairs_out, long cap_pairs,
                                long* npairs, int* trip_out, long cap_trip, long* ntrip, int nthreads) {
    DriverIn in{imcon, cell, nw, listttm2, x, y, z, vx, vy, vz, natms, dense};
    if (nthreads < 1) nthreads = 1;
    if (pairs_out || trip_out) nthreads = 1;  // lists are reported in the reference's loop order
    std::vector<HeatAcc> accs(nthreads);
    int rc = 0;
    long np = 0, nt = 0;
#pragma omp parallel for num_threads(nthreads) schedule(static, 1) reduction(| : rc) reduction(+ : np, nt)
    for (int r = 0; r < nthreads; ++r) {
        HeatAcc& a = accs[r];
        a.f.assign(3 * (size_t)natms, 0.0);
        a.ae.assign(natms, 0.0);
        if (dense) a.fm.assign((size_t)natms * natms * 3, 0.0);
        long p = 0, t = 0;
        rc |= run_rank(in, r, nthreads, a, pairs_out, cap_pairs, &p, trip_out, cap_trip, &t);
        np += p;
        nt += t;
    }
    // final_sum: combine the ranks (SOURCE/heatcurrent.f90:1129-1294, gdsum)
    for (int r = 0; r < nthreads; ++r) {
        const HeatAcc& a = accs[r];
        for (int i = 0; i < natms; ++i) {
            fx[i] += a.f[3 * i];
            fy[i] += a.f[3 * i + 1];
            fz[i] += a.f[3 * i + 2];
            if (atomic_energy) atomic_energy[i] += a.ae[i];
        }
        *eng2 += a.eng2;
        *eng3 += a.eng3;
        *vir += a.vir;
        for (int q = 0; q < 9; ++q) stress[q] += a.stress[q];
        if (jpot && !dense)
            for (int c = 0; c < 3; ++c) jpot[c] += a.jpot[c];
    }
    if (jpot && dense && vx) {
        // compute_heat_flux2's jpot double loop over the summed dense matrix
        std::vector<double> fm((size_t)natms * natms * 3, 0.0);
        for (int r = 0; r < nthreads; ++r)
            for (size_t q = 0; q < fm.size(); ++q) fm[q] += accs[r].fm[q];
        double jp[3] = {0, 0, 0};
        for (int i = 0; i < natms; ++i) {
            for (int j = 0; j < natms; ++j) {
                if (i == j) continue;
                const double* f = &fm[((size_t)i * natms + j) * 3];
                const double fv = f[0] * vx[i] + f[1] * vy[i] + f[2] * vz[i];
                jp[0] += (x[i] - x[j]) * fv;
                jp[1] += (y[i] - y[j]) * fv;
                jp[2] += (z[i] - z[j]) * fv;
            }
        }
        for (int c = 0; c < 3; ++c) jpot[c] += jp[c];
    }
    if (npairs) *npairs = np;
    if (ntrip) *ntrip = nt;
    return rc;
}

// ---------------------------------------------------------------------------
// Timed samples over explicit lists (CPU baseline): the same per-dimer/trimer work as
// do_dimer/do_trimer (imaging, model, energy, forces, virial), no heat bookkeeping.
namespace {
double sample_impl(int imcon, const double* cell, int nw, const double* monomers, const int* list,
                   long n, int nthreads, int body) {
    double etot = 0.0;
#pragma omp parallel num_threads(nthreads) reduction(+ : etot)
    {
        std::vector<double> mono(monomers, monomers + 9 * (size_t)nw);
        std::vector<double> f(9 * (size_t)nw, 0.0);
        std::vector<int> lst(3 * (size_t)nw);
        for (int t = 0; t < 3 * nw; ++t) lst[t] = t + 1;
        std::vector<double> xs(3 * (size_t)nw), ys(3 * (size_t)nw), zs(3 * (size_t)nw);
        for (int t = 0; t < 3 * nw; ++t) {
            xs[t] = monomers[3 * t];
            ys[t] = monomers[3 * t + 1];
            zs[t] = monomers[3 * t + 2];
        }
        DriverIn in{imcon, cell, nw, lst.data(), xs.data(), ys.data(), zs.data(), nullptr, nullptr, nullptr,
                    3 * nw, 0};
        HeatAcc acc;
        acc.f.assign(9 * (size_t)nw, 0.0);
        acc.ae.assign(3 * (size_t)nw, 0.0);
#pragma omp for schedule(static)
        for (long q = 0; q < n; ++q) {
            if (body == 2) {
                const int i = list[2 * q], j = list[2 * q + 1];
                do_dimer(in, &mono[9 * (size_t)i], &mono[9 * (size_t)j], 3 * i, 3 * j, acc);
            } else {
                const int i = list[3 * q], j = list[3 * q + 1], k = list[3 * q + 2];
                do_trimer(in, &mono[9 * (size_t)i], &mono[9 * (size_t)j], &mono[9 * (size_t)k], 3 * i, 3 * j,
                          3 * k, acc);
            }
        }
        etot += acc.eng2 + acc.eng3;
    }
    return etot;
}
}  // namespace

extern "C" double orc_trimer_sample(int imcon, const double* cell, int nw, const double* monomers,
                                    const int* trip, long n, int nthreads) {
    return sample_impl(imcon, cell, nw, monomers, trip, n, nthreads < 1 ? 1 : nthreads, 3);
}

extern "C" double orc_dimer_sample(int imcon, const double* cell, int nw, const double* monomers,
                                   const int* pairs, long n, int nthreads) {
    return sample_impl(imcon, cell, nw, monomers, pairs, n, nthreads < 1 ? 1 : nthreads, 2);
}

// CPU baseline: ranks [rank_begin, rank_end) of a bead_size = `size` decomposition
// (SOURCE/mbpol.f90:215-226, :311-314), one OpenMP thread per rank.  Returns the summed
// energy; the work done is (rank_end - rank_begin)/size of one full evaluation.
extern "C" double orc_mbpol_ranks(int imcon, const double* cell, int nw, const int* listttm2, const double* x,
                                  const double* y, const double* z, int natms, int rank_begin, int rank_end,
                                  int size, int nthreads) {
    DriverIn in{imcon, cell, nw, listttm2, x, y, z, nullptr, nullptr, nullptr, natms, 0};
    double e = 0.0;
    const int n = rank_end - rank_begin;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1) reduction(+ : e)
    for (int q = 0; q < n; ++q) {
        HeatAcc a;
        a.f.assign(3 * (size_t)natms, 0.0);
        a.ae.assign(natms, 0.0);
        long p = 0, t = 0;
        run_rank(in, rank_begin + q, size, a, nullptr, 0, &p, nullptr, 0, &t);
        e += a.eng2 + a.eng3;
    }
    return e;
}
