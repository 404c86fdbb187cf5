// Oracle for the TTM4-F polarizable electrostatics of MB-pol water as the reference's
// polar Ewald branch computes it (keyword vmbpol: Thole exp-4 damping, all charges and
// dipoles smeared, DMS charges; SOURCE/simdef_cmd.f:1040-1060).
//
// Parity unpinned: the reference's Fortran cannot be compiled in this image and the
// reference ships no input or output files, so this restatement is checked by
// self-consistency (forces against finite differences of the energy, momentum, the
// dense-matrix heat form, the published erfcc and gammq methods), not against a
// reference run.
// TEST INFRASTRUCTURE ONLY (see oracle.h).  Restates, operation by operation:
//   - erfcc (SOURCE/erfcc.f; its literals are default REAL, i.e. single precision)
//     and the table ercp(i, 0:3) of erfcgenp (SOURCE/erfcgenp.f:26-46);
//   - gammq / gser / gcf / gammln (SOURCE/gammq.f; the published Numerical Recipes
//     incomplete-gamma method, EPS and FPMIN single-precision literals as there);
//   - the induced-dipole loop of forces (SOURCE/forces.f:271-366): rfield
//     (SOURCE/rfield.f:59-569), ewald1p with iflag 0 (SOURCE/ewald1p.f), iter
//     (SOURCE/iter.f:43-100) with SOR weight sor_omega, until the RMS dipole change
//     is <= toler;
//   - coulomb_polar (SOURCE/coulomb_polar.f:47-84) and the final ewald1p (iflag 1)
//     with its HEAT_CURRENT per-atom stress/energy (SOURCE/ewald1p.f:575-698) and
//     the DMS potentials vesp_k, vesp_dc_k, vesp_s;
//   - ewald2p over the Verlet pairs (SOURCE/ewald2p.f:120-590), ewald3p over the
//     excluded intramolecular pairs (SOURCE/ewald3p.f:63-350), qdforce
//     (SOURCE/qdforce.f90:13-565) with vesp = sum of the seven potentials
//     (SOURCE/forces.f:829-833);
//   - the heat-current bookkeeping: update_forces entries of ewald2p/ewald3p/qdforce,
//     the M-site row redistribution (distribute_forces / _stress / _energy,
//     SOURCE/heatcurrent.f90:302-559, called from SOURCE/dlpoly_cmd.f:2585-2606) and
//     compute_heat_flux2's contraction (SOURCE/heatcurrent.f90:703-728), either
//     literally on a dense N x N force matrix or entry by entry.
//
// Layout: standard MB-pol water, 4*nw sites: water w has O, H1, H2 at 3w, 3w+1, 3w+2
// and its M site at 3nw + w (0-based).  Pair sets: the Verlet pairs are all site
// pairs of different waters within rcut; the excluded pairs (lexatm) are the six
// intramolecular pairs of each water (FIELD exclusions O-H1, O-H2, H1-H2 plus
// exclude_ttm's M-site pairs).  lexatm2 (intramolecular pairs that FIELD does not
// exclude) is empty for water, so ewald4p and rfield's lexatm2 branch add nothing.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

extern "C" void orc_image_vectors(int imcon, const double* cell, int n, double* dx);   // mbpol_oracle.cpp

namespace {

const double kR4pie0 = 138935.4835, kSqrpi = 1.7724538509055159, kPi = 3.141592653589793;

double erfcc(double x) {
    const double z = std::fabs(x);
    const double t = 1.0 / (1.0 + 0.5 * z);
    const double p = (double)1.00002368f +
                     t * ((double)0.37409196f +
                          t * ((double)0.09678418f +
                               t * (-(double)0.18628806f +
                                    t * ((double)0.27886807f +
                                         t * (-(double)1.13520398f +
                                              t * ((double)1.48851587f +
                                                   t * (-(double)0.82215223f + t * (double)0.17087277f)))))));
    double e = -(z * z) - (double)1.26551223f;
    e = e + t * p;
    double r = t * std::exp(e);
    if (x < 0.0) r = 2.0 - r;
    return r;
}

double gammln(double xx) {
    static const double cof[6] = {76.18009172947146, -86.50532032941677, 24.01409824083091,
                                  -1.231739572450155, .1208650973866179e-2, -.5395239384953e-5};
    const double stp = 2.5066282746310005;
    double x = xx, y = x;
    double tmp = x + 5.5;
    tmp = (x + 0.5) * std::log(tmp) - tmp;
    double ser = 1.000000000190015;
    for (int j = 0; j < 6; ++j) {
        y = y + 1.0;
        ser = ser + cof[j] / y;
    }
    return tmp + std::log(stp * ser / x);
}

double gammq(double a, double x) {
    const double eps = (double)3.e-7f, fpmin = (double)1.e-30f;
    if (x < a + 1.0) {   // gser
        const double gln = gammln(a);
        if (x <= 0.0) return 1.0;
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 1; n <= 800; ++n) {
            ap = ap + 1.0;
            del = del * x / ap;
            sum = sum + del;
            if (std::fabs(del) < std::fabs(sum) * eps) break;
        }
        return 1.0 - sum * std::exp(-x + a * std::log(x) - gln);
    }
    const double gln = gammln(a);   // gcf
    double b = x + 1.0 - a, c = 1.0 / fpmin, d = 1.0 / b, h = d;
    for (int i = 1; i <= 100; ++i) {
        const double an = -i * (i - a);
        b = b + 2.0;
        d = an * d + b;
        if (std::fabs(d) < fpmin) d = fpmin;
        c = b + an / c;
        if (std::fabs(c) < fpmin) c = fpmin;
        d = 1.0 / d;
        const double del = d * c;
        h = h * del;
        if (std::fabs(del - 1.0) < eps) break;
    }
    return std::exp(-x + a * std::log(x) - gln) * h;
}

// B_0..B_3 of the real-space Ewald sum at r (analytic form of rfield/ewald3p).
void bfun_exact(double alpha, double rr, double rri, double rsqi, double bbb[4]) {
    const double a = alpha * rr;
    bbb[0] = (erfcc(a) - 1.0) * rri;
    const double exp2a = std::exp(-a * a);
    for (int m = 1; m <= 3; ++m) {
        const double fm = m;
        bbb[m] = rsqi * ((2.0 * fm - 1.0) * bbb[m - 1] + std::pow(2.0 * (alpha * alpha), fm) * exp2a / alpha / kSqrpi);
    }
}

struct Params {
    double alpha, rcut, epsq, toler, omega, athole, athole12, athole13, ascc, ascd, gamma;
    int kmax[3], maxit;
};

struct Table {
    int mxegrd = 0;
    double drewd = 0;
    std::vector<double> e;   // e[4 * i + n] = ercp(i, n), i = 0..mxegrd (row 0 unused)
    void build(double alpha, double rcut) {
        mxegrd = std::max(1000, (int)(rcut / 0.0001 + 0.5) + 4);
        drewd = rcut / double(mxegrd - 4);
        e.assign(4 * (size_t)(mxegrd + 1), 0.0);
        for (int i = 1; i <= mxegrd; ++i) {
            const double rrr = double(i) * drewd;
            const double rsqi = 1.0 / rrr / rrr;
            const double a = alpha * rrr;
            double* c = &e[4 * (size_t)i];
            c[0] = (erfcc(a) - 1.0) / rrr;
            const double exp2a = std::exp(-a * a);
            for (int n = 1; n <= 3; ++n) {
                const double fn = n;
                c[n] = rsqi * ((2.0 * fn - 1.0) * c[n - 1] + std::pow(2.0 * (alpha * alpha), fn) * exp2a / alpha / kSqrpi);
            }
        }
    }
    void interp(double rr, double bbb[4]) const {
        const int ll = (int)(rr / drewd);
        const double ppp = rr / drewd - double(ll);
        for (int n = 0; n <= 3; ++n) {
            const double vk = e[4 * (size_t)ll + n], vk1 = e[4 * (size_t)(ll + 1) + n], vk2 = e[4 * (size_t)(ll + 2) + n];
            const double t1 = vk + (vk1 - vk) * ppp;
            const double t2 = vk1 + (vk2 - vk1) * (ppp - 1.0);
            bbb[n] = t1 + (t2 - t1) * ppp * 0.5;
        }
    }
};

// Heat-current bookkeeping of the force-matrix entries, the ew1p per-atom stress and the
// per-atom energies, after the M-site redistribution.
struct Heat {
    int nw = 0, nsite = 0;
    double gamma = 0;
    const double *x = nullptr, *y = nullptr, *z = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr;
    bool dense = false;
    std::vector<double> fm;       // dense: fm[(a * nsite + b) * 3 + c]
    std::vector<double> s1p;      // dense: per-site ew1p stress (9)
    double jpot[3] = {0, 0, 0};   // entry-by-entry contraction

    bool on() const { return vx != nullptr; }
    // water atoms that row a is carried to, with weights
    int expand(int a, int* c, double* w) const {
        if (a < 3 * nw) {
            c[0] = a;
            w[0] = 1.0;
            return 1;
        }
        const int m = a - 3 * nw;
        c[0] = 3 * m; c[1] = 3 * m + 1; c[2] = 3 * m + 2;
        w[0] = 1.0 - gamma; w[1] = 0.5 * gamma; w[2] = 0.5 * gamma;
        return 3;
    }
    // update_forces(a, b, f)
    void entry(int a, int b, double fx, double fy, double fz) {
        if (!on()) return;
        if (dense) {
            double* p = &fm[((size_t)a * nsite + b) * 3];
            p[0] += fx; p[1] += fy; p[2] += fz;
            return;
        }
        if (b >= 3 * nw) return;   // M columns are never read by compute_heat_flux2
        int c[3];
        double w[3];
        const int n = expand(a, c, w);
        for (int k = 0; k < n; ++k) {
            if (c[k] == b) continue;
            const double fv = w[k] * (fx * vx[c[k]] + fy * vy[c[k]] + fz * vz[c[k]]);
            jpot[0] += (x[c[k]] - x[b]) * fv;
            jpot[1] += (y[c[k]] - y[b]) * fv;
            jpot[2] += (z[c[k]] - z[b]) * fv;
        }
    }
    // update_stress_ew1p(a, :, :, -strs) for one k vector
    void stress1p(int a, const double strs[9]) {
        if (!on()) return;
        if (dense) {
            for (int q = 0; q < 9; ++q) s1p[9 * (size_t)a + q] -= strs[q];
            return;
        }
        int c[3];
        double w[3];
        const int n = expand(a, c, w);
        for (int k = 0; k < n; ++k) {
            const double v[3] = {vx[c[k]], vy[c[k]], vz[c[k]]};
            // jpot -= S . v with S's upper triangle; S = -strs
            jpot[0] += w[k] * (strs[0] * v[0] + strs[1] * v[1] + strs[2] * v[2]);
            jpot[1] += w[k] * (strs[1] * v[0] + strs[4] * v[1] + strs[5] * v[2]);
            jpot[2] += w[k] * (strs[2] * v[0] + strs[5] * v[1] + strs[8] * v[2]);
        }
    }
    void finish(double* jpot_out) {
        if (!on()) return;
        if (!dense) {
            for (int k = 0; k < 3; ++k) jpot_out[k] += jpot[k];
            return;
        }
        // distribute_forces / distribute_stress, then compute_heat_flux2 over water atoms
        for (int m = 0; m < nw; ++m) {
            const int mt = 3 * nw + m;
            int c[3];
            double w[3];
            expand(mt, c, w);
            for (int b = 0; b < nsite; ++b)
                for (int k = 0; k < 3; ++k) {
                    const double* src = &fm[((size_t)mt * nsite + b) * 3];
                    double* dst = &fm[((size_t)c[k] * nsite + b) * 3];
                    for (int q = 0; q < 3; ++q) dst[q] += w[k] * src[q];
                }
            for (int b = 0; b < nsite; ++b)
                for (int q = 0; q < 3; ++q) fm[((size_t)mt * nsite + b) * 3 + q] = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int q = 0; q < 9; ++q) s1p[9 * (size_t)c[k] + q] += w[k] * s1p[9 * (size_t)mt + q];
            for (int q = 0; q < 9; ++q) s1p[9 * (size_t)mt + q] = 0.0;
        }
        double jp[3] = {0, 0, 0};
        for (int i = 0; i < 3 * nw; ++i) {
            const double v[3] = {vx[i], vy[i], vz[i]};
            for (int j = 0; j < 3 * nw; ++j) {
                if (i == j) continue;
                const double* f = &fm[((size_t)i * nsite + j) * 3];
                const double fv = f[0] * v[0] + f[1] * v[1] + f[2] * v[2];
                jp[0] += (x[i] - x[j]) * fv;
                jp[1] += (y[i] - y[j]) * fv;
                jp[2] += (z[i] - z[j]) * fv;
            }
            const double* s = &s1p[9 * (size_t)i];
            jp[0] -= s[0] * v[0] + s[1] * v[1] + s[2] * v[2];
            jp[1] -= s[1] * v[0] + s[4] * v[1] + s[5] * v[2];
            jp[2] -= s[2] * v[0] + s[5] * v[1] + s[8] * v[2];
        }
        for (int k = 0; k < 3; ++k) jpot_out[k] += jp[k];
    }
};

struct Sys {
    int imcon, nw, n;
    const double* cell;
    const double *x, *y, *z, *q, *polr, *polr2;
    int mol(int i) const { return i < 3 * nw ? i / 3 : i - 3 * nw; }
    void sep(int i, int j, double d[3]) const {
        d[0] = x[i] - x[j];
        d[1] = y[i] - y[j];
        d[2] = z[i] - z[j];
        orc_image_vectors(imcon, cell, 1, d);
    }
};

struct PairL {
    int i, j;
};

// Thole exp-4 smearing of the dipole tensor: dum1, dum2 (rfield/ewald2p, nthole = 4)
inline void thole4(double a, double rr, double bb, double& dum1, double& dum2) {
    const double arob4 = a * std::pow(rr / bb, 4);
    dum1 = std::exp(-arob4);
    dum2 = (1.0 + (4.0 / 3.0) * arob4) * dum1;
}

struct KVec {
    int l, m, n;
    double kx, ky, kz, rksq;
};

}  // namespace

/*
 * prm[15] = {alpha, rcut, epsq, toler (e*Angstrom), sor_omega, athole, athole12, athole13,
 *            ascc, ascd, gamma, kmax1, kmax2, kmax3, maxit}
 * out[16] = {engcpe, vircpe, stress[9], iterations, deltadip, eng_polar, eng_kspace, jkin_u}
 *           (engcpe includes every electrostatic term; eng_polar is coulomb_polar's part,
 *           eng_kspace the final ewald1p energy; jkin_u = sum over water atoms of the
 *           redistributed electrostatic per-atom energy times the velocity, 3 values
 *           replacing nothing: it is returned in jkin[3])
 * fx.. ACCUMULATED site forces (M sites not redistributed); atomic_energy (per site,
 * not redistributed) ACCUMULATED, may be NULL; jpot/jkin ACCUMULATED, need v* != NULL.
 * dip* in: starting dipoles; out: converged dipoles.
 * Returns 0, or 1 when the dipoles did not converge within maxit iterations.
 */
static int polar_run(const double* prm, int imcon, const double* cell, int nw, const double* x, const double* y,
                     const double* z, const double* chge, const double* dp, const double* polr,
                     const double* polr2, double* dipx, double* dipy, double* dipz, double* fx, double* fy,
                     double* fz, double* out, double* atomic_energy, const double* vx, const double* vy,
                     const double* vz, double* jpot, double* jkin, int dense, double* resid) {
    Params P;
    P.alpha = prm[0]; P.rcut = prm[1]; P.epsq = prm[2]; P.toler = prm[3]; P.omega = prm[4];
    P.athole = prm[5]; P.athole12 = prm[6]; P.athole13 = prm[7]; P.ascc = prm[8]; P.ascd = prm[9];
    P.gamma = prm[10];
    P.kmax[0] = (int)prm[11]; P.kmax[1] = (int)prm[12]; P.kmax[2] = (int)prm[13]; P.maxit = (int)prm[14];
    const int N = 4 * nw;
    Sys S{imcon, nw, N, cell, x, y, z, chge, polr, polr2};
    const double r4 = kR4pie0, eps = P.epsq, eps2 = 2.0 * P.epsq;
    (void)eps2;
    Table T;
    T.build(P.alpha, P.rcut);

    // ---- pair sets
    std::vector<PairL> pairs;
    std::vector<double> pd;   // imaged separations (3 per pair)
    for (int i = 0; i < N; ++i)
        for (int j = i + 1; j < N; ++j) {
            if (S.mol(i) == S.mol(j)) continue;
            double d[3];
            S.sep(i, j, d);
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(P.rcut * P.rcut > r2) && !(P.rcut > std::sqrt(r2))) continue;
            pairs.push_back({i, j});
            pd.insert(pd.end(), d, d + 3);
        }
    std::vector<PairL> excl;
    std::vector<double> ed;
    for (int w = 0; w < nw; ++w) {
        const int o = 3 * w, h1 = o + 1, h2 = o + 2, m = 3 * nw + w;
        const int pr[6][2] = {{o, h1}, {o, h2}, {h1, h2}, {o, m}, {h1, m}, {h2, m}};
        for (auto& p : pr) {
            double d[3];
            S.sep(p[0], p[1], d);
            excl.push_back({p[0], p[1]});
            ed.insert(ed.end(), d, d + 3);
        }
    }

    // ---- k vectors (ewald1p's loop order and rcpcut)
    double rc[9];
    {
        const double* a = cell;
        double b[9];
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
        const double r = std::fabs(d) > 0.0 ? 1.0 / d : 0.0;
        for (int k = 0; k < 9; ++k) rc[k] = r * b[k];
    }
    auto dcell = [](const double* aa, double* bb) {
        bb[0] = std::sqrt(aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2]);
        bb[1] = std::sqrt(aa[3] * aa[3] + aa[4] * aa[4] + aa[5] * aa[5]);
        bb[2] = std::sqrt(aa[6] * aa[6] + aa[7] * aa[7] + aa[8] * aa[8]);
        const double axb1 = aa[1] * aa[5] - aa[2] * aa[4], axb2 = aa[2] * aa[3] - aa[0] * aa[5],
                     axb3 = aa[0] * aa[4] - aa[1] * aa[3];
        const double bxc1 = aa[4] * aa[8] - aa[5] * aa[7], bxc2 = aa[5] * aa[6] - aa[3] * aa[8],
                     bxc3 = aa[3] * aa[7] - aa[4] * aa[6];
        const double cxa1 = aa[7] * aa[2] - aa[1] * aa[8], cxa2 = aa[0] * aa[8] - aa[2] * aa[6],
                     cxa3 = aa[1] * aa[6] - aa[0] * aa[7];
        bb[9] = std::fabs(aa[0] * bxc1 + aa[1] * bxc2 + aa[2] * bxc3);
        bb[6] = bb[9] / std::sqrt(bxc1 * bxc1 + bxc2 * bxc2 + bxc3 * bxc3);
        bb[7] = bb[9] / std::sqrt(cxa1 * cxa1 + cxa2 * cxa2 + cxa3 * cxa3);
        bb[8] = bb[9] / std::sqrt(axb1 * axb1 + axb2 * axb2 + axb3 * axb3);
    };
    double cd[10], rd[10];
    dcell(cell, cd);
    dcell(rc, rd);
    const double volm = cd[9];
    const double twopi = 2.0 * kPi;
    const double rvolm = twopi / volm, ralph = -0.25 / (P.alpha * P.alpha);
    double rcpcut = std::min(std::min(double(P.kmax[0]) * rd[6], double(P.kmax[1]) * rd[7]), double(P.kmax[2]) * rd[8]);
    rcpcut = rcpcut * 1.05 * twopi;
    const double rcpct2 = rcpcut * rcpcut;
    std::vector<KVec> kv;
    {
        int mmin = 0, nmin = 1;
        for (int ll = 0; ll <= P.kmax[0]; ++ll) {
            const double t0 = twopi * double(ll);
            const double rkx1 = t0 * rc[0], rky1 = t0 * rc[3], rkz1 = t0 * rc[6];
            for (int mm = mmin; mm <= P.kmax[1]; ++mm) {
                const double t1 = twopi * double(mm);
                const double rkx2 = rkx1 + t1 * rc[1], rky2 = rky1 + t1 * rc[4], rkz2 = rkz1 + t1 * rc[7];
                for (int nn = nmin; nn <= P.kmax[2]; ++nn) {
                    const double t2 = twopi * double(nn);
                    const double rkx3 = rkx2 + t2 * rc[2], rky3 = rky2 + t2 * rc[5], rkz3 = rkz2 + t2 * rc[8];
                    const double rksq = rkx3 * rkx3 + rky3 * rky3 + rkz3 * rkz3;
                    if (rksq <= rcpct2) kv.push_back({ll, mm, nn, rkx3, rky3, rkz3, rksq});
                }
                nmin = -P.kmax[2];
            }
            mmin = -P.kmax[1];
        }
    }
    // exp(ikr) per k vector and site by ewald1p's recurrences
    const int K = (int)kv.size();
    std::vector<double> ckr((size_t)K * N), skr((size_t)K * N);
    {
        const int km = std::max(P.kmax[0], std::max(P.kmax[1], P.kmax[2]));
        std::vector<double> ec(km + 1), es(km + 1), mc(km + 1), ms(km + 1), nc(km + 1), ns(km + 1);
        for (int j = 0; j < N; ++j) {
            const double ssx = rc[0] * x[j] + rc[3] * y[j] + rc[6] * z[j];
            const double ssy = rc[1] * x[j] + rc[4] * y[j] + rc[7] * z[j];
            const double ssz = rc[2] * x[j] + rc[5] * y[j] + rc[8] * z[j];
            ec[0] = mc[0] = nc[0] = 1.0;
            es[0] = ms[0] = ns[0] = 0.0;
            ec[1] = std::cos(twopi * ssx); es[1] = std::sin(twopi * ssx);
            mc[1] = std::cos(twopi * ssy); ms[1] = std::sin(twopi * ssy);
            nc[1] = std::cos(twopi * ssz); ns[1] = std::sin(twopi * ssz);
            for (int l = 2; l <= P.kmax[1]; ++l) {
                mc[l] = mc[l - 1] * mc[1] - ms[l - 1] * ms[1];
                ms[l] = ms[l - 1] * mc[1] + mc[l - 1] * ms[1];
            }
            for (int l = 2; l <= P.kmax[2]; ++l) {
                nc[l] = nc[l - 1] * nc[1] - ns[l - 1] * ns[1];
                ns[l] = ns[l - 1] * nc[1] + nc[l - 1] * ns[1];
            }
            // elc(i,0) for L = ll by the running recurrence
            double lc = 1.0, ls = 0.0;
            int lcur = 0;
            for (int k = 0; k < K; ++k) {
                const KVec& v = kv[k];
                while (lcur < v.l) {
                    ++lcur;
                    if (lcur == 1) {
                        lc = ec[1];
                        ls = es[1];
                    } else {
                        const double cs = lc;
                        lc = cs * ec[1] - ls * es[1];
                        ls = ls * ec[1] + cs * es[1];
                    }
                }
                const int m = std::abs(v.m), n = std::abs(v.n);
                double clm, slm;
                if (v.m >= 0) {
                    clm = lc * mc[m] - ls * ms[m];
                    slm = ls * mc[m] + ms[m] * lc;
                } else {
                    clm = lc * mc[m] + ls * ms[m];
                    slm = ls * mc[m] - ms[m] * lc;
                }
                if (v.n >= 0) {
                    ckr[(size_t)k * N + j] = clm * nc[n] - slm * ns[n];
                    skr[(size_t)k * N + j] = slm * nc[n] + clm * ns[n];
                } else {
                    ckr[(size_t)k * N + j] = clm * nc[n] + slm * ns[n];
                    skr[(size_t)k * N + j] = slm * nc[n] - clm * ns[n];
                }
            }
        }
    }
    const double scale = 4.0 * rvolm * r4 / eps;

    std::vector<double> efk(3 * (size_t)N, 0.0), efc(3 * (size_t)N, 0.0), emu(3 * (size_t)N), efm(3 * (size_t)N);
    auto bb_of = [&](int i, int j) { return std::pow(polr[i] * polr[j], 1.0 / 6.0); };

    int iloop = 1, iflag = 0;
    double deltadip = 0.0;
    int status = 0;
    for (;;) {
        std::fill(efm.begin(), efm.end(), 0.0);
        std::fill(emu.begin(), emu.end(), 0.0);
        // ---- rfield: Verlet pairs
        for (size_t p = 0; p < pairs.size(); ++p) {
            const int i = pairs[p].i, j = pairs[p].j;
            const double* d = &pd[3 * p];
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const double rr = std::sqrt(r2);
            if (!(P.rcut > rr)) continue;
            double bbb[4];
            T.interp(rr, bbb);
            const double rsqi = 1.0 / r2, r3i = 1.0 / (rr * rr * rr), r5i = r3i * rsqi;
            if (iloop == 1) {
                double eki = r4 * chge[j] * (bbb[1] + r3i);
                double ekj = r4 * chge[i] * (bbb[1] + r3i);
                const double bb = bb_of(i, j);
                const double dum1 = std::exp(-(P.ascd * std::pow(rr / bb, 4)));
                eki = eki - r4 * chge[j] * dum1 * r3i;
                ekj = ekj - r4 * chge[i] * dum1 * r3i;
                for (int c = 0; c < 3; ++c) {
                    efk[3 * i + c] += eki * d[c];
                    efk[3 * j + c] -= ekj * d[c];
                }
            }
            if (polr2[i] > 1e-6 && polr2[j] > 1e-6) {
                double t[6];
                const int ab[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
                for (int q = 0; q < 6; ++q) {
                    const double rirj = d[ab[q][0]] * d[ab[q][1]];
                    const bool diag = ab[q][0] == ab[q][1];
                    t[q] = diag ? r4 * ((3.0 * rirj * r5i - r3i) + rirj * bbb[2] - bbb[1])
                                : r4 * ((3.0 * rirj * r5i) + rirj * bbb[2]);
                }
                double dum1, dum2;
                thole4(P.athole, rr, bb_of(i, j), dum1, dum2);
                for (int q = 0; q < 6; ++q) {
                    const double rirj = d[ab[q][0]] * d[ab[q][1]];
                    const bool diag = ab[q][0] == ab[q][1];
                    t[q] = diag ? t[q] - (3.0 * rirj * r5i * dum2 - dum1 * r3i) * r4 : t[q] - 3.0 * rirj * r5i * dum2 * r4;
                }
                const double mi[3] = {dipx[i], dipy[i], dipz[i]}, mj[3] = {dipx[j], dipy[j], dipz[j]};
                emu[3 * i + 0] += t[0] * mj[0] + t[1] * mj[1] + t[2] * mj[2];
                emu[3 * i + 1] += t[1] * mj[0] + t[3] * mj[1] + t[4] * mj[2];
                emu[3 * i + 2] += t[2] * mj[0] + t[4] * mj[1] + t[5] * mj[2];
                emu[3 * j + 0] += t[0] * mi[0] + t[1] * mi[1] + t[2] * mi[2];
                emu[3 * j + 1] += t[1] * mi[0] + t[3] * mi[1] + t[4] * mi[2];
                emu[3 * j + 2] += t[2] * mi[0] + t[4] * mi[1] + t[5] * mi[2];
            }
        }
        // ---- rfield: excluded (intramolecular) pairs
        for (size_t p = 0; p < excl.size(); ++p) {
            const int i = excl[p].i, j = excl[p].j;
            const double* d = &ed[3 * p];
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const double rr = std::sqrt(r2);
            const double rri = 1.0 / rr, rsqi = 1.0 / r2, rr3 = rr * r2, r3i = 1.0 / rr3, r5i = r3i * rsqi;
            double bbb[4];
            bfun_exact(P.alpha, rr, rri, rsqi, bbb);
            if (iloop == 1) {
                const double eki = r4 * chge[j] * bbb[1] / eps, ekj = r4 * chge[i] * bbb[1] / eps;
                for (int c = 0; c < 3; ++c) {
                    efk[3 * i + c] += eki * d[c];
                    efk[3 * j + c] -= ekj * d[c];
                }
            }
            if (polr2[i] > 1e-6 && polr2[j] > 1e-6) {
                double t[6];
                const int ab[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
                for (int q = 0; q < 6; ++q) {
                    const double rirj = d[ab[q][0]] * d[ab[q][1]];
                    t[q] = ab[q][0] == ab[q][1] ? rirj * bbb[2] - bbb[1] : rirj * bbb[2];
                }
                for (int q = 0; q < 6; ++q) {
                    const double rirj = d[ab[q][0]] * d[ab[q][1]];
                    t[q] = ab[q][0] == ab[q][1] ? t[q] + 3.0 * rirj * r5i - r3i : t[q] + 3.0 * rirj * r5i;
                }
                const double bb = bb_of(i, j);
                const double ath = (i % 3 == 0 || j % 3 == 0) ? P.athole12 : P.athole13;
                double dum1, dum2;
                thole4(ath, rr, bb, dum1, dum2);
                for (int q = 0; q < 6; ++q) {
                    const double rirj = d[ab[q][0]] * d[ab[q][1]];
                    t[q] = ab[q][0] == ab[q][1] ? t[q] - 3.0 * rirj * r5i * dum2 + dum1 * r3i
                                                : t[q] - 3.0 * rirj * r5i * dum2;
                }
                double mi[3] = {dipx[i], dipy[i], dipz[i]}, mj[3] = {dipx[j], dipy[j], dipz[j]};
                for (int c = 0; c < 3; ++c) {
                    mi[c] = mi[c] * r4 / eps;
                    mj[c] = mj[c] * r4 / eps;
                }
                emu[3 * i + 0] += t[0] * mj[0] + t[1] * mj[1] + t[2] * mj[2];
                emu[3 * i + 1] += t[1] * mj[0] + t[3] * mj[1] + t[4] * mj[2];
                emu[3 * i + 2] += t[2] * mj[0] + t[4] * mj[1] + t[5] * mj[2];
                emu[3 * j + 0] += t[0] * mi[0] + t[1] * mi[1] + t[2] * mi[2];
                emu[3 * j + 1] += t[1] * mi[0] + t[3] * mi[1] + t[4] * mi[2];
                emu[3 * j + 2] += t[2] * mi[0] + t[4] * mi[1] + t[5] * mi[2];
            }
        }
        // ---- ewald1p, iflag 0: static k field (first pass) and dipole k field
        for (int k = 0; k < K; ++k) {
            const KVec& v = kv[k];
            const double* c = &ckr[(size_t)k * N];
            const double* s = &skr[(size_t)k * N];
            double ckcs = 0, ckss = 0, mc[3] = {0, 0, 0}, ms[3] = {0, 0, 0};
            for (int j = 0; j < N; ++j) {
                if (polr2[j] > 1e-6) {
                    mc[0] += c[j] * dipx[j]; mc[1] += c[j] * dipy[j]; mc[2] += c[j] * dipz[j];
                    ms[0] += s[j] * dipx[j]; ms[1] += s[j] * dipy[j]; ms[2] += s[j] * dipz[j];
                }
            }
            for (int j = 0; j < N; ++j) {
                ckcs += chge[j] * c[j];
                ckss += chge[j] * s[j];
            }
            const double skc = v.kx * mc[0] + v.ky * mc[1] + v.kz * mc[2];
            const double sks = v.kx * ms[0] + v.ky * ms[1] + v.kz * ms[2];
            const double akk = std::exp(ralph * v.rksq) * (1.0 / v.rksq);
            for (int j = 0; j < N; ++j) {
                if (iloop == 1) {
                    const double tt = -s[j] * ckcs + c[j] * ckss;
                    efc[3 * j + 0] -= v.kx * akk * tt;
                    efc[3 * j + 1] -= v.ky * akk * tt;
                    efc[3 * j + 2] -= v.kz * akk * tt;
                }
                if (polr2[j] > 1e-6) {
                    const double vv = s[j] * sks + c[j] * skc;
                    efm[3 * j + 0] -= v.kx * akk * vv;
                    efm[3 * j + 1] -= v.ky * akk * vv;
                    efm[3 * j + 2] -= v.kz * akk * vv;
                }
            }
        }
        {
            const double dum = 4.0 * r4 * std::pow(P.alpha, 3) / kSqrpi / 3.0;
            for (int j = 0; j < N; ++j) {
                if (iloop == 1)
                    for (int c = 0; c < 3; ++c) efc[3 * j + c] = scale * efc[3 * j + c];
                for (int c = 0; c < 3; ++c) efm[3 * j + c] = scale * efm[3 * j + c];
                efm[3 * j + 0] += dum * dipx[j];
                efm[3 * j + 1] += dum * dipy[j];
                efm[3 * j + 2] += dum * dipz[j];
            }
        }
        // ---- induced_error (SOURCE/induced_error.f90:3-66): the residual of the dipole
        // equations, mu - polr2 E(mu) / r4pie0 over the polarizable sites, with the fields of
        // this pass (those of the dipoles entering it); L2 norm and largest component
        {
            double l2 = 0.0, linf = 0.0;
            for (int i = 0; i < N; ++i) {
                if (polr2[i] <= 1e-6) continue;
                const double mu[3] = {dipx[i], dipy[i], dipz[i]};
                for (int c = 0; c < 3; ++c) {
                    const double dm = mu[c] - polr2[i] * (efk[3 * i + c] + emu[3 * i + c] + efm[3 * i + c] +
                                                          efc[3 * i + c] + 0.0) / r4;
                    l2 += dm * dm;
                    linf = std::max(linf, std::fabs(dm));
                }
            }
            if (resid) {
                resid[0] = std::sqrt(l2);
                resid[1] = linf;
            }
        }
        // ---- iter
        {
            const double oldfac = P.omega, fac = 1.0 - oldfac;
            double dd = 0.0;
            int ndip = 0;
            for (int i = 0; i < N; ++i) {
                if (!(polr2[i] > P.toler)) continue;
                ++ndip;
                const double o[3] = {dipx[i], dipy[i], dipz[i]};
                double* dv[3] = {&dipx[i], &dipy[i], &dipz[i]};
                for (int c = 0; c < 3; ++c)
                    *dv[c] = oldfac * o[c] + fac * polr2[i] *
                                                 (efk[3 * i + c] + emu[3 * i + c] + efm[3 * i + c] + efc[3 * i + c] + 0.0) / r4;
                dd = dd + ((dipx[i] - o[0]) * (dipx[i] - o[0]) + (dipy[i] - o[1]) * (dipy[i] - o[1]) +
                           (dipz[i] - o[2]) * (dipz[i] - o[2]));
            }
            if (ndip == 0) ndip = 1;
            deltadip = std::sqrt(dd / double(ndip));
            if (deltadip <= P.toler) iflag = 1;
        }
        ++iloop;
        if (iflag) break;
        if (iloop > P.maxit) {
            status = 1;
            break;
        }
    }

    Heat H;
    H.nw = nw; H.nsite = N; H.gamma = P.gamma;
    H.x = x; H.y = y; H.z = z; H.vx = vx; H.vy = vy; H.vz = vz;
    H.dense = dense != 0;
    if (H.on() && H.dense) {
        H.fm.assign((size_t)N * N * 3, 0.0);
        H.s1p.assign(9 * (size_t)N, 0.0);
    }
    std::vector<double> ae(N, 0.0);
    std::vector<double> f(3 * (size_t)N, 0.0);
    double stress[9] = {0};

    // ---- coulomb_polar
    double engpol = 0.0;
    for (int i = 0; i < N; ++i) {
        if (!(polr2[i] > 1e-6)) continue;
        const double e = -(dipx[i] * (efk[3 * i] + efc[3 * i] + 0.5 * (emu[3 * i] + efm[3 * i]) + 0.0) +
                           dipy[i] * (efk[3 * i + 1] + efc[3 * i + 1] + 0.5 * (emu[3 * i + 1] + efm[3 * i + 1]) + 0.0) +
                           dipz[i] * (efk[3 * i + 2] + efc[3 * i + 2] + 0.5 * (emu[3 * i + 2] + efm[3 * i + 2]) + 0.0));
        engpol += e;
        ae[i] += e;
        const double edum = dipx[i] * dipx[i] + dipy[i] * dipy[i] + dipz[i] * dipz[i];
        engpol += r4 * edum / polr2[i] / 2.0;
        ae[i] += r4 * edum / polr2[i] / 2.0;
    }

    // ---- ewald1p, iflag 1
    std::vector<double> vesp(N, 0.0), vk(N, 0.0), vdk(N, 0.0);
    double engk = 0.0, vir = 0.0;
    {
        double engsic = 0.0;
        for (int i = 0; i < N; ++i) engsic = engsic + chge[i] * chge[i];
        engsic = -r4 / eps * P.alpha * engsic / kSqrpi;
        for (int i = 0; i < N; ++i) ae[i] += -r4 / eps * P.alpha * chge[i] * chge[i] / kSqrpi;
        double omg[9] = {0}, engc = 0.0, engdum = 0.0;
        std::vector<double> fk(3 * (size_t)N, 0.0);
        const double scalefactor = 2.0 * rvolm * r4 / eps;
        for (int k = 0; k < K; ++k) {
            const KVec& v = kv[k];
            const double* c = &ckr[(size_t)k * N];
            const double* s = &skr[(size_t)k * N];
            double ckcs = 0, ckss = 0, mc[3] = {0, 0, 0}, ms[3] = {0, 0, 0};
            for (int j = 0; j < N; ++j)
                if (polr2[j] > 1e-6) {
                    mc[0] += c[j] * dipx[j]; mc[1] += c[j] * dipy[j]; mc[2] += c[j] * dipz[j];
                    ms[0] += s[j] * dipx[j]; ms[1] += s[j] * dipy[j]; ms[2] += s[j] * dipz[j];
                }
            for (int j = 0; j < N; ++j) {
                ckcs += chge[j] * c[j];
                ckss += chge[j] * s[j];
            }
            const double skc = v.kx * mc[0] + v.ky * mc[1] + v.kz * mc[2];
            const double sks = v.kx * ms[0] + v.ky * ms[1] + v.kz * ms[2];
            const double summu1 = ckcs - sks, summu2 = ckss + skc;
            const double rrksq = 1.0 / v.rksq;
            const double akk = std::exp(ralph * v.rksq) * rrksq;
            const double akv = 2.0 * akk * (rrksq - ralph);
            const double akv2 = 2.0 * (rrksq - ralph);
            if (H.on() || atomic_energy) {
                const double kvec[3] = {v.kx, v.ky, v.kz};
                double B[9];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) B[3 * a + b] = (a == b ? 1.0 : 0.0) - akv2 * kvec[a] * kvec[b];
                for (int j = 0; j < N; ++j) {
                    const double dv[3] = {dipx[j], dipy[j], dipz[j]};
                    const double Cqi = chge[j] * c[j], Sqi = chge[j] * s[j];
                    const double CMi[3] = {dv[0] * c[j], dv[1] * c[j], dv[2] * c[j]};
                    const double SMi[3] = {dv[0] * s[j], dv[1] * s[j], dv[2] * s[j]};
                    const double dpkCMi = kvec[0] * CMi[0] + kvec[1] * CMi[1] + kvec[2] * CMi[2];
                    const double dpkSMi = kvec[0] * SMi[0] + kvec[1] * SMi[1] + kvec[2] * SMi[2];
                    const double dpkMc = kvec[0] * mc[0] + kvec[1] * mc[1] + kvec[2] * mc[2];
                    const double dpkMs = kvec[0] * ms[0] + kvec[1] * ms[1] + kvec[2] * ms[2];
                    double strs[9];
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) {
                            const int p = 3 * a + b;
                            const double cc = B[p] * (Cqi * ckcs + Sqi * ckss);
                            const double cdd = B[p] * (Sqi * dpkMc - Cqi * dpkMs - dpkSMi * ckcs + dpkCMi * ckss) +
                                               (Sqi * kvec[a] * mc[b] - Cqi * kvec[a] * ms[b] - kvec[a] * SMi[b] * ckcs +
                                                kvec[a] * CMi[b] * ckss);
                            const double ddd = B[p] * (dpkCMi * dpkMc + dpkSMi * dpkMs) +
                                               (kvec[a] * CMi[b] * dpkMc + kvec[a] * SMi[b] * dpkMs +
                                                dpkCMi * kvec[a] * mc[b] + dpkSMi * kvec[a] * ms[b]);
                            strs[p] = cc * scalefactor * akk + cdd * scalefactor * akk + ddd * scalefactor * akk;
                        }
                    H.stress1p(j, strs);
                    ae[j] += scalefactor * akk * (Cqi * ckcs + Sqi * ckss);
                }
            }
            engc = engc + akk * (ckcs * ckcs + ckss * ckss);
            engdum = engdum + akk * (summu1 * summu1 + summu2 * summu2);
            const double virprs = akv * (summu1 * summu1 + summu2 * summu2);
            const double k3[3] = {v.kx, v.ky, v.kz};
            const int oi[6] = {0, 4, 8, 1, 2, 5};
            const int oa[6] = {0, 1, 2, 0, 0, 1}, ob[6] = {0, 1, 2, 1, 2, 2};
            for (int q = 0; q < 6; ++q)
                omg[oi[q]] = omg[oi[q]] - virprs * k3[oa[q]] * k3[ob[q]] - 2.0 * akk * k3[oa[q]] * ms[ob[q]] * summu1 +
                             2.0 * akk * k3[oa[q]] * mc[ob[q]] * summu2;
            for (int j = 0; j < N; ++j) {
                double djmuk = 0.0;
                if (polr2[j] > 1e-6) djmuk = dipx[j] * v.kx + dipy[j] * v.ky + dipz[j] * v.kz;
                const double ssmu = summu1 * (-s[j] * chge[j] - c[j] * djmuk) + summu2 * (-s[j] * djmuk + c[j] * chge[j]);
                fk[3 * j + 0] -= v.kx * akk * ssmu;
                fk[3 * j + 1] -= v.ky * akk * ssmu;
                fk[3 * j + 2] -= v.kz * akk * ssmu;
                vk[j] += akk * (c[j] * ckcs + s[j] * ckss);
                vdk[j] += akk * (s[j] * skc - c[j] * sks);
            }
        }
        const double eng1 = engdum;
        engk = 2.0 * rvolm * r4 * engc / eps + engsic;
        const double scal1 = 2.0 * rvolm * r4 / eps;
        for (int j = 0; j < N; ++j) {
            for (int c = 0; c < 3; ++c) f[3 * j + c] += scale * fk[3 * j + c];
            vesp[j] += scale * vk[j] + scale * vdk[j] - 2.0 * r4 * chge[j] * P.alpha / kSqrpi / eps;
        }
        stress[0] += scal1 * (omg[0] + eng1);
        stress[1] += scal1 * omg[1];
        stress[2] += scal1 * omg[2];
        stress[3] += scal1 * omg[1];
        stress[4] += scal1 * (omg[4] + eng1);
        stress[5] += scal1 * omg[5];
        stress[6] += scal1 * omg[2];
        stress[7] += scal1 * omg[5];
        stress[8] += scal1 * (omg[8] + eng1);
        vir += -scal1 * (omg[0] + omg[4] + omg[8] + 3.0 * eng1);
    }

    // ---- ewald2p over the Verlet pairs
    double eng2 = 0.0;
    const double g34 = std::exp(gammln(3.0 / 4.0));
    for (size_t p = 0; p < pairs.size(); ++p) {
        const int ia = pairs[p].i, ja = pairs[p].j;
        const double* d = &pd[3 * p];
        const double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (!(P.rcut * P.rcut > rsq)) continue;
        const double rrr = std::sqrt(rsq);
        double bbb[4];
        T.interp(rrr, bbb);
        const double rri = 1.0 / rrr, rsqi = 1.0 / rsq, r3i = 1.0 / (rrr * rrr * rrr), r5i = r3i * rsqi;
        const double cicj = chge[ia] * chge[ja];
        const double edum = cicj * (bbb[0] + 1.0 / rrr) * r4;
        eng2 += edum;
        ae[ia] += 0.5 * edum;
        ae[ja] += 0.5 * edum;
        double espdum = (bbb[0] + 1.0 / rrr) * r4;
        double ffac = cicj * (r3i - 0.0 * rsqi + bbb[1]) * r4;
        const double bb = bb_of(ia, ja);
        {
            const double arob4 = P.ascc * std::pow(rrr / bb, 4);
            const double dum1 = std::exp(-arob4);
            const double sm = (dum1 - std::pow(arob4, 1.0 / 4.0) * g34 * gammq(3.0 / 4.0, arob4)) / rrr * r4;
            eng2 = eng2 - cicj * sm;
            ae[ia] += -cicj * 0.5 * (dum1 - std::pow(arob4, 0.25) * g34 * gammq(0.75, arob4)) / rrr * r4;
            ae[ja] += -cicj * 0.5 * (dum1 - std::pow(arob4, 0.25) * g34 * gammq(0.75, arob4)) / rrr * r4;
            espdum = espdum - sm;
            ffac = ffac - cicj * r3i * dum1 * r4;
        }
        const double rdmui = dipx[ia] * d[0] + dipy[ia] * d[1] + dipz[ia] * d[2];
        const double rdmuj = dipx[ja] * d[0] + dipy[ja] * d[1] + dipz[ja] * d[2];
        const double facmu0 = (chge[ja] * rdmui - chge[ia] * rdmuj) * (rrr * 0.0 - 3.0 * 1.0) * r5i * r4;
        const double facmui0 = 1.0 * r3i * chge[ja] * r4;
        const double facmuj0 = -1.0 * r3i * chge[ia] * r4;
        double facmu = facmu0 - (chge[ja] * rdmui - chge[ia] * rdmuj) * bbb[2] * r4;
        double dfacmui = facmui0 + bbb[1] * chge[ja] * r4;
        double dfacmuj = facmuj0 - bbb[1] * chge[ia] * r4;
        double espdcdum = (bbb[1] + r3i) * r4;
        {
            double dum1, dum2;
            thole4(P.ascd, rrr, bb, dum1, dum2);
            facmu = facmu - facmu0 * dum2;
            dfacmui = dfacmui - facmui0 * dum1;
            dfacmuj = dfacmuj - facmuj0 * dum1;
            espdcdum = espdcdum - r3i * dum1 * r4;
        }
        if (polr2[ia] > 1e-6 && polr2[ja] > 1e-6) {
            const double dpidpj = dipx[ia] * dipx[ja] + dipy[ia] * dipy[ja] + dipz[ia] * dipz[ja];
            facmu = facmu + ((dpidpj * (3.0 * 1.0 - 0.0 / rrr) + rdmui * rdmuj * rsqi * (3.0 * 0.0 * rrr - 15.0 * 1.0)) * r5i +
                             bbb[2] * dpidpj - bbb[3] * rdmui * rdmuj) * r4;
            dfacmui = dfacmui + (1.0 * 3.0 * r5i + bbb[2]) * rdmuj * r4;
            dfacmuj = dfacmuj + (1.0 * 3.0 * r5i + bbb[2]) * rdmui * r4;
            const double facmu1 = -15.0 * rdmui * rdmuj * rsqi * r5i * r4;
            const double facmu2 = 3.0 * dpidpj * r5i * r4;
            const double dfacmui1 = 3.0 * rdmuj * r5i * r4;
            const double dfacmuj1 = 3.0 * rdmui * r5i * r4;
            const double arob4 = P.athole * std::pow(rrr / bb, 4);
            const double dum1 = std::exp(-arob4);
            const double dum2 = (1.0 + (4.0 / 3.0) * arob4) * dum1;
            const double dum3 = 4.0 * P.athole * (4.0 * arob4 - 1.0) * dum1 * rsqi / std::pow(bb, 4);
            const double dum4 = 4.0 * P.athole * dum1 * rrr / std::pow(bb, 4);
            facmu = facmu - facmu1 * dum2 - facmu2 * dum1 + rdmui * rdmuj * dum3 * rri * r4 - dpidpj * rsqi * dum4 * r4;
            dfacmui = dfacmui - dfacmui1 * dum2;
            dfacmuj = dfacmuj - dfacmuj1 * dum2;
        }
        const double dfx = dfacmui * dipx[ia] + dfacmuj * dipx[ja];
        const double dfy = dfacmui * dipy[ia] + dfacmuj * dipy[ja];
        const double dfz = dfacmui * dipz[ia] + dfacmuj * dipz[ja];
        ffac = ffac + facmu;
        const double virdum = dfx * d[0] + dfy * d[1] + dfz * d[2];
        vir = vir - ffac * rsq - virdum;
        const double fxp = ffac * d[0] + dfx, fyp = ffac * d[1] + dfy, fzp = ffac * d[2] + dfz;
        f[3 * ia] += fxp; f[3 * ia + 1] += fyp; f[3 * ia + 2] += fzp;
        f[3 * ja] -= fxp; f[3 * ja + 1] -= fyp; f[3 * ja + 2] -= fzp;
        H.entry(ja, ia, -fxp, -fyp, -fzp);
        H.entry(ia, ja, fxp, fyp, fzp);
        vesp[ia] += chge[ja] * espdum + rdmuj * espdcdum;
        vesp[ja] += chge[ia] * espdum - rdmui * espdcdum;
        stress[0] += d[0] * fxp; stress[1] += d[0] * fyp; stress[2] += d[0] * fzp;
        stress[3] += d[0] * fyp; stress[4] += d[1] * fyp; stress[5] += d[1] * fzp;
        stress[6] += d[0] * fzp; stress[7] += d[1] * fzp; stress[8] += d[2] * fzp;
    }

    // ---- ewald3p over the excluded pairs
    double eng3 = 0.0;
    for (size_t p = 0; p < excl.size(); ++p) {
        const int ia = excl[p].i, ja = excl[p].j;
        const double* d = &ed[3 * p];
        const double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const double rrr = std::sqrt(rsq);
        const double rri = 1.0 / rrr, rsqi = 1.0 / rsq, r3i = 1.0 / (rrr * rrr * rrr), r5i = r3i * rsqi;
        double bbb[4];
        bfun_exact(P.alpha, rrr, rri, rsqi, bbb);
        const double cicj = chge[ia] * chge[ja];
        eng3 = eng3 + cicj * bbb[0] * r4 / eps;
        ae[ia] += 0.5 * cicj * bbb[0] * r4 / eps;
        ae[ja] += 0.5 * cicj * bbb[0] * r4 / eps;
        const double espdum = bbb[0] * r4 / eps, espdcdum = bbb[1] * r4 / eps;
        double ffac = cicj * bbb[1] * r4 / eps;
        const double rdmui = dipx[ia] * d[0] + dipy[ia] * d[1] + dipz[ia] * d[2];
        const double rdmuj = dipx[ja] * d[0] + dipy[ja] * d[1] + dipz[ja] * d[2];
        double facmu = (chge[ja] * rdmui - chge[ia] * rdmuj) * (-bbb[2]) * r4 / eps;
        double dfacmui = bbb[1] * chge[ja] * r4 / eps;
        double dfacmuj = -bbb[1] * chge[ia] * r4 / eps;
        if (polr2[ia] > 1e-6 && polr2[ja] > 1e-6) {
            const double dpidpj = dipx[ia] * dipx[ja] + dipy[ia] * dipy[ja] + dipz[ia] * dipz[ja];
            facmu = facmu + (bbb[2] * dpidpj - bbb[3] * rdmui * rdmuj) * r4 / eps;
            dfacmui = dfacmui + bbb[2] * rdmuj * r4 / eps;
            dfacmuj = dfacmuj + bbb[2] * rdmui * r4 / eps;
            const double facmu1 = -15.0 * rdmui * rdmuj * rsqi * r5i * r4 / eps;
            const double facmu2 = 3.0 * dpidpj * r5i * r4 / eps;
            facmu = facmu + facmu1 + facmu2;
            const double dfacmuidd = 3.0 * rdmuj * r5i * r4 / eps;
            const double dfacmujdd = 3.0 * rdmui * r5i * r4 / eps;
            dfacmui = dfacmui + dfacmuidd;
            dfacmuj = dfacmuj + dfacmujdd;
            const double bb = bb_of(ia, ja);
            const double ath = (ia % 3 == 0 || ja % 3 == 0) ? P.athole12 : P.athole13;
            const double arob4 = ath * std::pow(rrr / bb, 4);
            const double dum1 = std::exp(-arob4);
            const double dum2 = (1.0 + (4.0 / 3.0) * arob4) * dum1;
            const double dum3 = 4.0 * ath * (4.0 * arob4 - 1.0) * dum1 * rsqi / std::pow(bb, 4);
            const double dum4 = 4.0 * ath * dum1 * rrr / std::pow(bb, 4);
            facmu = facmu - facmu1 * dum2 - facmu2 * dum1 + rdmui * rdmuj * dum3 * rri * r4 / eps -
                    dpidpj * rsqi * dum4 * r4 / eps;
            dfacmui = dfacmui - dfacmuidd * dum2;
            dfacmuj = dfacmuj - dfacmujdd * dum2;
        }
        const double dfx = dfacmui * dipx[ia] + dfacmuj * dipx[ja];
        const double dfy = dfacmui * dipy[ia] + dfacmuj * dipy[ja];
        const double dfz = dfacmui * dipz[ia] + dfacmuj * dipz[ja];
        ffac = ffac + facmu;
        const double fxp = ffac * d[0] + dfx, fyp = ffac * d[1] + dfy, fzp = ffac * d[2] + dfz;
        f[3 * ia] += fxp; f[3 * ia + 1] += fyp; f[3 * ia + 2] += fzp;
        f[3 * ja] -= fxp; f[3 * ja + 1] -= fyp; f[3 * ja + 2] -= fzp;
        H.entry(ia, ja, fxp, fyp, fzp);
        H.entry(ja, ia, -fxp, -fyp, -fzp);
        const double virdum = dfx * d[0] + dfy * d[1] + dfz * d[2];
        vir = vir - ffac * rsq - virdum;
        vesp[ia] += chge[ja] * espdum;
        vesp[ja] += chge[ia] * espdum;
        vesp[ia] += rdmuj * espdcdum;
        vesp[ja] -= rdmui * espdcdum;
        stress[0] += d[0] * fxp; stress[1] += d[0] * fyp; stress[2] += d[0] * fzp;
        stress[3] += d[0] * fyp; stress[4] += d[1] * fyp; stress[5] += d[1] * fzp;
        stress[6] += d[0] * fzp; stress[7] += d[1] * fzp; stress[8] += d[2] * fzp;
    }

    // ---- qdforce (new charge assignment)
    double virq = 0.0;
    {
        const double g = P.gamma;
        double sq[6] = {0, 0, 0, 0, 0, 0};   // strs1, 2, 3, 5, 6, 9
        for (int w = 0; w < nw; ++w) {
            const int io = 3 * w, h1 = io + 1, h2 = io + 2, mt = 3 * nw + w;
            const double* D = dp + 6 * (size_t)w;   // dp1dr1, dp1dr2, dp2dr1, dp2dr2, dp1dcos, dp2dcos
            const double dp1dr1 = D[0], dp1dr2 = D[1], dp2dr1 = D[2], dp2dr2 = D[3], dp1dcos = D[4], dp2dcos = D[5];
            double r1v[3], r2v[3];
            S.sep(h1, io, r1v);
            S.sep(h2, io, r2v);
            const double r1 = std::sqrt(r1v[0] * r1v[0] + r1v[1] * r1v[1] + r1v[2] * r1v[2]);
            const double r2 = std::sqrt(r2v[0] * r2v[0] + r2v[1] * r2v[1] + r2v[2] * r2v[2]);
            const double rdot = r1v[0] * r2v[0] + r1v[1] * r2v[1] + r1v[2] * r2v[2];
            const double cost = rdot / (r1 * r2);
            const double r3 = std::sqrt(r1 * r1 + r2 * r2 - 2.0 * r1 * r2 * cost);
            const double sint = std::sqrt(1.0 - cost * cost);
            const double cott = cost / sint;
            const double r1sqr = r1 * r1, r2sqr = r2 * r2;
            double dr[3][4][3];   // drint(k, site, xyz)
            std::memset(dr, 0, sizeof dr);
            for (int c = 0; c < 3; ++c) {
                dr[0][1][c] = r1v[c] / r1;
                dr[0][0][c] = -dr[0][1][c];
                dr[1][2][c] = r2v[c] / r2;
                dr[1][0][c] = -dr[1][2][c];
                dr[2][1][c] = cott * (r1v[c] / r1sqr - r2v[c] / rdot);
                dr[2][2][c] = cott * (r2v[c] / r2sqr - r1v[c] / rdot);
                dr[2][0][c] = -dr[2][1][c] - dr[2][2][c];
            }
            double dp1s[4][3], dp2s[4][3];
            for (int i = 0; i < 4; ++i)
                for (int c = 0; c < 3; ++c) {
                    dp1s[i][c] = dp1dr1 * dr[0][i][c] + dp1dr2 * dr[1][i][c] - sint * dp1dcos * dr[2][i][c];
                    dp2s[i][c] = dp2dr1 * dr[0][i][c] + dp2dr2 * dr[1][i][c] - sint * dp2dcos * dr[2][i][c];
                }
            const double tmp = g / 2.0 / (1.0 - g);
            double dqdr12[4] = {0, 0, 0, 0}, dqdr13[4] = {0, 0, 0, 0}, dqdcos[4] = {0, 0, 0, 0};
            dqdr12[1] = dp1dr1 + (dp1dr1 + dp2dr1) * tmp;
            dqdr13[1] = dp1dr2 + (dp1dr2 + dp2dr2) * tmp;
            dqdcos[1] = dp1dcos + (dp1dcos + dp2dcos) * tmp;
            dqdr12[2] = dp2dr1 + (dp1dr1 + dp2dr1) * tmp;
            dqdr13[2] = dp2dr2 + (dp1dr2 + dp2dr2) * tmp;
            dqdcos[2] = dp2dcos + (dp1dcos + dp2dcos) * tmp;
            dqdr12[3] = -(dp1dr1 + dp2dr1) / (1.0 - g);
            dqdr13[3] = -(dp1dr2 + dp2dr2) / (1.0 - g);
            dqdcos[3] = -(dp1dcos + dp2dcos) / (1.0 - g);
            const double dcosdr12 = (r1 - r2 * cost) / r1 / r2;
            const double dcosdr13 = (r2 - r1 * cost) / r1 / r2;
            const double dcosdr23 = -r3 / r1 / r2;
            double dq[4][4][3];   // dq(charge j, site, xyz)
            std::memset(dq, 0, sizeof dq);
            const double factor = g / 2.0 / (1.0 - g);
            for (int j = 0; j < 4; ++j)
                for (int c = 0; c < 3; ++c) {
                    dq[1][j][c] = dp1s[j][c] * (factor + 1.0) + dp2s[j][c] * factor;
                    dq[2][j][c] = dp2s[j][c] * (factor + 1.0) + dp1s[j][c] * factor;
                    dq[3][j][c] = -(dq[1][j][c] + dq[2][j][c]);
                }
            const int site[4] = {io, h1, h2, mt};
            for (int j = 0; j < 4; ++j) {
                const double vt = vesp[site[j]];
                const int idx = j == 3 ? nw + w : 3 * w + j;   // the reference's column (heatcurrent entries)
                for (int s2 = 0; s2 < 4; ++s2) {
                    const double fq[3] = {-dq[j][s2][0] * vt, -dq[j][s2][1] * vt, -dq[j][s2][2] * vt};
                    for (int c = 0; c < 3; ++c) f[3 * site[s2] + c] += fq[c];
                    H.entry(site[s2], idx, fq[0], fq[1], fq[2]);
                }
            }
            // pressure tensor and virial
            for (int i = 0; i < 4; ++i) {
                const double vt = vesp[site[i]];
                for (int lab = 1; lab <= 2; ++lab) {
                    const double dqdr_tmp = lab == 1 ? dqdr12[i] : dqdr13[i];
                    const int hh = lab == 1 ? h1 : h2;
                    double r[3] = {x[io] - x[hh], y[io] - y[hh], z[io] - z[hh]};
                    orc_image_vectors(imcon, cell, 1, r);
                    const double rjk = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                    sq[0] = sq[0] - vt * dqdr_tmp * r[0] * r[0] / rjk;
                    sq[1] = sq[1] - vt * dqdr_tmp * r[0] * r[1] / rjk;
                    sq[2] = sq[2] - vt * dqdr_tmp * r[0] * r[2] / rjk;
                    sq[3] = sq[3] - vt * dqdr_tmp * r[1] * r[1] / rjk;
                    sq[4] = sq[4] - vt * dqdr_tmp * r[1] * r[2] / rjk;
                    sq[5] = sq[5] - vt * dqdr_tmp * r[2] * r[2] / rjk;
                    virq = virq + vt * rjk * dqdr_tmp;
                }
                double a1[3] = {x[io] - x[h1], y[io] - y[h1], z[io] - z[h1]};
                double a2[3] = {x[io] - x[h2], y[io] - y[h2], z[io] - z[h2]};
                double a3[3] = {x[h1] - x[h2], y[h1] - y[h2], z[h1] - z[h2]};
                orc_image_vectors(imcon, cell, 1, a1);
                orc_image_vectors(imcon, cell, 1, a2);
                orc_image_vectors(imcon, cell, 1, a3);
                const double q1 = std::sqrt(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
                const double q2 = std::sqrt(a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2]);
                const double q3 = std::sqrt(a3[0] * a3[0] + a3[1] * a3[1] + a3[2] * a3[2]);
                const int ta[6] = {0, 0, 0, 1, 1, 2}, tb[6] = {0, 1, 2, 1, 2, 2};
                double dc[6];
                for (int q = 0; q < 6; ++q)
                    dc[q] = dcosdr12 * a1[ta[q]] * a1[tb[q]] / q1 + dcosdr13 * a2[ta[q]] * a2[tb[q]] / q2 +
                            dcosdr23 * a3[ta[q]] * a3[tb[q]] / q3;
                for (int q = 0; q < 6; ++q) sq[q] = sq[q] - vt * dqdcos[i] * dc[q];
                virq = virq + vt * (dc[0] + dc[3] + dc[5]) * dqdcos[i];
            }
        }
        stress[0] += sq[0]; stress[1] += sq[1]; stress[2] += sq[2];
        stress[3] += sq[1]; stress[4] += sq[3]; stress[5] += sq[4];
        stress[6] += sq[2]; stress[7] += sq[4]; stress[8] += sq[5];
        vir += virq;
    }

    for (int i = 0; i < N; ++i) {
        fx[i] += f[3 * i];
        fy[i] += f[3 * i + 1];
        fz[i] += f[3 * i + 2];
        if (atomic_energy) atomic_energy[i] += ae[i];
    }
    if (H.on()) {
        H.finish(jpot);
        // jkin's potential part: redistributed per-atom energies times velocities
        for (int i = 0; i < N; ++i) {
            int c[3];
            double w[3];
            const int n = H.expand(i, c, w);
            for (int k = 0; k < n; ++k) {
                jkin[0] += w[k] * ae[i] * vx[c[k]];
                jkin[1] += w[k] * ae[i] * vy[c[k]];
                jkin[2] += w[k] * ae[i] * vz[c[k]];
            }
        }
    }
    const double engcpe = engk + eng2 + eng3 + engpol;
    out[0] = engcpe;
    out[1] = vir;
    for (int k = 0; k < 9; ++k) out[2 + k] = stress[k];
    out[11] = iloop - 1;
    out[12] = deltadip;
    out[13] = engpol;
    out[14] = engk;
    out[15] = eng2 + eng3;
    return status;
}

// The pieces the GPU path shares with the oracle, exposed for unit tests.
extern "C" int orc_polar(const double* prm, int imcon, const double* cell, int nw, const double* x, const double* y,
                         const double* z, const double* chge, const double* dp, const double* polr,
                         const double* polr2, double* dipx, double* dipy, double* dipz, double* fx, double* fy,
                         double* fz, double* out, double* atomic_energy, const double* vx, const double* vy,
                         const double* vz, double* jpot, double* jkin, int dense) {
    return polar_run(prm, imcon, cell, nw, x, y, z, chge, dp, polr, polr2, dipx, dipy, dipz, fx, fy, fz, out,
                     atomic_energy, vx, vy, vz, jpot, jkin, dense, nullptr);
}

/*
 * induced_error (SOURCE/induced_error.f90:3-66) of given dipoles: one pass of the fields at
 * dip* (rfield and ewald1p of the polar branch) and the residual of the dipole equations,
 * resid[2] = {L2 norm, largest component} over the polarizable sites.  prm as orc_polar;
 * the dipoles are not changed.
 */
extern "C" void orc_induced_error(const double* prm, int imcon, const double* cell, int nw, const double* x,
                                  const double* y, const double* z, const double* chge, const double* dp,
                                  const double* polr, const double* polr2, const double* dipx, const double* dipy,
                                  const double* dipz, double* resid) {
    const int N = 4 * nw;
    double p1[15];
    for (int q = 0; q < 15; ++q) p1[q] = prm[q];
    p1[14] = 1;   // one pass: the fields at the given dipoles
    std::vector<double> mx(dipx, dipx + N), my(dipy, dipy + N), mz(dipz, dipz + N), f(3 * (size_t)N, 0.0);
    double out[16];
    polar_run(p1, imcon, cell, nw, x, y, z, chge, dp, polr, polr2, mx.data(), my.data(), mz.data(), f.data(),
              f.data() + N, f.data() + 2 * (size_t)N, out, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0,
              resid);
}

extern "C" double orc_erfcc(double x) { return erfcc(x); }
extern "C" double orc_gammq(double a, double x) { return gammq(a, x); }
extern "C" double orc_gammln(double x) { return gammln(x); }
