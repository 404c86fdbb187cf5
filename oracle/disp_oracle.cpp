// Oracle for the short-range dispersion term: DL_POLY van der Waals type 12
// (Tang-Toennies damped C6/r^6 + C8/r^8) as the reference tabulates and applies it.
//
// Parity unpinned: restated from the reference's Fortran, which cannot be compiled in
// this image; checked against the tabulated formula, finite differences, momentum and
// the virial sum, not against a reference run.
// TEST INFRASTRUCTURE ONLY (see oracle.h).  Restates, operation by operation:
//   - tang_toennies / tang_toennies_lr (SOURCE/tang-toennies.f90:6-74), including the
//     reference's factorial, which multiplies by its argument at every step (z^z);
//   - the type-12 tables vv12/gg12 at r = i*dlrpot, i = 1..mxgrid (SOURCE/forgen.f:97,
//     :262-270, :337-357);
//   - srfrce2 (SOURCE/srfrce2.f:80-270): 3-point interpolation of energy and force,
//     virial, stress, per-atom energy halves (update_energy_srf) and the heat-current
//     pair entries update_forces(j,i,-f), update_forces(i,j,f) contracted as
//     (r_i - r_j) (f . (v_i + v_j)) with raw coordinates;
//   - the pair set of the Verlet list: every pair of atoms of different molecules
//     (intramolecular pairs are excluded, SOURCE/exclude_ttm.f) with the separation
//     x_i - x_j imaged as SOURCE/images.f does (SOURCE/forces.f:509-523);
//   - lrcorrect for type 12 (SOURCE/lrcorrect.f:112-223, el12/pl12 :285-302).
#include <cmath>
#include <vector>

extern "C" void orc_image_vectors(int imcon, const double* cell, int n, double* dx);   // mbpol_oracle.cpp

namespace {

double tang_toennies(int n, double x) {
    double sum = 1.0;
    for (int nn = n; nn >= 1; --nn) sum = 1.0 + sum * x / nn;
    double tt = 1.0 - sum * std::exp(-x);
    if (std::fabs(tt) < 1.0e-8) {
        double term = 1.0;
        for (int nn = n; nn >= 1; --nn) term = term * x / nn;
        sum = 0.0;
        for (int nn = n + 1; nn <= 1000; ++nn) {
            term = term * x / nn;
            sum = sum + term;
            if (std::fabs(term / sum) < 1.0e-8) break;
        }
        tt = sum * std::exp(-x);
    }
    return tt;
}

double factorial_as_reference(int z) {
    double f = 1.0;
    for (int i = z; i >= 1; --i) f = f * z;
    return f;
}

double tang_toennies_lr(int n, double x) {
    double v = tang_toennies(n, x) / std::pow(x, n - 3) +
               std::exp(-x) * (x * x * (3.0 + x) + 6 * (1.0 + x)) / factorial_as_reference(n);
    return v / (n - 3);
}

// A term whose coefficient is 0 adds a signed zero in the reference; it is skipped here
// (same value; and tang_toennies(n, 0) would run its series loop to the end).
double vv12(double r, double c6, double a6, double c8, double a8) {
    double v = 0.0;
    if (c6 != 0.0) v = -c6 * tang_toennies(6, a6 * r) / std::pow(r, 6);
    if (c8 != 0.0) v = v - c8 * tang_toennies(8, a8 * r) / std::pow(r, 8);
    return v;
}

double gg12(double r, double c6, double a6, double c8, double a8) {
    double g6 = 0.0, g8 = 0.0, e6 = 0.0, e8 = 0.0;
    if (c6 != 0.0) {
        g6 = -6 * c6 * tang_toennies(6, a6 * r) / std::pow(r, 6);
        e6 = r * c6 * std::pow(a6, 7) * std::exp(-a6 * r) / 720;
    }
    if (c8 != 0.0) {
        g8 = -8 * c8 * tang_toennies(8, a8 * r) / std::pow(r, 8);
        e8 = r * c8 * std::pow(a8, 9) * std::exp(-a8 * r) / 40320;
    }
    return g6 + g8 + e6 + e8;
}

// pair-type index of 1-based atom types (SOURCE/srfrce2.f:112-118), 0-based
int pair_index(int ai, int aj) { return ai > aj ? ai * (ai - 1) / 2 + aj - 1 : aj * (aj - 1) / 2 + ai - 1; }

}  // namespace

extern "C" double orc_tang_toennies(int n, double x) { return tang_toennies(n, x); }
extern "C" double orc_tang_toennies_lr(int n, double x) { return tang_toennies_lr(n, x); }

// vvv/ggg[k * mxgrid + (i - 1)] = vv12/gg12(i * dlrpot) for every pair type k (prm: 4 per type).
extern "C" void orc_disp_tables(int npair, const double* prm, int mxgrid, double dlrpot, double* vvv, double* ggg) {
    for (int k = 0; k < npair; ++k) {
        const double* p = prm + 4 * k;
        if (p[0] == 0.0 && p[2] == 0.0) {   // no interaction: the table is all zeros
            for (int i = 0; i < mxgrid; ++i) vvv[(size_t)k * mxgrid + i] = ggg[(size_t)k * mxgrid + i] = 0.0;
            continue;
        }
        for (int i = 1; i <= mxgrid; ++i) {
            const double rrr = i * dlrpot;
            vvv[(size_t)k * mxgrid + i - 1] = vv12(rrr, p[0], p[1], p[2], p[3]);
            ggg[(size_t)k * mxgrid + i - 1] = gg12(rrr, p[0], p[1], p[2], p[3]);
        }
    }
}

// srfrce2 over every intermolecular pair within rcut.  Types are 1-based (0: no
// dispersion); prm holds 4 values per pair type in the order of pair_index.
// f*, eng, vir, stress, atomic_energy and jpot are ACCUMULATED.  Returns the pair count.
extern "C" long orc_dispersion(int imcon, const double* cell, int natms, const int* ltype, const int* mol,
                               int ntypes, const double* prm, double rcut, int mxgrid, const double* x,
                               const double* y, const double* z, double* fx, double* fy, double* fz, double* eng,
                               double* vir, double* stress, double* atomic_energy, const double* vx,
                               const double* vy, const double* vz, double* jpot) {
    const int npair = ntypes * (ntypes + 1) / 2;
    const double dlrpot = rcut / double(mxgrid - 4);
    std::vector<double> vvv((size_t)npair * mxgrid), ggg((size_t)npair * mxgrid);
    orc_disp_tables(npair, prm, mxgrid, dlrpot, vvv.data(), ggg.data());
    const double rcsq = rcut * rcut, rdr = 1.0 / dlrpot;
    double engsrp = 0.0, virsrp = 0.0, s1 = 0, s2 = 0, s3 = 0, s5 = 0, s6 = 0, s9 = 0;
    long npairs = 0;
    for (int i = 0; i < natms; ++i) {
        if (ltype[i] <= 0) continue;
        for (int j = i + 1; j < natms; ++j) {
            if (ltype[j] <= 0 || mol[i] == mol[j]) continue;
            const int k = pair_index(ltype[i], ltype[j]);
            const double* vk_ = vvv.data() + (size_t)k * mxgrid;   // vk_[l - 1] = vvv(l, k)
            const double* gk_ = ggg.data() + (size_t)k * mxgrid;
            if (!(vk_[0] != 0.0)) continue;
            double d[3] = {x[i] - x[j], y[i] - y[j], z[i] - z[j]};
            orc_image_vectors(imcon, cell, 1, d);
            const double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (!(rcsq > rsq)) continue;
            ++npairs;
            const double rrr = std::sqrt(rsq);
            const int l = int(rrr * rdr);
            const double ppp = rrr * rdr - double(l);
            const double vk = vk_[l - 1], vk1 = vk_[l], vk2 = vk_[l + 1];
            double t1 = vk + (vk1 - vk) * ppp;
            double t2 = vk1 + (vk2 - vk1) * (ppp - 1.0);
            const double e = t1 + (t2 - t1) * ppp * 0.5;
            engsrp = e + engsrp;
            if (atomic_energy) {
                atomic_energy[i] += 0.5 * e;
                atomic_energy[j] += 0.5 * e;
            }
            const double gk = gk_[l - 1], gk1 = gk_[l], gk2 = gk_[l + 1];
            t1 = gk + (gk1 - gk) * ppp;
            t2 = gk1 + (gk2 - gk1) * (ppp - 1.0);
            const double gamma = (t1 + (t2 - t1) * ppp * 0.5) / rsq;
            const double f0 = gamma * d[0], f1 = gamma * d[1], f2 = gamma * d[2];
            fx[i] += f0; fy[i] += f1; fz[i] += f2;
            fx[j] -= f0; fy[j] -= f1; fz[j] -= f2;
            if (vx) {
                const double fv = f0 * (vx[i] + vx[j]) + f1 * (vy[i] + vy[j]) + f2 * (vz[i] + vz[j]);
                jpot[0] += (x[i] - x[j]) * fv;
                jpot[1] += (y[i] - y[j]) * fv;
                jpot[2] += (z[i] - z[j]) * fv;
            }
            s1 += d[0] * f0; s2 += d[0] * f1; s3 += d[0] * f2;
            s5 += d[1] * f1; s6 += d[1] * f2; s9 += d[2] * f2;
            virsrp = virsrp - gamma * rsq;
        }
    }
    *eng += engsrp;
    *vir += virsrp;
    stress[0] += s1; stress[1] += s2; stress[2] += s3;
    stress[3] += s2; stress[4] += s5; stress[5] += s6;
    stress[6] += s3; stress[7] += s6; stress[8] += s9;
    return npairs;
}

// lrcorrect for type 12: numtyp[t] atoms of each 1-based type t = 1..ntypes (no frozen
// atoms), cell volume volm.  Writes elrc and virlrc.
extern "C" void orc_disp_lrc(int ntypes, const double* prm, const int* numtyp, double rcut, double volm,
                             double* elrc_out, double* virlrc_out) {
    const double twopi = 6.283185307179586;
    double plrc = 0.0, elrc = 0.0;
    for (int i = 1; i <= ntypes; ++i) {
        for (int j = 1; j <= i; ++j) {
            const double* p = prm + 4 * pair_index(i, j);
            // el12 and pl12 (a term whose coefficient is 0 is skipped, as in the tables)
            double e6 = 0.0, e8 = 0.0, p6 = 0.0, p8 = 0.0;
            if (p[0] != 0.0) {
                e6 = -p[0] * std::pow(p[1], 3) * tang_toennies_lr(6, p[1] * rcut);
                p6 = p[0] * tang_toennies(6, p[1] * rcut) / std::pow(rcut, 3);
            }
            if (p[2] != 0.0) {
                e8 = p[2] * std::pow(p[3], 5) * tang_toennies_lr(8, p[3] * rcut);
                p8 = p[2] * tang_toennies(8, p[3] * rcut) / std::pow(rcut, 5);
            }
            double eadd = e6 - e8;
            double padd = 3 * eadd - p6 - p8;
            if (i != j) {
                eadd = eadd * 2.0;
                padd = padd * 2.0;
            }
            const double denprd = twopi * (double(numtyp[i - 1]) * double(numtyp[j - 1])) / (volm * volm);
            elrc = elrc + volm * denprd * eadd;
            plrc = plrc + denprd * padd / 3.0;
        }
    }
    *elrc_out = elrc;
    *virlrc_out = plrc * (-3.0 * volm);
}
