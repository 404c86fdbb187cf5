// Oracle restatement of the 1-body Partridge-Schwenke water PES used for the MB-pol
// monomer term: init_ps_type_pes (SOURCE/module.f90:507-595), ps_type_couple
// (SOURCE/ps_type_couple.f90:15-274) and its caller angfrc with keya = 9
// (SOURCE/angfrc.f:150-212, :344-410, :533-543) including the HEAT_CURRENT hooks.
// TEST INFRASTRUCTURE ONLY (see oracle.h).
// Parity unpinned: restated from the reference's Fortran, which cannot be compiled in
// this image; checked by finite differences, not against a reference run.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct Pes {
    int idx[245][3];
    int idxm[9][3];
    double c5z[245];
    double cmass[9];
    double cose = 0, xm1 = 0, xm2 = 0;
    bool loaded = false;
} g_pes;

const double reoh = 0.958649;
const double b1 = 2.0;

int load_pes(const char* path) {
    FILE* fp = std::fopen(path, "r");
    if (!fp) return 1;
    std::map<std::string, std::vector<double>> arr;
    char name[64];
    int n;
    while (std::fscanf(fp, "%63s", name) == 1) {
        if (name[0] == '#') {
            int c;
            while ((c = std::fgetc(fp)) != '\n' && c != EOF) {
            }
            continue;
        }
        if (std::fscanf(fp, "%d", &n) != 1) break;
        std::vector<double> v(n);
        for (int i = 0; i < n; ++i)
            if (std::fscanf(fp, "%lf", &v[i]) != 1) {
                std::fclose(fp);
                return 2;
            }
        arr[name] = v;
    }
    std::fclose(fp);
    const char* need[] = {"idx1", "idx2", "idx3", "c5z", "cbasis", "ccore", "crest", "cmass0", "idxm1", "idxm2", "idxm3"};
    for (const char* k : need)
        if (!arr.count(k)) return 3;
    // init_ps_type_pes (SOURCE/module.f90:507-595)
    const double hhmass = 1836.152697, hdmass = 3670.483031;
    const double engcnv = 1.19627, f5z = 0.99967788500000, fbasis = 0.15860145369897;
    const double fcore = -1.6351695982132, frest = 1.0;
    const double pi = 3.141592653589793;
    Pes& p = g_pes;
    std::vector<double> crest = arr["crest"];
    for (int i = 0; i < 245; ++i) {
        p.idx[i][0] = (int)arr["idx1"][i];
        p.idx[i][1] = (int)arr["idx2"][i];
        p.idx[i][2] = (int)arr["idx3"][i];
    }
    for (int i = 0; i < 9; ++i) {
        p.idxm[i][0] = (int)arr["idxm1"][i];
        p.idxm[i][1] = (int)arr["idxm2"][i];
        p.idxm[i][2] = (int)arr["idxm3"][i];
    }
    for (int i = 0; i < 9; ++i) {
        p.cmass[i] = arr["cmass0"][i] / (1.0 / hdmass - 1.0 / hhmass);
        double fac_corr = p.cmass[i] / hhmass;
        if (p.idxm[i][0] == p.idxm[i][1]) fac_corr = fac_corr * 0.5;
        for (int j = 0; j < 245; ++j)
            if (p.idx[j][0] == p.idxm[i][0] && p.idx[j][1] == p.idxm[i][1] && p.idx[j][2] == p.idxm[i][2]) {
                crest[j] = crest[j] - fac_corr;
                break;
            }
        for (int j = 0; j < 245; ++j)
            if (p.idx[j][1] == p.idxm[i][0] && p.idx[j][0] == p.idxm[i][1] && p.idx[j][2] == p.idxm[i][2]) {
                crest[j] = crest[j] - fac_corr;
                break;
            }
    }
    p.xm1 = 1.0 / hhmass;
    p.xm2 = 1.0 / hhmass;
    for (int i = 0; i < 245; ++i)
        p.c5z[i] = f5z * arr["c5z"][i] + fbasis * arr["cbasis"][i] + fcore * arr["ccore"][i] + frest * crest[i];
    for (int i = 0; i < 245; ++i) p.c5z[i] = p.c5z[i] * engcnv;
    for (int i = 0; i < 9; ++i) p.cmass[i] = p.cmass[i] * frest * engcnv;
    const double thetae = 104.3475 * pi / 180.0;
    p.cose = std::cos(thetae);
    p.c5z[0] = p.c5z[0] * 2.0;
    p.loaded = true;
    return 0;
}

void images1(int imcon, const double* cell, double& x, double& y, double& z) {
    // images (SOURCE/images.f:58-100) for one vector
    if (imcon == 1) {
        const double aaa = 1.0 / cell[0];
        x = x - cell[0] * std::round(aaa * x);
        y = y - cell[0] * std::round(aaa * y);
        z = z - cell[0] * std::round(aaa * z);
    } else if (imcon == 2) {
        const double aaa = 1.0 / cell[0], bbb = 1.0 / cell[4], ccc = 1.0 / cell[8];
        x = x - cell[0] * std::round(aaa * x);
        y = y - cell[4] * std::round(bbb * y);
        z = z - cell[8] * std::round(ccc * z);
    } else {
        double rc[9];
        const double* a = cell;
        rc[0] = a[4] * a[8] - a[5] * a[7];
        rc[1] = a[2] * a[7] - a[1] * a[8];
        rc[2] = a[1] * a[5] - a[2] * a[4];
        rc[3] = a[5] * a[6] - a[3] * a[8];
        rc[4] = a[0] * a[8] - a[2] * a[6];
        rc[5] = a[2] * a[3] - a[0] * a[5];
        rc[6] = a[3] * a[7] - a[4] * a[6];
        rc[7] = a[1] * a[6] - a[0] * a[7];
        rc[8] = a[0] * a[4] - a[1] * a[3];
        const double d = a[0] * rc[0] + a[3] * rc[1] + a[6] * rc[2];
        const double r = std::fabs(d) > 0.0 ? 1.0 / d : 0.0;
        for (int i = 0; i < 9; ++i) rc[i] = r * rc[i];
        const double ssx = (rc[0] * x + rc[3] * y + rc[6] * z);
        const double ssy = (rc[1] * x + rc[4] * y + rc[7] * z);
        const double ssz = (rc[2] * x + rc[5] * y + rc[8] * z);
        const double xss = ssx - std::round(ssx), yss = ssy - std::round(ssy), zss = ssz - std::round(ssz);
        x = (cell[0] * xss + cell[3] * yss + cell[6] * zss);
        y = (cell[1] * xss + cell[4] * yss + cell[7] * zss);
        z = (cell[2] * xss + cell[5] * yss + cell[8] * zss);
    }
}

}  // namespace

extern "C" int orc_pes_load(const char* path) { return load_pes(path); }

// ps_type_couple (SOURCE/ps_type_couple.f90:15-274); xoh1.. are unit vectors.
extern "C" void orc_ps_couple(double roh1, double xoh1, double yoh1, double zoh1, double roh2, double xoh2,
                              double yoh2, double zoh2, double theta, double* pterm_out, double* fdum,
                              double* vterm_out) {
    const Pes& P = g_pes;
    if (!P.loaded) {
        std::fprintf(stderr, "oracle: PES tables not loaded\n");
        std::abort();
    }
    const double cost = std::cos(theta);
    const double x1 = (roh1 - reoh) / reoh;
    const double x2 = (roh2 - reoh) / reoh;
    const double x3 = cost - P.cose;
    double fmat[16][3];
    std::memset(fmat, 0, sizeof fmat);
    fmat[1][0] = 1.0;
    fmat[1][1] = 1.0;
    fmat[1][2] = 1.0;
    for (int j = 2; j <= 15; ++j) {
        fmat[j][0] = fmat[j - 1][0] * x1;
        fmat[j][1] = fmat[j - 1][1] * x2;
        fmat[j][2] = fmat[j - 1][2] * x3;
    }
    double pterm = 0.0, vterm = 0.0;
    double fxa = 0, fya = 0, fza = 0, fxc = 0, fyc = 0, fzc = 0;
    for (int j = 1; j < 245; ++j) {  // Fortran j = 2..245
        const int i1 = P.idx[j][0], i2 = P.idx[j][1], i3 = P.idx[j][2];
        const double dum = fmat[i1][0] * fmat[i2][1] + fmat[i2][0] * fmat[i1][1];
        const double term = P.c5z[j] * dum * fmat[i3][2];
        pterm = pterm + term;
        double dum1x = (i1 - 1) * fmat[i1 - 1][0] * xoh1 / reoh;
        double dum1y = (i1 - 1) * fmat[i1 - 1][0] * yoh1 / reoh;
        double dum1z = (i1 - 1) * fmat[i1 - 1][0] * zoh1 / reoh;
        double dum2x = (i2 - 1) * fmat[i2 - 1][0] * xoh1 / reoh;
        double dum2y = (i2 - 1) * fmat[i2 - 1][0] * yoh1 / reoh;
        double dum2z = (i2 - 1) * fmat[i2 - 1][0] * zoh1 / reoh;
        double dum3x = (i3 - 1) * fmat[i3 - 1][2] * (xoh2 - cost * xoh1) / roh1;
        double dum3y = (i3 - 1) * fmat[i3 - 1][2] * (yoh2 - cost * yoh1) / roh1;
        double dum3z = (i3 - 1) * fmat[i3 - 1][2] * (zoh2 - cost * zoh1) / roh1;
        double dumx = dum1x * fmat[i2][1] * fmat[i3][2] + dum2x * fmat[i1][1] * fmat[i3][2] + dum * dum3x;
        double dumy = dum1y * fmat[i2][1] * fmat[i3][2] + dum2y * fmat[i1][1] * fmat[i3][2] + dum * dum3y;
        double dumz = dum1z * fmat[i2][1] * fmat[i3][2] + dum2z * fmat[i1][1] * fmat[i3][2] + dum * dum3z;
        fxa = fxa - P.c5z[j] * dumx;
        fya = fya - P.c5z[j] * dumy;
        fza = fza - P.c5z[j] * dumz;
        dum1x = (i2 - 1) * fmat[i2 - 1][1] * xoh2 / reoh;
        dum1y = (i2 - 1) * fmat[i2 - 1][1] * yoh2 / reoh;
        dum1z = (i2 - 1) * fmat[i2 - 1][1] * zoh2 / reoh;
        dum2x = (i1 - 1) * fmat[i1 - 1][1] * xoh2 / reoh;
        dum2y = (i1 - 1) * fmat[i1 - 1][1] * yoh2 / reoh;
        dum2z = (i1 - 1) * fmat[i1 - 1][1] * zoh2 / reoh;
        dum3x = (i3 - 1) * fmat[i3 - 1][2] * (xoh1 - cost * xoh2) / roh2;
        dum3y = (i3 - 1) * fmat[i3 - 1][2] * (yoh1 - cost * yoh2) / roh2;
        dum3z = (i3 - 1) * fmat[i3 - 1][2] * (zoh1 - cost * zoh2) / roh2;
        dumx = fmat[i1][0] * dum1x * fmat[i3][2] + fmat[i2][0] * dum2x * fmat[i3][2] + dum * dum3x;
        dumy = fmat[i1][0] * dum1y * fmat[i3][2] + fmat[i2][0] * dum2y * fmat[i3][2] + dum * dum3y;
        dumz = fmat[i1][0] * dum1z * fmat[i3][2] + fmat[i2][0] * dum2z * fmat[i3][2] + dum * dum3z;
        fxc = fxc - P.c5z[j] * dumx;
        fyc = fyc - P.c5z[j] * dumy;
        fzc = fzc - P.c5z[j] * dumz;
        vterm = vterm + P.c5z[j] *
                            (roh1 * fmat[i2][1] * (i1 - 1) * fmat[i1 - 1][0] / reoh +
                             roh2 * fmat[i1][0] * (i2 - 1) * fmat[i2 - 1][1] / reoh +
                             roh1 * fmat[i1][1] * (i2 - 1) * fmat[i2 - 1][0] / reoh +
                             roh2 * fmat[i2][0] * (i1 - 1) * fmat[i1 - 1][1] / reoh) *
                            fmat[i3][2];
    }
    double v1 = 0.0, v2 = 0.0;
    const double xm1 = P.xm1, xm2 = P.xm2;
    for (int j = 0; j < 9; ++j) {
        const int m1 = P.idxm[j][0], m2 = P.idxm[j][1], m3 = P.idxm[j][2];
        v1 = v1 + P.cmass[j] * fmat[m1][0] * fmat[m2][1] * fmat[m3][2];
        v2 = v2 + P.cmass[j] * fmat[m2][0] * fmat[m1][1] * fmat[m3][2];
        double dum1x = (m1 - 1) * fmat[m1 - 1][0] * xoh1 / reoh;
        double dum1y = (m1 - 1) * fmat[m1 - 1][0] * yoh1 / reoh;
        double dum1z = (m1 - 1) * fmat[m1 - 1][0] * zoh1 / reoh;
        double dum2x = (m2 - 1) * fmat[m2 - 1][0] * xoh1 / reoh;
        double dum2y = (m2 - 1) * fmat[m2 - 1][0] * yoh1 / reoh;
        double dum2z = (m2 - 1) * fmat[m2 - 1][0] * zoh1 / reoh;
        double dum3x = (m3 - 1) * fmat[m3 - 1][2] * (xoh2 - cost * xoh1) / roh1;
        double dum3y = (m3 - 1) * fmat[m3 - 1][2] * (yoh2 - cost * yoh1) / roh1;
        double dum3z = (m3 - 1) * fmat[m3 - 1][2] * (zoh2 - cost * zoh1) / roh1;
        double cx = xm1 * (dum1x * fmat[m2][1] * fmat[m3][2] + fmat[m1][0] * fmat[m2][1] * dum3x) +
                    xm2 * (dum2x * fmat[m1][1] * fmat[m3][2] + fmat[m2][0] * fmat[m1][1] * dum3x);
        double cy = xm1 * (dum1y * fmat[m2][1] * fmat[m3][2] + fmat[m1][0] * fmat[m2][1] * dum3y) +
                    xm2 * (dum2y * fmat[m1][1] * fmat[m3][2] + fmat[m2][0] * fmat[m1][1] * dum3y);
        double cz = xm1 * (dum1z * fmat[m2][1] * fmat[m3][2] + fmat[m1][0] * fmat[m2][1] * dum3z) +
                    xm2 * (dum2z * fmat[m1][1] * fmat[m3][2] + fmat[m2][0] * fmat[m1][1] * dum3z);
        fxa = fxa - P.cmass[j] * cx;
        fya = fya - P.cmass[j] * cy;
        fza = fza - P.cmass[j] * cz;
        dum1x = (m2 - 1) * fmat[m2 - 1][1] * xoh2 / reoh;
        dum1y = (m2 - 1) * fmat[m2 - 1][1] * yoh2 / reoh;
        dum1z = (m2 - 1) * fmat[m2 - 1][1] * zoh2 / reoh;
        dum2x = (m1 - 1) * fmat[m1 - 1][1] * xoh2 / reoh;
        dum2y = (m1 - 1) * fmat[m1 - 1][1] * yoh2 / reoh;
        dum2z = (m1 - 1) * fmat[m1 - 1][1] * zoh2 / reoh;
        dum3x = (m3 - 1) * fmat[m3 - 1][2] * (xoh1 - cost * xoh2) / roh2;
        dum3y = (m3 - 1) * fmat[m3 - 1][2] * (yoh1 - cost * yoh2) / roh2;
        dum3z = (m3 - 1) * fmat[m3 - 1][2] * (zoh1 - cost * zoh2) / roh2;
        cx = xm1 * (fmat[m1][0] * dum1x * fmat[m3][2] + fmat[m1][0] * fmat[m2][1] * dum3x) +
             xm2 * (fmat[m2][0] * dum2x * fmat[m3][2] + fmat[m2][0] * fmat[m1][1] * dum3x);
        cy = xm1 * (fmat[m1][0] * dum1y * fmat[m3][2] + fmat[m1][0] * fmat[m2][1] * dum3y) +
             xm2 * (fmat[m2][0] * dum2y * fmat[m3][2] + fmat[m2][0] * fmat[m1][1] * dum3y);
        cz = xm1 * (fmat[m1][0] * dum1z * fmat[m3][2] + fmat[m1][0] * fmat[m2][1] * dum3z) +
             xm2 * (fmat[m2][0] * dum2z * fmat[m3][2] + fmat[m2][0] * fmat[m1][1] * dum3z);
        fxc = fxc - P.cmass[j] * cx;
        fyc = fyc - P.cmass[j] * cy;
        fzc = fzc - P.cmass[j] * cz;
        vterm = vterm + P.cmass[j] *
                            (xm1 * roh1 * fmat[m2][1] * (m1 - 1) * fmat[m1 - 1][0] / reoh +
                             xm1 * roh2 * fmat[m1][0] * (m2 - 1) * fmat[m2 - 1][1] / reoh +
                             xm2 * roh1 * fmat[m1][1] * (m2 - 1) * fmat[m2 - 1][0] / reoh +
                             xm2 * roh2 * fmat[m2][0] * (m1 - 1) * fmat[m1 - 1][1] / reoh) *
                            fmat[m3][2];
    }
    pterm = pterm + xm1 * v1 + xm2 * v2;
    const double efac = std::exp(-b1 * ((roh1 - reoh) * (roh1 - reoh) + (roh2 - reoh) * (roh2 - reoh)));
    const double term = pterm;
    pterm = term * efac + P.c5z[0];
    pterm = pterm + 2.0384848702093006e-6 * 2625.50 / 100.0;
    fxa = fxa * efac + 2.0 * b1 * (roh1 - reoh) * xoh1 * efac * term;
    fya = fya * efac + 2.0 * b1 * (roh1 - reoh) * yoh1 * efac * term;
    fza = fza * efac + 2.0 * b1 * (roh1 - reoh) * zoh1 * efac * term;
    fxc = fxc * efac + 2.0 * b1 * (roh2 - reoh) * xoh2 * efac * term;
    fyc = fyc * efac + 2.0 * b1 * (roh2 - reoh) * yoh2 * efac * term;
    fzc = fzc * efac + 2.0 * b1 * (roh2 - reoh) * zoh2 * efac * term;
    const double dummy1 = -2.0 * b1 * (roh1 - reoh) * roh1 * efac;
    const double dummy2 = -2.0 * b1 * (roh2 - reoh) * roh2 * efac;
    vterm = dummy1 * term + dummy2 * term + efac * vterm;
    fdum[0] = fxa; fdum[1] = fya; fdum[2] = fza;
    fdum[3] = fxc; fdum[4] = fyc; fdum[5] = fzc;
    *pterm_out = pterm;
    *vterm_out = vterm;
}

// angfrc with keya = 9 for every angle (SOURCE/angfrc.f:150-212, :344-545) and its
// HEAT_CURRENT hooks: per-atom energy pterm/3, force-matrix entries (ia,ib), (ib,ia),
// (ic,ib), (ib,ic) contracted as in compute_heat_flux2 (raw coordinates).
extern "C" int orc_angfrc_ps(int imcon, const double* cell, int nang, const int* listang, const double* x,
                             const double* y, const double* z, double* fx, double* fy, double* fz, double* engang,
                             double* virang, double* stress, double* atomic_energy, const double* vx,
                             const double* vy, const double* vz, double* jpot) {
    double eng = 0.0, vir = 0.0;
    double s1 = 0, s2 = 0, s3 = 0, s5 = 0, s6 = 0, s9 = 0;
    for (int ii = 0; ii < nang; ++ii) {
        const int ia = listang[3 * ii] - 1, ib = listang[3 * ii + 1] - 1, ic = listang[3 * ii + 2] - 1;
        double xdab = x[ia] - x[ib], ydab = y[ia] - y[ib], zdab = z[ia] - z[ib];
        double xdbc = x[ic] - x[ib], ydbc = y[ic] - y[ib], zdbc = z[ic] - z[ib];
        images1(imcon, cell, xdab, ydab, zdab);
        images1(imcon, cell, xdbc, ydbc, zdbc);
        const double rab = std::sqrt(xdab * xdab + ydab * ydab + zdab * zdab);
        const double rrab = 1.0 / rab;
        const double xab = xdab * rrab, yab = ydab * rrab, zab = zdab * rrab;
        const double rbc = std::sqrt(xdbc * xdbc + ydbc * ydbc + zdbc * zdbc);
        const double rrbc = 1.0 / rbc;
        const double xbc = xdbc * rrbc, ybc = ydbc * rrbc, zbc = zdbc * rrbc;
        const double cost = (xab * xbc + yab * ybc + zab * zbc);
        const double theta = std::acos(cost);
        double pterm, vterm, f[6];
        orc_ps_couple(rab, xab, yab, zab, rbc, xbc, ybc, zbc, theta, &pterm, f, &vterm);
        eng = eng + pterm;
        if (atomic_energy) {
            atomic_energy[ia] += pterm / 3;
            atomic_energy[ib] += pterm / 3;
            atomic_energy[ic] += pterm / 3;
        }
        fx[ia] += f[0]; fy[ia] += f[1]; fz[ia] += f[2];
        fx[ib] = fx[ib] - f[0] - f[3];
        fy[ib] = fy[ib] - f[1] - f[4];
        fz[ib] = fz[ib] - f[2] - f[5];
        fx[ic] += f[3]; fy[ic] += f[4]; fz[ic] += f[5];
        if (vx && jpot) {
            // update_forces(ia,ib,fa), (ib,ia,-fa), (ic,ib,fc), (ib,ic,-fc) contracted
            const double fva = f[0] * (vx[ia] + vx[ib]) + f[1] * (vy[ia] + vy[ib]) + f[2] * (vz[ia] + vz[ib]);
            const double fvc = f[3] * (vx[ic] + vx[ib]) + f[4] * (vy[ic] + vy[ib]) + f[5] * (vz[ic] + vz[ib]);
            jpot[0] += (x[ia] - x[ib]) * fva + (x[ic] - x[ib]) * fvc;
            jpot[1] += (y[ia] - y[ib]) * fva + (y[ic] - y[ib]) * fvc;
            jpot[2] += (z[ia] - z[ib]) * fva + (z[ic] - z[ib]) * fvc;
        }
        vir = vir + vterm;
        s1 = s1 + rab * xab * f[0] + rbc * xbc * f[3];
        s2 = s2 + rab * xab * f[1] + rbc * xbc * f[4];
        s3 = s3 + rab * xab * f[2] + rbc * xbc * f[5];
        s5 = s5 + rab * yab * f[1] + rbc * ybc * f[4];
        s6 = s6 + rab * yab * f[2] + rbc * ybc * f[5];
        s9 = s9 + rab * zab * f[2] + rbc * zbc * f[5];
    }
    *engang += eng;
    *virang += vir;
    stress[0] += s1; stress[1] += s2; stress[2] += s3;
    stress[3] += s2; stress[4] += s5; stress[5] += s6;
    stress[6] += s3; stress[7] += s6; stress[8] += s9;
    return 0;
}

// ---------------------------------------------------------------------------
// M sites and the Partridge-Schwenke dipole-moment surface charges.
namespace {
struct Dms {
    int idx[84][3];
    double coef[84];
    int isump = 0;
    bool loaded = false;
} g_dms;
}  // namespace

extern "C" int orc_dms_load(const char* path) {
    FILE* fp = std::fopen(path, "r");
    if (!fp) return 1;
    std::map<std::string, std::vector<double>> arr;
    char name[64];
    int n;
    while (std::fscanf(fp, "%63s", name) == 1) {
        if (name[0] == '#') {
            int c;
            while ((c = std::fgetc(fp)) != '\n' && c != EOF) {
            }
            continue;
        }
        if (std::fscanf(fp, "%d", &n) != 1) break;
        std::vector<double> v(n);
        for (int i = 0; i < n; ++i)
            if (std::fscanf(fp, "%lf", &v[i]) != 1) {
                std::fclose(fp);
                return 2;
            }
        arr[name] = v;
    }
    std::fclose(fp);
    if (!arr.count("idx1") || !arr.count("coef")) return 3;
    // init_ps_type_dms (SOURCE/module.f90:890-916)
    g_dms.isump = 0;
    for (int i = 0; i < 84; ++i) {
        g_dms.idx[i][0] = (int)arr["idx1"][i];
        g_dms.idx[i][1] = (int)arr["idx2"][i];
        g_dms.idx[i][2] = (int)arr["idx3"][i];
        g_dms.coef[i] = arr["coef"][i];
        for (int k = 0; k < 3; ++k) g_dms.isump = std::max(g_dms.isump, g_dms.idx[i][k]);
    }
    g_dms.loaded = true;
    return 0;
}

// M-site coordinates, SOURCE/dlpoly_cmd.f:2041-2057: r_M = r_O + gamma/2 (r_OH1 + r_OH2).
extern "C" void orc_msites(int imcon, const double* cell, int nw, const int* listttm2, double* x, double* y, double* z,
                           double gamma) {
    if (nw <= 0) return;
    int mttm2 = listttm2[3 * nw - 1];  // 1-based
    for (int i = 0; i < nw; ++i) {
        mttm2 = mttm2 + 1;
        const int io = listttm2[3 * i] - 1, h1 = listttm2[3 * i + 1] - 1, h2 = listttm2[3 * i + 2] - 1;
        double x1 = x[h1] - x[io], y1 = y[h1] - y[io], z1 = z[h1] - z[io];
        double x2 = x[h2] - x[io], y2 = y[h2] - y[io], z2 = z[h2] - z[io];
        images1(imcon, cell, x1, y1, z1);
        images1(imcon, cell, x2, y2, z2);
        x[mttm2 - 1] = x[io] + (x1 + x2) * gamma / 2.0;
        y[mttm2 - 1] = y[io] + (y1 + y2) * gamma / 2.0;
        z[mttm2 - 1] = z[io] + (z1 + z2) * gamma / 2.0;
    }
}

// qdetermine with ldms, .not. lttm3, .not. lttmfold (the MB-pol settings of
// SOURCE/simdef_cmd.f:1040-1060): H and M charges and dq/d(r1, r2, cos) into
// dp[6*nw] = {dp1dr1, dp1dr2, dp2dr1, dp2dr2, dp1dcos, dp2dcos} per water
// (SOURCE/qdetermine.f90:112-285).  Returns the largest |sum of water charges|.
extern "C" double orc_qdetermine(int imcon, const double* cell, int nw, const int* listttm2, const double* x,
                                 const double* y, const double* z, double gamma, double* chge, double* dp) {
    if (!g_dms.loaded || !g_pes.loaded) {
        std::fprintf(stderr, "oracle: DMS/PES tables not loaded\n");
        std::abort();
    }
    const double bohr = 0.529177249;
    const double b1dms = 1.0, adms = 0.2999 * bohr, bdms = -0.6932;
    const double c0 = 1.0099, c1 = -0.1801, c2 = 0.0892;
    const Dms& D = g_dms;
    double worst = 0.0;
    int mttm2 = nw > 0 ? listttm2[3 * nw - 1] : 0;
    for (int i = 0; i < nw; ++i) {
        mttm2 = mttm2 + 1;
        const int io = listttm2[3 * i] - 1, h1 = listttm2[3 * i + 1] - 1, h2 = listttm2[3 * i + 2] - 1;
        double r1x = x[h1] - x[io], r1y = y[h1] - y[io], r1z = z[h1] - z[io];
        images1(imcon, cell, r1x, r1y, r1z);
        const double r1 = std::sqrt(r1x * r1x + r1y * r1y + r1z * r1z);
        double r2x = x[h2] - x[io], r2y = y[h2] - y[io], r2z = z[h2] - z[io];
        images1(imcon, cell, r2x, r2y, r2z);
        const double r2 = std::sqrt(r2x * r2x + r2y * r2y + r2z * r2z);
        const double cost = (r1x * r2x + r1y * r2y + r1z * r2z) / (r1 * r2);
        const double x1 = (r1 - reoh) / reoh, x2 = (r2 - reoh) / reoh, x3 = cost - g_pes.cose;
        double fmat[11][3];
        std::memset(fmat, 0, sizeof fmat);
        fmat[1][0] = fmat[1][1] = fmat[1][2] = 1.0;
        for (int j = 2; j <= D.isump; ++j) {
            fmat[j][0] = fmat[j - 1][0] * x1;
            fmat[j][1] = fmat[j - 1][1] * x2;
            fmat[j][2] = fmat[j - 1][2] * x3;
        }
        double p1 = 0.0, p2 = 0.0, d11 = 0, d12 = 0, d21 = 0, d22 = 0, d1c = 0, d2c = 0;
        for (int j = 1; j < 84; ++j) {
            const int i1 = D.idx[j][0], i2 = D.idx[j][1], i3 = D.idx[j][2];
            const double c = D.coef[j];
            p1 = p1 + c * fmat[i1][0] * fmat[i2][1] * fmat[i3][2];
            p2 = p2 + c * fmat[i2][0] * fmat[i1][1] * fmat[i3][2];
            d11 = d11 + c * (i1 - 1) * fmat[i1 - 1][0] * fmat[i2][1] * fmat[i3][2] / reoh;
            d12 = d12 + c * (i2 - 1) * fmat[i1][0] * fmat[i2 - 1][1] * fmat[i3][2] / reoh;
            d21 = d21 + c * (i2 - 1) * fmat[i2 - 1][0] * fmat[i1][1] * fmat[i3][2] / reoh;
            d22 = d22 + c * (i1 - 1) * fmat[i2][0] * fmat[i1 - 1][1] * fmat[i3][2] / reoh;
            d1c = d1c + c * (i3 - 1) * fmat[i1][0] * fmat[i2][1] * fmat[i3 - 1][2];
            d2c = d2c + c * (i3 - 1) * fmat[i2][0] * fmat[i1][1] * fmat[i3 - 1][2];
        }
        const double pl1 = cost;
        const double pl2 = 0.5 * (3.0 * pl1 * pl1 - 1.0);
        const double damp = std::exp(-b1dms * ((r1 - reoh) * (r1 - reoh) + (r2 - reoh) * (r2 - reoh)));
        const double ddampdr1 = -2.0 * b1dms * (r1 - reoh) * damp;
        const double ddampdr2 = -2.0 * b1dms * (r2 - reoh) * damp;
        const double ang = c0 + pl1 * c1 + pl2 * c2;
        const double pc0 = adms * (std::pow(r1, bdms) + std::pow(r2, bdms)) * ang;
        const double dpc0dr1 = adms * (bdms * std::pow(r1, bdms - 1)) * ang;
        const double dpc0dr2 = adms * (bdms * std::pow(r2, bdms - 1)) * ang;
        const double dpc0dcos = adms * (std::pow(r1, bdms) + std::pow(r2, bdms)) * (c1 + 3.0 * c2 * pl1);
        d11 = d11 * damp + p1 * ddampdr1 + dpc0dr1;
        d12 = d12 * damp + p1 * ddampdr2 + dpc0dr2;
        d21 = d21 * damp + p2 * ddampdr1 + dpc0dr1;
        d22 = d22 * damp + p2 * ddampdr2 + dpc0dr2;
        d1c = d1c * damp + dpc0dcos;
        d2c = d2c * damp + dpc0dcos;
        p1 = D.coef[0] + p1 * damp + pc0;
        p2 = D.coef[0] + p2 * damp + pc0;
        const double factor = gamma / 2.0 / (1.0 - gamma);
        chge[h1] = p1 + factor * (p1 + p2);
        chge[h2] = p2 + factor * (p1 + p2);
        chge[mttm2 - 1] = -(chge[h1] + chge[h2]);
        if (dp) {
            double* o = dp + 6 * (size_t)i;
            o[0] = d11; o[1] = d12; o[2] = d21; o[3] = d22; o[4] = d1c; o[5] = d2c;
        }
        worst = std::max(worst, std::fabs(chge[mttm2 - 1] + chge[h1] + chge[h2] + chge[io]));
    }
    return worst;
}
