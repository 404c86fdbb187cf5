// TTM4-F polarizable electrostatics of MB-pol water (the reference's polar Ewald branch
// with the vmbpol settings, SOURCE/simdef_cmd.f:1040-1060) with its heat-current terms.
//
//   list      site pairs of different waters within rcut (the Verlet pairs of SOURCE/parlst.f
//             with the TTM exclusions of SOURCE/exclude_ttm.f); directed, one row per site
//   static    rfield's first pass (SOURCE/rfield.f:59-201, :330-421): charge field of the
//             Verlet pairs (table B functions, Thole exp-4 smearing) and of the excluded
//             intramolecular pairs (analytic B functions); the dipole tensors of every pair
//             are stored for the iterations
//   k space   ewald1p (SOURCE/ewald1p.f): exp(ik.r) per k vector and site is tabulated once
//             per call; each pass is a structure-factor reduction over sites (block per k)
//             and a field / force gather over k vectors (thread per site)
//   iterate   rfield's dipole field + ewald1p's dipole field + iter (SOURCE/iter.f:43-100)
//             until the RMS dipole change is <= toler (SOURCE/forces.f:271-366)
//   final     coulomb_polar, ewald1p iflag 1 (forces, energy, virial, stress, DMS potentials,
//             HEAT_CURRENT per-atom stress and energy), ewald2p over the Verlet pairs,
//             ewald3p over the excluded pairs, qdforce (SOURCE/qdforce.f90) with the summed
//             DMS potentials
//   heat      update_forces entries, the M-site row redistribution and compute_heat_flux2's
//             contraction applied entry by entry (SOURCE/heatcurrent.f90:529-559, :703-728)
//
// Standard layout: 4*nw sites, water w has O, H1, H2 at 3w..3w+2 and its M site at 3nw+w.
// FP64 throughout; erfcc and gammq are the reference's published approximations
// (Numerical Recipes' erfc fit with single-precision constants; the incomplete gamma
// series / continued fraction with EPS 3e-7).
#include "mbx_kernels.cuh"

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <vector>

namespace mbx {

namespace {

constexpr double kR4pie0 = 138935.4835;   // SOURCE/dl_params.inc:60
constexpr double kSqrpi = 1.7724538509055159;
constexpr double kPi = 3.141592653589793;
constexpr int kSfThreads = 256;
// Beyond a Thole / smearing argument of 40 every damping factor is below exp(-40) = 4e-18
// of the undamped term it multiplies (and gammq's term likewise): the exponentials are not
// evaluated there, which changes no result beyond 1e-16 relative.
constexpr double kDampCut = 40.0;
constexpr int kKTile = 64;

// --- special functions (host and device) --------------------------------------------
__host__ __device__ inline double erfcc(double x) {
    const double z = fabs(x);
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
    double r = t * exp(e);
    if (x < 0.0) r = 2.0 - r;
    return r;
}

__host__ __device__ inline double gammln(double xx) {
    const double cof[6] = {76.18009172947146, -86.50532032941677, 24.01409824083091,
                           -1.231739572450155, .1208650973866179e-2, -.5395239384953e-5};
    double x = xx, y = x;
    double tmp = x + 5.5;
    tmp = (x + 0.5) * log(tmp) - tmp;
    double ser = 1.000000000190015;
    for (int j = 0; j < 6; ++j) {
        y = y + 1.0;
        ser = ser + cof[j] / y;
    }
    return tmp + log(2.5066282746310005 * ser / x);
}

// gammq(a, x) with gln = gammln(a) given (a per-call constant of the smeared-charge term)
__device__ inline double gammq_g(double a, double x, double gln) {
    const double eps = (double)3.e-7f, fpmin = (double)1.e-30f;
    if (x < a + 1.0) {
        if (x <= 0.0) return 1.0;
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 1; n <= 800; ++n) {
            ap = ap + 1.0;
            del = del * x / ap;
            sum = sum + del;
            if (fabs(del) < fabs(sum) * eps) break;
        }
        return 1.0 - sum * exp(-x + a * log(x) - gln);
    }
    double b = x + 1.0 - a, c = 1.0 / fpmin, d = 1.0 / b, h = d;
    for (int i = 1; i <= 100; ++i) {
        const double an = -i * (i - a);
        b = b + 2.0;
        d = an * d + b;
        if (fabs(d) < fpmin) d = fpmin;
        c = b + an / c;
        if (fabs(c) < fpmin) c = fpmin;
        d = 1.0 / d;
        const double del = d * c;
        h = h * del;
        if (fabs(del - 1.0) < eps) break;
    }
    return exp(-x + a * log(x) - gln) * h;
}

__device__ inline double gammq(double a, double x) { return gammq_g(a, x, gammln(a)); }

// B_0..B_3 of the real-space sum from erfcc (rfield / ewald3p intramolecular form)
__device__ inline void bfun_exact(double alpha, double rr, double rri, double rsqi, double bbb[4]) {
    const double a = alpha * rr;
    bbb[0] = (erfcc(a) - 1.0) * rri;
    const double exp2a = exp(-a * a);
    const double a2 = 2.0 * (alpha * alpha);
    double pw = 1.0;
    for (int m = 1; m <= 3; ++m) {
        pw = m == 1 ? a2 : (m == 2 ? a2 * a2 : pow(a2, 3.0));
        bbb[m] = rsqi * ((2.0 * m - 1.0) * bbb[m - 1] + pw * exp2a / alpha / kSqrpi);
    }
}

struct PolArgs {
    Cell cl;
    int nw, n, cap;
    const double *x, *y, *z, *q, *polr, *polr2, *dp;
    const double* polr6;   // polr^(1/6) per site: the Thole width of a pair is polr6_i polr6_j
    const double* rpolr6;  // 1 / polr6 per site
    double *mx, *my, *mz;
    const double *vx, *vy, *vz;
    double *fx, *fy, *fz;
    double gamma, alpha, rcut, rcsq, eps, athole, athole12, athole13, ascc, ascd, toler, omega;
    const double4* ercp;
    const float4* ercp32;   // C_n = B_n + (2n-1)!! / r^(2n+1) per table row, FP32 (mixed path), or null
    double drewd, rdrewd;   // the erfcgenp grid step and its reciprocal
    const int *nn, *nbr;
    const int* npol;   // per row: its first npol partners are the polarizable ones (polr2 > 1e-6)
    const int2* nup;   // per row: partners j > i at the head of each group (x polarizable, y the others)
    double* tens;   // 6 blocks of n * cap: the first npol entries of the polarizable rows
    float* tens32;  // the same in FP32 (mixed precision), or null
    double* intra;  // 18 per water
    float* intra32; // the same in FP32 (the FP32 real-space field)
    double *efk, *efc, *emu, *efm;   // 3 blocks of n each
    double *vesp, *ae;
    double* acc;
};

__device__ __forceinline__ int site_mol(const PolArgs& a, int i) { return i < 3 * a.nw ? i / 3 : i - 3 * a.nw; }

__device__ __forceinline__ void sep(const PolArgs& a, int i, int j, double& dx, double& dy, double& dz) {
    dx = dsub(a.x[i], a.x[j]);
    dy = dsub(a.y[i], a.y[j]);
    dz = dsub(a.z[i], a.z[j]);
    image(a.cl, dx, dy, dz);
}

__device__ __forceinline__ double norm2(double dx, double dy, double dz) {
    return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}

// interp with the grid index from r / drewd as a product with the reciprocal step (the
// index and fraction agree with the quotient's to rounding)
__device__ __forceinline__ void interp_r(const PolArgs& a, double rr, double bbb[4]) {
    const double u = rr * a.rdrewd;
    const int ll = (int)u;
    const double ppp = u - double(ll);
    const double4 v0 = a.ercp[ll], v1 = a.ercp[ll + 1], v2 = a.ercp[ll + 2];
    const double vk[4] = {v0.x, v0.y, v0.z, v0.w}, vk1[4] = {v1.x, v1.y, v1.z, v1.w}, vk2[4] = {v2.x, v2.y, v2.z, v2.w};
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        const double t1 = vk[n] + (vk1[n] - vk[n]) * ppp;
        const double t2 = vk1[n] + (vk2[n] - vk1[n]) * (ppp - 1.0);
        bbb[n] = t1 + (t2 - t1) * ppp * 0.5;
    }
}

__device__ __forceinline__ void interp(const PolArgs& a, double rr, double bbb[4]) {
    const int ll = (int)(rr / a.drewd);
    const double ppp = rr / a.drewd - double(ll);
    const double4 v0 = a.ercp[ll], v1 = a.ercp[ll + 1], v2 = a.ercp[ll + 2];
    const double vk[4] = {v0.x, v0.y, v0.z, v0.w}, vk1[4] = {v1.x, v1.y, v1.z, v1.w}, vk2[4] = {v2.x, v2.y, v2.z, v2.w};
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        const double t1 = vk[n] + (vk1[n] - vk[n]) * ppp;
        const double t2 = vk1[n] + (vk2[n] - vk1[n]) * (ppp - 1.0);
        bbb[n] = t1 + (t2 - t1) * ppp * 0.5;
    }
}

__device__ __forceinline__ double pow4(double t) {
    const double t2 = t * t;
    return t2 * t2;
}


// Heat-current contribution of the force-matrix entry (row a, column b, F) after the
// M-site row redistribution (columns of M sites are never read).
__device__ __forceinline__ void heat_entry(const PolArgs& a, int row, int col, double Fx, double Fy, double Fz,
                                           double jp[3]) {
    const int na = 3 * a.nw;
    if (col >= na) return;
    int c[3];
    double w[3];
    int m = 1;
    if (row < na) {
        c[0] = row;
        w[0] = 1.0;
    } else {
        const int wt = row - na;
        c[0] = 3 * wt; c[1] = 3 * wt + 1; c[2] = 3 * wt + 2;
        w[0] = 1.0 - a.gamma; w[1] = 0.5 * a.gamma; w[2] = 0.5 * a.gamma;
        m = 3;
    }
    for (int k = 0; k < m; ++k) {
        if (c[k] == col) continue;
        const double fv = w[k] * (Fx * a.vx[c[k]] + Fy * a.vy[c[k]] + Fz * a.vz[c[k]]);
        jp[0] += (a.x[c[k]] - a.x[col]) * fv;
        jp[1] += (a.y[c[k]] - a.y[col]) * fv;
        jp[2] += (a.z[c[k]] - a.z[col]) * fv;
    }
}

// Velocity a per-site quantity is carried with after the redistribution
__device__ __forceinline__ void vhat(const PolArgs& a, int j, double v[3]) {
    const int na = 3 * a.nw;
    if (j < na) {
        v[0] = a.vx[j]; v[1] = a.vy[j]; v[2] = a.vz[j];
        return;
    }
    const int o = 3 * (j - na);
    const double g1 = 1.0 - a.gamma, g2 = 0.5 * a.gamma;
    v[0] = g1 * a.vx[o] + g2 * a.vx[o + 1] + g2 * a.vx[o + 2];
    v[1] = g1 * a.vy[o] + g2 * a.vy[o + 1] + g2 * a.vy[o + 2];
    v[2] = g1 * a.vz[o] + g2 * a.vz[o + 1] + g2 * a.vz[o + 2];
}

// --- list -----------------------------------------------------------------------------
__global__ void k_pol_f32(int n, const double* __restrict__ x, const double* __restrict__ y,
                          const double* __restrict__ z, float4* __restrict__ xf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xf[i] = make_float4((float)x[i], (float)y[i], (float)z[i], 0.f);
}

// Partners of site i: every site of another water whose imaged separation passes the
// reference's cut (rcut > r in rfield, rcut^2 > r^2 in ewald2p), in increasing index.
// An FP32 test with a margin far above its rounding screens the candidates first.
// Cell of a site along one axis (orthorhombic cells, positions wrapped into the box).
__device__ __forceinline__ int pol_wrap(double s, int nc) {
    s = s - floor(s);
    const int c = (int)(s * nc);
    return c >= nc ? nc - 1 : (c < 0 ? 0 : c);
}

__global__ void k_pol_keys(int n, const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ z, Cell cl, int3 nc, unsigned* __restrict__ key,
                           int* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = (unsigned)((pol_wrap(z[i] * cl.inv[2], nc.z) * nc.y + pol_wrap(y[i] * cl.inv[1], nc.y)) * nc.x +
                        pol_wrap(x[i] * cl.inv[0], nc.x));
    idx[i] = i;
}

__global__ void k_pol_bounds(int n, const unsigned* __restrict__ skey, int* __restrict__ start,
                             int* __restrict__ end) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned c = skey[i];
    if (i == 0 || skey[i - 1] != c) start[c] = i;
    if (i == n - 1 || skey[i + 1] != c) end[c] = i + 1;
}

// The site pair list (the reference's Verlet pairs with exclude_ttm's exclusions: every
// site of another water within rcut), one directed row per site, warp per site.
// Candidates: the sites of the 27 cells around the site's cell (orthorhombic boxes with
// at least 3 cells of width >= rcut + 0.02 A per side), else every site.  An FP32
// prefilter with a 0.001 A margin, then the reference's FP64 test.
// A pair whose FP32 distance is inside rcut - 0.001 A (r2in) is inside rcut in FP64 too (the
// FP32 error of r^2 is below 1e-3 A^2 for coordinates under 1e3 A), so only the thin shell
// between r2in and r2f takes the reference's FP64 test.
// Row order: the polarizable partners first (npol of them), then the others; within each
// group the partners j > i first (nup.x and nup.y of them), so a kernel can take every pair
// once from its lower site (k_pol_ewald2p32) while the dipole kernels read whole rows.
__global__ void k_pol_list(PolArgs a, int* __restrict__ nn, int* __restrict__ nbr, int* __restrict__ npol,
                           int2* __restrict__ nup, int rowcap, double lc, const float4* __restrict__ xf, float r2f,
                           float r2in, int* __restrict__ flag, int3 nc, int cells, const int* __restrict__ sidx,
                           const int* __restrict__ cstart, const int* __restrict__ cend) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.n) return;
    const int mi = site_mol(a, i);
    const float4 pi = xf[i];
    int* my = nbr + (size_t)i * rowcap;
    int cnt = 0;
    const double lc2 = lc * lc;
    const int ncand = cells ? 27 : 1;
    // FP32 box constants once (converting them per candidate occupies the FP64 pipe)
    const float bx = (float)a.cl.c[0], by = (float)a.cl.c[4], bz = (float)a.cl.c[8];
    const float ibx = (float)a.cl.inv[0], iby = (float)a.cl.inv[1], ibz = (float)a.cl.inv[2];
    // four passes: polarizable j > i, polarizable j < i, the others j > i, the others j < i
    // (the dipole tensors are kept for the polarizable partners only)
    int c1 = 0, c2 = 0, c3 = 0;
    for (int pass = 0; pass < 4; ++pass) {
        if (pass == 1) c1 = cnt;
        if (pass == 2) c2 = cnt;
        if (pass == 3) c3 = cnt;
        const bool polpass = pass < 2, uppass = pass % 2 == 0;
        for (int c = 0; c < ncand; ++c) {
            int beg = 0, end = a.n;
            if (cells) {
                const int cx = pol_wrap(a.x[i] * a.cl.inv[0], nc.x), cy = pol_wrap(a.y[i] * a.cl.inv[1], nc.y),
                          cz = pol_wrap(a.z[i] * a.cl.inv[2], nc.z);
                const int ox = c % 3 - 1, oy = (c / 3) % 3 - 1, oz = c / 9 - 1;
                const int cc = (((cz + oz + nc.z) % nc.z) * nc.y + (cy + oy + nc.y) % nc.y) * nc.x + (cx + ox + nc.x) % nc.x;
                beg = cstart[cc];
                end = cend[cc];
            }
            for (int b = beg; b < end; b += 32) {
                const int q = b + lane;
                bool hit = false;
                int j = 0;
                if (q < end) {
                    j = cells ? sidx[q] : q;
                    bool near = false, inside = false;
                    if (j != i && site_mol(a, j) != mi && (a.polr2[j] > 1e-6) == polpass && (j > i) == uppass) {
                        const float4 pj = xf[j];
                        float d2;
                        if (cells) {   // orthorhombic
                            float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                            dx -= bx * rintf(dx * ibx);
                            dy -= by * rintf(dy * iby);
                            dz -= bz * rintf(dz * ibz);
                            d2 = dx * dx + dy * dy + dz * dz;
                        } else {
                            d2 = dist2_img_f(a.cl, pi, pj);
                        }
                        near = d2 < r2f;
                        inside = d2 < r2in;
                    }
                    if (inside) {
                        hit = true;
                    } else if (near) {
                        double dx, dy, dz;
                        sep(a, i, j, dx, dy, dz);
                        const double r2 = norm2(dx, dy, dz);
                        // the reference's test; the root only where rounding could decide it
                        hit = lc2 > r2 || (r2 < lc2 * (1.0 + 1e-14) && lc > __dsqrt_rn(r2));
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int slot = cnt + __popc(bal & ((1u << lane) - 1u));
                    if (slot < rowcap) my[slot] = j;
                }
                cnt += __popc(bal);
            }
        }
    }
    if (lane == 0) {
        nn[i] = min(cnt, rowcap);
        npol[i] = min(c2, rowcap);
        nup[i] = make_int2(min(c1, rowcap), min(c3, rowcap) - min(c2, rowcap));
        if (cnt > rowcap) atomicOr(flag, 1);
    }
}

// Verlet list with a skin (SOURCE/parlst.f with the rebuild test of SOURCE/centroid_vertest.f):
// the pairs within rcut + delr are kept between calls and the list is rebuilt once a site
// has moved more than delr / 2 since the build (flag set).
__global__ void k_pol_moved(int n, const double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ z, const double* __restrict__ xref, Cell cl, double half2,
                            int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double dx = x[i] - xref[i], dy = y[i] - xref[n + i], dz = z[i] - xref[2 * (size_t)n + i];
    image(cl, dx, dy, dz);
    if (dx * dx + dy * dy + dz * dz > half2) atomicOr(flag, 1);
}

__global__ void k_pol_ref(int n, const double* __restrict__ x, const double* __restrict__ y,
                          const double* __restrict__ z, double* __restrict__ xref) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    xref[i] = x[i];
    xref[n + i] = y[i];
    xref[2 * (size_t)n + i] = z[i];
}

// The exact list from the skin list: each row's pairs within rcut, tested as k_pol_list does
// (FP32 with margins, the reference's FP64 test in the shell around the cut), in the skin
// list's order.
__global__ void k_pol_filter(PolArgs a, const int* __restrict__ nn_s, const int* __restrict__ nbr_s,
                             const int* __restrict__ npol_s, const int2* __restrict__ nup_s, int cap_s,
                             int* __restrict__ nn, int* __restrict__ nbr, int* __restrict__ npol,
                             int2* __restrict__ nup, const float4* __restrict__ xf, float r2f, float r2in,
                             int* __restrict__ flag) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.n) return;
    const float4 pi = xf[i];
    // the skin row's segments (k_pol_list): [0, up.x) polarizable j > i, [up.x, mp) polarizable
    // j < i, [mp, mp + up.y) the others j > i, then the others j < i; kept in order
    const int m = nn_s[i], mp = npol_s[i];
    const int2 up = nup_s[i];
    int cntp = 0, cntu = 0, cntn = 0;
    const int* src = nbr_s + (size_t)i * cap_s;
    int* my = nbr + (size_t)i * a.cap;
    const bool ortho = a.cl.imcon == 1 || a.cl.imcon == 2;
    const float bx = (float)a.cl.c[0], by = (float)a.cl.c[4], bz = (float)a.cl.c[8];
    const float ibx = (float)a.cl.inv[0], iby = (float)a.cl.inv[1], ibz = (float)a.cl.inv[2];
    int cnt = 0;
    // two 32-entry chunks per step: both chunks' index and position loads are issued
    // before the first test
    int jn = lane < m ? src[lane] : 0;
    float4 pn = lane < m ? xf[jn] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int b = 0; b < m; b += 32) {
        const int q = b + lane;
        bool hit = false;
        const int j = jn;
        const float4 pj = pn;
        if (q + 32 < m) {   // the next chunk's loads, in flight during this chunk's tests
            jn = src[q + 32];
            pn = xf[jn];
        }
        if (q < m) {
            float d2;
            if (ortho) {
                float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                dx -= bx * rintf(dx * ibx);
                dy -= by * rintf(dy * iby);
                dz -= bz * rintf(dz * ibz);
                d2 = dx * dx + dy * dy + dz * dz;
            } else {
                d2 = dist2_img_f(a.cl, pi, pj);
            }
            if (d2 < r2in) {
                hit = true;
            } else if (d2 < r2f) {
                double dx, dy, dz;
                sep(a, i, j, dx, dy, dz);
                const double r2 = norm2(dx, dy, dz);
                hit = a.rcsq > r2 || (r2 < a.rcsq * (1.0 + 1e-14) && a.rcut > __dsqrt_rn(r2));
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int slot = cnt + __popc(bal & ((1u << lane) - 1u));
            if (slot < a.cap) my[slot] = j;
        }
        cnt += __popc(bal);
        // hits among the first B entries of the skin row, for the segment ends B
        auto below = [&](int B) {
            const int l = min(32, max(0, B - b));
            return __popc(bal & (l == 32 ? 0xffffffffu : ((1u << l) - 1u)));
        };
        cntu += below(up.x);
        cntp += below(mp);
        cntn += below(mp + up.y) - below(mp);
    }
    if (lane == 0) {
        nn[i] = min(cnt, a.cap);
        npol[i] = min(cntp, a.cap);
        nup[i] = make_int2(min(cntu, a.cap), min(cntp + cntn, a.cap) - min(cntp, a.cap));
        if (cnt > a.cap) atomicOr(flag, 1);
    }
}

// polr^(1/6) per site and its reciprocal (n further), once per call (the pair kernels
// multiply two of them).
__global__ void k_pol_polr6(PolArgs a, double* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < a.n) {
        const double p6 = pow(a.polr[j], 1.0 / 6.0);
        out[j] = p6;
        out[a.n + j] = 1.0 / p6;
    }
}

// --- static real-space field and dipole tensors ---------------------------------------
// rfield's first pass per pair (SOURCE/rfield.f:59-201): the charge field q_j (B_1 + 1/r^3
// - exp(-a_cd (r/bb)^4) / r^3) r, and for the polarizable partners the dipole tensor
// r r^T A - B I with A = 3/r^5 + B_2 and B = 1/r^3 + B_1, less its Thole damping (h1, h2 of
// exp(-a_dd (r/bb)^4)).  The damping is nonzero within ~3.5 A (charge) and ~5.5 A (dipole)
// only, a few pairs of a row of ~400, but one lane that needs the FP64 exp makes its whole
// warp execute it: so every lane first adds its pair's undamped field and writes its
// undamped tensor, and the damped pairs are queued per warp (their slots in the row) and
// evaluated 32 at a time, their damping subtracted from the field sum and from the tensor
// written before (read back and rewritten by the same warp).
__device__ __forceinline__ void static_damp(const PolArgs& a, int i, int k, size_t row, size_t blk, int np,
                                            double rpi, double e[3]) {
    const int j = a.nbr[row + k];
    double d[3];
    sep(a, i, j, d[0], d[1], d[2]);
    const double r2 = norm2(d[0], d[1], d[2]);
    const double rri = rsqrt_nr(r2);
    const double rr = r2 * rri;
    const double r3i = rri * rri * rri, r5i = r3i * rri * rri;
    const double u = pow4(rr * (rpi * a.rpolr6[j]));
    const double arq = a.ascd * u;
    if (arq < kDampCut) {
        const double f = kR4pie0 * a.q[j] * exp(-arq) * r3i;
        e[0] -= f * d[0];
        e[1] -= f * d[1];
        e[2] -= f * d[2];
    }
    if (k >= np) return;
    const double arob4 = a.athole * u;
    const bool dd = arob4 < kDampCut;
    const double h1 = dd ? exp(-arob4) : 0.0;
    const double h2 = (1.0 + (4.0 / 3.0) * arob4) * h1;
    const double C = 3.0 * kR4pie0 * r5i * h2, D = kR4pie0 * h1 * r3i;
    const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        double t = a.tens[p * blk + row + k];
        if (dd) {
            const double rirj = d[ia[p]] * d[ib[p]];
            t -= ia[p] == ib[p] ? fma(rirj, C, -D) : rirj * C;
            a.tens[p * blk + row + k] = t;
        }
        if (a.tens32) a.tens32[p * blk + row + k] = (float)t;   // not written by the first pass
    }
}

__global__ void __launch_bounds__(kThreads) k_pol_static(PolArgs a) {
    __shared__ int dq[kThreads / 32][64];   // per warp: row slots of the damped pairs
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.n) return;
    // the static field is read only at sites that carry a dipole (iter, the residual,
    // coulomb_polar): the rows of the others (the M sites) are skipped
    if (!(a.polr2[i] > a.toler) && !(a.polr2[i] > 1e-6)) {
        if (lane < 3) a.efk[lane * (size_t)a.n + i] = 0.0;
        return;
    }
    const int nn = a.nn[i];
    const size_t row = (size_t)i * a.cap, blk = (size_t)a.n * a.cap;
    const bool poli = a.polr2[i] > 1e-6;
    const int np = poli ? a.npol[i] : 0;   // tensors of the polarizable partners (the row's first np)
    const double rpi = a.rpolr6[i];
    int* q = dq[threadIdx.x >> 5];
    int qn = 0;                            // queued pairs (warp-uniform)
    double e[3] = {0, 0, 0};
    for (int base = 0; base < nn; base += 32) {
        const int k = base + lane;
        bool damped = false;
        if (k < nn) {
            const int j = a.nbr[row + k];
            double d[3];
            sep(a, i, j, d[0], d[1], d[2]);
            const double r2 = norm2(d[0], d[1], d[2]);
            // one reciprocal root gives r, 1/r^2, 1/r^3 and 1/r^5; the table index and the
            // Thole arguments multiply by reciprocals (FP64 divisions are the costliest
            // FP64-pipe operations of this kernel)
            const double rri = rsqrt_nr(r2);
            const double rr = r2 * rri;
            double t[6] = {0, 0, 0, 0, 0, 0};
            if (a.rcut > rr) {
                double bbb[4];
                interp_r(a, rr, bbb);
                const double rsqi = rri * rri, r3i = rsqi * rri, r5i = r3i * rsqi;
                const double eki = kR4pie0 * a.q[j] * (bbb[1] + r3i);
                e[0] += eki * d[0];
                e[1] += eki * d[1];
                e[2] += eki * d[2];
                const double u = pow4(rr * (rpi * a.rpolr6[j]));   // (r / bb)^4
                damped = a.ascd * u < kDampCut || (k < np && a.athole * u < kDampCut);
                if (k < np) {
                    const double A = kR4pie0 * (3.0 * r5i + bbb[2]), B = kR4pie0 * (r3i + bbb[1]);
                    const double ax = A * d[0], ay = A * d[1], az = A * d[2];
                    t[0] = fma(ax, d[0], -B);
                    t[1] = ax * d[1];
                    t[2] = ax * d[2];
                    t[3] = fma(ay, d[1], -B);
                    t[4] = ay * d[2];
                    t[5] = fma(az, d[2], -B);
                }
            }
            if (k < np) {
#pragma unroll
                for (int p = 0; p < 6; ++p) a.tens[p * blk + row + k] = t[p];
                // a damped pair's FP32 copy is written with its damping
                if (a.tens32 && !damped)
                    for (int p = 0; p < 6; ++p) a.tens32[p * blk + row + k] = (float)t[p];
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, damped);
        if (damped) q[qn + __popc(bal & ((1u << lane) - 1u))] = k;
        qn += __popc(bal);
        if (qn >= 32) {   // a full warp of damped pairs
            __syncwarp();
            static_damp(a, i, q[lane], row, blk, np, rpi, e);
            __syncwarp();
            if (lane < qn - 32) q[lane] = q[32 + lane];
            qn -= 32;
            __syncwarp();
        }
    }
    __syncwarp();
    if (lane < qn) static_damp(a, i, q[lane], row, blk, np, rpi, e);
    for (int c = 0; c < 3; ++c) e[c] = warp_sum(e[c]);
    if (lane == 0) {
        a.efk[i] = e[0];
        a.efk[a.n + i] = e[1];
        a.efk[2 * a.n + i] = e[2];
    }
}

// Intramolecular (excluded) pairs: static charge field and the three O/H dipole tensors.
// One thread per excluded pair (6 per water); the field sums by atomics.
__global__ void k_pol_intra_static(PolArgs a) {
    const int tt = blockIdx.x * blockDim.x + threadIdx.x;
    if (tt >= 6 * a.nw) return;
    const int w = tt / 6, p = tt % 6;
    const int o = 3 * w, m = 3 * a.nw + w;
    const int pr[6][2] = {{o, o + 1}, {o, o + 2}, {o + 1, o + 2}, {o, m}, {o + 1, m}, {o + 2, m}};
    double* T = a.intra + 18 * (size_t)w;
    {
        const int i = pr[p][0], j = pr[p][1];
        double d[3];
        sep(a, i, j, d[0], d[1], d[2]);
        const double r2 = norm2(d[0], d[1], d[2]);
        const double rr = __dsqrt_rn(r2);
        const double rri = 1.0 / rr, rsqi = 1.0 / r2, r3i = 1.0 / (rr * r2), r5i = r3i * rsqi;
        double bbb[4];
        bfun_exact(a.alpha, rr, rri, rsqi, bbb);
        const double eki = kR4pie0 * a.q[j] * bbb[1] / a.eps, ekj = kR4pie0 * a.q[i] * bbb[1] / a.eps;
        for (int c = 0; c < 3; ++c) {
            atomicAdd(a.efk + c * a.n + i, eki * d[c]);
            atomicAdd(a.efk + c * a.n + j, -ekj * d[c]);
        }
        if (p < 3) {
            double t[6] = {0, 0, 0, 0, 0, 0};
            if (a.polr2[i] > 1e-6 && a.polr2[j] > 1e-6) {
                const double bb = pow(a.polr[i] * a.polr[j], 1.0 / 6.0);
                const double ath = (i % 3 == 0 || j % 3 == 0) ? a.athole12 : a.athole13;
                const double arob4 = ath * pow4(rr / bb);
                const double h1 = exp(-arob4);
                const double h2 = (1.0 + (4.0 / 3.0) * arob4) * h1;
                const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
                for (int q = 0; q < 6; ++q) {
                    const double rirj = d[ia[q]] * d[ib[q]];
                    const bool dg = ia[q] == ib[q];
                    double v = dg ? rirj * bbb[2] - bbb[1] : rirj * bbb[2];
                    v = dg ? v + 3.0 * rirj * r5i - r3i : v + 3.0 * rirj * r5i;
                    v = dg ? v - 3.0 * rirj * r5i * h2 + h1 * r3i : v - 3.0 * rirj * r5i * h2;
                    t[q] = v * (kR4pie0 / a.eps);
                }
            }
            for (int q = 0; q < 6; ++q) T[6 * p + q] = t[q];
            for (int q = 0; q < 6; ++q) a.intra32[18 * (size_t)w + 6 * p + q] = (float)t[q];
        }
    }
}

// --- dipole field of the real-space pairs ------------------------------------------------
__global__ void k_pol_dd(PolArgs a) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.n) return;
    double e[3] = {0, 0, 0};
    if (a.polr2[i] > 1e-6) {
        const int nn = a.npol[i];   // the other partners carry no dipole
        const size_t row = (size_t)i * a.cap, blk = (size_t)a.n * a.cap;
        // two entries per lane and step (the loads of both in flight together), as k_pol_dd32
        for (int k = lane; k < nn; k += 64) {
            const bool two = k + 32 < nn;
            const int j0 = a.nbr[row + k], j1 = two ? a.nbr[row + k + 32] : j0;
            double t0[6], t1[6];
#pragma unroll
            for (int p = 0; p < 6; ++p) {
                t0[p] = a.tens[p * blk + row + k];
                t1[p] = two ? a.tens[p * blk + row + k + 32] : 0.0;
            }
            const double m0[3] = {a.mx[j0], a.my[j0], a.mz[j0]}, m1[3] = {a.mx[j1], a.my[j1], a.mz[j1]};
            e[0] += t0[0] * m0[0] + t0[1] * m0[1] + t0[2] * m0[2];
            e[1] += t0[1] * m0[0] + t0[3] * m0[1] + t0[4] * m0[2];
            e[2] += t0[2] * m0[0] + t0[4] * m0[1] + t0[5] * m0[2];
            e[0] += t1[0] * m1[0] + t1[1] * m1[1] + t1[2] * m1[2];
            e[1] += t1[1] * m1[0] + t1[3] * m1[1] + t1[4] * m1[2];
            e[2] += t1[2] * m1[0] + t1[4] * m1[1] + t1[5] * m1[2];
        }
        for (int c = 0; c < 3; ++c) e[c] = warp_sum(e[c]);
        if (lane == 0 && i < 3 * a.nw) {
            const int w = i / 3, s = i % 3;
            // pairs 0 (O,H1), 1 (O,H2), 2 (H1,H2)
            const int pj[3][2] = {{1, 2}, {0, 2}, {0, 1}};   // partner sites of s
            const int pp[3][2] = {{0, 1}, {0, 2}, {1, 2}};   // their pair index
            const double* T = a.intra + 18 * (size_t)w;
            for (int u = 0; u < 2; ++u) {
                const int j = 3 * w + pj[s][u];
                const double* t = T + 6 * pp[s][u];
                const double mj[3] = {a.mx[j], a.my[j], a.mz[j]};
                e[0] += t[0] * mj[0] + t[1] * mj[1] + t[2] * mj[2];
                e[1] += t[1] * mj[0] + t[3] * mj[1] + t[4] * mj[2];
                e[2] += t[2] * mj[0] + t[4] * mj[1] + t[5] * mj[2];
            }
        }
    }
    if (lane == 0) {
        a.emu[i] = e[0];
        a.emu[a.n + i] = e[1];
        a.emu[2 * a.n + i] = e[2];
    }
}

// --- k space ------------------------------------------------------------------------------
struct KArgs {
    int K, n, kmax[3];
    const double4* kv;     // kx, ky, kz, akk
    const double2* kx2;    // rksq, akv2
    const int4* lmn;
    double2* fac;          // per-site phase factors exp(2 pi i l s): x (l = 0..kmax1), y, z (-kmax..kmax)
    double2* eik;          // exp(ik.r) [k * n + j] = (cos, sin)
    float2* fac32;         // the per-site axis factors in FP32 (mixed precision), or null
    const int4* ktile;     // per kSfThreads k vectors: first (l, m) column, columns (FP32 structure factors)
    const int4* kaux;      // per k: column within its tile, next column (l << 16 | y row), column, z offset
    const int* kcol;       // per (l, m) column: l << 16 | y row
    const int2* colk;      // per (l, m) column: first k vector, count
    float* kco32;          // 16 per k: the CG gather's kx, ky, kz, akk k.Ds, akk k.Dc, then the FP32 force gather's
    double* sf;            // 8 per k: ckcs, ckss, Mc(3), Ms(3)
    double* kco;           // 16 per k: coefficients of the gathers
    double* kterm;         // 16 per k (final pass): engc, engdum, omg 11 22 33 12 13 23, jpot(3)
    const double4* md;     // dipoles of the polarizable sites (0 elsewhere)
    const double* q;       // site charges
    const double* vh;      // per-site products of the heat sums: q v (3 blocks of n), mu_c v_b (9 blocks)
    double rc[9];
    double scale, ralph, sfac;   // 4 rvolm r4pie0 / epsq, -1 / (4 alpha^2), 2 rvolm r4pie0 / epsq
    const int* stop = nullptr;   // the CG sweeps' FP32 kernels: nonzero state = return at once
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// exp(2 pi i l s) for the fractional coordinates of each site and every l of each axis
__global__ void k_pol_factors(KArgs k, const double* __restrict__ x, const double* __restrict__ y,
                              const double* __restrict__ z) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.n) return;
    const double s3[3] = {k.rc[0] * x[j] + k.rc[3] * y[j] + k.rc[6] * z[j],
                          k.rc[1] * x[j] + k.rc[4] * y[j] + k.rc[7] * z[j],
                          k.rc[2] * x[j] + k.rc[5] * y[j] + k.rc[8] * z[j]};
    int off = 0;
    for (int ax = 0; ax < 3; ++ax) {
        const int lo = ax == 0 ? 0 : -k.kmax[ax];
        for (int l = lo; l <= k.kmax[ax]; ++l) {
            const double t = (double)l * s3[ax];
            double sn, cs;
            sincospi(2.0 * (t - rint(t)), &sn, &cs);
            k.fac[(size_t)(off + l - lo) * k.n + j] = make_double2(cs, sn);
            if (k.fac32) k.fac32[(size_t)(off + l - lo) * k.n + j] = make_float2((float)cs, (float)sn);
        }
        off += k.kmax[ax] - lo + 1;
    }
}

// exp(ik.r_j) = (fx_l fy_m) fz_n per (l, m) column (blockIdx.x) and site: the product
// fx_l fy_m once per column and site, then one complex product per k vector.
__global__ void k_pol_phase(KArgs k) {
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    if (j >= k.n) return;
    const int2 ck = k.colk[blockIdx.x];   // first k vector, count
    const int c = k.kcol[blockIdx.x];
    const int oz = k.kmax[0] + 2 * k.kmax[1] + 2 + k.kmax[2];
    const double2 fxy = cmul(k.fac[(size_t)(c >> 16) * k.n + j], k.fac[(size_t)(c & 0xffff) * k.n + j]);
    for (int q = 0; q < ck.y; ++q) {
        const int kk = ck.x + q;
        const double2 fz = k.fac[(size_t)(oz + k.lmn[kk].z) * k.n + j];
        k.eik[(size_t)kk * k.n + j] = cmul(fxy, fz);
    }
}

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double* out) {
    __shared__ double red[kSfThreads / 32][NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const double s = warp_sum(v[q]);
        if (lane == 0) red[w][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int i = 0; i < kSfThreads / 32; ++i) s += red[i][threadIdx.x];
        out[threadIdx.x] = s;
    }
}

__global__ void k_pol_mask(PolArgs a, double4* __restrict__ md) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    md[j] = a.polr2[j] > 1e-6 ? make_double4(a.mx[j], a.my[j], a.mz[j], 0.0) : make_double4(0, 0, 0, 0);
}

// Charge structure factors (fixed for the call): ckcs, ckss per k vector.
__global__ void __launch_bounds__(kSfThreads) k_pol_sfq(KArgs k, const double* __restrict__ q) {
    const int kk = blockIdx.x;
    const double2* e = k.eik + (size_t)kk * k.n;
    double v[2] = {0, 0};
    for (int j = threadIdx.x; j < k.n; j += kSfThreads) {
        const double2 cs = e[j];
        v[0] += q[j] * cs.x;
        v[1] += q[j] * cs.y;
    }
    __shared__ double tot[2];
    block_reduce_store<2>(v, tot);
    __syncthreads();
    if (threadIdx.x < 2) k.sf[8 * (size_t)kk + threadIdx.x] = tot[threadIdx.x];
}

// Dipole structure factors of one k vector and the coefficients of the field gather.
__global__ void __launch_bounds__(kSfThreads) k_pol_sfd(KArgs k) {
    const int kk = blockIdx.x;
    const double2* e = k.eik + (size_t)kk * k.n;
    double v[6] = {0, 0, 0, 0, 0, 0};
    for (int j = threadIdx.x; j < k.n; j += kSfThreads) {
        const double2 cs = e[j];
        const double4 m = k.md[j];
        v[0] += cs.x * m.x; v[1] += cs.x * m.y; v[2] += cs.x * m.z;
        v[3] += cs.y * m.x; v[4] += cs.y * m.y; v[5] += cs.y * m.z;
    }
    __shared__ double tot[6];
    block_reduce_store<6>(v, tot);
    __syncthreads();
    if (threadIdx.x == 0) {
        double* sf = k.sf + 8 * (size_t)kk;
        for (int c = 0; c < 6; ++c) sf[2 + c] = tot[c];
        const double4 kv = k.kv[kk];
        const double skc = kv.x * tot[0] + kv.y * tot[1] + kv.z * tot[2];
        const double sks = kv.x * tot[3] + kv.y * tot[4] + kv.z * tot[5];
        double* c = k.kco + 16 * (size_t)kk;
        c[0] = kv.x; c[1] = kv.y; c[2] = kv.z;
        c[3] = kv.w * sks;      // dipole field: -k akk (s k.Ms + c k.Mc)
        c[4] = kv.w * skc;
        c[5] = kv.w * sf[0];    // static field: -k akk (-s ckcs + c ckss)
        c[6] = kv.w * sf[1];
    }
}

// Per k vector, from its 6 (NV = 6) or 30 (NV = 30, with velocities) structure-factor sums:
// the final dipole structure factors, the k vector's energy, virial and heat-current terms
// (SOURCE/ewald1p.f:575-733) and the coefficients of the force gather.
template <int HEAT>
__device__ __forceinline__ void final_k(const KArgs& k, int kk, const double* tot) {
    double* sf = k.sf + 8 * (size_t)kk;
    for (int c = 0; c < 6; ++c) sf[2 + c] = tot[c];
    const double4 kv = k.kv[kk];
    const double2 k2 = k.kx2[kk];
    const double kx[3] = {kv.x, kv.y, kv.z};
    const double ckcs = sf[0], ckss = sf[1];
    const double Mc[3] = {tot[0], tot[1], tot[2]}, Ms[3] = {tot[3], tot[4], tot[5]};
    const double skc = kx[0] * Mc[0] + kx[1] * Mc[1] + kx[2] * Mc[2];
    const double sks = kx[0] * Ms[0] + kx[1] * Ms[1] + kx[2] * Ms[2];
    const double s1 = ckcs - sks, s2 = ckss + skc;
    const double akk = kv.w, akv = 2.0 * akk * (1.0 / k2.x - k.ralph), akv2 = k2.y;
    const double s12 = s1 * s1 + s2 * s2;
    const double virprs = akv * s12;
    double* t = k.kterm + 16 * (size_t)kk;
    t[0] = akk * (ckcs * ckcs + ckss * ckss);
    t[1] = akk * s12;
    const int oa[6] = {0, 1, 2, 0, 0, 1}, ob[6] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; ++q)
        t[2 + q] = -virprs * kx[oa[q]] * kx[ob[q]] - 2.0 * akk * kx[oa[q]] * Ms[ob[q]] * s1 +
                   2.0 * akk * kx[oa[q]] * Mc[ob[q]] * s2;
    t[8] = t[9] = t[10] = 0.0;
    if (HEAT) {
        const double* V1 = tot + 6;
        const double* V2 = tot + 9;
        const double* W1 = tot + 12;
        const double* W2 = tot + 21;
        double kW1[3], kW2[3], P[3];
        for (int b = 0; b < 3; ++b) {
            kW1[b] = kx[0] * W1[b] + kx[1] * W1[3 + b] + kx[2] * W1[6 + b];
            kW2[b] = kx[0] * W2[b] + kx[1] * W2[3 + b] + kx[2] * W2[6 + b];
            P[b] = s1 * V1[b] + s2 * kW1[b] + s2 * V2[b] - s1 * kW2[b];
        }
        const double kp = kx[0] * P[0] + kx[1] * P[1] + kx[2] * P[2];
        double Q[3][3];   // Q[b'][b] = sum_j Y_jb' v_jb
        for (int bp = 0; bp < 3; ++bp)
            for (int b = 0; b < 3; ++b)
                Q[bp][b] = -Ms[bp] * V1[b] + s2 * W1[3 * bp + b] + Mc[bp] * kW1[b] + Mc[bp] * V2[b] -
                           s1 * W2[3 * bp + b] + Ms[bp] * kW2[b];
        const double f = k.sfac * akk;
        for (int aa = 0; aa < 3; ++aa) {
            double y = 0.0;
            for (int b = 0; b < 3; ++b) {
                const int lo = aa < b ? aa : b, hi = aa < b ? b : aa;
                y += kx[lo] * Q[hi][b];
            }
            t[8 + aa] = f * (P[aa] - akv2 * kx[aa] * kp + y);
        }
    }
    // coefficients of the force gather: k, akk summu1, akk summu2, akk ckcs, akk ckss,
    // akk k.Mc, akk k.Ms
    double* c = k.kco + 16 * (size_t)kk;
    c[0] = kx[0]; c[1] = kx[1]; c[2] = kx[2];
    c[3] = akk * s1; c[4] = akk * s2; c[5] = akk * ckcs; c[6] = akk * ckss; c[7] = akk * skc; c[8] = akk * sks;
    if (k.kco32) {
        float* f = k.kco32 + 16 * (size_t)kk;
        for (int q = 0; q < 9; ++q) f[q] = (float)c[q];
    }
}

// Final structure factors (dipoles, and with velocities the 24 sums of the ew1p
// per-atom stress contraction), the k vector's energy, virial and heat-current terms
// (SOURCE/ewald1p.f:575-733) and the coefficients of the force gather.
template <int HEAT>
__global__ void __launch_bounds__(kSfThreads) k_pol_sf_final(KArgs k) {
    constexpr int NV = HEAT ? 30 : 6;
    const int kk = blockIdx.x;
    const double2* e = k.eik + (size_t)kk * k.n;
    double v[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = 0.0;
    for (int j = threadIdx.x; j < k.n; j += kSfThreads) {
        const double2 cs = e[j];
        const double4 m = k.md[j];
        v[0] += cs.x * m.x; v[1] += cs.x * m.y; v[2] += cs.x * m.z;
        v[3] += cs.y * m.x; v[4] += cs.y * m.y; v[5] += cs.y * m.z;
        if (HEAT) {
            // per-site products q v (3) and mu_c v_b (9), rows of k.vh
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const double qv = k.vh[(size_t)b * k.n + j];
                v[6 + b] += cs.x * qv;    // V1
                v[9 + b] += cs.y * qv;    // V2
            }
#pragma unroll
            for (int cb = 0; cb < 9; ++cb) {
                const double mv = k.vh[(size_t)(3 + cb) * k.n + j];
                v[12 + cb] += cs.x * mv;   // W1[c][b]
                v[21 + cb] += cs.y * mv;   // W2[c][b]
            }
        }
    }
    __shared__ double tot[NV];
    block_reduce_store<NV>(v, tot);
    __syncthreads();
    if (threadIdx.x == 0) final_k<HEAT>(k, kk, tot);
}

// k-space fields per site (iflag 0): the dipole field and, in the first pass, the static
// charge field.  Blocks split the sites (two per thread) and the k vectors (blockIdx.y
// chunks of kchunk); each writes its partial sums, which k_pol_kfield_sum adds in order.
__global__ void __launch_bounds__(kThreads) k_pol_kfield(KArgs k, int first, int kchunk, double* __restrict__ part) {
    __shared__ double sh[kKTile][8];
    const int j0 = blockIdx.x * 2 * blockDim.x + threadIdx.x, j1 = j0 + blockDim.x;
    const bool in0 = j0 < k.n, in1 = j1 < k.n;
    const int kb = blockIdx.y * kchunk, ke = min(k.K, kb + kchunk);
    double em0[3] = {0, 0, 0}, ec0[3] = {0, 0, 0}, em1[3] = {0, 0, 0}, ec1[3] = {0, 0, 0};
    for (int t0 = kb; t0 < ke; t0 += kKTile) {
        const int nt = min(kKTile, ke - t0);
        __syncthreads();
        for (int u = threadIdx.x; u < nt * 8; u += blockDim.x) sh[u >> 3][u & 7] = k.kco[16 * (size_t)(t0 + (u >> 3)) + (u & 7)];
        __syncthreads();
        const double2* e = k.eik + (size_t)t0 * k.n;
        for (int u = 0; u < nt; ++u, e += k.n) {
            const double* c = sh[u];
            if (in0) {
                const double2 cs = e[j0];
                const double vv = cs.y * c[3] + cs.x * c[4];
                em0[0] -= c[0] * vv; em0[1] -= c[1] * vv; em0[2] -= c[2] * vv;
                if (first) {
                    const double tt = -cs.y * c[5] + cs.x * c[6];
                    ec0[0] -= c[0] * tt; ec0[1] -= c[1] * tt; ec0[2] -= c[2] * tt;
                }
            }
            if (in1) {
                const double2 cs = e[j1];
                const double vv = cs.y * c[3] + cs.x * c[4];
                em1[0] -= c[0] * vv; em1[1] -= c[1] * vv; em1[2] -= c[2] * vv;
                if (first) {
                    const double tt = -cs.y * c[5] + cs.x * c[6];
                    ec1[0] -= c[0] * tt; ec1[1] -= c[1] * tt; ec1[2] -= c[2] * tt;
                }
            }
        }
    }
    double* p = part + (size_t)blockIdx.y * 6 * k.n;
    for (int c = 0; c < 3; ++c) {
        if (in0) {
            p[c * (size_t)k.n + j0] = em0[c];
            p[(3 + c) * (size_t)k.n + j0] = ec0[c];
        }
        if (in1) {
            p[c * (size_t)k.n + j1] = em1[c];
            p[(3 + c) * (size_t)k.n + j1] = ec1[c];
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_pol_kfield_sum(KArgs k, PolArgs a, int first, int nchunk,
                                                             const double* __restrict__ part) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.n) return;
    double em[3] = {0, 0, 0}, ec[3] = {0, 0, 0};
    for (int q = 0; q < nchunk; ++q) {
        const double* p = part + (size_t)q * 6 * k.n;
        for (int c = 0; c < 3; ++c) {
            em[c] += p[c * (size_t)k.n + j];
            if (first) ec[c] += p[(3 + c) * (size_t)k.n + j];
        }
    }
    const double dum = 4.0 * kR4pie0 * (a.alpha * a.alpha * a.alpha) / kSqrpi / 3.0;
    const bool pol = a.polr2[j] > 1e-6;
    const double m[3] = {a.mx[j], a.my[j], a.mz[j]};
    for (int c = 0; c < 3; ++c) {
        if (first) a.efc[c * k.n + j] = k.scale * ec[c];
        a.efm[c * k.n + j] = (pol ? k.scale * em[c] : 0.0) + dum * m[c];
    }
}

// iter (SOURCE/iter.f): SOR update of the dipoles; sum of squared changes and count;
// refreshes the masked dipoles of the structure factors.
// With dlt (mixed precision) the update of the masked dipoles is also written in FP32.
__global__ void __launch_bounds__(kThreads) k_pol_iter(PolArgs a, double4* __restrict__ md, float4* __restrict__ dlt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0, 0};
    if (dlt && i < a.n) dlt[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < a.n && a.polr2[i] > a.toler) {
        const double oldfac = a.omega, fac = 1.0 - oldfac;
        double* m[3] = {a.mx + i, a.my + i, a.mz + i};
        double dd = 0.0, nm[3];
        for (int c = 0; c < 3; ++c) {
            const double o = *m[c];
            const double f = a.efk[c * a.n + i] + a.emu[c * a.n + i] + a.efm[c * a.n + i] + a.efc[c * a.n + i] + 0.0;
            const double nv = oldfac * o + fac * a.polr2[i] * f / kR4pie0;
            *m[c] = nv;
            nm[c] = nv;
            dd += (nv - o) * (nv - o);
        }
        if (a.polr2[i] > 1e-6) {
            if (dlt) {
                const double4 o = md[i];
                dlt[i] = make_float4((float)(nm[0] - o.x), (float)(nm[1] - o.y), (float)(nm[2] - o.z), 0.f);
            }
            md[i] = make_double4(nm[0], nm[1], nm[2], 0.0);
        }
        v[0] = dd;
        v[1] = 1.0;
    }
    block_sum_atomic<2>(v, a.acc + 27);
}

// --- mixed precision: FP32 correction solves under FP64 refinement -----------------------
struct MixArgs {
    float4* r32;      // FP64 residual, rounded (polarizable sites; 0 elsewhere)
    float4* d32;      // vector the FP32 field is evaluated for (the CG direction)
    float* e32;       // FP32 field of d32: real space (3 blocks of n), then k space (3 blocks)
    float4 *x, *rho, *q;   // CG: solution, residual, A d32
    const int* stop = nullptr;   // CG state on the device (nonzero: the sweep kernels return at once)
};

// FP64 residual of the dipole equations at the current dipoles: r = polr2 E / r4pie0 - mu
// with E the four fields of the last FP64 evaluation; rounds it for the FP32 solve and
// clears the correction.  Sums |r|^2, the count and |mu|^2 into acc[29..31].
__global__ void __launch_bounds__(kThreads) k_pol_resid(PolArgs a, MixArgs m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0, 0, 0};
    if (i < a.n) {
        float4 r = make_float4(0, 0, 0, 0);
        if (a.polr2[i] > a.toler) {
            double rr[3];
            const double mu[3] = {a.mx[i], a.my[i], a.mz[i]};
            for (int c = 0; c < 3; ++c) {
                const double f = a.efk[c * a.n + i] + a.emu[c * a.n + i] + a.efm[c * a.n + i] + a.efc[c * a.n + i] + 0.0;
                rr[c] = a.polr2[i] * f / kR4pie0 - mu[c];
            }
            v[0] = rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2];
            v[1] = 1.0;
            v[2] = mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2];
            r = make_float4((float)rr[0], (float)rr[1], (float)rr[2], 0.f);
        }
        m.r32[i] = r;
        m.d32[i] = make_float4(0, 0, 0, 0);
    }
    block_sum_atomic<3>(v, a.acc + 29);
}

// FP32 real-space dipole field (warp per site) of `in`, written to `out` (3 blocks of n).
__global__ void k_pol_dd32(PolArgs a, const float4* __restrict__ in, float* __restrict__ out,
                           const int* __restrict__ stop = nullptr) {
    if (stop && *stop) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.n) return;
    float e[3] = {0, 0, 0};
    if (a.polr2[i] > 1e-6) {
        const int nn = a.npol[i];   // the other partners carry no dipole
        const size_t row = (size_t)i * a.cap, blk = (size_t)a.n * a.cap;
        // two entries per lane and step: both index loads, then both dipole and tensor loads,
        // in flight together (the index -> dipole chain is two memory latencies)
        for (int k = lane; k < nn; k += 64) {
            const bool two = k + 32 < nn;
            const int j0 = a.nbr[row + k], j1 = two ? a.nbr[row + k + 32] : j0;
            float t0[6], t1[6];
#pragma unroll
            for (int p = 0; p < 6; ++p) {
                t0[p] = a.tens32[p * blk + row + k];
                t1[p] = two ? a.tens32[p * blk + row + k + 32] : 0.f;
            }
            const float4 d0 = in[j0], d1 = in[j1];
            e[0] += t0[0] * d0.x + t0[1] * d0.y + t0[2] * d0.z;
            e[1] += t0[1] * d0.x + t0[3] * d0.y + t0[4] * d0.z;
            e[2] += t0[2] * d0.x + t0[4] * d0.y + t0[5] * d0.z;
            e[0] += t1[0] * d1.x + t1[1] * d1.y + t1[2] * d1.z;
            e[1] += t1[1] * d1.x + t1[3] * d1.y + t1[4] * d1.z;
            e[2] += t1[2] * d1.x + t1[4] * d1.y + t1[5] * d1.z;
        }
        for (int c = 0; c < 3; ++c) e[c] = warp_sum(e[c]);
        if (lane == 0 && i < 3 * a.nw) {
            const int w = i / 3, s = i % 3;
            const int pj[3][2] = {{1, 2}, {0, 2}, {0, 1}};
            const int pp[3][2] = {{0, 1}, {0, 2}, {1, 2}};
            // the FP32 copy: FP64 loads and conversions would occupy the FP64 pipe (1/64 rate)
            const float* T = a.intra32 + 18 * (size_t)w;
            for (int u = 0; u < 2; ++u) {
                const float4 d = in[3 * w + pj[s][u]];
                const float* t = T + 6 * pp[s][u];
                e[0] += t[0] * d.x + t[1] * d.y + t[2] * d.z;
                e[1] += t[1] * d.x + t[3] * d.y + t[4] * d.z;
                e[2] += t[2] * d.x + t[4] * d.y + t[5] * d.z;
            }
        }
    }
    if (lane == 0)
        for (int c = 0; c < 3; ++c) out[c * a.n + i] = e[c];
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Rows of the per-site axis factors: x rows l = 0..kmax1, then y rows m = -kmax2..kmax2,
// then z rows n = -kmax3..kmax3 (each row n sites).
__device__ __forceinline__ int row_z(const KArgs& k, int n) { return k.kmax[0] + 2 * k.kmax[1] + 2 + k.kmax[2] + n; }

// FP32 dipole structure factors of the correction, phases formed on the fly:
// exp(ik.r_j) = fx_l(j) fy_m(j) fz_n(j) from the FP32 axis factors.  One k vector per
// thread (blockIdx.x: kSfThreads consecutive vectors), sites split over blockIdx.y.  The
// block stages tiles of kSfTile sites in shared memory: the x and y rows its vectors use
// (ktile), every z row, and d32.  Per k and site chunk: sum_j e_j (k.d_j), summed in FP32
// within a tile and in FP64 across tiles; k_pol_sfd32_sum adds the chunks in order.
constexpr int kSfTile = 64;
constexpr int kMaxRows = 448;   // factor rows a tile of k vectors may use (kmax up to ~100)
constexpr size_t kMaxDynSmem = 200 * 1024;   // dynamic shared memory of the FP32 k-space kernels

// kSfTile sites (from s0, ns of them real) of the tile's factor rows, transposed
// (fs[t * rowp + r]; rowp odd spreads the stores over the banks): rows 0..ncol-1 the
// products fx_l fy_m of the tile's (l, m) columns, then the z rows n = -kmax3..kmax3.
__device__ __forceinline__ void stage_tile(const KArgs& k, int4 tl, int rowp, int s0, int ns, float2* fs) {
    const int nrow = tl.y + 2 * k.kmax[2] + 1;
    for (int idx = threadIdx.x; idx < nrow * kSfTile; idx += blockDim.x) {
        const int r = idx / kSfTile, t = idx % kSfTile;
        float2 v = make_float2(0.f, 0.f);
        if (t < ns) {
            const size_t j = (size_t)s0 + t;
            if (r < tl.y) {
                const int c = k.kcol[tl.x + r];
                v = cmulf(k.fac32[(size_t)(c >> 16) * k.n + j], k.fac32[(size_t)(c & 0xffff) * k.n + j]);
            } else {
                v = k.fac32[(size_t)row_z(k, r - tl.y - k.kmax[2]) * k.n + j];
            }
        }
        fs[t * rowp + r] = v;
    }
}

// Two k vectors per thread: the block takes two consecutive tiles of kSfThreads vectors
// (their columns are contiguous), so each staged site tile serves 512 vectors.
__global__ void __launch_bounds__(kSfThreads) k_pol_sfd32(KArgs k, MixArgs m, int schunk, int rowp,
                                                          double* __restrict__ part) {
    if (k.stop && *k.stop) return;
    extern __shared__ float4 sfd_smem[];
    float4* ds = sfd_smem;                                   // [kSfTile]
    float2* fs = reinterpret_cast<float2*>(sfd_smem + kSfTile);   // [kSfTile][rowp]
    const int nkt = (k.K + kSfThreads - 1) / kSfThreads;
    const int4 ta = k.ktile[2 * blockIdx.x];
    const int4 tb = 2 * blockIdx.x + 1 < nkt ? k.ktile[2 * blockIdx.x + 1] : ta;
    const int4 tl = make_int4(ta.x, max(ta.x + ta.y, tb.x + tb.y) - ta.x, 0, 0);   // first column, columns
    int rc[2] = {0, 0}, rn[2] = {0, 0};
    float kx[2] = {0.f, 0.f}, ky[2] = {0.f, 0.f}, kz[2] = {0.f, 0.f};
    const int kk0 = 2 * blockIdx.x * kSfThreads + threadIdx.x;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int kk = kk0 + h * kSfThreads;
        if (kk < k.K) {
            rc[h] = k.kaux[kk].z - tl.x;
            rn[h] = tl.y + k.lmn[kk].z + k.kmax[2];
            const double4 kv = k.kv[kk];
            kx[h] = (float)kv.x;
            ky[h] = (float)kv.y;
            kz[h] = (float)kv.z;
        }
    }
    const int sb = blockIdx.y * schunk, se = min(k.n, sb + schunk);
    double ac[2] = {0.0, 0.0}, as[2] = {0.0, 0.0};
    for (int s0 = sb; s0 < se; s0 += kSfTile) {
        const int ns = min(kSfTile, se - s0);
        __syncthreads();
        stage_tile(k, tl, rowp, s0, ns, fs);
        for (int t = threadIdx.x; t < kSfTile; t += kSfThreads)
            ds[t] = t < ns ? m.d32[s0 + t] : make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        float c0 = 0.f, s0_ = 0.f, c1 = 0.f, s1 = 0.f;
#pragma unroll 4
        for (int t = 0; t < kSfTile; ++t) {
            const float2* f = fs + t * rowp;
            const float4 d = ds[t];
            const float2 e0 = cmulf(f[rc[0]], f[rn[0]]);
            const float2 e1 = cmulf(f[rc[1]], f[rn[1]]);
            const float p0 = kx[0] * d.x + ky[0] * d.y + kz[0] * d.z;
            const float p1 = kx[1] * d.x + ky[1] * d.y + kz[1] * d.z;
            c0 += e0.x * p0;
            s0_ += e0.y * p0;
            c1 += e1.x * p1;
            s1 += e1.y * p1;
        }
        ac[0] += (double)c0;
        as[0] += (double)s0_;
        ac[1] += (double)c1;
        as[1] += (double)s1;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int kk = kk0 + h * kSfThreads;
        if (kk < k.K) {
            double* p = part + 2 * ((size_t)blockIdx.y * k.K + kk);
            p[0] = ac[h];
            p[1] = as[h];
        }
    }
}

// The site chunks of k_pol_sfd32 added in order; the coefficients of the FP32 gather.
__global__ void __launch_bounds__(kThreads) k_pol_sfd32_sum(KArgs k, int nchunk, const double* __restrict__ part) {
    if (k.stop && *k.stop) return;
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= k.K) return;
    double skc = 0.0, sks = 0.0;
    for (int q = 0; q < nchunk; ++q) {
        const double* p = part + 2 * ((size_t)q * k.K + kk);
        skc += p[0];
        sks += p[1];
    }
    const double4 kv = k.kv[kk];
    float* c = k.kco32 + 16 * (size_t)kk;
    c[0] = (float)kv.x; c[1] = (float)kv.y; c[2] = (float)kv.z;
    c[3] = (float)(kv.w * sks);
    c[4] = (float)(kv.w * skc);
}

// Mixed precision, final pass: the final dipoles differ from those of the last FP64
// structure factors (k.sf) only by the last SOR update `dlt` (at the dipole tolerance), so
// the final dipole structure factors are k.sf plus the FP32 structure factors of dlt.
// With velocities the 24 sums of the ew1p per-atom stress contraction (weights q v_b and
// mu_c v_b, FP32, 12 per site in vh32) come from the same pass.  One k vector per thread,
// phases formed on the fly as in k_pol_sfd32; FP32 within a site tile, FP64 across tiles;
// per site chunk NV sums, added in order by k_pol_sfx32_fin.
template <int HEAT>
__global__ void __launch_bounds__(kSfThreads, 2) k_pol_sfx32(KArgs k, const float4* __restrict__ dlt,
                                                             const float4* __restrict__ vh32, int schunk, int rowp,
                                                             double* __restrict__ part) {
    constexpr int NV = HEAT ? 30 : 6;
    constexpr int NW = HEAT ? 4 : 1;   // float4 per site: dlt, then the 12 heat weights
    extern __shared__ float4 sfx_smem[];
    float4* ws = sfx_smem;                                       // [kSfTile][NW]
    float2* fs = reinterpret_cast<float2*>(sfx_smem + kSfTile * NW);   // [kSfTile][rowp]
    const int kk = blockIdx.x * kSfThreads + threadIdx.x;
    const int4 tl = k.ktile[blockIdx.x];
    int rc = 0, rn = 0;
    if (kk < k.K) {
        rc = k.kaux[kk].x;
        rn = tl.y + k.lmn[kk].z + k.kmax[2];
    }
    const int sb = blockIdx.y * schunk, se = min(k.n, sb + schunk);
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = 0.0;
    for (int s0 = sb; s0 < se; s0 += kSfTile) {
        const int ns = min(kSfTile, se - s0);
        __syncthreads();
        stage_tile(k, tl, rowp, s0, ns, fs);
        for (int t = threadIdx.x; t < kSfTile * NW; t += kSfThreads) {
            const int site = t / NW, w = t % NW;
            float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
            if (site < ns) val = w == 0 ? dlt[s0 + site] : vh32[3 * (size_t)(s0 + site) + w - 1];
            ws[t] = val;
        }
        __syncthreads();
        float v[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q] = 0.f;
#pragma unroll 2
        for (int t = 0; t < kSfTile; ++t) {
            const float2* f = fs + t * rowp;
            const float2 e = cmulf(f[rc], f[rn]);
            const float4 d = ws[t * NW];
            v[0] += e.x * d.x; v[1] += e.x * d.y; v[2] += e.x * d.z;
            v[3] += e.y * d.x; v[4] += e.y * d.y; v[5] += e.y * d.z;
            if (HEAT) {
                const float4 w0 = ws[t * NW + 1], w1 = ws[t * NW + 2], w2 = ws[t * NW + 3];
                const float w[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    v[6 + b] += e.x * w[b];    // V1
                    v[9 + b] += e.y * w[b];    // V2
                }
#pragma unroll
                for (int cb = 0; cb < 9; ++cb) {
                    v[12 + cb] += e.x * w[3 + cb];   // W1[c][b]
                    v[21 + cb] += e.y * w[3 + cb];   // W2[c][b]
                }
            }
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] += (double)v[q];
    }
    if (kk < k.K) {
        double* p = part + NV * ((size_t)blockIdx.y * k.K + kk);
#pragma unroll
        for (int q = 0; q < NV; ++q) p[q] = acc[q];
    }
}

template <int HEAT>
__global__ void __launch_bounds__(kThreads) k_pol_sfx32_fin(KArgs k, int nchunk, const double* __restrict__ part) {
    constexpr int NV = HEAT ? 30 : 6;
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= k.K) return;
    double tot[NV];
    for (int q = 0; q < NV; ++q) tot[q] = 0.0;
    for (int c = 0; c < nchunk; ++c) {
        const double* p = part + NV * ((size_t)c * k.K + kk);
        for (int q = 0; q < NV; ++q) tot[q] += p[q];
    }
    const double* sf = k.sf + 8 * (size_t)kk;
    for (int q = 0; q < 6; ++q) tot[q] = sf[2 + q] + tot[q];
    final_k<HEAT>(k, kk, tot);
}

// Shared-memory bytes of the FP32 gathers: the z rows of the block's sites.
inline size_t gather_smem(const int* kmax) { return (size_t)(2 * kmax[2] + 1) * kThreads * sizeof(float2); }

// The FP32 gathers (one site per thread, k vectors in ewald1p's order): the block's sites
// keep their z-row factors in shared memory ([row][kThreads]); the product fx_l fy_m of the
// current (l, m) column stays in registers, and the next column's factors are loaded (from
// L2) when a column starts, so they have arrived when it ends.  Out-of-range threads work
// on the last site and store nothing.
struct GatherPhase {
    const float2* fac32;
    size_t n, jc;
    int col = -1;
    float2 fxy = make_float2(0.f, 0.f), px, py;
    __device__ GatherPhase(const KArgs& k, float2* smem, int jc_, int kfirst) : fac32(k.fac32), n(k.n), jc(jc_) {
        const int nz = 2 * k.kmax[2] + 1;
        for (int r = 0; r < nz; ++r) smem[r * kThreads + threadIdx.x] = fac32[(size_t)row_z(k, r - k.kmax[2]) * n + jc];
        const int c = k.kcol[k.kaux[kfirst].z];
        px = fac32[(size_t)(c >> 16) * n + jc];
        py = fac32[(size_t)(c & 0xffff) * n + jc];
    }
    // exp(ik.r_j) for the k vector with auxiliary record x (column, z offset)
    __device__ __forceinline__ float2 operator()(int4 x, const float2* smem) {
        if (x.z != col) {   // uniform across the block
            col = x.z;
            fxy = cmulf(px, py);
            px = fac32[(size_t)(x.y >> 16) * n + jc];
            py = fac32[(size_t)(x.y & 0xffff) * n + jc];
        }
        return cmulf(fxy, smem[x.w + threadIdx.x]);
    }
};

// FP32 k-space field of the correction: one site per thread, k vectors split over
// blockIdx.y; each tile of kKTile vectors summed in FP32, the tiles in FP64; the partial
// sums of the chunks added in order by k_pol_kfield32_sum.
__global__ void __launch_bounds__(kThreads) k_pol_kfield32(KArgs k, int kchunk, float* __restrict__ part) {
    if (k.stop && *k.stop) return;
    extern __shared__ float2 gat_smem[];
    __shared__ float4 cf[kKTile][2];   // kx ky kz c3, c4 ...
    __shared__ int4 ax[kKTile];
    const int j = blockIdx.x * kThreads + threadIdx.x;
    const int kb = blockIdx.y * kchunk, ke = min(k.K, kb + kchunk);
    GatherPhase ph(k, gat_smem, min(j, k.n - 1), kb);
    double ed[3] = {0, 0, 0};
    for (int t0 = kb; t0 < ke; t0 += kKTile) {
        const int nt = min(kKTile, ke - t0);
        __syncthreads();
        for (int u = threadIdx.x; u < 2 * nt; u += kThreads)
            cf[u >> 1][u & 1] = reinterpret_cast<const float4*>(k.kco32)[4 * (size_t)(t0 + (u >> 1)) + (u & 1)];
        for (int u = threadIdx.x; u < nt; u += kThreads) ax[u] = k.kaux[t0 + u];
        __syncthreads();
        float e[3] = {0, 0, 0};
#pragma unroll 4
        for (int u = 0; u < nt; ++u) {
            const float4 c0 = cf[u][0];
            const float c4 = cf[u][1].x;
            const float2 a = ph(ax[u], gat_smem);
            const float w = a.y * c0.w + a.x * c4;
            e[0] -= c0.x * w; e[1] -= c0.y * w; e[2] -= c0.z * w;
        }
        for (int c = 0; c < 3; ++c) ed[c] += (double)e[c];
    }
    if (j < k.n) {
        float* p = part + (size_t)blockIdx.y * 3 * k.n;
        for (int c = 0; c < 3; ++c) p[c * (size_t)k.n + j] = (float)ed[c];
    }
}

__global__ void __launch_bounds__(kThreads) k_pol_kfield32_sum(KArgs k, PolArgs a, MixArgs m, int nchunk,
                                                               const float* __restrict__ part) {
    if (k.stop && *k.stop) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.n) return;
    float ev[3] = {0, 0, 0};
    for (int q = 0; q < nchunk; ++q)
        for (int c = 0; c < 3; ++c) ev[c] += part[((size_t)q * 3 + c) * k.n + j];
    const float dum = (float)(4.0 * kR4pie0 * (a.alpha * a.alpha * a.alpha) / kSqrpi / 3.0);
    const float sc = (float)k.scale;
    const bool pol = a.polr2[j] > 1e-6;
    const float4 d = m.d32[j];
    const float dd[3] = {d.x, d.y, d.z};
    for (int c = 0; c < 3; ++c) m.e32[(3 + c) * (size_t)k.n + j] = (pol ? sc * ev[c] : 0.f) + dum * dd[c];
}

// Conjugate gradients for the correction: A x = b with A = r4pie0 / polr2 - T (T the
// dipole field operator: real-space tensors, k-space sum, self term; symmetric) and
// b = r4pie0 / polr2 * r, preconditioned by the diagonal r4pie0 / polr2.  Scalars live in
// acc: 33 rho.z, 34 d.Ad, 35 new rho.z, 36 |z|^2, 37 count.
__global__ void __launch_bounds__(kThreads) k_pcg_init(PolArgs a, MixArgs m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0};
    if (i < a.n) {
        const float4 r = m.r32[i];
        const float w = a.polr2[i] > a.toler ? (float)(kR4pie0 / a.polr2[i]) : 0.f;
        m.x[i] = make_float4(0, 0, 0, 0);
        m.rho[i] = make_float4(w * r.x, w * r.y, w * r.z, 0.f);
        m.d32[i] = r;   // z = M^-1 rho = r
        v[0] = (double)w * ((double)r.x * r.x + (double)r.y * r.y + (double)r.z * r.z);
    }
    block_sum_atomic<1>(v, a.acc + 33);
}

__global__ void __launch_bounds__(kThreads) k_pcg_ad(PolArgs a, MixArgs m, int nk) {
    if (m.stop && *m.stop) return;   // the CG solve has stopped (uniform per launch)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0};
    if (i < a.n) {
        float4 q = make_float4(0, 0, 0, 0);
        if (a.polr2[i] > a.toler) {
            const float w = (float)(kR4pie0 / a.polr2[i]);
            const float4 d = m.d32[i];
            const float dv[3] = {d.x, d.y, d.z};
            float qv[3];
            for (int c = 0; c < 3; ++c)
                qv[c] = w * dv[c] - (m.e32[c * (size_t)a.n + i] + (nk ? m.e32[(3 + c) * (size_t)a.n + i] : 0.f));
            q = make_float4(qv[0], qv[1], qv[2], 0.f);
            v[0] = (double)dv[0] * qv[0] + (double)dv[1] * qv[1] + (double)dv[2] * qv[2];
        }
        m.q[i] = q;
    }
    block_sum_atomic<1>(v, a.acc + 34);
}

__device__ void pcg_next_body(double* acc, int* st, double target, bool keep_beta);

// With `st` (the diagonal preconditioner), the last block to finish also runs the sweep's
// stopping test (pcg_next_body, as k_pcg_next) on the complete sums; `ticket` counts the
// finished blocks and is left at 0.
__global__ void __launch_bounds__(kThreads) k_pcg_step(PolArgs a, MixArgs m, int* st, double target, int* ticket,
                                                       int skip_rz) {
    if (m.stop && *m.stop) return;   // the CG solve has stopped (uniform per launch)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0, 0, 0};
    const double pq = a.acc[34];
    const float g = pq != 0.0 ? (float)(a.acc[33] / pq) : 0.f;
    if (i < a.n && a.polr2[i] > a.toler) {
        const float w = (float)(a.polr2[i] / kR4pie0);
        const float4 d = m.d32[i], q = m.q[i];
        float4 x = m.x[i], r = m.rho[i];
        x.x += g * d.x; x.y += g * d.y; x.z += g * d.z;
        r.x -= g * q.x; r.y -= g * q.y; r.z -= g * q.z;
        m.x[i] = x;
        m.rho[i] = r;
        const double z[3] = {(double)w * r.x, (double)w * r.y, (double)w * r.z};
        v[0] = skip_rz ? 0.0 : z[0] * r.x + z[1] * r.y + z[2] * r.z;   // the block kernel's rho.z instead
        v[1] = z[0] * z[0] + z[1] * z[1] + z[2] * z[2];
        v[2] = 1.0;
    }
    block_sum_atomic<3>(v, a.acc + 35);
    if (!st) return;
    __shared__ int last;
    __threadfence();   // this block's sums (threads 0..2) before its ticket
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    *ticket = 0;
    pcg_next_body(a.acc, st, target, true);
}

// d = z + beta d, z = M^-1 rho: the diagonal (z null) or the polynomial preconditioner's z.
// beta: the new rho.z over the previous one, or (fused: the stopping test has run in
// k_pcg_step and moved the sums on) the beta it kept in acc[38].
__global__ void __launch_bounds__(kThreads) k_pcg_dir(PolArgs a, MixArgs m, const float4* __restrict__ z,
                                                      int fused) {
    if (m.stop && *m.stop) return;   // the CG solve has stopped (uniform per launch)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !(a.polr2[i] > a.toler)) return;
    const double rz = a.acc[33];
    const float b = fused ? (float)a.acc[38] : (rz != 0.0 ? (float)(a.acc[35] / rz) : 0.f);
    const float4 d = m.d32[i];
    float4 zz;
    if (z) {
        zz = z[i];
    } else {
        const float w = (float)(a.polr2[i] / kR4pie0);
        const float4 r = m.rho[i];
        zz = make_float4(w * r.x, w * r.y, w * r.z, 0.f);
    }
    m.d32[i] = make_float4(zz.x + b * d.x, zz.y + b * d.y, zz.z + b * d.z, 0.f);
}

__device__ void pcg_next_body(double* acc, int* st, double target, bool keep_beta);

// Block-Jacobi preconditioner: per water, the inverse of the 9x9 block of the CG matrix
// A = r4pie0/polr2 - dum - T over its three sites (the diagonal, the self term and the
// intramolecular tensors O-H1, O-H2, H1-H2; the k-space coupling inside the block left
// out), by Cholesky in FP32, stored whole (81 floats per water).  A water whose block is not
// positive definite, or with a site that carries no dipole, keeps the diagonal.
__global__ void k_pcg_block_setup(PolArgs a, float dum, float* __restrict__ binv) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= a.nw) return;
    float B[9][9];
    float d[3];
    bool ok = true;
    for (int s = 0; s < 3; ++s) {
        const double p2 = a.polr2[3 * w + s];
        ok = ok && p2 > a.toler;
        d[s] = p2 > a.toler ? (float)(kR4pie0 / p2) : 0.f;
    }
#pragma unroll
    for (int r = 0; r < 9; ++r)
#pragma unroll
        for (int c = 0; c < 9; ++c) B[r][c] = 0.f;
#pragma unroll
    for (int s = 0; s < 3; ++s)
#pragma unroll
        for (int c = 0; c < 3; ++c) B[3 * s + c][3 * s + c] = d[s] - dum;
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
    const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
    const float* T = a.intra32 + 18 * (size_t)w;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float t = T[6 * p + q];
            const int r = 3 * pa[p] + ia[q], c = 3 * pb[p] + ib[q];
            const int r2 = 3 * pa[p] + ib[q], c2 = 3 * pb[p] + ia[q];
            B[r][c] = -t;   // the (a, b) block and its transpose
            B[c][r] = -t;
            B[r2][c2] = -t;
            B[c2][r2] = -t;
        }
    // B = L L^T in place (lower triangle)
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        float v = B[j][j];
#pragma unroll
        for (int k = 0; k < j; ++k) v -= B[j][k] * B[j][k];
        ok = ok && v > 0.f;
        const float ljj = sqrtf(fmaxf(v, 1e-30f)), rl = 1.f / ljj;
        B[j][j] = ljj;
#pragma unroll
        for (int i = j + 1; i < 9; ++i) {
            float u = B[i][j];
#pragma unroll
            for (int k = 0; k < j; ++k) u -= B[i][k] * B[j][k];
            B[i][j] = u * rl;
        }
    }
    float* out = binv + 81 * (size_t)w;
    if (!ok) {   // the diagonal
        for (int r = 0; r < 9; ++r)
            for (int c = 0; c < 9; ++c) out[9 * r + c] = (r == c && d[r / 3] > 0.f) ? 1.f / d[r / 3] : 0.f;
        return;
    }
    // M = L^-1 (lower), written into the upper triangle of B transposed: Mt[k][i] = M[i][k]
    float M[9][9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
#pragma unroll
        for (int k = 0; k < 9; ++k) M[i][k] = 0.f;
        M[i][i] = 1.f / B[i][i];
#pragma unroll
        for (int k = 0; k < i; ++k) {
            float u = 0.f;
#pragma unroll
            for (int q = k; q < i; ++q) u += B[i][q] * M[q][k];
            M[i][k] = -u * M[i][i];
        }
    }
    // B^-1 = M^T M
#pragma unroll
    for (int r = 0; r < 9; ++r)
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            float u = 0.f;
#pragma unroll
            for (int q = 0; q < 9; ++q) u += M[q][r] * M[q][c];
            out[9 * r + c] = u;
        }
}

// z = M^-1 rho with the block inverses: a thread per site, the three rows of its water's
// inverse times the water's residual; the sites of no water (M sites) 0.
// With `slot` >= 0 also rho.z into acc[slot], and with `st` the sweep's stopping test in the
// last block to finish (as k_pcg_step's; `ticket` counts the finished blocks).
__global__ void __launch_bounds__(kThreads) k_pcg_block(PolArgs a, MixArgs m, const float* __restrict__ binv,
                                                        float4* __restrict__ z, int slot, int* st, double target,
                                                        int* ticket) {
    if (m.stop && *m.stop) return;   // the CG solve has stopped (uniform per launch)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (i < a.n) {
        float o[3] = {0.f, 0.f, 0.f};
        if (i < 3 * a.nw) {
            const int w = i / 3, s = i % 3;
            const float4 r0 = m.rho[3 * w], r1 = m.rho[3 * w + 1], r2 = m.rho[3 * w + 2];
            const float rv[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
            const float* B = binv + 81 * (size_t)w + 27 * s;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float u = 0.f;
#pragma unroll
                for (int q = 0; q < 9; ++q) u += B[9 * c + q] * rv[q];
                o[c] = u;
            }
            const float* ri = rv + 3 * s;
            v[0] = (double)ri[0] * o[0] + (double)ri[1] * o[1] + (double)ri[2] * o[2];
        }
        z[i] = make_float4(o[0], o[1], o[2], 0.f);
    }
    if (slot < 0) return;
    block_sum_atomic<1>(v, a.acc + slot);
    if (!st) return;
    __shared__ int last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    *ticket = 0;
    pcg_next_body(a.acc, st, target, true);
}

// Polynomial preconditioner: p Jacobi sweeps on the real-space part of the system,
// (D - T_real) z = rho with D = r4pie0 / polr2, from z = 0:
//   z <- D^-1 (rho + T_real z)   (t = T_real z; t null: the first sweep, z = D^-1 rho),
// i.e. z = sum_{i<p} (D^-1 T_real)^i D^-1 rho, symmetric; positive definite for even p.
__global__ void __launch_bounds__(kThreads) k_pcg_jacobi(PolArgs a, MixArgs m, const float* __restrict__ t,
                                                         float4* __restrict__ z) {
    if (m.stop && *m.stop) return;   // the CG solve has stopped (uniform per launch)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.polr2[i] > a.toler) {
        const float w = (float)(a.polr2[i] / kR4pie0);
        const float4 r = m.rho[i];
        v = t ? make_float4(w * (r.x + t[i]), w * (r.y + t[(size_t)a.n + i]), w * (r.z + t[2 * (size_t)a.n + i]), 0.f)
              : make_float4(w * r.x, w * r.y, w * r.z, 0.f);
    }
    z[i] = v;
}

// rho.z into acc[slot]; with `dir`, also d32 = z (the first direction).
__global__ void __launch_bounds__(kThreads) k_pcg_rz(PolArgs a, MixArgs m, const float4* __restrict__ z, int slot,
                                                     int dir) {
    if (m.stop && *m.stop) return;   // the CG solve has stopped (uniform per launch)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0};
    if (i < a.n) {
        const float4 r = m.rho[i], zz = z[i];
        v[0] = (double)r.x * zz.x + (double)r.y * zz.y + (double)r.z * zz.z;
        if (dir) m.d32[i] = zz;
    }
    block_sum_atomic<1>(v, a.acc + slot);
}

// End of a CG sweep, on the device: the stopping test of the correction solve (|z| <= target
// with z the diagonally preconditioned residual; a breakdown when d.Ad <= 0 or a sum is not
// finite), then rho.z <- new rho.z and the sums cleared for the next sweep.
// st[0]: 0 running, 1 converged, 2 breakdown; st[1]: sweeps run; acc[42..45] the sums of the
// sweep that stopped it.
__device__ void pcg_next_body(double* acc, int* st, double target, bool keep_beta) {
    if (st[0] != 0) return;
    st[1] += 1;
    // L2 reads: the sums were added by atomics of other blocks
    const double dad = __ldcg(acc + 34), rz = __ldcg(acc + 35), zz = __ldcg(acc + 36), cnt = __ldcg(acc + 37);
    if (keep_beta) {
        const double rz0 = __ldcg(acc + 33);
        acc[38] = rz0 != 0.0 ? rz / rz0 : 0.0;
    }
    int state = 0;
    if (!(dad > 0.0) || !isfinite(rz) || !isfinite(zz)) state = 2;
    else if (sqrt(zz / (cnt > 0.0 ? cnt : 1.0)) <= target) state = 1;
    if (state) {
        acc[42] = dad;
        acc[43] = rz;
        acc[44] = zz;
        acc[45] = cnt;
        st[0] = state;
    }
    acc[33] = rz;
    acc[34] = acc[35] = acc[36] = acc[37] = 0.0;
}

__global__ void k_pcg_next(double* __restrict__ acc, int* __restrict__ st, double target) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    pcg_next_body(acc, st, target, false);
}

// The evaluation after a correction: the fields are linear in the dipoles, so each is the
// previous FP64 one plus the FP32 field of the correction (e32: real space in the first 3
// blocks, SPME k space with its self term in the next 3): emu += real (with `real`), efm +=
// k space (with `kspace`).  The correction is at the size of the residual, ~1e-4 of the
// dipoles in an MD step, so the FP32 rounding enters ~1e-11 of the fields.
__global__ void k_pol_field_add(PolArgs a, const float* __restrict__ e32, int real, int kspace) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const size_t n = a.n;
    for (int c = 0; c < 3; ++c) {
        if (real) a.emu[c * n + i] += (double)e32[c * n + i];
        if (kspace) a.efm[c * n + i] += (double)e32[(3 + c) * n + i];
    }
}

// mu += d in FP64; refreshes the masked dipoles.
// Also writes the update of the masked dipoles (the structure factors' dipoles) to d32,
// for the next field evaluation's k-space part (k_pol_kfield32_dsum).
__global__ void k_pol_apply(PolArgs a, MixArgs m, double4* __restrict__ md) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float4 dm = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.polr2[i] > a.toler) {
        const float4 d = m.x[i];
        a.mx[i] += (double)d.x;
        a.my[i] += (double)d.y;
        a.mz[i] += (double)d.z;
        if (a.polr2[i] > 1e-6) {
            md[i] = make_double4(a.mx[i], a.my[i], a.mz[i], 0.0);
            dm = make_float4(d.x, d.y, d.z, 0.f);
        }
    }
    m.d32[i] = dm;
}

// Mixed precision, FP64 field evaluations after a correction: the k-space dipole field is
// linear in the dipoles, so it is the previous one (efm, FP64) plus the field of the
// correction (FP32 phases and sums, on a quantity at the size of the residual).  Per k:
// the chunks of k_pol_sfx32<0> over the correction added in order; the dipole structure
// factors k.sf updated in FP64; the coefficients of the FP32 gather of the correction.
__global__ void __launch_bounds__(kThreads) k_pol_sfd_dfin(KArgs k, int nchunk, const double* __restrict__ part) {
    const int kk = blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= k.K) return;
    double t[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < nchunk; ++c) {
        const double* p = part + 6 * ((size_t)c * k.K + kk);
        for (int q = 0; q < 6; ++q) t[q] += p[q];
    }
    double* sf = k.sf + 8 * (size_t)kk;
    for (int q = 0; q < 6; ++q) sf[2 + q] += t[q];
    const double4 kv = k.kv[kk];
    float* c = k.kco32 + 16 * (size_t)kk;
    c[0] = (float)kv.x; c[1] = (float)kv.y; c[2] = (float)kv.z;
    c[3] = (float)(kv.w * (kv.x * t[3] + kv.y * t[4] + kv.z * t[5]));
    c[4] = (float)(kv.w * (kv.x * t[0] + kv.y * t[1] + kv.z * t[2]));
}

// efm += scale * (k-space field of the correction) + self term of the dipole change.
__global__ void __launch_bounds__(kThreads) k_pol_kfield32_dsum(KArgs k, PolArgs a, MixArgs m, int nchunk,
                                                                const float* __restrict__ part) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k.n) return;
    double em[3] = {0, 0, 0};
    for (int q = 0; q < nchunk; ++q)
        for (int c = 0; c < 3; ++c) em[c] += (double)part[((size_t)q * 3 + c) * k.n + j];
    const double dum = 4.0 * kR4pie0 * (a.alpha * a.alpha * a.alpha) / kSqrpi / 3.0;
    const bool pol = a.polr2[j] > 1e-6;
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.polr2[j] > a.toler) x = m.x[j];   // the dipole change of k_pol_apply
    const double dx[3] = {(double)x.x, (double)x.y, (double)x.z};
    for (int c = 0; c < 3; ++c) a.efm[c * k.n + j] += (pol ? k.scale * em[c] : 0.0) + dum * dx[c];
}

// Final k-space pass (ewald1p iflag 1): per site and chunk of k vectors, the force and the
// two DMS potentials (5 partial sums per site; the k-space charge energy of a site is its
// charge times the first potential).  Two sites per thread.
//   akk ssmu = q (c akk s2 - s akk s1) - (k.mu) (c akk s1 + s akk s2)
template <typename R, typename V2>
__device__ __forceinline__ void kforce_site(const R* r, V2 cs, R qj, const R* dv, bool pol, R* acc) {
    const R c = cs.x, s = cs.y;
    const R kap = pol ? dv[0] * r[0] + dv[1] * r[1] + dv[2] * r[2] : R(0);
    const R t1 = c * r[4] - s * r[3], t2 = c * r[3] + s * r[4];
    const R fv = qj * t1 - kap * t2;
    acc[0] -= r[0] * fv;
    acc[1] -= r[1] * fv;
    acc[2] -= r[2] * fv;
    acc[3] += c * r[5] + s * r[6];
    acc[4] += s * r[7] - c * r[8];
}

__global__ void __launch_bounds__(kThreads) k_pol_kforce(KArgs k, PolArgs a, int kchunk, double* __restrict__ part) {
    __shared__ double sh[kKTile][9];
    const int j0 = blockIdx.x * 2 * blockDim.x + threadIdx.x, j1 = j0 + blockDim.x;
    const int kb = blockIdx.y * kchunk, ke = min(k.K, kb + kchunk);
    const bool in0 = j0 < k.n, in1 = j1 < k.n;
    const double q0 = in0 ? a.q[j0] : 0.0, q1 = in1 ? a.q[j1] : 0.0;
    const bool p0 = in0 && a.polr2[j0] > 1e-6, p1 = in1 && a.polr2[j1] > 1e-6;
    const double d0[3] = {in0 ? a.mx[j0] : 0.0, in0 ? a.my[j0] : 0.0, in0 ? a.mz[j0] : 0.0};
    const double d1[3] = {in1 ? a.mx[j1] : 0.0, in1 ? a.my[j1] : 0.0, in1 ? a.mz[j1] : 0.0};
    double acc0[5] = {0, 0, 0, 0, 0}, acc1[5] = {0, 0, 0, 0, 0};
    for (int t0 = kb; t0 < ke; t0 += kKTile) {
        const int nt = min(kKTile, ke - t0);
        __syncthreads();
        for (int u = threadIdx.x; u < nt * 9; u += blockDim.x)
            sh[u / 9][u % 9] = k.kco[16 * (size_t)(t0 + u / 9) + u % 9];
        __syncthreads();
        const double2* e = k.eik + (size_t)t0 * k.n;
        for (int u = 0; u < nt; ++u, e += k.n) {
            if (in0) kforce_site<double, double2>(sh[u], e[j0], q0, d0, p0, acc0);
            if (in1) kforce_site<double, double2>(sh[u], e[j1], q1, d1, p1, acc1);
        }
    }
    double* p = part + (size_t)blockIdx.y * 5 * k.n;
    for (int c = 0; c < 5; ++c) {
        if (in0) p[c * (size_t)k.n + j0] = acc0[c];
        if (in1) p[c * (size_t)k.n + j1] = acc1[c];
    }
}

// The same in FP32 (mixed precision): FP32 coefficients and phases formed on the fly from
// the FP32 axis factors (one site per thread), each tile of kKTile k vectors summed in FP32
// and the tiles added in FP64.
__global__ void __launch_bounds__(kThreads) k_pol_kforce32(KArgs k, PolArgs a, int kchunk, double* __restrict__ part) {
    extern __shared__ float2 gat_smem[];
    __shared__ float4 cf[kKTile][3];   // the 9 coefficients
    __shared__ int4 ax[kKTile];
    const int j = blockIdx.x * kThreads + threadIdx.x;
    const bool in = j < k.n;
    const int jc = min(j, k.n - 1);
    const int kb = blockIdx.y * kchunk, ke = min(k.K, kb + kchunk);
    GatherPhase ph(k, gat_smem, jc, kb);
    const float qj = (float)a.q[jc];
    const bool pj = a.polr2[jc] > 1e-6;
    const float dj[3] = {(float)a.mx[jc], (float)a.my[jc], (float)a.mz[jc]};
    double acc[5] = {0, 0, 0, 0, 0};
    for (int t0 = kb; t0 < ke; t0 += kKTile) {
        const int nt = min(kKTile, ke - t0);
        __syncthreads();
        for (int u = threadIdx.x; u < 3 * nt; u += kThreads)
            cf[u / 3][u % 3] = reinterpret_cast<const float4*>(k.kco32)[4 * (size_t)(t0 + u / 3) + u % 3];
        for (int u = threadIdx.x; u < nt; u += kThreads) ax[u] = k.kaux[t0 + u];
        __syncthreads();
        float f[5] = {0, 0, 0, 0, 0};
        for (int u = 0; u < nt; ++u) {
            const float4 c0 = cf[u][0], c1 = cf[u][1], c2 = cf[u][2];
            const float r[9] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w, c2.x};
            kforce_site<float, float2>(r, ph(ax[u], gat_smem), qj, dj, pj, f);
        }
        for (int c = 0; c < 5; ++c) acc[c] += (double)f[c];
    }
    if (in) {
        double* p = part + (size_t)blockIdx.y * 5 * k.n;
        for (int c = 0; c < 5; ++c) p[c * (size_t)k.n + j] = acc[c];
    }
}

// Per site: the k-space sums of all chunks, the self terms and coulomb_polar.
__global__ void __launch_bounds__(kThreads) k_pol_kforce_sum(KArgs k, PolArgs a, int nchunk,
                                                             const double* __restrict__ part) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double red[2] = {0, 0};   // engsic, eng_polar
    if (j < k.n) {
        double v[6] = {0, 0, 0, 0, 0, 0};
        for (int q = 0; q < nchunk; ++q)
            for (int c = 0; c < 5; ++c) v[c] += part[((size_t)q * 5 + c) * k.n + j];
        const double qj = a.q[j];
        v[5] = qj * v[3];   // k-space charge energy of the site (update_energy_ew1p)
        const double dv[3] = {a.mx[j], a.my[j], a.mz[j]};
        a.fx[j] += k.scale * v[0];
        a.fy[j] += k.scale * v[1];
        a.fz[j] += k.scale * v[2];
        a.vesp[j] = k.scale * v[3] + k.scale * v[4] - 2.0 * kR4pie0 * qj * a.alpha / kSqrpi / a.eps;
        const double self = -kR4pie0 / a.eps * a.alpha * qj * qj / kSqrpi;
        double ae = self + k.sfac * v[5];
        red[0] = self;
        if (a.polr2[j] > 1e-6) {   // coulomb_polar
            double e = 0.0;
            for (int c = 0; c < 3; ++c)
                e += dv[c] * (a.efk[c * k.n + j] + a.efc[c * k.n + j] + 0.5 * (a.emu[c * k.n + j] + a.efm[c * k.n + j]) + 0.0);
            e = -e;
            const double edum = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
            const double sp = kR4pie0 * edum / a.polr2[j] / 2.0;
            ae += e + sp;
            red[1] = e + sp;
        }
        a.ae[j] = ae;
    }
    block_sum_atomic<2>(red, a.acc + 40);
}

// ---------------------------------------------------------------------------------------
// --- final real-space terms ----------------------------------------------------------------
// ewald2p for the directed pair (i, j): force on i, its per-atom energy half, its DMS
// potential; pair scalars only from i < j.
__global__ void __launch_bounds__(kThreads) k_pol_ewald2p(PolArgs a, double g34, int heat) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double red[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};   // eng, vir, stress(6), jpot(3)
    if (i < a.n) {
        const int nn = a.nn[i];
        const size_t row = (size_t)i * a.cap;
        const double qi = a.q[i];
        const double mi[3] = {a.mx[i], a.my[i], a.mz[i]};
        const bool poli = a.polr2[i] > 1e-6;
        double f[3] = {0, 0, 0}, aei = 0, vsp = 0;
        for (int k = lane; k < nn; k += 32) {
            const int j = a.nbr[row + k];
            double d[3];
            sep(a, i, j, d[0], d[1], d[2]);
            const double rsq = norm2(d[0], d[1], d[2]);
            if (!(a.rcsq > rsq)) continue;
            const double rrr = __dsqrt_rn(rsq);
            double bbb[4];
            interp(a, rrr, bbb);
            const double rri = 1.0 / rrr, rsqi = 1.0 / rsq, r3i = 1.0 / (rrr * rrr * rrr), r5i = r3i * rsqi;
            const double qj = a.q[j];
            const double cicj = qi * qj;
            const double edum = cicj * (bbb[0] + 1.0 / rrr) * kR4pie0;
            double eng = edum;
            aei += 0.5 * edum;
            double espdum = (bbb[0] + 1.0 / rrr) * kR4pie0;
            double ffac = cicj * (r3i + bbb[1]) * kR4pie0;
            const double bb = a.polr6[i] * a.polr6[j];
            {
                const double arob4 = a.ascc * pow4(rrr / bb);
                if (arob4 < kDampCut) {
                    const double dum1 = exp(-arob4);
                    const double gq = gammq(0.75, arob4);
                    const double sm = (dum1 - pow(arob4, 0.25) * g34 * gq) / rrr * kR4pie0;
                    eng -= cicj * sm;
                    aei += -cicj * 0.5 * (dum1 - pow(arob4, 0.25) * g34 * gq) / rrr * kR4pie0;
                    espdum -= sm;
                    ffac = ffac - cicj * r3i * dum1 * kR4pie0;
                }
            }
            const double mj[3] = {a.mx[j], a.my[j], a.mz[j]};
            const double rdmui = mi[0] * d[0] + mi[1] * d[1] + mi[2] * d[2];
            const double rdmuj = mj[0] * d[0] + mj[1] * d[1] + mj[2] * d[2];
            const double facmu0 = (qj * rdmui - qi * rdmuj) * (-3.0) * r5i * kR4pie0;
            const double facmui0 = r3i * qj * kR4pie0;
            const double facmuj0 = -r3i * qi * kR4pie0;
            double facmu = facmu0 - (qj * rdmui - qi * rdmuj) * bbb[2] * kR4pie0;
            double dfi = facmui0 + bbb[1] * qj * kR4pie0;
            double dfj = facmuj0 - bbb[1] * qi * kR4pie0;
            double espdc = (bbb[1] + r3i) * kR4pie0;
            {
                const double arob4 = a.ascd * pow4(rrr / bb);
                const double dum1 = arob4 < kDampCut ? exp(-arob4) : 0.0;
                const double dum2 = (1.0 + (4.0 / 3.0) * arob4) * dum1;
                facmu = facmu - facmu0 * dum2;
                dfi = dfi - facmui0 * dum1;
                dfj = dfj - facmuj0 * dum1;
                espdc = espdc - r3i * dum1 * kR4pie0;
            }
            if (poli && a.polr2[j] > 1e-6) {
                const double dpidpj = mi[0] * mj[0] + mi[1] * mj[1] + mi[2] * mj[2];
                facmu = facmu + ((dpidpj * 3.0 + rdmui * rdmuj * rsqi * (-15.0)) * r5i + bbb[2] * dpidpj -
                                 bbb[3] * rdmui * rdmuj) * kR4pie0;
                dfi = dfi + (3.0 * r5i + bbb[2]) * rdmuj * kR4pie0;
                dfj = dfj + (3.0 * r5i + bbb[2]) * rdmui * kR4pie0;
                const double facmu1 = -15.0 * rdmui * rdmuj * rsqi * r5i * kR4pie0;
                const double facmu2 = 3.0 * dpidpj * r5i * kR4pie0;
                const double dfi1 = 3.0 * rdmuj * r5i * kR4pie0;
                const double dfj1 = 3.0 * rdmui * r5i * kR4pie0;
                const double bb4 = pow4(bb);
                const double arob4 = a.athole * pow4(rrr / bb);
                const double dum1 = arob4 < kDampCut ? exp(-arob4) : 0.0;
                const double dum2 = (1.0 + (4.0 / 3.0) * arob4) * dum1;
                const double dum3 = 4.0 * a.athole * (4.0 * arob4 - 1.0) * dum1 * rsqi / bb4;
                const double dum4 = 4.0 * a.athole * dum1 * rrr / bb4;
                facmu = facmu - facmu1 * dum2 - facmu2 * dum1 + rdmui * rdmuj * dum3 * rri * kR4pie0 -
                        dpidpj * rsqi * dum4 * kR4pie0;
                dfi = dfi - dfi1 * dum2;
                dfj = dfj - dfj1 * dum2;
            }
            const double dfx = dfi * mi[0] + dfj * mj[0];
            const double dfy = dfi * mi[1] + dfj * mj[1];
            const double dfz = dfi * mi[2] + dfj * mj[2];
            ffac = ffac + facmu;
            const double fx = ffac * d[0] + dfx, fy = ffac * d[1] + dfy, fz = ffac * d[2] + dfz;
            f[0] += fx; f[1] += fy; f[2] += fz;
            vsp += qj * espdum + rdmuj * espdc;
            if (heat) heat_entry(a, i, j, fx, fy, fz, red + 8);
            if (j > i) {
                const double virdum = dfx * d[0] + dfy * d[1] + dfz * d[2];
                red[0] += eng;
                red[1] += -ffac * rsq - virdum;
                red[2] += d[0] * fx; red[3] += d[0] * fy; red[4] += d[0] * fz;
                red[5] += d[1] * fy; red[6] += d[1] * fz; red[7] += d[2] * fz;
            }
        }
        for (int c = 0; c < 3; ++c) f[c] = warp_sum(f[c]);
        aei = warp_sum(aei);
        vsp = warp_sum(vsp);
        if (lane == 0) {
            a.fx[i] += f[0];
            a.fy[i] += f[1];
            a.fz[i] += f[2];
            a.ae[i] += aei;
            a.vesp[i] += vsp;
        }
    }
    block_sum_atomic<11>(red, a.acc + 0);
}

// The mixed path's ewald2p: the same terms as k_pol_ewald2p.  The pair energies stay FP64
// (the screened 1/r interpolated from the FP64 table, the smeared charge-charge term with
// the FP64 gammq: the per-site energies feed jkin, whose budget FP32 pair energies would
// exceed); the forces, the potentials and the dipole terms are FP32 per pair (the B
// functions from the FP32 table of C_n = B_n + (2n-1)!!/r^(2n+1), free of the cancellation
// between B_n and the bare 1/r^(2n+1)); separation, cut test and heat entries FP64; every
// sum FP64.
// The pairs of a row whose smeared charge-charge term is not negligible (ascc (r/bb)^4 below
// kDampCut: about 1 in 20 listed pairs, within ~3.5 A) need an FP64 gammq, pow and exp,
// several hundred FP64-pipe instructions.  Taken in the pair loop, a warp ran them for
// whichever of its lanes had such a pair, and most warp steps had one.  They are queued
// instead (32 per warp) and evaluated with every lane active when the queue fills and at
// the end of the row.
struct SmearQueue {
    int j[32];
    double r[32];
};

__device__ __forceinline__ void smear_flush(const PolArgs& a, int i, const SmearQueue& q, int cnt, int lane,
                                            double gln, double g34d, double qid, double& eng, double& aei,
                                            double& vsp) {
    if (lane >= cnt) return;
    const int j = q.j[lane];
    const double rrd = q.r[lane];
    const double arob4d = a.ascc * pow4(rrd * (a.rpolr6[i] * a.rpolr6[j]));
    const double dum1d = exp(-arob4d);
    const double gq = gammq_g(0.75, arob4d, gln);
    const double sm = (dum1d - pow(arob4d, 0.25) * g34d * gq) / rrd * kR4pie0;
    const double qjd = a.q[j];
    const double cicjd = qid * qjd;
    eng -= cicjd * sm;                      // every queued pair has j > i: its energy once
    aei -= cicjd * 0.5 * sm;
    vsp -= qjd * sm;
    atomicAdd(a.ae + j, -cicjd * 0.5 * sm);   // the partner's share
    atomicAdd(a.vesp + j, -qid * sm);
}

// The mixed path's ewald2p: the same terms as k_pol_ewald2p.  The pair energies stay FP64
// (the screened 1/r interpolated from the FP64 table, the smeared charge-charge term with
// the FP64 gammq: the per-site energies feed jkin, whose budget FP32 pair energies would
// exceed); the forces, the potentials and the dipole terms are FP32 per pair (the B
// functions from the FP32 table of C_n = B_n + (2n-1)!!/r^(2n+1), free of the cancellation
// between B_n and the bare 1/r^(2n+1)); separation, cut test and heat entries FP64; every
// sum FP64.  Every pair is taken once, from its lower site (the rows' j > i segments): the
// partner's force (the pair forces are antisymmetric), energy half, potential and heat
// entry go to it by FP64 atomics, which halves the FP64-pipe work of the pair loop.
__global__ void __launch_bounds__(kThreads) k_pol_ewald2p32(PolArgs a, double g34d, double gln, int heat) {
    __shared__ SmearQueue sq[kThreads / 32];
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double red[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};   // eng, vir, stress(6), jpot(3)
    if (i < a.n) {
        SmearQueue& q = sq[threadIdx.x >> 5];
        int qn = 0;   // queued pairs (warp-uniform)
        const size_t row = (size_t)i * a.cap;
        const float r4 = (float)kR4pie0;
        const double qid = a.q[i];
        const float qi = (float)qid;
        const float mi[3] = {(float)a.mx[i], (float)a.my[i], (float)a.mz[i]};
        const bool poli = a.polr2[i] > 1e-6;
        const float p6i = (float)a.polr6[i];
        const float ascc = (float)a.ascc, ascd = (float)a.ascd, athole = (float)a.athole;
        const float rdw = (float)(1.0 / a.drewd);
        const double rdwd = a.rdrewd;
        double f[3] = {0, 0, 0}, aei = 0, vsp = 0, engq = 0;
        // the partners j > i: [0, up.x) and [npol, npol + up.y) of the row
        const int2 up = a.nup[i];
        const int np = a.npol[i], nu = up.x + up.y;
        for (int b = 0; b < nu; b += 32) {
            const int v = b + lane;
            bool smear = false;
            int j = 0;
            double rrd = 0.0;
            if (v < nu) {
                const int k = v < up.x ? v : np + (v - up.x);
                j = a.nbr[row + k];
                double dd[3];
                sep(a, i, j, dd[0], dd[1], dd[2]);
                const double rsqd = norm2(dd[0], dd[1], dd[2]);
                if (a.rcsq > rsqd) {
                    const float d[3] = {(float)dd[0], (float)dd[1], (float)dd[2]};
                    const float rsq = (float)rsqd;
                    const float rrr = sqrtf(rsq);
                    // 3-point interpolation of the C_n table (erfcgenp's grid)
                    float bbb[4];
                    {
                        const float u = rrr * rdw;
                        const int ll = (int)u;
                        const float ppp = u - (float)ll;
                        const float4 v0 = a.ercp32[ll], v1 = a.ercp32[ll + 1], v2 = a.ercp32[ll + 2];
                        const float vk[4] = {v0.x, v0.y, v0.z, v0.w}, vk1[4] = {v1.x, v1.y, v1.z, v1.w},
                                    vk2[4] = {v2.x, v2.y, v2.z, v2.w};
#pragma unroll
                        for (int qq = 0; qq < 4; ++qq) {
                            const float t1 = vk[qq] + (vk1[qq] - vk[qq]) * ppp;
                            const float t2 = vk1[qq] + (vk2[qq] - vk1[qq]) * (ppp - 1.f);
                            bbb[qq] = t1 + (t2 - t1) * ppp * 0.5f;
                        }
                    }
                    const float rri = 1.f / rrr, rsqi = 1.f / rsq, r3i = rri * rsqi, r5i = r3i * rsqi;
                    const double qjd = a.q[j];
                    const float qj = (float)qjd;
                    const float cicj = qi * qj;
                    // FP64 energy: the screened 1/r (bbb[0] + 1/r of the FP64 table); the
                    // smeared term is queued
                    const double rrid = rsqrt_nr(rsqd);
                    rrd = rsqd * rrid;
                    double c0;
                    {
                        const double u = rrd * rdwd;
                        const int ll = (int)u;
                        const double ppp = u - double(ll);
                        const double v0 = a.ercp[ll].x, v1 = a.ercp[ll + 1].x, v2 = a.ercp[ll + 2].x;
                        const double t1 = v0 + (v1 - v0) * ppp;
                        const double t2 = v1 + (v2 - v1) * (ppp - 1.0);
                        c0 = t1 + (t2 - t1) * ppp * 0.5 + rrid;
                    }
                    const double cicjd = qid * qjd;
                    const double edum = cicjd * c0 * kR4pie0;
                    // bbb[1] = the screened 1/r^3 (C_1), bbb[2] = C_2, bbb[3] = C_3
                    const float espdum = bbb[0] * r4;
                    float ffac = cicj * bbb[1] * r4;
                    const float bb = p6i * (float)a.polr6[j];
                    const float rb = rrr / bb, rb2 = rb * rb, rb4 = rb2 * rb2;
                    {
                        const float arob4 = ascc * rb4;
                        if (arob4 < (float)kDampCut) {
                            smear = true;
                            ffac = ffac - cicj * r3i * expf(-arob4) * r4;
                        }
                    }
                    const float mj[3] = {(float)a.mx[j], (float)a.my[j], (float)a.mz[j]};
                    const float rdmui = mi[0] * d[0] + mi[1] * d[1] + mi[2] * d[2];
                    const float rdmuj = mj[0] * d[0] + mj[1] * d[1] + mj[2] * d[2];
                    const float x0 = qj * rdmui - qi * rdmuj;
                    const float facmu0 = x0 * (-3.f) * r5i * r4;
                    const float facmui0 = r3i * qj * r4;
                    const float facmuj0 = -r3i * qi * r4;
                    // facmu0 - x0 B_2 = -x0 C_2; facmui0 + B_1 qj = C_1 qj
                    float facmu = -x0 * bbb[2] * r4;
                    float dfi = bbb[1] * qj * r4;
                    float dfj = -bbb[1] * qi * r4;
                    float espdc = bbb[1] * r4;
                    {
                        const float arob4 = ascd * rb4;
                        const float dum1 = arob4 < (float)kDampCut ? expf(-arob4) : 0.f;
                        const float dum2 = (1.f + (4.f / 3.f) * arob4) * dum1;
                        facmu = facmu - facmu0 * dum2;
                        dfi = dfi - facmui0 * dum1;
                        dfj = dfj - facmuj0 * dum1;
                        espdc = espdc - r3i * dum1 * r4;
                    }
                    if (poli && a.polr2[j] > 1e-6) {
                        const float dpidpj = mi[0] * mj[0] + mi[1] * mj[1] + mi[2] * mj[2];
                        // (3 dpidpj - 15 rdmui rdmuj / r^2) r5i + B_2 dpidpj - B_3 rdmui rdmuj = C_2 dpidpj - C_3 rdmui rdmuj
                        facmu = facmu + (bbb[2] * dpidpj - bbb[3] * rdmui * rdmuj) * r4;
                        dfi = dfi + bbb[2] * rdmuj * r4;
                        dfj = dfj + bbb[2] * rdmui * r4;
                        const float facmu1 = -15.f * rdmui * rdmuj * rsqi * r5i * r4;
                        const float facmu2 = 3.f * dpidpj * r5i * r4;
                        const float dfi1 = 3.f * rdmuj * r5i * r4;
                        const float dfj1 = 3.f * rdmui * r5i * r4;
                        const float bb2 = bb * bb, bb4 = bb2 * bb2;
                        const float arob4 = athole * rb4;
                        const float dum1 = arob4 < (float)kDampCut ? expf(-arob4) : 0.f;
                        const float dum2 = (1.f + (4.f / 3.f) * arob4) * dum1;
                        const float dum3 = 4.f * athole * (4.f * arob4 - 1.f) * dum1 * rsqi / bb4;
                        const float dum4 = 4.f * athole * dum1 * rrr / bb4;
                        facmu = facmu - facmu1 * dum2 - facmu2 * dum1 + rdmui * rdmuj * dum3 * rri * r4 -
                                dpidpj * rsqi * dum4 * r4;
                        dfi = dfi - dfi1 * dum2;
                        dfj = dfj - dfj1 * dum2;
                    }
                    const float dfx = dfi * mi[0] + dfj * mj[0];
                    const float dfy = dfi * mi[1] + dfj * mj[1];
                    const float dfz = dfi * mi[2] + dfj * mj[2];
                    ffac = ffac + facmu;
                    const double fx = (double)(ffac * d[0] + dfx), fy = (double)(ffac * d[1] + dfy),
                                 fz = (double)(ffac * d[2] + dfz);
                    f[0] += fx; f[1] += fy; f[2] += fz;
                    aei += 0.5 * edum;
                    vsp += (double)(qj * espdum + rdmuj * espdc);
                    // the partner: the opposite force, its energy half, its potential (r_j - r_i =
                    // -d), its heat entry
                    atomicAdd(a.fx + j, -fx);
                    atomicAdd(a.fy + j, -fy);
                    atomicAdd(a.fz + j, -fz);
                    atomicAdd(a.ae + j, 0.5 * edum);
                    atomicAdd(a.vesp + j, (double)(qi * espdum - rdmui * espdc));
                    if (heat) {
                        heat_entry(a, i, j, fx, fy, fz, red + 8);
                        heat_entry(a, j, i, -fx, -fy, -fz, red + 8);
                    }
                    const double virdum = (double)(dfx * d[0] + dfy * d[1] + dfz * d[2]);
                    red[0] += edum;
                    red[1] += -(double)ffac * rsqd - virdum;
                    red[2] += dd[0] * fx; red[3] += dd[0] * fy; red[4] += dd[0] * fz;
                    red[5] += dd[1] * fy; red[6] += dd[1] * fz; red[7] += dd[2] * fz;
                }
            }
            // queue this step's smeared pairs; flush a full queue first
            const unsigned sb = __ballot_sync(0xffffffffu, smear);
            if (sb) {
                const int cnt = __popc(sb);
                if (qn + cnt > 32) {
                    __syncwarp();
                    smear_flush(a, i, q, qn, lane, gln, g34d, qid, engq, aei, vsp);
                    qn = 0;
                    __syncwarp();
                }
                if (smear) {
                    const int slot = qn + __popc(sb & ((1u << lane) - 1u));
                    q.j[slot] = j;
                    q.r[slot] = rrd;
                }
                qn += cnt;
            }
        }
        __syncwarp();
        if (qn) smear_flush(a, i, q, qn, lane, gln, g34d, qid, engq, aei, vsp);
        red[0] += engq;
        for (int c = 0; c < 3; ++c) f[c] = warp_sum(f[c]);
        aei = warp_sum(aei);
        vsp = warp_sum(vsp);
        if (lane == 0) {   // atomics: other rows add their pairs with this site concurrently
            atomicAdd(a.fx + i, f[0]);
            atomicAdd(a.fy + i, f[1]);
            atomicAdd(a.fz + i, f[2]);
            atomicAdd(a.ae + i, aei);
            atomicAdd(a.vesp + i, vsp);
        }
    }
    block_sum_atomic<11>(red, a.acc + 0);
}

// ewald3p over the six excluded pairs of one water (thread per water).
// One thread per excluded pair (6 per water): the pairs of a water add to the same sites,
// by atomics.
__global__ void __launch_bounds__(kThreads) k_pol_ewald3p(PolArgs a, int heat) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double red[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (t < 6 * a.nw) {
        const int w = t / 6, p = t % 6;
        const int o = 3 * w, m = 3 * a.nw + w;
        const int pr[6][2] = {{o, o + 1}, {o, o + 2}, {o + 1, o + 2}, {o, m}, {o + 1, m}, {o + 2, m}};
        const double r4e = kR4pie0 / a.eps;
        {
            const int ia = pr[p][0], ja = pr[p][1];
            double d[3];
            sep(a, ia, ja, d[0], d[1], d[2]);
            const double rsq = norm2(d[0], d[1], d[2]);
            const double rrr = __dsqrt_rn(rsq);
            const double rri = 1.0 / rrr, rsqi = 1.0 / rsq, r3i = 1.0 / (rrr * rrr * rrr), r5i = r3i * rsqi;
            double bbb[4];
            bfun_exact(a.alpha, rrr, rri, rsqi, bbb);
            const double qi = a.q[ia], qj = a.q[ja];
            const double cicj = qi * qj;
            red[0] += cicj * bbb[0] * r4e;
            atomicAdd(a.ae + ia, 0.5 * cicj * bbb[0] * r4e);
            atomicAdd(a.ae + ja, 0.5 * cicj * bbb[0] * r4e);
            const double espdum = bbb[0] * r4e, espdc = bbb[1] * r4e;
            double ffac = cicj * bbb[1] * r4e;
            const double mi[3] = {a.mx[ia], a.my[ia], a.mz[ia]}, mj[3] = {a.mx[ja], a.my[ja], a.mz[ja]};
            const double rdmui = mi[0] * d[0] + mi[1] * d[1] + mi[2] * d[2];
            const double rdmuj = mj[0] * d[0] + mj[1] * d[1] + mj[2] * d[2];
            double facmu = (qj * rdmui - qi * rdmuj) * (-bbb[2]) * r4e;
            double dfi = bbb[1] * qj * r4e;
            double dfj = -bbb[1] * qi * r4e;
            if (a.polr2[ia] > 1e-6 && a.polr2[ja] > 1e-6) {
                const double dpidpj = mi[0] * mj[0] + mi[1] * mj[1] + mi[2] * mj[2];
                facmu = facmu + (bbb[2] * dpidpj - bbb[3] * rdmui * rdmuj) * r4e;
                dfi = dfi + bbb[2] * rdmuj * r4e;
                dfj = dfj + bbb[2] * rdmui * r4e;
                const double facmu1 = -15.0 * rdmui * rdmuj * rsqi * r5i * r4e;
                const double facmu2 = 3.0 * dpidpj * r5i * r4e;
                facmu = facmu + facmu1 + facmu2;
                const double dfidd = 3.0 * rdmuj * r5i * r4e, dfjdd = 3.0 * rdmui * r5i * r4e;
                dfi = dfi + dfidd;
                dfj = dfj + dfjdd;
                const double bb = pow(a.polr[ia] * a.polr[ja], 1.0 / 6.0);
                const double bb4 = pow4(bb);
                const double ath = (ia % 3 == 0 || ja % 3 == 0) ? a.athole12 : a.athole13;
                const double arob4 = ath * pow4(rrr / bb);
                const double dum1 = exp(-arob4);
                const double dum2 = (1.0 + (4.0 / 3.0) * arob4) * dum1;
                const double dum3 = 4.0 * ath * (4.0 * arob4 - 1.0) * dum1 * rsqi / bb4;
                const double dum4 = 4.0 * ath * dum1 * rrr / bb4;
                facmu = facmu - facmu1 * dum2 - facmu2 * dum1 + rdmui * rdmuj * dum3 * rri * r4e - dpidpj * rsqi * dum4 * r4e;
                dfi = dfi - dfidd * dum2;
                dfj = dfj - dfjdd * dum2;
            }
            const double dfx = dfi * mi[0] + dfj * mj[0];
            const double dfy = dfi * mi[1] + dfj * mj[1];
            const double dfz = dfi * mi[2] + dfj * mj[2];
            ffac = ffac + facmu;
            const double fx = ffac * d[0] + dfx, fy = ffac * d[1] + dfy, fz = ffac * d[2] + dfz;
            atomicAdd(a.fx + ia, fx); atomicAdd(a.fy + ia, fy); atomicAdd(a.fz + ia, fz);
            atomicAdd(a.fx + ja, -fx); atomicAdd(a.fy + ja, -fy); atomicAdd(a.fz + ja, -fz);
            if (heat) {
                heat_entry(a, ia, ja, fx, fy, fz, red + 8);
                heat_entry(a, ja, ia, -fx, -fy, -fz, red + 8);
            }
            const double virdum = dfx * d[0] + dfy * d[1] + dfz * d[2];
            red[1] += -ffac * rsq - virdum;
            atomicAdd(a.vesp + ia, qj * espdum + rdmuj * espdc);
            atomicAdd(a.vesp + ja, qi * espdum - rdmui * espdc);
            red[2] += d[0] * fx; red[3] += d[0] * fy; red[4] += d[0] * fz;
            red[5] += d[1] * fy; red[6] += d[1] * fz; red[7] += d[2] * fz;
        }
    }
    block_sum_atomic<11>(red, a.acc + 0);
}

// qdforce (new charge assignment) with the summed DMS potentials: a thread per (water,
// site s) - four per water, each repeating the water's geometry - takes the force on site
// s from the four charges and site s's share of the stress.
__global__ void __launch_bounds__(kThreads) k_pol_qdforce(PolArgs a, int heat) {
    const int tq = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = tq >> 2, s = tq & 3;
    double red[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};   // -, vir, stress(6), jpot(3)
    if (w < a.nw) {
        const int io = 3 * w, h1 = io + 1, h2 = io + 2, mt = 3 * a.nw + w;
        const double* D = a.dp + 6 * (size_t)w;
        const double dp1dr1 = D[0], dp1dr2 = D[1], dp2dr1 = D[2], dp2dr2 = D[3], dp1dcos = D[4], dp2dcos = D[5];
        double r1v[3], r2v[3];
        sep(a, h1, io, r1v[0], r1v[1], r1v[2]);
        sep(a, h2, io, r2v[0], r2v[1], r2v[2]);
        const double r1 = sqrt(r1v[0] * r1v[0] + r1v[1] * r1v[1] + r1v[2] * r1v[2]);
        const double r2 = sqrt(r2v[0] * r2v[0] + r2v[1] * r2v[1] + r2v[2] * r2v[2]);
        const double rdot = r1v[0] * r2v[0] + r1v[1] * r2v[1] + r1v[2] * r2v[2];
        const double cost = rdot / (r1 * r2);
        const double r3 = sqrt(r1 * r1 + r2 * r2 - 2.0 * r1 * r2 * cost);
        const double sint = sqrt(1.0 - cost * cost);
        const double cott = cost / sint;
        const double r1sqr = r1 * r1, r2sqr = r2 * r2;
        double dr[3][4][3];
        for (int u = 0; u < 4; ++u)
            for (int c = 0; c < 3; ++c) dr[0][u][c] = dr[1][u][c] = dr[2][u][c] = 0.0;
        for (int c = 0; c < 3; ++c) {
            dr[0][1][c] = r1v[c] / r1;
            dr[0][0][c] = -dr[0][1][c];
            dr[1][2][c] = r2v[c] / r2;
            dr[1][0][c] = -dr[1][2][c];
            dr[2][1][c] = cott * (r1v[c] / r1sqr - r2v[c] / rdot);
            dr[2][2][c] = cott * (r2v[c] / r2sqr - r1v[c] / rdot);
            dr[2][0][c] = -dr[2][1][c] - dr[2][2][c];
        }
        const double g = a.gamma;
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
        const int site[4] = {io, h1, h2, mt};
        double vt[4];
        for (int u = 0; u < 4; ++u) vt[u] = a.vesp[site[u]];
        double fs[3] = {0.0, 0.0, 0.0};
        {   // site s, whose position moves the charges
            double dp1[3], dp2[3];
            for (int c = 0; c < 3; ++c) {
                dp1[c] = dp1dr1 * dr[0][s][c] + dp1dr2 * dr[1][s][c] - sint * dp1dcos * dr[2][s][c];
                dp2[c] = dp2dr1 * dr[0][s][c] + dp2dr2 * dr[1][s][c] - sint * dp2dcos * dr[2][s][c];
            }
            double dq[4][3];
            const double factor = g / 2.0 / (1.0 - g);
            for (int c = 0; c < 3; ++c) {
                dq[0][c] = 0.0;
                dq[1][c] = dp1[c] * (factor + 1.0) + dp2[c] * factor;
                dq[2][c] = dp2[c] * (factor + 1.0) + dp1[c] * factor;
                dq[3][c] = -(dq[1][c] + dq[2][c]);
            }
            for (int j = 0; j < 4; ++j) {   // charge j, in the reference's loop order
                const double F[3] = {-dq[j][0] * vt[j], -dq[j][1] * vt[j], -dq[j][2] * vt[j]};
                for (int c = 0; c < 3; ++c) fs[c] += F[c];
                if (heat) heat_entry(a, site[s], j == 3 ? a.nw + w : 3 * w + j, F[0], F[1], F[2], red + 8);
            }
        }
        a.fx[site[s]] += fs[0]; a.fy[site[s]] += fs[1]; a.fz[site[s]] += fs[2];
        double sq[6] = {0, 0, 0, 0, 0, 0}, virq = 0.0;
        const int ta[6] = {0, 0, 0, 1, 1, 2}, tb[6] = {0, 1, 2, 1, 2, 2};
        {   // the stress of charge s's potential
            const double v = vt[s];
            for (int lab = 1; lab <= 2; ++lab) {
                const double dqdr_tmp = lab == 1 ? dqdr12[s] : dqdr13[s];
                const int hh = lab == 1 ? h1 : h2;
                double r[3];
                sep(a, io, hh, r[0], r[1], r[2]);
                const double rjk = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                for (int q = 0; q < 6; ++q) sq[q] = sq[q] - v * dqdr_tmp * r[ta[q]] * r[tb[q]] / rjk;
                virq = virq + v * rjk * dqdr_tmp;
            }
            double a1[3], a2[3], a3[3];
            sep(a, io, h1, a1[0], a1[1], a1[2]);
            sep(a, io, h2, a2[0], a2[1], a2[2]);
            sep(a, h1, h2, a3[0], a3[1], a3[2]);
            const double q1 = sqrt(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
            const double q2 = sqrt(a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2]);
            const double q3 = sqrt(a3[0] * a3[0] + a3[1] * a3[1] + a3[2] * a3[2]);
            double dc[6];
            for (int q = 0; q < 6; ++q)
                dc[q] = dcosdr12 * a1[ta[q]] * a1[tb[q]] / q1 + dcosdr13 * a2[ta[q]] * a2[tb[q]] / q2 +
                        dcosdr23 * a3[ta[q]] * a3[tb[q]] / q3;
            for (int q = 0; q < 6; ++q) sq[q] = sq[q] - v * dqdcos[s] * dc[q];
            virq = virq + v * (dc[0] + dc[3] + dc[5]) * dqdcos[s];
        }
        red[1] = virq;
        for (int q = 0; q < 6; ++q) red[2 + q] = sq[q];
    }
    block_sum_atomic<11>(red, a.acc + 0);
}

// jkin's electrostatic part: redistributed per-site energies times velocities; the
// per-site energies are added to the caller's array.
__global__ void __launch_bounds__(kThreads) k_pol_jkin(PolArgs a, double* __restrict__ ae_out, int heat) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double red[3] = {0, 0, 0};
    if (j < a.n) {
        const double e = a.ae[j];
        if (ae_out) ae_out[j] += e;
        if (heat) {
            double v[3];
            vhat(a, j, v);
            red[0] = e * v[0]; red[1] = e * v[1]; red[2] = e * v[2];
        }
    }
    block_sum_atomic<3>(red, a.acc + 24);
}

__global__ void k_pol_kreduce(int K, const double* __restrict__ kterm, double* __restrict__ out) {
    // one block: out[q] = sum over k of kterm[16k + q], q < 11
    constexpr int NV = 11;
    double v[NV];
    for (int q = 0; q < NV; ++q) v[q] = 0.0;
    for (int k = threadIdx.x; k < K; k += blockDim.x)
        for (int q = 0; q < NV; ++q) v[q] += kterm[16 * (size_t)k + q];
    __shared__ double red[kSfThreads / 32][NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < NV; ++q) {
        const double s = warp_sum(v[q]);
        if (lane == 0) red[w][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int i = 0; i < kSfThreads / 32; ++i) s += red[i][threadIdx.x];
        out[threadIdx.x] = s;
    }
}

// Per-site products of the ew1p heat sums, with v the velocity each site's terms are
// carried with: q v (3 rows), then mu_c v_b (9 rows, c major), mu the masked dipole.
// vh (FP64, 12 blocks of n) or vh32 (FP32, 12 per site as 3 float4): q v_b, mu_c v_b.
__global__ void k_pol_vhat(PolArgs a, const double4* __restrict__ md, double* __restrict__ vh,
                           float4* __restrict__ vh32) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    double v[3];
    vhat(a, j, v);
    const double q = a.q[j];
    const double4 m = md[j];
    const double mu[3] = {m.x, m.y, m.z};
    double w[12];
    for (int b = 0; b < 3; ++b) w[b] = q * v[b];
    for (int c = 0; c < 3; ++c)
        for (int b = 0; b < 3; ++b) w[3 + 3 * c + b] = mu[c] * v[b];
    if (vh)
        for (int q_ = 0; q_ < 12; ++q_) vh[(size_t)q_ * a.n + j] = w[q_];
    if (vh32)
        for (int u = 0; u < 3; ++u)
            vh32[3 * (size_t)j + u] = make_float4((float)w[4 * u], (float)w[4 * u + 1], (float)w[4 * u + 2], (float)w[4 * u + 3]);
}

inline unsigned blocks(long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// M-site force redistribution (SOURCE/dlpoly_cmd.f:2585-2601), standard layout.
__global__ void k_msite_redistribute(int nw, double gamma, double* __restrict__ fx, double* __restrict__ fy,
                                     double* __restrict__ fz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    const int m = 3 * nw + i, o = 3 * i;
    double* f[3] = {fx, fy, fz};
    for (int c = 0; c < 3; ++c) {
        f[c][o] = f[c][o] + (1.0 - gamma) * f[c][m];
        f[c][o + 1] = f[c][o + 1] + f[c][m] * gamma / 2.0;
        f[c][o + 2] = f[c][o + 2] + f[c][m] * gamma / 2.0;
    }
}

__global__ void k_add(int n, const double* __restrict__ x, double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += x[i];
}

// --- host -------------------------------------------------------------------------------
cudaError_t launch_add(int n, const double* x, double* y, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_add<<<blocks(n, kThreads), kThreads, 0, s>>>(n, x, y);
    return cudaGetLastError();
}

cudaError_t launch_msite_redistribute(int nw, double gamma, double* fx, double* fy, double* fz, cudaStream_t s) {
    if (nw <= 0) return cudaSuccess;
    k_msite_redistribute<<<blocks(nw, kThreads), kThreads, 0, s>>>(nw, gamma, fx, fy, fz);
    return cudaGetLastError();
}

void PolarState::release() {
    void* p[] = {ercp, ercp32, nn_s, nbr_s, npol_s, nup_s, xref, nn, nbr, npol, nup, flag, xf, tens, intra, fld, vesp, ae, eik, kv, kx2, lmn, sf, kterm, acc, kco, fac, md, vh, polr6,
                 ckey, cskey, cidx, csidx, csort, cstart, cend,
                 tens32, r32, d32, e32, kco32, fac32, ktile, kaux, kcol, colk, kpart, cg_x, cg_r, cg_q, cg_z, vh32,
                 aspc_hist, binv};
    for (void* q : p)
        if (q) cudaFree(q);
    if (acc_h) cudaFreeHost(acc_h);
    for (auto& v : ev)
        if (v) {
            cudaEventDestroy(v);
            v = nullptr;
        }
    for (auto& pr : kfev)
        for (auto& v : pr)
            if (v) {
                cudaEventDestroy(v);
                v = nullptr;
            }
    ercp = nullptr;
    ercp32 = nullptr;
    nn_s = nbr_s = npol_s = nullptr;
    nup_s = nup = nullptr;
    xref = nullptr;
    ns_cap = cap_s_alloc = 0;
    skin_ok = false;
    nn = nbr = flag = npol = nullptr;
    xf = nullptr;
    tens = intra = fld = vesp = ae = sf = kterm = acc = kco = vh = polr6 = nullptr;
    ckey = cskey = nullptr;
    cidx = csidx = cstart = cend = nullptr;
    csort = nullptr;
    cell_n_cap = ncell_cap = 0;
    csort_bytes = 0;
    eik = fac = nullptr;
    md = nullptr;
    fac_cap = 0;
    tens32 = e32 = kco32 = nullptr;
    r32 = d32 = cg_x = cg_r = cg_q = cg_z = vh32 = nullptr;
    fac32 = nullptr;
    ktile = nullptr;
    kaux = nullptr;
    kcol = nullptr;
    colk = nullptr;
    ktile_cap = 0;
    cap32 = n32 = k32 = 0;
    fac32_cap = 0;
    kpart = nullptr;
    part_cap = 0;
    kv = nullptr;
    kx2 = nullptr;
    lmn = nullptr;
    acc_h = nullptr;
    n_cap = nw_cap = k_cap = 0;
    eik_cap = 0;
    tab_alpha = tab_rcut = -1.0;
    aspc_hist = nullptr;
    aspc_n = aspc_head = 0;
    binv = nullptr;
    binv_cap = 0;
}

PolarState::~PolarState() { release(); }

cudaError_t PolarState::aspc_reset(int k, int niter) {
    aspc_k = k;
    aspc_niter = niter;
    if (k) guess_order = 0;
    aspc_step = 0;
    aspc_head = 0;
    if (aspc_hist) cudaFree(aspc_hist);   // reallocated (zeroed) by the next call
    aspc_hist = nullptr;
    aspc_n = 0;
    return cudaSuccess;
}

void PolarState::aspc_restart() { aspc_step = 0; }

cudaError_t PolarState::guess_reset(int order) {
    const cudaError_t e = aspc_reset(0, 0);
    guess_order = order;
    return e;
}

// Kolafa's predictor coefficients B_1..B_{k+2} (J. Comput. Chem. 25 (2004) 335, eq. 6):
// B_j = (-1)^(j+1) j (4k+6)/(k+3) prod_{m<j} (k+2-m)/(k+3+m), as SOURCE/aspc.f90:110-114
// builds them (k = 2: 14/5, -14/5, 6/5, -1/5)
struct AspcCoef {
    double b[6];
};

static AspcCoef aspc_coefficients(int k) {
    AspcCoef c{};
    const double rk = k;
    double t = 1.0 / (rk + 3.0);
    for (int j = 1; j <= k + 2 && j <= 6; ++j) {
        c.b[j - 1] = ((j & 1) ? 1.0 : -1.0) * double(j) * (4.0 * rk + 6.0) * t;
        t = t * (rk + 2.0 - double(j)) / (rk + 3.0 + double(j));
    }
    return c;
}

// The initial guess of a converged solve: the polynomial of degree `order` through the last
// order+1 steps' dipoles, extrapolated one step, c_j = (-1)^(j+1) C(order+1, j) (newest first:
// 2, -1 linear; 3, -3, 1 quadratic).
static AspcCoef extrapolation_coefficients(int order) {
    AspcCoef c{};
    double b = 1.0;
    for (int j = 1; j <= order + 1 && j <= 6; ++j) {
        b = b * double(order + 2 - j) / double(j);   // C(order+1, j)
        c.b[j - 1] = (j & 1) ? b : -b;
    }
    return c;
}

// mu = sum_j B_j mu(t - j h) over the history, newest first (SOURCE/aspc.f90:143-170).
// With `carried` (the initial guess of a converged solve) a site keeps the caller's dipole
// unless it is the newest history entry (the caller carried the last step's dipoles over).
__global__ void k_aspc_predict(int n, int m, int head, AspcCoef c, const double* __restrict__ hist,
                               double* __restrict__ mx, double* __restrict__ my, double* __restrict__ mz,
                               int carried) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* out[3] = {mx, my, mz};
    if (carried) {
        const double* h0 = hist + (size_t)head * 3 * n;
        if (mx[i] != h0[i] || my[i] != h0[n + i] || mz[i] != h0[2 * (size_t)n + i]) return;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double v = 0.0;
        for (int j = 0; j < m; ++j) {
            const int slot = (head + j) % m;
            v += c.b[j] * hist[((size_t)slot * 3 + d) * n + i];
        }
        out[d][i] = v;
    }
}

cudaError_t PolarState::aspc_predict(int n, double* mx, double* my, double* mz, cudaStream_t s) {
    cudaError_t e;
    const int m = aspc_slots();
    if (!aspc_hist || aspc_n != n) {   // a new history (aspc_init): zeroed, the step count restarts
        if (aspc_hist) cudaFree(aspc_hist);
        aspc_hist = nullptr;
        if ((e = cudaMalloc(&aspc_hist, (size_t)m * 3 * n * sizeof(double)))) return e;
        if ((e = cudaMemsetAsync(aspc_hist, 0, (size_t)m * 3 * n * sizeof(double), s))) return e;
        aspc_n = n;
        aspc_head = 0;
        aspc_step = 0;
    }
    ++aspc_step;
    if (aspc_k && aspc_step > aspc_niter) {   // as aspc_predict's test (slots not yet filled are zeros)
        k_aspc_predict<<<blocks(n, kThreads), kThreads, 0, s>>>(n, m, aspc_head, aspc_coefficients(aspc_k),
                                                                aspc_hist, mx, my, mz, 0);
        ++launches;
    } else if (guess_order && aspc_step > m) {   // m steps in the history
        k_aspc_predict<<<blocks(n, kThreads), kThreads, 0, s>>>(n, m, aspc_head,
                                                                extrapolation_coefficients(guess_order), aspc_hist,
                                                                mx, my, mz, 1);
        ++launches;
    }
    return cudaSuccess;
}

cudaError_t PolarState::aspc_push(int n, const double* mx, const double* my, const double* mz, cudaStream_t s) {
    const int m = aspc_slots();
    aspc_head = (aspc_head + m - 1) % m;
    const double* src[3] = {mx, my, mz};
    for (int d = 0; d < 3; ++d) {
        const cudaError_t e = cudaMemcpyAsync(aspc_hist + ((size_t)aspc_head * 3 + d) * n, src[d], n * sizeof(double),
                                              cudaMemcpyDeviceToDevice, s);
        if (e) return e;
    }
    return cudaSuccess;
}

cudaError_t PolarState::table(double alpha, double rcut, cudaStream_t s) {
    if (ercp && alpha == tab_alpha && rcut == tab_rcut) return cudaSuccess;
    if (ercp) cudaFree(ercp);
    if (ercp32) cudaFree(ercp32);
    ercp = nullptr;
    ercp32 = nullptr;
    mxegrd = std::max(1000, (int)(rcut / 0.0001 + 0.5) + 4);
    drewd = rcut / double(mxegrd - 4);
    std::vector<double4> h((size_t)mxegrd + 1, make_double4(0, 0, 0, 0));
    for (int i = 1; i <= mxegrd; ++i) {   // erfcgenp (SOURCE/erfcgenp.f:26-46)
        const double rrr = double(i) * drewd;
        const double rsqi = 1.0 / rrr / rrr;
        const double a = alpha * rrr;
        double c[4];
        c[0] = (erfcc(a) - 1.0) / rrr;
        const double exp2a = std::exp(-a * a);
        for (int n = 1; n <= 3; ++n) {
            const double fn = n;
            c[n] = rsqi * ((2.0 * fn - 1.0) * c[n - 1] + std::pow(2.0 * (alpha * alpha), fn) * exp2a / alpha / kSqrpi);
        }
        h[i] = make_double4(c[0], c[1], c[2], c[3]);
    }
    // the mixed path's FP32 table: C_n = B_n + (2n-1)!!/r^(2n+1), the screened functions
    // themselves (row 0, r = 0, is never read: sites of different waters are not that close)
    std::vector<float4> h32(h.size(), make_float4(0.f, 0.f, 0.f, 0.f));
    for (int i = 1; i <= mxegrd; ++i) {
        const double r = double(i) * drewd, ri = 1.0 / r, r2i = ri * ri;
        const double c0 = h[i].x + ri, c1 = h[i].y + ri * r2i, c2 = h[i].z + 3.0 * ri * r2i * r2i,
                     c3 = h[i].w + 15.0 * ri * r2i * r2i * r2i;
        h32[i] = make_float4((float)c0, (float)c1, (float)c2, (float)c3);
    }
    cudaError_t e;
    if ((e = cudaMalloc(&ercp, h.size() * sizeof(double4)))) return e;
    if ((e = cudaMalloc(&ercp32, h32.size() * sizeof(float4)))) return e;
    // stream-ordered and complete before the host vector goes (a plain cudaMemcpy from
    // pageable memory may return before its DMA lands, unordered with non-blocking streams)
    if ((e = cudaMemcpyAsync(ercp, h.data(), h.size() * sizeof(double4), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaMemcpyAsync(ercp32, h32.data(), h32.size() * sizeof(float4), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    tab_alpha = alpha;
    tab_rcut = rcut;
    return cudaSuccess;
}

// Cell-list buffers of the pair-list build: sort keys and indices (n) and cell bounds.
cudaError_t PolarState::reserve_cells(int n, int ncell) {
    cudaError_t e;
    if (n > cell_n_cap) {
        void* p[] = {ckey, cskey, cidx, csidx, csort};
        for (void* q : p)
            if (q) cudaFree(q);
        ckey = cskey = nullptr;
        cidx = csidx = nullptr;
        csort = nullptr;
        cell_n_cap = 0;
        const size_t m = (size_t)std::max(n, 1);
        if ((e = cudaMalloc(&ckey, m * sizeof(unsigned)))) return e;
        if ((e = cudaMalloc(&cskey, m * sizeof(unsigned)))) return e;
        if ((e = cudaMalloc(&cidx, m * sizeof(int)))) return e;
        if ((e = cudaMalloc(&csidx, m * sizeof(int)))) return e;
        size_t b = 0;
        if ((e = cub::DeviceRadixSort::SortPairs(nullptr, b, ckey, cskey, cidx, csidx, (int)m))) return e;
        if ((e = cudaMalloc(&csort, std::max(b, (size_t)1)))) return e;
        csort_bytes = b;
        cell_n_cap = n;
    }
    if (ncell > ncell_cap) {
        if (cstart) cudaFree(cstart);
        if (cend) cudaFree(cend);
        cstart = cend = nullptr;
        ncell_cap = 0;
        if ((e = cudaMalloc(&cstart, ncell * sizeof(int)))) return e;
        if ((e = cudaMalloc(&cend, ncell * sizeof(int)))) return e;
        ncell_cap = ncell;
    }
    return cudaSuccess;
}

// The skin list (cap_s partners per site) and the positions of its build.
cudaError_t PolarState::reserve_skin(int n) {
    cudaError_t e;
    if (n > ns_cap || cap_s != cap_s_alloc) {
        void* p[] = {nn_s, nbr_s, npol_s, nup_s, xref};
        for (void* q : p)
            if (q) cudaFree(q);
        nn_s = nbr_s = npol_s = nullptr;
        nup_s = nullptr;
        xref = nullptr;
        ns_cap = cap_s_alloc = 0;
        skin_ok = false;
        const size_t m = (size_t)std::max(n, 1);
        if ((e = cudaMalloc(&nn_s, m * sizeof(int)))) return e;
        if ((e = cudaMalloc(&npol_s, m * sizeof(int)))) return e;
        if ((e = cudaMalloc(&nup_s, m * sizeof(int2)))) return e;
        if ((e = cudaMalloc(&nbr_s, m * cap_s * sizeof(int)))) return e;
        if ((e = cudaMalloc(&xref, 3 * m * sizeof(double)))) return e;
        ns_cap = n;
        cap_s_alloc = cap_s;
    }
    return cudaSuccess;
}

cudaError_t PolarState::reserve_part(size_t nd) {
    if (nd <= part_cap) return cudaSuccess;
    if (kpart) cudaFree(kpart);
    kpart = nullptr;
    part_cap = 0;
    cudaError_t e = cudaMalloc(&kpart, std::max(nd, (size_t)1) * sizeof(double));
    if (!e) part_cap = nd;
    return e;
}

cudaError_t PolarState::reserve_mixed(int n, int K, size_t nfac) {
    cudaError_t e;
    if (!tens32 || cap32 != cap || n > n32) {
        void* p[] = {tens32, r32, d32, e32, cg_x, cg_r, cg_q, cg_z, vh32};
        for (void* q : p)
            if (q) cudaFree(q);
        tens32 = e32 = nullptr;
        r32 = d32 = cg_x = cg_r = cg_q = cg_z = vh32 = nullptr;
        cap32 = n32 = 0;
        const size_t m = (size_t)std::max(n, 1);
        if ((e = cudaMalloc(&tens32, 6 * m * cap * sizeof(float)))) return e;
        if ((e = cudaMalloc(&r32, m * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&d32, m * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&e32, 6 * m * sizeof(float)))) return e;
        if ((e = cudaMalloc(&cg_x, m * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&cg_r, m * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&cg_q, m * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&vh32, 3 * m * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&cg_z, m * sizeof(float4)))) return e;
        cap32 = cap;
        n32 = n;
    }
    if (K > k32) {
        void* p[] = {kco32, kaux};
        for (void* q : p)
            if (q) cudaFree(q);
        kco32 = nullptr;
        kaux = nullptr;
        k32 = 0;
        const size_t kk = (size_t)std::max(K, 1);
        if ((e = cudaMalloc(&kco32, 16 * kk * sizeof(float)))) return e;
        if ((e = cudaMalloc(&kaux, kk * sizeof(int4)))) return e;
        k32 = K;
    }
    const size_t need = nfac * n;
    if (need > fac32_cap) {
        if (fac32) cudaFree(fac32);
        fac32 = nullptr;
        fac32_cap = 0;
        if ((e = cudaMalloc(&fac32, std::max(need, (size_t)1) * sizeof(float2)))) return e;
        fac32_cap = need;
    }
    const int nt = (K + kSfThreads - 1) / kSfThreads;
    if (nt > ktile_cap) {
        if (ktile) cudaFree(ktile);
        ktile = nullptr;
        ktile_cap = 0;
        if ((e = cudaMalloc(&ktile, std::max(nt, 1) * sizeof(int4)))) return e;
        ktile_cap = nt;
    }
    return cudaSuccess;
}

cudaError_t PolarState::reserve(int nw, int K, size_t nfac) {
    cudaError_t e;
    const int n = 4 * nw;
    if (!acc && (e = cudaMalloc(&acc, 64 * sizeof(double)))) return e;
    if (!acc_h && (e = cudaMallocHost(&acc_h, 64 * sizeof(double)))) return e;
    if (!flag && (e = cudaMalloc(&flag, 8 * sizeof(int)))) return e;
    // a capacity is zeroed before its buffers are replaced, so a failed allocation leaves
    // nothing that a later call would take for allocated
    if (n > n_cap || cap != cap_alloc) {
        void* p[] = {nn, nbr, npol, nup, xf, tens, fld, vesp, ae, md, vh, polr6};
        for (void* q : p)
            if (q) cudaFree(q);
        n_cap = 0;
        cap_alloc = 0;
        nn = nbr = npol = nullptr;
        nup = nullptr;
        xf = nullptr;
        tens = fld = vesp = ae = vh = polr6 = nullptr;
        md = nullptr;
        const size_t m = (size_t)std::max(n, 1);
        if ((e = cudaMalloc(&nn, m * sizeof(int)))) return e;
        if ((e = cudaMalloc(&npol, m * sizeof(int)))) return e;
        if ((e = cudaMalloc(&nup, m * sizeof(int2)))) return e;
        if ((e = cudaMalloc(&nbr, m * cap * sizeof(int)))) return e;
        if ((e = cudaMalloc(&xf, m * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&tens, 6 * m * cap * sizeof(double)))) return e;
        if ((e = cudaMalloc(&fld, 12 * m * sizeof(double)))) return e;
        if ((e = cudaMalloc(&vesp, m * sizeof(double)))) return e;
        if ((e = cudaMalloc(&ae, m * sizeof(double)))) return e;
        if ((e = cudaMalloc(&md, m * sizeof(double4)))) return e;
        if ((e = cudaMalloc(&vh, 12 * m * sizeof(double)))) return e;
        if ((e = cudaMalloc(&polr6, 2 * m * sizeof(double)))) return e;
        n_cap = n;
        cap_alloc = cap;
    }
    if (nw > nw_cap) {
        if (intra) cudaFree(intra);
        intra = nullptr;
        nw_cap = 0;
        // FP64 tensors, then their FP32 copy
        if ((e = cudaMalloc(&intra, 18 * (size_t)std::max(nw, 1) * (sizeof(double) + sizeof(float))))) return e;
        nw_cap = nw;
    }
    if (K > k_cap) {
        void* p[] = {kv, kx2, lmn, sf, kterm, kco, kcol, colk};
        for (void* q : p)
            if (q) cudaFree(q);
        kv = nullptr;
        kx2 = nullptr;
        lmn = nullptr;
        sf = kterm = kco = nullptr;
        kcol = nullptr;
        colk = nullptr;
        k_cap = 0;
        if ((e = cudaMalloc(&kv, K * sizeof(double4)))) return e;
        if ((e = cudaMalloc(&kx2, K * sizeof(double2)))) return e;
        if ((e = cudaMalloc(&lmn, K * sizeof(int4)))) return e;
        if ((e = cudaMalloc(&sf, 8 * (size_t)K * sizeof(double)))) return e;
        if ((e = cudaMalloc(&kterm, 16 * (size_t)K * sizeof(double)))) return e;
        if ((e = cudaMalloc(&kco, 16 * (size_t)K * sizeof(double)))) return e;
        if ((e = cudaMalloc(&kcol, K * sizeof(int)))) return e;
        if ((e = cudaMalloc(&colk, K * sizeof(int2)))) return e;
        k_cap = K;
    }
    const size_t need = (size_t)K * n;
    if (need > eik_cap) {
        if (eik) cudaFree(eik);
        eik = nullptr;
        eik_cap = 0;
        if ((e = cudaMalloc(&eik, std::max(need, (size_t)1) * sizeof(double2)))) return e;
        eik_cap = need;
    }
    if (nfac * n > fac_cap) {
        if (fac) cudaFree(fac);
        fac = nullptr;
        fac_cap = 0;
        if ((e = cudaMalloc(&fac, std::max(nfac * n, (size_t)1) * sizeof(double2)))) return e;
        fac_cap = nfac * n;
    }
    return cudaSuccess;
}

// The dynamic shared-memory cap of the FP32 k-space kernels.  The attribute is process-wide
// (per device), so it is raised once to a fixed bound rather than per call: contexts on other
// threads launch the same kernels with their own sizes.
static cudaError_t allow_dynamic_smem() {
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(dev)) return cudaSuccess;
    const void* f[] = {(const void*)k_pol_sfd32, (const void*)k_pol_sfx32<0>, (const void*)k_pol_sfx32<1>,
                       (const void*)k_pol_kfield32, (const void*)k_pol_kforce32};
    for (const void* q : f)
        if ((e = cudaFuncSetAttribute(q, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxDynSmem))) return e;
    done.insert(dev);
    return cudaSuccess;
}

cudaError_t PolarState::run(int precision, const Cell& cl, const double* prm, int nw, const double* x, const double* y,
                            const double* z, const double* q, const double* dp, const double* polr,
                            const double* polr2, double* mx, double* my, double* mz, double* fx, double* fy,
                            double* fz, double* ae_out, const double* vx, const double* vy, const double* vz,
                            double* out16, double* jpot, double* jkin, cudaStream_t s) {
    cudaError_t e;
    converged = false;
    bool forked = false;   // fork_hook called (the caller's work runs beside the solve)
    iterations = 0;
    launches = 0;
    const int n = 4 * nw;
    const double alpha = prm[0], rcut = prm[1], epsq = prm[2];
    const int kmax[3] = {(int)prm[11], (int)prm[12], (int)prm[13]};
    const int maxit = (int)prm[14];
    if ((e = table(alpha, rcut, s))) return e;

    // k vectors in ewald1p's order (SOURCE/ewald1p.f:159-172, :279-348)
    double rc[9];
    {
        const double* a = cl.c;
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
    auto widths = [](const double* aa, double* w3, double* vol) {
        const double axb1 = aa[1] * aa[5] - aa[2] * aa[4], axb2 = aa[2] * aa[3] - aa[0] * aa[5],
                     axb3 = aa[0] * aa[4] - aa[1] * aa[3];
        const double bxc1 = aa[4] * aa[8] - aa[5] * aa[7], bxc2 = aa[5] * aa[6] - aa[3] * aa[8],
                     bxc3 = aa[3] * aa[7] - aa[4] * aa[6];
        const double cxa1 = aa[7] * aa[2] - aa[1] * aa[8], cxa2 = aa[0] * aa[8] - aa[2] * aa[6],
                     cxa3 = aa[1] * aa[6] - aa[0] * aa[7];
        const double v = std::fabs(aa[0] * bxc1 + aa[1] * bxc2 + aa[2] * bxc3);
        w3[0] = v / std::sqrt(bxc1 * bxc1 + bxc2 * bxc2 + bxc3 * bxc3);
        w3[1] = v / std::sqrt(cxa1 * cxa1 + cxa2 * cxa2 + cxa3 * cxa3);
        w3[2] = v / std::sqrt(axb1 * axb1 + axb2 * axb2 + axb3 * axb3);
        *vol = v;
    };
    double wc[3], wr[3], volm, vr;
    widths(cl.c, wc, &volm);
    widths(rc, wr, &vr);
    const double twopi = 2.0 * kPi;
    const double rvolm = twopi / volm, ralph = -0.25 / (alpha * alpha);
    double rcpcut = std::min(std::min(double(kmax[0]) * wr[0], double(kmax[1]) * wr[1]), double(kmax[2]) * wr[2]);
    rcpcut = rcpcut * 1.05 * twopi;
    const double rcpct2 = rcpcut * rcpcut;
    hk.clear();
    hk2.clear();
    hlmn.clear();
    const bool spme_on = spme_order > 0;
    if (!spme_on) {
        int mmin = 0, nmin = 1;
        for (int ll = 0; ll <= kmax[0]; ++ll) {
            const double t0 = twopi * double(ll);
            const double rkx1 = t0 * rc[0], rky1 = t0 * rc[3], rkz1 = t0 * rc[6];
            for (int mm = mmin; mm <= kmax[1]; ++mm) {
                const double t1 = twopi * double(mm);
                const double rkx2 = rkx1 + t1 * rc[1], rky2 = rky1 + t1 * rc[4], rkz2 = rkz1 + t1 * rc[7];
                for (int nn_ = nmin; nn_ <= kmax[2]; ++nn_) {
                    const double t2 = twopi * double(nn_);
                    const double rkx3 = rkx2 + t2 * rc[2], rky3 = rky2 + t2 * rc[5], rkz3 = rkz2 + t2 * rc[8];
                    const double rksq = rkx3 * rkx3 + rky3 * rky3 + rkz3 * rkz3;
                    if (rksq <= rcpct2) {
                        const double rrksq = 1.0 / rksq;
                        hk.push_back(make_double4(rkx3, rky3, rkz3, std::exp(ralph * rksq) * rrksq));
                        hk2.push_back(make_double2(rksq, 2.0 * (rrksq - ralph)));
                        hlmn.push_back(make_int4(ll, mm, nn_, 0));
                    }
                }
                nmin = -kmax[2];
            }
            mmin = -kmax[1];
        }
    }
    const int K = (int)hk.size();
    if (n > 65535L * kThreads) return cudaErrorInvalidValue;
    const size_t nfac = (size_t)(kmax[0] + 1) + (2 * kmax[1] + 1) + (2 * kmax[2] + 1);
    if ((e = reserve(nw, K, nfac))) return e;
    if (precision == 1 && (e = reserve_mixed(n, K, nfac))) return e;
    if (K) {
        if ((e = cudaMemcpyAsync(kv, hk.data(), K * sizeof(double4), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaMemcpyAsync(kx2, hk2.data(), K * sizeof(double2), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaMemcpyAsync(lmn, hlmn.data(), K * sizeof(int4), cudaMemcpyHostToDevice, s))) return e;
    }
    const bool heat = vx && vy && vz;
    const bool mixed = precision == 1;
    inner_sweeps = 0;
    // FP32 structure factors: per tile of kSfThreads k vectors the x and y factor rows it
    // uses (k vectors come l-major, so a tile spans few l); the widest tile sizes the
    // shared-memory rows (odd, so the transposed stores spread over the banks)
    int rowp = 1, rowp2 = 1;
    const int nkt = (K + kSfThreads - 1) / kSfThreads, nkt2 = (nkt + 1) / 2;
    // the (l, m) columns of the k vectors (runs of n): l << 16 | y row, first k and count
    hkcol.clear();
    hcolk.clear();
    std::vector<int> col(K);
    for (int q = 0; q < K; ++q) {
        if (q == 0 || hlmn[q].x != hlmn[q - 1].x || hlmn[q].y != hlmn[q - 1].y) {
            hkcol.push_back((hlmn[q].x << 16) | (kmax[0] + 1 + kmax[1] + hlmn[q].y));
            hcolk.push_back(make_int2(q, 0));
        }
        col[q] = (int)hkcol.size() - 1;
        ++hcolk.back().y;
    }
    const int ncols = (int)hkcol.size();
    if (K) {
        if ((e = cudaMemcpyAsync(kcol, hkcol.data(), ncols * sizeof(int), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaMemcpyAsync(colk, hcolk.data(), ncols * sizeof(int2), cudaMemcpyHostToDevice, s))) return e;
    }
    if (mixed && K) {
        // each tile's first column and count, and per k its column within the tile, the
        // next column, its column and the offset of its z row in the gathers' shared memory
        hktile.resize(nkt);
        hkaux.resize(K);
        for (int t = 0; t < nkt; ++t) {
            const int b = t * kSfThreads, e_ = std::min(K, b + kSfThreads);
            hktile[t] = make_int4(col[b], col[e_ - 1] - col[b] + 1, 0, 0);
            rowp = std::max(rowp, hktile[t].y + 2 * kmax[2] + 1);
            for (int q = b; q < e_; ++q)
                hkaux[q] = make_int4(col[q] - col[b], hkcol[std::min(col[q] + 1, ncols - 1)], col[q],
                                     (hlmn[q].z + kmax[2]) * kThreads);
        }
        rowp |= 1;
        // k_pol_sfd32 takes two tiles per block: the rows of both
        for (int t = 0; t < nkt; t += 2) {
            const int4 ta = hktile[t], tb = t + 1 < nkt ? hktile[t + 1] : ta;
            rowp2 = std::max(rowp2, std::max(ta.x + ta.y, tb.x + tb.y) - ta.x + 2 * kmax[2] + 1);
        }
        rowp2 |= 1;
        if ((e = cudaMemcpyAsync(ktile, hktile.data(), nkt * sizeof(int4), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaMemcpyAsync(kaux, hkaux.data(), K * sizeof(int4), cudaMemcpyHostToDevice, s))) return e;
    }
    const size_t sfd_smem = kSfTile * (sizeof(float4) + (size_t)rowp2 * sizeof(float2));
    const size_t sfx_smem0 = kSfTile * (sizeof(float4) + (size_t)rowp * sizeof(float2)),
                 sfx_smem1 = kSfTile * (4 * sizeof(float4) + (size_t)rowp * sizeof(float2));
    const size_t gat_smem = gather_smem(kmax);
    if (mixed && K) {
        // the FP32 k-space passes keep their factor rows in shared memory (kmax up to ~100)
        if (rowp > kMaxRows || sfx_smem1 > kMaxDynSmem || sfd_smem > kMaxDynSmem || gat_smem > kMaxDynSmem)
            return cudaErrorInvalidValue;
        if ((e = allow_dynamic_smem())) return e;
    }

    PolArgs a;
    auto bind = [&](PolArgs& b) {
        b.cap = cap;
        b.ercp = ercp;
        b.ercp32 = ercp32;
        b.drewd = drewd;
        b.rdrewd = 1.0 / drewd;
        b.nn = nn;
        b.nbr = nbr;
        b.npol = npol;
        b.nup = nup;
        b.tens = tens;
        b.tens32 = mixed ? tens32 : nullptr;
        b.intra = intra;
        b.intra32 = reinterpret_cast<float*>(intra + 18 * (size_t)std::max(nw, 1));
        b.efk = fld;
        b.efc = fld + 3 * (size_t)n;
        b.emu = fld + 6 * (size_t)n;
        b.efm = fld + 9 * (size_t)n;
        b.vesp = vesp;
        b.ae = ae;
        b.polr6 = polr6;
        b.rpolr6 = polr6 + n;
        b.acc = acc;
    };
    a.cl = cl;
    a.nw = nw;
    a.n = n;
    a.x = x; a.y = y; a.z = z; a.q = q; a.polr = polr; a.polr2 = polr2; a.dp = dp;
    a.mx = mx; a.my = my; a.mz = mz;
    a.vx = vx; a.vy = vy; a.vz = vz;
    a.fx = fx; a.fy = fy; a.fz = fz;
    a.gamma = prm[10];
    a.alpha = alpha;
    a.rcut = rcut;
    a.rcsq = rcut * rcut;
    a.eps = epsq;
    a.athole = prm[5]; a.athole12 = prm[6]; a.athole13 = prm[7]; a.ascc = prm[8]; a.ascd = prm[9];
    a.toler = prm[3];
    a.omega = prm[4];
    // ASPC (SOURCE/forces.f:334-366): once aspc_niter steps are past, the dipoles predicted
    // from the history (aspc_predict before forces, SOURCE/dlpoly_cmd.f:2273-2283) and one
    // corrector iteration; SOR weight 0.3 for the first four steps
    bool aspc_one = false;
    if (aspc_k) {
        if ((e = aspc_predict(n, mx, my, mz, s))) return e;
        if (aspc_step < 5) a.omega = 0.3;
        aspc_one = aspc_step > aspc_niter;
    } else if (guess_order && (e = aspc_predict(n, mx, my, mz, s))) {   // the start of a converged solve
        return e;
    }
    bind(a);

    KArgs k;
    // every buffer pointer of the k-space kernels; bound again whenever a reserve may have
    // reallocated them (the list growth below)
    auto bindk = [&](KArgs& b) {
        b.kv = kv;
        b.kx2 = kx2;
        b.lmn = lmn;
        b.fac = fac;
        b.eik = eik;
        b.fac32 = mixed ? fac32 : nullptr;
        b.ktile = mixed ? ktile : nullptr;
        b.kaux = mixed ? kaux : nullptr;
        b.kcol = kcol;
        b.colk = colk;
        b.kco32 = mixed ? kco32 : nullptr;
        b.sf = sf;
        b.kco = kco;
        b.kterm = kterm;
        b.md = md;
        b.vh = vh;
    };
    k.K = K;
    k.n = n;
    for (int c = 0; c < 3; ++c) k.kmax[c] = kmax[c];
    k.q = q;
    bindk(k);
    for (int c = 0; c < 9; ++c) k.rc[c] = rc[c];
    k.scale = 4.0 * rvolm * kR4pie0 / epsq;
    k.ralph = ralph;
    k.sfac = 2.0 * rvolm * kR4pie0 / epsq;

    if ((e = cudaMemsetAsync(acc, 0, 64 * sizeof(double), s))) return e;
    K_last = K;
    if (profiling) {
        for (auto& v : ev)
            if (!v && (e = cudaEventCreate(&v))) return e;
        if ((e = cudaEventRecord(ev[0], s))) return e;
    }
    if (n == 0) {
        for (int c = 0; c < 16; ++c) out16[c] = 0.0;
        converged = true;
        return cudaSuccess;
    }
    // list (grows until every row fits); cell-sorted candidates where the box allows.  With a
    // skin the pairs within rcut + skin are kept between calls (rebuilt when a site moved more
    // than skin / 2) and the exact list is filtered from them each call.
    const double skin = list_skin > 0.0 ? list_skin : 0.0;
    last_n = n;
    // the shell of the FP64 test: +-0.001 A about rcut, 0.018 A^2 in r^2 at 9 A, 18 times the
    // FP32 error bound of r^2 below (a warp holding one shell entry runs its FP64 test: a
    // thinner shell is fewer such warps)
    const float r2f = (float)((rcut + 0.001) * (rcut + 0.001));
    const float r2in = rcut > 0.002 ? (float)((rcut - 0.001) * (rcut - 0.001)) : 0.f;
    auto build = [&](int* lnn, int* lnbr, int* lnpol, int2* lnup, int rowcap, double lcut) -> cudaError_t {
        // one pass of k_pol_list at cut lcut into (lnn, lnbr); the overflow flag is read by the caller
        cudaError_t err;
        int3 nc = make_int3(1, 1, 1);
        int cells = 0;
        if (cl.imcon == 1 || cl.imcon == 2) {
            const double wcell = lcut + 0.02;
            nc = make_int3((int)(cl.c[0] / wcell), (int)(cl.c[4] / wcell), (int)(cl.c[8] / wcell));
            cells = nc.x >= 3 && nc.y >= 3 && nc.z >= 3 && (long)nc.x * nc.y * nc.z < (1L << 24);
            if (!cells) nc = make_int3(1, 1, 1);
        }
        if (cells) {
            if ((err = reserve_cells(n, nc.x * nc.y * nc.z))) return err;
            k_pol_keys<<<blocks(n, kThreads), kThreads, 0, s>>>(n, x, y, z, cl, nc, ckey, cidx);
            size_t b = csort_bytes;
            if ((err = cub::DeviceRadixSort::SortPairs(csort, b, ckey, cskey, cidx, csidx, n, 0, 32, s))) return err;
            if ((err = cudaMemsetAsync(cstart, 0, (size_t)nc.x * nc.y * nc.z * sizeof(int), s))) return err;
            if ((err = cudaMemsetAsync(cend, 0, (size_t)nc.x * nc.y * nc.z * sizeof(int), s))) return err;
            k_pol_bounds<<<blocks(n, kThreads), kThreads, 0, s>>>(n, cskey, cstart, cend);
            launches += 3;
        }
        const float lf = (float)((lcut + 0.01) * (lcut + 0.01));
        const float li = lcut > 0.02 ? (float)((lcut - 0.01) * (lcut - 0.01)) : 0.f;
        k_pol_list<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, lnn, lnbr, lnpol, lnup, rowcap, lcut, xf, lf,
                                                                   li, flag, nc, cells, csidx, cstart, cend);
        ++launches;
        return cudaGetLastError();
    };
    auto read_flags = [&](int* h2) -> cudaError_t {
        cudaError_t err;
        if ((err = cudaMemcpyAsync(acc_h, flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s))) return err;
        if ((err = cudaStreamSynchronize(s))) return err;
        std::memcpy(h2, acc_h, 2 * sizeof(int));
        return cudaSuccess;
    };
    bind(a);
    k_pol_f32<<<blocks(n, kThreads), kThreads, 0, s>>>(n, x, y, z, xf);
    ++launches;
    if (skin > 0.0) {
        if ((e = reserve_skin(n))) return e;
        bool same = skin_ok && skin_n == n && skin_rcut == rcut && skin_delr == skin && skin_imcon == cl.imcon &&
                    std::equal(cl.c, cl.c + 9, skin_cell);
        for (;;) {
            if (same) {
                // the movement test and the filter of the kept list, one host read for both
                bind(a);
                if ((e = cudaMemsetAsync(flag, 0, 2 * sizeof(int), s))) return e;
                k_pol_moved<<<blocks(n, kThreads), kThreads, 0, s>>>(n, x, y, z, xref, cl, 0.25 * skin * skin,
                                                                     flag + 1);
                k_pol_filter<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, nn_s, nbr_s, npol_s, nup_s, cap_s, nn,
                                                                            nbr, npol, nup, xf, r2f, r2in, flag);
                launches += 2;
                int fh[2];
                if ((e = read_flags(fh))) return e;
                if (fh[1]) {
                    same = false;
                } else if (fh[0]) {
                    cap = std::min(2 * cap, std::max(n, 32));
                    if ((e = reserve(nw, K, nfac))) return e;
                    if (mixed && (e = reserve_mixed(n, K, nfac))) return e;
                    // reserve() reallocates the FP32 positions with the rows
                    k_pol_f32<<<blocks(n, kThreads), kThreads, 0, s>>>(n, x, y, z, xf);
                    ++launches;
                    continue;
                } else {
                    break;
                }
            }
            // (re)build the skin list at rcut + skin until every row fits
            for (;;) {
                if ((e = cudaMemsetAsync(flag, 0, 2 * sizeof(int), s))) return e;
                bind(a);
                if ((e = build(nn_s, nbr_s, npol_s, nup_s, cap_s, rcut + skin))) return e;
                int fh[2];
                if ((e = read_flags(fh))) return e;
                if (!fh[0]) break;
                cap_s = std::min(2 * cap_s, std::max(n, 32));
                if ((e = reserve_skin(n))) return e;
            }
            k_pol_ref<<<blocks(n, kThreads), kThreads, 0, s>>>(n, x, y, z, xref);
            ++launches;
            ++list_builds;
            skin_ok = true;
            skin_n = n;
            skin_rcut = rcut;
            skin_delr = skin;
            skin_imcon = cl.imcon;
            std::copy(cl.c, cl.c + 9, skin_cell);
            same = true;
        }
    } else {
        skin_ok = false;
        for (;;) {
            bind(a);
            if ((e = cudaMemsetAsync(flag, 0, 2 * sizeof(int), s))) return e;
            if ((e = build(nn, nbr, npol, nup, cap, rcut))) return e;
            int fh[2];
            if ((e = read_flags(fh))) return e;
            if (!fh[0]) break;
            cap = std::min(2 * cap, std::max(n, 32));   // a row holds at most n - 1 sites
            if ((e = reserve(nw, K, nfac))) return e;
            if (mixed && (e = reserve_mixed(n, K, nfac))) return e;
            k_pol_f32<<<blocks(n, kThreads), kThreads, 0, s>>>(n, x, y, z, xf);
            ++launches;
        }
        ++list_builds;
    }
    bind(a);
    bindk(k);
    k_pol_polr6<<<blocks(n, kThreads), kThreads, 0, s>>>(a, polr6);
    k_pol_static<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a);
    k_pol_intra_static<<<blocks(6L * nw, 64), 64, 0, s>>>(a);   // a thread per excluded pair
    launches += 3;
    k_pol_mask<<<blocks(n, kThreads), kThreads, 0, s>>>(a, md);
    ++launches;
    if (spme_on) {
        int Kg[3];
        for (int c = 0; c < 3; ++c)
            Kg[c] = spme_grid[0] > 0 ? spme_grid[c] : spme_smooth_even(wc[c] / spme_spacing);
        for (int c = 0; c < 3; ++c) spme_K_last[c] = Kg[c];
        if ((e = spme.prepare(cl.c, alpha, spme_order, Kg, mixed, heat ? 9 : 1, s))) return e;
        // the site frame of this call's positions (grid indices, FP32 fractions, FP64 splines)
        if ((e = spme.frame(n, x, y, z, s))) return e;
        ++launches;
    }
    if (K) {
        k_pol_factors<<<blocks(n, kThreads), kThreads, 0, s>>>(k, x, y, z);
        dim3 g(ncols, blocks(n, kThreads));   // sites per column along y (n < 65535 * 128)
        k_pol_phase<<<g, kThreads, 0, s>>>(k);
        k_pol_sfq<<<K, kSfThreads, 0, s>>>(k, q);
        launches += 3;
    }
    if (profiling && (e = cudaEventRecord(ev[1], s))) return e;
    double deltadip = 0.0;
    // k vectors per chunk of the field / force gathers: about four blocks per SM in all
    const int sblk2 = (int)blocks(n, 2 * kThreads), sblk1 = (int)blocks(n, kThreads);
    // A grid that is not a multiple of the SM count leaves some SMs one block (or a last
    // short wave) longer than the rest: take the smallest chunk count from the four-per-SM
    // target up to four times it that makes sites x chunks a multiple of the SMs, when
    // there is one.
    auto chunking = [&](int sblk, int& kchunk, int& nchunk) {
        int want = std::max(1, (4 * nsm + sblk - 1) / sblk);
        for (int c = want; c <= 4 * want; ++c)
            if (((long)sblk * c) % nsm == 0) {
                want = c;
                break;
            }
        kchunk = std::max(kKTile, (int)(((K + want - 1) / want + kKTile - 1) / kKTile) * kKTile);
        nchunk = K ? (K + kchunk - 1) / kchunk : 0;
    };
    int kc2, nc2, kc1, nc1;
    chunking(sblk2, kc2, nc2);
    chunking(sblk1, kc1, nc1);
    // FP32 structure factors: site chunks so that the grid holds about four blocks per SM
    const int nsc = nkt ? std::max(1, std::min((n + kSfTile - 1) / kSfTile, (4 * nsm + nkt - 1) / nkt)) : 1;
    const int schunk = ((n + nsc - 1) / nsc + kSfTile - 1) / kSfTile * kSfTile;
    const int nsc_used = (n + schunk - 1) / schunk;
    // k_pol_sfd32 (two tiles per block): its own site chunks for about four blocks per SM
    const int nsc2 = nkt2 ? std::max(1, std::min((n + kSfTile - 1) / kSfTile, (4 * nsm + nkt2 - 1) / nkt2)) : 1;
    const int schunk2 = ((n + nsc2 - 1) / nsc2 + kSfTile - 1) / kSfTile * kSfTile;
    const int nsc2_used = (n + schunk2 - 1) / schunk2;
    if ((e = reserve_part(std::max(std::max(std::max((size_t)6 * std::max(nc1, nc2) * n, (size_t)30 * nsc_used * K),
                                            (size_t)2 * nsc2_used * K),
                                   spme_on ? (size_t)5 * n : (size_t)0))))
        return e;
    // self term of the k-space dipole field (SOURCE/ewald1p.f), added with every field
    const double dum_self = 4.0 * kR4pie0 * (alpha * alpha * alpha) / kSqrpi / 3.0;
    cudaError_t field_err = cudaSuccess;   // a failed SPME field evaluation (checked after each)
    int kf_calls = 0;          // profiling: k_pol_kfield launches of this call with events
    double kf_call_flops = 0.0;
    auto fields64 = [&](bool first) {
        k_pol_dd<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a);
        if (spme_on) {
            const cudaError_t fe =
                spme.field64(n, x, y, z, first ? q : nullptr, md, polr2, mx, my, mz, k.sfac, dum_self, a.efm, a.efc, s);
            if (fe && !field_err) field_err = fe;
            launches += 1 + spme.launches;
            return;
        }
        if (K) {
            k_pol_sfd<<<K, kSfThreads, 0, s>>>(k);
            const bool timed = profiling && kf_calls < kKfEvents;
            if (timed) {
                for (auto& v : kfev[kf_calls])
                    if (!v) cudaEventCreate(&v);
                cudaEventRecord(kfev[kf_calls][0], s);
            }
            k_pol_kfield<<<dim3(sblk2, nc2), kThreads, 0, s>>>(k, first, kc2, kpart);
            if (timed) {
                cudaEventRecord(kfev[kf_calls][1], s);
                // algorithmic flops per (k vector, site): 9, and 9 more for the static field
                kf_call_flops += (first ? 18.0 : 9.0) * K * (double)n;
                ++kf_calls;
            }
        }
        k_pol_kfield_sum<<<sblk1, kThreads, 0, s>>>(k, a, first, nc2, kpart);
        launches += K ? 4 : 2;
    };
    auto sor64 = [&]() -> cudaError_t {   // iter, then read the rms change
        cudaError_t err;
        if (field_err) return field_err;
        if ((err = cudaMemsetAsync(acc + 27, 0, 2 * sizeof(double), s))) return err;
        k_pol_iter<<<blocks(n, kThreads), kThreads, 0, s>>>(a, md, mixed ? d32 : nullptr);
        ++launches;
        if ((err = cudaMemcpyAsync(acc_h + 27, acc + 27, 2 * sizeof(double), cudaMemcpyDeviceToHost, s))) return err;
        if ((err = cudaStreamSynchronize(s))) return err;
        deltadip = std::sqrt(acc_h[27] / (acc_h[28] > 0.0 ? acc_h[28] : 1.0));
        return cudaSuccess;
    };
    if (aspc_one) {   // one iteration, then marked converged (SOURCE/forces.f:361-366)
        fields64(true);
        if ((e = sor64())) return e;
        iterations = 1;
        converged = true;
    } else if (!mixed) {
        for (int it = 1;; ++it) {
            fields64(it == 1);
            if ((e = sor64())) return e;
            iterations = it;
            if (deltadip <= prm[3]) {
                converged = true;
                break;
            }
            if (it >= maxit) break;
        }
    } else {
        // FP64 refinement: the residual of the FP64 fields decides; the correction is solved
        // by FP32 conjugate gradients; the last step is the FP64 SOR update of the reference.
        MixArgs m;
        m.r32 = r32;
        m.d32 = d32;
        m.e32 = e32;
        m.x = cg_x;
        m.rho = cg_r;
        m.q = cg_q;
        const double fac = 1.0 - a.omega;
        // z = M^-1 rho into cg_z, rho.z into acc[slot] (and the first direction); `pre`
        // Jacobi sweeps (odd: the polynomial is positive definite for every eigenvalue of
        // D^-1 T_real below 1, which the dipole equations guarantee)
        // with SPME a CG sweep's k space is cheap beside two more real-space sweeps: the
        // diagonal; with the Ewald sum the polynomial's fewer sweeps pay
        int pre = (precond_sweeps > 0 ? precond_sweeps : (spme_on ? 1 : 3)) | 1;
        // the block-Jacobi preconditioner (per-water 9x9 inverses), in place of the sweeps
        bool blk = precond_block && nw > 0;
        if (blk) {
            if (binv_cap < nw) {
                if (binv) cudaFree(binv);
                binv = nullptr;
                binv_cap = 0;
                if ((e = cudaMalloc(&binv, 81 * (size_t)nw * sizeof(float)))) return e;
                binv_cap = nw;
            }
            k_pcg_block_setup<<<blocks(nw, 64), 64, 0, s>>>(a, (float)dum_self, binv);
            ++launches;
        }
        auto precondition = [&](int slot, int dir) -> cudaError_t {
            if (blk) {
                k_pcg_block<<<blocks(n, kThreads), kThreads, 0, s>>>(a, m, binv, cg_z, -1, nullptr, 0.0, nullptr);
                ++launches;
            } else {
                k_pcg_jacobi<<<blocks(n, kThreads), kThreads, 0, s>>>(a, m, nullptr, cg_z);
                for (int q = 1; q < pre; ++q) {
                    k_pol_dd32<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, cg_z, e32 + 3 * (size_t)n);
                    k_pcg_jacobi<<<blocks(n, kThreads), kThreads, 0, s>>>(a, m, e32 + 3 * (size_t)n, cg_z);
                    launches += 2;
                }
            }
            cudaError_t err;
            if ((err = cudaMemsetAsync(acc + slot, 0, sizeof(double), s))) return err;
            k_pcg_rz<<<blocks(n, kThreads), kThreads, 0, s>>>(a, m, cg_z, slot, dir);
            launches += 2;
            return cudaSuccess;
        };
        double rms_prev = HUGE_VAL;
        bool corrected = false;   // the dipoles changed by k_pol_apply since the last evaluation
        // the field evaluation after a correction: FP64 real space; k space the previous
        // FP64 fields plus the FP32 ones of the correction
        auto fields_delta = [&]() {
            // real space: the previous FP64 field + the FP32 field of the correction
            k_pol_dd32<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, d32, e32);
            if (spme_on) {   // k space likewise: the FP32 SPME field of the correction
                const cudaError_t fe =
                    spme.field32(n, x, y, z, d32, polr2, k.sfac, dum_self, e32 + 3 * (size_t)n, s, nullptr);
                if (fe && !field_err) field_err = fe;
                k_pol_field_add<<<blocks(n, kThreads), kThreads, 0, s>>>(a, e32, 1, 1);
                launches += 2 + spme.launches;
                return;
            }
            k_pol_field_add<<<blocks(n, kThreads), kThreads, 0, s>>>(a, e32, 1, 0);
            launches += 2;
            if (K) {
                k_pol_sfx32<0><<<dim3(nkt, nsc_used), kSfThreads, sfx_smem0, s>>>(k, d32, vh32, schunk, rowp, kpart);
                k_pol_sfd_dfin<<<blocks(K, kThreads), kThreads, 0, s>>>(k, nsc_used, kpart);
                k_pol_kfield32<<<dim3(sblk1, nc1), kThreads, gat_smem, s>>>(k, kc1, (float*)kpart);
                launches += 3;
            }
            k_pol_kfield32_dsum<<<sblk1, kThreads, 0, s>>>(k, a, m, K ? nc1 : 0, (const float*)kpart);
            launches += 2;
        };
        for (int it = 1;; ++it) {
            if (corrected) fields_delta();
            else fields64(it == 1);
            corrected = false;
            if (field_err) return field_err;
            if ((e = cudaMemsetAsync(acc + 29, 0, 3 * sizeof(double), s))) return e;
            k_pol_resid<<<blocks(n, kThreads), kThreads, 0, s>>>(a, m);
            ++launches;
            if ((e = cudaMemcpyAsync(acc_h + 29, acc + 29, 3 * sizeof(double), cudaMemcpyDeviceToHost, s))) return e;
            if ((e = cudaStreamSynchronize(s))) return e;
            const double rms = std::sqrt(acc_h[29] / (acc_h[30] > 0.0 ? acc_h[30] : 1.0));
            const double rms_mu = std::sqrt(acc_h[31] / (acc_h[30] > 0.0 ? acc_h[30] : 1.0));
            iterations = it;
            if (fac * rms <= prm[3] || it >= maxit) {
                if ((e = sor64())) return e;
                converged = deltadip <= prm[3];
                break;
            }
            // an outer step that did not halve the FP64 residual: the diagonal preconditioner
            // from here on
            if ((pre > 1 || blk) && !(rms <= 0.5 * rms_prev)) {
                pre = 1;
                blk = false;
            }
            rms_prev = rms;
            // |z| (the preconditioned residual of the correction, a dipole) down to
            // 1e-6 of the FP64 residual or 5x below toler
            const double target = std::max(1e-6 * rms, 0.2 * prm[3]);
            bool broke = false;
            // The sweeps are enqueued in batches without host round trips: the stopping test
            // runs on the device (k_pcg_next), and once it has stopped the solve, the rest of
            // the batch returns at once.  The host reads the state after each batch; the first
            // batch is as long as the previous solve took.
            if (fork_hook && !forked) {
                if ((e = fork_hook())) return e;
                forked = true;
            }
            int* cgs = flag + 2;
            MixArgs ms = m;
            ms.stop = cgs;
            KArgs ks = k;
            ks.stop = cgs;
            for (bool restart = true; restart;) {
                restart = false;
                broke = false;
                if ((e = cudaMemsetAsync(acc + 33, 0, 5 * sizeof(double), s))) return e;
                if ((e = cudaMemsetAsync(cgs, 0, 3 * sizeof(int), s))) return e;   // state, sweeps, ticket
                k_pcg_init<<<blocks(n, kThreads), kThreads, 0, s>>>(a, m);
                ++launches;
                const bool poly = pre > 1 || blk;
                if (poly && (e = precondition(33, 1))) return e;
                int queued = 0, batch = std::max(2, std::min(cg_hint, 40));
                int st[2] = {0, 0};
                while (queued < 100) {
                    for (int b = 0; b < batch && queued < 100; ++b, ++queued) {
                        k_pol_dd32<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, d32, e32, cgs);
                        if (spme_on) {
                            if ((e = spme.field32(n, x, y, z, d32, polr2, k.sfac, dum_self, e32 + 3 * (size_t)n, s,
                                                  cgs)))
                                return e;
                            launches += spme.launches;
                        } else if (K) {
                            k_pol_sfd32<<<dim3(nkt2, nsc2_used), kSfThreads, sfd_smem, s>>>(ks, ms, schunk2, rowp2,
                                                                                            kpart);
                            k_pol_sfd32_sum<<<blocks(K, kThreads), kThreads, 0, s>>>(ks, nsc2_used, kpart);
                            k_pol_kfield32<<<dim3(sblk1, nc1), kThreads, gat_smem, s>>>(ks, kc1, (float*)kpart);
                            k_pol_kfield32_sum<<<sblk1, kThreads, 0, s>>>(ks, a, ms, nc1, (const float*)kpart);
                            launches += 4;
                        }
                        k_pcg_ad<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ms, (K || spme_on) ? 1 : 0);
                        // the diagonal preconditioner: the stopping test in k_pcg_step's last block
                        k_pcg_step<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ms, poly ? nullptr : cgs, target,
                                                                            cgs + 2, blk ? 1 : 0);
                        if (poly && blk) {
                            // z, rho.z (in place of k_pcg_step's diagonal one) and the stopping test
                            k_pcg_block<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ms, binv, cg_z, 35, cgs, target,
                                                                                 cgs + 2);
                            ++launches;
                        } else if (poly) {
                            k_pcg_jacobi<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ms, nullptr, cg_z);
                            for (int qq = 1; qq < pre; ++qq) {
                                k_pol_dd32<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, cg_z, e32 + 3 * (size_t)n,
                                                                                           cgs);
                                k_pcg_jacobi<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ms, e32 + 3 * (size_t)n,
                                                                                     cg_z);
                                launches += 2;
                            }
                            // rho.z of the polynomial z replaces k_pcg_step's diagonal one
                            if ((e = cudaMemsetAsync(acc + 35, 0, sizeof(double), s))) return e;
                            k_pcg_rz<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ms, cg_z, 35, 0);
                            launches += 2;
                        }
                        // fused stopping test (diagonal: in k_pcg_step; block: in k_pcg_block)
                        const bool fused = !poly || blk;
                        k_pcg_dir<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ms, poly ? cg_z : nullptr, fused ? 1 : 0);
                        if (!fused) {
                            k_pcg_next<<<1, 32, 0, s>>>(acc, cgs, target);
                            ++launches;
                        }
                        launches += 4;
                    }
                    if ((e = cudaMemcpyAsync(acc_h + 60, cgs, 2 * sizeof(int), cudaMemcpyDeviceToHost, s))) return e;
                    if ((e = cudaStreamSynchronize(s))) return e;
                    std::memcpy(st, acc_h + 60, 2 * sizeof(int));
                    if (st[0] != 0) break;
                    batch = 2;
                }
                inner_sweeps += st[1];
                cg_hint = std::max(2, st[1]);
                // d.Ad <= 0 (or a non-finite sum): the preconditioned operator is not
                // positive definite in FP32 here; the diagonal preconditioner takes over,
                // and with it an FP64 SOR step replaces this correction
                if (st[0] == 2) {
                    if (pre > 1 || blk) {
                        pre = 1;
                        blk = false;
                        restart = true;
                    } else {
                        broke = true;
                    }
                }
            }
            if (broke) {
                if ((e = sor64())) return e;
            } else {
                k_pol_apply<<<blocks(n, kThreads), kThreads, 0, s>>>(a, m, md);
                ++launches;
                // the next FP64 evaluation adds the FP32 k-space field of this correction to the
                // previous one; its FP32 rounding (1e-7 of the correction's field) stays in the
                // fields of every later residual, so a correction that is not small against
                // the dipoles (a cold start's first) is followed by a full FP64 evaluation
                corrected = rms <= 1e-4 * rms_mu;
            }
        }
    }
    // aspc_set (SOURCE/dlpoly_cmd.f:2318-2320): the step's dipoles join the history
    if ((aspc_k || guess_order) && (e = aspc_push(n, mx, my, mz, s))) return e;
    // final pass: after the caller's work that ran beside the solve (its kernels may add to
    // the same force arrays); with no CG solve, that work runs here, before the pass
    if (fork_hook && !forked) {
        if ((e = fork_hook())) return e;
        forked = true;
    }
    if (forked && join_hook && (e = join_hook())) return e;
    const double g34 = std::exp(gammln(3.0 / 4.0));
    const bool mfin = mixed && !final_fp64;   // the final pass's FP32 forms
    if (heat) {
        const bool w32 = mfin && !spme_on;   // the FP32 Ewald heat sums take FP32 weights
        k_pol_vhat<<<blocks(n, kThreads), kThreads, 0, s>>>(a, md, w32 ? nullptr : vh, w32 ? vh32 : nullptr);
        ++launches;
    }
    if (profiling && (e = cudaEventRecord(ev[2], s))) return e;
    if (K) {
        if (mfin) {   // the last FP64 structure factors plus FP32 ones of the last update
            const dim3 g(nkt, nsc_used);
            if (heat) {
                k_pol_sfx32<1><<<g, kSfThreads, sfx_smem1, s>>>(k, d32, vh32, schunk, rowp, kpart);
                k_pol_sfx32_fin<1><<<blocks(K, kThreads), kThreads, 0, s>>>(k, nsc_used, kpart);
            } else {
                k_pol_sfx32<0><<<g, kSfThreads, sfx_smem0, s>>>(k, d32, vh32, schunk, rowp, kpart);
                k_pol_sfx32_fin<0><<<blocks(K, kThreads), kThreads, 0, s>>>(k, nsc_used, kpart);
            }
            launches += 2;
        } else {
            if (heat) k_pol_sf_final<1><<<K, kSfThreads, 0, s>>>(k);
            else k_pol_sf_final<0><<<K, kSfThreads, 0, s>>>(k);
            ++launches;
        }
    }
    if (spme_on) {
        if ((e = spme.final(n, x, y, z, q, md, heat ? vh : nullptr, k.sfac, kpart, acc, nullptr, s, mfin))) return e;
        launches += spme.launches;
    }
    if (profiling && (e = cudaEventRecord(ev[3], s))) return e;
    if (K) {
        if (mfin) k_pol_kforce32<<<dim3(sblk1, nc1), kThreads, gat_smem, s>>>(k, a, kc1, kpart);
        else k_pol_kforce<<<dim3(sblk2, nc2), kThreads, 0, s>>>(k, a, kc2, kpart);
        ++launches;
    }
    k_pol_kforce_sum<<<sblk1, kThreads, 0, s>>>(k, a, spme_on ? 1 : (mfin ? nc1 : nc2), kpart);
    if (mfin && !ewald2p_fp64)
        k_pol_ewald2p32<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, g34, gammln(0.75), heat);
    else
        k_pol_ewald2p<<<blocks(32L * n, kThreads), kThreads, 0, s>>>(a, g34, heat);
    // thread per water, FP64-latency bound: one-warp blocks spread them over every SM
    k_pol_ewald3p<<<blocks(6L * nw, 64), 64, 0, s>>>(a, heat);   // a thread per excluded pair
    k_pol_qdforce<<<blocks(4L * nw, 64), 64, 0, s>>>(a, heat);   // a thread per (water, site)
    k_pol_jkin<<<blocks(n, kThreads), kThreads, 0, s>>>(a, ae_out, heat);
    launches += 5;
    if (K) {
        k_pol_kreduce<<<1, kSfThreads, 0, s>>>(K, kterm, acc + 48);
        ++launches;
    }
    if ((e = cudaGetLastError())) return e;
    if (profiling && (e = cudaEventRecord(ev[4], s))) return e;
    if ((e = cudaMemcpyAsync(acc_h, acc, 64 * sizeof(double), cudaMemcpyDeviceToHost, s))) return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    if (profiling) {
        for (int q = 0; q < 4; ++q)
            if ((e = cudaEventElapsedTime(&phase_ms[q], ev[q], ev[q + 1]))) return e;
        kf_ms = 0.f;
        for (int q = 0; q < kf_calls; ++q) {
            float t = 0.f;
            if ((e = cudaEventElapsedTime(&t, kfev[q][0], kfev[q][1]))) return e;
            kf_ms += t;
        }
        kf_launches = kf_calls;
        kf_flops = kf_call_flops;
    }
    const double* h = acc_h;
    // acc: 0 eng_real, 1 vir, 2..7 stress (11 12 13 22 23 33), 8..10 jpot (real + qd),
    //      24..26 jkin, 27..28 iteration sums, 40 engsic, 41 eng_polar,
    //      48 engc, 49 engdum, 50..55 omg (11 22 33 12 13 23), 56..58 jpot (k space)
    const double scal1 = 2.0 * rvolm * kR4pie0 / epsq;
    const bool kon = K || spme_on;
    const double engc = kon ? h[48] : 0.0, eng1 = kon ? h[49] : 0.0;
    const double omg11 = kon ? h[50] : 0.0, omg22 = kon ? h[51] : 0.0, omg33 = kon ? h[52] : 0.0;
    const double omg12 = kon ? h[53] : 0.0, omg13 = kon ? h[54] : 0.0, omg23 = kon ? h[55] : 0.0;
    const double engk = 2.0 * rvolm * kR4pie0 * engc / epsq + h[40];
    const double virk = -scal1 * (omg11 + omg22 + omg33 + 3.0 * eng1);
    double st[9];
    st[0] = h[2] + scal1 * (omg11 + eng1);
    st[1] = h[3] + scal1 * omg12;
    st[2] = h[4] + scal1 * omg13;
    st[3] = st[1];
    st[4] = h[5] + scal1 * (omg22 + eng1);
    st[5] = h[6] + scal1 * omg23;
    st[6] = st[2];
    st[7] = st[5];
    st[8] = h[7] + scal1 * (omg33 + eng1);
    out16[0] = engk + h[0] + h[41];
    out16[1] = h[1] + virk;
    for (int c = 0; c < 9; ++c) out16[2 + c] = st[c];
    out16[11] = iterations;
    out16[12] = deltadip;
    out16[13] = h[41];
    out16[14] = engk;
    out16[15] = h[0];
    if (heat) {
        for (int c = 0; c < 3; ++c) {
            jpot[c] += h[8 + c] + (kon ? h[56 + c] : 0.0);
            jkin[c] += h[24 + c];
        }
    }
    return cudaSuccess;
}

}  // namespace mbx
