// Short-range dispersion: DL_POLY van der Waals type 12, Tang-Toennies damped C6/r^6 +
// C8/r^8, with the reference's tables, Verlet list and heat-current bookkeeping.
//
//   tables   vv12/gg12 at r = i * dlrpot, i = 1..mxgrid, dlrpot = rcut / (mxgrid - 4)
//            (SOURCE/forgen.f:97, :262-270, :337-357; tang_toennies SOURCE/tang-toennies.f90)
//   list     pairs of atoms of different molecules within rcut + delr, kept until an atom
//            has moved more than delr / 2 (the Verlet list of SOURCE/parlst.f with the
//            intramolecular exclusions of SOURCE/exclude_ttm.f); built on the device from a
//            cell list
//   forces   srfrce2 (SOURCE/srfrce2.f:80-270): separation x_i - x_j imaged as
//            SOURCE/images.f, cut at rcut, 3-point interpolation of energy and -r dV/dr,
//            forces, virial, stress, per-atom energy halves, heat-current pair entries
//            (r_i - r_j)(f . (v_i + v_j)) with raw coordinates
//   lrc      lrcorrect for type 12 (SOURCE/lrcorrect.f:112-223), on the host
//
// One warp per atom; lanes take its list partners.  FP64 throughout.
#include "mbx_kernels.cuh"

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

namespace mbx {

namespace {

// --- tables (host) -----------------------------------------------------------------
double tt(int n, double x) {
    double sum = 1.0;
    for (int nn = n; nn >= 1; --nn) sum = 1.0 + sum * x / nn;
    double v = 1.0 - sum * std::exp(-x);
    if (std::fabs(v) < 1.0e-8) {   // small-x series branch of the reference
        double term = 1.0;
        for (int nn = n; nn >= 1; --nn) term = term * x / nn;
        sum = 0.0;
        for (int nn = n + 1; nn <= 1000; ++nn) {
            term = term * x / nn;
            sum = sum + term;
            if (std::fabs(term / sum) < 1.0e-8) break;
        }
        v = sum * std::exp(-x);
    }
    return v;
}

// tang_toennies_lr with the reference's factorial (it multiplies by its argument at
// every step, giving z^z); kept because it defines the reference's correction.
double tt_lr(int n, double x) {
    double fact = 1.0;
    for (int i = n; i >= 1; --i) fact = fact * n;
    const double v = tt(n, x) / std::pow(x, n - 3) + std::exp(-x) * (x * x * (3.0 + x) + 6 * (1.0 + x)) / fact;
    return v / (n - 3);
}

// vv12 and gg12 = -r dV/dr; a term whose coefficient is 0 adds a signed zero in the
// reference and is skipped here (same value; tt(n, 0) would run its series loop out).
double v12(double r, const double* p) {
    double v = 0.0;
    if (p[0] != 0.0) v = -p[0] * tt(6, p[1] * r) / std::pow(r, 6);
    if (p[2] != 0.0) v = v - p[2] * tt(8, p[3] * r) / std::pow(r, 8);
    return v;
}

double g12(double r, const double* p) {
    double g6 = 0.0, g8 = 0.0, e6 = 0.0, e8 = 0.0;
    if (p[0] != 0.0) {
        g6 = -6 * p[0] * tt(6, p[1] * r) / std::pow(r, 6);
        e6 = r * p[0] * std::pow(p[1], 7) * std::exp(-p[1] * r) / 720;
    }
    if (p[2] != 0.0) {
        g8 = -8 * p[2] * tt(8, p[3] * r) / std::pow(r, 8);
        e8 = r * p[2] * std::pow(p[3], 9) * std::exp(-p[3] * r) / 40320;
    }
    return g6 + g8 + e6 + e8;
}

// --- device --------------------------------------------------------------------------
constexpr int kMaxTypes = 16;

struct DispArgs {
    int natms;
    Cell cl;
    const int* ltype;        // 1-based types, 0 = none
    const int* mol;
    const double *x, *y, *z;
    double *fx, *fy, *fz;
    const double *vx, *vy, *vz;
    double* ae;
    double* acc14;
    const double* vvv;       // [pair][mxgrid]
    const double* ggg;
    int mxgrid;
    double rcsq, rdr;
    unsigned vdw_types;      // bit t: type t has at least one dispersion partner
    unsigned long long vdw_pairs[3];   // bit k: pair type k has a nonzero table (k < 136)
};

__device__ __forceinline__ int pair_index(int ai, int aj) {
    return ai > aj ? ai * (ai - 1) / 2 + aj - 1 : aj * (aj - 1) / 2 + ai - 1;
}

__device__ __forceinline__ bool vdw_atom(const DispArgs& a, int i) {
    const int t = a.ltype[i];
    return t > 0 && t < kMaxTypes && ((a.vdw_types >> t) & 1u);
}

__device__ __forceinline__ int wrap(double s, int nc) {
    s = s - floor(s);
    int c = (int)(s * nc);
    return c >= nc ? nc - 1 : (c < 0 ? 0 : c);
}

__global__ void k_disp_keys(int natms, const double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ z, Cell cl, int3 nc, unsigned* __restrict__ key,
                            int* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= natms) return;
    key[i] = (unsigned)((wrap(z[i] * cl.inv[2], nc.z) * nc.y + wrap(y[i] * cl.inv[1], nc.y)) * nc.x +
                        wrap(x[i] * cl.inv[0], nc.x));
    idx[i] = i;
}

__global__ void k_disp_bounds(int n, const unsigned* __restrict__ skey, int* __restrict__ start,
                              int* __restrict__ end) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned c = skey[i];
    if (i == 0 || skey[i - 1] != c) start[c] = i;
    if (i == n - 1 || skey[i + 1] != c) end[c] = i + 1;
}

__device__ __forceinline__ double sep2(const Cell& cl, double dx, double dy, double dz) {
    image(cl, dx, dy, dz);
    return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}

// |image(d)|^2 in FP32, for the list build only (the forces cut at rcut in FP64).
__device__ __forceinline__ float sep2f(const Cell& cl, float dx, float dy, float dz) {
    if (cl.imcon == 1 || cl.imcon == 2) {
        dx -= (float)cl.c[0] * rintf(dx * (float)cl.inv[0]);
        dy -= (float)cl.c[4] * rintf(dy * (float)cl.inv[1]);
        dz -= (float)cl.c[8] * rintf(dz * (float)cl.inv[2]);
    } else {
        const double* r = cl.rc;
        const double* c = cl.c;
        float sx = (float)r[0] * dx + (float)r[3] * dy + (float)r[6] * dz;
        float sy = (float)r[1] * dx + (float)r[4] * dy + (float)r[7] * dz;
        float sz = (float)r[2] * dx + (float)r[5] * dy + (float)r[8] * dz;
        sx -= rintf(sx);
        sy -= rintf(sy);
        sz -= rintf(sz);
        dx = (float)c[0] * sx + (float)c[3] * sy + (float)c[6] * sz;
        dy = (float)c[1] * sx + (float)c[4] * sy + (float)c[7] * sz;
        dz = (float)c[2] * sx + (float)c[5] * sy + (float)c[8] * sz;
    }
    return dx * dx + dy * dy + dz * dz;
}

__global__ void k_disp_f32(int natms, const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ z, float4* __restrict__ xf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < natms) xf[i] = make_float4((float)x[i], (float)y[i], (float)z[i], 0.f);
}

// Verlet list: partners j > i of different molecules within rlist; warp per atom,
// candidates from the 27 cells around the atom's cell (or every atom), appended in
// candidate order.  The distance test runs in FP32 against rlist plus a margin far above
// FP32 rounding (rlist2f), so the list holds every pair within rlist; the force kernel
// applies the exact FP64 cut at rcut.
__global__ void k_disp_build(DispArgs a, int3 nc, int all_pairs, const int* __restrict__ sidx,
                             const int* __restrict__ cstart, const int* __restrict__ cend,
                             const float4* __restrict__ xf, float rlist2f, int cap, int* __restrict__ nn,
                             int* __restrict__ nbr, int* __restrict__ flag) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= a.natms) return;   // warp-uniform
    int cnt = 0;
    if (vdw_atom(a, i)) {
        const double xi = a.x[i], yi = a.y[i], zi = a.z[i];
        const float4 pi = xf[i];
        const int mi = a.mol[i];
        int* my = nbr + (size_t)i * cap;
        const int ncand_cells = all_pairs ? 1 : 27;
        for (int c = 0; c < ncand_cells; ++c) {
            int beg = 0, end = a.natms;
            if (!all_pairs) {
                const int cx = wrap(xi * a.cl.inv[0], nc.x), cy = wrap(yi * a.cl.inv[1], nc.y),
                          cz = wrap(zi * a.cl.inv[2], nc.z);
                const int ox = c % 3 - 1, oy = (c / 3) % 3 - 1, oz = c / 9 - 1;
                const int cc = (((cz + oz + nc.z) % nc.z) * nc.y + (cy + oy + nc.y) % nc.y) * nc.x +
                               (cx + ox + nc.x) % nc.x;
                beg = cstart[cc];
                end = cend[cc];
            }
            for (int b = beg; b < end; b += 32) {
                const int q = b + lane;
                bool hit = false;
                int j = 0;
                if (q < end) {
                    j = all_pairs ? q : sidx[q];
                    if (j > i && vdw_atom(a, j) && a.mol[j] != mi) {
                        const float4 pj = xf[j];
                        hit = sep2f(a.cl, pi.x - pj.x, pi.y - pj.y, pi.z - pj.z) < rlist2f;
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, hit);
                if (hit) {
                    const int slot = cnt + __popc(bal & ((1u << lane) - 1u));
                    if (slot < cap) my[slot] = j;
                }
                cnt += __popc(bal);
            }
        }
    }
    if (lane == 0) {
        nn[i] = min(cnt, cap);
        if (cnt > cap) atomicOr(flag, 1);
    }
}

// An atom that moved more than half the skin since the list was built asks for a rebuild.
__global__ void k_disp_moved(DispArgs a, const double* __restrict__ xref, double half_skin2, int* flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.natms || !vdw_atom(a, i)) return;
    if (sep2(a.cl, a.x[i] - xref[i], a.y[i] - xref[a.natms + i], a.z[i] - xref[2 * (size_t)a.natms + i]) >
        half_skin2)
        atomicOr(flag, 2);
}

__global__ void k_disp_ref(int natms, const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ z, double* __restrict__ xref) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= natms) return;
    xref[i] = x[i];
    xref[natms + i] = y[i];
    xref[2 * (size_t)natms + i] = z[i];
}

__global__ void __launch_bounds__(kThreads) k_disp_forces(DispArgs a, const int* __restrict__ nn,
                                                           const int* __restrict__ nbr, int cap) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double red[14];
#pragma unroll
    for (int q = 0; q < 14; ++q) red[q] = 0.0;
    double fi[3] = {0.0, 0.0, 0.0}, aei = 0.0;
    if (i < a.natms) {   // warp-uniform
        const int n = nn[i];
        const int ti = a.ltype[i];
        const double xi = a.x[i], yi = a.y[i], zi = a.z[i];
        for (int m = lane; m < n; m += 32) {
            const int j = nbr[(size_t)i * cap + m];
            const int k = pair_index(ti, a.ltype[j]);
            if (!((a.vdw_pairs[k >> 6] >> (k & 63)) & 1ull)) continue;
            double dx = dsub(xi, a.x[j]), dy = dsub(yi, a.y[j]), dz = dsub(zi, a.z[j]);
            const double rx = dx, ry = dy, rz = dz;   // the raw separation (the heat term's)
            image(a.cl, dx, dy, dz);
            const double rsq = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
            if (!(a.rcsq > rsq)) continue;
            const double rri = rsqrt_nr(rsq);   // r and 1/r^2 without an FP64 root and division
            const double rrr = rsq * rri;
            // l >= 1 unless two atoms are closer than one table step (the reference would
            // read before its table there); r < rcut keeps l + 2 <= mxgrid
            const int l = max((int)dmul(rrr, a.rdr), 1);
            const double ppp = dsub(dmul(rrr, a.rdr), (double)l);
            const double* vt = a.vvv + (size_t)k * a.mxgrid + (l - 1);
            const double* gt = a.ggg + (size_t)k * a.mxgrid + (l - 1);
            const double vk = vt[0], vk1 = vt[1], vk2 = vt[2];
            double t1 = dadd(vk, dmul(dsub(vk1, vk), ppp));
            double t2 = dadd(vk1, dmul(dsub(vk2, vk1), dsub(ppp, 1.0)));
            const double e = dadd(t1, dmul(dmul(dsub(t2, t1), ppp), 0.5));
            const double gk = gt[0], gk1 = gt[1], gk2 = gt[2];
            t1 = dadd(gk, dmul(dsub(gk1, gk), ppp));
            t2 = dadd(gk1, dmul(dsub(gk2, gk1), dsub(ppp, 1.0)));
            const double gamma = dadd(t1, dmul(dmul(dsub(t2, t1), ppp), 0.5)) * (rri * rri);
            const double f0 = gamma * dx, f1 = gamma * dy, f2 = gamma * dz;
            fi[0] += f0;
            fi[1] += f1;
            fi[2] += f2;
            atomicAdd(a.fx + j, -f0);
            atomicAdd(a.fy + j, -f1);
            atomicAdd(a.fz + j, -f2);
            red[0] += e;
            if (a.ae) {   // the row's half summed per lane, the partner's by an atomic
                aei += 0.5 * e;
                atomicAdd(a.ae + j, 0.5 * e);
            }
            red[1] -= gamma * rsq;
            // the stress's lower triangle (5, 8, 9) repeats 3, 4, 7: copied after the loop
            red[2] += dx * f0; red[3] += dx * f1; red[4] += dx * f2;
            red[6] += dy * f1; red[7] += dy * f2; red[10] += dz * f2;
            if (a.vx) {
                const double fv = f0 * (a.vx[i] + a.vx[j]) + f1 * (a.vy[i] + a.vy[j]) + f2 * (a.vz[i] + a.vz[j]);
                red[11] += rx * fv;
                red[12] += ry * fv;
                red[13] += rz * fv;
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) fi[c] = warp_sum(fi[c]);
        aei = warp_sum(aei);
        if (lane == 0 && (fi[0] != 0.0 || fi[1] != 0.0 || fi[2] != 0.0)) {
            atomicAdd(a.fx + i, fi[0]);
            atomicAdd(a.fy + i, fi[1]);
            atomicAdd(a.fz + i, fi[2]);
        }
        if (lane == 0 && a.ae && aei != 0.0) atomicAdd(a.ae + i, aei);
    }
    red[5] = red[3];
    red[8] = red[4];
    red[9] = red[7];
    block_sum_atomic<14>(red, a.acc14);
}

// The mixed-precision form of k_disp_forces: the separation, the image and the cut test in
// FP64 as there (the same pairs), the rest in FP32: the distance, the 3-point interpolation of
// FP32 copies of the tables, the forces, and per-lane FP32 partial sums of the forces,
// energies, virial, stress and heat terms, turned into FP64 for the warp and block sums
// and for the partner atomics.
__global__ void __launch_bounds__(kThreads) k_disp_forces32(DispArgs a, const int* __restrict__ nn,
                                                             const int* __restrict__ nbr, int cap,
                                                             const float* __restrict__ vvv32,
                                                             const float* __restrict__ ggg32,
                                                             const float4* __restrict__ vf, float rdr32) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    float rf[14];
#pragma unroll
    for (int q = 0; q < 14; ++q) rf[q] = 0.f;
    float fi[3] = {0.f, 0.f, 0.f}, aei = 0.f;
    if (i < a.natms) {   // warp-uniform
        const int n = nn[i];
        const int ti = a.ltype[i];
        const double xi = a.x[i], yi = a.y[i], zi = a.z[i];
        const float4 vi = vf ? vf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int m = lane; m < n; m += 32) {
            const int j = nbr[(size_t)i * cap + m];
            const int k = pair_index(ti, a.ltype[j]);
            if (!((a.vdw_pairs[k >> 6] >> (k & 63)) & 1ull)) continue;
            double dx = dsub(xi, a.x[j]), dy = dsub(yi, a.y[j]), dz = dsub(zi, a.z[j]);
            const float rx = (float)dx, ry = (float)dy, rz = (float)dz;   // the raw separation
            image(a.cl, dx, dy, dz);
            const double rsq = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
            if (!(a.rcsq > rsq)) continue;
            const float d0 = (float)dx, d1 = (float)dy, d2 = (float)dz;
            const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
            const float ri = rsqrtf(r2);
            const float u = r2 * ri * rdr32;
            const int l = max((int)u, 1);
            const float ppp = u - (float)l;
            const float* vt = vvv32 + (size_t)k * a.mxgrid + (l - 1);
            const float* gt = ggg32 + (size_t)k * a.mxgrid + (l - 1);
            float t1 = vt[0] + (vt[1] - vt[0]) * ppp;
            float t2 = vt[1] + (vt[2] - vt[1]) * (ppp - 1.f);
            const float e = t1 + (t2 - t1) * ppp * 0.5f;
            t1 = gt[0] + (gt[1] - gt[0]) * ppp;
            t2 = gt[1] + (gt[2] - gt[1]) * (ppp - 1.f);
            const float gamma = (t1 + (t2 - t1) * ppp * 0.5f) * (ri * ri);
            const float f0 = gamma * d0, f1 = gamma * d1, f2 = gamma * d2;
            fi[0] += f0;
            fi[1] += f1;
            fi[2] += f2;
            atomicAdd(a.fx + j, -(double)f0);
            atomicAdd(a.fy + j, -(double)f1);
            atomicAdd(a.fz + j, -(double)f2);
            rf[0] += e;
            if (a.ae) {
                aei += 0.5f * e;
                atomicAdd(a.ae + j, (double)(0.5f * e));
            }
            rf[1] -= gamma * r2;
            rf[2] += d0 * f0; rf[3] += d0 * f1; rf[4] += d0 * f2;
            rf[6] += d1 * f1; rf[7] += d1 * f2; rf[10] += d2 * f2;
            if (vf) {
                const float4 vj = vf[j];
                const float fv = f0 * (vi.x + vj.x) + f1 * (vi.y + vj.y) + f2 * (vi.z + vj.z);
                rf[11] += rx * fv;
                rf[12] += ry * fv;
                rf[13] += rz * fv;
            }
        }
        double fd[3] = {(double)fi[0], (double)fi[1], (double)fi[2]};
#pragma unroll
        for (int c = 0; c < 3; ++c) fd[c] = warp_sum(fd[c]);
        const double aed = warp_sum((double)aei);
        if (lane == 0 && (fd[0] != 0.0 || fd[1] != 0.0 || fd[2] != 0.0)) {
            atomicAdd(a.fx + i, fd[0]);
            atomicAdd(a.fy + i, fd[1]);
            atomicAdd(a.fz + i, fd[2]);
        }
        if (lane == 0 && a.ae && aed != 0.0) atomicAdd(a.ae + i, aed);
    }
    rf[5] = rf[3];
    rf[8] = rf[4];
    rf[9] = rf[7];
    double red[14];
#pragma unroll
    for (int q = 0; q < 14; ++q) red[q] = (double)rf[q];
    block_sum_atomic<14>(red, a.acc14);
}

// FP32 copies of the velocities (the mixed form's heat terms)
__global__ void k_disp_vf(int natms, const double* __restrict__ vx, const double* __restrict__ vy,
                          const double* __restrict__ vz, float4* __restrict__ vf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < natms) vf[i] = make_float4((float)vx[i], (float)vy[i], (float)vz[i], 0.f);
}

int grid(long threads) { return (int)((threads + kThreads - 1) / kThreads); }

}  // namespace

DispState::~DispState() { release(); }

void DispState::release() {
    void* p[] = {vvv, ggg, nn, nbr, xref, flag, key, skey, idx, sidx, cstart, cend, sort_tmp, vvv32, vf};
    for (void* q : p)
        if (q) cudaFree(q);
    vvv = ggg = xref = nullptr;
    vvv32 = nullptr;
    vf = nullptr;
    vf_cap = 0;
    nn = nbr = flag = idx = sidx = cstart = cend = nullptr;
    key = skey = nullptr;
    sort_tmp = nullptr;
    natms_cap = ncell_cap = 0;
    sort_bytes = 0;
    valid = false;
}

cudaError_t DispState::setup(int ntypes_, const double* prm_, double rcut_, double delr_, int mxgrid_) {
    cudaError_t e;
    if (vvv) cudaFree(vvv);
    if (ggg) cudaFree(ggg);
    if (vvv32) cudaFree(vvv32);
    vvv = ggg = nullptr;
    vvv32 = ggg32 = nullptr;
    ntypes = ntypes_;
    rcut = rcut_;
    delr = delr_;
    mxgrid = mxgrid_ > 0 ? mxgrid_ : std::max(1000, (int)(rcut / 0.0001 + 0.5) + 4);
    const int npair = ntypes * (ntypes + 1) / 2;
    prm.assign(prm_, prm_ + 4 * npair);
    const double dlrpot = rcut / double(mxgrid - 4);
    std::vector<double> hv((size_t)npair * mxgrid), hg((size_t)npair * mxgrid);
    vdw_types = 0;
    vdw_pairs[0] = vdw_pairs[1] = vdw_pairs[2] = 0;
    for (int k = 0; k < npair; ++k) {
        const double* p = prm.data() + 4 * k;
        if (p[0] == 0.0 && p[2] == 0.0) continue;   // no interaction: the table stays all zeros
        for (int i = 1; i <= mxgrid; ++i) {
            hv[(size_t)k * mxgrid + i - 1] = v12(i * dlrpot, p);
            hg[(size_t)k * mxgrid + i - 1] = g12(i * dlrpot, p);
        }
        if (hv[(size_t)k * mxgrid] != 0.0) {   // srfrce2 skips pair types whose table starts at 0
            vdw_pairs[k >> 6] |= 1ull << (k & 63);
            int ai = 1;
            while (ai * (ai + 1) / 2 <= k) ++ai;
            const int aj = k - ai * (ai - 1) / 2 + 1;
            vdw_types |= (1u << ai) | (1u << aj);
        }
    }
    if ((e = cudaMalloc(&vvv, hv.size() * sizeof(double)))) return e;
    if ((e = cudaMalloc(&ggg, hg.size() * sizeof(double)))) return e;
    if ((e = cudaMemcpy(vvv, hv.data(), hv.size() * sizeof(double), cudaMemcpyHostToDevice))) return e;
    if ((e = cudaMemcpy(ggg, hg.data(), hg.size() * sizeof(double), cudaMemcpyHostToDevice))) return e;
    {   // the FP32 copies of the mixed form (vvv32 then ggg32 in one allocation)
        std::vector<float> h32(2 * hv.size());
        for (size_t q = 0; q < hv.size(); ++q) {
            h32[q] = (float)hv[q];
            h32[hv.size() + q] = (float)hg[q];
        }
        if ((e = cudaMalloc(&vvv32, h32.size() * sizeof(float)))) return e;
        ggg32 = vvv32 + hv.size();
        if ((e = cudaMemcpy(vvv32, h32.data(), h32.size() * sizeof(float), cudaMemcpyHostToDevice))) return e;
    }
    // a copy from pageable memory may return before its DMA lands; the tables are read by
    // kernels on non-blocking streams, so wait for the copies here
    if ((e = cudaStreamSynchronize(cudaStreamLegacy))) return e;
    valid = false;
    return cudaSuccess;
}

// One evaluation on device arrays; out14 (device) = {E, virial, stress[9], jpot[3]}
// ACCUMULATED.  The list is rebuilt when it is missing, stale (an atom moved more than
// delr / 2), built for other inputs, or too small; `*rebuilt` reports it.
cudaError_t DispState::forces(const Cell& cl, int natms, const int* ltype, const int* mol, const double* x,
                              const double* y, const double* z, double* fx, double* fy, double* fz,
                              const double* vx, const double* vy, const double* vz, double* ae, double* out14,
                              int* flag_host, cudaStream_t s, bool* rebuilt, bool fp32) {
    cudaError_t e;
    *rebuilt = false;
    if (!vvv) return cudaErrorInvalidValue;
    DispArgs a;
    a.natms = natms;
    a.cl = cl;
    a.ltype = ltype;
    a.mol = mol;
    a.x = x; a.y = y; a.z = z;
    a.fx = fx; a.fy = fy; a.fz = fz;
    a.vx = vx; a.vy = vy; a.vz = vz;
    a.ae = ae;
    a.acc14 = out14;
    a.vvv = vvv;
    a.ggg = ggg;
    a.mxgrid = mxgrid;
    a.rcsq = rcut * rcut;
    a.rdr = 1.0 / (rcut / double(mxgrid - 4));
    a.vdw_types = vdw_types;
    for (int q = 0; q < 3; ++q) a.vdw_pairs[q] = vdw_pairs[q];
    if (natms > natms_cap) {
        void* p[] = {nn, nbr, xref, key, skey, idx, sidx, sort_tmp};
        for (void* q : p)
            if (q) cudaFree(q);
        nn = nbr = idx = sidx = nullptr;
        xref = nullptr;
        key = skey = nullptr;
        sort_tmp = nullptr;
        natms_cap = 0;   // until every buffer below exists
        cap_alloc = 0;
        const size_t n = (size_t)natms + 1;
        if ((e = cudaMalloc(&nn, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&nbr, n * cap * sizeof(int)))) return e;
        if ((e = cudaMalloc(&xref, 3 * n * sizeof(double)))) return e;
        if ((e = cudaMalloc(&key, n * sizeof(unsigned)))) return e;
        if ((e = cudaMalloc(&skey, n * sizeof(unsigned)))) return e;
        if ((e = cudaMalloc(&idx, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&sidx, n * sizeof(int)))) return e;
        size_t b = 0;
        if ((e = cub::DeviceRadixSort::SortPairs(nullptr, b, key, skey, idx, sidx, (int)n))) return e;
        sort_bytes = b;
        if ((e = cudaMalloc(&sort_tmp, sort_bytes))) return e;
        natms_cap = natms;
        cap_alloc = cap;
        valid = false;
    }
    if (!flag && (e = cudaMalloc(&flag, 4 * sizeof(int)))) return e;
    bool same = valid && natms == natms_last && ltype == ltype_last && mol == mol_last &&
                std::equal(cl.c, cl.c + 9, cell_last) && cl.imcon == imcon_last;
    if (same) {   // skin check
        if ((e = cudaMemsetAsync(flag, 0, sizeof(int), s))) return e;
        k_disp_moved<<<grid(natms), kThreads, 0, s>>>(a, xref, 0.25 * delr * delr, flag);
        if ((e = cudaMemcpyAsync(flag_host, flag, sizeof(int), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaStreamSynchronize(s))) return e;
        same = *flag_host == 0;
        ++launches;
    }
    for (int attempt = 0; !same; ++attempt) {
        // cells of at least rcut + delr; all pairs when fewer than 3 per side or triclinic
        const double rlist = rcut + delr;
        int3 nc = make_int3(1, 1, 1);
        int all_pairs = 1;
        if (cl.imcon == 1 || cl.imcon == 2) {
            nc = make_int3((int)(cl.c[0] / rlist), (int)(cl.c[4] / rlist), (int)(cl.c[8] / rlist));
            if (nc.x >= 3 && nc.y >= 3 && nc.z >= 3) all_pairs = 0;
            else nc = make_int3(1, 1, 1);
        }
        const int ncell = nc.x * nc.y * nc.z;
        if (ncell > ncell_cap) {
            if (cstart) cudaFree(cstart);
            if (cend) cudaFree(cend);
            cstart = cend = nullptr;
            ncell_cap = 0;
            if ((e = cudaMalloc(&cstart, ncell * sizeof(int)))) return e;
            if ((e = cudaMalloc(&cend, ncell * sizeof(int)))) return e;
            ncell_cap = ncell;
        }
        if (!all_pairs) {
            k_disp_keys<<<grid(natms), kThreads, 0, s>>>(natms, x, y, z, cl, nc, key, idx);
            size_t b = sort_bytes;
            if ((e = cub::DeviceRadixSort::SortPairs(sort_tmp, b, key, skey, idx, sidx, natms, 0, 32, s))) return e;
            if ((e = cudaMemsetAsync(cstart, 0, ncell * sizeof(int), s))) return e;
            if ((e = cudaMemsetAsync(cend, 0, ncell * sizeof(int), s))) return e;
            k_disp_bounds<<<grid(natms), kThreads, 0, s>>>(natms, skey, cstart, cend);
            launches += 3;
        }
        if ((e = cudaMemsetAsync(flag, 0, sizeof(int), s))) return e;
        // FP32 copies of the positions for the distance tests live in xref until the
        // build is done (the reference positions are written into it afterwards)
        float4* xf = (float4*)xref;
        k_disp_f32<<<grid(natms), kThreads, 0, s>>>(natms, x, y, z, xf);
        const double margin = 1.0e-3;   // Angstrom, >> FP32 rounding of coordinates below ~1e3 A
        const float rlist2f = (float)((rlist + margin) * (rlist + margin));
        k_disp_build<<<grid(32L * natms), kThreads, 0, s>>>(a, nc, all_pairs, sidx, cstart, cend, xf, rlist2f, cap,
                                                            nn, nbr, flag);
        k_disp_ref<<<grid(natms), kThreads, 0, s>>>(natms, x, y, z, xref);
        launches += 3;
        if ((e = cudaMemcpyAsync(flag_host, flag, sizeof(int), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaStreamSynchronize(s))) return e;
        if (!(*flag_host & 1)) {
            same = true;
            ++builds;
            *rebuilt = true;
            valid = true;
            natms_last = natms;
            ltype_last = ltype;
            mol_last = mol;
            imcon_last = cl.imcon;
            std::copy(cl.c, cl.c + 9, cell_last);
            break;
        }
        if (attempt >= 6 || cap >= natms + 32) return cudaErrorInvalidValue;
        cap = std::min(2 * cap, natms + 32);
        if (nbr) cudaFree(nbr);
        nbr = nullptr;
        const int keep = natms_cap;
        natms_cap = 0;   // the rows are gone until the new ones exist
        if ((e = cudaMalloc(&nbr, ((size_t)keep + 1) * cap * sizeof(int)))) return e;
        natms_cap = keep;
        cap_alloc = cap;
    }
    if (fp32) {
        const float4* vfp = nullptr;
        if (vx) {
            if (vf_cap < natms) {
                if (vf) cudaFree(vf);
                vf = nullptr;
                vf_cap = 0;
                if ((e = cudaMalloc(&vf, (size_t)natms * sizeof(float4)))) return e;
                vf_cap = natms;
            }
            k_disp_vf<<<grid(natms), kThreads, 0, s>>>(natms, vx, vy, vz, vf);
            vfp = vf;
            ++launches;
        }
        k_disp_forces32<<<grid(32L * natms), kThreads, 0, s>>>(a, nn, nbr, cap, vvv32, ggg32, vfp, (float)a.rdr);
    } else {
        k_disp_forces<<<grid(32L * natms), kThreads, 0, s>>>(a, nn, nbr, cap);
    }
    ++launches;
    return cudaGetLastError();
}

void disp_lrc(int ntypes, const double* prm, const int* numtyp, double rcut, double volm, double* elrc_out,
              double* virlrc_out) {
    const double twopi = 6.283185307179586;
    double plrc = 0.0, elrc = 0.0;
    for (int i = 1; i <= ntypes; ++i) {
        for (int j = 1; j <= i; ++j) {
            const double* p = prm + 4 * (i * (i - 1) / 2 + j - 1);
            // el12 and pl12 (a term whose coefficient is 0 is skipped, as in the tables)
            double e6 = 0.0, e8 = 0.0, p6 = 0.0, p8 = 0.0;
            if (p[0] != 0.0) {
                e6 = -p[0] * std::pow(p[1], 3) * tt_lr(6, p[1] * rcut);
                p6 = p[0] * tt(6, p[1] * rcut) / std::pow(rcut, 3);
            }
            if (p[2] != 0.0) {
                e8 = p[2] * std::pow(p[3], 5) * tt_lr(8, p[3] * rcut);
                p8 = p[2] * tt(8, p[3] * rcut) / std::pow(rcut, 5);
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

}  // namespace mbx
