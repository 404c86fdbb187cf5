// 1-body Partridge-Schwenke water PES (the MB-pol monomer term) with the angfrc
// bookkeeping: ps_type_couple (SOURCE/ps_type_couple.f90:15-274) called from angfrc
// for keya = 9 (SOURCE/angfrc.f:150-212, :344-545).  Eight lanes per H-O-H angle, FP64.
#include "mbx_kernels.cuh"
#include "mbx_pes_gen.cuh"

namespace mbx {

namespace {

__device__ __forceinline__ double c5z(int j) { return __longlong_as_double((long long)pes::kC5z[j]); }
__device__ __forceinline__ double cmass(int j) { return __longlong_as_double((long long)pes::kCmass[j]); }

// Lanes per angle: a group of kGroup lanes shares one angle's expansion terms.  The
// FP64 pipe of this part takes one warp instruction per 64 cycles however many lanes are
// active, so work that one lane does for an angle (the geometry, the exponential
// prefactor) is best done for several angles at once: four angles per warp.
constexpr int kGroup = 8;

__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = kGroup / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ps_type_couple for one angle on the kGroup lanes of a group (sub-lane s): the lanes
// share the 244 expansion terms and the 9 mass-correction terms, partial sums are
// reduced within the group.  Outputs (valid on every lane of the group): potential,
// the forces on the two H atoms (fa = f[0..2], fc = f[3..5]) and the virial term.
// Per term the derivative factors (i-1) x^(i-2) / reoh come from per-angle tables, and
// the virial term is assembled from the radial sums (vterm = roh1 * ra + roh2 * rc term
// by term, the same sum the reference accumulates separately).
__device__ void ps_couple_group(int s, double roh1, double xoh1, double yoh1, double zoh1, double roh2,
                                double xoh2, double yoh2, double zoh2, double theta, double& pterm_out, double* f,
                                double& vterm_out) {
    const double reoh = pes::kReoh, ireoh = 1.0 / pes::kReoh;
    const double cose = __longlong_as_double((long long)pes::kCose);
    const double cost = cos(theta);
    const double x1 = (roh1 - reoh) / reoh;
    const double x2 = (roh2 - reoh) / reoh;
    const double x3 = cost - cose;
    const double ir1 = 1.0 / roh1, ir2 = 1.0 / roh2;
    // fm[j][k] = x_k^(j-1); dm[j][k] = (j-1) x_k^(j-2) (/ reoh for the bond variables)
    double fm[16][3], dm[16][3];
    fm[0][0] = fm[0][1] = fm[0][2] = 0.0;
    fm[1][0] = fm[1][1] = fm[1][2] = 1.0;
    dm[0][0] = dm[0][1] = dm[0][2] = 0.0;
    dm[1][0] = dm[1][1] = dm[1][2] = 0.0;
#pragma unroll
    for (int j = 2; j <= 15; ++j) {
        fm[j][0] = fm[j - 1][0] * x1;
        fm[j][1] = fm[j - 1][1] * x2;
        fm[j][2] = fm[j - 1][2] * x3;
        dm[j][0] = (j - 1) * fm[j - 1][0] * ireoh;
        dm[j][1] = (j - 1) * fm[j - 1][1] * ireoh;
        dm[j][2] = (j - 1) * fm[j - 1][2];
    }
    double pterm = 0.0, ra = 0.0, aa = 0.0, rc = 0.0;
    for (int j = 1 + s; j < pes::kTerms; j += kGroup) {
        const int i1 = pes::kIdx[j][0], i2 = pes::kIdx[j][1], i3 = pes::kIdx[j][2];
        const double c = c5z(j);
        const double cz = c * fm[i3][2];
        const double dum = fm[i1][0] * fm[i2][1] + fm[i2][0] * fm[i1][1];
        pterm += cz * dum;
        ra += cz * (dm[i1][0] * fm[i2][1] + dm[i2][0] * fm[i1][1]);
        aa += c * dum * dm[i3][2];
        rc += cz * (fm[i1][0] * dm[i2][1] + fm[i2][0] * dm[i1][1]);
    }
    // mass-correction terms, one per lane (lane 0 also takes the ninth)
    const double xm = __longlong_as_double((long long)pes::kXm);
    const double e1x = xoh2 - cost * xoh1, e1y = yoh2 - cost * yoh1, e1z = zoh2 - cost * zoh1;
    const double e2x = xoh1 - cost * xoh2, e2y = yoh1 - cost * yoh2, e2z = zoh1 - cost * zoh2;
    double v12 = 0.0, pa = 0.0, q3 = 0.0, qa = 0.0, q4 = 0.0;
    for (int j = s; j < pes::kMass; j += kGroup) {
        const int m1 = pes::kIdxm[j][0], m2 = pes::kIdxm[j][1], m3 = pes::kIdxm[j][2];
        const double c = cmass(j);
        v12 += c * (fm[m1][0] * fm[m2][1] + fm[m2][0] * fm[m1][1]) * fm[m3][2];
        pa += c * xm * (dm[m1][0] * fm[m2][1] + dm[m2][0] * fm[m1][1]) * fm[m3][2];
        q3 += c * xm * (fm[m1][0] * fm[m2][1] + fm[m2][0] * fm[m1][1]) * dm[m3][2] * ir1;
        qa += c * xm * (fm[m1][0] * dm[m2][1] + fm[m2][0] * dm[m1][1]) * fm[m3][2];
        q4 += c * xm * (fm[m1][0] * fm[m2][1] + fm[m2][0] * fm[m1][1]) * dm[m3][2] * ir2;
    }
    pterm = group_sum(pterm);
    ra = group_sum(ra);
    aa = group_sum(aa);
    rc = group_sum(rc);
    v12 = group_sum(v12);
    pa = group_sum(pa);
    q3 = group_sum(q3);
    qa = group_sum(qa);
    q4 = group_sum(q4);
    double fa[3], fc[3];
    fa[0] = -(ra * xoh1 + aa * ir1 * e1x) - (pa * xoh1 + q3 * e1x);
    fa[1] = -(ra * yoh1 + aa * ir1 * e1y) - (pa * yoh1 + q3 * e1y);
    fa[2] = -(ra * zoh1 + aa * ir1 * e1z) - (pa * zoh1 + q3 * e1z);
    fc[0] = -(rc * xoh2 + aa * ir2 * e2x) - (qa * xoh2 + q4 * e2x);
    fc[1] = -(rc * yoh2 + aa * ir2 * e2y) - (qa * yoh2 + q4 * e2y);
    fc[2] = -(rc * zoh2 + aa * ir2 * e2z) - (qa * zoh2 + q4 * e2z);
    double vterm = roh1 * ra + roh2 * rc + roh1 * pa + roh2 * qa;
    pterm = pterm + xm * v12;
    const double b1 = pes::kB1;
    const double efac = exp(-b1 * ((roh1 - reoh) * (roh1 - reoh) + (roh2 - reoh) * (roh2 - reoh)));
    const double term = pterm;
    pterm = term * efac + c5z(0) + 2.0384848702093006e-6 * 2625.50 / 100.0;
    const double ga = 2.0 * b1 * (roh1 - reoh) * efac * term;
    const double gc = 2.0 * b1 * (roh2 - reoh) * efac * term;
    f[0] = fa[0] * efac + ga * xoh1;
    f[1] = fa[1] * efac + ga * yoh1;
    f[2] = fa[2] * efac + ga * zoh1;
    f[3] = fc[0] * efac + gc * xoh2;
    f[4] = fc[1] * efac + gc * yoh2;
    f[5] = fc[2] * efac + gc * zoh2;
    vterm = -2.0 * b1 * (roh1 - reoh) * roh1 * efac * term - 2.0 * b1 * (roh2 - reoh) * roh2 * efac * term + efac * vterm;
    pterm_out = pterm;
    vterm_out = vterm;
}

// Four angles per warp (kGroup lanes each); the first lane of each group accumulates.
__global__ void __launch_bounds__(kThreads) k_ps_pes(int nang, const int* __restrict__ listang, Cell cl,
                                                      const double* __restrict__ x, const double* __restrict__ y,
                                                      const double* __restrict__ z, double* fx, double* fy,
                                                      double* fz, double* ae, const double* __restrict__ vx,
                                                      const double* __restrict__ vy, const double* __restrict__ vz,
                                                      double* acc, const Cell* __restrict__ cells,
                                                      const int* __restrict__ abox, double* acc_box,
                                                      const int* __restrict__ skip) {
    if (skip && *skip) return;   // block-uniform
    const int lane = threadIdx.x & 31;
    const int sub = lane % kGroup;
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) / kGroup;
    const bool lead = sub == 0 && t < nang;
    // red = {E, virial, stress[9], jpot[3]} (the leading lane of each group)
    double red[14];
#pragma unroll
    for (int q = 0; q < 14; ++q) red[q] = 0.0;
    const int warp_first = (blockIdx.x * blockDim.x + (threadIdx.x & ~31)) / kGroup;
    if (warp_first < nang) {   // warp-uniform: every lane takes part in the group sums
        const int ta = min(t, nang - 1);   // groups past the end repeat the last angle, unused
        const int ia = listang[3 * ta] - 1, ib = listang[3 * ta + 1] - 1, ic = listang[3 * ta + 2] - 1;
        double xab = x[ia] - x[ib], yab = y[ia] - y[ib], zab = z[ia] - z[ib];
        double xbc = x[ic] - x[ib], ybc = y[ic] - y[ib], zbc = z[ic] - z[ib];
        if (cells) {
            image(cells[abox[ta]], xab, yab, zab);
            image(cells[abox[ta]], xbc, ybc, zbc);
        } else {
            image(cl, xab, yab, zab);
            image(cl, xbc, ybc, zbc);
        }
        const double rab = sqrt(xab * xab + yab * yab + zab * zab);
        const double rbc = sqrt(xbc * xbc + ybc * ybc + zbc * zbc);
        const double rrab = 1.0 / rab, rrbc = 1.0 / rbc;
        xab *= rrab; yab *= rrab; zab *= rrab;
        xbc *= rrbc; ybc *= rrbc; zbc *= rrbc;
        const double cost = xab * xbc + yab * ybc + zab * zbc;
        double pterm = 0, vterm = 0, f[6];
        ps_couple_group(sub, rab, xab, yab, zab, rbc, xbc, ybc, zbc, acos(cost), pterm, f, vterm);
        if (lead) {
            red[0] = pterm;
            red[1] = vterm;
            const double s1 = rab * xab * f[0] + rbc * xbc * f[3], s2 = rab * xab * f[1] + rbc * xbc * f[4];
            const double s3 = rab * xab * f[2] + rbc * xbc * f[5], s5 = rab * yab * f[1] + rbc * ybc * f[4];
            const double s6 = rab * yab * f[2] + rbc * ybc * f[5], s9 = rab * zab * f[2] + rbc * zbc * f[5];
            red[2] = s1; red[3] = s2; red[4] = s3;
            red[5] = s2; red[6] = s5; red[7] = s6;
            red[8] = s3; red[9] = s6; red[10] = s9;
            atomicAdd(fx + ia, f[0]); atomicAdd(fy + ia, f[1]); atomicAdd(fz + ia, f[2]);
            atomicAdd(fx + ib, -f[0] - f[3]); atomicAdd(fy + ib, -f[1] - f[4]); atomicAdd(fz + ib, -f[2] - f[5]);
            atomicAdd(fx + ic, f[3]); atomicAdd(fy + ic, f[4]); atomicAdd(fz + ic, f[5]);
            if (ae) {
                atomicAdd(ae + ia, pterm / 3);
                atomicAdd(ae + ib, pterm / 3);
                atomicAdd(ae + ic, pterm / 3);
            }
            if (vx) {
                // force-matrix entries (ia,ib),(ib,ia),(ic,ib),(ib,ic) contracted (raw coordinates)
                const double fva = f[0] * (vx[ia] + vx[ib]) + f[1] * (vy[ia] + vy[ib]) + f[2] * (vz[ia] + vz[ib]);
                const double fvc = f[3] * (vx[ic] + vx[ib]) + f[4] * (vy[ic] + vy[ib]) + f[5] * (vz[ic] + vz[ib]);
                red[11] = (x[ia] - x[ib]) * fva + (x[ic] - x[ib]) * fvc;
                red[12] = (y[ia] - y[ib]) * fva + (y[ic] - y[ib]) * fvc;
                red[13] = (z[ia] - z[ib]) * fva + (z[ic] - z[ib]) * fvc;
            }
        }
    }
    if (!acc_box) {
        block_sum_atomic<14>(red, acc);
        return;
    }
    // several boxes: one block sum when the block's angles share a box (the usual case,
    // boxes are contiguous), otherwise lane 0 of each warp adds its own angle
    __shared__ int span[2];
    if (threadIdx.x == 0) {
        span[0] = 0x7fffffff;
        span[1] = -1;
    }
    __syncthreads();
    const int box = lead ? abox[t] : -1;
    if (box >= 0) {
        atomicMin(&span[0], box);
        atomicMax(&span[1], box);
    }
    __syncthreads();
    const int lo = span[0], hi = span[1];
    if (hi < 0) return;   // block-uniform
    if (lo == hi) {
        block_sum_atomic<14>(red, acc_box + 14 * (size_t)hi);
    } else if (box >= 0) {
#pragma unroll
        for (int q = 0; q < 14; ++q)
            if (red[q] != 0.0) atomicAdd(acc_box + 14 * (size_t)box + q, red[q]);
    }
}

// M-site placement (SOURCE/dlpoly_cmd.f:2041-2057) and qdetermine with the MB-pol
// settings (ldms, new charge assignment; SOURCE/qdetermine.f90:112-285): one thread per
// water writes r_M, q_H1, q_H2, q_M and dq/d(r1, r2, cos) (6 values) for qdforce.
// Eight lanes per water: every lane places the M site's geometry, lane l takes the DMS
// expansion terms j = l (mod 8), and the group adds its partial sums by shuffles (one
// thread per water left 4096 waters at 128 warps: latency-bound at 0.29 ms).  The 1/reoh
// factor of the r derivatives is applied once to the sums.
constexpr int kDmsLanes = 8;

__global__ void __launch_bounds__(kThreads) k_msites_dms(int nw, const int* __restrict__ list, Cell cl, double* x,
                                                          double* y, double* z, double gamma, double* chge,
                                                          double* dp) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int i = (int)(t / kDmsLanes), l = (int)(t % kDmsLanes);
    if (i >= nw) return;   // whole lane groups leave together
    const int io = list[3 * i] - 1, h1 = list[3 * i + 1] - 1, h2 = list[3 * i + 2] - 1;
    const int m = list[3 * nw - 1] + i;   // 0-based index of this water's M site
    double r1x = x[h1] - x[io], r1y = y[h1] - y[io], r1z = z[h1] - z[io];
    double r2x = x[h2] - x[io], r2y = y[h2] - y[io], r2z = z[h2] - z[io];
    image(cl, r1x, r1y, r1z);
    image(cl, r2x, r2y, r2z);
    if (l == 0) {
        x[m] = x[io] + (r1x + r2x) * gamma / 2.0;
        y[m] = y[io] + (r1y + r2y) * gamma / 2.0;
        z[m] = z[io] + (r1z + r2z) * gamma / 2.0;
    }
    if (!chge) return;
    const double reoh = pes::kReoh;
    const double r1 = sqrt(r1x * r1x + r1y * r1y + r1z * r1z);
    const double r2 = sqrt(r2x * r2x + r2y * r2y + r2z * r2z);
    const double cost = (r1x * r2x + r1y * r2y + r1z * r2z) / (r1 * r2);
    const double x1 = (r1 - reoh) / reoh, x2 = (r2 - reoh) / reoh;
    const double x3 = cost - __longlong_as_double((long long)pes::kCose);
    double fm[pes::kDmsIsump + 1][3];
    fm[0][0] = fm[0][1] = fm[0][2] = 0.0;
    fm[1][0] = fm[1][1] = fm[1][2] = 1.0;
#pragma unroll
    for (int j = 2; j <= pes::kDmsIsump; ++j) {
        fm[j][0] = fm[j - 1][0] * x1;
        fm[j][1] = fm[j - 1][1] * x2;
        fm[j][2] = fm[j - 1][2] * x3;
    }
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // p1, p2, d11, d12, d21, d22 (times reoh), d1c, d2c
    for (int j = 1 + l; j < pes::kDmsTerms; j += kDmsLanes) {
        const int i1 = pes::kDmsIdx[j][0], i2 = pes::kDmsIdx[j][1], i3 = pes::kDmsIdx[j][2];
        const double c = __longlong_as_double((long long)pes::kDmsCoef[j]);
        v[0] += c * fm[i1][0] * fm[i2][1] * fm[i3][2];
        v[1] += c * fm[i2][0] * fm[i1][1] * fm[i3][2];
        v[2] += c * (i1 - 1) * fm[i1 - 1][0] * fm[i2][1] * fm[i3][2];
        v[3] += c * (i2 - 1) * fm[i1][0] * fm[i2 - 1][1] * fm[i3][2];
        v[4] += c * (i2 - 1) * fm[i2 - 1][0] * fm[i1][1] * fm[i3][2];
        v[5] += c * (i1 - 1) * fm[i2][0] * fm[i1 - 1][1] * fm[i3][2];
        v[6] += c * (i3 - 1) * fm[i1][0] * fm[i2][1] * fm[i3 - 1][2];
        v[7] += c * (i3 - 1) * fm[i2][0] * fm[i1][1] * fm[i3 - 1][2];
    }
    const unsigned gm = 0xffu << (threadIdx.x & 24);   // this water's lane group
#pragma unroll
    for (int q = 0; q < 8; ++q)
#pragma unroll
        for (int o = kDmsLanes / 2; o > 0; o >>= 1) v[q] += __shfl_xor_sync(gm, v[q], o, kDmsLanes);
    if (l != 0) return;
    double p1 = v[0], p2 = v[1];
    double d11 = v[2] / reoh, d12 = v[3] / reoh, d21 = v[4] / reoh, d22 = v[5] / reoh, d1c = v[6], d2c = v[7];
    const double bohr = 0.529177249, b1dms = 1.0, adms = 0.2999 * bohr, bdms = -0.6932;
    const double c0 = 1.0099, c1 = -0.1801, c2 = 0.0892;
    const double pl1 = cost, pl2 = 0.5 * (3.0 * pl1 * pl1 - 1.0);
    const double damp = exp(-b1dms * ((r1 - reoh) * (r1 - reoh) + (r2 - reoh) * (r2 - reoh)));
    const double dd1 = -2.0 * b1dms * (r1 - reoh) * damp, dd2 = -2.0 * b1dms * (r2 - reoh) * damp;
    const double ang = c0 + pl1 * c1 + pl2 * c2;
    const double q1b = pow(r1, bdms), q2b = pow(r2, bdms);
    const double pc0 = adms * (q1b + q2b) * ang;
    const double dpc0dr1 = adms * (bdms * pow(r1, bdms - 1)) * ang;
    const double dpc0dr2 = adms * (bdms * pow(r2, bdms - 1)) * ang;
    const double dpc0dcos = adms * (q1b + q2b) * (c1 + 3.0 * c2 * pl1);
    d11 = d11 * damp + p1 * dd1 + dpc0dr1;
    d12 = d12 * damp + p1 * dd2 + dpc0dr2;
    d21 = d21 * damp + p2 * dd1 + dpc0dr1;
    d22 = d22 * damp + p2 * dd2 + dpc0dr2;
    d1c = d1c * damp + dpc0dcos;
    d2c = d2c * damp + dpc0dcos;
    const double c00 = __longlong_as_double((long long)pes::kDmsCoef[0]);
    p1 = c00 + p1 * damp + pc0;
    p2 = c00 + p2 * damp + pc0;
    const double factor = gamma / 2.0 / (1.0 - gamma);
    const double qh1 = p1 + factor * (p1 + p2), qh2 = p2 + factor * (p1 + p2);
    chge[h1] = qh1;
    chge[h2] = qh2;
    chge[m] = -(qh1 + qh2);
    if (dp) {
        double* o = dp + 6 * (size_t)i;
        o[0] = d11; o[1] = d12; o[2] = d21; o[3] = d22; o[4] = d1c; o[5] = d2c;
    }
}

}  // namespace

cudaError_t launch_msites_dms(int nw, const int* list, const Cell& cl, double* x, double* y, double* z, double gamma,
                              double* chge, double* dp, cudaStream_t s) {
    if (nw <= 0) return cudaSuccess;
    const long threads = (long)kDmsLanes * nw;
    k_msites_dms<<<(unsigned)((threads + kThreads - 1) / kThreads), kThreads, 0, s>>>(nw, list, cl, x, y, z, gamma,
                                                                                       chge, dp);
    return cudaGetLastError();
}

cudaError_t launch_ps_pes(int nang, const int* listang, const Cell& cl, const double* x, const double* y,
                          const double* z, double* fx, double* fy, double* fz, double* ae, const double* vx,
                          const double* vy, const double* vz, double* acc14, cudaStream_t s) {
    if (nang <= 0) return cudaSuccess;
    const int blocks = (int)(((long)nang * kGroup + kThreads - 1) / kThreads);   // kGroup lanes per angle
    k_ps_pes<<<blocks, kThreads, 0, s>>>(nang, listang, cl, x, y, z, fx, fy, fz, ae, vx, vy, vz, acc14, nullptr,
                                         nullptr, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_ps_pes_boxes(int nang, const int* listang, const Cell* cells, const int* abox, const double* x,
                                const double* y, const double* z, double* fx, double* fy, double* fz, double* ae,
                                const double* vx, const double* vy, const double* vz, double* acc14_box,
                                const int* skip, cudaStream_t s) {
    if (nang <= 0) return cudaSuccess;
    const int blocks = (int)(((long)nang * kGroup + kThreads - 1) / kThreads);
    k_ps_pes<<<blocks, kThreads, 0, s>>>(nang, listang, Cell{}, x, y, z, fx, fy, fz, ae, vx, vy, vz, nullptr, cells,
                                         abox, acc14_box, skip);
    return cudaGetLastError();
}

}  // namespace mbx
