// Fused MB-pol 2B and 3B cluster kernels.
//
// One thread evaluates one dimer (or trimer) end to end:
//   1. gather the two (three) imaged monomers and re-image them around the
//      second one, as do_dimer / do_trimer do (SOURCE/mbpol.f90:505-509, :867-876);
//   2. build the model's variables (2B: X sites + 31 exp / exp-over-r terms,
//      SOURCE/mbpol-2b-poly.cpp:358-445; 3B: 36 exp terms, SOURCE/mbpol-3b-poly.cpp:148-206);
//   3. call the generated polynomial value+gradient functions (PTX, linked in);
//   4. chain rule back to the atoms, X-site redistribution and switching function
//      (SOURCE/mbpol-2b-poly.cpp:447-682, SOURCE/mbpol-3b-poly.cpp:208-312);
//   5. accumulate forces, per-atom energies (1/6, 1/9 per atom), energy, virial,
//      stress and the cluster's exact share of the heat-current jpot term
//      (the force-matrix rows of SOURCE/mbpol.f90:533-556 and :920-952 contracted as
//      in SOURCE/heatcurrent.f90:703-728).
//
// T = double reproduces the reference's arithmetic (FP64 path).  T = float is
// the mixed path: positions are re-imaged in FP64, shifted to the cluster's
// frame, and everything per cluster runs in FP32; forces, energies, virial and the
// heat current are accumulated in FP64.
#include "mbx_kernels.cuh"
#include "mbx_poly_gen.cuh"

namespace mbx {

__device__ __forceinline__ double t_exp(double v) { return exp(v); }
__device__ __forceinline__ float t_exp(float v) { return expf(v); }
__device__ __forceinline__ double t_sqrt(double v) { return sqrt(v); }
__device__ __forceinline__ float t_sqrt(float v) { return sqrtf(v); }
__device__ __forceinline__ double t_sin(double v) { return sin(v); }
__device__ __forceinline__ float t_sin(float v) { return sinf(v); }
__device__ __forceinline__ double t_cos(double v) { return cos(v); }
__device__ __forceinline__ float t_cos(float v) { return cosf(v); }

// ---------------------------------------------------------------------------
// 2B model (x2b_v6x_p), constants of SOURCE/mbpol-2b-poly.cpp:1846-1866
namespace m2b {
constexpr double k_HH_intra = -6.480884773303821e-01;
constexpr double k_OH_intra = 1.674518993682975e+00;
constexpr double k_HH_coul = 1.148231864355956e+00;
constexpr double k_OH_coul = 1.205989761123099e+00;
constexpr double k_OO_coul = 1.395357065790959e+00;
constexpr double k_XH_main = 7.347036852042255e-01;
constexpr double k_XO_main = 7.998249864422826e-01;
constexpr double k_XX_main = 7.960663960630585e-01;
constexpr double in_plane_gamma = -9.721486914088159e-02;
constexpr double out_of_plane_gamma = 9.859272078406150e-02;
enum { Oa = 0, Ha1 = 3, Ha2 = 6, Ob = 9, Hb1 = 12, Hb2 = 15, Xa1 = 18, Xa2 = 21, Xb1 = 24, Xb2 = 27 };
// variable kind (0 exp, 1 exp/r), r0, k, site1, site2 (SOURCE/mbpol-2b-poly.cpp:415-445)
struct V { int coul; double r0, k; int s1, s2; };
__device__ constexpr V kV[31] = {
    {0, 1.0, k_HH_intra, Ha1, Ha2}, {0, 1.0, k_HH_intra, Hb1, Hb2}, {0, 1.0, k_OH_intra, Oa, Ha1},
    {0, 1.0, k_OH_intra, Oa, Ha2},  {0, 1.0, k_OH_intra, Ob, Hb1},  {0, 1.0, k_OH_intra, Ob, Hb2},
    {1, 4.0, k_HH_coul, Ha1, Hb1},  {1, 4.0, k_HH_coul, Ha1, Hb2},  {1, 4.0, k_HH_coul, Ha2, Hb1},
    {1, 4.0, k_HH_coul, Ha2, Hb2},  {1, 4.0, k_OH_coul, Oa, Hb1},   {1, 4.0, k_OH_coul, Oa, Hb2},
    {1, 4.0, k_OH_coul, Ob, Ha1},   {1, 4.0, k_OH_coul, Ob, Ha2},   {1, 4.0, k_OO_coul, Oa, Ob},
    {0, 4.0, k_XH_main, Xa1, Hb1},  {0, 4.0, k_XH_main, Xa1, Hb2},  {0, 4.0, k_XH_main, Xa2, Hb1},
    {0, 4.0, k_XH_main, Xa2, Hb2},  {0, 4.0, k_XH_main, Xb1, Ha1},  {0, 4.0, k_XH_main, Xb1, Ha2},
    {0, 4.0, k_XH_main, Xb2, Ha1},  {0, 4.0, k_XH_main, Xb2, Ha2},  {0, 4.0, k_XO_main, Oa, Xb1},
    {0, 4.0, k_XO_main, Oa, Xb2},   {0, 4.0, k_XO_main, Ob, Xa1},   {0, 4.0, k_XO_main, Ob, Xa2},
    {0, 4.0, k_XX_main, Xa1, Xb1},  {0, 4.0, k_XX_main, Xa1, Xb2},  {0, 4.0, k_XX_main, Xa2, Xb1},
    {0, 4.0, k_XX_main, Xa2, Xb2},
};
}  // namespace m2b

// monomer::setup (SOURCE/mbpol-2b-poly.cpp:118-140)
template <typename T>
__device__ __forceinline__ void xsites(const T* ohh, T* oh1, T* oh2, T* x1, T* x2) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        oh1[i] = ohh[i + 3] - ohh[i];
        oh2[i] = ohh[i + 6] - ohh[i];
    }
    const T v[3] = {oh1[1] * oh2[2] - oh1[2] * oh2[1], oh1[2] * oh2[0] - oh1[0] * oh2[2],
                    oh1[0] * oh2[1] - oh1[1] * oh2[0]};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const T in_plane = ohh[i] + T(0.5) * T(m2b::in_plane_gamma) * (oh1[i] + oh2[i]);
        const T out_of_plane = T(m2b::out_of_plane_gamma) * v[i];
        x1[i] = in_plane + out_of_plane;
        x2[i] = in_plane - out_of_plane;
    }
}

// monomer::grads (SOURCE/mbpol-2b-poly.cpp:144-177)
template <typename T>
__device__ __forceinline__ void xsite_grads(const T* oh1, const T* oh2, const T* g1, const T* g2, T* grd) {
    const T gm[3] = {g1[0] - g2[0], g1[1] - g2[1], g1[2] - g2[2]};
    const T t1[3] = {oh2[1] * gm[2] - oh2[2] * gm[1], oh2[2] * gm[0] - oh2[0] * gm[2],
                     oh2[0] * gm[1] - oh2[1] * gm[0]};
    const T t2[3] = {oh1[1] * gm[2] - oh1[2] * gm[1], oh1[2] * gm[0] - oh1[0] * gm[2],
                     oh1[0] * gm[1] - oh1[1] * gm[0]};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const T gsum = g1[i] + g2[i];
        const T in_plane = T(0.5) * T(m2b::in_plane_gamma) * gsum;
        const T gh1 = in_plane + T(m2b::out_of_plane_gamma) * t1[i];
        const T gh2 = in_plane - T(m2b::out_of_plane_gamma) * t2[i];
        grd[i + 0] += gsum - (gh1 + gh2);
        grd[i + 3] += gh1;
        grd[i + 6] += gh2;
    }
}

// f_switch (SOURCE/mbpol-2b-poly.cpp:340-354 and SOURCE/mbpol-3b-poly.cpp:130-144)
template <typename T>
__device__ __forceinline__ T f_switch(T r, T ri, T rf, T& g) {
    if (r > rf) {
        g = T(0);
        return T(0);
    } else if (r > ri) {
        const T t1 = T(M_PI) / (rf - ri);
        const T x = (r - ri) * t1;
        g = -t_sin(x) * t1 / T(2);
        return (T(1) + t_cos(x)) / T(2);
    }
    g = T(0);
    return T(1);
}

// One FP64 dimer evaluated as kPoly2BF64Parts tasks, one polynomial chunk each: every
// task computes the variables and its chunk, publishes the chunk's [E, dE/dx] (32
// doubles) in partial[(t * parts + p) * 32], and the task that completes the count in
// done[t] sums the chunks in chunk order -- the same sums as one thread calling the
// chunks in turn -- and finishes the dimer.
struct Part2B {
    int t, p;
    double* partial;
    int* done;
};

// x2b_v6x_p::operator() on coordinates already in the working frame.
// Returns E (kcal/mol); g1/g2 assigned.  For T = float the polynomial is evaluated
// in the shifted variables x - kShift2B; if any of them lies further than `limit`
// from its centre the cluster is left to the FP64 pass (*hard = true, nothing set).
// With `part` (T = double) only that polynomial chunk is evaluated here; unless this
// task completes the dimer, *deferred is set and nothing else is.
template <typename T>
__device__ __forceinline__ T model_2b(const T* w1, const T* w2, T* g1, T* g2, float limit = 0.f,
                                      bool* hard = nullptr, const Part2B* part = nullptr,
                                      bool* deferred = nullptr) {
    const T dOO[3] = {w1[0] - w2[0], w1[1] - w2[1], w1[2] - w2[2]};
    const T rOO = t_sqrt(dOO[0] * dOO[0] + dOO[1] * dOO[1] + dOO[2] * dOO[2]);
    if (rOO > T(kR2f)) {
#pragma unroll
        for (int i = 0; i < 9; ++i) g1[i] = g2[i] = T(0);
        return T(0);
    }
    T xc[30];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        xc[i] = w1[i];
        xc[9 + i] = w2[i];
    }
    T oha[2][3], ohb[2][3];
    xsites(xc + m2b::Oa, oha[0], oha[1], xc + m2b::Xa1, xc + m2b::Xa2);
    xsites(xc + m2b::Ob, ohb[0], ohb[1], xc + m2b::Xb1, xc + m2b::Xb2);
    T v[31], gg[31];
#pragma unroll
    for (int q = 0; q < 31; ++q) {
        const m2b::V d = m2b::kV[q];
        const T dx = xc[d.s1] - xc[d.s2], dy = xc[d.s1 + 1] - xc[d.s2 + 1], dz = xc[d.s1 + 2] - xc[d.s2 + 2];
        const T r = t_sqrt(dx * dx + dy * dy + dz * dz);
        const T e = t_exp(T(d.k) * (T(d.r0) - r));
        if (!d.coul) {
            v[q] = e;
            gg[q] = -T(d.k) * e / r;
        } else {
            const T rinv = T(1) / r;
            v[q] = e * rinv;
            gg[q] = -(T(d.k) + rinv) * v[q] * rinv;
        }
    }
    if constexpr (sizeof(T) == 4) {
        float dev = 0.f;
#pragma unroll
        for (int q = 0; q < 31; ++q) {
            v[q] -= kShift2B[q];
            dev = fmaxf(dev, fabsf(v[q]));
        }
        if (hard && dev > limit) {
            *hard = true;
            return T(0);
        }
    }
    T acc[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) acc[q] = T(0);
    if constexpr (sizeof(T) == 8) {
        if (part) {
            poly2b_f64_part(part->p, v, acc);
            double* slot = part->partial + (size_t)part->t * (kPoly2BF64Parts * 32);
#pragma unroll
            for (int q = 0; q < 32; ++q) __stcg(slot + part->p * 32 + q, acc[q]);
            __threadfence();
            if (atomicAdd(part->done + part->t, 1) != kPoly2BF64Parts - 1) {
                *deferred = true;
                return T(0);
            }
            __threadfence();
#pragma unroll
            for (int q = 0; q < 32; ++q) acc[q] = T(0);
            for (int pp = 0; pp < kPoly2BF64Parts; ++pp) {
#pragma unroll
                for (int q = 0; q < 32; ++q) acc[q] = acc[q] + __ldcg(slot + pp * 32 + q);
            }
        } else {
            poly2b<T>(v, acc);
        }
    } else {
        poly2b<T>(v, acc);
    }
    const T E_poly = acc[0];
    T xgrd[30];
#pragma unroll
    for (int q = 0; q < 30; ++q) xgrd[q] = T(0);
#pragma unroll
    for (int q = 0; q < 31; ++q) {
        const m2b::V d = m2b::kV[q];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T gv = (xc[d.s1 + c] - xc[d.s2 + c]) * gg[q];
            const T t = acc[1 + q] * gv;
            xgrd[d.s1 + c] += t;
            xgrd[d.s2 + c] -= t;
        }
    }
    xsite_grads(oha[0], oha[1], xgrd + m2b::Xa1, xgrd + m2b::Xa2, xgrd + m2b::Oa);
    xsite_grads(ohb[0], ohb[1], xgrd + m2b::Xb1, xgrd + m2b::Xb2, xgrd + m2b::Ob);
    T gsw;
    const T sw = f_switch(rOO, T(kR2i), T(kR2f), gsw);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        g1[i] = sw * xgrd[i];
        g2[i] = sw * xgrd[i + 9];
    }
    gsw *= E_poly / rOO;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const T d = gsw * dOO[i];
        g1[i] += d;
        g2[i] -= d;
    }
    return sw * E_poly;
}

// ---------------------------------------------------------------------------
// 3B model (x3b_v2x_p), constants of SOURCE/mbpol-3b-poly.cpp:1486-1506
namespace m3b {
constexpr double kHH_intra = -2.254303257872797e+00;
constexpr double kOH_intra = -2.564771901404151e-01;
constexpr double kHH = 4.247920544074333e-01;
constexpr double kOH = 8.128985941165371e-01;
constexpr double kOO = 3.749457984616480e-02;
constexpr double dHH_intra = 1.690594510379166e+00;
constexpr double dOH_intra = -2.999999868517452e+00;
constexpr double dHH = 3.499031358429095e+00;
constexpr double dOH = 4.854042963514281e+00;
constexpr double dOO = 4.816312044947604e-08;
enum { Oa = 0, Ha1 = 3, Ha2 = 6, Ob = 9, Hb1 = 12, Hb2 = 15, Oc = 18, Hc1 = 21, Hc2 = 24 };
struct V { double k, r0; int a1, a2; };
// SOURCE/mbpol-3b-poly.cpp:170-206
__device__ constexpr V kV[36] = {
    {kHH_intra, dHH_intra, Ha1, Ha2}, {kHH_intra, dHH_intra, Hb1, Hb2}, {kHH_intra, dHH_intra, Hc1, Hc2},
    {kOH_intra, dOH_intra, Oa, Ha1},  {kOH_intra, dOH_intra, Oa, Ha2},  {kOH_intra, dOH_intra, Ob, Hb1},
    {kOH_intra, dOH_intra, Ob, Hb2},  {kOH_intra, dOH_intra, Oc, Hc1},  {kOH_intra, dOH_intra, Oc, Hc2},
    {kHH, dHH, Ha1, Hb1}, {kHH, dHH, Ha1, Hb2}, {kHH, dHH, Ha1, Hc1}, {kHH, dHH, Ha1, Hc2},
    {kHH, dHH, Ha2, Hb1}, {kHH, dHH, Ha2, Hb2}, {kHH, dHH, Ha2, Hc1}, {kHH, dHH, Ha2, Hc2},
    {kHH, dHH, Hb1, Hc1}, {kHH, dHH, Hb1, Hc2}, {kHH, dHH, Hb2, Hc1}, {kHH, dHH, Hb2, Hc2},
    {kOH, dOH, Oa, Hb1},  {kOH, dOH, Oa, Hb2},  {kOH, dOH, Oa, Hc1},  {kOH, dOH, Oa, Hc2},
    {kOH, dOH, Ob, Ha1},  {kOH, dOH, Ob, Ha2},  {kOH, dOH, Ob, Hc1},  {kOH, dOH, Ob, Hc2},
    {kOH, dOH, Oc, Ha1},  {kOH, dOH, Oc, Ha2},  {kOH, dOH, Oc, Hb1},  {kOH, dOH, Oc, Hb2},
    {kOO, dOO, Oa, Ob},   {kOO, dOO, Oa, Oc},   {kOO, dOO, Ob, Oc},
};
}  // namespace m3b

// 3B variables (SOURCE/mbpol-3b-poly.cpp:170-206) and the factor -k e/r of their
// gradient (g_intra/g_main, :26-87).  For T = float the variables are returned
// shifted by kShift3B (the FP32 polynomial's expansion point); returns the largest
// |shifted variable| (0 for double).
template <typename T>
__device__ __forceinline__ float vars_3b(const T* t, T* x, T* fk) {
    float dev = 0.f;
#pragma unroll
    for (int q = 0; q < 36; ++q) {
        const m3b::V d = m3b::kV[q];
        const T dx = t[d.a1] - t[d.a2], dy = t[d.a1 + 1] - t[d.a2 + 1], dz = t[d.a1 + 2] - t[d.a2 + 2];
        const T r = t_sqrt(dx * dx + dy * dy + dz * dz);
        const T e = t_exp(-T(d.k) * (r - T(d.r0)));
        x[q] = e;
        fk[q] = -T(d.k) * e / r;
        if constexpr (sizeof(T) == 4) {
            x[q] -= kShift3B[q];
            dev = fmaxf(dev, fabsf(x[q]));
        }
    }
    return dev;
}

// Chain rule and switching of x3b_v2x_p::operator() (SOURCE/mbpol-3b-poly.cpp:208-312)
// given the polynomial's [E, dE/dx]; gradients ADDED to gt; returns the energy.
template <typename T>
__device__ __forceinline__ T finish_3b(const T* t, const T* acc, const T* fk, T* gt) {
    T retval = acc[0];
    T rab[3], rac[3], rbc[3];
    T drab = T(0), drac = T(0), drbc = T(0);
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        rab[n] = t[m3b::Oa + n] - t[m3b::Ob + n];
        drab += rab[n] * rab[n];
        rac[n] = t[m3b::Oa + n] - t[m3b::Oc + n];
        drac += rac[n] * rac[n];
        rbc[n] = t[m3b::Ob + n] - t[m3b::Oc + n];
        drbc += rbc[n] * rbc[n];
    }
    drab = t_sqrt(drab);
    drac = t_sqrt(drac);
    drbc = t_sqrt(drbc);
    T gab, gac, gbc;
    const T sab = f_switch(drab, T(0), T(kR3f), gab);
    const T sac = f_switch(drac, T(0), T(kR3f), gac);
    const T sbc = f_switch(drbc, T(0), T(kR3f), gbc);
    const T s = sab * sac + sab * sbc + sac * sbc;
#pragma unroll
    for (int q = 0; q < 36; ++q) {
        const m3b::V d = m3b::kV[q];
        const T gg = (acc[1 + q] * s) * fk[q];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T dd = t[d.a1 + c] - t[d.a2 + c];
            gt[d.a1 + c] += gg * dd;
            gt[d.a2 + c] -= gg * dd;
        }
    }
    gab *= (sac + sbc) * retval / drab;
    gac *= (sab + sbc) * retval / drac;
    gbc *= (sab + sac) * retval / drbc;
    retval *= s;
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        gt[m3b::Oa + n] += gab * rab[n] + gac * rac[n];
        gt[m3b::Ob + n] += gbc * rbc[n] - gab * rab[n];
        gt[m3b::Oc + n] -= gac * rac[n] + gbc * rbc[n];
    }
    return retval;
}

// x3b_v2x_p::operator() on the 27 trimer coordinates; gradients ADDED to gt.
// T = float: shifted variables and the FP64 hand-off, as in model_2b.
template <typename T>
__device__ __forceinline__ T model_3b(const T* t, T* gt, float limit = 0.f, bool* hard = nullptr) {
    T x[36], fk[36];
    const float dev = vars_3b<T>(t, x, fk);
    if (hard && dev > limit) {
        *hard = true;
        return T(0);
    }
    T acc[37];
#pragma unroll
    for (int q = 0; q < 37; ++q) acc[q] = T(0);
    poly3b<T>(x, acc);
    return finish_3b<T>(t, acc, fk, gt);
}

// ---------------------------------------------------------------------------
// Cluster bookkeeping shared by 2B and 3B: forces, per-atom energy, virial,
// stress (do_dimer :574-667, do_trimer :967-1071) and the exact heat-current share.
// red = {E, vir, stress[9], jpot[3]} (14), plus the 2B energy in red[14] when the
// caller accumulates both bodies (eidx = 14 for dimers, 0 otherwise).
template <int NA>
__device__ __forceinline__ void cluster_accumulate(const MbpolArgs& a, const int* at, double e_kcal,
                                                   const double* w, const double* g_kcal, double* red,
                                                   int eidx = 0) {
    const double e = e_kcal * kEngUnit;
    red[eidx] += e;
    if (a.ae) {
        const double ea = (1.0 / NA) * e_kcal * kEngUnit;
#pragma unroll
        for (int q = 0; q < NA; ++q) atomicAdd(a.ae + at[q], ea);
    }
    if (a.vx) {
        double rs[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            rs[0] += a.x[at[q]];
            rs[1] += a.y[at[q]];
            rs[2] += a.z[at[q]];
        }
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            const int i = at[q];
            const double f0 = -((1.0 / NA) * g_kcal[3 * q + 0]) * kEngUnit;
            const double f1 = -((1.0 / NA) * g_kcal[3 * q + 1]) * kEngUnit;
            const double f2 = -((1.0 / NA) * g_kcal[3 * q + 2]) * kEngUnit;
            const double fv = f0 * a.vx[i] + f1 * a.vy[i] + f2 * a.vz[i];
            red[11] += fv * (NA * a.x[i] - rs[0]);
            red[12] += fv * (NA * a.y[i] - rs[1]);
            red[13] += fv * (NA * a.z[i] - rs[2]);
        }
    }
    double sv[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int q = 0; q < NA; ++q) {
        const double g0 = g_kcal[3 * q] * kEngUnit, g1 = g_kcal[3 * q + 1] * kEngUnit,
                     g2 = g_kcal[3 * q + 2] * kEngUnit;
        const double w0 = w[3 * q], w1 = w[3 * q + 1], w2 = w[3 * q + 2];
        red[1] += w0 * g0 + w1 * g1 + w2 * g2;
        sv[0] += w0 * g0;
        sv[1] += w0 * g1;
        sv[2] += w0 * g2;
        sv[3] += w1 * g1;
        sv[4] += w1 * g2;
        sv[5] += w2 * g2;
        atomicAdd(a.fx + at[q], -g0);
        atomicAdd(a.fy + at[q], -g1);
        atomicAdd(a.fz + at[q], -g2);
    }
    red[2] -= sv[0]; red[3] -= sv[1]; red[4] -= sv[2];
    red[5] -= sv[1]; red[6] -= sv[3]; red[7] -= sv[4];
    red[8] -= sv[2]; red[9] -= sv[4]; red[10] -= sv[5];
}

// Slot of red[q]: q = 0 the energy of `eslot`, 1 the virial, 2..10 stress, 11..13
// jpot, 14 (when present) the 2B energy of a block that evaluated both bodies.
__device__ __forceinline__ int red_slot(int q, int eslot) {
    return q == 0 ? eslot
                  : (q == 1 ? S_VIR : (q <= 10 ? S_STRESS + (q - 2) : (q <= 13 ? S_JPOT + (q - 11) : S_E2)));
}

// Reduce red[NR] of the block (NT threads) into acc.
template <int NT, int NR>
__device__ __forceinline__ void flush_block_n(double (&red)[NR], double* acc, int eslot) {
    __shared__ double sh[NT / 32][NR];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const double s = warp_sum(red[q]);
        if (lane == 0) sh[w][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < NR) {
        double s = 0.0;
        for (int i = 0; i < NT / 32; ++i) s += sh[i][threadIdx.x];
        if (s != 0.0) atomicAdd(acc + red_slot(threadIdx.x, eslot), s);
    }
}

template <int NR>
__device__ __forceinline__ void flush_block(double (&red)[NR], double* acc, int eslot) {
    flush_block_n<kThreads, NR>(red, acc, eslot);
}

// Several boxes in one launch: clusters are grouped by box, so a warp almost always
// holds one box -- reduce it with shuffles; a warp straddling boxes adds per lane.
// box < 0: this thread holds no cluster.
template <int NR>
__device__ __forceinline__ void flush_boxes(double (&red)[NR], double* acc_box, int box, int eslot) {
    int lo = box < 0 ? 0x7fffffff : box, hi = box;
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (hi < 0) return;
    if (lo == hi) {
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            const double v = warp_sum(red[q]);
            if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(acc_box + (size_t)hi * S_NSLOTS + red_slot(q, eslot), v);
        }
    } else if (box >= 0) {
#pragma unroll
        for (int q = 0; q < NR; ++q)
            if (red[q] != 0.0) atomicAdd(acc_box + (size_t)box * S_NSLOTS + red_slot(q, eslot), red[q]);
    }
}

// Mixed-precision hand-off: clusters whose FP32 variables stray beyond the limit
// are appended to `hard` and evaluated by the FP64 kernel afterwards.
struct HardList {
    void* items;        // int2 (dimers) or int4 (trimers)
    int* count;
    float limit;
};

// One dimer: image, model, then forces/energy/virial/stress/heat into red (or the
// hand-off list when the FP32 variables stray beyond the limit).
template <typename T>
__device__ __forceinline__ void eval_dimer(const MbpolArgs& a, int2 p, double* red, int eidx, const HardList& hl,
                                           const Part2B* part = nullptr) {
    const int i = p.x, j = p.y;
    const Cell& cl = a.cells ? a.cells[a.wbox[i]] : a.cell;
    double w1[9], w2[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        w1[q] = a.mono[9 * (size_t)i + q];
        w2[q] = a.mono[9 * (size_t)j + q];
    }
    double r12[3];
    dist2_img(cl, w1, w2, r12);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        w1[3 + k] = dadd(dsub(w1[3 + k], w1[k]), dadd(w2[k], r12[k]));
        w1[6 + k] = dadd(dsub(w1[6 + k], w1[k]), dadd(w2[k], r12[k]));
        w1[k] = dadd(w2[k], r12[k]);
    }
    // working frame: absolute for FP64, shifted to the second O for FP32
    T p1[9], p2[9], g1[9], g2[9];
    double w[18];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double o = (sizeof(T) == 8) ? 0.0 : w2[q % 3];
        w[q] = w1[q] - o;
        w[9 + q] = w2[q] - o;
        p1[q] = (T)w[q];
        p2[q] = (T)w[9 + q];
    }
    bool hard = false, deferred = false;
    const T e = model_2b<T>(p1, p2, g1, g2, hl.limit, hl.items ? &hard : nullptr, part, &deferred);
    if (deferred) return;
    if (hard) {
        ((int2*)hl.items)[atomicAdd(hl.count, 1)] = p;
        return;
    }
    const int o1 = a.list[3 * i] - 1, o2 = a.list[3 * j] - 1;
    const int at[6] = {o1, o1 + 1, o1 + 2, o2, o2 + 1, o2 + 2};
    double g[18];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        g[q] = (double)g1[q];
        g[9 + q] = (double)g2[q];
    }
    cluster_accumulate<6>(a, at, (double)e, w, g, red, eidx);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_mbpol_2b(MbpolArgs a, const int2* __restrict__ pairs, int n,
                                                        const int* __restrict__ n_dev, HardList hl) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n = *n_dev;
    double red[14];
#pragma unroll
    for (int q = 0; q < 14; ++q) red[q] = 0.0;
    int box = -1;
    if (t < n) {
        const int2 p = pairs[t];
        if (a.cells) box = a.wbox[p.x];
        eval_dimer<T>(a, p, red, 0, hl);
    }
    if (a.acc_box) flush_boxes(red, a.acc_box, box, S_E2);
    else flush_block(red, a.acc, S_E2);
}

// Gather the trimer's monomers and re-image them around the second one as do_trimer
// does (SOURCE/mbpol.f90:867-876); w = working-frame positions (absolute for FP64,
// shifted to the second O for FP32), p = the same in T.
template <typename T>
__device__ __forceinline__ void prep_3b(const MbpolArgs& a, int4 c, double* w, T* p) {
    double w1[9], w2[9], w3[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        w1[q] = a.mono[9 * (size_t)c.x + q];
        w2[q] = a.mono[9 * (size_t)c.y + q];
        w3[q] = a.mono[9 * (size_t)c.z + q];
    }
    double r12[3], r23[3];
    const Cell& cl = a.cells ? a.cells[a.wbox[c.x]] : a.cell;
    dist2_img(cl, w1, w2, r12);
    dist2_img(cl, w2, w3, r23);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        w1[3 + k] = dadd(dsub(w1[3 + k], w1[k]), dadd(w2[k], r12[k]));
        w1[6 + k] = dadd(dsub(w1[6 + k], w1[k]), dadd(w2[k], r12[k]));
        w1[k] = dadd(w2[k], r12[k]);
        w3[3 + k] = dadd(dsub(w3[3 + k], w3[k]), dsub(w2[k], r23[k]));
        w3[6 + k] = dadd(dsub(w3[6 + k], w3[k]), dsub(w2[k], r23[k]));
        w3[k] = dsub(w2[k], r23[k]);
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double o = (sizeof(T) == 8) ? 0.0 : w2[q % 3];
        w[q] = w1[q] - o;
        w[9 + q] = w2[q] - o;
        w[18 + q] = w3[q] - o;
    }
#pragma unroll
    for (int q = 0; q < 27; ++q) p[q] = (T)w[q];
}

// The FP32 working frame of a trimer directly: positions relative to the second O, with
// the monomers re-imaged around it as do_trimer does (SOURCE/mbpol.f90:867-876).  The
// same frame as prep_3b<float> up to the FP64 rounding before the cast, in fewer FP64
// operations (the FP64 pipe is the mixed kernel's bound).
__device__ __forceinline__ void prep_3b_shifted(const MbpolArgs& a, int4 c, float* p) {
    double w1[9], w2[9], w3[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        w1[q] = a.mono[9 * (size_t)c.x + q];
        w2[q] = a.mono[9 * (size_t)c.y + q];
        w3[q] = a.mono[9 * (size_t)c.z + q];
    }
    double r12[3], r23[3];
    const Cell& cl = a.cells ? a.cells[a.wbox[c.x]] : a.cell;
    dist2_img(cl, w1, w2, r12);   // image(O1 - O2)
    dist2_img(cl, w2, w3, r23);   // image(O2 - O3)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        p[k] = (float)r12[k];
        p[3 + k] = (float)dadd(dsub(w1[3 + k], w1[k]), r12[k]);
        p[6 + k] = (float)dadd(dsub(w1[6 + k], w1[k]), r12[k]);
        p[9 + k] = 0.f;
        p[12 + k] = (float)dsub(w2[3 + k], w2[k]);
        p[15 + k] = (float)dsub(w2[6 + k], w2[k]);
        p[18 + k] = (float)(-r23[k]);
        p[21 + k] = (float)dsub(dsub(w3[3 + k], w3[k]), r23[k]);
        p[24 + k] = (float)dsub(dsub(w3[6 + k], w3[k]), r23[k]);
    }
}

// cluster_accumulate for an FP32 trimer: the same quantities with the per-cluster
// virial and stress products in FP32 on the shifted frame (a cluster's gradient sums to
// zero, so the shift does not change them) and FP64 for the energy, the force and
// per-atom energy atomics and the heat current (raw coordinates, FP64).
__device__ __forceinline__ void trimer_accumulate_f32(const MbpolArgs& a, const int* at, float e_kcal,
                                                      const float* p, const float* gt, double* red) {
    const double e = (double)e_kcal * kEngUnit;
    red[0] += e;
    if (a.ae) {
        const double ea = (1.0 / 9) * (double)e_kcal * kEngUnit;
#pragma unroll
        for (int q = 0; q < 9; ++q) atomicAdd(a.ae + at[q], ea);
    }
    double gd[27];
#pragma unroll
    for (int q = 0; q < 27; ++q) gd[q] = (double)(gt[q] * (float)kEngUnit);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        atomicAdd(a.fx + at[q], -gd[3 * q + 0]);
        atomicAdd(a.fy + at[q], -gd[3 * q + 1]);
        atomicAdd(a.fz + at[q], -gd[3 * q + 2]);
    }
    float sv[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const float w0 = p[3 * q], w1 = p[3 * q + 1], w2 = p[3 * q + 2];
        const float g0 = gt[3 * q], g1 = gt[3 * q + 1], g2 = gt[3 * q + 2];
        sv[0] += w0 * g0;
        sv[1] += w0 * g1;
        sv[2] += w0 * g2;
        sv[3] += w1 * g1;
        sv[4] += w1 * g2;
        sv[5] += w2 * g2;
    }
    double s[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) s[k] = (double)sv[k] * kEngUnit;
    red[1] += (s[0] + s[3]) + s[5];
    red[2] -= s[0]; red[3] -= s[1]; red[4] -= s[2];
    red[5] -= s[1]; red[6] -= s[3]; red[7] -= s[4];
    red[8] -= s[2]; red[9] -= s[4]; red[10] -= s[5];
    if (a.vx) {
        // sum_q (F_q . v_q)(9 r_q - sum_j r_j) = 9 sum_q fv_q r_q - (sum_j r_j) sum_q fv_q
        double rs[3] = {0.0, 0.0, 0.0}, A[3] = {0.0, 0.0, 0.0}, B = 0.0;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const int i = at[q];
            const double xi = a.x[i], yi = a.y[i], zi = a.z[i];
            const double fv = -(1.0 / 9) * (gd[3 * q] * a.vx[i] + gd[3 * q + 1] * a.vy[i] + gd[3 * q + 2] * a.vz[i]);
            rs[0] += xi;
            rs[1] += yi;
            rs[2] += zi;
            A[0] += fv * xi;
            A[1] += fv * yi;
            A[2] += fv * zi;
            B += fv;
        }
        red[11] += 9.0 * A[0] - rs[0] * B;
        red[12] += 9.0 * A[1] - rs[1] * B;
        red[13] += 9.0 * A[2] - rs[2] * B;
    }
}

__device__ __forceinline__ void trimer_atoms(const MbpolArgs& a, int4 c, int* at) {
    const int o1 = a.list[3 * c.x] - 1, o2 = a.list[3 * c.y] - 1, o3 = a.list[3 * c.z] - 1;
    at[0] = o1; at[1] = o1 + 1; at[2] = o1 + 2;
    at[3] = o2; at[4] = o2 + 1; at[5] = o2 + 2;
    at[6] = o3; at[7] = o3 + 1; at[8] = o3 + 2;
}

template <typename T>
__device__ __forceinline__ void eval_trimer(const MbpolArgs& a, int4 c, double* red, const HardList& hl) {
    if constexpr (sizeof(T) == 4) {
        float p[27], gt[27];
        prep_3b_shifted(a, c, p);
#pragma unroll
        for (int q = 0; q < 27; ++q) gt[q] = 0.f;
        bool hard = false;
        const float e = model_3b<float>(p, gt, hl.limit, hl.items ? &hard : nullptr);
        if (hard) {
            ((int4*)hl.items)[atomicAdd(hl.count, 1)] = c;
            return;
        }
        int at[9];
        trimer_atoms(a, c, at);
        trimer_accumulate_f32(a, at, e, p, gt, red);
        return;
    }
    T p[27], gt[27];
    double w[27];
    prep_3b<T>(a, c, w, p);
#pragma unroll
    for (int q = 0; q < 27; ++q) gt[q] = T(0);
    bool hard = false;
    const T e = model_3b<T>(p, gt, hl.limit, hl.items ? &hard : nullptr);
    if (hard) {
        ((int4*)hl.items)[atomicAdd(hl.count, 1)] = c;
        return;
    }
    int at[9];
    trimer_atoms(a, c, at);
    double g[27];
#pragma unroll
    for (int q = 0; q < 27; ++q) g[q] = (double)gt[q];
    cluster_accumulate<9>(a, at, (double)e, w, g, red, 0);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_mbpol_3b(MbpolArgs a, const int4* __restrict__ trip, int n,
                                                        const int* __restrict__ n_dev, HardList hl) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n = *n_dev;
    double red[14];
#pragma unroll
    for (int q = 0; q < 14; ++q) red[q] = 0.0;
    int box = -1;
    if (t < n) {
        const int4 c = trip[t];
        if (a.cells) box = a.wbox[c.x];
        eval_trimer<T>(a, c, red, hl);
    }
    if (a.acc_box) flush_boxes(red, a.acc_box, box, S_E3);
    else flush_block(red, a.acc, S_E3);
}

// Both bodies of the mixed method in one persistent launch: one 384-thread block per
// SM (12 warps at <= 168 registers).  Warps 0-3 (one per SM sub-partition) take FP64
// dimers first and keep the FP64 pipe busy; warps 4-11 take FP32 trimers; a warp whose
// queue runs dry moves to the other one.  The two bodies so overlap on their own pipes
// instead of following each other.  The FP64 pipe takes one warp instruction per 64
// cycles whatever the number of active lanes, so a 32-dimer chunk is the unit of FP64
// work (~1 ms); with a partial buffer each dimer chunk is split into one task per FP64
// polynomial chunk, all part-0 tasks first, which halves the unit and the last round's
// tail while the dimer warps of an SM still walk the same code.  Measured on the
// 4096-water box: 4.67 ms (two kernels in sequence: 6.7 ms; unsplit dimers 4.85 ms;
// 4+4 warps at 255 registers 5.2 ms).  Work is claimed 32 tasks at a time from ctr[0]
// (dimers) and ctr[1] (trimers), which start at zero.
constexpr int kFusedThreads = 384;
// The block of the overlapped form (mbx_set_overlap): 8 warps at <= 168 registers, 43K of an
// SM's 64K registers, so the electrostatics' FP32 CG kernels fit beside it on every SM.
constexpr int kFusedThreadsShared = 256;
constexpr int kFusedDimerWarps = 4;   // the default split (dimer_warps 0)
// Registers per thread of both blocks, the budget the polynomial functions are compiled to.
// It is set with __maxnreg__ (launch bounds of 256 threads, one block, would let the kernel
// body take 255 registers and the whole register file).
constexpr int kFusedMaxRegs = 168;

template <typename T2, typename T3, int NT>
__global__ void __maxnreg__(kFusedMaxRegs)
    k_mbpol_23(MbpolArgs a, const int2* __restrict__ pairs, int n2, const int* __restrict__ n2_dev,
               const int4* __restrict__ trip, int n3, const int* __restrict__ n3_dev, int* ctr,
               double* partial, int* done, long part_cap, int dimer_warps) {
    if (n2_dev) n2 = *n2_dev;
    if (n3_dev) n3 = *n3_dev;
    // dimer tasks: 32-dimer chunks, each split into `parts` polynomial chunks (chunk c,
    // part p at task block c * parts + p) when the partial buffer holds every dimer
    if (n2 > part_cap) partial = nullptr;
    const int parts = partial ? kPoly2BF64Parts : 1;
    const int ntask2 = ((n2 + 31) / 32) * 32 * parts;
    const int lane = threadIdx.x & 31;
    int role = (int)(threadIdx.x >> 5) < dimer_warps ? 0 : 1;
    bool switched = false;
    const HardList none{nullptr, nullptr, 0.f};
    double red[15];
#pragma unroll
    for (int q = 0; q < 15; ++q) red[q] = 0.0;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(ctr + role, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (role ? n3 : ntask2)) {
            if (switched) break;
            switched = true;
            role ^= 1;
            continue;
        }
        const int t = base + lane;
        int box = -1;
        if (role == 0) {
            const int blk = base >> 5;
            const int nchunk = (n2 + 31) / 32;
            // all chunks of polynomial part 0 first, then part 1, ...: the dimer warps of an
            // SM walk the same part's code at the same time
            const int td = (blk % nchunk) * 32 + lane;
            if (td < n2) {
                const int2 p = pairs[td];
                if (a.cells) box = a.wbox[p.x];
                if (partial) {
                    const Part2B part{td, blk / nchunk, partial, done};
                    eval_dimer<T2>(a, p, red, 14, none, &part);
                } else {
                    eval_dimer<T2>(a, p, red, 14, none);
                }
            }
        } else if (t < n3) {
            const int4 c = trip[t];
            if (a.cells) box = a.wbox[c.x];
            eval_trimer<T3>(a, c, red, none);
        }
        if (a.acc_box) {   // several boxes: flush this chunk per box
            flush_boxes(red, a.acc_box, box, S_E3);
#pragma unroll
            for (int q = 0; q < 15; ++q) red[q] = 0.0;
        }
    }
    if (!a.acc_box) flush_block_n<NT, 15>(red, a.acc, S_E3);
}

// Per-call model evaluation (drop-in for mbpol_2b_poly_/mbpol_3b_poly_ over many clusters).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_2b_direct(int n, const double* __restrict__ w1s,
                                                         const double* __restrict__ w2s, double* E, double* g1s,
                                                         double* g2s) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    T p1[9], p2[9], g1[9], g2[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double o = (sizeof(T) == 8) ? 0.0 : w2s[9 * (size_t)t + q % 3];
        p1[q] = (T)(w1s[9 * (size_t)t + q] - o);
        p2[q] = (T)(w2s[9 * (size_t)t + q] - o);
    }
    E[t] = (double)model_2b<T>(p1, p2, g1, g2);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        g1s[9 * (size_t)t + q] = (double)g1[q];
        g2s[9 * (size_t)t + q] = (double)g2[q];
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_3b_direct(int n, const double* __restrict__ w1s,
                                                         const double* __restrict__ w2s,
                                                         const double* __restrict__ w3s, double* E, double* g1s,
                                                         double* g2s, double* g3s) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    T p[27], gt[27];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double o = (sizeof(T) == 8) ? 0.0 : w2s[9 * (size_t)t + q % 3];
        p[q] = (T)(w1s[9 * (size_t)t + q] - o);
        p[9 + q] = (T)(w2s[9 * (size_t)t + q] - o);
        p[18 + q] = (T)(w3s[9 * (size_t)t + q] - o);
    }
#pragma unroll
    for (int q = 0; q < 27; ++q) gt[q] = T(0);
    E[t] = (double)model_3b<T>(p, gt);
#pragma unroll
    for (int q = 0; q < 9; ++q) {  // accumulate like the reference (SOURCE/mbpol-3b-poly.cpp:39-42)
        g1s[9 * (size_t)t + q] += (double)gt[q];
        g2s[9 * (size_t)t + q] += (double)gt[9 + q];
        g3s[9 * (size_t)t + q] += (double)gt[18 + q];
    }
}

// --- the per-cluster force matrices of the reference's C entry points --------------------
// mbpol_2b_poly_ / mbpol_3b_poly_ also return a pairwise split of the cluster gradient,
// read by the reference's HEAT_STRESS build (SOURCE/mbpol.f90:564-566, :951-953): entry
// (i, j, :) of the sites of a cluster is the gradient of the polynomial variable that links
// sites i and j (g_v dv/d(r_i - r_j)), +/- for the two orders.

// 2B (SOURCE/mbpol-2b-poly.cpp:449-653): the 10 x 10 x 3 matrix over O, H, H, O, H, H and
// the four X sites, the X rows redistributed onto their monomer's O, H, H through the
// X-site geometry and the X columns of atom rows moved onto the other monomer's O, then the
// 6 x 6 x 3 block of the atoms times the switch, the switch's gradient added to the two O-O
// entries.  The diagonal has no variable: the reference copies it from an uninitialised
// array, here it is 0.  Beyond the cutoff the matrix is not touched, as in the reference.
__device__ __forceinline__ void fm_xrows(const double* oh1, const double* oh2, double* gX1, double* gX2,
                                         double* grd, bool clear) {
    // rows X1, X2 (entries at gX1, gX2) onto rows O, H1, H2 (grd + 30 k) of the same column
    const double gm[3] = {gX1[0] - gX2[0], gX1[1] - gX2[1], gX1[2] - gX2[2]};
    const double t1[3] = {oh2[1] * gm[2] - oh2[2] * gm[1], oh2[2] * gm[0] - oh2[0] * gm[2],
                          oh2[0] * gm[1] - oh2[1] * gm[0]};
    const double t2[3] = {oh1[1] * gm[2] - oh1[2] * gm[1], oh1[2] * gm[0] - oh1[0] * gm[2],
                          oh1[0] * gm[1] - oh1[1] * gm[0]};
    for (int i = 0; i < 3; ++i) {
        const double gsum = gX1[i] + gX2[i];
        const double in_plane = 0.5 * m2b::in_plane_gamma * gsum;
        const double gh1 = in_plane + m2b::out_of_plane_gamma * t1[i];
        const double gh2 = in_plane - m2b::out_of_plane_gamma * t2[i];
        grd[i] += gsum - (gh1 + gh2);
        grd[i + 30] += gh1;
        grd[i + 60] += gh2;
        if (clear) {
            gX1[i] = 0.0;
            gX2[i] = 0.0;
        }
    }
}

__device__ void fm_2b(const double* w1, const double* w2, double* fm) {
    const double dOO[3] = {w1[0] - w2[0], w1[1] - w2[1], w1[2] - w2[2]};
    const double rOO = sqrt(dOO[0] * dOO[0] + dOO[1] * dOO[1] + dOO[2] * dOO[2]);
    if (rOO > kR2f) return;
    double xc[30];
    for (int i = 0; i < 9; ++i) {
        xc[i] = w1[i];
        xc[9 + i] = w2[i];
    }
    double oha[2][3], ohb[2][3];
    xsites(xc + m2b::Oa, oha[0], oha[1], xc + m2b::Xa1, xc + m2b::Xa2);
    xsites(xc + m2b::Ob, ohb[0], ohb[1], xc + m2b::Xb1, xc + m2b::Xb2);
    double v[31], gg[31];
    for (int q = 0; q < 31; ++q) {
        const m2b::V d = m2b::kV[q];
        const double dx = xc[d.s1] - xc[d.s2], dy = xc[d.s1 + 1] - xc[d.s2 + 1], dz = xc[d.s1 + 2] - xc[d.s2 + 2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double e = exp(d.k * (d.r0 - r));
        if (!d.coul) {
            v[q] = e;
            gg[q] = -d.k * e / r;
        } else {
            const double rinv = 1.0 / r;
            v[q] = e * rinv;
            gg[q] = -(d.k + rinv) * v[q] * rinv;
        }
    }
    double acc[32];
    for (int q = 0; q < 32; ++q) acc[q] = 0.0;
    poly2b<double>(v, acc);
    double tmp[300];
    for (int q = 0; q < 300; ++q) tmp[q] = 0.0;
    for (int q = 0; q < 31; ++q) {
        const m2b::V d = m2b::kV[q];
        for (int c = 0; c < 3; ++c) {
            const double t = acc[1 + q] * ((xc[d.s1 + c] - xc[d.s2 + c]) * gg[q]);
            tmp[10 * d.s1 + d.s2 + c] = t;    // row site s1, column site s2 (10 sites x 3 per row)
            tmp[10 * d.s2 + d.s1 + c] = -t;
        }
    }
    // site s at row 30 s, column 3 s: Oa 0, Ha1 1, Ha2 2, Ob 3, Hb1 4, Hb2 5, Xa1 6, Xa2 7, Xb1 8, Xb2 9
    auto at = [&](int r, int c) { return tmp + 30 * r + 3 * c; };
    fm_xrows(oha[0], oha[1], at(6, 3), at(7, 3), at(0, 3), false);   // X rows of a, column Ob
    fm_xrows(oha[0], oha[1], at(6, 4), at(7, 4), at(0, 4), false);   // column Hb1
    fm_xrows(oha[0], oha[1], at(6, 5), at(7, 5), at(0, 5), false);   // column Hb2
    fm_xrows(ohb[0], ohb[1], at(8, 0), at(9, 0), at(3, 0), false);   // X rows of b, column Oa
    fm_xrows(ohb[0], ohb[1], at(8, 1), at(9, 1), at(3, 1), false);
    fm_xrows(ohb[0], ohb[1], at(8, 2), at(9, 2), at(3, 2), false);
    // X columns of atom rows onto the other monomer's O column
    const int ra[3] = {0, 1, 2}, rb[3] = {3, 4, 5};
    for (int k = 0; k < 3; ++k)
        for (int x = 8; x <= 9; ++x)
            for (int c = 0; c < 3; ++c) {
                at(ra[k], 3)[c] += at(ra[k], x)[c];
                at(ra[k], x)[c] = 0.0;
            }
    for (int k = 0; k < 3; ++k)
        for (int x = 6; x <= 7; ++x)
            for (int c = 0; c < 3; ++c) {
                at(rb[k], 0)[c] += at(rb[k], x)[c];
                at(rb[k], x)[c] = 0.0;
            }
    // X-X entries: X rows onto O, H, H rows, the entries to the other monomer's O column
    fm_xrows(oha[0], oha[1], at(6, 8), at(7, 8), at(0, 3), true);
    fm_xrows(oha[0], oha[1], at(6, 9), at(7, 9), at(0, 3), true);
    fm_xrows(ohb[0], ohb[1], at(8, 6), at(9, 6), at(3, 0), true);
    fm_xrows(ohb[0], ohb[1], at(8, 7), at(9, 7), at(3, 0), true);
    double gsw;
    const double sw = f_switch(rOO, kR2i, kR2f, gsw);
    for (int r = 0; r < 6; ++r)
        for (int i = 0; i < 18; ++i) fm[i + 18 * r] = sw * tmp[i + 30 * r];
    gsw *= acc[0] / rOO;
    for (int i = 0; i < 3; ++i) {
        const double d = gsw * dOO[i];
        fm[i + 18 * 0 + 3 * 3] += d;
        fm[i + 18 * 3 + 3 * 0] -= d;
    }
}

// 3B (SOURCE/mbpol-3b-poly.cpp:208-312): the 9 x 9 x 3 matrix over the three monomers'
// O, H, H, every off-diagonal entry assigned from its variable (the gradient including
// the switching product), the switch's gradients added to the O-O entries; the diagonal is
// not written, as in the reference.
__device__ void fm_3b(const double* t, double* fm) {
    double x[36], fk[36];
    vars_3b<double>(t, x, fk);
    double acc[37];
    for (int q = 0; q < 37; ++q) acc[q] = 0.0;
    poly3b<double>(x, acc);
    double rab[3], rac[3], rbc[3], drab = 0.0, drac = 0.0, drbc = 0.0;
    for (int n = 0; n < 3; ++n) {
        rab[n] = t[m3b::Oa + n] - t[m3b::Ob + n];
        drab += rab[n] * rab[n];
        rac[n] = t[m3b::Oa + n] - t[m3b::Oc + n];
        drac += rac[n] * rac[n];
        rbc[n] = t[m3b::Ob + n] - t[m3b::Oc + n];
        drbc += rbc[n] * rbc[n];
    }
    drab = sqrt(drab);
    drac = sqrt(drac);
    drbc = sqrt(drbc);
    double gab, gac, gbc;
    const double sab = f_switch(drab, 0.0, kR3f, gab);
    const double sac = f_switch(drac, 0.0, kR3f, gac);
    const double sbc = f_switch(drbc, 0.0, kR3f, gbc);
    const double s = sab * sac + sab * sbc + sac * sbc;
    for (int q = 0; q < 36; ++q) {
        const m3b::V d = m3b::kV[q];
        const double gq = (acc[1 + q] * s) * fk[q];
        const int i = d.a1 / 3, j = d.a2 / 3;
        for (int c = 0; c < 3; ++c) {
            const double v = gq * (t[d.a1 + c] - t[d.a2 + c]);
            fm[27 * i + 3 * j + c] = v;
            fm[27 * j + 3 * i + c] = -v;
        }
    }
    const double e = acc[0];
    gab *= (sac + sbc) * e / drab;
    gac *= (sab + sbc) * e / drac;
    gbc *= (sab + sac) * e / drbc;
    for (int n = 0; n < 3; ++n) {
        fm[27 * 0 + 3 * 3 + n] += gab * rab[n];
        fm[27 * 3 + 3 * 0 + n] -= gab * rab[n];
        fm[27 * 0 + 3 * 6 + n] += gac * rac[n];
        fm[27 * 6 + 3 * 0 + n] -= gac * rac[n];
        fm[27 * 3 + 3 * 6 + n] += gbc * rbc[n];
        fm[27 * 6 + 3 * 3 + n] -= gbc * rbc[n];
    }
}

__global__ void __launch_bounds__(kThreads) k_2b_fm(int n, const double* __restrict__ w1s,
                                                     const double* __restrict__ w2s, double* __restrict__ fms) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    fm_2b(w1s + 9 * (size_t)t, w2s + 9 * (size_t)t, fms + 108 * (size_t)t);
}

__global__ void __launch_bounds__(kThreads) k_3b_fm(int n, const double* __restrict__ w1s,
                                                     const double* __restrict__ w2s, const double* __restrict__ w3s,
                                                     double* __restrict__ fms) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double p[27];
    for (int q = 0; q < 9; ++q) {
        p[q] = w1s[9 * (size_t)t + q];
        p[9 + q] = w2s[9 * (size_t)t + q];
        p[18 + q] = w3s[9 * (size_t)t + q];
    }
    fm_3b(p, fms + 243 * (size_t)t);
}

__global__ void __launch_bounds__(kThreads) k_jkin(int n, const double* __restrict__ vx,
                                                    const double* __restrict__ vy, const double* __restrict__ vz,
                                                    const double* __restrict__ mass, const double* __restrict__ ae,
                                                    double* acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double j[3] = {0.0, 0.0, 0.0};
    if (i < n) {
        const double v0 = vx[i], v1 = vy[i], v2 = vz[i];
        const double kin = 0.5 * mass[i] * (v0 * v0 + v1 * v1 + v2 * v2);
        const double eng = kin + (ae ? ae[i] : 0.0);
        j[0] = eng * v0;
        j[1] = eng * v1;
        j[2] = eng * v2;
    }
    __shared__ double sh[kThreads / 32][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double s = warp_sum(j[q]);
        if (lane == 0) sh[w][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int k = 0; k < kThreads / 32; ++k) s += sh[k][threadIdx.x];
        atomicAdd(acc + S_JKIN + threadIdx.x, s);
    }
}

static int blocks(int n) { return (n + kThreads - 1) / kThreads; }

cudaError_t launch_2b(const MbpolArgs& a, const int2* pairs, int n, int precision, const MixedPass& mp,
                      cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (precision == 0 || !(mp.limit2 > 0.f)) {
        k_mbpol_2b<double><<<blocks(n), kThreads, 0, s>>>(a, pairs, n, nullptr, HardList{nullptr, nullptr, 0.f});
    } else {
        k_mbpol_2b<float><<<blocks(n), kThreads, 0, s>>>(a, pairs, n, nullptr,
                                                         HardList{mp.hard2, mp.count + 0, mp.limit2});
        k_mbpol_2b<double><<<blocks(n), kThreads, 0, s>>>(a, mp.hard2, n, mp.count + 0,
                                                          HardList{nullptr, nullptr, 0.f});
    }
    return cudaGetLastError();
}

cudaError_t launch_3b(const MbpolArgs& a, const int4* trip, int n, int precision, const MixedPass& mp,
                      cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (precision == 0 || !(mp.limit3 > 0.f)) {
        k_mbpol_3b<double><<<blocks(n), kThreads, 0, s>>>(a, trip, n, nullptr, HardList{nullptr, nullptr, 0.f});
    } else if (!(mp.limit3 < 3.0e38f)) {
        // no hand-off requested: every trimer in FP32
        k_mbpol_3b<float><<<blocks(n), kThreads, 0, s>>>(a, trip, n, nullptr, HardList{nullptr, nullptr, 0.f});
    } else {
        k_mbpol_3b<float><<<blocks(n), kThreads, 0, s>>>(a, trip, n, nullptr,
                                                         HardList{mp.hard3, mp.count + 1, mp.limit3});
        k_mbpol_3b<double><<<blocks(n), kThreads, 0, s>>>(a, mp.hard3, n, mp.count + 1,
                                                          HardList{nullptr, nullptr, 0.f});
    }
    return cudaGetLastError();
}

static int blocks_l(long n) { return (int)((n + kThreads - 1) / kThreads); }

cudaError_t launch_2b_dev(const MbpolArgs& a, const int2* pairs, long cap, const int* n_dev, int precision,
                          const MixedPass& mp, cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    const int g = blocks_l(cap);
    if (precision == 0 || !(mp.limit2 > 0.f)) {
        k_mbpol_2b<double><<<g, kThreads, 0, s>>>(a, pairs, 0, n_dev, HardList{nullptr, nullptr, 0.f});
    } else {
        k_mbpol_2b<float><<<g, kThreads, 0, s>>>(a, pairs, 0, n_dev, HardList{mp.hard2, mp.count + 0, mp.limit2});
        k_mbpol_2b<double><<<g, kThreads, 0, s>>>(a, mp.hard2, 0, mp.count + 0, HardList{nullptr, nullptr, 0.f});
    }
    return cudaGetLastError();
}

cudaError_t launch_3b_dev(const MbpolArgs& a, const int4* trip, long cap, const int* n_dev, int precision,
                          const MixedPass& mp, cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    const int g = blocks_l(cap);
    if (precision == 0 || !(mp.limit3 > 0.f)) {
        k_mbpol_3b<double><<<g, kThreads, 0, s>>>(a, trip, 0, n_dev, HardList{nullptr, nullptr, 0.f});
    } else if (!(mp.limit3 < 3.0e38f)) {
        k_mbpol_3b<float><<<g, kThreads, 0, s>>>(a, trip, 0, n_dev, HardList{nullptr, nullptr, 0.f});
    } else {
        k_mbpol_3b<float><<<g, kThreads, 0, s>>>(a, trip, 0, n_dev, HardList{mp.hard3, mp.count + 1, mp.limit3});
        k_mbpol_3b<double><<<g, kThreads, 0, s>>>(a, mp.hard3, 0, mp.count + 1, HardList{nullptr, nullptr, 0.f});
    }
    return cudaGetLastError();
}

bool fused_applies(int precision, const MixedPass& mp) {
    // the mixed method's default split only (2B in FP64, every trimer in FP32, no
    // hand-off).  In FP64 both bodies compete for the FP64 pipe and the separate
    // kernels (full register file) are faster.
    return precision != 0 && !(mp.limit2 > 0.f) && !(mp.limit3 < 3.0e38f);
}

int dimer_parts() { return kPoly2BF64Parts; }

cudaError_t launch_23(const MbpolArgs& a, const int2* pairs, int n2, const int* n2_dev, const int4* trip, int n3,
                      const int* n3_dev, int precision, int* ctr, int nsm, cudaStream_t s, double* partial,
                      int* done, long part_cap, int dimer_warps, bool shared_sm) {
    const int nt = shared_sm ? kFusedThreadsShared : kFusedThreads;
    if (dimer_warps <= 0) dimer_warps = kFusedDimerWarps;
    if (dimer_warps >= nt / 32) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(ctr, 0, 2 * sizeof(int), s);
    if (e) return e;
    if (precision == 0) return cudaErrorInvalidValue;   // see fused_applies
    if (!partial || !done) part_cap = 0;
    if (part_cap > 0 && (e = cudaMemsetAsync(done, 0, (size_t)part_cap * sizeof(int), s))) return e;
    if (shared_sm)
        k_mbpol_23<double, float, kFusedThreadsShared><<<nsm, kFusedThreadsShared, 0, s>>>(
            a, pairs, n2, n2_dev, trip, n3, n3_dev, ctr, partial, done, part_cap, dimer_warps);
    else
        k_mbpol_23<double, float, kFusedThreads><<<nsm, kFusedThreads, 0, s>>>(
            a, pairs, n2, n2_dev, trip, n3, n3_dev, ctr, partial, done, part_cap, dimer_warps);
    return cudaGetLastError();
}

cudaError_t launch_2b_direct(int n, const double* w1, const double* w2, double* E, double* g1, double* g2,
                             int precision, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (precision == 0) k_2b_direct<double><<<blocks(n), kThreads, 0, s>>>(n, w1, w2, E, g1, g2);
    else k_2b_direct<float><<<blocks(n), kThreads, 0, s>>>(n, w1, w2, E, g1, g2);
    return cudaGetLastError();
}

cudaError_t launch_3b_direct(int n, const double* w1, const double* w2, const double* w3, double* E, double* g1,
                             double* g2, double* g3, int precision, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (precision == 0) k_3b_direct<double><<<blocks(n), kThreads, 0, s>>>(n, w1, w2, w3, E, g1, g2, g3);
    else k_3b_direct<float><<<blocks(n), kThreads, 0, s>>>(n, w1, w2, w3, E, g1, g2, g3);
    return cudaGetLastError();
}

cudaError_t launch_2b_fm(int n, const double* w1, const double* w2, double* fm, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_2b_fm<<<blocks(n), kThreads, 0, s>>>(n, w1, w2, fm);
    return cudaGetLastError();
}

cudaError_t launch_3b_fm(int n, const double* w1, const double* w2, const double* w3, double* fm, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_3b_fm<<<blocks(n), kThreads, 0, s>>>(n, w1, w2, w3, fm);
    return cudaGetLastError();
}

cudaError_t launch_jkin(int n, const double* vx, const double* vy, const double* vz, const double* mass,
                        const double* ae, double* acc, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_jkin<<<blocks(n), kThreads, 0, s>>>(n, vx, vy, vz, mass, ae, acc);
    return cudaGetLastError();
}

}  // namespace mbx
