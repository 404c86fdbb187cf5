// Smooth particle-mesh Ewald for point charges and induced point dipoles (mbx_spme.cu),
// and the k-vector heat-current term shared with the explicit Ewald sum (mbx_polar.cu).
#pragma once

#include "mbx_common.cuh"

namespace mbx {

// ew1p's HEAT_CURRENT per-atom stress contracted with the velocities, for one k vector
// (SOURCE/ewald1p.f:575-690), regrouped into sums over the sites.  s1 + i s2 is the total
// structure factor sum_j (q_j + i k.mu_j) e^{ik.r_j}, Mc + i Ms the dipole one
// sum_j mu_j e^{ik.r_j}, V1 + i V2 that of q_j v_j (v_b), W1 + i W2 that of mu_jc v_jb
// ([c][b], c major); f = sfac akk and akv2 = 2 (1 / k^2 + 1 / (4 alpha^2)).  The reference
// reads only the upper triangle of the per-atom stress, and the regrouping keeps that.
__host__ __device__ inline void ew1p_heat_kterm(const double kx[3], double s1, double s2, const double Mc[3],
                                                const double Ms[3], const double V1[3], const double V2[3],
                                                const double W1[9], const double W2[9], double f, double akv2,
                                                double out[3]) {
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
    for (int aa = 0; aa < 3; ++aa) {
        double y = 0.0;
        for (int b = 0; b < 3; ++b) {
            const int lo = aa < b ? aa : b, hi = aa < b ? b : aa;
            y += kx[lo] * Q[hi][b];
        }
        out[aa] = f * (P[aa] - akv2 * kx[aa] * kp + y);
    }
}

// One axis of the hand-written FFT: length n = product of the radices r[0..nst-1]
// (each 2, 3, 4 or 5), twiddles exp(2 pi i m / n) at tw + tw_off.
struct FftAxis {
    int n = 0, nst = 0, tw_off = 0;
    int r[16] = {};
};

// SPME k space on a K1 x K2 x K3 grid with cardinal B-splines of order p (4..8).
//
// The charge part is the reference's ewald_spme (SOURCE/ewald_spme.f:1-362 with
// bspgen.f, bspcoe.f, spme_for.f): fractional coordinates t_a = K_a (s_a + 1/2), weights
// M_p(t_a - g_a) at the p grid points g_a = floor(t_a) - j, the Euler-spline moduli
// |b(m)|^2 in the influence function, the spherical k cut at 1.05 x half the grid,
// forces with the mean (the SPME drift) removed.  The reference has no SPME for induced
// dipoles (its polar branch runs the explicit Ewald sum only); here a dipole is spread as
// mu . grad M_p, so the grid density is that of charges plus point dipoles, the energy is
// (2 pi / V) r4pie0 / epsq sum_m G(m) |F[Q](m)|^2, the field at a site is minus the
// gradient of the convolved grid, and the forces are the exact gradient of that energy
// (second derivatives of the splines for the dipoles).
//
// Grids are complex, x fastest (K1), FFT with exp(+2 pi i m.g / K) forward and the
// opposite sign backward, both unnormalised; two real densities share one complex grid
// (real and imaginary part), which the even, real influence function keeps apart.
// The Nyquist frequencies of even grids carry no weight (G = 0 there; the reference
// gives them to m = -K/2, where the Gaussian factor is below 1e-12 at the grids used).
struct SpmeState {
    int order = 0;                 // B-spline order of the prepared tables (0: none)
    int K[3] = {0, 0, 0};
    size_t ng = 0;                 // K1 K2 K3
    double alpha = -1.0;
    double cellc[9] = {};
    double rc[9] = {};             // reciprocal cell (the k-vector rows of mbx_polar.cu)
    double jac[9] = {};            // dt_a / dr_c = K_a rc[a + 3c], [a][c]
    FftAxis ax[3];
    double* G = nullptr;           // influence function per grid point (moduli included)
    float* G32 = nullptr;
    double2* tw = nullptr;         // twiddles, the three axes one after the other
    float2* tw32 = nullptr;
    double2* grid = nullptr;       // complex grids, ngrid_cap of them
    float2* grid32 = nullptr;
    float2* hgrid32 = nullptr;     // the mixed final pass's 8 heat grids in FP32
    size_t hgrid_cap_ng = 0;
    int4* sib = nullptr;           // per site floor(t_a) mod K_a (frame)
    float4* sw = nullptr;          //   FP32 passes: t_a - floor(t_a)
    double* spl = nullptr;         //   FP64 passes: B-spline values and derivatives per axis
    int site_cap = 0;
    double* part = nullptr;        // per-block partial sums of the k-vector terms
    size_t g_cap = 0, part_cap = 0;
    int tw_cap = 0, ngrid_cap = 0, grid32_cap_ng = 0;
    size_t grid_cap_ng = 0;
    bool have32 = false;
    long launches = 0;             // kernels issued by the last call of each kind

    ~SpmeState();
    void release();
    // Tables for this cell, splitting parameter, order and grid (kept while they are
    // unchanged); `ngrids` complex FP64 grids (1, or 9 with the heat current), and the
    // FP32 grid and tables when fp32.
    cudaError_t prepare(const double* cell, double alpha, int order, const int* K, bool fp32, int ngrids,
                        cudaStream_t s);
    // k-space field of the masked dipoles md at every site, with the self term:
    // efm = (polr2 > 1e-6 ? field : 0) + dum * mu (3 blocks of n, mu from mx/my/mz); with
    // q non-null (the first evaluation) also the charges' field efc (3 blocks of n).
    cudaError_t field64(int n, const double* x, const double* y, const double* z, const double* q,
                        const double4* md, const double* polr2, const double* mx, const double* my,
                        const double* mz, double sfac, double dum, double* efm, double* efc, cudaStream_t s);
    // The site frame for these positions (once per call, after prepare and before any spread
    // or gather): grid indices, FP32 fractions and the FP64 spline table.
    cudaError_t frame(int n, const double* x, const double* y, const double* z, cudaStream_t s);
    // The same in FP32 for the correction solve: e32k = (polr2 > 1e-6 ? field(d) : 0) + dum d.
    // stop (device, or null): when nonzero the kernels return at once (a CG solve that has
    // stopped while further sweeps were queued).
    cudaError_t field32(int n, const double* x, const double* y, const double* z, const float4* d,
                        const double* polr2, double sfac, double dum, float* e32k, cudaStream_t s,
                        const int* stop = nullptr);
    // Final pass at the converged dipoles.  part5 (5 blocks of n): per site the k-space
    // force / scale (mean removed), half the charges' potential, half the dipoles'
    // potential (the layout of the Ewald force gather, scale = 2 sfac); acc[48..58] =
    // {engc, engdum, omg 11 22 33 12 13 23, jpot (the ew1p heat term, with vh)} in the
    // half-space convention of the Ewald sums; acc[11..19] scratch.  vh: the 12 per-site
    // heat weights (q v, mu_c v_b) or null.  field (3 blocks of n) receives the total
    // k-space field without the self term, or null.
    // heat32 (mixed precision, with vh): the heat densities on FP32 grids (FP32 spread, FFT and
    // products; the k sums in FP64), the charges and dipoles in FP64 as always.
    cudaError_t final(int n, const double* x, const double* y, const double* z, const double* q,
                      const double4* md, const double* vh, double sfac, double* part5, double* acc, double* field,
                      cudaStream_t s, bool heat32 = false);
    // Forward (sign +1) or backward (-1) unnormalised 3D FFT of `count` FP64 grids in place.
    cudaError_t fft64(double2* data, int count, int sign, cudaStream_t s);
};

// Smallest even K >= x whose only prime factors are 2, 3 and 5.
int spme_smooth_even(double x);

}  // namespace mbx
