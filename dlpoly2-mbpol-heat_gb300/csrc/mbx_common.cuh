// Shared device helpers for the MB-pol GB300 path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mbx {

constexpr double kEngUnit = 418.4;        // SOURCE/mbpol.f90:37, internal units per kcal/mol
constexpr double kR2f = 6.5;              // 2B outer cutoff, SOURCE/mbpol-2b-poly.cpp:1863
constexpr double kR2i = 4.5;              // 2B switch start, SOURCE/mbpol-2b-poly.cpp:1862
constexpr double kR3f = 4.5;              // 3B cutoff, SOURCE/mbpol-3b-poly.cpp:1489
constexpr int kThreads = 128;

// Simulation-cell description passed by value to kernels.
struct Cell {
    int imcon;          // 1 cubic, 2 orthorhombic, 3 triclinic (DL_POLY keys)
    double c[9];        // cell vectors, DL_POLY order
    double rc[9];       // inverse (imcon 3)
    double inv[3];      // 1/c[0], 1/c[4], 1/c[8]
};

// Unfused double arithmetic: list tests and imaging must round exactly like the
// reference's x86-64 build (no contraction into FMA).
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// 1 / sqrt(x) for x > 0 (a squared pair distance): the FP32 estimate refined by two
// Newton-Raphson steps y <- y (3 - x y^2) / 2, each squaring the relative error (~1e-7 ->
// ~1e-14 -> rounding level).  Eight FP64-pipe operations where a correctly rounded root
// and a division take about twice that; results agree with them to a few ulp.
__device__ __forceinline__ double rsqrt_nr(double x) {
    double y = (double)rsqrtf((float)x);
    y = y * (1.5 - 0.5 * x * y * y);
    return y * (1.5 - 0.5 * x * y * y);
}

// Fortran NINT on a double: round half away from zero.
// The image shift: the reference's NINT rounds halves away from zero, rint to even; the two
// differ only at a scaled separation of exactly k + 1/2, a separation of half a box or more,
// outside every cutoff of the path (rcut <= half the box), so every pair within reach gets
// the same shift bit for bit.  rint is one FP64 instruction, round several.
__device__ __forceinline__ double nint(double x) { return rint(x); }

// image_vectors (SOURCE/mbpol.f90:1305-1361) applied to one vector.
__device__ __forceinline__ void image(const Cell& cl, double& x, double& y, double& z) {
    if (cl.imcon == 1) {
        x = dsub(x, dmul(cl.c[0], nint(dmul(x, cl.inv[0]))));
        y = dsub(y, dmul(cl.c[0], nint(dmul(y, cl.inv[0]))));
        z = dsub(z, dmul(cl.c[0], nint(dmul(z, cl.inv[0]))));
    } else if (cl.imcon == 2) {
        x = dsub(x, dmul(cl.c[0], nint(dmul(x, cl.inv[0]))));
        y = dsub(y, dmul(cl.c[4], nint(dmul(y, cl.inv[1]))));
        z = dsub(z, dmul(cl.c[8], nint(dmul(z, cl.inv[2]))));
    } else {
        const double* r = cl.rc;
        const double ssx = dadd(dadd(dmul(r[0], x), dmul(r[3], y)), dmul(r[6], z));
        const double ssy = dadd(dadd(dmul(r[1], x), dmul(r[4], y)), dmul(r[7], z));
        const double ssz = dadd(dadd(dmul(r[2], x), dmul(r[5], y)), dmul(r[8], z));
        const double xss = dsub(ssx, nint(ssx));
        const double yss = dsub(ssy, nint(ssy));
        const double zss = dsub(ssz, nint(ssz));
        const double* c = cl.c;
        x = dadd(dadd(dmul(c[0], xss), dmul(c[3], yss)), dmul(c[6], zss));
        y = dadd(dadd(dmul(c[1], xss), dmul(c[4], yss)), dmul(c[7], zss));
        z = dadd(dadd(dmul(c[2], xss), dmul(c[5], yss)), dmul(c[8], zss));
    }
}

// |image(a - b)|^2 with the reference's association ((x^2 + y^2) + z^2).
__device__ __forceinline__ double dist2_img(const Cell& cl, const double* a, const double* b,
                                            double* d = nullptr) {
    double x = dsub(a[0], b[0]), y = dsub(a[1], b[1]), z = dsub(a[2], b[2]);
    image(cl, x, y, z);
    if (d) { d[0] = x; d[1] = y; d[2] = z; }
    return dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z));
}

// Dimer test of do_dimer (SOURCE/mbpol.f90:496-503): keep iff r^2 <= r2f^2.
__device__ __forceinline__ bool dimer_in(double r2) { return !(r2 > kR2f * kR2f); }
// 3B pair test of do_trimer (SOURCE/mbpol.f90:839-862): the distance itself is compared.
__device__ __forceinline__ bool tri_edge(double r2) { return !(__dsqrt_rn(r2) > kR3f); }

// FP32 |image(a - b)|^2 of two O positions, for list pre-tests only.
__device__ __forceinline__ float dist2_img_f(const Cell& cl, float4 a, float4 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
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

// The two list tests of a water pair: the dimer test of do_dimer (r^2 <= 6.5^2) and the
// 3B edge test of do_trimer (r <= 4.5).  They are decided in FP32 (from the FP32 copies
// `of` of the O positions) when r^2 is more than 0.05 A^2 from both cutoffs -- far above
// FP32 rounding, which also covers an image chosen differently at half a box length,
// where both images have the same length -- and with the reference's FP64 arithmetic
// otherwise, so the lists are the reference's.
__device__ __forceinline__ void pair_tests(const Cell& cl, const float4* of, const double* mono, int i, int j,
                                           bool& in2, bool& in3) {
    const float r2f = dist2_img_f(cl, of[i], of[j]);
    const float c2 = (float)(kR2f * kR2f), c3 = (float)(kR3f * kR3f);
    if (fabsf(r2f - c2) < 0.05f || fabsf(r2f - c3) < 0.05f) {
        const double r2 = dist2_img(cl, mono + 9 * (size_t)i, mono + 9 * (size_t)j);
        in2 = dimer_in(r2);
        in3 = tri_edge(r2);
    } else {
        in2 = r2f < c2;
        in3 = r2f < c3;
    }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NV doubles; thread 0 of the block adds the totals atomically.
template <int NV>
__device__ __forceinline__ void block_sum_atomic(double (&v)[NV], double* out) {
    __shared__ double red[kThreads / 32][NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = warp_sum(v[q]);
        if (lane == 0) red[w][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        const int nwarp = ((int)blockDim.x + 31) >> 5;   // blocks of up to kThreads
        for (int i = 0; i < nwarp; ++i) s += red[i][threadIdx.x];
        atomicAdd(out + threadIdx.x, s);
    }
}

// Pair k (0 <= k < n(n-1)/2) of the pairs (p, q), p < q < n, in lexicographic order.
__device__ __forceinline__ void pair_of_index(int n, int k, int& p, int& q) {
    const double b = 2.0 * n - 1.0;
    int pp = (int)((b - sqrt(b * b - 8.0 * k)) * 0.5);
    auto off = [n](int r) { return r * (2 * n - r - 1) / 2; };
    if (pp < 0) pp = 0;
    while (pp > 0 && off(pp) > k) --pp;
    while (off(pp + 1) <= k) ++pp;
    p = pp;
    q = k - off(pp) + pp + 1;
}

}  // namespace mbx
