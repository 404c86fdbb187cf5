// Smooth particle-mesh Ewald for the charges and induced dipoles of the TTM4-F
// electrostatics, with a hand-written 3D FFT.  See mbx_spme.cuh for the method and the
// conventions; the reference's charge-only SPME is SOURCE/ewald_spme.f (B-splines
// SOURCE/bspgen.f, moduli SOURCE/bspcoe.f, forces SOURCE/spme_for.f, FFT SOURCE/dlpfft3.f).
//
//   spread    8 lanes per site, one z plane of its p^3-point B-spline support each, FP64
//             (FP32 for the correction solve) atomic adds into the complex grid
//   fft       one axis per launch: a block loads nl lines into shared memory ([element][line],
//             line pitch nl + 1), runs the Stockham radix-2/3/4/5 stages there and stores
//             them back; the z pass of a convolution does forward FFT, influence function
//             and backward FFT of its lines in one launch
//   gather    8 lanes per site, one z plane each, summed per x row, then over the lanes
//   k terms   thread per grid point: energies, virial and heat-current terms of every k
//             vector, block partial sums added in order by one block
#include "mbx_kernels.cuh"
#include "mbx_spme.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <vector>

namespace mbx {

namespace {

constexpr double kPiS = 3.141592653589793;
constexpr int kFftThreads = 256;
constexpr int kFftPlaneThreads = 1024;  // one block per plane: 64 blocks of a 64^3 grid, so
                                         // each block needs many warps to hide its latencies
constexpr int kSpThreads = 128;
constexpr int kKtThreads = 256;
constexpr int kMaxGrid = 1024;     // points per axis
constexpr int kMaxFftSmem = 200 * 1024;
constexpr int kKtBlocks = 1024;  // blocks of the k-term reduction (partial sums kept in order)

template <typename T>
struct Cx;
template <>
struct Cx<double> {
    typedef double2 t;
};
template <>
struct Cx<float> {
    typedef float2 t;
};

template <typename C>
__device__ __forceinline__ C cadd(C a, C b) {
    C r;
    r.x = a.x + b.x;
    r.y = a.y + b.y;
    return r;
}
template <typename C>
__device__ __forceinline__ C csub(C a, C b) {
    C r;
    r.x = a.x - b.x;
    r.y = a.y - b.y;
    return r;
}
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// sg * i * a
template <typename C>
__device__ __forceinline__ C cmuli(C a, int sg) {
    C r;
    r.x = sg > 0 ? -a.y : a.y;
    r.y = sg > 0 ? a.x : -a.x;
    return r;
}
template <typename C, typename T>
__device__ __forceinline__ C cscale(C a, T f) {
    C r;
    r.x = a.x * f;
    r.y = a.y * f;
    return r;
}

// y_u = sum_t v_t exp(sg 2 pi i t u / R)
template <typename T, int R>
__device__ __forceinline__ void bfly(typename Cx<T>::t* v, int sg) {
    typedef typename Cx<T>::t C;
    if constexpr (R == 2) {
        const C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        const C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        const C b0 = cadd(v[1], v[3]), b1 = cmuli(csub(v[1], v[3]), sg);
        v[0] = cadd(a0, b0);
        v[2] = csub(a0, b0);
        v[1] = cadd(a1, b1);
        v[3] = csub(a1, b1);
    } else if constexpr (R == 3) {
        const T h = T(0.5), s3 = T(0.86602540378443864676);
        const C sm = cadd(v[1], v[2]), df = csub(v[1], v[2]);
        const C c = csub(v[0], cscale(sm, h));
        const C d = cmuli(cscale(df, s3), sg);
        v[0] = cadd(v[0], sm);
        v[1] = cadd(c, d);
        v[2] = csub(c, d);
    } else {   // R == 5
        const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);
        const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);
        const C sa = cadd(v[1], v[4]), da = csub(v[1], v[4]);
        const C sb = cadd(v[2], v[3]), db = csub(v[2], v[3]);
        const C p1 = cadd(v[0], cadd(cscale(sa, c1), cscale(sb, c2)));
        const C p2 = cadd(v[0], cadd(cscale(sa, c2), cscale(sb, c1)));
        const C q1 = cmuli(cadd(cscale(da, s1), cscale(db, s2)), sg);
        const C q2 = cmuli(csub(cscale(da, s2), cscale(db, s1)), sg);
        v[0] = cadd(v[0], cadd(sa, sb));
        v[1] = cadd(p1, q1);
        v[4] = csub(p1, q1);
        v[2] = cadd(p2, q2);
        v[3] = csub(p2, q2);
    }
}

// a / d and a % d for d > 0: a shift and a mask when d is a power of two (the usual grid
// sizes and line counts), the integer division otherwise (the branch is uniform).
struct IDiv {
    int d, sh;
    __device__ __forceinline__ explicit IDiv(int d_) : d(d_), sh(-1) {
        if ((d_ & (d_ - 1)) == 0) {
            sh = 0;
            while ((1 << sh) < d_) ++sh;
        }
    }
    __device__ __forceinline__ int div(int a) const { return sh >= 0 ? a >> sh : a / d; }
    __device__ __forceinline__ int mod(int a) const { return sh >= 0 ? a & (d - 1) : a % d; }
};

// One Stockham stage of radix R over nl lines of length n in shared memory ([e][l], pitch P):
// sub-transforms of length Ns are combined into length Ns R; the output is in natural
// order after the last stage.
template <typename T, int R>
__device__ __forceinline__ void fft_stage(const typename Cx<T>::t* src, typename Cx<T>::t* dst, int n, int Ns,
                                          int P, int nl, const typename Cx<T>::t* tws, int sg) {
    typedef typename Cx<T>::t C;
    const int nb = n / R;
    const int step = n / (Ns * R);
    const IDiv dl(nl), ds(Ns);
    for (int b = threadIdx.x; b < nl * nb; b += blockDim.x) {
        const int l = dl.mod(b), j = dl.div(b);
        const int k = ds.mod(j);
        C v[R];
#pragma unroll
        for (int t = 0; t < R; ++t) v[t] = src[(j + t * nb) * P + l];
        if (Ns > 1) {
#pragma unroll
            for (int t = 1; t < R; ++t) {
                C w = tws[k * t * step];
                if (sg < 0) w.y = -w.y;
                v[t] = cmul(v[t], w);
            }
        }
        bfly<T, R>(v, sg);
        const int o = ds.div(j) * Ns * R + k;
#pragma unroll
        for (int t = 0; t < R; ++t) dst[(o + t * Ns) * P + l] = v[t];
    }
}

// All stages of one axis; returns the buffer holding the result.
template <typename T>
__device__ typename Cx<T>::t* fft_lines(typename Cx<T>::t* a, typename Cx<T>::t* b, const FftAxis& ax, int P, int nl,
                                        const typename Cx<T>::t* tws, int sg) {
    int Ns = 1;
    for (int st = 0; st < ax.nst; ++st) {
        const int R = ax.r[st];
        if (R == 4) fft_stage<T, 4>(a, b, ax.n, Ns, P, nl, tws, sg);
        else if (R == 2) fft_stage<T, 2>(a, b, ax.n, Ns, P, nl, tws, sg);
        else if (R == 3) fft_stage<T, 3>(a, b, ax.n, Ns, P, nl, tws, sg);
        else fft_stage<T, 5>(a, b, ax.n, Ns, P, nl, tws, sg);
        __syncthreads();
        Ns *= R;
        typename Cx<T>::t* t = a;
        a = b;
        b = t;
    }
    return a;
}

struct GridDims {
    int K1, K2, K3;
};

// One axis of the 3D FFT of the grids data + blockIdx.y * gstride.  MODE 0 forward,
// 1 backward, 2 forward then multiply by G then backward (the convolution's last axis),
// 3 multiply by G then backward.  Blocks: axis 0 takes nl consecutive x lines; axes 1
// and 2 take nl consecutive x positions (tile blockIdx.x % ntile) at one z (axis 1) or
// one y (axis 2).
template <typename T, int MODE>
__global__ void __launch_bounds__(kFftThreads) k_fft_axis(typename Cx<T>::t* data, size_t gstride, int axis,
                                                          FftAxis ax, GridDims d, int nl, int ntile,
                                                          const typename Cx<T>::t* tw, const T* G,
                                                          const int* __restrict__ stop) {
    typedef typename Cx<T>::t C;
    if (stop && *stop) return;   // the CG solve that queued this pass has stopped
    extern __shared__ __align__(16) unsigned char fft_smem[];
    const int n = ax.n, P = nl + 1;
    C* s0 = reinterpret_cast<C*>(fft_smem);
    C* s1 = s0 + (size_t)n * P;
    C* tws = s1 + (size_t)n * P;
    C* g = data + (size_t)blockIdx.y * gstride;
    size_t base, estride, lstride;
    int lcount;
    if (axis == 0) {
        const int L0 = blockIdx.x * nl;
        lcount = min(nl, d.K2 * d.K3 - L0);
        base = (size_t)L0 * d.K1;
        estride = 1;
        lstride = d.K1;
    } else {
        const int tile = blockIdx.x % ntile, o = blockIdx.x / ntile;
        const int x0 = tile * nl;
        lcount = min(nl, d.K1 - x0);
        base = axis == 1 ? (size_t)o * d.K1 * d.K2 + x0 : (size_t)o * d.K1 + x0;
        estride = axis == 1 ? (size_t)d.K1 : (size_t)d.K1 * d.K2;
        lstride = 1;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) tws[i] = tw[ax.tw_off + i];
    // element i of the block's tile: line l and element e (axis 0: l = i / n; else l = i % nl)
    const IDiv dn(n), dl(nl);
    const int tot = nl * n, bs = blockDim.x;
    constexpr int U = 4;   // loads in flight per thread
    for (int i0 = threadIdx.x; i0 < tot; i0 += U * bs) {
        C v[U];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const int i = i0 + q * bs;
            const int l = axis == 0 ? dn.div(i) : dl.mod(i), e = axis == 0 ? dn.mod(i) : dl.div(i);
            v[q].x = 0;
            v[q].y = 0;
            if (i < tot && l < lcount) {
                const size_t off = axis == 0 ? base + (size_t)l * lstride + e : base + (size_t)e * estride + l;
                v[q] = g[off];
                if (MODE == 3) v[q] = cscale(v[q], G[off]);
            }
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const int i = i0 + q * bs;
            const int l = axis == 0 ? dn.div(i) : dl.mod(i), e = axis == 0 ? dn.mod(i) : dl.div(i);
            if (i < tot) s0[e * P + l] = v[q];
        }
    }
    __syncthreads();
    C* r = fft_lines<T>(s0, s1, ax, P, nl, tws, (MODE == 0 || MODE == 2) ? 1 : -1);
    if (MODE == 2) {
        for (int i = threadIdx.x; i < tot; i += bs) {
            const int l = dl.mod(i), e = dl.div(i);
            if (l < lcount) r[e * P + l] = cscale(r[e * P + l], G[base + (size_t)e * estride + (size_t)l * lstride]);
        }
        __syncthreads();
        r = fft_lines<T>(r, r == s0 ? s1 : s0, ax, P, nl, tws, -1);
    }
    if (axis == 0) {
        for (int i = threadIdx.x; i < lcount * n; i += bs) {
            const int l = dn.div(i), e = dn.mod(i);
            g[base + (size_t)l * lstride + e] = r[e * P + l];
        }
    } else {
        for (int i = threadIdx.x; i < tot; i += bs) {
            const int l = dl.mod(i), e = dl.div(i);
            if (l < lcount) g[base + (size_t)e * estride + l] = r[e * P + l];
        }
    }
}

// --- B-splines ---------------------------------------------------------------------------
struct SpArgs {
    int n, K1, K2, K3;
    double rc[9];    // s_a = rc[a] x + rc[a + 3] y + rc[a + 6] z
    double jac[9];   // dt_a / dr_c = K_a rc[a + 3c] at [3a + c]
    const int* stop; // FP32 CG sweeps: nonzero = the solve has stopped, return at once
    // FP32 kernels: the per-call site frame (base grid index and fractional part per axis,
    // from the FP64 positions once per call) and the Jacobian in FP32
    const int4* sib;
    const float4* sw;
    float jac32[9];
    // FP64 kernels: the per-call spline table, per site [axis][th, d1, d2][kSplStride]
    const double* spl;
};

constexpr int kSplStride = 8;                    // entries per (axis, kind): orders up to 8
constexpr int kSplSite = 3 * 3 * kSplStride;     // doubles per site

// M_p(w + j), j = 0..p-1, for w in [0, 1) (bspgen's values bspx(i, j + 1)), and with
// ND >= 1 (2) the first (second) derivatives.  Recursion over the order from M_2:
// M_{m+1}(u) = (u M_m(u) + (m + 1 - u) M_m(u - 1)) / m; M_p' and M_p'' are the first and
// second differences of M_{p-1} and M_{p-2}.
template <typename T, int P, int ND>
__device__ __forceinline__ void bspline(T w, T* th, T* d1, T* d2) {
    T a[P];
    a[0] = w;
    a[1] = T(1) - w;
#pragma unroll
    for (int j = 2; j < P; ++j) a[j] = T(0);
#pragma unroll
    for (int m = 2; m < P; ++m) {
        if (ND >= 2 && m == P - 2) {
#pragma unroll
            for (int j = 0; j < P; ++j)
                d2[j] = a[j] - T(2) * (j >= 1 ? a[j - 1] : T(0)) + (j >= 2 ? a[j - 2] : T(0));
        }
        if (ND >= 1 && m == P - 1) {
#pragma unroll
            for (int j = 0; j < P; ++j) d1[j] = a[j] - (j >= 1 ? a[j - 1] : T(0));
        }
#pragma unroll
        for (int j = m; j >= 0; --j) {
            const T lo = j >= 1 ? a[j - 1] : T(0);
            a[j] = ((w + T(j)) * a[j] + (T(m + 1) - w - T(j)) * lo) / T(m);
        }
    }
#pragma unroll
    for (int j = 0; j < P; ++j) th[j] = a[j];
}

// Splines of one site along the three axes and the grid indices of its support:
// gi[a][j] = (floor(t_a) - j) mod K_a.
template <typename T, int P, int ND>
__device__ __forceinline__ void site_splines(const SpArgs& s, double x, double y, double z, int (&gi)[3][P],
                                             T (&th)[3][P], T (&d1)[3][P], T (&d2)[3][P]) {
    const int Ka[3] = {s.K1, s.K2, s.K3};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double t = (double)Ka[a] * (s.rc[a] * x + s.rc[a + 3] * y + s.rc[a + 6] * z + 0.5);
        const double fl = floor(t);
        long long ib = (long long)fl % Ka[a];
        if (ib < 0) ib += Ka[a];
#pragma unroll
        for (int j = 0; j < P; ++j) {
            int g = (int)ib - j;
            gi[a][j] = g < 0 ? g + Ka[a] : g;
        }
        bspline<T, P, ND>((T)(t - fl), th[a], d1[a], d2[a]);
    }
}

// The site frame, once per call: per site floor(t_a) mod K_a, for the FP32 passes the
// fraction t_a - floor(t_a) (FP64, rounded to FP32: 6e-8 absolute), and for the FP64 passes
// the B-spline values with their first and second derivatives (the table site_splines
// would compute in every lane of every FP64 spread and gather).  Thread per (site, axis).
template <int P>
__global__ void k_spme_frame(SpArgs s, const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ z, int4* __restrict__ sib, float4* __restrict__ sw,
                             double* __restrict__ spl) {
    const long t3 = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int j = (int)(t3 / 3), a = (int)(t3 % 3);
    if (j >= s.n) return;
    const int Ka = a == 0 ? s.K1 : (a == 1 ? s.K2 : s.K3);
    const double t = (double)Ka * (s.rc[a] * x[j] + s.rc[a + 3] * y[j] + s.rc[a + 6] * z[j] + 0.5);
    const double fl = floor(t);
    long long b = (long long)fl % Ka;
    if (b < 0) b += Ka;
    reinterpret_cast<int*>(sib + j)[a] = (int)b;
    reinterpret_cast<float*>(sw + j)[a] = (float)(t - fl);
    double th[P], d1[P], d2[P];
    bspline<double, P, 2>(t - fl, th, d1, d2);
    double* o = spl + (size_t)j * kSplSite + a * 3 * kSplStride;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        o[q] = th[q];
        o[kSplStride + q] = d1[q];
        o[2 * kSplStride + q] = d2[q];
    }
}

// site_splines of the FP64 passes from the per-call table (the same values)
template <int P, int ND>
__device__ __forceinline__ void site_splines_tab(const SpArgs& s, int j, int (&gi)[3][P], double (&th)[3][P],
                                                 double (&d1)[3][P], double (&d2)[3][P]) {
    const int4 ib = s.sib[j];
    const int Ka[3] = {s.K1, s.K2, s.K3}, b[3] = {ib.x, ib.y, ib.z};
    const double* row = s.spl + (size_t)j * kSplSite;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int g = b[a] - q;
            gi[a][q] = g < 0 ? g + Ka[a] : g;
            th[a][q] = row[a * 3 * kSplStride + q];
            if (ND >= 1) d1[a][q] = row[a * 3 * kSplStride + kSplStride + q];
            if (ND >= 2) d2[a][q] = row[a * 3 * kSplStride + 2 * kSplStride + q];
        }
    }
}

// site_splines of the FP32 passes from the site frame (no FP64 arithmetic per lane)
template <int P, int ND>
__device__ __forceinline__ void site_splines32(const SpArgs& s, int j, int (&gi)[3][P], float (&th)[3][P],
                                               float (&d1)[3][P], float (&d2)[3][P]) {
    const int4 ib = s.sib[j];
    const float4 w = s.sw[j];
    const int Ka[3] = {s.K1, s.K2, s.K3}, b[3] = {ib.x, ib.y, ib.z};
    const float wa[3] = {w.x, w.y, w.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int g = b[a] - q;
            gi[a][q] = g < 0 ? g + Ka[a] : g;
        }
        bspline<float, P, ND>(wa[a], th[a], d1[a], d2[a]);
    }
}

// dipole in t space: mu_t[a] = sum_c jac[a][c] mu_c
template <typename T>
__device__ __forceinline__ void to_t(const SpArgs& s, double mx, double my, double mz, T* mt) {
#pragma unroll
    for (int a = 0; a < 3; ++a) mt[a] = (T)(s.jac[3 * a] * mx + s.jac[3 * a + 1] * my + s.jac[3 * a + 2] * mz);
}

__device__ __forceinline__ void atomic_add_re(double2* p, double v) { atomicAdd(&p->x, v); }
__device__ __forceinline__ void atomic_add_im(double2* p, double v) { atomicAdd(&p->y, v); }
__device__ __forceinline__ void atomic_add_re(float2* p, float v) { atomicAdd(&p->x, v); }
__device__ __forceinline__ void atomic_add_im(float2* p, float v) { atomicAdd(&p->y, v); }

template <typename DV>
__device__ __forceinline__ void dip_of(const DV* d, int j, double& x, double& y, double& z) {
    const DV v = d[j];
    x = v.x;
    y = v.y;
    z = v.z;
}

// The spread and gather kernels give each site a group of kLanes (8) consecutive lanes, lane
// jz of the group handling the z plane jz of the site's support (lanes jz >= p idle): eight
// times the threads of a thread-per-site form, which left the SMs latency-bound.
constexpr int kLanes = 8;

// a[jz] with jz a run-time lane index, by unrolled selects (a dynamic index would move the
// spline arrays to local memory)
template <typename T, int P>
__device__ __forceinline__ T pick(const T (&a)[P], int jz) {
    T v = a[0];
#pragma unroll
    for (int k = 1; k < P; ++k) v = jz == k ? a[k] : v;
    return v;
}

// Sum of v over the site's lane group (width kLanes, the group's own mask).
template <typename T>
__device__ __forceinline__ T group_sum(T v) {
    const unsigned gm = 0xffu << (threadIdx.x & 24);
#pragma unroll
    for (int o = kLanes / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gm, v, o, kLanes);
    return v;
}

// Spread one density (or two: real and imaginary part) onto the grid.
//   MODE 0: re += mu . grad M                      (dipole field evaluations)
//   MODE 1: re += mu . grad M, im += q M           (the first evaluation: dipoles and charges)
//   MODE 2: re += q M + mu . grad M, im += q M     (final pass: total density and charges)
// Dipoles of sites with polr2 <= 1e-6 are left out (the masked dipoles); polr2 null: dv is
// masked already.
template <typename T, int P, int MODE, typename DV>
__global__ void __launch_bounds__(kSpThreads) k_spme_spread(SpArgs s, const double* __restrict__ x,
                                                            const double* __restrict__ y, const double* __restrict__ z,
                                                            const double* __restrict__ q, const DV* __restrict__ dv,
                                                            const double* __restrict__ polr2,
                                                            typename Cx<T>::t* __restrict__ grid) {
    typedef typename Cx<T>::t C;
    if (s.stop && *s.stop) return;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int j = (int)(t / kLanes), jz = (int)(t % kLanes);
    if (j >= s.n || jz >= P) return;
    // MODE 0 spreads dipoles alone: a masked site (the M sites) adds nothing
    if (MODE == 0 && polr2 && !(polr2[j] > 1e-6)) return;
    int gi[3][P];
    T th[3][P], d1[3][P], d2[3][P];
    T mt[3];
    if constexpr (sizeof(T) == 4 && MODE == 0) {   // the CG sweeps: site frame, FP32 dipoles
        site_splines32<P, 1>(s, j, gi, th, d1, d2);
        const DV d = dv[j];
#pragma unroll
        for (int a = 0; a < 3; ++a) mt[a] = s.jac32[3 * a] * d.x + s.jac32[3 * a + 1] * d.y + s.jac32[3 * a + 2] * d.z;
    } else {
        if constexpr (sizeof(T) == 8) site_splines_tab<P, 1>(s, j, gi, th, d1, d2);
        else site_splines<T, P, 1>(s, x[j], y[j], z[j], gi, th, d1, d2);
        double mxd = 0, myd = 0, mzd = 0;
        if (!polr2 || polr2[j] > 1e-6) dip_of(dv, j, mxd, myd, mzd);
        to_t<T>(s, mxd, myd, mzd, mt);
    }
    const T qj = MODE >= 1 ? (T)q[j] : T(0);
    const size_t K12 = (size_t)s.K1 * s.K2;
    const T tz = pick(th[2], jz), dz = pick(d1[2], jz);
    C* plane = grid + pick(gi[2], jz) * K12;
#pragma unroll
    for (int jy = 0; jy < P; ++jy) {
        const T tyz = th[1][jy] * tz;
        // w = dx (mt_x ty tz) + tx (mt_y dy tz + mt_z ty dz) (+ q tx ty tz)
        const T r1 = mt[0] * tyz;
        T r2 = mt[1] * d1[1][jy] * tz + mt[2] * th[1][jy] * dz;
        if (MODE == 2) r2 += qj * tyz;
        C* row = plane + (size_t)gi[1][jy] * s.K1;
#pragma unroll
        for (int jx = 0; jx < P; ++jx) {
            const T w = d1[0][jx] * r1 + th[0][jx] * r2;
            atomic_add_re(row + gi[0][jx], w);
            if (MODE >= 1) atomic_add_im(row + gi[0][jx], qj * th[0][jx] * tyz);
        }
    }
}

// The ew1p heat weights spread as charge-like densities: mu (3) and the 12 rows of vh
// (q v_b, mu_c v_b), two per complex grid (grids h = 0..7 at grid + h * gstride).
template <int P>
__global__ void __launch_bounds__(kSpThreads) k_spme_spread_heat(SpArgs s, const double* __restrict__ x,
                                                                 const double* __restrict__ y,
                                                                 const double* __restrict__ z,
                                                                 const double4* __restrict__ md,
                                                                 const double* __restrict__ vh,
                                                                 double2* __restrict__ grid, size_t gstride) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int j = (int)(t / kLanes), jz = (int)(t % kLanes);
    if (j >= s.n || jz >= P) return;
    int gi[3][P];
    double th[3][P], d1[3][P], d2[3][P];
    site_splines_tab<P, 0>(s, j, gi, th, d1, d2);
    double w[16];
    const double4 m = md[j];
    w[0] = m.x;
    w[1] = m.y;
    w[2] = m.z;
#pragma unroll
    for (int r = 0; r < 12; ++r) w[3 + r] = vh[(size_t)r * s.n + j];
    w[15] = 0.0;
    const size_t K12 = (size_t)s.K1 * s.K2;
    const double tz = pick(th[2], jz);
    const size_t plane = pick(gi[2], jz) * K12;
#pragma unroll
    for (int jy = 0; jy < P; ++jy) {
        const double tyz = th[1][jy] * tz;
        const size_t row = plane + (size_t)gi[1][jy] * s.K1;
#pragma unroll
        for (int jx = 0; jx < P; ++jx) {
            const double tt = th[0][jx] * tyz;
            const size_t g = row + gi[0][jx];
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                if (w[2 * h] != 0.0) atomicAdd(&grid[h * gstride + g].x, w[2 * h] * tt);
                if (w[2 * h + 1] != 0.0) atomicAdd(&grid[h * gstride + g].y, w[2 * h + 1] * tt);
            }
        }
    }
}

// The same heat densities on 8 FP32 grids (the mixed path's final pass): splines from the
// site frame, one float2 atomic per grid point and grid.
template <int P>
__global__ void __launch_bounds__(kSpThreads) k_spme_spread_heat32(SpArgs s, const double4* __restrict__ md,
                                                                   const double* __restrict__ vh,
                                                                   float2* __restrict__ grid, size_t gstride) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int j = (int)(t / kLanes), jz = (int)(t % kLanes);
    if (j >= s.n || jz >= P) return;
    int gi[3][P];
    float th[3][P], d1[3][P], d2[3][P];
    site_splines32<P, 0>(s, j, gi, th, d1, d2);
    float w[16];
    const double4 m = md[j];
    w[0] = (float)m.x;
    w[1] = (float)m.y;
    w[2] = (float)m.z;
#pragma unroll
    for (int r = 0; r < 12; ++r) w[3 + r] = (float)vh[(size_t)r * s.n + j];
    w[15] = 0.f;
    bool any[8];
#pragma unroll
    for (int h = 0; h < 8; ++h) any[h] = w[2 * h] != 0.f || w[2 * h + 1] != 0.f;
    const size_t K12 = (size_t)s.K1 * s.K2;
    const float tz = pick(th[2], jz);
    const size_t plane = pick(gi[2], jz) * K12;
#pragma unroll
    for (int jy = 0; jy < P; ++jy) {
        const float tyz = th[1][jy] * tz;
        const size_t row = plane + (size_t)gi[1][jy] * s.K1;
#pragma unroll
        for (int jx = 0; jx < P; ++jx) {
            const float tt = th[0][jx] * tyz;
            const size_t g = row + gi[0][jx];
#pragma unroll
            for (int h = 0; h < 8; ++h)
                if (any[h]) atomicAdd(&grid[h * gstride + g], make_float2(w[2 * h] * tt, w[2 * h + 1] * tt));
        }
    }
}

// Field gathers of the dipole iterations: D_t = sum_g phi(g) grad_t M, D = J^T D_t and the
// field -sfac D; with FIRST the charges' field from the imaginary part as well.
//   FP64 (T double): efm = (polr2 > 1e-6 ? -sfac D : 0) + dum mu, efc = -sfac D_q
//   FP32 (T float):  e32k = (polr2 > 1e-6 ? -sfac D : 0) + dum d
template <typename T, int P, bool FIRST>
__global__ void __launch_bounds__(kSpThreads) k_spme_field(SpArgs s, const double* __restrict__ x,
                                                           const double* __restrict__ y, const double* __restrict__ z,
                                                           const typename Cx<T>::t* __restrict__ grid,
                                                           const double* __restrict__ polr2, double sfac, double dum,
                                                           const double* __restrict__ mx, const double* __restrict__ my,
                                                           const double* __restrict__ mz, double* __restrict__ efm,
                                                           double* __restrict__ efc, const float4* __restrict__ d32,
                                                           float* __restrict__ e32k) {
    typedef typename Cx<T>::t C;
    if (s.stop && *s.stop) return;
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int j = (int)(t / kLanes), jz = (int)(t % kLanes);
    if (j >= s.n) return;   // whole lane groups leave together
    const bool pol = polr2[j] > 1e-6;
    T D[3] = {0, 0, 0}, Dq[3] = {0, 0, 0};
    // without the charges' field a masked site needs no gather (its field is not used)
    if (jz < P && (FIRST || pol)) {
        int gi[3][P];
        T th[3][P], d1[3][P], d2[3][P];
        if constexpr (sizeof(T) == 4) site_splines32<P, 1>(s, j, gi, th, d1, d2);
        else site_splines_tab<P, 1>(s, j, gi, th, d1, d2);
        const size_t K12 = (size_t)s.K1 * s.K2;
        const C* plane = grid + pick(gi[2], jz) * K12;
        const T tz = pick(th[2], jz), dz = pick(d1[2], jz);
#pragma unroll
        for (int jy = 0; jy < P; ++jy) {
            const C* row = plane + (size_t)gi[1][jy] * s.K1;
            T s0 = 0, s1 = 0, q0 = 0, q1 = 0;
#pragma unroll
            for (int jx = 0; jx < P; ++jx) {
                const C p = row[gi[0][jx]];
                s0 += p.x * th[0][jx];
                s1 += p.x * d1[0][jx];
                if (FIRST) {
                    q0 += p.y * th[0][jx];
                    q1 += p.y * d1[0][jx];
                }
            }
            const T a = th[1][jy] * tz, b = d1[1][jy] * tz, c = th[1][jy] * dz;
            D[0] += a * s1;
            D[1] += b * s0;
            D[2] += c * s0;
            if (FIRST) {
                Dq[0] += a * q1;
                Dq[1] += b * q0;
                Dq[2] += c * q0;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        D[c] = group_sum(D[c]);
        if (FIRST) Dq[c] = group_sum(Dq[c]);
    }
    if (jz != 0) return;
    const int n = s.n;
    for (int c = 0; c < 3; ++c) {
        if (efm) {
            const double Dr = s.jac[c] * (double)D[0] + s.jac[3 + c] * (double)D[1] + s.jac[6 + c] * (double)D[2];
            const double mu = c == 0 ? mx[j] : (c == 1 ? my[j] : mz[j]);
            efm[(size_t)c * n + j] = (pol ? -sfac * Dr : 0.0) + dum * mu;
            if (FIRST)
                efc[(size_t)c * n + j] =
                    -sfac * (s.jac[c] * (double)Dq[0] + s.jac[3 + c] * (double)Dq[1] + s.jac[6 + c] * (double)Dq[2]);
        } else {
            const float4 dd = d32[j];
            const float dc = c == 0 ? dd.x : (c == 1 ? dd.y : dd.z);
            const float Drf = s.jac32[c] * (float)D[0] + s.jac32[3 + c] * (float)D[1] + s.jac32[6 + c] * (float)D[2];
            e32k[(size_t)c * n + j] = (pol ? (float)(-sfac) * Drf : 0.f) + (float)dum * dc;
        }
    }
}

// Final gather at the converged dipoles from the grid phi_tot + i phi_q: per site the
// force / scale = -(q D + W) / 2 with W = J^T sum_g phi_tot grad_t(mu_t . grad_t M), half
// the charges' potential and half the dipoles' (part5, 5 blocks of n); the dipole part of
// the virial sum_j mu_jb D_ja (acc[11..16]: 11 22 33 12 13 23) and the force sums
// (acc[17..19]); the total k-space field -sfac D (field, or null).
template <int P>
__global__ void __launch_bounds__(kSpThreads) k_spme_final_gather(SpArgs s, const double* __restrict__ x,
                                                                  const double* __restrict__ y,
                                                                  const double* __restrict__ z,
                                                                  const double2* __restrict__ grid,
                                                                  const double* __restrict__ q,
                                                                  const double4* __restrict__ md, double sfac,
                                                                  double* __restrict__ part5, double* __restrict__ acc,
                                                                  double* __restrict__ field) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int j = (int)(t / kLanes), jz = (int)(t % kLanes);
    double red[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (j < s.n) {   // whole lane groups in or out: the group sums below see all 8 lanes
        double Pt = 0, Pq = 0, D[3] = {0, 0, 0}, W[3] = {0, 0, 0};
        const double4 m = md[j];
        if (jz < P) {
            int gi[3][P];
            double th[3][P], d1[3][P], d2[3][P];
            site_splines_tab<P, 2>(s, j, gi, th, d1, d2);
            double mt[3];
            to_t<double>(s, m.x, m.y, m.z, mt);
            const size_t K12 = (size_t)s.K1 * s.K2;
            const double2* plane = grid + pick(gi[2], jz) * K12;
            const double tz = pick(th[2], jz), dz = pick(d1[2], jz), ddz = pick(d2[2], jz);
#pragma unroll
            for (int jy = 0; jy < P; ++jy) {
                const double2* row = plane + (size_t)gi[1][jy] * s.K1;
                double s0 = 0, s1 = 0, s2 = 0, q0 = 0;
#pragma unroll
                for (int jx = 0; jx < P; ++jx) {
                    const double2 p = row[gi[0][jx]];
                    s0 += p.x * th[0][jx];
                    s1 += p.x * d1[0][jx];
                    s2 += p.x * d2[0][jx];
                    q0 += p.y * th[0][jx];
                }
                const double ty = th[1][jy], dy = d1[1][jy], ddy = d2[1][jy];
                const double a = ty * tz, b = dy * tz, c = ty * dz;
                Pt += a * s0;
                Pq += a * q0;
                D[0] += a * s1;
                D[1] += b * s0;
                D[2] += c * s0;
                // gradient (t space) of w = mt . grad_t M over the row
                const double e = ddy * tz, f = dy * dz, h = ty * ddz;
                W[0] += mt[0] * a * s2 + (mt[1] * b + mt[2] * c) * s1;
                W[1] += mt[0] * b * s1 + (mt[1] * e + mt[2] * f) * s0;
                W[2] += mt[0] * c * s1 + (mt[1] * f + mt[2] * h) * s0;
            }
        }
        Pt = group_sum(Pt);
        Pq = group_sum(Pq);
        for (int c = 0; c < 3; ++c) {
            D[c] = group_sum(D[c]);
            W[c] = group_sum(W[c]);
        }
        if (jz == 0) {
            const double qj = q[j];
            double Dr[3], Wr[3];
            for (int c = 0; c < 3; ++c) {
                Dr[c] = s.jac[c] * D[0] + s.jac[3 + c] * D[1] + s.jac[6 + c] * D[2];
                Wr[c] = s.jac[c] * W[0] + s.jac[3 + c] * W[1] + s.jac[6 + c] * W[2];
            }
            const int n = s.n;
            for (int c = 0; c < 3; ++c) {
                const double v = -0.5 * (qj * Dr[c] + Wr[c]);
                part5[(size_t)c * n + j] = v;
                red[6 + c] = v;
                if (field) field[(size_t)c * n + j] = -sfac * Dr[c];
            }
            part5[3 * (size_t)n + j] = 0.5 * Pq;
            part5[4 * (size_t)n + j] = 0.5 * (Pt - Pq);
            const double mu[3] = {m.x, m.y, m.z};
            red[0] = mu[0] * Dr[0];
            red[1] = mu[1] * Dr[1];
            red[2] = mu[2] * Dr[2];
            red[3] = mu[1] * Dr[0];
            red[4] = mu[2] * Dr[0];
            red[5] = mu[2] * Dr[1];
        }
    }
    block_sum_atomic<9>(red, acc + 11);
}

// The SPME drift: the mean k-space force over the sites is removed (SOURCE/spme_for.f:86-112).
__global__ void k_spme_drift(int n, const double* __restrict__ acc, double* __restrict__ part5) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    for (int c = 0; c < 3; ++c) part5[(size_t)c * n + j] -= acc[17 + c] / (double)n;
}

__device__ __forceinline__ int mfreq(int i, int K) { return i < K / 2 ? i : i - K; }

// Per grid point m (the full grid, each term halved: the Ewald sums' half-space form):
// engc = G |F_q|^2, engdum = G |F_tot|^2, the k k part of omg and, with HEAT, the ew1p heat
// term from the structure factors of grids 1..8 (mu, q v, mu v).  F(m) of a density packed
// as the real or imaginary part of grid Z is (Z(m) + conj Z(-m)) / 2 or
// (Z(m) - conj Z(-m)) / 2i.  Block partial sums go to part[block * 11 + q].
template <int HEAT, typename HC>
__global__ void __launch_bounds__(kKtThreads) k_spme_kterms(SpArgs s, const double2* __restrict__ grid,
                                                            const HC* __restrict__ hgrid, size_t hstride,
                                                            const double* __restrict__ G, double ralph, double sfac,
                                                            double* __restrict__ part) {
    double acc[11];
#pragma unroll
    for (int q = 0; q < 11; ++q) acc[q] = 0.0;
    const size_t ng = (size_t)s.K1 * s.K2 * s.K3;
    const double twopi = 2.0 * kPiS;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ng; i += (size_t)gridDim.x * blockDim.x) {
        const double gm = G[i];
        if (gm == 0.0) continue;
        const int ix = (int)(i % s.K1), iy = (int)((i / s.K1) % s.K2), iz = (int)(i / ((size_t)s.K1 * s.K2));
        const int m1 = mfreq(ix, s.K1), m2 = mfreq(iy, s.K2), m3 = mfreq(iz, s.K3);
        const size_t jm = (size_t)((s.K3 - iz) % s.K3) * s.K1 * s.K2 + (size_t)((s.K2 - iy) % s.K2) * s.K1 +
                          (size_t)((s.K1 - ix) % s.K1);
        const double kx[3] = {twopi * (m1 * s.rc[0] + m2 * s.rc[1] + m3 * s.rc[2]),
                              twopi * (m1 * s.rc[3] + m2 * s.rc[4] + m3 * s.rc[5]),
                              twopi * (m1 * s.rc[6] + m2 * s.rc[7] + m3 * s.rc[8])};
        const double rksq = kx[0] * kx[0] + kx[1] * kx[1] + kx[2] * kx[2];
        const double akv2 = 2.0 * (1.0 / rksq - ralph);
        const double2 z0 = grid[i], z0m = grid[jm];
        // total density (real part) and charges (imaginary part)
        const double s1 = 0.5 * (z0.x + z0m.x), s2 = 0.5 * (z0.y - z0m.y);
        const double cq = 0.5 * (z0.y + z0m.y), sq = -0.5 * (z0.x - z0m.x);
        const double s12 = s1 * s1 + s2 * s2;
        acc[0] += 0.5 * gm * (cq * cq + sq * sq);
        acc[1] += 0.5 * gm * s12;
        const int oa[6] = {0, 1, 2, 0, 0, 1}, ob[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
        for (int q = 0; q < 6; ++q) acc[2 + q] -= 0.5 * gm * akv2 * s12 * kx[oa[q]] * kx[ob[q]];
        if (HEAT) {
            double re[16], im[16];
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                const HC a = hgrid[h * hstride + i], b = hgrid[h * hstride + jm];
                re[2 * h] = 0.5 * (a.x + b.x);
                im[2 * h] = 0.5 * (a.y - b.y);
                re[2 * h + 1] = 0.5 * (a.y + b.y);
                im[2 * h + 1] = -0.5 * (a.x - b.x);
            }
            double out[3];
            ew1p_heat_kterm(kx, s1, s2, re, im, re + 3, im + 3, re + 6, im + 6, sfac * gm, akv2, out);
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[8 + c] += 0.5 * out[c];
        }
    }
    __shared__ double red[kKtThreads / 32][11];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 11; ++q) {
        const double v = warp_sum(acc[q]);
        if (lane == 0) red[w][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < 11) {
        double v = 0.0;
        for (int i = 0; i < kKtThreads / 32; ++i) v += red[i][threadIdx.x];
        part[(size_t)blockIdx.x * 11 + threadIdx.x] = v;
    }
}

// One block: acc[48 + q] = sum over blocks of part (in block order); the dipole part of
// the virial (acc[11..16]) is added to omg.
__global__ void k_spme_kreduce(int nblk, const double* __restrict__ part, double* __restrict__ acc) {
    __shared__ double red[32][11];
    double v[11];
    for (int q = 0; q < 11; ++q) v[q] = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        for (int q = 0; q < 11; ++q) v[q] += part[(size_t)b * 11 + q];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < 11; ++q) {
        const double t = warp_sum(v[q]);
        if (lane == 0) red[w][q] = t;
    }
    __syncthreads();
    if (threadIdx.x < 11) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x / 32); ++i) t += red[i][threadIdx.x];
        if (threadIdx.x >= 2 && threadIdx.x < 8) t += acc[11 + threadIdx.x - 2];
        acc[48 + threadIdx.x] = t;
    }
}

// Influence function: G(m) = |b1 b2 b3|^2 exp(-k^2 / (4 alpha^2)) / k^2 inside the
// reference's sphere (1e-6 < k^2 <= rcpct2), 0 elsewhere and at the Nyquist frequencies.
__global__ void k_spme_influence(SpArgs s, const double* __restrict__ bsq, double ralph, double rcpct2,
                                 double* __restrict__ G, float* __restrict__ G32) {
    const size_t ng = (size_t)s.K1 * s.K2 * s.K3;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= ng) return;
    const int ix = (int)(i % s.K1), iy = (int)((i / s.K1) % s.K2), iz = (int)(i / ((size_t)s.K1 * s.K2));
    double g = 0.0;
    const bool nyq = (s.K1 % 2 == 0 && ix == s.K1 / 2) || (s.K2 % 2 == 0 && iy == s.K2 / 2) ||
                     (s.K3 % 2 == 0 && iz == s.K3 / 2);
    if (!nyq) {
        const int m1 = mfreq(ix, s.K1), m2 = mfreq(iy, s.K2), m3 = mfreq(iz, s.K3);
        const double twopi = 2.0 * kPiS;
        const double kx = twopi * (m1 * s.rc[0] + m2 * s.rc[1] + m3 * s.rc[2]);
        const double ky = twopi * (m1 * s.rc[3] + m2 * s.rc[4] + m3 * s.rc[5]);
        const double kz = twopi * (m1 * s.rc[6] + m2 * s.rc[7] + m3 * s.rc[8]);
        const double rksq = kx * kx + ky * ky + kz * kz;
        if (rksq > 1e-6 && rksq <= rcpct2)
            g = bsq[ix] * bsq[s.K1 + iy] * bsq[s.K1 + s.K2 + iz] * exp(ralph * rksq) / rksq;
    }
    G[i] = g;
    if (G32) G32[i] = (float)g;
}

inline unsigned nblocks(long n, int t) { return (unsigned)((n + t - 1) / t); }

// Radices of n (4 first, then 2, 3, 5); false when n has another prime factor.
bool factor(int n, FftAxis& a) {
    a.n = n;
    a.nst = 0;
    int m = n;
    while (m % 4 == 0 && a.nst < 16) {
        a.r[a.nst++] = 4;
        m /= 4;
    }
    const int pr[3] = {2, 3, 5};
    for (int p : pr)
        while (m % p == 0 && a.nst < 16) {
            a.r[a.nst++] = p;
            m /= p;
        }
    return m == 1;
}

// The x and y axes of the 3D FFT in one pass: one block per z plane (blockIdx.x) of grid
// blockIdx.y.  The plane is loaded once (coalesced), transformed along x ([x][y] layout,
// pitch K2 + 1), transposed in shared memory and transformed along y ([y][x], pitch K1 + 1),
// then stored once: two passes over the grid and two launches fewer than one pass per axis.
// sg +1 forward, -1 backward.
template <typename T>
__global__ void __launch_bounds__(kFftPlaneThreads) k_fft_plane(typename Cx<T>::t* data, size_t gstride, FftAxis ax,
                                                                FftAxis ay, int sg, const typename Cx<T>::t* tw,
                                                                const int* __restrict__ stop) {
    typedef typename Cx<T>::t C;
    if (stop && *stop) return;   // the CG solve that queued this pass has stopped
    extern __shared__ __align__(16) unsigned char fft_smem[];
    const int K1 = ax.n, K2 = ay.n, P1 = K2 + 1, P2 = K1 + 1;
    const int words = max(K1 * P1, K2 * P2);
    C* s0 = reinterpret_cast<C*>(fft_smem);
    C* s1 = s0 + words;
    C* twx = s1 + words;
    C* twy = twx + K1;
    C* g = data + (size_t)blockIdx.y * gstride + (size_t)blockIdx.x * K1 * K2;
    for (int i = threadIdx.x; i < K1; i += blockDim.x) twx[i] = tw[ax.tw_off + i];
    for (int i = threadIdx.x; i < K2; i += blockDim.x) twy[i] = tw[ay.tw_off + i];
    const IDiv dk(K1);
    const int nxy = K1 * K2, bs = blockDim.x;
    // the plane's loads issued U at a time per thread (all in flight before the first store)
    constexpr int U = 4;
    for (int i0 = threadIdx.x; i0 < nxy; i0 += U * bs) {
        C v[U];
#pragma unroll
        for (int q = 0; q < U; ++q)
            if (i0 + q * bs < nxy) v[q] = g[i0 + q * bs];
#pragma unroll
        for (int q = 0; q < U; ++q) {
            const int i = i0 + q * bs;
            if (i < nxy) s0[dk.mod(i) * P1 + dk.div(i)] = v[q];
        }
    }
    __syncthreads();
    C* r = fft_lines<T>(s0, s1, ax, P1, K2, twx, sg);
    C* t = r == s0 ? s1 : s0;
    for (int i = threadIdx.x; i < nxy; i += bs) {
        const int x = dk.mod(i), y = dk.div(i);
        t[y * P2 + x] = r[x * P1 + y];
    }
    __syncthreads();
    C* u = fft_lines<T>(t, r, ay, P2, K1, twy, sg);
    for (int i = threadIdx.x; i < nxy; i += bs) g[i] = u[dk.div(i) * P2 + dk.mod(i)];
}

// Shared memory of the plane pass: two buffers and the x and y twiddles.
inline size_t plane_smem_bytes(int K1, int K2, size_t csize) {
    return (2 * (size_t)std::max(K1 * (K2 + 1), K2 * (K1 + 1)) + K1 + K2) * csize;
}

// Lines per FFT block: about 1024 complex values per block.
inline int lines_per_block(int n) { return std::max(2, std::min(16, 1024 / n)); }

inline size_t fft_smem_bytes(int n, int nl, size_t csize) { return (2 * (size_t)n * (nl + 1) + n) * csize; }

cudaError_t allow_fft_smem() {
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(dev)) return cudaSuccess;
    const void* f[] = {(const void*)k_fft_axis<double, 0>, (const void*)k_fft_axis<double, 1>,
                       (const void*)k_fft_axis<double, 2>, (const void*)k_fft_axis<double, 3>,
                       (const void*)k_fft_axis<float, 0>,  (const void*)k_fft_axis<float, 1>,
                       (const void*)k_fft_axis<float, 2>,  (const void*)k_fft_axis<float, 3>,
                       (const void*)k_fft_plane<double>,   (const void*)k_fft_plane<float>};
    for (const void* q : f)
        if ((e = cudaFuncSetAttribute(q, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxFftSmem))) return e;
    done.insert(dev);
    return cudaSuccess;
}

// One axis pass over `count` grids.
template <typename T>
cudaError_t fft_pass(int mode, typename Cx<T>::t* data, size_t gstride, int count, int axis, const FftAxis& ax,
                     const int* K, const typename Cx<T>::t* tw, const T* G, cudaStream_t s,
                     const int* stop = nullptr) {
    const int n = ax.n;
    const int nl = lines_per_block(n);
    const GridDims d{K[0], K[1], K[2]};
    int ntile = 1;
    unsigned nb;
    if (axis == 0) {
        nb = nblocks((long)K[1] * K[2], nl);
    } else {
        ntile = (K[0] + nl - 1) / nl;
        nb = (unsigned)ntile * (axis == 1 ? K[2] : K[1]);
    }
    const size_t sm = fft_smem_bytes(n, nl, sizeof(typename Cx<T>::t));
    if (sm > (size_t)kMaxFftSmem) return cudaErrorInvalidValue;
    const dim3 g(nb, count);
    switch (mode) {
        case 0: k_fft_axis<T, 0><<<g, kFftThreads, sm, s>>>(data, gstride, axis, ax, d, nl, ntile, tw, G, stop); break;
        case 1: k_fft_axis<T, 1><<<g, kFftThreads, sm, s>>>(data, gstride, axis, ax, d, nl, ntile, tw, G, stop); break;
        case 2: k_fft_axis<T, 2><<<g, kFftThreads, sm, s>>>(data, gstride, axis, ax, d, nl, ntile, tw, G, stop); break;
        default: k_fft_axis<T, 3><<<g, kFftThreads, sm, s>>>(data, gstride, axis, ax, d, nl, ntile, tw, G, stop); break;
    }
    return cudaGetLastError();
}

// The convolution phi = F^-1[G F[Q]] of one grid: forward x, forward y, (forward z, G,
// backward z), backward y, backward x.
template <typename T>
cudaError_t convolve(typename Cx<T>::t* data, const FftAxis* ax, const int* K, const typename Cx<T>::t* tw, const T* G,
                     cudaStream_t s, long& launches, const int* stop = nullptr) {
    cudaError_t e;
    typedef typename Cx<T>::t C;
    const size_t psm = plane_smem_bytes(K[0], K[1], sizeof(C));
    // FP32: x and y in one pass per plane (64 x 64: 14 us against 2 x 8.8 us).  FP64 keeps the
    // axis passes: its plane pass (one 135 KB block per plane, 64 of the 152 SMs) is FP64-pipe
    // bound and took 62 us against 2 x 16 us (with 256 and again with 1024 threads).
    if (sizeof(T) == 4 && psm <= (size_t)kMaxFftSmem) {
        k_fft_plane<T><<<dim3(K[2], 1), kFftPlaneThreads, psm, s>>>(data, 0, ax[0], ax[1], 1, tw, stop);
        if ((e = cudaGetLastError())) return e;
        if ((e = fft_pass<T>(2, data, 0, 1, 2, ax[2], K, tw, G, s, stop))) return e;
        k_fft_plane<T><<<dim3(K[2], 1), kFftPlaneThreads, psm, s>>>(data, 0, ax[0], ax[1], -1, tw, stop);
        launches += 3;
        return cudaGetLastError();
    }
    if ((e = fft_pass<T>(0, data, 0, 1, 0, ax[0], K, tw, G, s, stop))) return e;
    if ((e = fft_pass<T>(0, data, 0, 1, 1, ax[1], K, tw, G, s, stop))) return e;
    if ((e = fft_pass<T>(2, data, 0, 1, 2, ax[2], K, tw, G, s, stop))) return e;
    if ((e = fft_pass<T>(1, data, 0, 1, 1, ax[1], K, tw, G, s, stop))) return e;
    if ((e = fft_pass<T>(1, data, 0, 1, 0, ax[0], K, tw, G, s, stop))) return e;
    launches += 5;
    return cudaSuccess;
}

SpArgs sp_args(const SpmeState& st, int n) {
    SpArgs a;
    a.n = n;
    a.K1 = st.K[0];
    a.K2 = st.K[1];
    a.K3 = st.K[2];
    a.stop = nullptr;
    a.sib = st.sib;
    a.sw = st.sw;
    a.spl = st.spl;
    for (int i = 0; i < 9; ++i) {
        a.rc[i] = st.rc[i];
        a.jac[i] = st.jac[i];
        a.jac32[i] = (float)st.jac[i];
    }
    return a;
}

#define SPME_ORDER_SWITCH(p, CALL) \
    switch (p) {                   \
        case 4: { constexpr int P_ = 4; CALL; } break; \
        case 5: { constexpr int P_ = 5; CALL; } break; \
        case 6: { constexpr int P_ = 6; CALL; } break; \
        case 7: { constexpr int P_ = 7; CALL; } break; \
        case 8: { constexpr int P_ = 8; CALL; } break; \
        default: return cudaErrorInvalidValue;          \
    }

}  // namespace

int spme_smooth_even(double x) {
    int k = std::max(2, (int)std::ceil(x - 1e-9));
    for (;; ++k) {
        if (k % 2) continue;
        int m = k;
        for (int p : {2, 3, 5})
            while (m % p == 0) m /= p;
        if (m == 1) return k;
    }
}

SpmeState::~SpmeState() { release(); }

void SpmeState::release() {
    void* p[] = {G, G32, tw, tw32, grid, grid32, hgrid32, part, sib, sw, spl};
    for (void* q : p)
        if (q) cudaFree(q);
    hgrid32 = nullptr;
    hgrid_cap_ng = 0;
    sib = nullptr;
    sw = nullptr;
    spl = nullptr;
    site_cap = 0;
    G = nullptr;
    G32 = nullptr;
    tw = nullptr;
    tw32 = nullptr;
    grid = nullptr;
    grid32 = nullptr;
    part = nullptr;
    g_cap = part_cap = grid_cap_ng = 0;
    tw_cap = ngrid_cap = grid32_cap_ng = 0;
    order = 0;
    have32 = false;
}

cudaError_t SpmeState::prepare(const double* cell, double alpha_, int order_, const int* Kin, bool fp32, int ngrids,
                               cudaStream_t s) {
    cudaError_t e;
    if (order_ < 4 || order_ > 8) return cudaErrorInvalidValue;
    for (int a = 0; a < 3; ++a)
        if (Kin[a] < order_ || Kin[a] > kMaxGrid) return cudaErrorInvalidValue;
    if ((e = allow_fft_smem())) return e;
    bool same = order == order_ && alpha == alpha_ && K[0] == Kin[0] && K[1] == Kin[1] && K[2] == Kin[2] && G &&
                (!fp32 || have32);
    for (int i = 0; i < 9 && same; ++i) same = cellc[i] == cell[i];
    const size_t ngn = (size_t)Kin[0] * Kin[1] * Kin[2];
    // grids
    if ((size_t)ngrids > (size_t)ngrid_cap || ngn > grid_cap_ng) {
        const size_t ngr = std::max((size_t)ngrids, (size_t)ngrid_cap);
        if (grid) cudaFree(grid);
        grid = nullptr;
        ngrid_cap = 0;
        grid_cap_ng = 0;
        if ((e = cudaMalloc(&grid, ngr * ngn * sizeof(double2)))) return e;
        ngrid_cap = (int)ngr;
        grid_cap_ng = ngn;
    }
    if (fp32 && ngn > (size_t)grid32_cap_ng) {
        if (grid32) cudaFree(grid32);
        grid32 = nullptr;
        grid32_cap_ng = 0;
        if ((e = cudaMalloc(&grid32, ngn * sizeof(float2)))) return e;
        grid32_cap_ng = (int)ngn;
    }
    if (fp32 && ngrids > 1 && ngn > hgrid_cap_ng) {   // the mixed final pass's 8 FP32 heat grids
        if (hgrid32) cudaFree(hgrid32);
        hgrid32 = nullptr;
        hgrid_cap_ng = 0;
        if ((e = cudaMalloc(&hgrid32, 8 * ngn * sizeof(float2)))) return e;
        hgrid_cap_ng = ngn;
    }
    if (same) return cudaSuccess;
    // tables for this cell, alpha, order and grid
    order = 0;
    have32 = false;
    for (int a = 0; a < 3; ++a) {
        K[a] = Kin[a];
        if (!factor(K[a], ax[a])) return cudaErrorInvalidValue;
    }
    ax[0].tw_off = 0;
    ax[1].tw_off = K[0];
    ax[2].tw_off = K[0] + K[1];
    ng = ngn;
    alpha = alpha_;
    for (int i = 0; i < 9; ++i) cellc[i] = cell[i];
    // reciprocal cell (the inverse of the DL_POLY cell matrix, as the Ewald k vectors use it)
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
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) jac[3 * a + c] = K[a] * rc[a + 3 * c];
    // widths of the reciprocal cell (dcell's celprp(7..9) of rcell) and the k cut
    double wr[3];
    {
        const double* aa = rc;
        const double axb1 = aa[1] * aa[5] - aa[2] * aa[4], axb2 = aa[2] * aa[3] - aa[0] * aa[5],
                     axb3 = aa[0] * aa[4] - aa[1] * aa[3];
        const double bxc1 = aa[4] * aa[8] - aa[5] * aa[7], bxc2 = aa[5] * aa[6] - aa[3] * aa[8],
                     bxc3 = aa[3] * aa[7] - aa[4] * aa[6];
        const double cxa1 = aa[7] * aa[2] - aa[1] * aa[8], cxa2 = aa[0] * aa[8] - aa[2] * aa[6],
                     cxa3 = aa[1] * aa[6] - aa[0] * aa[7];
        const double v = std::fabs(aa[0] * bxc1 + aa[1] * bxc2 + aa[2] * bxc3);
        wr[0] = v / std::sqrt(bxc1 * bxc1 + bxc2 * bxc2 + bxc3 * bxc3);
        wr[1] = v / std::sqrt(cxa1 * cxa1 + cxa2 * cxa2 + cxa3 * cxa3);
        wr[2] = v / std::sqrt(axb1 * axb1 + axb2 * axb2 + axb3 * axb3);
    }
    const double twopi = 2.0 * kPiS;
    double rcpcut = 0.5 * std::min(std::min(K[0] * wr[0], K[1] * wr[1]), K[2] * wr[2]);
    rcpcut = rcpcut * 1.05 * twopi;
    const double rcpct2 = rcpcut * rcpcut;
    // |b(m)|^2 per axis (bspcoe): 1 / |sum_{k=0}^{p-2} M_p(k + 1) exp(2 pi i m k / K)|^2
    std::vector<double> csp(order_ + 1, 0.0);   // csp[j] = M_p(j), j = 0..p
    {
        std::vector<double> a(order_ + 1, 0.0);
        a[1] = 1.0;   // M_2 at the knots 0, 1, 2: 0, 1, 0
        for (int k = 3; k <= order_; ++k)
            for (int j = k; j >= 1; --j) a[j] = (double(j) * a[j] + double(k - j) * a[j - 1]) / double(k - 1);
        csp = a;
    }
    const int Ktot = K[0] + K[1] + K[2];
    std::vector<double> bsq(Ktot, 0.0);
    {
        int off = 0;
        for (int a = 0; a < 3; ++a) {
            for (int i = 0; i < K[a]; ++i) {
                double re = 0.0, im = 0.0;
                for (int k = 0; k <= order_ - 2; ++k) {
                    const long long mk = ((long long)i * k) % K[a];
                    const double ang = twopi * double(mk) / double(K[a]);
                    re += csp[k + 1] * std::cos(ang);
                    im += csp[k + 1] * std::sin(ang);
                }
                const double d2 = re * re + im * im;
                bsq[off + i] = d2 > 1e-30 ? 1.0 / d2 : 0.0;
            }
            off += K[a];
        }
    }
    std::vector<double2> htw(Ktot);
    std::vector<float2> htw32(Ktot);
    {
        int off = 0;
        for (int a = 0; a < 3; ++a) {
            for (int i = 0; i < K[a]; ++i) {
                const long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)i / K[a];
                const double c = (double)std::cos(ang), sn = (double)std::sin(ang);
                htw[off + i] = make_double2(c, sn);
                htw32[off + i] = make_float2((float)c, (float)sn);
            }
            off += K[a];
        }
    }
    if (ngn > g_cap || (fp32 && !G32)) {
        if (G) cudaFree(G);
        if (G32) cudaFree(G32);
        G = nullptr;
        G32 = nullptr;
        g_cap = 0;
        if ((e = cudaMalloc(&G, ngn * sizeof(double)))) return e;
        if ((e = cudaMalloc(&G32, ngn * sizeof(float)))) return e;
        g_cap = ngn;
    }
    if (Ktot > tw_cap) {
        if (tw) cudaFree(tw);
        if (tw32) cudaFree(tw32);
        tw = nullptr;
        tw32 = nullptr;
        tw_cap = 0;
        if ((e = cudaMalloc(&tw, Ktot * sizeof(double2)))) return e;
        if ((e = cudaMalloc(&tw32, Ktot * sizeof(float2)))) return e;
        tw_cap = Ktot;
    }
    if (!part) {
        if ((e = cudaMalloc(&part, (size_t)kKtBlocks * 11 * sizeof(double)))) return e;
        part_cap = (size_t)kKtBlocks * 11;
    }
    double* dbsq = nullptr;
    if ((e = cudaMalloc(&dbsq, Ktot * sizeof(double)))) return e;
    e = cudaMemcpyAsync(dbsq, bsq.data(), Ktot * sizeof(double), cudaMemcpyHostToDevice, s);
    if (!e) e = cudaMemcpyAsync(tw, htw.data(), Ktot * sizeof(double2), cudaMemcpyHostToDevice, s);
    if (!e) e = cudaMemcpyAsync(tw32, htw32.data(), Ktot * sizeof(float2), cudaMemcpyHostToDevice, s);
    if (!e) {
        const SpArgs sa = sp_args(*this, 0);
        k_spme_influence<<<nblocks((long)ngn, 256), 256, 0, s>>>(sa, dbsq, -0.25 / (alpha_ * alpha_), rcpct2, G, G32);
        e = cudaGetLastError();
    }
    // the host vectors and the moduli buffer must outlive the copies and the kernel
    const cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(dbsq);
    if (e) return e;
    if (e2) return e2;
    order = order_;
    have32 = true;
    return cudaSuccess;
}

cudaError_t SpmeState::field64(int n, const double* x, const double* y, const double* z, const double* q,
                               const double4* md, const double* polr2, const double* mx, const double* my,
                               const double* mz, double sfac, double dum, double* efm, double* efc, cudaStream_t s) {
    cudaError_t e;
    launches = 0;
    if ((e = cudaMemsetAsync(grid, 0, ng * sizeof(double2), s))) return e;
    const SpArgs sa = sp_args(*this, n);
    const unsigned nb = nblocks((long)kLanes * n, kSpThreads);
    if (n > 0) {
        if (q) {
            SPME_ORDER_SWITCH(order, (k_spme_spread<double, P_, 1, double4><<<nb, kSpThreads, 0, s>>>(
                                         sa, x, y, z, q, md, polr2, grid)));
        } else {
            SPME_ORDER_SWITCH(order, (k_spme_spread<double, P_, 0, double4><<<nb, kSpThreads, 0, s>>>(
                                         sa, x, y, z, q, md, polr2, grid)));
        }
    }
    if ((e = cudaGetLastError())) return e;
    if ((e = convolve<double>(grid, ax, K, tw, G, s, launches))) return e;
    if (n > 0) {
        if (q) {
            SPME_ORDER_SWITCH(order, (k_spme_field<double, P_, true><<<nb, kSpThreads, 0, s>>>(
                                         sa, x, y, z, grid, polr2, sfac, dum, mx, my, mz, efm, efc, nullptr, nullptr)));
        } else {
            SPME_ORDER_SWITCH(order, (k_spme_field<double, P_, false><<<nb, kSpThreads, 0, s>>>(
                                         sa, x, y, z, grid, polr2, sfac, dum, mx, my, mz, efm, efc, nullptr, nullptr)));
        }
    }
    launches += 3;
    return cudaGetLastError();
}

cudaError_t SpmeState::frame(int n, const double* x, const double* y, const double* z, cudaStream_t s) {
    cudaError_t e;
    if (!order) return cudaErrorInvalidValue;
    if (n > site_cap) {
        if (sib) cudaFree(sib);
        if (sw) cudaFree(sw);
        if (spl) cudaFree(spl);
        sib = nullptr;
        sw = nullptr;
        spl = nullptr;
        site_cap = 0;
        if ((e = cudaMalloc(&sib, (size_t)n * sizeof(int4)))) return e;
        if ((e = cudaMalloc(&sw, (size_t)n * sizeof(float4)))) return e;
        if ((e = cudaMalloc(&spl, (size_t)n * kSplSite * sizeof(double)))) return e;
        site_cap = n;
    }
    if (n > 0) {
        const SpArgs sa = sp_args(*this, n);
        SPME_ORDER_SWITCH(order, (k_spme_frame<P_><<<nblocks(3L * n, 256), 256, 0, s>>>(sa, x, y, z, sib, sw, spl)));
    }
    return cudaGetLastError();
}

cudaError_t SpmeState::field32(int n, const double* x, const double* y, const double* z, const float4* d,
                               const double* polr2, double sfac, double dum, float* e32k, cudaStream_t s,
                               const int* stop) {
    cudaError_t e;
    launches = 0;
    if (!have32) return cudaErrorInvalidValue;
    if ((e = cudaMemsetAsync(grid32, 0, ng * sizeof(float2), s))) return e;
    SpArgs sa = sp_args(*this, n);
    sa.stop = stop;
    const unsigned nb = nblocks((long)kLanes * n, kSpThreads);
    if (n > 0)
        SPME_ORDER_SWITCH(order, (k_spme_spread<float, P_, 0, float4><<<nb, kSpThreads, 0, s>>>(
                                     sa, x, y, z, nullptr, d, polr2, grid32)));
    if ((e = cudaGetLastError())) return e;
    if ((e = convolve<float>(grid32, ax, K, tw32, G32, s, launches, stop))) return e;
    if (n > 0)
        SPME_ORDER_SWITCH(order, (k_spme_field<float, P_, false><<<nb, kSpThreads, 0, s>>>(
                                     sa, x, y, z, grid32, polr2, sfac, dum, nullptr, nullptr, nullptr, nullptr,
                                     nullptr, d, e32k)));
    launches += 3;
    return cudaGetLastError();
}

cudaError_t SpmeState::final(int n, const double* x, const double* y, const double* z, const double* q,
                             const double4* md, const double* vh, double sfac, double* part5, double* acc,
                             double* field, cudaStream_t s, bool heat32) {
    cudaError_t e;
    launches = 0;
    const bool heat = vh != nullptr;
    heat32 = heat && heat32 && hgrid32;
    const int ngr = heat && !heat32 ? 9 : 1;   // FP64 grids: the densities, and the heat ones in FP64
    if (ngr > ngrid_cap || !order) return cudaErrorInvalidValue;
    const size_t gs = grid_cap_ng;
    if ((e = cudaMemsetAsync(grid, 0, (size_t)ngr * gs * sizeof(double2), s))) return e;
    if (heat32 && (e = cudaMemsetAsync(hgrid32, 0, 8 * ng * sizeof(float2), s))) return e;
    if ((e = cudaMemsetAsync(acc + 11, 0, 9 * sizeof(double), s))) return e;
    const SpArgs sa = sp_args(*this, n);
    const unsigned nb = nblocks((long)kLanes * n, kSpThreads);
    if (n > 0) {
        SPME_ORDER_SWITCH(order, (k_spme_spread<double, P_, 2, double4><<<nb, kSpThreads, 0, s>>>(
                                     sa, x, y, z, q, md, nullptr, grid)));
        if (heat32) {
            SPME_ORDER_SWITCH(order, (k_spme_spread_heat32<P_><<<nb, kSpThreads, 0, s>>>(sa, md, vh, hgrid32, ng)));
        } else if (heat) {
            SPME_ORDER_SWITCH(order, (k_spme_spread_heat<P_><<<nb, kSpThreads, 0, s>>>(sa, x, y, z, md, vh, grid + gs,
                                                                                      gs)));
        }
    }
    if ((e = cudaGetLastError())) return e;
    for (int a = 0; a < 3; ++a)
        if ((e = fft_pass<double>(0, grid, gs, ngr, a, ax[a], K, tw, G, s))) return e;
    if (heat32) {   // the 8 FP32 heat grids forward: plane passes (x, y) and the z pass
        const size_t psm = plane_smem_bytes(K[0], K[1], sizeof(float2));
        if (psm <= (size_t)kMaxFftSmem) {
            k_fft_plane<float><<<dim3(K[2], 8), kFftPlaneThreads, psm, s>>>(hgrid32, ng, ax[0], ax[1], 1, tw32,
                                                                           nullptr);
            if ((e = cudaGetLastError())) return e;
        } else {
            for (int a = 0; a < 2; ++a)
                if ((e = fft_pass<float>(0, hgrid32, ng, 8, a, ax[a], K, tw32, G32, s))) return e;
        }
        if ((e = fft_pass<float>(0, hgrid32, ng, 8, 2, ax[2], K, tw32, G32, s))) return e;
        launches += 2;
    }
    const int nblk = (int)std::min<long>(nblocks((long)ng, kKtThreads), kKtBlocks);
    const double ralph = -0.25 / (alpha * alpha);
    if (heat32)
        k_spme_kterms<1, float2><<<nblk, kKtThreads, 0, s>>>(sa, grid, hgrid32, ng, G, ralph, sfac, part);
    else if (heat)
        k_spme_kterms<1, double2><<<nblk, kKtThreads, 0, s>>>(sa, grid, grid + gs, gs, G, ralph, sfac, part);
    else
        k_spme_kterms<0, double2><<<nblk, kKtThreads, 0, s>>>(sa, grid, grid, gs, G, ralph, sfac, part);
    if ((e = fft_pass<double>(3, grid, 0, 1, 2, ax[2], K, tw, G, s))) return e;
    if ((e = fft_pass<double>(1, grid, 0, 1, 1, ax[1], K, tw, G, s))) return e;
    if ((e = fft_pass<double>(1, grid, 0, 1, 0, ax[0], K, tw, G, s))) return e;
    if (n > 0) {
        SPME_ORDER_SWITCH(order, (k_spme_final_gather<P_><<<nb, kSpThreads, 0, s>>>(sa, x, y, z, grid, q, md, sfac,
                                                                                   part5, acc, field)));
        k_spme_drift<<<nblocks(n, kSpThreads), kSpThreads, 0, s>>>(n, acc, part5);
    }
    k_spme_kreduce<<<1, 1024, 0, s>>>(nblk, part, acc);
    launches += (heat ? 2 : 1) + 3 + 1 + 3 + (n > 0 ? 2 : 0) + 1;
    return cudaGetLastError();
}

cudaError_t SpmeState::fft64(double2* data, int count, int sign, cudaStream_t s) {
    cudaError_t e;
    if (!order) return cudaErrorInvalidValue;
    const size_t gs = ng;
    const size_t psm = plane_smem_bytes(K[0], K[1], sizeof(double2));
    if (psm <= (size_t)kMaxFftSmem) {   // the FP32 convolutions' form: x and y in one plane pass
        k_fft_plane<double><<<dim3(K[2], count), kFftPlaneThreads, psm, s>>>(data, gs, ax[0], ax[1], sign > 0 ? 1 : -1,
                                                                            tw, nullptr);
        if ((e = cudaGetLastError())) return e;
        return fft_pass<double>(sign > 0 ? 0 : 1, data, gs, count, 2, ax[2], K, tw, G, s);
    }
    for (int a = 0; a < 3; ++a)
        if ((e = fft_pass<double>(sign > 0 ? 0 : 1, data, gs, count, a, ax[a], K, tw, G, s))) return e;
    return cudaSuccess;
}

}  // namespace mbx
