// Path-integral bead coupling on the device: the normal-mode transformation of the
// reference's PIMD/CMD mode (transformation_matrix and the cart <-> normal-mode transforms,
// SOURCE/centroid_matrix.f:3-270) and its ring-polymer spring forces
// (SOURCE/centroid_spring_force.f:1-157), with the beads as a leading array axis on one GPU
// instead of MPI ring ranks.  P beads of n atoms are stored bead after bead: value j of bead
// b at b * n + j in every per-atom array (the layout of mbx_water_step_multi's boxes).
#include "../../include/mbx.h"
#include "mbx_kernels.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace mbx {

namespace {

constexpr int kPimdThreads = 128;
constexpr int kMaxBeads = 256;

// out[p * m + j] = sum_b A[p * P + b] in[b * m + j]: the P x P matrix in shared memory,
// one value index j per thread.
__global__ void __launch_bounds__(kPimdThreads) k_pimd_transform(int P, long m, const double* __restrict__ A,
                                                                 const double* __restrict__ in,
                                                                 double* __restrict__ out) {
    extern __shared__ double a_sm[];
    for (int i = threadIdx.x; i < P * P; i += blockDim.x) a_sm[i] = A[i];
    __syncthreads();
    const long j = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (j >= m) return;
    for (int p = 0; p < P; ++p) {
        double s = 0.0;
        for (int b = 0; b < P; ++b) s += a_sm[p * P + b] * in[b * m + j];
        out[p * m + j] = s;
    }
}

// centroid_spring_force for every bead of atom i (thread per atom): the centroid
// c = fac1 sum_b C2N[0][b] x_b (the first normal mode, as a position), then per bead k
// d1 = x_k - c, d2 = x_k - x_{k-1}, d3 = x_k - x_{k+1} (ring), the centroid-virial sum
// -d1 . f_k (physical forces), the spring sum m |d2|^2 and f_k -= coeff m (d2 + d3) fac3.
// acc[0] += sum_e, acc[1] += sum_d.
__global__ void __launch_bounds__(kThreads) k_pimd_springs(int P, int n, const double* __restrict__ c2n0,
                                                           const double* __restrict__ x,
                                                           const double* __restrict__ y,
                                                           const double* __restrict__ z, double* __restrict__ fx,
                                                           double* __restrict__ fy, double* __restrict__ fz,
                                                           const double* __restrict__ mass, double coeff,
                                                           double fac1, double fac3, double* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double red[2] = {0.0, 0.0};
    if (i < n) {
        const double* r[3] = {x, y, z};
        double* f[3] = {fx, fy, fz};
        double c[3] = {0.0, 0.0, 0.0};
        for (int b = 0; b < P; ++b)
            for (int q = 0; q < 3; ++q) c[q] += c2n0[b] * r[q][(size_t)b * n + i];
        for (int q = 0; q < 3; ++q) c[q] *= fac1;
        const double m = mass[i];
        for (int k = 0; k < P; ++k) {
            const int kp = k == 0 ? P - 1 : k - 1, kn = k == P - 1 ? 0 : k + 1;
            const size_t o = (size_t)k * n + i;
            double d2s = 0.0;
            for (int q = 0; q < 3; ++q) {
                const double xk = r[q][o];
                const double d1 = xk - c[q], d2 = xk - r[q][(size_t)kp * n + i], d3 = xk - r[q][(size_t)kn * n + i];
                red[1] -= d1 * f[q][o];
                d2s += d2 * d2;
                f[q][o] -= coeff * m * (d2 + d3) * fac3;
            }
            red[0] += m * d2s;
        }
    }
    block_sum_atomic<2>(red, acc);
}

}  // namespace

// transformation_matrix (SOURCE/centroid_matrix.f:3-135), 0-based: nmode_to_cart[bead][mode],
// cart_to_nmode[mode][bead], lambda[mode].
void pimd_matrices(int P, bool langevin, std::vector<double>& n2c, std::vector<double>& c2n,
                   std::vector<double>& lam) {
    n2c.assign((size_t)P * P, 0.0);
    c2n.assign((size_t)P * P, 0.0);
    lam.assign(P, 0.0);
    const double pi = 3.141592653589793;
    auto c = [&](int b, int m) -> double& { return n2c[(size_t)b * P + m]; };
    if (!langevin) {
        for (int b = 0; b < P; ++b) c(b, 0) = 1.0;
        for (int n1 = 1; n1 <= P / 2; ++n1) {
            c(2 * n1 - 1, P - 1) = -1.0;
            c(2 * n1 - 2, P - 1) = 1.0;
        }
        for (int n1 = 1; n1 <= P; ++n1) {
            const double t = 2.0 * pi * (n1 - 1) / P;
            for (int n2 = 1; n2 < P / 2; ++n2) {
                c(n1 - 1, 2 * n2 - 1) = std::sqrt(2.0) * std::cos(t * n2);
                c(n1 - 1, 2 * n2) = -std::sqrt(2.0) * std::sin(t * n2);
            }
        }
        for (int m = 0; m < P; ++m)
            for (int b = 0; b < P; ++b) c2n[(size_t)m * P + b] = c(b, m) / P;
        for (int k = 1; k < P / 2; ++k) {
            const double v = 2.0 * (1.0 - std::cos(2.0 * pi * k / P)) * P;
            lam[2 * k - 1] = v;
            lam[2 * k] = v;
        }
        lam[P - 1] = 4.0 * P;
    } else {
        for (int n1 = 1; n1 <= P; ++n1) {
            const double a = std::sqrt(1.0 / P);
            c(n1 - 1, 0) = a;
            c(n1 - 1, P / 2) = a * ((n1 % 2) ? -1.0 : 1.0);
            const double b = std::sqrt(2.0 / P);
            const double t = 2.0 * pi * n1 / P;
            for (int n2 = 2; n2 <= P / 2; ++n2) {
                c(n1 - 1, n2 - 1) = b * std::cos(t * (n2 - 1));
                c(n1 - 1, n2 + P / 2 - 1) = b * std::sin(t * (n2 + P / 2.0 - 1.0));
            }
        }
        for (int m = 0; m < P; ++m)
            for (int b = 0; b < P; ++b) c2n[(size_t)m * P + b] = c(b, m);
        for (int m = 0; m < P; ++m) lam[m] = 1.0;
    }
}

cudaError_t launch_pimd_transform(int P, long m, const double* A, const double* in, double* out, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    const unsigned nb = (unsigned)((m + kPimdThreads - 1) / kPimdThreads);
    k_pimd_transform<<<nb, kPimdThreads, (size_t)P * P * sizeof(double), s>>>(P, m, A, in, out);
    return cudaGetLastError();
}

cudaError_t launch_pimd_springs(int P, int n, const double* c2n0, const double* x, const double* y, const double* z,
                                double* fx, double* fy, double* fz, const double* mass, double coeff, double fac1,
                                double fac3, double* acc, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_pimd_springs<<<(n + kThreads - 1) / kThreads, kThreads, 0, s>>>(P, n, c2n0, x, y, z, fx, fy, fz, mass, coeff,
                                                                      fac1, fac3, acc);
    return cudaGetLastError();
}

int pimd_max_beads() { return kMaxBeads; }

}  // namespace mbx
