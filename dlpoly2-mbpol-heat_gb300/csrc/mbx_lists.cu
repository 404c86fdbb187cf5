// Monomer imaging, O-atom cell list, and the MB-pol dimer / trimer lists.
//
// The reference enumerates every pair and every triple of waters and tests
// O-O distances inside the loop (SOURCE/mbpol.f90:226-272 and :314-374; the
// tests are in do_dimer :496-503 and do_trimer :839-862).  Here the same tests,
// evaluated with the same floating-point operations, run only on candidates from
// a cell list, so the lists are identical as sets while the work is O(N).
//
// Layout: monomers are 9 doubles per water (O, H1, H2; H imaged next to O), the
// pair list is int2 (i < j) grouped by i, the trimer list is int4 (i < j < k, w
// unused) grouped by the centre water that generated it.
#include "mbx_kernels.cuh"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>

namespace mbx {

// image_monomers (SOURCE/mbpol.f90:1275-1301) fused with the gather of
// mbpol_forces (SOURCE/mbpol.f90:194-200): listttm2 is 1-based.
__global__ void k_image_monomers(int nw, const int* __restrict__ list, const double* __restrict__ x,
                                 const double* __restrict__ y, const double* __restrict__ z, Cell cl,
                                 double* __restrict__ mono, float4* __restrict__ of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    double w[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int at = list[3 * i + a] - 1;
        w[3 * a + 0] = x[at];
        w[3 * a + 1] = y[at];
        w[3 * a + 2] = z[at];
    }
#pragma unroll
    for (int h = 1; h < 3; ++h) {
        double ox = dsub(w[3 * h + 0], w[0]), oy = dsub(w[3 * h + 1], w[1]), oz = dsub(w[3 * h + 2], w[2]);
        image(cl, ox, oy, oz);
        w[3 * h + 0] = dadd(w[0], ox);
        w[3 * h + 1] = dadd(w[1], oy);
        w[3 * h + 2] = dadd(w[2], oz);
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) mono[9 * (size_t)i + q] = w[q];
    of[i] = make_float4((float)w[0], (float)w[1], (float)w[2], 0.f);
}

__device__ __forceinline__ int wrap_cell(double s, int nc) {
    s = s - floor(s);
    int c = (int)(s * nc);
    return c >= nc ? nc - 1 : (c < 0 ? 0 : c);
}

__global__ void k_cell_keys(int nw, const double* __restrict__ mono, Cell cl, int3 nc,
                            unsigned* __restrict__ key, int* __restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    const double* o = mono + 9 * (size_t)i;
    const int cx = wrap_cell(o[0] * cl.inv[0], nc.x);
    const int cy = wrap_cell(o[1] * cl.inv[1], nc.y);
    const int cz = wrap_cell(o[2] * cl.inv[2], nc.z);
    key[i] = (unsigned)((cz * nc.y + cy) * nc.x + cx);
    idx[i] = i;
}

__global__ void k_cell_bounds(int nw, int ncell, const unsigned* __restrict__ skey, int* __restrict__ start,
                              int* __restrict__ end) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    const unsigned c = skey[i];
    if (i == 0 || skey[i - 1] != c) start[c] = i;
    if (i == nw - 1 || skey[i + 1] != c) end[c] = i + 1;
}

// Per water i (one warp): dimer partners j > i (2B test) and 3B neighbours j != i
// (3B edge test).  Lanes test candidates in parallel and append the hits in candidate
// order through a warp ballot, so the lists are deterministic.  Candidates come from
// the 27 surrounding cells (in a fixed order, waters by index within a cell), or from
// every water when the grid is too coarse (all_pairs).
__global__ void k_neighbours(int nw, const double* __restrict__ mono, const float4* __restrict__ of, Cell cl,
                             int3 nc, int all_pairs,
                             const unsigned* __restrict__ skey, const int* __restrict__ sidx,
                             const int* __restrict__ cstart, const int* __restrict__ cend, int cap2, int cap3,
                             int* __restrict__ n2, int* __restrict__ l2, int* __restrict__ n3,
                             int* __restrict__ l3, int* __restrict__ overflow) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nw) return;   // warp-uniform
    const double* oi = mono + 9 * (size_t)i;
    int* my2 = l2 + (size_t)i * cap2;
    int* my3 = l3 + (size_t)i * cap3;
    // candidate ranges: lane c < 27 owns neighbour cell c
    int cs = 0, cn = 0;
    int total;
    if (all_pairs) {
        total = nw;
    } else {
        if (lane < 27) {
            const int cx = wrap_cell(oi[0] * cl.inv[0], nc.x);
            const int cy = wrap_cell(oi[1] * cl.inv[1], nc.y);
            const int cz = wrap_cell(oi[2] * cl.inv[2], nc.z);
            const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
            const int x = (cx + dx + nc.x) % nc.x, y = (cy + dy + nc.y) % nc.y, z = (cz + dz + nc.z) % nc.z;
            const int c = (z * nc.y + y) * nc.x + x;
            cs = cstart[c];
            cn = cend[c] - cs;
        }
        // inclusive prefix of the counts over lanes
        int incl = cn;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        total = __shfl_sync(0xffffffffu, incl, 31);
        cn = incl;   // lane c now holds the end offset of cell c in the candidate sequence
    }
    int c2 = 0, c3 = 0;
    for (int base = 0; base < total; base += 32) {
        const int k = base + lane;
        const bool valid = k < total;
        int j = -1;
        if (all_pairs) {
            if (valid) j = k;
        } else {
            // the cell holding candidate k: the first cell whose end offset exceeds k
            // (all lanes take part in the shuffles; total > 0 inside this loop)
            const int kk = valid ? k : total - 1;
            int cell = 0;
            for (int c = 0; c < 27; ++c) {
                const int end = __shfl_sync(0xffffffffu, cn, c);
                if (kk >= end) cell = c + 1;
            }
            const int start = __shfl_sync(0xffffffffu, cs, cell);
            const int prev_end = __shfl_sync(0xffffffffu, cn, cell > 0 ? cell - 1 : 0);
            if (valid) j = sidx[start + (kk - (cell > 0 ? prev_end : 0))];
        }
        bool in2 = false, in3 = false;
        if (j >= 0 && j != i) {
            pair_tests(cl, of, mono, i, j, in2, in3);
            in2 = in2 && j > i;
        }
        const unsigned b2 = __ballot_sync(0xffffffffu, in2);
        const unsigned b3 = __ballot_sync(0xffffffffu, in3);
        const unsigned lt = (1u << lane) - 1u;
        if (in2) {
            const int q = c2 + __popc(b2 & lt);
            if (q < cap2) my2[q] = j;
        }
        if (in3) {
            const int q = c3 + __popc(b3 & lt);
            if (q < cap3) my3[q] = j;
        }
        c2 += __popc(b2);
        c3 += __popc(b3);
    }
    if (lane == 0) {
        n2[i] = c2;
        n3[i] = c3;
        if (c2 > cap2 || c3 > cap3) atomicOr(overflow, 1);
    }
}

__global__ void k_pairs_compact(int nw, int cap2, const int* __restrict__ n2, const int* __restrict__ off2,
                                const int* __restrict__ l2, int2* __restrict__ pairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    const int n = min(n2[i], cap2), o = off2[i];
    for (int q = 0; q < n; ++q) pairs[o + q] = make_int2(i, l2[(size_t)i * cap2 + q]);
}

// Trimers {c, a, b} with a, b 3B neighbours of the centre c (one warp per centre).
// A trimer is kept by the reference iff some water is within the 3B cutoff of the
// other two (istoobig1..3 in SOURCE/mbpol.f90:858-862); it is generated here by the
// smallest such centre only, so every trimer appears exactly once.  Lanes test the
// pairs (p < q) of the neighbour list in parallel, 32 pairs per step in lexicographic
// order (the FP64 distance tests keep every lane busy); hits are appended in pair order.
template <bool FILL>
__global__ void k_trimers(int nw, const double* __restrict__ mono, const float4* __restrict__ of, Cell cl, int cap3,
                          const int* __restrict__ n3,
                          const int* __restrict__ l3, int* __restrict__ cnt, const int* __restrict__ off,
                          int4* __restrict__ trip) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nw) return;   // warp-uniform
    const int n = min(n3[c], cap3);
    const int* nb = l3 + (size_t)c * cap3;
    const int npair = n * (n - 1) / 2;
    int m = 0;
    const int base = FILL ? off[c] : 0;
    for (int k0 = 0; k0 < npair; k0 += 32) {
        const int k = k0 + lane;
        bool keep = false;
        int a = 0, b = 0;
        if (k < npair) {
            int p, q;
            pair_of_index(n, k, p, q);
            a = nb[p];
            b = nb[q];
            bool in2, ab;
            pair_tests(cl, of, mono, a, b, in2, ab);
            keep = !(ab && (a < c || b < c));
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (FILL && keep) {
            int i = c, j = a, kk = b;  // sort the three indices
            if (i > j) { int t = i; i = j; j = t; }
            if (j > kk) { int t = j; j = kk; kk = t; }
            if (i > j) { int t = i; i = j; j = t; }
            trip[base + m + __popc(bal & ((1u << lane) - 1u))] = make_int4(i, j, kk, 0);
        }
        m += __popc(bal);
    }
    if (!FILL && lane == 0) cnt[c] = m;
}

// ---------------------------------------------------------------------------
ListBuilder::~ListBuilder() { release(); }

static void free_ptr(void*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}
template <typename T>
static void free_t(T*& p) {
    void* q = p;
    free_ptr(q);
    p = nullptr;
}

void ListBuilder::release() {
    if (external) return;
    free_t(key); free_t(skey); free_t(idx); free_t(sidx); free_t(cstart); free_t(cend);
    free_t(n2); free_t(l2); free_t(off2); free_t(n3); free_t(l3); free_t(tcnt); free_t(toff);
    free_t(flag); free_t(of); free_ptr(scan_tmp); free_ptr(sort_tmp);
    nw_cap = ncell_cap = 0;
    cap2_alloc = cap3_alloc = 0;
}

cudaError_t ListBuilder::reserve(int nw, int ncell) {
    cudaError_t e = cudaSuccess;
    if (external) return (nw <= nw_cap && ncell <= ncell_cap) ? cudaSuccess : cudaErrorInvalidValue;
    if (nw > nw_cap || cap2 != cap2_alloc || cap3 != cap3_alloc) {
        free_t(key); free_t(skey); free_t(idx); free_t(sidx);
        free_t(n2); free_t(l2); free_t(off2); free_t(n3); free_t(l3); free_t(tcnt); free_t(toff); free_t(of);
        free_ptr(scan_tmp); free_ptr(sort_tmp);
        const int n = std::max(nw, nw_cap) + 1;
        nw_cap = 0;   // until every buffer below exists
        cap2_alloc = cap3_alloc = 0;
        if ((e = cudaMalloc(&key, n * sizeof(unsigned)))) return e;
        if ((e = cudaMalloc(&skey, n * sizeof(unsigned)))) return e;
        if ((e = cudaMalloc(&idx, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&sidx, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&n2, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&off2, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&n3, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&tcnt, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&toff, n * sizeof(int)))) return e;
        if ((e = cudaMalloc(&l2, (size_t)n * cap2 * sizeof(int)))) return e;
        if ((e = cudaMalloc(&l3, (size_t)n * cap3 * sizeof(int)))) return e;
        if ((e = cudaMalloc(&of, (size_t)n * sizeof(float4)))) return e;
        size_t a = 0, b = 0;
        if ((e = cub::DeviceScan::ExclusiveSum(nullptr, a, n2, off2, n))) return e;
        if ((e = cub::DeviceRadixSort::SortPairs(nullptr, b, key, skey, idx, sidx, n))) return e;
        scan_bytes = a;
        sort_bytes = b;
        if ((e = cudaMalloc(&scan_tmp, scan_bytes))) return e;
        if ((e = cudaMalloc(&sort_tmp, sort_bytes))) return e;
        nw_cap = n - 1;
        cap2_alloc = cap2;
        cap3_alloc = cap3;
    }
    if (ncell > ncell_cap) {
        free_t(cstart);
        free_t(cend);
        ncell_cap = 0;
        if ((e = cudaMalloc(&cstart, ncell * sizeof(int)))) return e;
        if ((e = cudaMalloc(&cend, ncell * sizeof(int)))) return e;
        ncell_cap = ncell;
    }
    if (!flag && (e = cudaMalloc(&flag, 4 * sizeof(int)))) return e;
    return e;
}

static int grid_for(int n) { return (n + kThreads - 1) / kThreads; }

// Phase 1: image monomers, cell list, neighbour lists, counts and offsets.  The
// caller reads back `totals` (pairs, trimers, overflow) before phase 2.
cudaError_t ListBuilder::phase1(int nw, const int* list, const double* x, const double* y, const double* z,
                                const Cell& cl, double* mono, int* totals_dev, cudaStream_t s) {
    // grid: cells of at least the 2B cutoff; all-pairs if fewer than 3 per side or triclinic
    int3 nc = make_int3(1, 1, 1);
    int all_pairs = 1;
    if ((cl.imcon == 1 || cl.imcon == 2) && !external) {
        nc.x = (int)(cl.c[0] / kR2f);
        nc.y = (int)(cl.c[4] / kR2f);
        nc.z = (int)(cl.c[8] / kR2f);
        if (nc.x >= 3 && nc.y >= 3 && nc.z >= 3) all_pairs = 0;
        else nc = make_int3(1, 1, 1);
    }
    const int ncell = nc.x * nc.y * nc.z;
    cudaError_t e = reserve(nw, ncell);
    if (e) return e;
    nc_last = nc;
    all_pairs_last = all_pairs;
    // launch count: image, [keys, radix sort (CUB), bounds], neighbours, scan (CUB), trimer count,
    // scan (CUB), totals.  CUB's DeviceScan is 2 kernels; its one-sweep radix sort of <= 16 key bits
    // is a histogram, an exclusive-sum and one pass per 8-bit digit.
    launches_last = 1 + 1 + 2 + 1 + 2 + 1;
    const int g = grid_for(nw);
    k_image_monomers<<<g, kThreads, 0, s>>>(nw, list, x, y, z, cl, mono, of);
    if (!all_pairs) {
        cudaMemsetAsync(cstart, 0, ncell * sizeof(int), s);
        cudaMemsetAsync(cend, 0, ncell * sizeof(int), s);
        k_cell_keys<<<g, kThreads, 0, s>>>(nw, mono, cl, nc, key, idx);
        size_t b = sort_bytes;
        int bits = 1;
        while ((1 << bits) < ncell) ++bits;
        cub::DeviceRadixSort::SortPairs(sort_tmp, b, key, skey, idx, sidx, nw, 0, bits, s);
        launches_last += 2 + 2 + (bits + 7) / 8;
        k_cell_bounds<<<g, kThreads, 0, s>>>(nw, ncell, skey, cstart, cend);
    }
    cudaMemsetAsync(flag, 0, sizeof(int), s);
    const int gw = (int)(((long)nw * 32 + kThreads - 1) / kThreads);   // one warp per water
    k_neighbours<<<gw, kThreads, 0, s>>>(nw, mono, of, cl, nc, all_pairs, skey, sidx, cstart, cend, cap2, cap3, n2, l2,
                                         n3, l3, flag);
    size_t a = scan_bytes;
    cub::DeviceScan::ExclusiveSum(scan_tmp, a, n2, off2, nw, s);
    k_trimers<false><<<gw, kThreads, 0, s>>>(nw, mono, of, cl, cap3, n3, l3, tcnt, nullptr, nullptr);
    a = scan_bytes;
    cub::DeviceScan::ExclusiveSum(scan_tmp, a, tcnt, toff, nw, s);
    k_list_totals<<<1, 1, 0, s>>>(nw, n2, off2, tcnt, toff, flag, totals_dev);
    return cudaGetLastError();
}

cudaError_t ListBuilder::phase2(int nw, const Cell& cl, const double* mono, int2* pairs, int4* trip,
                                cudaStream_t s) {
    const int g = grid_for(nw);
    k_pairs_compact<<<g, kThreads, 0, s>>>(nw, cap2, n2, off2, l2, pairs);
    const int gw = (int)(((long)nw * 32 + kThreads - 1) / kThreads);
    k_trimers<true><<<gw, kThreads, 0, s>>>(nw, mono, of, cl, cap3, n3, l3, nullptr, toff, trip);
    launches_last += 2;
    return cudaGetLastError();
}

void launch_pairs_compact(int nw, int cap2, const int* n2, const int* off2, const int* l2, int2* pairs,
                          cudaStream_t s) {
    if (nw <= 0) return;
    k_pairs_compact<<<grid_for(nw), kThreads, 0, s>>>(nw, cap2, n2, off2, l2, pairs);
}

__global__ void k_list_totals(int nw, const int* n2, const int* off2, const int* tcnt, const int* toff,
                              const int* flag, int* totals) {
    totals[0] = nw > 0 ? off2[nw - 1] + min(n2[nw - 1], 0x7fffffff) : 0;
    totals[1] = nw > 0 ? toff[nw - 1] + tcnt[nw - 1] : 0;
    totals[2] = flag[0];
}

}  // namespace mbx
