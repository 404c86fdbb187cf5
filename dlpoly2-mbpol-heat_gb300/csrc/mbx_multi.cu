// Many independent water boxes in one evaluation (path-integral beads, uneven boxes):
// one set of launches covers every box, list sizes stay on the device (no host
// synchronisation inside the step), so a repeated configuration can be captured once
// and replayed as a CUDA graph.
//
// Layout: box b holds nw_b waters in DL_POLY order (3*nw_b water atoms, then nw_b M
// sites) at atom offset 4 * sum_{b'<b} nw_b'.  Waters carry global indices; each
// water knows its box.  Candidates for the cluster lists are the waters of the same box
// (all pairs within the box), tested with the reference's exact O-O criteria.
#include "mbx_kernels.cuh"

#include <cub/device/device_scan.cuh>

namespace mbx {

namespace {

__global__ void k_multi_mono(int nw, const int* __restrict__ list, const int* __restrict__ wbox,
                             const Cell* __restrict__ cells, const double* __restrict__ x,
                             const double* __restrict__ y, const double* __restrict__ z, double* __restrict__ mono,
                             float4* __restrict__ of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    const Cell& cl = cells[wbox[i]];
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

// One warp per water: dimer partners j > i and 3B neighbours among the waters of its box.
__global__ void k_multi_neighbours(int nw, const double* __restrict__ mono, const float4* __restrict__ of,
                                   const int* __restrict__ wbox,
                                   const Cell* __restrict__ cells, const int* __restrict__ bstart,
                                   const int* __restrict__ bcount, int cap2, int cap3, int* __restrict__ n2,
                                   int* __restrict__ l2, int* __restrict__ n3, int* __restrict__ l3,
                                   int* __restrict__ overflow) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nw) return;   // warp-uniform
    const int b = wbox[i];
    const Cell& cl = cells[b];
    const int j0 = bstart[b], nb = bcount[b];
    int* my2 = l2 + (size_t)i * cap2;
    int* my3 = l3 + (size_t)i * cap3;
    int c2 = 0, c3 = 0;
    for (int base = 0; base < nb; base += 32) {
        const int k = base + lane;
        const int j = j0 + k;
        bool in2 = false, in3 = false;
        if (k < nb && j != i) {
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
        n2[i] = min(c2, cap2);
        n3[i] = min(c3, cap3);
        if (c2 > cap2 || c3 > cap3) atomicOr(overflow, 1);
    }
}

// Trimers of each centre (one warp per centre), as the single-box k_trimers, with the
// centre's box cell; writes beyond `cap` are dropped and flagged.
template <bool FILL>
__global__ void k_multi_trimers(int nw, const double* __restrict__ mono, const float4* __restrict__ of,
                                const int* __restrict__ wbox,
                                const Cell* __restrict__ cells, int cap3, const int* __restrict__ n3,
                                const int* __restrict__ l3, int* __restrict__ cnt, const int* __restrict__ off,
                                int4* __restrict__ trip, long cap, int* __restrict__ overflow) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nw) return;
    const Cell& cl = cells[wbox[c]];
    const int n = n3[c];
    const int* nb = l3 + (size_t)c * cap3;
    const int npair = n * (n - 1) / 2;
    int m = 0;
    const long base = FILL ? off[c] : 0;
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
            int i = c, j = a, kk = b;
            if (i > j) { int t = i; i = j; j = t; }
            if (j > kk) { int t = j; j = kk; kk = t; }
            if (i > j) { int t = i; i = j; j = t; }
            const long slot = base + m + __popc(bal & ((1u << lane) - 1u));
            if (slot < cap) trip[slot] = make_int4(i, j, kk, 0);
            else atomicOr(overflow, 2);
        }
        m += __popc(bal);
    }
    if (!FILL && lane == 0) cnt[c] = m;
}

__global__ void k_multi_totals(int nw, const int* n2, const int* off2, const int* tcnt, const int* toff, long cap2,
                               long cap3, int* totals, int* overflow) {
    const long np = nw > 0 ? (long)off2[nw - 1] + n2[nw - 1] : 0;
    const long nt = nw > 0 ? (long)toff[nw - 1] + tcnt[nw - 1] : 0;
    if (nt > cap3) atomicOr(overflow, 2);
    // a list that outgrew its capacity: evaluate nothing (the host grows the lists and
    // repeats the step, so no partial forces are ever accumulated)
    const bool bad = *(volatile int*)overflow != 0;
    totals[0] = bad ? 0 : (int)min(np, cap2);
    totals[1] = bad ? 0 : (int)min(nt, cap3);
}

// jkin per box: atoms are contiguous per box, so warps rarely straddle boxes.
__global__ void __launch_bounds__(kThreads) k_multi_jkin(int natms, const int* __restrict__ abox,
                                                          const unsigned char* __restrict__ is_water,
                                                          const double* __restrict__ vx, const double* __restrict__ vy,
                                                          const double* __restrict__ vz,
                                                          const double* __restrict__ mass,
                                                          const double* __restrict__ ae, double* acc_box,
                                                          const int* __restrict__ skip) {
    if (*skip) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double j[3] = {0.0, 0.0, 0.0};
    int box = -1;
    if (i < natms && is_water[i]) {
        box = abox[i];
        const double v0 = vx[i], v1 = vy[i], v2 = vz[i];
        const double kin = 0.5 * mass[i] * (v0 * v0 + v1 * v1 + v2 * v2);
        const double eng = kin + (ae ? ae[i] : 0.0);
        j[0] = eng * v0;
        j[1] = eng * v1;
        j[2] = eng * v2;
    }
    int lo = box < 0 ? 0x7fffffff : box, hi = box;
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (hi < 0) return;
    if (lo == hi) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double v = warp_sum(j[q]);
            if ((threadIdx.x & 31) == 0) atomicAdd(acc_box + (size_t)hi * S_NSLOTS + S_JKIN + q, v);
        }
    } else if (box >= 0) {
#pragma unroll
        for (int q = 0; q < 3; ++q) atomicAdd(acc_box + (size_t)box * S_NSLOTS + S_JKIN + q, j[q]);
    }
}

int blocks_for(long threads) { return (int)((threads + kThreads - 1) / kThreads); }

}  // namespace

MultiBoxes::~MultiBoxes() { release(); }

void MultiBoxes::release() {
    void* ptrs[] = {list,  listang, wbox,  abox,     is_water, cells,   bstart,     bcount, mono,   n2,
                    l2,    off2,    n3,    l3,       tcnt,     toff,    pairs,      trip,   hard2,  hard3,
                    hard_count, scan_tmp, acc_box, pes_box, ae_scratch, totals, flag, ctr, partial, done, of};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    list = listang = wbox = abox = bstart = bcount = n2 = l2 = off2 = n3 = l3 = tcnt = toff = nullptr;
    hard_count = totals = flag = ctr = done = nullptr;
    partial = nullptr;
    part_cap = 0;
    is_water = nullptr;
    cells = nullptr;
    mono = acc_box = pes_box = ae_scratch = nullptr;
    of = nullptr;
    pairs = hard2 = nullptr;
    trip = hard3 = nullptr;
    scan_tmp = nullptr;
    scan_bytes = 0;
    pair_cap = trip_cap = 0;
    nbox = nw = natms = 0;
    nw_of_box.clear();
}

cudaError_t MultiBoxes::setup(int nbox_, const int* nw_box, bool need_hard, cudaStream_t s) {
    cudaError_t e;
    std::vector<int> nwb(nw_box, nw_box + nbox_);
    if (nbox_ == nbox && nwb == nw_of_box && pairs) {
        if (need_hard && !hard2) {
            if ((e = cudaMalloc(&hard2, (pair_cap + 1) * sizeof(int2)))) return e;
            if ((e = cudaMalloc(&hard3, (trip_cap + 1) * sizeof(int4)))) return e;
        }
        return cudaSuccess;
    }
    release();
    ++gen;
    nbox = nbox_;
    nw_of_box = nwb;
    for (int b = 0; b < nbox; ++b) nw += nwb[b];
    natms = 4 * nw;
    // host-side layout tables: 1-based water atoms and H-O-H angles, box of every water/atom
    std::vector<int> hl(3 * (size_t)nw), ha(3 * (size_t)nw), hw(nw), hab(natms), hbs(nbox), hbc(nbox);
    std::vector<unsigned char> hwat(natms, 0);
    int w0 = 0, a0 = 0;
    for (int b = 0; b < nbox; ++b) {
        hbs[b] = w0;
        hbc[b] = nwb[b];
        for (int i = 0; i < nwb[b]; ++i) {
            const int o = a0 + 3 * i + 1;
            const size_t k = 3 * (size_t)(w0 + i);
            hl[k] = o;
            hl[k + 1] = o + 1;
            hl[k + 2] = o + 2;
            ha[k] = o + 1;
            ha[k + 1] = o;
            ha[k + 2] = o + 2;
            hw[w0 + i] = b;
        }
        for (int q = 0; q < 4 * nwb[b]; ++q) {
            hab[a0 + q] = b;
            hwat[a0 + q] = q < 3 * nwb[b];
        }
        w0 += nwb[b];
        a0 += 4 * nwb[b];
    }
    const size_t n = (size_t)nw + 1;
    if ((e = cudaMalloc(&list, 3 * n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&listang, 3 * n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&wbox, n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&abox, ((size_t)natms + 1) * sizeof(int)))) return e;
    if ((e = cudaMalloc(&is_water, (size_t)natms + 1))) return e;
    if ((e = cudaMalloc(&cells, (size_t)nbox * sizeof(Cell)))) return e;
    if ((e = cudaMalloc(&bstart, (size_t)nbox * sizeof(int)))) return e;
    if ((e = cudaMalloc(&bcount, (size_t)nbox * sizeof(int)))) return e;
    if ((e = cudaMalloc(&mono, 9 * n * sizeof(double)))) return e;
    if ((e = cudaMalloc(&of, n * sizeof(float4)))) return e;
    if ((e = cudaMalloc(&n2, n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&off2, n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&n3, n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&tcnt, n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&toff, n * sizeof(int)))) return e;
    if ((e = cudaMalloc(&l2, n * cap2 * sizeof(int)))) return e;
    if ((e = cudaMalloc(&l3, n * cap3 * sizeof(int)))) return e;
    pair_cap = (long)nw * cap2;
    trip_cap = (long)nw * trip_per_water;
    if ((e = cudaMalloc(&pairs, (pair_cap + 1) * sizeof(int2)))) return e;
    if ((e = cudaMalloc(&trip, (trip_cap + 1) * sizeof(int4)))) return e;
    if (need_hard) {
        if ((e = cudaMalloc(&hard2, (pair_cap + 1) * sizeof(int2)))) return e;
        if ((e = cudaMalloc(&hard3, (trip_cap + 1) * sizeof(int4)))) return e;
    }
    if ((e = cudaMalloc(&hard_count, 2 * sizeof(int)))) return e;
    size_t a = 0;
    if ((e = cub::DeviceScan::ExclusiveSum(nullptr, a, n2, off2, (int)n))) return e;
    scan_bytes = a;
    if ((e = cudaMalloc(&scan_tmp, scan_bytes))) return e;
    if ((e = cudaMalloc(&acc_box, (size_t)nbox * S_NSLOTS * sizeof(double)))) return e;
    if ((e = cudaMalloc(&pes_box, (size_t)nbox * 14 * sizeof(double)))) return e;
    if ((e = cudaMalloc(&ae_scratch, ((size_t)natms + 1) * sizeof(double)))) return e;
    if ((e = cudaMalloc(&totals, 4 * sizeof(int)))) return e;
    if ((e = cudaMalloc(&flag, 4 * sizeof(int)))) return e;
    if ((e = cudaMalloc(&ctr, 2 * sizeof(int)))) return e;
    // split FP64 dimers for up to 32 dimers per water (liquid water has ~20-25 within
    // the 2B cutoff); more dimers fall back to one task per dimer
    part_cap = 32L * nw + 32;
    if ((e = cudaMalloc(&partial, (size_t)part_cap * dimer_parts() * 32 * sizeof(double)))) return e;
    if ((e = cudaMalloc(&done, (size_t)part_cap * sizeof(int)))) return e;
    int dev = 0;
    if ((e = cudaGetDevice(&dev))) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev))) return e;
    // pageable sources: each copy has read them before it returns
    if ((e = cudaMemcpyAsync(list, hl.data(), hl.size() * sizeof(int), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaMemcpyAsync(listang, ha.data(), ha.size() * sizeof(int), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaMemcpyAsync(wbox, hw.data(), hw.size() * sizeof(int), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaMemcpyAsync(abox, hab.data(), hab.size() * sizeof(int), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaMemcpyAsync(is_water, hwat.data(), hwat.size(), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaMemcpyAsync(bstart, hbs.data(), nbox * sizeof(int), cudaMemcpyHostToDevice, s))) return e;
    if ((e = cudaMemcpyAsync(bcount, hbc.data(), nbox * sizeof(int), cudaMemcpyHostToDevice, s))) return e;
    return cudaStreamSynchronize(s);
}

// The whole multi-box step, asynchronous on `s` (no host synchronisation, no allocation).
cudaError_t MultiBoxes::enqueue(int precision, const MixedPass& limits, bool fused, const double* x,
                                const double* y, const double* z, double* fx, double* fy, double* fz, const double* vx,
                                const double* vy, const double* vz, const double* mass, double* ae,
                                cudaStream_t s) {
    cudaError_t e;
    launches = 0;
    const bool heat = vx && vy && vz;
    double* ae_use = ae;
    if (!ae_use && heat && mass) {
        ae_use = ae_scratch;
        if ((e = cudaMemsetAsync(ae_use, 0, (size_t)natms * sizeof(double), s))) return e;
    }
    if ((e = cudaMemsetAsync(acc_box, 0, (size_t)nbox * S_NSLOTS * sizeof(double), s))) return e;
    if ((e = cudaMemsetAsync(pes_box, 0, (size_t)nbox * 14 * sizeof(double), s))) return e;
    if ((e = cudaMemsetAsync(flag, 0, 4 * sizeof(int), s))) return e;
    if ((e = cudaMemsetAsync(hard_count, 0, 2 * sizeof(int), s))) return e;
    if (nw == 0) return cudaSuccess;
    // cluster lists
    k_multi_mono<<<blocks_for(nw), kThreads, 0, s>>>(nw, list, wbox, cells, x, y, z, mono, of);
    k_multi_neighbours<<<blocks_for(32L * nw), kThreads, 0, s>>>(nw, mono, of, wbox, cells, bstart, bcount, cap2, cap3,
                                                                  n2, l2, n3, l3, flag);
    size_t a = scan_bytes;
    if ((e = cub::DeviceScan::ExclusiveSum(scan_tmp, a, n2, off2, nw, s))) return e;
    launch_pairs_compact(nw, cap2, n2, off2, l2, pairs, s);
    k_multi_trimers<false><<<blocks_for(32L * nw), kThreads, 0, s>>>(nw, mono, of, wbox, cells, cap3, n3, l3, tcnt,
                                                                      nullptr, nullptr, 0, flag);
    a = scan_bytes;
    if ((e = cub::DeviceScan::ExclusiveSum(scan_tmp, a, tcnt, toff, nw, s))) return e;
    k_multi_trimers<true><<<blocks_for(32L * nw), kThreads, 0, s>>>(nw, mono, of, wbox, cells, cap3, n3, l3, nullptr,
                                                                     toff, trip, trip_cap, flag);
    k_multi_totals<<<1, 1, 0, s>>>(nw, n2, off2, tcnt, toff, pair_cap, trip_cap, totals, flag);
    launches += 6 + 2 * 2;   // own kernels + two CUB scans (two kernels each)
    if ((e = cudaGetLastError())) return e;
    // 1-body term of every water (skipped when a list overflowed)
    if ((e = launch_ps_pes_boxes(nw, listang, cells, wbox, x, y, z, fx, fy, fz, ae_use, heat ? vx : nullptr,
                                 heat ? vy : nullptr, heat ? vz : nullptr, pes_box, flag, s)))
        return e;
    ++launches;
    // 2B / 3B terms with the heat current
    MbpolArgs args;
    args.nw = nw;
    args.cell = Cell{};
    args.list = list;
    args.x = x;
    args.y = y;
    args.z = z;
    args.vx = heat ? vx : nullptr;
    args.vy = heat ? vy : nullptr;
    args.vz = heat ? vz : nullptr;
    args.mono = mono;
    args.fx = fx;
    args.fy = fy;
    args.fz = fz;
    args.ae = ae_use;
    args.acc = nullptr;
    args.cells = cells;
    args.wbox = wbox;
    args.acc_box = acc_box;
    MixedPass mp = limits;
    mp.hard2 = hard2;
    mp.hard3 = hard3;
    mp.count = hard_count;
    if (!hard2) {   // no hand-off lists: the default split (2B FP64, 3B FP32)
        mp.limit2 = 0.f;
        mp.limit3 = 3.4e38f;
    }
    if (fused && fused_applies(precision, mp)) {
        if ((e = launch_23(args, pairs, 0, totals + 0, trip, 0, totals + 1, precision, ctr, nsm, s, partial, done,
                           part_cap)))
            return e;
        launches += 1;
    } else {
        if ((e = launch_2b_dev(args, pairs, pair_cap, totals + 0, precision, mp, s))) return e;
        if ((e = launch_3b_dev(args, trip, trip_cap, totals + 1, precision, mp, s))) return e;
        launches += (precision == 1 && mp.limit2 > 0.f) ? 2 : 1;
        launches += (precision == 1 && mp.limit3 > 0.f && mp.limit3 < 3.0e38f) ? 2 : 1;
    }
    if (heat && mass) {
        k_multi_jkin<<<blocks_for(natms), kThreads, 0, s>>>(natms, abox, is_water, vx, vy, vz, mass, ae_use,
                                                            acc_box, flag);
        ++launches;
    }
    return cudaGetLastError();
}

}  // namespace mbx
