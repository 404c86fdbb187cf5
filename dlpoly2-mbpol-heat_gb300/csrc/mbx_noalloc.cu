// mbx_mbpol_forces_noalloc: the MB-pol evaluation without any device allocation.
//
// Some callers cannot call cudaMalloc at the point where they need forces: hosts whose
// device memory is owned by another allocator or pool and must not be fragmented or
// raced by a second allocator, and real-time MD drivers that forbid allocation after
// start-up (an allocation can synchronise the device and take milliseconds).  For them
// this entry point keeps every intermediate (imaged monomers, neighbour and cluster
// lists, scan workspace, accumulators) in one file-scope __device__ array of fixed
// size, and the caller passes only its inputs and outputs.
//
// The call synchronises the caller's stream twice: once to read the list totals (they
// size the cluster launches) and once at the end to read the scalars.
//
// Limits: at most kMaxWaters waters, at most kCap2 dimer partners and kCap3 3B
// neighbours per water, at most kMaxTrimers trimers; beyond them the call returns
// MBX_ERR_ARG / MBX_ERR_CAPACITY with a message on stderr.  Candidates are all waters
// (no cell sort, so no sort workspace), which is cheap at these sizes.
#include "../../include/mbx.h"
#include "mbx_kernels.cuh"

#include <cub/device/device_scan.cuh>

#include <cstdio>
#include <cstring>
#include <mutex>

namespace {

using namespace mbx;

constexpr int kMaxWaters = 512;
constexpr int kCap2 = 64;
constexpr int kCap3 = 48;
constexpr long kMaxTrimers = 256L * kMaxWaters;
constexpr size_t kScanBytes = 64 << 10;

constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// layout of the scratch array (byte offsets)
constexpr size_t kN = kMaxWaters + 1;
constexpr size_t oMono = 0;
constexpr size_t oAcc = align256(oMono + 9 * sizeof(double) * kN);
constexpr size_t oTotals = align256(oAcc + MBX_NSCALARS * sizeof(double));
constexpr size_t oFlag = align256(oTotals + 4 * sizeof(int));
constexpr size_t oOf = align256(oFlag + 4 * sizeof(int));
constexpr size_t oCtr = align256(oOf + kN * sizeof(float4));
constexpr size_t oN2 = align256(oCtr + 4 * sizeof(int));
constexpr size_t oOff2 = align256(oN2 + kN * sizeof(int));
constexpr size_t oN3 = align256(oOff2 + kN * sizeof(int));
constexpr size_t oTcnt = align256(oN3 + kN * sizeof(int));
constexpr size_t oToff = align256(oTcnt + kN * sizeof(int));
constexpr size_t oL2 = align256(oToff + kN * sizeof(int));
constexpr size_t oL3 = align256(oL2 + kN * kCap2 * sizeof(int));
constexpr size_t oScan = align256(oL3 + kN * kCap3 * sizeof(int));
constexpr size_t oPairs = align256(oScan + kScanBytes);
constexpr size_t oTrip = align256(oPairs + (size_t)kMaxWaters * kCap2 * sizeof(int2));
constexpr size_t kScratchBytes = align256(oTrip + (size_t)kMaxTrimers * sizeof(int4));

}  // namespace

// The scratch.  Every GPU that loads libmbx holds it (~2.7 MB) until the process exits.
static __device__ __align__(256) unsigned char g_mbx_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_mu;
unsigned char* g_scratch_ptr[64] = {nullptr};

int report(int code, const char* msg) {
    std::fprintf(stderr, "mbx_mbpol_forces_noalloc: %s\n", msg);
    return code;
}

// Device address of the scratch on the current device, looked up once per device.
// In host code g_mbx_noalloc_scratch is only a host-side stand-in for the symbol, so
// the address must come from cudaGetSymbolAddress with that device current.  The
// address is cached for the life of the process: do not use this entry point across a
// cudaDeviceReset of the device (the module, and with it the array, may move).
unsigned char* scratch_for_current_device(int* dev_out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    *dev_out = dev;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_mbx_noalloc_scratch);
        if (e != cudaSuccess) {
            std::fprintf(stderr, "mbx_mbpol_forces_noalloc: cudaGetSymbolAddress failed: %s\n",
                         cudaGetErrorString(e));
            return nullptr;
        }
        g_scratch_ptr[dev] = (unsigned char*)p;
    }
    return g_scratch_ptr[dev];
}

}  // namespace

#define NA_CK(call)                                                                                  \
    do {                                                                                             \
        const cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                                     \
            std::fprintf(stderr, "mbx_mbpol_forces_noalloc: %s failed: %s\n", #call,                 \
                         cudaGetErrorString(e_));                                                    \
            return MBX_ERR_CUDA;                                                                     \
        }                                                                                            \
    } while (0)

extern "C" int mbx_mbpol_forces_noalloc(int precision, int imcon, const double* cell, int nttm2,
                                        const int* listttm2, int natms, const double* xxx, const double* yyy,
                                        const double* zzz, double* fxx, double* fyy, double* fzz,
                                        const double* vxx, const double* vyy, const double* vzz,
                                        const double* weight, double* atomic_energy, double* scalars,
                                        void* stream) {
    if (precision != MBX_FP64 && precision != MBX_MIXED) return report(MBX_ERR_ARG, "bad precision");
    if (nttm2 < 0 || nttm2 % 3) return report(MBX_ERR_ARG, "nttm2 must be a non-negative multiple of 3");
    const int nw = nttm2 / 3;
    if (nw > kMaxWaters) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "%d waters exceed the fixed scratch limit of %d waters", nw, kMaxWaters);
        return report(MBX_ERR_ARG, msg);
    }
    if (natms < nttm2 || !cell || (nw > 0 && !listttm2) || !xxx || !yyy || !zzz || !fxx || !fyy || !fzz)
        return report(MBX_ERR_ARG, "NULL or inconsistent argument");
    if (imcon < 1 || imcon > 3 || !(cell[0] > 0.0) || !(cell[4] > 0.0) || !(cell[8] > 0.0))
        return report(MBX_ERR_ARG, "bad imcon or cell");
    int dev = -1;
    unsigned char* base = scratch_for_current_device(&dev);
    if (!base) return report(MBX_ERR_CUDA, "no device scratch");
    cudaStream_t s = (cudaStream_t)stream;

    Cell cl;
    cl.imcon = imcon;
    for (int i = 0; i < 9; ++i) cl.c[i] = cell[i];
    cl.inv[0] = 1.0 / cell[0];
    cl.inv[1] = 1.0 / cell[4];
    cl.inv[2] = 1.0 / cell[8];
    {
        const double* a = cell;
        double* b = cl.rc;
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
        const double r = d != 0.0 ? 1.0 / d : 0.0;
        for (int i = 0; i < 9; ++i) b[i] *= r;
    }

    double* mono = (double*)(base + oMono);
    double* acc = (double*)(base + oAcc);
    int* totals = (int*)(base + oTotals);

    // the array keeps the previous call's contents: clear what must start at zero
    NA_CK(cudaMemsetAsync(acc, 0, MBX_NSCALARS * sizeof(double), s));

    const bool heat = vxx && vyy && vzz;
    int np = 0, nt = 0;
    if (nw >= 2) {
        ListBuilder lb;
        lb.external = true;
        lb.cap2 = lb.cap2_alloc = kCap2;
        lb.cap3 = lb.cap3_alloc = kCap3;
        lb.nw_cap = kMaxWaters;
        lb.ncell_cap = 1;
        lb.n2 = (int*)(base + oN2);
        lb.off2 = (int*)(base + oOff2);
        lb.n3 = (int*)(base + oN3);
        lb.tcnt = (int*)(base + oTcnt);
        lb.toff = (int*)(base + oToff);
        lb.l2 = (int*)(base + oL2);
        lb.l3 = (int*)(base + oL3);
        lb.flag = (int*)(base + oFlag);
        lb.of = (float4*)(base + oOf);
        lb.scan_tmp = base + oScan;
        size_t need = 0;
        NA_CK(cub::DeviceScan::ExclusiveSum(nullptr, need, lb.n2, lb.off2, nw));   // size query only
        if (need > kScanBytes) return report(MBX_ERR_CAPACITY, "scan workspace too small");
        lb.scan_bytes = kScanBytes;
        NA_CK(lb.phase1(nw, listttm2, xxx, yyy, zzz, cl, mono, totals, s));
        int th[4] = {0, 0, 0, 0};
        NA_CK(cudaMemcpyAsync(th, totals, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        if (th[2]) return report(MBX_ERR_CAPACITY, "a water has more neighbours than the fixed lists hold");
        np = th[0];
        nt = th[1];
        if (np > kMaxWaters * kCap2 || nt > kMaxTrimers)
            return report(MBX_ERR_CAPACITY, "more dimers or trimers than the fixed lists hold");
        int2* pairs = (int2*)(base + oPairs);
        int4* trip = (int4*)(base + oTrip);
        NA_CK(lb.phase2(nw, cl, mono, pairs, trip, s));
        MbpolArgs a;
        a.nw = nw;
        a.cell = cl;
        a.list = listttm2;
        a.x = xxx; a.y = yyy; a.z = zzz;
        a.vx = heat ? vxx : nullptr;
        a.vy = heat ? vyy : nullptr;
        a.vz = heat ? vzz : nullptr;
        a.mono = mono;
        a.fx = fxx; a.fy = fyy; a.fz = fzz;
        a.ae = atomic_energy;
        a.acc = acc;
        // default mixed split (2B in FP64, 3B in FP32, no hand-off lists): one persistent
        // launch, its work counters in the scratch (zeroed by launch_23); FP64: two kernels
        MixedPass mp{nullptr, nullptr, nullptr, 0.0f, 3.4e38f};
        if (fused_applies(precision, mp)) {
            int nsm = 0;
            NA_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            NA_CK(launch_23(a, pairs, np, nullptr, trip, nt, nullptr, precision, (int*)(base + oCtr), nsm, s));
        } else {
            NA_CK(launch_2b(a, pairs, np, precision, mp, s));
            NA_CK(launch_3b(a, trip, nt, precision, mp, s));
        }
    }
    if (heat && weight) NA_CK(launch_jkin(3 * nw, vxx, vyy, vzz, weight, atomic_energy, acc, s));
    double h[MBX_NSCALARS];
    NA_CK(cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, s));
    NA_CK(cudaStreamSynchronize(s));
    if (scalars) std::memcpy(scalars, h, sizeof h);
    return MBX_OK;
}
