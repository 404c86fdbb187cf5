// C ABI of libmbx: contexts, host/device entry points and the per-call drop-ins.
#include "../../include/mbx.h"
#include "mbx_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

using namespace mbx;

struct mbx_context {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    ListBuilder lb;
    int nw_cap = 0, natms_cap = 0;
    double* mono = nullptr;       // 9 per water
    int* list = nullptr;          // device copy of listttm2 (host entry point)
    double* atoms = nullptr;      // host entry point staging: x y z vx vy vz m f(3) ae  (11 * natms)
    double* ae_scratch = nullptr; // per-atom energy when the caller passes none
    double* acc = nullptr;        // MBX_NSCALARS accumulators
    int* totals = nullptr;        // device list totals
    int* totals_h = nullptr;      // pinned
    double* acc_h = nullptr;      // pinned
    int2* pairs = nullptr;
    long pairs_cap = 0;
    int4* trip = nullptr;
    long trip_cap = 0;
    int2* hard2 = nullptr;          // mixed path: clusters handed to the FP64 kernels
    int4* hard3 = nullptr;
    int* hard_count = nullptr;      // device [2]
    // mixed-path defaults: the 2B term in FP64 (its FP32 gradient is a small difference of
    // large partials), the 3B term entirely in shifted FP32
    float limit2 = 0.0f, limit3 = 3.4e38f;
    // 2B and 3B in one persistent launch (launch_23) where it applies; 0 = separate kernels
    int fused = 1;
    int fused_split = 0;            // dimer warps of the 12 per block (0: the default, 4)
    // the whole step (mbx_water_step*): the MB-pol terms on a second stream, beside the
    // electrostatics' FP32 CG sweeps (mbx_set_overlap)
    int overlap = 0;
    int overlap_split = 0;          // dimer warps of the 8-warp block (0: 4)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the whole step: the 1-body and dispersion terms on a third stream beside the
    // electrostatics' setup and solve (mbx_set_overlap_terms), their scalars in side_acc
    int overlap_terms = 0;
    cudaStream_t side2 = nullptr;
    cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr;
    double* side_acc = nullptr;     // device [28]: 1-body 14, dispersion 14
    double* side_acc_h = nullptr;   // pinned copy
    int nsm = 0;                    // SMs of the device (the persistent grid)
    int* fuse_ctr = nullptr;        // device [2]: work counters of the persistent kernel
    double* part2 = nullptr;        // split FP64 dimers: per-chunk partial sums (pairs_cap dimers)
    int* done2 = nullptr;
    long hard_last[2] = {0, 0};
    long npairs = 0, ntrip = 0;
    // batch-API staging
    double* batch = nullptr;
    size_t batch_bytes = 0;
    // optional per-phase timing on the context's stream (mbx_set_profiling)
    int profiling = 0;
    cudaEvent_t ev[8] = {nullptr};
    float phase_ms[4] = {0, 0, 0, 0};  // lists, 2B, 3B, heat/jkin
    long launches = 0;                 // kernel launches issued by the last evaluation
    // many boxes in one evaluation (mbx_mbpol_multi*): buffers, and the step captured as
    // a CUDA graph that is replayed while its key (arrays, layout, precision) is unchanged
    MultiBoxes multi;
    int use_graphs = 1;
    cudaGraphExec_t mexec = nullptr;
    const void* mkey[15] = {nullptr};
    long mkey_gen = -1;
    int mkey_prec = -1;
    float mkey_lim[2] = {0, 0};
    cudaStream_t mkey_stream = nullptr;
    Cell* cells_h = nullptr;           // pinned, one per box
    double* mout_h = nullptr;          // pinned: per-box MB-pol and 1-body scalars
    int* mint_h = nullptr;             // pinned: totals[2], flag, hand-off counts[2]
    int mbox_cap = 0;
    long graph_replays = 0;
    double* hstage = nullptr;          // pinned host staging of per-atom results (4 * natms)
    size_t hstage_cap = 0;
    int* ints = nullptr;               // mbx_water_forces staging: listttm2, listang, ltype, molecule
    size_t ints_cap = 0;
    DispState disp;                    // dispersion tables and Verlet list
    PolarState polar;                  // TTM4-F electrostatics
    double* polar_stage = nullptr;     // host entry point staging (24 * sites)
    size_t polar_stage_cap = 0;
    double* step_stage = nullptr;      // mbx_water_step staging
    size_t step_stage_cap = 0;
    int* step_ints = nullptr;          // standard-layout water and angle lists
    int step_nw = -1;
    std::vector<int> disp_types_h, disp_mol_h;   // inputs of the host entry point's list
    // mbx_water_step_multi: worker lanes (child contexts, each with its own stream and
    // buffers, driven by one host thread per call) and the dispersion setup they replay
    std::vector<mbx_context*> lane;
    int nlanes = 8;
    std::vector<double> disp_prm_h;
    int disp_ntypes = 0, disp_mxgrid = 0;
    double disp_rcut = 0.0, disp_delr = 0.0;
    long disp_gen = 0;       // setups made on this context
    long disp_gen_seen = -1; // (on a lane) the parent's setup it holds
    // path-integral bead coupling: device copies of the normal-mode matrices for pimd_P
    // beads (nmode_to_cart then cart_to_nmode, P x P each) and two accumulators
    double* pimd_mat = nullptr;
    double* pimd_acc = nullptr;
    int pimd_P = 0, pimd_lang = -1;
    char err[512] = {0};
};

namespace {

int fail(mbx_context* c, int code, const char* fmt, ...) {
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(c->err, sizeof c->err, fmt, ap);
        va_end(ap);
    }
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(ctx, MBX_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                      \
    } while (0)

int make_cell(mbx_context* ctx, int imcon, const double* cell, Cell& cl) {
    if (!cell) return fail(ctx, MBX_ERR_ARG, "cell is NULL");
    if (imcon < 1 || imcon > 3) return fail(ctx, MBX_ERR_ARG, "imcon %d not supported (1, 2 or 3)", imcon);
    cl.imcon = imcon;
    for (int i = 0; i < 9; ++i) cl.c[i] = cell[i];
    cl.inv[0] = 1.0 / cell[0];
    cl.inv[1] = 1.0 / cell[4];
    cl.inv[2] = 1.0 / cell[8];
    // invert (SOURCE/invert.f), used for imcon 3
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
    const double r = std::fabs(d) > 0.0 ? 1.0 / d : 0.0;
    for (int i = 0; i < 9; ++i) b[i] *= r;
    if (!(cell[0] > 0.0) || !(cell[4] > 0.0) || !(cell[8] > 0.0))
        return fail(ctx, MBX_ERR_ARG, "cell diagonal must be positive");
    return MBX_OK;
}

int reserve_water(mbx_context* ctx, int nw, int natms) {
    // a capacity is zeroed before its buffers are replaced, so a failed allocation can
    // never leave a capacity that promises memory which is not there
    if (nw > ctx->nw_cap) {
        ctx->nw_cap = 0;
        if (ctx->mono) cudaFree(ctx->mono);
        if (ctx->list) cudaFree(ctx->list);
        ctx->mono = nullptr;
        ctx->list = nullptr;
        CK(cudaMalloc(&ctx->mono, 9 * (size_t)nw * sizeof(double)));
        CK(cudaMalloc(&ctx->list, 3 * (size_t)nw * sizeof(int)));
        ctx->nw_cap = nw;
    }
    if (natms > ctx->natms_cap) {
        ctx->natms_cap = 0;
        if (ctx->atoms) cudaFree(ctx->atoms);
        if (ctx->ae_scratch) cudaFree(ctx->ae_scratch);
        ctx->atoms = ctx->ae_scratch = nullptr;
        CK(cudaMalloc(&ctx->atoms, 11 * (size_t)natms * sizeof(double)));
        CK(cudaMalloc(&ctx->ae_scratch, (size_t)natms * sizeof(double)));
        ctx->natms_cap = natms;
    }
    return MBX_OK;
}

// Pinned host staging for copying per-atom results back (grown as needed).
double* host_stage(mbx_context* ctx, size_t n) {
    if (n > ctx->hstage_cap) {
        if (ctx->hstage) cudaFreeHost(ctx->hstage);
        ctx->hstage = nullptr;
        ctx->hstage_cap = 0;
        if (cudaMallocHost(&ctx->hstage, n * sizeof(double)) != cudaSuccess) return nullptr;
        ctx->hstage_cap = n;
    }
    return ctx->hstage;
}

// The whole MB-pol evaluation on device arrays.
int finish_mbpol(mbx_context* ctx, int precision, int nw, double* scalars);

// The 1-body-free MB-pol terms on ctx->stream.  wait: read the scalars back (the stream is
// synchronised); otherwise the work is only enqueued and finish_mbpol reads them later, and
// jkin (which reads every term's per-atom energy) is left to the caller.  shared_sm: the
// fused kernel in its 8-warp form, to share the SMs with other work.
int run_mbpol(mbx_context* ctx, int precision, const Cell& cl, int nw, const int* list_dev, int natms,
              const double* x, const double* y, const double* z, double* fx, double* fy, double* fz,
              const double* vx, const double* vy, const double* vz, const double* mass, double* ae,
              double* scalars, bool wait = true, bool shared_sm = false) {
    if (precision != MBX_FP64 && precision != MBX_MIXED)
        return fail(ctx, MBX_ERR_ARG, "precision must be MBX_FP64 or MBX_MIXED");
    if (nw < 0 || natms < 3 * nw) return fail(ctx, MBX_ERR_ARG, "bad sizes nw=%d natms=%d", nw, natms);
    if (!x || !y || !z || !fx || !fy || !fz) return fail(ctx, MBX_ERR_ARG, "NULL position/force array");
    const bool heat = vx && vy && vz;
    int rc = reserve_water(ctx, std::max(nw, 1), std::max(natms, 1));
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    CK(cudaMemsetAsync(ctx->acc, 0, MBX_NSCALARS * sizeof(double), s));
    double* ae_use = ae;
    if (!ae_use && heat && mass) {
        ae_use = ctx->ae_scratch;
        CK(cudaMemsetAsync(ae_use, 0, (size_t)natms * sizeof(double), s));
    }
    ctx->npairs = ctx->ntrip = 0;
    ctx->launches = 0;
    if (ctx->profiling) CK(cudaEventRecord(ctx->ev[0], s));
    if (nw >= 2) {
        // lists: count, read totals, grow capacities if needed, fill
        for (int attempt = 0;; ++attempt) {
            CK(ctx->lb.phase1(nw, list_dev, x, y, z, cl, ctx->mono, ctx->totals, s));
            CK(cudaMemcpyAsync(ctx->totals_h, ctx->totals, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (!ctx->totals_h[2]) break;
            if (attempt >= 6 || ctx->lb.cap2 >= nw + 8)
                return fail(ctx, MBX_ERR_CAPACITY, "neighbour list capacity exceeded");
            ctx->lb.cap2 = std::min(2 * ctx->lb.cap2, nw + 8);
            ctx->lb.cap3 = std::min(2 * ctx->lb.cap3, nw + 8);
        }
        const long np = ctx->totals_h[0], nt = ctx->totals_h[1];
        if (np > ctx->pairs_cap) {
            if (ctx->pairs) cudaFree(ctx->pairs);
            if (ctx->hard2) cudaFree(ctx->hard2);
            if (ctx->part2) cudaFree(ctx->part2);
            if (ctx->done2) cudaFree(ctx->done2);
            ctx->pairs_cap = 0;
            ctx->pairs = nullptr;
            ctx->hard2 = nullptr;
            ctx->part2 = nullptr;
            ctx->done2 = nullptr;
            const long cap = np + np / 4 + 64;
            CK(cudaMalloc(&ctx->pairs, cap * sizeof(int2)));
            CK(cudaMalloc(&ctx->hard2, cap * sizeof(int2)));
            CK(cudaMalloc(&ctx->part2, cap * dimer_parts() * 32 * sizeof(double)));
            CK(cudaMalloc(&ctx->done2, cap * sizeof(int)));
            ctx->pairs_cap = cap;
        }
        if (nt > ctx->trip_cap) {
            if (ctx->trip) cudaFree(ctx->trip);
            if (ctx->hard3) cudaFree(ctx->hard3);
            ctx->trip_cap = 0;
            ctx->trip = nullptr;
            ctx->hard3 = nullptr;
            const long cap = nt + nt / 4 + 64;
            CK(cudaMalloc(&ctx->trip, cap * sizeof(int4)));
            CK(cudaMalloc(&ctx->hard3, cap * sizeof(int4)));
            ctx->trip_cap = cap;
        }
        CK(ctx->lb.phase2(nw, cl, ctx->mono, ctx->pairs, ctx->trip, s));
        if (ctx->profiling) CK(cudaEventRecord(ctx->ev[1], s));
        ctx->launches += ctx->lb.launches_last;
        ctx->npairs = np;
        ctx->ntrip = nt;
        MbpolArgs a;
        a.nw = nw;
        a.cell = cl;
        a.list = list_dev;
        a.x = x; a.y = y; a.z = z;
        a.vx = heat ? vx : nullptr;
        a.vy = heat ? vy : nullptr;
        a.vz = heat ? vz : nullptr;
        a.mono = ctx->mono;
        a.fx = fx; a.fy = fy; a.fz = fz;
        a.ae = ae_use;
        a.acc = ctx->acc;
        MixedPass mp{ctx->hard2, ctx->hard3, ctx->hard_count, ctx->limit2, ctx->limit3};
        if (ctx->fused && fused_applies(precision, mp)) {
            CK(launch_23(a, ctx->pairs, (int)np, nullptr, ctx->trip, (int)nt, nullptr, precision, ctx->fuse_ctr,
                         ctx->nsm, s, ctx->part2, ctx->done2, ctx->pairs_cap,
                         shared_sm ? ctx->overlap_split : ctx->fused_split, shared_sm));
            if (ctx->profiling) {
                CK(cudaEventRecord(ctx->ev[2], s));
                CK(cudaEventRecord(ctx->ev[3], s));
            }
            ctx->launches += 1;
        } else {
            if (precision == MBX_MIXED) CK(cudaMemsetAsync(ctx->hard_count, 0, 2 * sizeof(int), s));
            CK(launch_2b(a, ctx->pairs, (int)np, precision, mp, s));
            if (ctx->profiling) CK(cudaEventRecord(ctx->ev[2], s));
            CK(launch_3b(a, ctx->trip, (int)nt, precision, mp, s));
            if (ctx->profiling) CK(cudaEventRecord(ctx->ev[3], s));
            const int p2 = (precision == MBX_MIXED && ctx->limit2 > 0.f) ? 2 : 1;
            const int p3 = (precision == MBX_MIXED && ctx->limit3 > 0.f && ctx->limit3 < 3.0e38f) ? 2 : 1;
            ctx->launches += p2 * (np > 0) + p3 * (nt > 0);
        }
    } else if (ctx->profiling) {
        for (int q = 1; q < 4; ++q) CK(cudaEventRecord(ctx->ev[q], s));
    }
    if (heat && mass && wait) {
        CK(launch_jkin(3 * nw, vx, vy, vz, mass, ae_use, ctx->acc, s));
        ctx->launches += nw > 0;
    }
    if (ctx->profiling) CK(cudaEventRecord(ctx->ev[4], s));
    if (!wait) return MBX_OK;
    return finish_mbpol(ctx, precision, nw, scalars);
}

// The scalars of run_mbpol (its stream is the context's stream when it was enqueued).
int finish_mbpol(mbx_context* ctx, int precision, int nw, double* scalars) {
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(ctx->acc_h, ctx->acc, MBX_NSCALARS * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (precision == MBX_MIXED && nw >= 2)
        CK(cudaMemcpyAsync(ctx->totals_h + 4, ctx->hard_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ctx->hard_last[0] = (precision == MBX_MIXED && nw >= 2) ? ctx->totals_h[4] : 0;
    ctx->hard_last[1] = (precision == MBX_MIXED && nw >= 2) ? ctx->totals_h[5] : 0;
    if (scalars) std::memcpy(scalars, ctx->acc_h, MBX_NSCALARS * sizeof(double));
    if (ctx->profiling)
        for (int q = 0; q < 4; ++q) CK(cudaEventElapsedTime(&ctx->phase_ms[q], ctx->ev[q], ctx->ev[q + 1]));
    return MBX_OK;
}

// One multi-box step on device arrays: the cell copy, every kernel and the copies of the
// per-box scalars back to pinned host memory are enqueued (or replayed as one graph),
// then the host waits once.  A list that outgrew its capacity makes the step a no-op on
// the device; the host then grows the lists and repeats it.
int run_multi(mbx_context* ctx, int precision, int nbox, const int* nw_box, const double* x, const double* y,
              const double* z, double* fx, double* fy, double* fz, const double* vx, const double* vy,
              const double* vz, const double* mass, double* ae, double* scalars) {
    cudaStream_t s = ctx->stream;
    MultiBoxes& m = ctx->multi;
    const bool need_hard =
        precision == MBX_MIXED && (ctx->limit2 > 0.f || (ctx->limit3 > 0.f && ctx->limit3 < 3.0e38f));
    const bool heat = vx && vy && vz;
    MixedPass lim{nullptr, nullptr, nullptr, ctx->limit2, ctx->limit3};
    if (ctx->profiling) CK(cudaEventRecord(ctx->ev[0], s));
    for (int attempt = 0;; ++attempt) {
        CK(m.setup(nbox, nw_box, need_hard, s));
        auto enqueue_all = [&]() -> cudaError_t {
            cudaError_t e;
            if ((e = cudaMemcpyAsync(m.cells, ctx->cells_h, nbox * sizeof(Cell), cudaMemcpyHostToDevice, s)))
                return e;
            if ((e = m.enqueue(precision, lim, ctx->fused != 0, x, y, z, fx, fy, fz, heat ? vx : nullptr,
                               heat ? vy : nullptr, heat ? vz : nullptr, heat ? mass : nullptr, ae, s)))
                return e;
            if ((e = cudaMemcpyAsync(ctx->mout_h, m.acc_box, (size_t)nbox * S_NSLOTS * sizeof(double),
                                     cudaMemcpyDeviceToHost, s)))
                return e;
            if ((e = cudaMemcpyAsync(ctx->mout_h + (size_t)nbox * S_NSLOTS, m.pes_box, (size_t)nbox * 14 * sizeof(double),
                                     cudaMemcpyDeviceToHost, s)))
                return e;
            if ((e = cudaMemcpyAsync(ctx->mint_h, m.totals, 2 * sizeof(int), cudaMemcpyDeviceToHost, s))) return e;
            if ((e = cudaMemcpyAsync(ctx->mint_h + 2, m.flag, sizeof(int), cudaMemcpyDeviceToHost, s))) return e;
            return cudaMemcpyAsync(ctx->mint_h + 3, m.hard_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
        };
        const void* key[15] = {x, y, z, fx, fy, fz, heat ? vx : nullptr, heat ? vy : nullptr, heat ? vz : nullptr,
                               heat ? mass : nullptr, ae, (const void*)(long)nbox, ctx->cells_h, ctx->mout_h,
                               ctx->mint_h};
        bool launched = false;
        if (ctx->use_graphs) {
            const bool same = ctx->mexec && m.gen == ctx->mkey_gen && precision + 2 * ctx->fused == ctx->mkey_prec &&
                              ctx->mkey_lim[0] == ctx->limit2 && ctx->mkey_lim[1] == ctx->limit3 &&
                              ctx->mkey_stream == s && std::memcmp(key, ctx->mkey, sizeof key) == 0;
            if (!same) {
                if (ctx->mexec) cudaGraphExecDestroy(ctx->mexec);
                ctx->mexec = nullptr;
                cudaGraph_t g = nullptr;
                if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                    const cudaError_t e1 = enqueue_all();
                    const cudaError_t e2 = cudaStreamEndCapture(s, &g);
                    if (e1 == cudaSuccess && e2 == cudaSuccess && g &&
                        cudaGraphInstantiate(&ctx->mexec, g, 0) == cudaSuccess) {
                        std::memcpy(ctx->mkey, key, sizeof key);
                        ctx->mkey_gen = m.gen;
                        ctx->mkey_prec = precision + 2 * ctx->fused;
                        ctx->mkey_lim[0] = ctx->limit2;
                        ctx->mkey_lim[1] = ctx->limit3;
                        ctx->mkey_stream = s;
                    } else {
                        ctx->mexec = nullptr;
                    }
                    if (g) cudaGraphDestroy(g);
                }
                cudaGetLastError();   // a failed capture leaves no sticky error; run uncaptured below
            }
            if (ctx->mexec) {
                CK(cudaGraphLaunch(ctx->mexec, s));
                ++ctx->graph_replays;
                launched = true;
            }
        }
        if (!launched) CK(enqueue_all());
        CK(cudaStreamSynchronize(s));
        if (!ctx->mint_h[2]) break;
        if (attempt >= 6 || m.cap2 > 4096) return fail(ctx, MBX_ERR_CAPACITY, "multi-box list capacity exceeded");
        // grow what overflowed and repeat the step (nothing was accumulated)
        if (ctx->mint_h[2] & 1) {
            m.cap2 *= 2;
            m.cap3 *= 2;
        }
        if (ctx->mint_h[2] & 2) m.trip_per_water *= 2;
        m.release();
    }
    if (ctx->profiling) {
        CK(cudaEventRecord(ctx->ev[1], s));
        CK(cudaEventSynchronize(ctx->ev[1]));
        CK(cudaEventElapsedTime(&ctx->phase_ms[0], ctx->ev[0], ctx->ev[1]));
        ctx->phase_ms[1] = ctx->phase_ms[2] = ctx->phase_ms[3] = 0.f;
    }
    ctx->npairs = ctx->mint_h[0];
    ctx->ntrip = ctx->mint_h[1];
    ctx->launches = m.launches;
    ctx->hard_last[0] = need_hard ? ctx->mint_h[3] : 0;
    ctx->hard_last[1] = need_hard ? ctx->mint_h[4] : 0;
    if (scalars)
        for (int b = 0; b < nbox; ++b) {
            std::memcpy(scalars + (size_t)b * MBX_NBOXSCALARS, ctx->mout_h + (size_t)b * S_NSLOTS,
                        S_NSLOTS * sizeof(double));
            std::memcpy(scalars + (size_t)b * MBX_NBOXSCALARS + MBX_NSCALARS,
                        ctx->mout_h + (size_t)nbox * S_NSLOTS + (size_t)b * 14, 14 * sizeof(double));
        }
    return MBX_OK;
}

// Validate the box layout and stage the cells (pinned) for run_multi.
int prepare_multi(mbx_context* ctx, int precision, int imcon, int nbox, const int* nw_box, const double* cells,
                  long* natms_out) {
    if (precision != MBX_FP64 && precision != MBX_MIXED)
        return fail(ctx, MBX_ERR_ARG, "precision must be MBX_FP64 or MBX_MIXED");
    if (nbox < 1 || !nw_box || !cells) return fail(ctx, MBX_ERR_ARG, "nbox must be >= 1 with nw_box and cells");
    long nw = 0;
    for (int b = 0; b < nbox; ++b) {
        if (nw_box[b] < 0) return fail(ctx, MBX_ERR_ARG, "nw_box[%d] = %d", b, nw_box[b]);
        nw += nw_box[b];
    }
    if (nw > (1L << 26)) return fail(ctx, MBX_ERR_ARG, "too many waters (%ld)", nw);
    CK(cudaSetDevice(ctx->device));
    if (nbox > ctx->mbox_cap) {
        if (ctx->cells_h) cudaFreeHost(ctx->cells_h);
        if (ctx->mout_h) cudaFreeHost(ctx->mout_h);
        ctx->mbox_cap = 0;
        ctx->cells_h = nullptr;
        ctx->mout_h = nullptr;
        CK(cudaMallocHost(&ctx->cells_h, nbox * sizeof(Cell)));
        CK(cudaMallocHost(&ctx->mout_h, (size_t)nbox * (S_NSLOTS + 14) * sizeof(double)));
        ctx->mbox_cap = nbox;
    }
    if (!ctx->mint_h) CK(cudaMallocHost(&ctx->mint_h, 8 * sizeof(int)));
    for (int b = 0; b < nbox; ++b) {
        const int rc = make_cell(ctx, imcon, cells + 9 * (size_t)b, ctx->cells_h[b]);
        if (rc) return rc;
    }
    *natms_out = 4 * nw;
    return MBX_OK;
}

int check_device(mbx_context* ctx, int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0)
        return fail(ctx, MBX_ERR_NO_DEVICE, "CUDA device %d not available", device);
    cudaDeviceProp p;
    CK(cudaGetDeviceProperties(&p, device));
    if (p.major != 10 || p.minor != 3)
        return fail(ctx, MBX_ERR_NO_DEVICE, "device %d is sm_%d%d; libmbx is built for sm_103a only", device,
                    p.major, p.minor);
    return MBX_OK;
}

}  // namespace

extern "C" int mbx_create(mbx_context** out, int device) {
    if (!out) return MBX_ERR_ARG;
    *out = nullptr;
    mbx_context* ctx = new mbx_context();
    int rc = check_device(ctx, device);
    if (rc) {
        std::fprintf(stderr, "mbx_create: %s\n", ctx->err);
        delete ctx;
        return rc;
    }
    ctx->device = device;
    auto init = [&]() -> int {
        CK(cudaSetDevice(device));
        // the fused cluster kernels call the generated polynomial functions, whose
        // frames need up to ~2.3 KB of stack per thread (FP64); reserve it up front
        size_t stack = 0;
        CK(cudaDeviceGetLimit(&stack, cudaLimitStackSize));
        if (stack < 4096) CK(cudaDeviceSetLimit(cudaLimitStackSize, 4096));
        CK(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
        ctx->stream = ctx->own_stream;
        CK(cudaMalloc(&ctx->acc, MBX_NSCALARS * sizeof(double)));
        CK(cudaMalloc(&ctx->totals, 4 * sizeof(int)));
        CK(cudaMalloc(&ctx->hard_count, 2 * sizeof(int)));
        CK(cudaMalloc(&ctx->fuse_ctr, 2 * sizeof(int)));
        CK(cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device));
        CK(cudaMallocHost(&ctx->totals_h, 8 * sizeof(int)));
        CK(cudaMallocHost(&ctx->acc_h, MBX_NSCALARS * sizeof(double)));
        return MBX_OK;
    };
    rc = init();
    if (rc) {
        std::fprintf(stderr, "mbx_create: %s\n", ctx->err);
        mbx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return MBX_OK;
}

extern "C" void mbx_destroy(mbx_context* ctx) {
    if (!ctx) return;
    for (mbx_context* c : ctx->lane) mbx_destroy(c);
    ctx->lane.clear();
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    void* dev[] = {ctx->mono, ctx->list, ctx->atoms, ctx->ae_scratch, ctx->acc, ctx->totals, ctx->pairs, ctx->trip,
                   ctx->batch, ctx->hard2, ctx->hard3, ctx->hard_count, ctx->fuse_ctr, ctx->part2, ctx->done2,
                   ctx->ints, ctx->polar_stage, ctx->step_stage, ctx->step_ints, ctx->pimd_mat, ctx->pimd_acc};
    for (void* p : dev)
        if (p) cudaFree(p);
    if (ctx->totals_h) cudaFreeHost(ctx->totals_h);
    if (ctx->acc_h) cudaFreeHost(ctx->acc_h);
    if (ctx->mexec) cudaGraphExecDestroy(ctx->mexec);
    if (ctx->cells_h) cudaFreeHost(ctx->cells_h);
    if (ctx->mout_h) cudaFreeHost(ctx->mout_h);
    if (ctx->mint_h) cudaFreeHost(ctx->mint_h);
    if (ctx->hstage) cudaFreeHost(ctx->hstage);
    ctx->multi.release();
    ctx->disp.release();
    ctx->polar.release();
    ctx->lb.release();
    for (cudaEvent_t e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->side2) {
        cudaStreamSynchronize(ctx->side2);
        cudaStreamDestroy(ctx->side2);
    }
    if (ctx->ev_fork2) cudaEventDestroy(ctx->ev_fork2);
    if (ctx->ev_join2) cudaEventDestroy(ctx->ev_join2);
    if (ctx->side_acc) cudaFree(ctx->side_acc);
    if (ctx->side_acc_h) cudaFreeHost(ctx->side_acc_h);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

extern "C" int mbx_set_profiling(mbx_context* ctx, int on) {
    if (!ctx) return MBX_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    if (on && !ctx->ev[0])
        for (cudaEvent_t& e : ctx->ev) CK(cudaEventCreate(&e));
    ctx->profiling = on ? 1 : 0;
    return MBX_OK;
}

extern "C" int mbx_last_timings(mbx_context* ctx, double* ms, long* counts) {
    if (!ctx) return MBX_ERR_ARG;
    if (ms)
        for (int q = 0; q < 4; ++q) ms[q] = ctx->profiling ? ctx->phase_ms[q] : -1.0;
    if (counts) {
        counts[0] = ctx->npairs;
        counts[1] = ctx->ntrip;
        counts[2] = ctx->launches;
        counts[3] = ctx->hard_last[0];
        counts[4] = ctx->hard_last[1];
    }
    return MBX_OK;
}

extern "C" int mbx_set_mixed_limits(mbx_context* ctx, double limit2b, double limit3b) {
    if (!ctx) return MBX_ERR_ARG;
    if (!(limit2b >= 0.0) || !(limit3b >= 0.0)) return fail(ctx, MBX_ERR_ARG, "limits must be >= 0");
    ctx->limit2 = (float)std::min(limit2b, 3.4e38);
    ctx->limit3 = (float)std::min(limit3b, 3.4e38);
    return MBX_OK;
}

extern "C" const char* mbx_error(const mbx_context* ctx) { return ctx ? ctx->err : "no context"; }

extern "C" int mbx_set_stream(mbx_context* ctx, void* stream) {
    if (!ctx) return MBX_ERR_ARG;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return MBX_OK;
}

extern "C" int mbx_mbpol_forces_device(mbx_context* ctx, int precision, int imcon, const double* cell, int nttm2,
                                       const int* listttm2, int natms, const double* xxx, const double* yyy,
                                       const double* zzz, double* fxx, double* fyy, double* fzz, const double* vxx,
                                       const double* vyy, const double* vzz, const double* weight,
                                       double* atomic_energy, double* scalars) {
    if (!ctx) return MBX_ERR_ARG;
    if (nttm2 < 0 || nttm2 % 3) return fail(ctx, MBX_ERR_ARG, "nttm2 must be a multiple of 3");
    if (nttm2 > 0 && !listttm2) return fail(ctx, MBX_ERR_ARG, "listttm2 is NULL");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    return run_mbpol(ctx, precision, cl, nttm2 / 3, listttm2, natms, xxx, yyy, zzz, fxx, fyy, fzz, vxx, vyy, vzz,
                     weight, atomic_energy, scalars);
}

extern "C" int mbx_mbpol_forces(mbx_context* ctx, int precision, int imcon, const double* cell, int nttm2,
                                const int* listttm2, int natms, const double* xxx, const double* yyy,
                                const double* zzz, double* fxx, double* fyy, double* fzz, double* engsrp,
                                double* virsrp, double* stress, const double* vxx, const double* vyy,
                                const double* vzz, const double* weight, double* atomic_energy, double* scalars) {
    if (!ctx) return MBX_ERR_ARG;
    if (nttm2 < 0 || nttm2 % 3) return fail(ctx, MBX_ERR_ARG, "nttm2 must be a multiple of 3");
    if (!xxx || !yyy || !zzz || !fxx || !fyy || !fzz || !engsrp || !virsrp || !stress)
        return fail(ctx, MBX_ERR_ARG, "NULL argument");
    if (nttm2 > 0 && !listttm2) return fail(ctx, MBX_ERR_ARG, "listttm2 is NULL");
    for (int t = 0; t < nttm2; ++t)
        if (listttm2[t] < 1 || listttm2[t] > natms || (t % 3 && listttm2[t] != listttm2[t - t % 3] + t % 3))
            return fail(ctx, MBX_ERR_ARG, "listttm2[%d]=%d: water atoms must be 1-based, O,H1,H2 consecutive", t,
                        listttm2[t]);
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    const int nw = nttm2 / 3;
    rc = reserve_water(ctx, std::max(nw, 1), std::max(natms, 1));
    if (rc) return rc;
    const bool heat = vxx && vyy && vzz && weight;
    cudaStream_t s = ctx->stream;
    const size_t nb = (size_t)natms * sizeof(double);
    double* d = ctx->atoms;
    double *dx = d, *dy = d + natms, *dz = d + 2 * (size_t)natms;
    double *dvx = d + 3 * (size_t)natms, *dvy = d + 4 * (size_t)natms, *dvz = d + 5 * (size_t)natms;
    double* dm = d + 6 * (size_t)natms;
    double *dfx = d + 7 * (size_t)natms, *dfy = d + 8 * (size_t)natms, *dfz = d + 9 * (size_t)natms;
    double* dae = d + 10 * (size_t)natms;
    if (nttm2) CK(cudaMemcpyAsync(ctx->list, listttm2, nttm2 * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
    if (heat) {
        CK(cudaMemcpyAsync(dvx, vxx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvy, vyy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvz, vzz, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dm, weight, nb, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemsetAsync(dfx, 0, 3 * nb, s));
    if (atomic_energy) CK(cudaMemsetAsync(dae, 0, nb, s));
    double sc[MBX_NSCALARS];
    rc = run_mbpol(ctx, precision, cl, nw, ctx->list, natms, dx, dy, dz, dfx, dfy, dfz, heat ? dvx : nullptr,
                   heat ? dvy : nullptr, heat ? dvz : nullptr, heat ? dm : nullptr, atomic_energy ? dae : nullptr,
                   sc);
    if (rc) return rc;
    // bring the per-atom results back and accumulate into the caller's arrays
    double* h = host_stage(ctx, 4 * (size_t)natms + 1);
    if (!h) return fail(ctx, MBX_ERR_CUDA, "pinned host staging allocation failed");
    CK(cudaMemcpyAsync(h, dfx, 3 * nb, cudaMemcpyDeviceToHost, s));
    if (atomic_energy) CK(cudaMemcpyAsync(h + 3 * (size_t)natms, dae, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < natms; ++i) {
        fxx[i] += h[i];
        fyy[i] += h[natms + i];
        fzz[i] += h[2 * (size_t)natms + i];
        if (atomic_energy) atomic_energy[i] += h[3 * (size_t)natms + i];
    }
    *engsrp += sc[MBX_S_ENG2] + sc[MBX_S_ENG3];
    *virsrp += sc[MBX_S_VIR];
    for (int q = 0; q < 9; ++q) stress[q] += sc[MBX_S_STRESS + q];
    if (scalars) std::memcpy(scalars, sc, sizeof sc);
    return MBX_OK;
}

extern "C" int mbx_disp_setup(mbx_context* ctx, int ntypes, const double* prm, double rcut, double delr,
                              int mxgrid) {
    if (!ctx) return MBX_ERR_ARG;
    if (ntypes < 1 || ntypes > 15 || !prm || !(rcut > 0.0) || !(delr >= 0.0) || (mxgrid != 0 && mxgrid < 8))
        return fail(ctx, MBX_ERR_ARG, "bad dispersion parameters (ntypes 1..15, rcut > 0, delr >= 0)");
    CK(cudaSetDevice(ctx->device));
    CK(ctx->disp.setup(ntypes, prm, rcut, delr, mxgrid));
    ctx->disp_types_h.clear();
    ctx->disp_prm_h.assign(prm, prm + 4 * (size_t)(ntypes * (ntypes + 1) / 2));   // replayed on the lanes
    ctx->disp_ntypes = ntypes;
    ctx->disp_rcut = rcut;
    ctx->disp_delr = delr;
    ctx->disp_mxgrid = mxgrid;
    ++ctx->disp_gen;
    return MBX_OK;
}

// The dispersion on device arrays; fp32: the mixed form (k_disp_forces32), used by the
// mixed whole evaluation.
static int disp_forces_dev(mbx_context* ctx, int imcon, const double* cell, int natms, const int* ltype,
                           const int* molecule, const double* xxx, const double* yyy, const double* zzz, double* fxx,
                           double* fyy, double* fzz, const double* vxx, const double* vyy, const double* vzz,
                           double* atomic_energy, double* out, bool fp32) {
    if (!ctx) return MBX_ERR_ARG;
    if (!ctx->disp.vvv) return fail(ctx, MBX_ERR_ARG, "mbx_disp_setup has not been called");
    if (natms < 0 || (natms > 0 && (!ltype || !molecule || !xxx || !yyy || !zzz || !fxx || !fyy || !fzz)))
        return fail(ctx, MBX_ERR_ARG, "bad argument");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const bool heat = vxx && vyy && vzz;
    CK(cudaMemsetAsync(ctx->acc, 0, 14 * sizeof(double), s));
    bool rebuilt = false;
    if (natms > 0) {
        const cudaError_t e = ctx->disp.forces(cl, natms, ltype, molecule, xxx, yyy, zzz, fxx, fyy, fzz,
                                               heat ? vxx : nullptr, heat ? vyy : nullptr, heat ? vzz : nullptr,
                                               atomic_energy, ctx->acc, ctx->totals_h, s, &rebuilt, fp32);
        if (e == cudaErrorInvalidValue) return fail(ctx, MBX_ERR_CAPACITY, "dispersion list capacity exceeded");
        CK(e);
    }
    CK(cudaMemcpyAsync(ctx->acc_h, ctx->acc, 14 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (out) std::memcpy(out, ctx->acc_h, 14 * sizeof(double));
    return MBX_OK;
}

extern "C" int mbx_disp_forces_device(mbx_context* ctx, int imcon, const double* cell, int natms, const int* ltype,
                                      const int* molecule, const double* xxx, const double* yyy, const double* zzz,
                                      double* fxx, double* fyy, double* fzz, const double* vxx, const double* vyy,
                                      const double* vzz, double* atomic_energy, double* out) {
    return disp_forces_dev(ctx, imcon, cell, natms, ltype, molecule, xxx, yyy, zzz, fxx, fyy, fzz, vxx, vyy, vzz,
                           atomic_energy, out, false);
}

extern "C" int mbx_disp_forces(mbx_context* ctx, int imcon, const double* cell, int natms, const int* ltype,
                               const int* molecule, const double* xxx, const double* yyy, const double* zzz,
                               double* fxx, double* fyy, double* fzz, double* engsrp, double* virsrp,
                               double* stress, const double* vxx, const double* vyy, const double* vzz,
                               double* atomic_energy, double* jpot) {
    if (!ctx) return MBX_ERR_ARG;
    if (natms < 0 || !ltype || !molecule || !xxx || !yyy || !zzz || !fxx || !fyy || !fzz || !engsrp || !virsrp ||
        !stress)
        return fail(ctx, MBX_ERR_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    int rc = reserve_water(ctx, std::max(natms / 3, 1), std::max(natms, 1));
    if (rc) return rc;
    const bool heat = vxx && vyy && vzz;
    cudaStream_t s = ctx->stream;
    const size_t nb = (size_t)natms * sizeof(double);
    double* d = ctx->atoms;
    double *dx = d, *dy = d + natms, *dz = d + 2 * (size_t)natms;
    double *dvx = d + 3 * (size_t)natms, *dvy = d + 4 * (size_t)natms, *dvz = d + 5 * (size_t)natms;
    int* dint = (int*)(d + 6 * (size_t)natms);   // ltype then molecule (2 * natms ints in natms doubles)
    double *dfx = d + 7 * (size_t)natms, *dfy = d + 8 * (size_t)natms, *dfz = d + 9 * (size_t)natms;
    double* dae = d + 10 * (size_t)natms;
    if (natms) {
        CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dint, ltype, natms * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dint + natms, molecule, natms * sizeof(int), cudaMemcpyHostToDevice, s));
        if (heat) {
            CK(cudaMemcpyAsync(dvx, vxx, nb, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dvy, vyy, nb, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dvz, vzz, nb, cudaMemcpyHostToDevice, s));
        }
        CK(cudaMemsetAsync(dfx, 0, 3 * nb, s));
        if (atomic_energy) CK(cudaMemsetAsync(dae, 0, nb, s));
    }
    // the staging arrays are rewritten every call: keep the list only while the types
    // and molecules are those it was built for (positions are checked against the skin)
    if (ctx->disp_types_h.size() != (size_t)natms ||
        !std::equal(ltype, ltype + natms, ctx->disp_types_h.begin()) ||
        !std::equal(molecule, molecule + natms, ctx->disp_mol_h.begin())) {
        ctx->disp.valid = false;
        ctx->disp_types_h.assign(ltype, ltype + natms);
        ctx->disp_mol_h.assign(molecule, molecule + natms);
    }
    double out[14];
    rc = mbx_disp_forces_device(ctx, imcon, cell, natms, dint, dint + natms, dx, dy, dz, dfx, dfy, dfz,
                                heat ? dvx : nullptr, heat ? dvy : nullptr, heat ? dvz : nullptr,
                                atomic_energy ? dae : nullptr, out);
    if (rc) return rc;
    double* h = host_stage(ctx, 4 * (size_t)natms + 1);
    if (!h) return fail(ctx, MBX_ERR_CUDA, "pinned host staging allocation failed");
    if (natms) {
        CK(cudaMemcpyAsync(h, dfx, 3 * nb, cudaMemcpyDeviceToHost, s));
        if (atomic_energy) CK(cudaMemcpyAsync(h + 3 * (size_t)natms, dae, nb, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    for (int i = 0; i < natms; ++i) {
        fxx[i] += h[i];
        fyy[i] += h[natms + i];
        fzz[i] += h[2 * (size_t)natms + i];
        if (atomic_energy) atomic_energy[i] += h[3 * (size_t)natms + i];
    }
    *engsrp += out[0];
    *virsrp += out[1];
    for (int q = 0; q < 9; ++q) stress[q] += out[2 + q];
    if (jpot)
        for (int q = 0; q < 3; ++q) jpot[q] += out[11 + q];
    return MBX_OK;
}

extern "C" int mbx_water_forces(mbx_context* ctx, int precision, int imcon, const double* cell, int nttm2,
                                const int* listttm2, int nang, const int* listang, const int* ltype,
                                const int* molecule, int natms, const double* xxx, const double* yyy,
                                const double* zzz, double* fxx, double* fyy, double* fzz, const double* vxx,
                                const double* vyy, const double* vzz, const double* weight, double* atomic_energy,
                                double* scalars) {
    if (!ctx) return MBX_ERR_ARG;
    if (nttm2 < 0 || nttm2 % 3 || nang < 0 || natms < nttm2 || (nttm2 && !listttm2) || (nang && !listang) || !xxx ||
        !yyy || !zzz || !fxx || !fyy || !fzz)
        return fail(ctx, MBX_ERR_ARG, "bad argument");
    for (int t = 0; t < nttm2; ++t)
        if (listttm2[t] < 1 || listttm2[t] > natms || (t % 3 && listttm2[t] != listttm2[t - t % 3] + t % 3))
            return fail(ctx, MBX_ERR_ARG, "listttm2[%d]=%d: water atoms must be 1-based, O,H1,H2 consecutive", t,
                        listttm2[t]);
    for (int q = 0; q < 3 * nang; ++q)
        if (listang[q] < 1 || listang[q] > natms) return fail(ctx, MBX_ERR_ARG, "listang[%d] out of range", q);
    const bool disp = ltype && molecule;
    if (disp && !ctx->disp.vvv) return fail(ctx, MBX_ERR_ARG, "dispersion asked for before mbx_disp_setup");
    CK(cudaSetDevice(ctx->device));
    const int nw = nttm2 / 3;
    int rc = reserve_water(ctx, std::max(nw, 1), std::max(natms, 1));
    if (rc) return rc;
    const size_t nint = (size_t)nttm2 + 3 * (size_t)nang + 2 * (size_t)natms + 1;
    if (nint > ctx->ints_cap) {
        if (ctx->ints) cudaFree(ctx->ints);
        ctx->ints_cap = 0;
        ctx->ints = nullptr;
        CK(cudaMalloc(&ctx->ints, nint * sizeof(int)));
        ctx->ints_cap = nint;
    }
    int* d_lst = ctx->ints;
    int* d_ang = d_lst + nttm2;
    int* d_typ = d_ang + 3 * (size_t)nang;
    int* d_mol = d_typ + natms;
    const bool heat = vxx && vyy && vzz && weight;
    cudaStream_t s = ctx->stream;
    const size_t nb = (size_t)natms * sizeof(double);
    double* d = ctx->atoms;
    double *dx = d, *dy = d + natms, *dz = d + 2 * (size_t)natms;
    double *dvx = d + 3 * (size_t)natms, *dvy = d + 4 * (size_t)natms, *dvz = d + 5 * (size_t)natms;
    double* dm = d + 6 * (size_t)natms;
    double *dfx = d + 7 * (size_t)natms, *dfy = d + 8 * (size_t)natms, *dfz = d + 9 * (size_t)natms;
    double* dae = d + 10 * (size_t)natms;
    // one copy of every input, one zeroing of the outputs
    if (nttm2) CK(cudaMemcpyAsync(d_lst, listttm2, nttm2 * sizeof(int), cudaMemcpyHostToDevice, s));
    if (nang) CK(cudaMemcpyAsync(d_ang, listang, 3 * (size_t)nang * sizeof(int), cudaMemcpyHostToDevice, s));
    if (disp) {
        CK(cudaMemcpyAsync(d_typ, ltype, natms * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_mol, molecule, natms * sizeof(int), cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
    if (heat) {
        CK(cudaMemcpyAsync(dvx, vxx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvy, vyy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvz, vzz, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dm, weight, nb, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemsetAsync(dfx, 0, 3 * nb, s));
    // per-atom energies are needed on the device for jkin even when the caller passes none
    CK(cudaMemsetAsync(dae, 0, nb, s));
    double sc[MBX_NWATERSCALARS];
    std::memset(sc, 0, sizeof sc);
    // 1-body, then dispersion, then MB-pol: jkin (at the end of the MB-pol evaluation)
    // sees every term's per-atom energy
    if (nang) {
        rc = mbx_ps_pes_forces_device(ctx, imcon, cell, nang, d_ang, natms, dx, dy, dz, dfx, dfy, dfz,
                                      heat ? dvx : nullptr, heat ? dvy : nullptr, heat ? dvz : nullptr, dae,
                                      sc + MBX_NSCALARS);
        if (rc) return rc;
    }
    if (disp && natms) {
        if (ctx->disp_types_h.size() != (size_t)natms || !std::equal(ltype, ltype + natms, ctx->disp_types_h.begin()) ||
            !std::equal(molecule, molecule + natms, ctx->disp_mol_h.begin())) {
            ctx->disp.valid = false;
            ctx->disp_types_h.assign(ltype, ltype + natms);
            ctx->disp_mol_h.assign(molecule, molecule + natms);
        }
        rc = disp_forces_dev(ctx, imcon, cell, natms, d_typ, d_mol, dx, dy, dz, dfx, dfy, dfz,
                             heat ? dvx : nullptr, heat ? dvy : nullptr, heat ? dvz : nullptr, dae,
                             sc + MBX_NSCALARS + 14, precision == MBX_MIXED);
        if (rc) return rc;
    }
    Cell cl;
    rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    rc = run_mbpol(ctx, precision, cl, nw, d_lst, natms, dx, dy, dz, dfx, dfy, dfz, heat ? dvx : nullptr,
                   heat ? dvy : nullptr, heat ? dvz : nullptr, heat ? dm : nullptr, dae, sc);
    if (rc) return rc;
    double* h = host_stage(ctx, 4 * (size_t)natms + 1);
    if (!h) return fail(ctx, MBX_ERR_CUDA, "pinned host staging allocation failed");
    if (natms) {
        CK(cudaMemcpyAsync(h, dfx, (atomic_energy ? 4 : 3) * nb, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    for (int i = 0; i < natms; ++i) {
        fxx[i] += h[i];
        fyy[i] += h[natms + i];
        fzz[i] += h[2 * (size_t)natms + i];
        if (atomic_energy) atomic_energy[i] += h[3 * (size_t)natms + i];
    }
    if (scalars) std::memcpy(scalars, sc, sizeof sc);
    return MBX_OK;
}

extern "C" int mbx_disp_lrc(int ntypes, const double* prm, const int* numtyp, double rcut, double volm,
                            double* elrc, double* virlrc) {
    if (ntypes < 1 || !prm || !numtyp || !(rcut > 0.0) || !(volm > 0.0) || !elrc || !virlrc) return MBX_ERR_ARG;
    disp_lrc(ntypes, prm, numtyp, rcut, volm, elrc, virlrc);
    return MBX_OK;
}

extern "C" long mbx_disp_list_builds(const mbx_context* ctx) { return ctx ? ctx->disp.builds : -1; }

namespace {
// An electrostatics call that failed part way leaves no half-built state behind: the next
// call allocates everything again.
int polar_failed(mbx_context* ctx, cudaError_t e) {
    cudaStreamSynchronize(ctx->stream);
    ctx->polar.release();
    return fail(ctx, MBX_ERR_CUDA, "electrostatics: %s", cudaGetErrorString(e));
}

bool polar_prm_ok(const double* prm) {
    return prm && prm[0] > 1e-6 && prm[1] > 0.0 && prm[2] > 0.0 && prm[3] > 0.0 && prm[4] >= 0.0 && prm[4] < 1.0 &&
           prm[11] >= 0 && prm[12] >= 0 && prm[13] >= 0 && prm[11] <= 512 && prm[12] <= 512 && prm[13] <= 512 &&
           prm[14] >= 1;
}
}  // namespace

extern "C" int mbx_polar_forces_device(mbx_context* ctx, int precision, const double* prm, int imcon, const double* cell, int nw,
                                       const double* xxx, const double* yyy, const double* zzz, const double* chge,
                                       const double* dqdr, const double* polr, const double* polr2, double* dipx,
                                       double* dipy, double* dipz, double* fxx, double* fyy, double* fzz,
                                       double* out16, double* atomic_energy, const double* vxx, const double* vyy,
                                       const double* vzz, double* jpot, double* jkin) {
    if (!ctx) return MBX_ERR_ARG;
    if ((precision != MBX_FP64 && precision != MBX_MIXED) || nw < 0 || !polar_prm_ok(prm) || !out16 ||
        (nw && (!xxx || !yyy || !zzz || !chge || !dqdr || !polr || !polr2 || !dipx || !dipy || !dipz || !fxx ||
                !fyy || !fzz)))
        return fail(ctx, MBX_ERR_ARG, "mbx_polar_forces: bad argument");
    const bool heat = vxx && vyy && vzz;
    if (heat && (!jpot || !jkin)) return fail(ctx, MBX_ERR_ARG, "mbx_polar_forces: jpot/jkin needed with velocities");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    double jp[3] = {0, 0, 0}, jk[3] = {0, 0, 0};
    if (ctx->nsm > 0) ctx->polar.nsm = ctx->nsm;
    ctx->polar.profiling = ctx->profiling != 0;
    const cudaError_t pe = ctx->polar.run(precision, cl, prm, nw, xxx, yyy, zzz, chge, dqdr, polr, polr2, dipx, dipy,
                                          dipz, fxx, fyy, fzz, atomic_energy, heat ? vxx : nullptr,
                                          heat ? vyy : nullptr, heat ? vzz : nullptr, out16, jp, jk, ctx->stream);
    if (pe != cudaSuccess) return polar_failed(ctx, pe);
    ctx->launches = ctx->polar.launches;
    if (heat)
        for (int c = 0; c < 3; ++c) {
            jpot[c] += jp[c];
            jkin[c] += jk[c];
        }
    if (!ctx->polar.converged)
        return fail(ctx, MBX_ERR_CONVERGE, "mbx_polar_forces: dipoles not converged after %d iterations (rms change %g)",
                    ctx->polar.iterations, out16[12]);
    return MBX_OK;
}

extern "C" int mbx_polar_forces(mbx_context* ctx, int precision, const double* prm, int imcon, const double* cell, int nw,
                                const double* xxx, const double* yyy, const double* zzz, const double* chge,
                                const double* dqdr, const double* polr, const double* polr2, double* dipx, double* dipy,
                                double* dipz, double* fxx, double* fyy, double* fzz, double* out16,
                                double* atomic_energy, const double* vxx, const double* vyy, const double* vzz,
                                double* jpot, double* jkin) {
    if (!ctx) return MBX_ERR_ARG;
    if ((precision != MBX_FP64 && precision != MBX_MIXED) || nw < 0 || !polar_prm_ok(prm) || !out16 ||
        (nw && (!xxx || !yyy || !zzz || !chge || !dqdr || !polr || !polr2 || !dipx || !dipy || !dipz || !fxx ||
                !fyy || !fzz)))
        return fail(ctx, MBX_ERR_ARG, "mbx_polar_forces: bad argument");
    const bool heat = vxx && vyy && vzz;
    if (heat && (!jpot || !jkin)) return fail(ctx, MBX_ERR_ARG, "mbx_polar_forces: jpot/jkin needed with velocities");
    CK(cudaSetDevice(ctx->device));
    const size_t n = 4 * (size_t)nw, na = 3 * (size_t)nw;
    // x y z q polr polr2 dip(3) f(3) ae (13 n) + dp (6 nw) + v (3 na)
    const size_t need = 13 * n + 6 * (size_t)nw + 3 * na + 1;
    if (need > ctx->polar_stage_cap) {
        if (ctx->polar_stage) cudaFree(ctx->polar_stage);
        ctx->polar_stage = nullptr;
        ctx->polar_stage_cap = 0;
        CK(cudaMalloc(&ctx->polar_stage, need * sizeof(double)));
        ctx->polar_stage_cap = need;
    }
    cudaStream_t s = ctx->stream;
    double* d = ctx->polar_stage;
    double *dx = d, *dy = d + n, *dz = d + 2 * n, *dq = d + 3 * n, *dpr = d + 4 * n, *dpr2 = d + 5 * n;
    double *dmx = d + 6 * n, *dmy = d + 7 * n, *dmz = d + 8 * n, *dfx = d + 9 * n, *dfy = d + 10 * n,
           *dfz = d + 11 * n, *dae = d + 12 * n, *ddp = d + 13 * n, *dv = d + 13 * n + 6 * (size_t)nw;
    const size_t nb = n * sizeof(double);
    if (n) {
        CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dq, chge, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dpr, polr, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dpr2, polr2, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dmx, dipx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dmy, dipy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dmz, dipz, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ddp, dqdr, 6 * (size_t)nw * sizeof(double), cudaMemcpyHostToDevice, s));
        if (heat) {
            CK(cudaMemcpyAsync(dv, vxx, na * sizeof(double), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dv + na, vyy, na * sizeof(double), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dv + 2 * na, vzz, na * sizeof(double), cudaMemcpyHostToDevice, s));
        }
        CK(cudaMemsetAsync(dfx, 0, 4 * nb, s));   // forces and per-site energies
    }
    const int rc = mbx_polar_forces_device(ctx, precision, prm, imcon, cell, nw, dx, dy, dz, dq, ddp, dpr, dpr2, dmx, dmy, dmz,
                                           dfx, dfy, dfz, out16, atomic_energy ? dae : nullptr,
                                           heat ? dv : nullptr, heat ? dv + na : nullptr, heat ? dv + 2 * na : nullptr,
                                           jpot, jkin);
    if (rc && rc != MBX_ERR_CONVERGE) return rc;
    double* h = host_stage(ctx, 7 * n + 1);
    if (!h) return fail(ctx, MBX_ERR_CUDA, "pinned host staging allocation failed");
    if (n) {
        CK(cudaMemcpyAsync(h, dfx, 4 * nb, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(h + 4 * n, dmx, 3 * nb, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    for (size_t i = 0; i < n; ++i) {
        fxx[i] += h[i];
        fyy[i] += h[n + i];
        fzz[i] += h[2 * n + i];
        if (atomic_energy) atomic_energy[i] += h[3 * n + i];
        dipx[i] = h[4 * n + i];
        dipy[i] = h[5 * n + i];
        dipz[i] = h[6 * n + i];
    }
    return rc;
}

namespace {
// Standard-layout water and angle lists on the device (1-based atoms; angles H1, O, H2),
// followed by room for per-atom types and molecules.
int step_lists(mbx_context* ctx, int nw, int natms) {
    if (ctx->step_nw == nw) return MBX_OK;
    if (ctx->step_ints) cudaFree(ctx->step_ints);
    ctx->step_ints = nullptr;
    ctx->step_nw = -1;
    const size_t na = 3 * (size_t)nw;
    std::vector<int> h(na + 3 * (size_t)nw + 2 * (size_t)natms);
    for (size_t t = 0; t < na; ++t) h[t] = (int)t + 1;
    for (int w = 0; w < nw; ++w) {
        h[na + 3 * w] = 3 * w + 2;
        h[na + 3 * w + 1] = 3 * w + 1;
        h[na + 3 * w + 2] = 3 * w + 3;
    }
    CK(cudaMalloc(&ctx->step_ints, h.size() * sizeof(int)));
    // on the context's stream and complete before returning: a plain cudaMemcpy from pageable
    // memory may return before its DMA lands, unordered with the (non-blocking) stream
    CK(cudaMemcpyAsync(ctx->step_ints, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->step_nw = nw;
    return MBX_OK;
}

// q, aep (per-site electrostatic energies) and dqdr device workspace of the step
int step_stage(mbx_context* ctx, size_t n, int nw, size_t extra) {
    const size_t need = 2 * n + 6 * (size_t)nw + extra + 1;
    if (need <= ctx->step_stage_cap) return MBX_OK;
    if (ctx->step_stage) cudaFree(ctx->step_stage);
    ctx->step_stage = nullptr;
    ctx->step_stage_cap = 0;
    CK(cudaMalloc(&ctx->step_stage, need * sizeof(double)));
    ctx->step_stage_cap = need;
    return MBX_OK;
}

// The step on device arrays: M sites + DMS charges, electrostatics, 1-body, dispersion,
// MB-pol, M-site redistribution.  dq, ddq, daep are workspace; dae must be valid.
int water_step_core(mbx_context* ctx, int precision, int imcon, const double* cell, const Cell& cl, int nw,
                    int natms, const double* prm, const double* dpr, const double* dpr2, const int* d_typ,
                    const int* d_mol, double* dx, double* dy, double* dz, double* dmx, double* dmy, double* dmz,
                    double* dfx, double* dfy, double* dfz, const double* dvx, const double* dvy, const double* dvz,
                    const double* dm, double* dae, double* dq, double* ddq, double* daep, double* sc) {
    cudaStream_t s = ctx->stream;
    const int* d_lst = ctx->step_ints;
    const int* d_ang = d_lst + 3 * (size_t)nw;
    const bool heat = dvx && dvy && dvz && dm;
    const double gamma = prm[10];
    CK(cudaMemsetAsync(dq, 0, natms * sizeof(double), s));   // O carries no charge
    CK(cudaMemsetAsync(daep, 0, natms * sizeof(double), s));
    CK(launch_msites_dms(nw, d_lst, cl, dx, dy, dz, gamma, dq, ddq, s));
    double* sp = sc + MBX_NWATERSCALARS;
    double jp[3] = {0, 0, 0}, jk[3] = {0, 0, 0};
    if (ctx->nsm > 0) ctx->polar.nsm = ctx->nsm;
    // the electrostatic per-site energies stay apart: their jkin carries them with the
    // M-site redistribution
    ctx->polar.profiling = ctx->profiling != 0;
    // overlapped form: the MB-pol 2B/3B terms (positions only) on the side stream, launched
    // when the mixed solve starts its FP32 CG sweeps, in the 8-warp fused kernel that leaves
    // room on every SM for the CG kernels; the final pass waits for it
    const MixedPass mpq{ctx->hard2, ctx->hard3, ctx->hard_count, ctx->limit2, ctx->limit3};
    const bool overlap = ctx->overlap && precision == MBX_MIXED && nw >= 2 && ctx->fused &&
                         fused_applies(precision, mpq);
    int mb_rc = MBX_OK;
    // the 1-body and dispersion terms (positions only) on the third stream, beside the
    // electrostatics' setup and solve; the final pass, whose kernels add to the same force
    // arrays, waits for them (join_hook)
    const bool side_terms = ctx->overlap_terms && nw > 0;
    const bool disp = d_typ && d_mol;
    if (side_terms) {
        if (disp && !ctx->disp.vvv) return fail(ctx, MBX_ERR_ARG, "mbx_disp_setup has not been called");
        if (!ctx->side2) CK(cudaStreamCreateWithFlags(&ctx->side2, cudaStreamNonBlocking));
        if (!ctx->ev_fork2) CK(cudaEventCreateWithFlags(&ctx->ev_fork2, cudaEventDisableTiming));
        if (!ctx->ev_join2) CK(cudaEventCreateWithFlags(&ctx->ev_join2, cudaEventDisableTiming));
        if (!ctx->side_acc) CK(cudaMalloc(&ctx->side_acc, 28 * sizeof(double)));
        if (!ctx->side_acc_h) CK(cudaMallocHost(&ctx->side_acc_h, 28 * sizeof(double)));
        cudaStream_t s2 = ctx->side2;
        CK(cudaEventRecord(ctx->ev_fork2, s));   // after the M sites
        CK(cudaStreamWaitEvent(s2, ctx->ev_fork2, 0));
        CK(cudaMemsetAsync(ctx->side_acc, 0, 28 * sizeof(double), s2));
        if (disp) {   // first: its skin test reads a flag back, a short wait here
            bool rebuilt = false;
            const cudaError_t e = ctx->disp.forces(cl, natms, d_typ, d_mol, dx, dy, dz, dfx, dfy, dfz,
                                                   heat ? dvx : nullptr, heat ? dvy : nullptr, heat ? dvz : nullptr,
                                                   dae, ctx->side_acc + 14, ctx->totals_h, s2, &rebuilt,
                                                   precision == MBX_MIXED);
            if (e == cudaErrorInvalidValue) return fail(ctx, MBX_ERR_CAPACITY, "dispersion list capacity exceeded");
            CK(e);
        }
        CK(launch_ps_pes(nw, d_ang, cl, dx, dy, dz, dfx, dfy, dfz, dae, heat ? dvx : nullptr, heat ? dvy : nullptr,
                         heat ? dvz : nullptr, ctx->side_acc, s2));
        CK(cudaMemcpyAsync(ctx->side_acc_h, ctx->side_acc, 28 * sizeof(double), cudaMemcpyDeviceToHost, s2));
        CK(cudaEventRecord(ctx->ev_join2, s2));
        if (!overlap) {   // the hooks of the solve: nothing to fork, the join before the final pass
            ctx->polar.fork_hook = []() -> cudaError_t { return cudaSuccess; };
            ctx->polar.join_hook = [&]() -> cudaError_t { return cudaStreamWaitEvent(s, ctx->ev_join2, 0); };
        }
    }
    if (overlap) {
        if (!ctx->side) CK(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        if (!ctx->ev_fork) CK(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
        if (!ctx->ev_join) CK(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
        ctx->polar.fork_hook = [&]() -> cudaError_t {
            cudaError_t e;
            if ((e = cudaEventRecord(ctx->ev_fork, s))) return e;
            if ((e = cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0))) return e;
            ctx->stream = ctx->side;
            mb_rc = run_mbpol(ctx, precision, cl, nw, d_lst, natms, dx, dy, dz, dfx, dfy, dfz, heat ? dvx : nullptr,
                              heat ? dvy : nullptr, heat ? dvz : nullptr, heat ? dm : nullptr, dae, sc, false, true);
            ctx->stream = s;
            if (mb_rc) return cudaErrorUnknown;
            return cudaEventRecord(ctx->ev_join, ctx->side);
        };
        ctx->polar.join_hook = [&]() -> cudaError_t {
            cudaError_t e;
            if (side_terms && (e = cudaStreamWaitEvent(s, ctx->ev_join2, 0))) return e;
            return cudaStreamWaitEvent(s, ctx->ev_join, 0);
        };
    }
    const cudaError_t pe = ctx->polar.run(precision, cl, prm, nw, dx, dy, dz, dq, ddq, dpr, dpr2, dmx, dmy, dmz, dfx,
                                          dfy, dfz, daep, heat ? dvx : nullptr, heat ? dvy : nullptr,
                                          heat ? dvz : nullptr, sp, jp, jk, s);
    ctx->polar.fork_hook = nullptr;
    ctx->polar.join_hook = nullptr;
    // the side terms are done before anything else touches the force arrays, on error too
    if (side_terms) CK(cudaStreamSynchronize(ctx->side2));
    if (mb_rc) return mb_rc;
    if (pe != cudaSuccess) return polar_failed(ctx, pe);
    if (overlap) {   // the MB-pol scalars (the side stream has finished with the join)
        CK(cudaStreamWaitEvent(s, ctx->ev_join, 0));
        ctx->stream = ctx->side;
        const int frc = finish_mbpol(ctx, precision, nw, sc);
        ctx->stream = s;
        if (frc) return frc;
    }
    const long mb_launches = overlap ? ctx->launches : 0;
    for (int c = 0; c < 3; ++c) {
        sp[16 + c] = jp[c];
        sp[19 + c] = jk[c];
    }
    const long polar_launches = ctx->polar.launches + 1;
    int rc = MBX_OK;
    if (side_terms) {   // their scalars (the final pass has waited for the stream)
        CK(cudaEventSynchronize(ctx->ev_join2));
        std::memcpy(sc + MBX_NSCALARS, ctx->side_acc_h, 14 * sizeof(double));
        if (disp) std::memcpy(sc + MBX_NSCALARS + 14, ctx->side_acc_h + 14, 14 * sizeof(double));
    } else {
        rc = mbx_ps_pes_forces_device(ctx, imcon, cell, nw, d_ang, natms, dx, dy, dz, dfx, dfy, dfz,
                                      heat ? dvx : nullptr, heat ? dvy : nullptr, heat ? dvz : nullptr, dae,
                                      sc + MBX_NSCALARS);
        if (rc) return rc;
        if (disp) {
            rc = disp_forces_dev(ctx, imcon, cell, natms, d_typ, d_mol, dx, dy, dz, dfx, dfy, dfz,
                                 heat ? dvx : nullptr, heat ? dvy : nullptr, heat ? dvz : nullptr, dae,
                                 sc + MBX_NSCALARS + 14, precision == MBX_MIXED);
            if (rc) return rc;
        }
    }
    if (!overlap) {
        rc = run_mbpol(ctx, precision, cl, nw, d_lst, natms, dx, dy, dz, dfx, dfy, dfz, heat ? dvx : nullptr,
                       heat ? dvy : nullptr, heat ? dvz : nullptr, heat ? dm : nullptr, dae, sc);
        if (rc) return rc;
    } else {
        ctx->launches = mb_launches;
        if (heat) {   // jkin once every term's per-atom energy is in (the sequential form's last step)
            CK(cudaMemsetAsync(ctx->acc, 0, MBX_NSCALARS * sizeof(double), s));
            CK(launch_jkin(3 * nw, dvx, dvy, dvz, dm, dae, ctx->acc, s));
            CK(cudaMemcpyAsync(ctx->acc_h, ctx->acc, MBX_NSCALARS * sizeof(double), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            for (int c = 0; c < 3; ++c) sc[S_JKIN + c] += ctx->acc_h[S_JKIN + c];
            ++ctx->launches;
        }
    }
    CK(launch_msite_redistribute(nw, gamma, dfx, dfy, dfz, s));
    // device atomic energies: the electrostatic part joins the others for the caller
    ctx->launches += polar_launches + 3;   // + 1-body + M sites + redistribution
    return MBX_OK;
}
}  // namespace

extern "C" int mbx_water_step_device(mbx_context* ctx, int precision, int imcon, const double* cell, int nw,
                                     int natms, const double* polar_prm, const double* polr, const double* polr2,
                                     const int* ltype, const int* molecule, double* xxx, double* yyy, double* zzz,
                                     double* dipx, double* dipy, double* dipz, double* fxx, double* fyy,
                                     double* fzz, const double* vxx, const double* vyy, const double* vzz,
                                     const double* weight, double* atomic_energy, double* chge, double* scalars) {
    if (!ctx) return MBX_ERR_ARG;
    if ((precision != MBX_FP64 && precision != MBX_MIXED) || nw < 0 || natms != 4 * nw ||
        !polar_prm_ok(polar_prm) || (nw && (!polr || !polr2 || !xxx || !yyy || !zzz || !dipx || !dipy || !dipz ||
                                            !fxx || !fyy || !fzz || !chge)))
        return fail(ctx, MBX_ERR_ARG, "mbx_water_step_device: bad argument");
    const bool disp = ltype && molecule;
    if (disp && !ctx->disp.vvv) return fail(ctx, MBX_ERR_ARG, "dispersion asked for before mbx_disp_setup");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    double sc[MBX_NSTEPSCALARS];
    std::memset(sc, 0, sizeof sc);
    if (nw > 0) {
        if ((rc = reserve_water(ctx, nw, natms)) || (rc = step_lists(ctx, nw, natms)) ||
            (rc = step_stage(ctx, natms, nw, atomic_energy ? 0 : (size_t)natms)))
            return rc;
        const size_t n = (size_t)natms;
        double* g = ctx->step_stage;
        double *daep = g, *ddq = g + n, *dae = atomic_energy ? atomic_energy : g + n + 6 * (size_t)nw;
        if (!atomic_energy) CK(cudaMemsetAsync(dae, 0, n * sizeof(double), ctx->stream));
        ctx->launches = 0;
        rc = water_step_core(ctx, precision, imcon, cell, cl, nw, natms, polar_prm, polr, polr2, ltype, molecule,
                             xxx, yyy, zzz, dipx, dipy, dipz, fxx, fyy, fzz, vxx, vyy, vzz, weight, dae, chge, ddq,
                             daep, sc);
        if (rc) return rc;
        if (atomic_energy) CK(launch_add(natms, daep, atomic_energy, ctx->stream));
    }
    if (scalars) std::memcpy(scalars, sc, sizeof sc);
    if (nw > 0 && !ctx->polar.converged)
        return fail(ctx, MBX_ERR_CONVERGE, "mbx_water_step: dipoles not converged after %d iterations",
                    ctx->polar.iterations);
    return MBX_OK;
}

extern "C" int mbx_water_step(mbx_context* ctx, int precision, int imcon, const double* cell, int nw, int natms,
                              const double* polar_prm, const double* polr, const double* polr2, const int* ltype,
                              const int* molecule, double* xxx, double* yyy, double* zzz, double* dipx,
                              double* dipy, double* dipz, double* fxx, double* fyy, double* fzz, const double* vxx,
                              const double* vyy, const double* vzz, const double* weight, double* atomic_energy,
                              double* chge, double* scalars) {
    if (!ctx) return MBX_ERR_ARG;
    if ((precision != MBX_FP64 && precision != MBX_MIXED) || nw < 0 || natms != 4 * nw ||
        !polar_prm_ok(polar_prm) || (nw && (!polr || !polr2 || !xxx || !yyy || !zzz || !dipx || !dipy || !dipz ||
                                            !fxx || !fyy || !fzz)))
        return fail(ctx, MBX_ERR_ARG, "mbx_water_step: bad argument");
    const bool disp = ltype && molecule;
    if (disp && !ctx->disp.vvv) return fail(ctx, MBX_ERR_ARG, "dispersion asked for before mbx_disp_setup");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    double sc[MBX_NSTEPSCALARS];
    std::memset(sc, 0, sizeof sc);
    if (nw == 0) {
        if (scalars) std::memcpy(scalars, sc, sizeof sc);
        return MBX_OK;
    }
    const size_t n = (size_t)natms, na = 3 * (size_t)nw;
    // x y z vx vy vz m f(3) ae in ctx->atoms; polr polr2 dip(3) q in the step workspace
    if ((rc = reserve_water(ctx, nw, natms)) || (rc = step_lists(ctx, nw, natms)) ||
        (rc = step_stage(ctx, n, nw, 6 * n)))
        return rc;
    cudaStream_t s = ctx->stream;
    int* d_typ = ctx->step_ints + na + 3 * (size_t)nw;
    int* d_mol = d_typ + n;
    const bool heat = vxx && vyy && vzz && weight;
    const size_t nb = n * sizeof(double);
    double* d = ctx->atoms;
    double *dx = d, *dy = d + n, *dz = d + 2 * n, *dvx = d + 3 * n, *dvy = d + 4 * n, *dvz = d + 5 * n, *dm = d + 6 * n;
    double *dfx = d + 7 * n, *dfy = d + 8 * n, *dfz = d + 9 * n, *dae = d + 10 * n;
    double* g = ctx->step_stage;
    double *daep = g, *ddq = g + n, *dpr = g + n + 6 * (size_t)nw, *dpr2 = dpr + n, *dmx = dpr2 + n, *dmy = dmx + n,
           *dmz = dmy + n, *dq = dmz + n;
    CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dpr, polr, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dpr2, polr2, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dmx, dipx, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dmy, dipy, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dmz, dipz, nb, cudaMemcpyHostToDevice, s));
    if (heat) {
        CK(cudaMemcpyAsync(dvx, vxx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvy, vyy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvz, vzz, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dm, weight, nb, cudaMemcpyHostToDevice, s));
    }
    if (disp) {
        CK(cudaMemcpyAsync(d_typ, ltype, n * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(d_mol, molecule, n * sizeof(int), cudaMemcpyHostToDevice, s));
        if (ctx->disp_types_h.size() != n || !std::equal(ltype, ltype + n, ctx->disp_types_h.begin()) ||
            !std::equal(molecule, molecule + n, ctx->disp_mol_h.begin())) {
            ctx->disp.valid = false;
            ctx->disp_types_h.assign(ltype, ltype + n);
            ctx->disp_mol_h.assign(molecule, molecule + n);
        }
    }
    CK(cudaMemsetAsync(dfx, 0, 4 * nb, s));   // forces and per-atom energies
    ctx->launches = 0;
    rc = water_step_core(ctx, precision, imcon, cell, cl, nw, natms, polar_prm, dpr, dpr2, disp ? d_typ : nullptr,
                         disp ? d_mol : nullptr, dx, dy, dz, dmx, dmy, dmz, dfx, dfy, dfz, heat ? dvx : nullptr,
                         heat ? dvy : nullptr, heat ? dvz : nullptr, heat ? dm : nullptr, dae, dq, ddq, daep, sc);
    if (rc) return rc;
    // forces, per-atom energies, dipoles, M-site positions, charges back through one staging area
    double* h = host_stage(ctx, 12 * n + 1);
    if (!h) return fail(ctx, MBX_ERR_CUDA, "pinned host staging allocation failed");
    CK(cudaMemcpyAsync(h, dfx, 4 * nb, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h + 4 * n, daep, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h + 5 * n, dmx, 3 * nb, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h + 8 * n, dx, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h + 9 * n, dy, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h + 10 * n, dz, nb, cudaMemcpyDeviceToHost, s));
    if (chge) CK(cudaMemcpyAsync(h + 11 * n, dq, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (size_t i = 0; i < n; ++i) {
        fxx[i] += h[i];
        fyy[i] += h[n + i];
        fzz[i] += h[2 * n + i];
        if (atomic_energy) atomic_energy[i] += h[3 * n + i] + h[4 * n + i];
        dipx[i] = h[5 * n + i];
        dipy[i] = h[6 * n + i];
        dipz[i] = h[7 * n + i];
        if (chge) chge[i] = h[11 * n + i];
    }
    for (size_t i = na; i < n; ++i) {
        xxx[i] = h[8 * n + i];
        yyy[i] = h[9 * n + i];
        zzz[i] = h[10 * n + i];
    }
    if (scalars) std::memcpy(scalars, sc, sizeof sc);
    if (!ctx->polar.converged)
        return fail(ctx, MBX_ERR_CONVERGE, "mbx_water_step: dipoles not converged after %d iterations",
                    ctx->polar.iterations);
    return MBX_OK;
}

// Many boxes, one call: box b runs mbx_water_step on its slice of the arrays on one of the
// context's worker lanes.  A lane is a child context (its own stream and device buffers,
// kept between calls) driven by its own host thread for the call, so the boxes' kernels
// and host round trips overlap; boxes are taken largest first from a shared counter.
void mbx_set_error_text(mbx_context* ctx, const char* msg) {
    if (ctx && msg) std::snprintf(ctx->err, sizeof ctx->err, "%s", msg);
}

extern "C" int mbx_set_precond_sweeps(mbx_context* ctx, int sweeps) {
    if (!ctx) return MBX_ERR_ARG;
    if (sweeps != 0 && (sweeps < 1 || sweeps > 9 || sweeps % 2 == 0))
        return fail(ctx, MBX_ERR_ARG, "preconditioner sweeps must be 0 (automatic) or odd, 1..9");
    ctx->polar.precond_sweeps = sweeps;
    return MBX_OK;
}

extern "C" int mbx_set_aspc(mbx_context* ctx, int k, int iter_nstep) {
    if (!ctx) return MBX_ERR_ARG;
    // aspc_init stops on any other order (SOURCE/aspc.f90:68-71)
    if (k != 0 && k != 2 && k != 4) return fail(ctx, MBX_ERR_ARG, "ASPC order must be 0 (off), 2 or 4");
    if (iter_nstep < 0) return fail(ctx, MBX_ERR_ARG, "ASPC iter_nstep must be >= 0");
    CK(cudaSetDevice(ctx->device));
    CK(ctx->polar.aspc_reset(k, iter_nstep));
    return MBX_OK;
}

extern "C" int mbx_set_dipole_guess(mbx_context* ctx, int order) {
    if (!ctx) return MBX_ERR_ARG;
    if (order < 0 || order > 3) return fail(ctx, MBX_ERR_ARG, "dipole guess order must be 0..3");
    CK(cudaSetDevice(ctx->device));
    CK(ctx->polar.guess_reset(order));
    return MBX_OK;
}

extern "C" int mbx_aspc_restart(mbx_context* ctx) {
    if (!ctx) return MBX_ERR_ARG;
    ctx->polar.aspc_restart();
    return MBX_OK;
}

extern "C" int mbx_aspc_step(mbx_context* ctx) { return ctx ? ctx->polar.aspc_step : -1; }

extern "C" int mbx_set_precond_block(mbx_context* ctx, int on) {
    if (!ctx) return MBX_ERR_ARG;
    ctx->polar.precond_block = on != 0;
    return MBX_OK;
}

extern "C" int mbx_set_spme(mbx_context* ctx, int order, double spacing, const int* grid) {
    if (!ctx) return MBX_ERR_ARG;
    if (order != 0 && (order < 4 || order > 8)) return fail(ctx, MBX_ERR_ARG, "SPME order must be 0 or 4..8");
    if (order && grid && grid[0] > 0) {
        for (int a = 0; a < 3; ++a)
            if (grid[a] < order || grid[a] > 1024 || grid[a] % 2 || spme_smooth_even(grid[a]) != grid[a])
                return fail(ctx, MBX_ERR_ARG, "SPME grid must be even, 2-3-5 smooth, order..1024 per axis");
    } else if (order && !(spacing > 0.05 && spacing < 100.0)) {
        return fail(ctx, MBX_ERR_ARG, "SPME spacing out of range");
    }
    ctx->polar.spme_order = order;
    ctx->polar.spme_spacing = spacing;
    for (int a = 0; a < 3; ++a) ctx->polar.spme_grid[a] = (order && grid && grid[0] > 0) ? grid[a] : 0;
    return MBX_OK;
}

extern "C" int mbx_set_polar_skin(mbx_context* ctx, double delr) {
    if (!ctx) return MBX_ERR_ARG;
    if (!(delr >= 0.0 && delr < 10.0)) return fail(ctx, MBX_ERR_ARG, "skin must be in [0, 10) Angstrom");
    ctx->polar.list_skin = delr;
    ctx->polar.skin_ok = false;
    return MBX_OK;
}

extern "C" long mbx_polar_list_builds(const mbx_context* ctx) { return ctx ? ctx->polar.list_builds : -1; }

extern "C" int mbx_polar_last_pairs(mbx_context* ctx, int* pairs, long cap, long* npairs) {
    if (!ctx || !npairs || cap < 0 || (cap && !pairs)) return MBX_ERR_ARG;
    PolarState& P = ctx->polar;
    *npairs = 0;
    if (!P.nn || P.n_cap == 0) return MBX_OK;
    const int n = P.last_n;
    if (n <= 0) return MBX_OK;
    CK(cudaSetDevice(ctx->device));
    std::vector<int> nn(n), nbr((size_t)n * P.cap);
    CK(cudaMemcpyAsync(nn.data(), P.nn, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(nbr.data(), P.nbr, nbr.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    long c = 0;
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < nn[i]; ++k) {
            const int j = nbr[(size_t)i * P.cap + k];
            if (j <= i) continue;
            if (c < cap) {
                pairs[2 * c] = i;
                pairs[2 * c + 1] = j;
            }
            ++c;
        }
    *npairs = c;
    return MBX_OK;
}

extern "C" int mbx_spme_last_grid(const mbx_context* ctx, int* grid) {
    if (!ctx || !grid) return MBX_ERR_ARG;
    for (int a = 0; a < 3; ++a) grid[a] = ctx->polar.spme_order ? ctx->polar.spme_K_last[a] : 0;
    return MBX_OK;
}

extern "C" int mbx_spme_grid_for_cell(const double* cell, double spacing, int* grid) {
    if (!cell || !grid || !(spacing > 0.0)) return MBX_ERR_ARG;
    const double* a = cell;   // perpendicular widths of the cell
    const double axb[3] = {a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5], a[0] * a[4] - a[1] * a[3]};
    const double bxc[3] = {a[4] * a[8] - a[5] * a[7], a[5] * a[6] - a[3] * a[8], a[3] * a[7] - a[4] * a[6]};
    const double cxa[3] = {a[7] * a[2] - a[1] * a[8], a[0] * a[8] - a[2] * a[6], a[1] * a[6] - a[0] * a[7]};
    const double v = std::fabs(a[0] * bxc[0] + a[1] * bxc[1] + a[2] * bxc[2]);
    auto nrm = [](const double* u) { return std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]); };
    const double w[3] = {v / nrm(bxc), v / nrm(cxa), v / nrm(axb)};
    for (int c = 0; c < 3; ++c) grid[c] = spme_smooth_even(w[c] / spacing);
    return MBX_OK;
}

extern "C" int mbx_fft3d(mbx_context* ctx, int n1, int n2, int n3, int count, int sign, double* data) {
    if (!ctx) return MBX_ERR_ARG;
    if (n1 < 1 || n2 < 1 || n3 < 1 || n1 > 1024 || n2 > 1024 || n3 > 1024 || count < 1 || !data ||
        (sign != 1 && sign != -1))
        return fail(ctx, MBX_ERR_ARG, "mbx_fft3d: bad argument");
    for (int n : {n1, n2, n3}) {
        int m = n;
        for (int p : {2, 3, 5})
            while (m % p == 0) m /= p;
        if (m != 1) return fail(ctx, MBX_ERR_ARG, "mbx_fft3d: sizes must have no prime factor above 5");
    }
    CK(cudaSetDevice(ctx->device));
    SpmeState st;
    const double cell[9] = {(double)n1, 0, 0, 0, (double)n2, 0, 0, 0, (double)n3};
    const int K[3] = {n1, n2, n3};
    // the FFT tables need no B-spline order beyond the grid: the smallest order that fits
    const int order = std::max(4, std::min(8, std::min(n1, std::min(n2, n3))));
    if (std::min(n1, std::min(n2, n3)) < 4) return fail(ctx, MBX_ERR_ARG, "mbx_fft3d: sizes must be >= 4");
    CK(st.prepare(cell, 1.0, order, K, false, 1, ctx->stream));
    const size_t ng = (size_t)n1 * n2 * n3 * count;
    double2* d = nullptr;
    CK(cudaMalloc(&d, ng * sizeof(double2)));
    cudaError_t e = cudaMemcpyAsync(d, data, ng * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream);
    if (!e) e = st.fft64(d, count, sign, ctx->stream);
    if (!e) e = cudaMemcpyAsync(data, d, ng * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream);
    if (!e) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    CK(e);
    return MBX_OK;
}

extern "C" int mbx_spme_kspace(mbx_context* ctx, const double* prm, int order, const int* grid, int imcon,
                               const double* cell, int n, const double* xxx, const double* yyy, const double* zzz,
                               const double* chge, const double* dip, const double* vel, double* forces, double* field,
                               double* pot, double* out) {
    if (!ctx) return MBX_ERR_ARG;
    if (!prm || !grid || !out || n < 0 || (n && (!xxx || !yyy || !zzz || !chge || !forces)) || !(prm[0] > 0.0) ||
        !(prm[1] > 0.0) || order < 4 || order > 8)
        return fail(ctx, MBX_ERR_ARG, "mbx_spme_kspace: bad argument");
    for (int a = 0; a < 3; ++a)
        if (grid[a] < order || grid[a] > 1024 || grid[a] % 2 || spme_smooth_even(grid[a]) != grid[a])
            return fail(ctx, MBX_ERR_ARG, "mbx_spme_kspace: grid must be even, 2-3-5 smooth, order..1024 per axis");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    SpmeState& st = ctx->polar.spme;
    const bool heat = vel != nullptr;
    CK(st.prepare(cell, prm[0], order, grid, false, heat ? 9 : 1, s));
    const size_t m = (size_t)std::max(n, 1);
    // device staging: x y z q (4 n), md (n double4), vh (12 n), part5 (5 n), field (3 n), acc (64)
    std::vector<double> h(4 * m + 4 * m + 12 * m, 0.0);
    for (int j = 0; j < n; ++j) {
        h[j] = xxx[j];
        h[m + j] = yyy[j];
        h[2 * m + j] = zzz[j];
        h[3 * m + j] = chge[j];
        const double mu[3] = {dip ? dip[j] : 0.0, dip ? dip[(size_t)n + j] : 0.0, dip ? dip[2 * (size_t)n + j] : 0.0};
        for (int c = 0; c < 3; ++c) h[4 * m + 4 * j + c] = mu[c];
        if (heat) {
            const double v[3] = {vel[j], vel[(size_t)n + j], vel[2 * (size_t)n + j]};
            for (int b = 0; b < 3; ++b) h[8 * m + (size_t)b * m + j] = chge[j] * v[b];
            for (int c = 0; c < 3; ++c)
                for (int b = 0; b < 3; ++b) h[8 * m + (size_t)(3 + 3 * c + b) * m + j] = mu[c] * v[b];
        }
    }
    double* d = nullptr;
    const size_t nd = h.size() + 8 * m + 64;
    CK(cudaMalloc(&d, nd * sizeof(double)));
    double* part5 = d + h.size();
    double* dfield = part5 + 5 * m;
    double* acc = dfield + 3 * m;
    std::vector<double> hp(8 * m + 64);
    double sc = 0.0;
    cudaError_t e = cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (!e) e = cudaMemsetAsync(acc, 0, 64 * sizeof(double), s);
    if (!e) {
        const double* a = cell;
        const double vol = std::fabs(a[0] * (a[4] * a[8] - a[5] * a[7]) + a[1] * (a[5] * a[6] - a[3] * a[8]) +
                                     a[2] * (a[3] * a[7] - a[4] * a[6]));
        sc = 2.0 * (2.0 * 3.141592653589793 / vol) * 138935.4835 / prm[1];   // sfac
        e = st.frame(n, d, d + m, d + 2 * m, s);
        if (!e)
            e = st.final(n, d, d + m, d + 2 * m, d + 3 * m, reinterpret_cast<const double4*>(d + 4 * m),
                         heat ? d + 8 * m : nullptr, sc, part5, acc, dfield, s);
    }
    if (!e) e = cudaMemcpyAsync(hp.data(), part5, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    cudaFree(d);
    CK(e);
    const double* p5 = hp.data();
    const double* hf = p5 + 5 * m;
    const double* ha = hf + 3 * m;
    for (int j = 0; j < n; ++j) {
        for (int c = 0; c < 3; ++c) {
            forces[(size_t)c * n + j] = 2.0 * sc * p5[(size_t)c * m + j];
            if (field) field[(size_t)c * n + j] = hf[(size_t)c * m + j];
        }
        if (pot) pot[j] = 2.0 * sc * (p5[3 * m + j] + p5[4 * m + j]);
    }
    const double engc = ha[48], eng1 = ha[49];
    out[0] = sc * engc;
    out[1] = sc * eng1;
    const double* o = ha + 50;   // omg 11 22 33 12 13 23
    const double st9[9] = {o[0] + eng1, o[3], o[4], o[3], o[1] + eng1, o[5], o[4], o[5], o[2] + eng1};
    for (int c = 0; c < 9; ++c) out[2 + c] = sc * st9[c];
    for (int c = 0; c < 3; ++c) out[11 + c] = heat ? ha[56 + c] : 0.0;
    return MBX_OK;
}

extern "C" int mbx_pimd_matrices(int nbead, int langevin, double* nmode_to_cart, double* cart_to_nmode,
                                 double* lambda) {
    if (nbead < 2 || nbead % 2 || nbead > pimd_max_beads()) return MBX_ERR_ARG;
    std::vector<double> n2c, c2n, lam;
    pimd_matrices(nbead, langevin != 0, n2c, c2n, lam);
    if (nmode_to_cart) std::memcpy(nmode_to_cart, n2c.data(), n2c.size() * sizeof(double));
    if (cart_to_nmode) std::memcpy(cart_to_nmode, c2n.data(), c2n.size() * sizeof(double));
    if (lambda) std::memcpy(lambda, lam.data(), lam.size() * sizeof(double));
    return MBX_OK;
}

namespace {
int pimd_prepare(mbx_context* ctx, int P, int langevin) {
    if (P < 2 || P % 2 || P > pimd_max_beads())
        return fail(ctx, MBX_ERR_ARG, "the number of beads must be even, 2..%d", pimd_max_beads());
    if (ctx->pimd_mat && ctx->pimd_P == P && ctx->pimd_lang == (langevin != 0)) return MBX_OK;
    std::vector<double> n2c, c2n, lam;
    pimd_matrices(P, langevin != 0, n2c, c2n, lam);
    if (ctx->pimd_mat) cudaFree(ctx->pimd_mat);
    ctx->pimd_mat = nullptr;
    ctx->pimd_P = 0;
    CK(cudaMalloc(&ctx->pimd_mat, 2 * (size_t)P * P * sizeof(double)));
    if (!ctx->pimd_acc) CK(cudaMalloc(&ctx->pimd_acc, 2 * sizeof(double)));
    CK(cudaMemcpyAsync(ctx->pimd_mat, n2c.data(), n2c.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->pimd_mat + (size_t)P * P, c2n.data(), c2n.size() * sizeof(double),
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));   // the host vectors go out of scope
    ctx->pimd_P = P;
    ctx->pimd_lang = langevin != 0;
    return MBX_OK;
}
}  // namespace

extern "C" int mbx_pimd_transform_device(mbx_context* ctx, int nbead, int langevin, int to_modes, long nvals,
                                         const double* in, double* out) {
    if (!ctx) return MBX_ERR_ARG;
    if (nvals < 0 || (nvals && (!in || !out)) || in == out)
        return fail(ctx, MBX_ERR_ARG, "mbx_pimd_transform_device: bad argument");
    CK(cudaSetDevice(ctx->device));
    int rc = pimd_prepare(ctx, nbead, langevin);
    if (rc) return rc;
    const double* A = ctx->pimd_mat + (to_modes ? (size_t)nbead * nbead : 0);
    CK(launch_pimd_transform(nbead, nvals, A, in, out, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MBX_OK;
}

extern "C" int mbx_pimd_spring_forces_device(mbx_context* ctx, int nbead, int langevin, int add_spring_to_forces,
                                             double hbar, double beta, double force_scale, int natms,
                                             const double* xxx, const double* yyy, const double* zzz, double* fxx,
                                             double* fyy, double* fzz, const double* mass, double* energies) {
    if (!ctx) return MBX_ERR_ARG;
    if (natms < 0 || !(hbar > 0.0) || !(beta > 0.0) || !(force_scale != 0.0) ||
        (natms && (!xxx || !yyy || !zzz || !fxx || !fyy || !fzz || !mass)))
        return fail(ctx, MBX_ERR_ARG, "mbx_pimd_spring_forces_device: bad argument");
    CK(cudaSetDevice(ctx->device));
    int rc = pimd_prepare(ctx, nbead, langevin);
    if (rc) return rc;
    const double coeff = double(nbead) / ((hbar * beta) * (hbar * beta));
    const double fac1 = langevin ? 1.0 / std::sqrt(double(nbead)) : 1.0;
    const double fac3 = (langevin && !add_spring_to_forces) ? 0.0 : force_scale;
    CK(cudaMemsetAsync(ctx->pimd_acc, 0, 2 * sizeof(double), ctx->stream));
    // row 0 of cart_to_nmode: the centroid mode's weights
    CK(launch_pimd_springs(nbead, natms, ctx->pimd_mat + (size_t)nbead * nbead, xxx, yyy, zzz, fxx, fyy, fzz, mass,
                           coeff, fac1, fac3, ctx->pimd_acc, ctx->stream));
    double h[2] = {0.0, 0.0};
    CK(cudaMemcpyAsync(h, ctx->pimd_acc, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (energies) {
        energies[0] = 0.5 * coeff * h[0];
        energies[1] = 0.5 * h[1] / force_scale;
    }
    return MBX_OK;
}

extern "C" int mbx_set_lanes(mbx_context* ctx, int lanes) {
    if (!ctx) return MBX_ERR_ARG;
    if (lanes < 1 || lanes > 64) return fail(ctx, MBX_ERR_ARG, "lanes must be 1..64");
    ctx->nlanes = lanes;
    return MBX_OK;
}

extern "C" int mbx_water_step_multi(mbx_context* ctx, int precision, int nbox, const int* imcon, const double* cell,
                                    const int* nw, const double* polar_prm, const double* polr, const double* polr2,
                                    const int* ltype, const int* molecule, double* xxx, double* yyy, double* zzz,
                                    double* dipx, double* dipy, double* dipz, double* fxx, double* fyy, double* fzz,
                                    const double* vxx, const double* vyy, const double* vzz, const double* weight,
                                    double* atomic_energy, double* chge, double* scalars, int* status) {
    if (!ctx) return MBX_ERR_ARG;
    if ((precision != MBX_FP64 && precision != MBX_MIXED) || nbox < 0 || (nbox && (!imcon || !cell || !nw ||
                                                                                     !polar_prm)))
        return fail(ctx, MBX_ERR_ARG, "mbx_water_step_multi: bad argument");
    std::vector<size_t> off(nbox + 1, 0);
    for (int b = 0; b < nbox; ++b) {
        if (nw[b] < 0) return fail(ctx, MBX_ERR_ARG, "mbx_water_step_multi: box %d has %d waters", b, nw[b]);
        if (!polar_prm_ok(polar_prm + 15 * (size_t)b))
            return fail(ctx, MBX_ERR_ARG, "mbx_water_step_multi: bad electrostatics parameters of box %d", b);
        off[b + 1] = off[b] + 4 * (size_t)nw[b];
    }
    if (off[nbox] && (!polr || !polr2 || !xxx || !yyy || !zzz || !dipx || !dipy || !dipz || !fxx || !fyy || !fzz))
        return fail(ctx, MBX_ERR_ARG, "mbx_water_step_multi: bad argument");
    const bool disp = ltype && molecule;
    if (disp && ctx->disp_gen == 0) return fail(ctx, MBX_ERR_ARG, "dispersion asked for before mbx_disp_setup");
    const bool heat = vxx && vyy && vzz && weight;
    const int nl = std::min(ctx->nlanes, std::max(nbox, 1));
    while ((int)ctx->lane.size() < nl) {
        mbx_context* c = nullptr;
        const int rc = mbx_create(&c, ctx->device);
        if (rc) return fail(ctx, rc, "mbx_water_step_multi: creating a lane failed");
        ctx->lane.push_back(c);
    }
    for (int l = 0; l < nl; ++l) {   // the parent's settings and dispersion tables
        mbx_context* c = ctx->lane[l];
        c->limit2 = ctx->limit2;
        c->limit3 = ctx->limit3;
        c->fused = ctx->fused;
        c->polar.precond_sweeps = ctx->polar.precond_sweeps;
        c->polar.final_fp64 = ctx->polar.final_fp64;
        c->polar.list_skin = ctx->polar.list_skin;
        c->polar.spme_order = ctx->polar.spme_order;
        c->polar.spme_spacing = ctx->polar.spme_spacing;
        for (int a = 0; a < 3; ++a) c->polar.spme_grid[a] = ctx->polar.spme_grid[a];
        if (disp && c->disp_gen_seen != ctx->disp_gen) {
            const int rc = mbx_disp_setup(c, ctx->disp_ntypes, ctx->disp_prm_h.data(), ctx->disp_rcut, ctx->disp_delr,
                                          ctx->disp_mxgrid);
            if (rc) return fail(ctx, rc, "mbx_water_step_multi: lane %d: %s", l, c->err);
            c->disp_gen_seen = ctx->disp_gen;
        }
    }
    std::vector<int> order(nbox), st(nbox, MBX_OK);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nw[a] > nw[b]; });
    std::atomic<int> next{0};
    std::mutex err_mu;   // the first lane error goes to the parent context
    std::vector<long> launches(nl, 0);
    auto work = [&](int l) {
        mbx_context* c = ctx->lane[l];
        for (int t; (t = next.fetch_add(1)) < nbox;) {
            const int b = order[t];
            const size_t o = off[b];
            double sc[MBX_NSTEPSCALARS];
            st[b] = mbx_water_step(c, precision, imcon[b], cell + 9 * (size_t)b, nw[b], 4 * nw[b],
                                   polar_prm + 15 * (size_t)b, polr + o, polr2 + o, disp ? ltype + o : nullptr,
                                   disp ? molecule + o : nullptr, xxx + o, yyy + o, zzz + o, dipx + o, dipy + o,
                                   dipz + o, fxx + o, fyy + o, fzz + o, heat ? vxx + o : nullptr,
                                   heat ? vyy + o : nullptr, heat ? vzz + o : nullptr, heat ? weight + o : nullptr,
                                   atomic_energy ? atomic_energy + o : nullptr, chge ? chge + o : nullptr, sc);
            if (scalars) std::memcpy(scalars + MBX_NSTEPSCALARS * (size_t)b, sc, sizeof sc);
            launches[l] += c->launches;
            if (st[b] != MBX_OK && st[b] != MBX_ERR_CONVERGE) {
                std::lock_guard<std::mutex> lk(err_mu);
                if (!ctx->err[0]) std::snprintf(ctx->err, sizeof ctx->err, "box %d: %s", b, c->err);
            }
        }
    };
    ctx->err[0] = 0;
    if (nl == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int l = 0; l < nl; ++l) th.emplace_back(work, l);
        for (auto& t : th) t.join();
    }
    ctx->launches = std::accumulate(launches.begin(), launches.end(), 0L);
    if (status) std::copy(st.begin(), st.end(), status);
    int rc = MBX_OK;
    for (int b = 0; b < nbox && rc == MBX_OK; ++b)
        if (st[b] != MBX_OK && st[b] != MBX_ERR_CONVERGE) rc = st[b];
    if (rc) return rc;
    for (int b = 0; b < nbox; ++b)
        if (st[b] == MBX_ERR_CONVERGE)
            return fail(ctx, MBX_ERR_CONVERGE, "mbx_water_step_multi: dipoles of box %d not converged", b);
    return MBX_OK;
}

extern "C" double mbx_trim(mbx_context* ctx, double keep_bytes) {
    if (!ctx) return -1.0;
    const double held = (double)ctx->polar.held_bytes();
    if (held > keep_bytes) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        ctx->polar.release();
        return held;
    }
    return 0.0;
}

extern "C" int mbx_polar_iterations(const mbx_context* ctx) { return ctx ? ctx->polar.iterations : -1; }

extern "C" long mbx_polar_inner_sweeps(const mbx_context* ctx) { return ctx ? ctx->polar.inner_sweeps : -1; }

extern "C" int mbx_polar_timings(const mbx_context* ctx, float* ms4, long* kvectors) {
    if (!ctx || !ms4) return MBX_ERR_ARG;
    for (int q = 0; q < 4; ++q) ms4[q] = ctx->polar.phase_ms[q];
    if (kvectors) *kvectors = ctx->polar.K_last;
    return MBX_OK;
}

extern "C" int mbx_polar_field_timing(const mbx_context* ctx, double* ms, double* flops, long* launches) {
    if (!ctx) return MBX_ERR_ARG;
    if (ms) *ms = ctx->polar.kf_ms;
    if (flops) *flops = ctx->polar.kf_flops;
    if (launches) *launches = ctx->polar.kf_launches;
    return MBX_OK;
}

extern "C" int mbx_msite_redistribute(int nw, double gamma, double* fxx, double* fyy, double* fzz) {
    if (nw < 0 || (nw && (!fxx || !fyy || !fzz))) return MBX_ERR_ARG;
    for (int i = 0; i < nw; ++i) {   // SOURCE/dlpoly_cmd.f:2585-2601 (standard layout)
        const int m = 3 * nw + i, o = 3 * i;
        double* f[3] = {fxx, fyy, fzz};
        for (int c = 0; c < 3; ++c) {
            f[c][o] = f[c][o] + (1.0 - gamma) * f[c][m];
            f[c][o + 1] = f[c][o + 1] + f[c][m] * gamma / 2.0;
            f[c][o + 2] = f[c][o + 2] + f[c][m] * gamma / 2.0;
        }
    }
    return MBX_OK;
}

extern "C" int mbx_set_fused(mbx_context* ctx, int on) {
    if (!ctx) return MBX_ERR_ARG;
    ctx->fused = on ? 1 : 0;
    return MBX_OK;
}

extern "C" int mbx_set_fused_split(mbx_context* ctx, int dimer_warps) {
    if (!ctx || dimer_warps < 0 || dimer_warps > 11) return MBX_ERR_ARG;
    ctx->fused_split = dimer_warps;
    return MBX_OK;
}

extern "C" int mbx_set_overlap(mbx_context* ctx, int on, int dimer_warps) {
    if (!ctx || dimer_warps < 0 || dimer_warps > 7) return MBX_ERR_ARG;
    ctx->overlap = on ? 1 : 0;
    ctx->overlap_split = dimer_warps;
    return MBX_OK;
}

extern "C" int mbx_set_overlap_terms(mbx_context* ctx, int on) {
    if (!ctx) return MBX_ERR_ARG;
    ctx->overlap_terms = on ? 1 : 0;
    return MBX_OK;
}

extern "C" int mbx_set_final_fp64(mbx_context* ctx, int on) {
    if (!ctx) return MBX_ERR_ARG;
    ctx->polar.final_fp64 = on != 0;
    return MBX_OK;
}

extern "C" int mbx_set_graphs(mbx_context* ctx, int on) {
    if (!ctx) return MBX_ERR_ARG;
    ctx->use_graphs = on ? 1 : 0;
    return MBX_OK;
}

extern "C" long mbx_graph_launches(const mbx_context* ctx) { return ctx ? ctx->graph_replays : -1; }

extern "C" int mbx_mbpol_multi_device(mbx_context* ctx, int precision, int imcon, int nbox, const int* nw_box,
                                      const double* cells, const double* xxx, const double* yyy, const double* zzz,
                                      double* fxx, double* fyy, double* fzz, const double* vxx, const double* vyy,
                                      const double* vzz, const double* weight, double* atomic_energy,
                                      double* scalars) {
    if (!ctx) return MBX_ERR_ARG;
    long natms = 0;
    int rc = prepare_multi(ctx, precision, imcon, nbox, nw_box, cells, &natms);
    if (rc) return rc;
    if (natms > 0 && (!xxx || !yyy || !zzz || !fxx || !fyy || !fzz))
        return fail(ctx, MBX_ERR_ARG, "NULL position/force array");
    const bool heat = vxx && vyy && vzz && weight;
    return run_multi(ctx, precision, nbox, nw_box, xxx, yyy, zzz, fxx, fyy, fzz, heat ? vxx : nullptr,
                     heat ? vyy : nullptr, heat ? vzz : nullptr, heat ? weight : nullptr, atomic_energy, scalars);
}

extern "C" int mbx_mbpol_multi(mbx_context* ctx, int precision, int imcon, int nbox, const int* nw_box,
                               const double* cells, const double* xxx, const double* yyy, const double* zzz,
                               double* fxx, double* fyy, double* fzz, const double* vxx, const double* vyy,
                               const double* vzz, const double* weight, double* atomic_energy, double* scalars) {
    if (!ctx) return MBX_ERR_ARG;
    long natms_l = 0;
    int rc = prepare_multi(ctx, precision, imcon, nbox, nw_box, cells, &natms_l);
    if (rc) return rc;
    const int natms = (int)natms_l;
    if (natms > 0 && (!xxx || !yyy || !zzz || !fxx || !fyy || !fzz))
        return fail(ctx, MBX_ERR_ARG, "NULL position/force array");
    rc = reserve_water(ctx, std::max(natms / 4, 1), std::max(natms, 1));
    if (rc) return rc;
    const bool heat = vxx && vyy && vzz && weight;
    cudaStream_t s = ctx->stream;
    const size_t nb = (size_t)natms * sizeof(double);
    double* d = ctx->atoms;
    double *dx = d, *dy = d + natms, *dz = d + 2 * (size_t)natms;
    double *dvx = d + 3 * (size_t)natms, *dvy = d + 4 * (size_t)natms, *dvz = d + 5 * (size_t)natms;
    double* dm = d + 6 * (size_t)natms;
    double *dfx = d + 7 * (size_t)natms, *dfy = d + 8 * (size_t)natms, *dfz = d + 9 * (size_t)natms;
    double* dae = d + 10 * (size_t)natms;
    if (natms) {
        CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
        if (heat) {
            CK(cudaMemcpyAsync(dvx, vxx, nb, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dvy, vyy, nb, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dvz, vzz, nb, cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(dm, weight, nb, cudaMemcpyHostToDevice, s));
        }
        CK(cudaMemsetAsync(dfx, 0, 3 * nb, s));
        if (atomic_energy) CK(cudaMemsetAsync(dae, 0, nb, s));
    }
    rc = run_multi(ctx, precision, nbox, nw_box, dx, dy, dz, dfx, dfy, dfz, heat ? dvx : nullptr,
                   heat ? dvy : nullptr, heat ? dvz : nullptr, heat ? dm : nullptr, atomic_energy ? dae : nullptr,
                   scalars);
    if (rc || !natms) return rc;
    double* h = host_stage(ctx, 4 * (size_t)natms + 1);
    if (!h) return fail(ctx, MBX_ERR_CUDA, "pinned host staging allocation failed");
    CK(cudaMemcpyAsync(h, dfx, 3 * nb, cudaMemcpyDeviceToHost, s));
    if (atomic_energy) CK(cudaMemcpyAsync(h + 3 * (size_t)natms, dae, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < natms; ++i) {
        fxx[i] += h[i];
        fyy[i] += h[natms + i];
        fzz[i] += h[2 * (size_t)natms + i];
        if (atomic_energy) atomic_energy[i] += h[3 * (size_t)natms + i];
    }
    return MBX_OK;
}

extern "C" int mbx_ps_pes_forces_device(mbx_context* ctx, int imcon, const double* cell, int nang,
                                        const int* listang, int natms, const double* xxx, const double* yyy,
                                        const double* zzz, double* fxx, double* fyy, double* fzz, const double* vxx,
                                        const double* vyy, const double* vzz, double* atomic_energy, double* out) {
    if (!ctx) return MBX_ERR_ARG;
    if (nang < 0 || (nang > 0 && !listang) || !xxx || !yyy || !zzz || !fxx || !fyy || !fzz || natms < 0)
        return fail(ctx, MBX_ERR_ARG, "bad argument");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const bool heat = vxx && vyy && vzz;
    CK(cudaMemsetAsync(ctx->acc, 0, 14 * sizeof(double), s));
    CK(launch_ps_pes(nang, listang, cl, xxx, yyy, zzz, fxx, fyy, fzz, atomic_energy, heat ? vxx : nullptr,
                     heat ? vyy : nullptr, heat ? vzz : nullptr, ctx->acc, s));
    CK(cudaMemcpyAsync(ctx->acc_h, ctx->acc, 14 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (out) std::memcpy(out, ctx->acc_h, 14 * sizeof(double));
    return MBX_OK;
}

extern "C" int mbx_ps_pes_forces(mbx_context* ctx, int imcon, const double* cell, int nang, const int* listang,
                                 int natms, const double* xxx, const double* yyy, const double* zzz, double* fxx,
                                 double* fyy, double* fzz, double* engang, double* virang, double* stress,
                                 const double* vxx, const double* vyy, const double* vzz, double* atomic_energy,
                                 double* jpot) {
    if (!ctx) return MBX_ERR_ARG;
    if (nang < 0 || natms < 0 || !xxx || !yyy || !zzz || !fxx || !fyy || !fzz || !engang || !virang || !stress)
        return fail(ctx, MBX_ERR_ARG, "NULL argument");
    for (int q = 0; q < 3 * nang; ++q)
        if (listang[q] < 1 || listang[q] > natms) return fail(ctx, MBX_ERR_ARG, "listang[%d] out of range", q);
    CK(cudaSetDevice(ctx->device));
    int rc = reserve_water(ctx, std::max((nang + 2) / 3, 1), std::max(natms, 1));
    if (rc) return rc;
    if ((long)3 * nang > 3L * ctx->nw_cap) {
        rc = reserve_water(ctx, nang, std::max(natms, 1));
        if (rc) return rc;
    }
    const bool heat = vxx && vyy && vzz;
    cudaStream_t s = ctx->stream;
    const size_t nb = (size_t)natms * sizeof(double);
    double* d = ctx->atoms;
    double *dx = d, *dy = d + natms, *dz = d + 2 * (size_t)natms;
    double *dvx = d + 3 * (size_t)natms, *dvy = d + 4 * (size_t)natms, *dvz = d + 5 * (size_t)natms;
    double *dfx = d + 7 * (size_t)natms, *dfy = d + 8 * (size_t)natms, *dfz = d + 9 * (size_t)natms;
    double* dae = d + 10 * (size_t)natms;
    if (nang) CK(cudaMemcpyAsync(ctx->list, listang, 3 * (size_t)nang * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
    if (heat) {
        CK(cudaMemcpyAsync(dvx, vxx, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvy, vyy, nb, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dvz, vzz, nb, cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemsetAsync(dfx, 0, 3 * nb, s));
    if (atomic_energy) CK(cudaMemsetAsync(dae, 0, nb, s));
    double out[14];
    rc = mbx_ps_pes_forces_device(ctx, imcon, cell, nang, ctx->list, natms, dx, dy, dz, dfx, dfy, dfz,
                                  heat ? dvx : nullptr, heat ? dvy : nullptr, heat ? dvz : nullptr,
                                  atomic_energy ? dae : nullptr, out);
    if (rc) return rc;
    double* h = host_stage(ctx, 4 * (size_t)natms + 1);
    if (!h) return fail(ctx, MBX_ERR_CUDA, "pinned host staging allocation failed");
    CK(cudaMemcpyAsync(h, dfx, 3 * nb, cudaMemcpyDeviceToHost, s));
    if (atomic_energy) CK(cudaMemcpyAsync(h + 3 * (size_t)natms, dae, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < natms; ++i) {
        fxx[i] += h[i];
        fyy[i] += h[natms + i];
        fzz[i] += h[2 * (size_t)natms + i];
        if (atomic_energy) atomic_energy[i] += h[3 * (size_t)natms + i];
    }
    *engang += out[0];
    *virang += out[1];
    for (int q = 0; q < 9; ++q) stress[q] += out[2 + q];
    if (jpot)
        for (int q = 0; q < 3; ++q) jpot[q] += out[11 + q];
    return MBX_OK;
}

extern "C" int mbx_msites_dms_device(mbx_context* ctx, int imcon, const double* cell, int nttm2,
                                     const int* listttm2, int natms, double gamma, double* xxx, double* yyy,
                                     double* zzz, double* chge, double* dqdr) {
    if (!ctx) return MBX_ERR_ARG;
    if (nttm2 < 0 || nttm2 % 3 || (nttm2 && !listttm2) || !xxx || !yyy || !zzz || natms < 4 * (nttm2 / 3))
        return fail(ctx, MBX_ERR_ARG, "bad argument");
    Cell cl;
    int rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    CK(launch_msites_dms(nttm2 / 3, listttm2, cl, xxx, yyy, zzz, gamma, chge, dqdr, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return MBX_OK;
}

extern "C" int mbx_msites_dms(mbx_context* ctx, int imcon, const double* cell, int nttm2, const int* listttm2,
                              int natms, double gamma, double* xxx, double* yyy, double* zzz, double* chge,
                              double* dqdr) {
    if (!ctx) return MBX_ERR_ARG;
    if (nttm2 < 0 || nttm2 % 3 || !xxx || !yyy || !zzz) return fail(ctx, MBX_ERR_ARG, "bad argument");
    const int nw = nttm2 / 3;
    if (nw == 0) return MBX_OK;
    for (int t = 0; t < nttm2; ++t)
        if (listttm2[t] < 1 || listttm2[t] > natms || (t % 3 && listttm2[t] != listttm2[t - t % 3] + t % 3))
            return fail(ctx, MBX_ERR_ARG, "listttm2[%d]=%d: 1-based, O,H1,H2 consecutive", t, listttm2[t]);
    if (listttm2[nttm2 - 1] + nw > natms) return fail(ctx, MBX_ERR_ARG, "M sites beyond natms");
    CK(cudaSetDevice(ctx->device));
    int rc = reserve_water(ctx, nw, natms);
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    const size_t nb = (size_t)natms * sizeof(double);
    double* d = ctx->atoms;
    double *dx = d, *dy = d + natms, *dz = d + 2 * (size_t)natms, *dq = d + 3 * (size_t)natms;
    double* ddp = d + 4 * (size_t)natms;   // 6*nw <= 6*natms/4 fits in the 7*natms that follow
    CK(cudaMemcpyAsync(ctx->list, listttm2, nttm2 * sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dx, xxx, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dy, yyy, nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dz, zzz, nb, cudaMemcpyHostToDevice, s));
    if (chge) CK(cudaMemcpyAsync(dq, chge, nb, cudaMemcpyHostToDevice, s));
    Cell cl;
    rc = make_cell(ctx, imcon, cell, cl);
    if (rc) return rc;
    CK(launch_msites_dms(nw, ctx->list, cl, dx, dy, dz, gamma, chge ? dq : nullptr, dqdr ? ddp : nullptr, s));
    CK(cudaMemcpyAsync(xxx, dx, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(yyy, dy, nb, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(zzz, dz, nb, cudaMemcpyDeviceToHost, s));
    if (chge) CK(cudaMemcpyAsync(chge, dq, nb, cudaMemcpyDeviceToHost, s));
    if (dqdr) CK(cudaMemcpyAsync(dqdr, ddp, 6 * (size_t)nw * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return MBX_OK;
}

extern "C" int mbx_last_lists(mbx_context* ctx, int* pairs, long cap_pairs, long* npairs, int* trimers,
                              long cap_trimers, long* ntrimers) {
    if (!ctx) return MBX_ERR_ARG;
    if (npairs) *npairs = ctx->npairs;
    if (ntrimers) *ntrimers = ctx->ntrip;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));   // the lists come from the context's stream
    if (pairs && ctx->npairs) {
        const long n = std::min(cap_pairs, ctx->npairs);
        CK(cudaMemcpy(pairs, ctx->pairs, n * sizeof(int2), cudaMemcpyDeviceToHost));
    }
    if (trimers && ctx->ntrip) {
        const long n = std::min(cap_trimers, ctx->ntrip);
        std::vector<int4> t(n);
        CK(cudaMemcpy(t.data(), ctx->trip, n * sizeof(int4), cudaMemcpyDeviceToHost));
        for (long q = 0; q < n; ++q) {
            trimers[3 * q] = t[q].x;
            trimers[3 * q + 1] = t[q].y;
            trimers[3 * q + 2] = t[q].z;
        }
    }
    return MBX_OK;
}

namespace {
int batch_reserve(mbx_context* ctx, size_t bytes) {
    if (bytes > ctx->batch_bytes) {
        if (ctx->batch) cudaFree(ctx->batch);
        ctx->batch = nullptr;
        CK(cudaMalloc(&ctx->batch, bytes));
        ctx->batch_bytes = bytes;
    }
    return MBX_OK;
}
}  // namespace

extern "C" int mbx_2b_poly_batch(mbx_context* ctx, int precision, long n, const double* w1, const double* w2,
                                 double* E, double* g1, double* g2) {
    if (!ctx) return MBX_ERR_ARG;
    if (n < 0 || n > 0x7fffffff) return fail(ctx, MBX_ERR_ARG, "bad n");
    if (n == 0) return MBX_OK;
    if (!w1 || !w2 || !E || !g1 || !g2) return fail(ctx, MBX_ERR_ARG, "NULL argument");
    if (precision != MBX_FP64 && precision != MBX_MIXED) return fail(ctx, MBX_ERR_ARG, "bad precision");
    CK(cudaSetDevice(ctx->device));
    const size_t b9 = 9 * (size_t)n * sizeof(double);
    int rc = batch_reserve(ctx, 4 * b9 + n * sizeof(double));
    if (rc) return rc;
    double *d1 = ctx->batch, *d2 = d1 + 9 * n, *dg1 = d2 + 9 * n, *dg2 = dg1 + 9 * n, *dE = dg2 + 9 * n;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d1, w1, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d2, w2, b9, cudaMemcpyHostToDevice, s));
    CK(launch_2b_direct((int)n, d1, d2, dE, dg1, dg2, precision, s));
    CK(cudaMemcpyAsync(E, dE, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(g1, dg1, b9, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(g2, dg2, b9, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return MBX_OK;
}

extern "C" int mbx_3b_poly_batch(mbx_context* ctx, int precision, long n, const double* w1, const double* w2,
                                 const double* w3, double* E, double* g1, double* g2, double* g3) {
    if (!ctx) return MBX_ERR_ARG;
    if (n < 0 || n > 0x7fffffff) return fail(ctx, MBX_ERR_ARG, "bad n");
    if (n == 0) return MBX_OK;
    if (!w1 || !w2 || !w3 || !E || !g1 || !g2 || !g3) return fail(ctx, MBX_ERR_ARG, "NULL argument");
    if (precision != MBX_FP64 && precision != MBX_MIXED) return fail(ctx, MBX_ERR_ARG, "bad precision");
    CK(cudaSetDevice(ctx->device));
    const size_t b9 = 9 * (size_t)n * sizeof(double);
    int rc = batch_reserve(ctx, 6 * b9 + n * sizeof(double));
    if (rc) return rc;
    double *d1 = ctx->batch, *d2 = d1 + 9 * n, *d3 = d2 + 9 * n, *dg1 = d3 + 9 * n, *dg2 = dg1 + 9 * n,
           *dg3 = dg2 + 9 * n, *dE = dg3 + 9 * n;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d1, w1, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d2, w2, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d3, w3, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dg1, g1, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dg2, g2, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dg3, g3, b9, cudaMemcpyHostToDevice, s));
    CK(launch_3b_direct((int)n, d1, d2, d3, dE, dg1, dg2, dg3, precision, s));
    CK(cudaMemcpyAsync(E, dE, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(g1, dg1, b9, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(g2, dg2, b9, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(g3, dg3, b9, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return MBX_OK;
}

// ---------------------------------------------------------------------------
// Per-call drop-ins: one process-wide context per device, created on first use.
namespace {
std::mutex g_mu;
mbx_context* g_ctx[64] = {nullptr};

mbx_context* global_ctx() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        std::fprintf(stderr, "libmbx: no CUDA device\n");
        std::abort();
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ctx[dev] && mbx_create(&g_ctx[dev], dev) != MBX_OK) {
        std::fprintf(stderr, "libmbx: cannot create a context on device %d\n", dev);
        std::abort();
    }
    return g_ctx[dev];
}
}  // namespace

extern "C" int mbx_2b_force_matrix_batch(mbx_context* ctx, long n, const double* w1, const double* w2, double* fm) {
    if (!ctx) return MBX_ERR_ARG;
    if (n < 0 || n > 0x7fffffff) return fail(ctx, MBX_ERR_ARG, "bad n");
    if (n == 0) return MBX_OK;
    if (!w1 || !w2 || !fm) return fail(ctx, MBX_ERR_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    const size_t b9 = 9 * (size_t)n * sizeof(double), bf = 108 * (size_t)n * sizeof(double);
    int rc = batch_reserve(ctx, 2 * b9 + bf);
    if (rc) return rc;
    double *d1 = ctx->batch, *d2 = d1 + 9 * n, *df = d2 + 9 * n;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d1, w1, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d2, w2, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(df, fm, bf, cudaMemcpyHostToDevice, s));   // entries not written keep their values
    CK(launch_2b_fm((int)n, d1, d2, df, s));
    CK(cudaMemcpyAsync(fm, df, bf, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return MBX_OK;
}

extern "C" int mbx_3b_force_matrix_batch(mbx_context* ctx, long n, const double* w1, const double* w2,
                                         const double* w3, double* fm) {
    if (!ctx) return MBX_ERR_ARG;
    if (n < 0 || n > 0x7fffffff) return fail(ctx, MBX_ERR_ARG, "bad n");
    if (n == 0) return MBX_OK;
    if (!w1 || !w2 || !w3 || !fm) return fail(ctx, MBX_ERR_ARG, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    const size_t b9 = 9 * (size_t)n * sizeof(double), bf = 243 * (size_t)n * sizeof(double);
    int rc = batch_reserve(ctx, 3 * b9 + bf);
    if (rc) return rc;
    double *d1 = ctx->batch, *d2 = d1 + 9 * n, *d3 = d2 + 9 * n, *df = d3 + 9 * n;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(d1, w1, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d2, w2, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d3, w3, b9, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(df, fm, bf, cudaMemcpyHostToDevice, s));
    CK(launch_3b_fm((int)n, d1, d2, d3, df, s));
    CK(cudaMemcpyAsync(fm, df, bf, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return MBX_OK;
}

extern "C" void mbpol_2b_poly_(const double* w1, const double* w2, double* E, double* g1, double* g2,
                               double* force_matrix) {
    mbx_context* c = global_ctx();
    std::lock_guard<std::mutex> lk(g_mu);
    if (force_matrix && mbx_2b_force_matrix_batch(c, 1, w1, w2, force_matrix) != MBX_OK) {
        std::fprintf(stderr, "mbpol_2b_poly_: %s\n", mbx_error(c));
        std::abort();
    }
    if (mbx_2b_poly_batch(c, MBX_FP64, 1, w1, w2, E, g1, g2) != MBX_OK) {
        std::fprintf(stderr, "mbpol_2b_poly_: %s\n", mbx_error(c));
        std::abort();
    }
}

extern "C" void mbpol_3b_poly_(const double* w1, const double* w2, const double* w3, double* E, double* g1,
                               double* g2, double* g3, double* force_matrix) {
    mbx_context* c = global_ctx();
    std::lock_guard<std::mutex> lk(g_mu);
    if (force_matrix && mbx_3b_force_matrix_batch(c, 1, w1, w2, w3, force_matrix) != MBX_OK) {
        std::fprintf(stderr, "mbpol_3b_poly_: %s\n", mbx_error(c));
        std::abort();
    }
    if (mbx_3b_poly_batch(c, MBX_FP64, 1, w1, w2, w3, E, g1, g2, g3) != MBX_OK) {
        std::fprintf(stderr, "mbpol_3b_poly_: %s\n", mbx_error(c));
        std::abort();
    }
}

extern "C" void mbpol_2b_cutoff_(double* r) { *r = kR2f; }
extern "C" void mbpol_3b_cutoff_(double* r) { *r = kR3f; }
