// Continuous-batching force server: independent water boxes (path-integral beads,
// separate simulations, remote clients) are evaluated concurrently on one GPU.
//
// A fixed set of worker slots each own an mbx_context (its own CUDA stream and device
// buffers, kept between requests as a warm start for memory).  Requests enter a FIFO
// queue; the head is admitted to a free slot as soon as its device-memory footprint
// fits the server's budget, so requests that arrive while others run start as slots
// and memory free up, and their kernels overlap on the device.  A request runs either the
// 1-body + 2B/3B MB-pol terms with the heat current (mbx_server_submit), or the whole force
// evaluation with the TTM4-F electrostatics (mbx_server_submit_step), whose induced
// dipoles start from the last converged ones of the same client; a client's requests run
// one at a time, in order.
// The reference has no serving loop; its i-PI client (SOURCE/ipi.f90:33-198) answers
// one force request at a time.
#include "../../include/mbx.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long id = 0;
    bool step = false;        // the whole force evaluation (mbx_water_step) with electrostatics
    long client = 0;          // step requests: whose dipoles warm-start this one
    int precision = MBX_MIXED;
    int imcon = 1;
    double cell[9] = {0};
    int nw = 0;
    int natms = 0;
    std::vector<double> x, y, z, vx, vy, vz, mass;
    bool heat = false;
    // results
    std::vector<double> fx, fy, fz, ae, dip;
    double scalars[MBX_NSTEPSCALARS] = {0};
    int status = MBX_OK;
    bool done = false;
    size_t footprint = 0;
    int spme_order = 0;       // step requests: k space (0: Ewald; else SPME of this order)
    double spme_spacing = 0.8;
    Clock::time_point t_submit, t_start, t_done;
};

// Device bytes one request needs (context buffers and lists), a conservative estimate.
size_t footprint_bytes(int nw) {
    const size_t natms = 4 * (size_t)nw;
    return 11 * natms * 8          // staging of positions/velocities/masses/forces/energies
           + 9 * (size_t)nw * 8    // monomers
           + (size_t)nw * (64 + 48 + 8) * 4   // neighbour lists and counters
           + (size_t)nw * 40 * 8 * 2          // dimers (and hand-off list)
           + (size_t)nw * 160 * 16 * 2        // trimers (and hand-off list)
           + (1u << 20);                      // scan/sort workspace
}

// Ewald settings of a step request, from its cell: rcut 9 A or less than half the narrowest
// width, alpha * rcut = 2.7 (config 0's 0.3 x 9), kmax keeping config 0's k-space cutoff
// 2 pi kmax / L per unit of alpha (kmax 8 at alpha 0.3, L 19.73 A); the vmbpol Thole
// settings, dipoles to 1e-8 D.
void step_params(const double* cell, double* prm, int* K_est) {
    double w[3];
    {
        const double* a = cell;
        const double bxc[3] = {a[4] * a[8] - a[5] * a[7], a[5] * a[6] - a[3] * a[8], a[3] * a[7] - a[4] * a[6]};
        const double cxa[3] = {a[7] * a[2] - a[1] * a[8], a[0] * a[8] - a[2] * a[6], a[1] * a[6] - a[0] * a[7]};
        const double axb[3] = {a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5], a[0] * a[4] - a[1] * a[3]};
        const double v = std::fabs(a[0] * bxc[0] + a[1] * bxc[1] + a[2] * bxc[2]);
        w[0] = v / std::sqrt(bxc[0] * bxc[0] + bxc[1] * bxc[1] + bxc[2] * bxc[2]);
        w[1] = v / std::sqrt(cxa[0] * cxa[0] + cxa[1] * cxa[1] + cxa[2] * cxa[2]);
        w[2] = v / std::sqrt(axb[0] * axb[0] + axb[1] * axb[1] + axb[2] * axb[2]);
    }
    const double wmin = std::min(w[0], std::min(w[1], w[2]));
    const double rcut = std::min(9.0, 0.49 * wmin);
    const double alpha = 2.7 / rcut;
    int km[3];
    double K = 2.6;   // the half ball of radius 1.05 kmax holds about 2.42 kmax^3 k vectors
    for (int c = 0; c < 3; ++c) {
        km[c] = std::max(1, (int)std::ceil(8.0 * alpha * w[c] / (0.3 * 19.73) - 1e-9));
        K *= km[c] + 1;
    }
    const double p[15] = {alpha, rcut, 1.0, 1e-8 / 4.803239, 0.3, 0.055, 0.626, 0.055, 0.4, 0.4, 0.426706882,
                          (double)km[0], (double)km[1], (double)km[2], 22581};
    std::memcpy(prm, p, sizeof p);
    *K_est = (int)std::min(K, (double)(1L << 30));   // an upper bound
}

// Extra device bytes of a step request: the exp(ik.r) tables (FP64 and FP32), the site pair
// list with its FP64 and FP32 tensors, and the per-site work arrays.
size_t step_footprint_bytes(int nw, int K) {
    const size_t n = 4 * (size_t)nw;
    return (size_t)K * n * 24 + n * 1024 * (4 + 48 + 24) + n * 300 * 8 + (size_t)K * 256 + (8u << 20);
}

// The SPME grids of a step request instead of the phase tables: nine FP64 and one FP32
// complex grids plus the influence functions, at the grid the spacing gives the cell.
size_t spme_grid_bytes(const double* cell, double spacing) {
    int g[3] = {0, 0, 0};
    if (mbx_spme_grid_for_cell(cell, spacing, g)) return 0;
    const size_t ng = (size_t)g[0] * g[1] * g[2];
    return ng * (9 * 16 + 8 + 12);
}

}  // namespace

extern "C" void mbx_polar_params_for_cell(const double* cell, double* prm) {
    int K = 0;
    step_params(cell, prm, &K);
}

struct mbx_server {
    int device = 0;
    size_t budget = 0;
    size_t in_use = 0;
    long next_id = 1;
    bool stop = false;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::map<long, std::shared_ptr<Request>> live;
    std::vector<std::thread> workers;
    std::map<long, std::vector<double>> client_dip;   // last converged dipoles per client
    int spme_order = 0;                                // k space of step requests (0: Ewald)
    double spme_spacing = 0.8;
    std::set<long> busy;                               // clients with a request on a slot
    long completed = 0;
    char err[256] = {0};

    void worker(int slot) {
        mbx_context* ctx = nullptr;
        if (mbx_create(&ctx, device) != MBX_OK) {
            std::lock_guard<std::mutex> lk(mu);
            std::snprintf(err, sizeof err, "slot %d: mbx_create failed", slot);
            return;
        }
        for (;;) {
            std::shared_ptr<Request> r;
            {
                std::unique_lock<std::mutex> lk(mu);
                // the first queued request whose client has none on a slot, once its footprint
                // fits (an oversized request runs alone)
                auto pick = [&]() -> std::deque<std::shared_ptr<Request>>::iterator {
                    for (auto it = queue.begin(); it != queue.end(); ++it) {
                        if ((*it)->step && busy.count((*it)->client)) continue;
                        if (in_use + (*it)->footprint <= budget || in_use == 0) return it;
                        return queue.end();   // arrival order: nothing overtakes a waiting request
                    }
                    return queue.end();
                };
                cv_work.wait(lk, [&] { return stop || pick() != queue.end(); });
                if (stop && queue.empty()) break;
                auto it = pick();
                if (it == queue.end()) continue;
                r = *it;
                queue.erase(it);
                in_use += r->footprint;
                if (r->step) {
                    busy.insert(r->client);
                    auto d = client_dip.find(r->client);
                    if (d != client_dip.end() && d->second.size() == 3 * (size_t)r->natms) r->dip = d->second;
                    else r->dip.assign(3 * (size_t)r->natms, 0.0);
                }
            }
            r->t_start = Clock::now();
            if (r->step) mbx_set_spme(ctx, r->spme_order, r->spme_spacing, nullptr);
            run(ctx, *r);
            r->t_done = Clock::now();
            {
                std::lock_guard<std::mutex> lk(mu);
                if (r->status != MBX_OK && !err[0])   // the first failure explains the rest
                    std::snprintf(err, sizeof err, "request %ld (%d waters): %s", r->id, r->nw, mbx_error(ctx));
                in_use -= r->footprint;
                if (r->step) {
                    if (r->status == MBX_OK) client_dip[r->client] = r->dip;
                    busy.erase(r->client);
                }
                r->done = true;
                ++completed;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
        mbx_destroy(ctx);
    }

    static void run(mbx_context* ctx, Request& r) {
        const int n = r.natms, nw = r.nw;
        r.fx.assign(n, 0.0);
        r.fy.assign(n, 0.0);
        r.fz.assign(n, 0.0);
        r.ae.assign(n, 0.0);
        std::vector<int> lst(3 * (size_t)nw), ang(3 * (size_t)nw);
        for (int t = 0; t < 3 * nw; ++t) lst[t] = t + 1;
        for (int i = 0; i < nw; ++i) {
            ang[3 * i] = 3 * i + 2;
            ang[3 * i + 1] = 3 * i + 1;
            ang[3 * i + 2] = 3 * i + 3;
        }
        if (r.step) {
            // the whole force evaluation; the dipoles start from the client's last ones
            double prm[15];
            int K = 0;
            step_params(r.cell, prm, &K);
            std::vector<double> polr(n), polr2(n);
            for (int i = 0; i < n; ++i) {
                const bool m = i >= 3 * nw;
                const bool o = !m && i % 3 == 0;
                polr[i] = (m || o) ? 1.310 : 0.294;
                polr2[i] = m ? 0.0 : polr[i];
            }
            double* d = r.dip.data();
            r.status = mbx_water_step(ctx, r.precision, r.imcon, r.cell, nw, n, prm, polr.data(), polr2.data(), nullptr,
                                      nullptr, r.x.data(), r.y.data(), r.z.data(), d, d + n, d + 2 * (size_t)n,
                                      r.fx.data(), r.fy.data(), r.fz.data(), r.heat ? r.vx.data() : nullptr,
                                      r.heat ? r.vy.data() : nullptr, r.heat ? r.vz.data() : nullptr,
                                      r.heat ? r.mass.data() : nullptr, r.ae.data(), nullptr, r.scalars);
            // admission counts a request's footprint only while it runs: return the big
            // electrostatics buffers (phase tables grow with k vectors x sites)
            mbx_trim(ctx, 1e9);
            return;
        }
        // 1-body + MB-pol in one call; scalars: the MB-pol block, then the 1-body block
        double sc[MBX_NWATERSCALARS];
        r.status = mbx_water_forces(ctx, r.precision, r.imcon, r.cell, 3 * nw, lst.data(), nw, ang.data(), nullptr,
                                    nullptr, n, r.x.data(), r.y.data(), r.z.data(), r.fx.data(), r.fy.data(),
                                    r.fz.data(), r.heat ? r.vx.data() : nullptr, r.heat ? r.vy.data() : nullptr,
                                    r.heat ? r.vz.data() : nullptr, r.heat ? r.mass.data() : nullptr, r.ae.data(),
                                    sc);
        std::memcpy(r.scalars, sc, (MBX_NSCALARS + 14) * sizeof(double));
    }
};

extern "C" int mbx_server_create(mbx_server** out, int device, int slots, double budget_bytes) {
    if (!out || slots < 1 || slots > 64 || !(budget_bytes > 0)) return MBX_ERR_ARG;
    mbx_server* s = new mbx_server();
    s->device = device;
    s->budget = (size_t)budget_bytes;
    for (int k = 0; k < slots; ++k) s->workers.emplace_back([s, k] { s->worker(k); });
    *out = s;
    return MBX_OK;
}

extern "C" int mbx_server_set_spme(mbx_server* s, int order, double spacing) {
    if (!s || (order != 0 && (order < 4 || order > 8)) || (order && !(spacing > 0.05 && spacing < 100.0)))
        return MBX_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->spme_order = order;
    s->spme_spacing = spacing;
    return MBX_OK;
}

extern "C" void mbx_server_destroy(mbx_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    delete s;
}

extern "C" long mbx_server_submit(mbx_server* s, int precision, int imcon, const double* cell, int nw, int natms,
                                  const double* xxx, const double* yyy, const double* zzz, const double* vxx,
                                  const double* vyy, const double* vzz, const double* weight) {
    if (!s || !cell || nw < 0 || natms < 3 * nw || !xxx || !yyy || !zzz) return -MBX_ERR_ARG;
    if (precision != MBX_FP64 && precision != MBX_MIXED) return -MBX_ERR_ARG;
    auto r = std::make_shared<Request>();
    r->precision = precision;
    r->imcon = imcon;
    std::memcpy(r->cell, cell, sizeof r->cell);
    r->nw = nw;
    r->natms = natms;
    r->x.assign(xxx, xxx + natms);
    r->y.assign(yyy, yyy + natms);
    r->z.assign(zzz, zzz + natms);
    r->heat = vxx && vyy && vzz && weight;
    if (r->heat) {
        r->vx.assign(vxx, vxx + natms);
        r->vy.assign(vyy, vyy + natms);
        r->vz.assign(vzz, vzz + natms);
        r->mass.assign(weight, weight + natms);
    }
    r->footprint = footprint_bytes(nw);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        s->queue.push_back(r);
        s->live[r->id] = r;
    }
    s->cv_work.notify_all();
    return r->id;
}

extern "C" long mbx_server_submit_step(mbx_server* s, int precision, long client, int imcon, const double* cell,
                                       int nw, const double* xxx, const double* yyy, const double* zzz,
                                       const double* vxx, const double* vyy, const double* vzz,
                                       const double* weight) {
    const int natms = 4 * nw;
    if (!s || !cell || nw < 1 || !xxx || !yyy || !zzz) return -MBX_ERR_ARG;
    if (precision != MBX_FP64 && precision != MBX_MIXED) return -MBX_ERR_ARG;
    auto r = std::make_shared<Request>();
    r->step = true;
    r->client = client;
    r->precision = precision;
    r->imcon = imcon;
    std::memcpy(r->cell, cell, sizeof r->cell);
    r->nw = nw;
    r->natms = natms;
    r->x.assign(xxx, xxx + natms);
    r->y.assign(yyy, yyy + natms);
    r->z.assign(zzz, zzz + natms);
    r->heat = vxx && vyy && vzz && weight;
    if (r->heat) {
        r->vx.assign(vxx, vxx + natms);
        r->vy.assign(vyy, vyy + natms);
        r->vz.assign(vzz, vzz + natms);
        r->mass.assign(weight, weight + natms);
    }
    double prm[15];
    int K = 0;
    step_params(cell, prm, &K);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->spme_order = s->spme_order;
        r->spme_spacing = s->spme_spacing;
    }
    r->footprint = footprint_bytes(nw) + (r->spme_order ? step_footprint_bytes(nw, 0) + spme_grid_bytes(cell, r->spme_spacing)
                                                        : step_footprint_bytes(nw, K));
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        s->queue.push_back(r);
        s->live[r->id] = r;
    }
    s->cv_work.notify_all();
    return r->id;
}

extern "C" int mbx_server_wait_step(mbx_server* s, long id, double* fxx, double* fyy, double* fzz,
                                    double* atomic_energy, double* dipoles, double* scalars, double* times) {
    if (!s) return MBX_ERR_ARG;
    std::shared_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->live.find(id);
        if (it == s->live.end() || !it->second->step) return MBX_ERR_ARG;
        r = it->second;
        s->cv_done.wait(lk, [&] { return r->done; });
        s->live.erase(id);
    }
    const int n = r->natms;
    if (r->status == MBX_OK) {
        if (fxx) std::memcpy(fxx, r->fx.data(), n * sizeof(double));
        if (fyy) std::memcpy(fyy, r->fy.data(), n * sizeof(double));
        if (fzz) std::memcpy(fzz, r->fz.data(), n * sizeof(double));
        if (atomic_energy) std::memcpy(atomic_energy, r->ae.data(), n * sizeof(double));
        if (dipoles) std::memcpy(dipoles, r->dip.data(), 3 * (size_t)n * sizeof(double));
        if (scalars) std::memcpy(scalars, r->scalars, sizeof r->scalars);
    }
    if (times) {
        times[0] = std::chrono::duration<double>(r->t_start - r->t_submit).count();
        times[1] = std::chrono::duration<double>(r->t_done - r->t_start).count();
        times[2] = std::chrono::duration<double>(r->t_done - r->t_submit).count();
    }
    return r->status;
}

extern "C" int mbx_server_wait(mbx_server* s, long id, double* fxx, double* fyy, double* fzz, double* atomic_energy,
                               double* scalars, double* times) {
    if (!s) return MBX_ERR_ARG;
    std::shared_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->live.find(id);
        if (it == s->live.end()) return MBX_ERR_ARG;
        r = it->second;
        s->cv_done.wait(lk, [&] { return r->done; });
        s->live.erase(id);
    }
    const int n = r->natms;
    if (r->status == MBX_OK) {
        if (fxx) std::memcpy(fxx, r->fx.data(), n * sizeof(double));
        if (fyy) std::memcpy(fyy, r->fy.data(), n * sizeof(double));
        if (fzz) std::memcpy(fzz, r->fz.data(), n * sizeof(double));
        if (atomic_energy) std::memcpy(atomic_energy, r->ae.data(), n * sizeof(double));
        if (scalars) std::memcpy(scalars, r->scalars, (MBX_NSCALARS + 14) * sizeof(double));
    }
    if (times) {
        times[0] = std::chrono::duration<double>(r->t_start - r->t_submit).count();   // queueing
        times[1] = std::chrono::duration<double>(r->t_done - r->t_start).count();     // on a slot
        times[2] = std::chrono::duration<double>(r->t_done - r->t_submit).count();    // latency
    }
    return r->status;
}

extern "C" const char* mbx_server_error(const mbx_server* s) { return s ? s->err : "no server"; }
