// Continuous-batching force server: independent water boxes (path-integral beads,
// separate simulations, remote clients) are evaluated concurrently on one GPU.
//
// A fixed set of worker slots each own an mbx_context (its own CUDA stream and device
// buffers, kept between requests as a warm start for memory).  Requests enter a FIFO
// queue; the head is admitted to a free slot as soon as its device-memory footprint
// fits the server's budget, so requests that arrive while others run start as slots
// and memory free up, and their kernels overlap on the device.  Each request runs the
// full path: the 1-body term, then the 2B/3B MB-pol terms with the heat current.
// The reference has no serving loop; its i-PI client (SOURCE/ipi.f90:33-198) answers
// one force request at a time.
#include "../../include/mbx.h"

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long id = 0;
    int precision = MBX_MIXED;
    int imcon = 1;
    double cell[9] = {0};
    int nw = 0;
    int natms = 0;
    std::vector<double> x, y, z, vx, vy, vz, mass;
    bool heat = false;
    // results
    std::vector<double> fx, fy, fz, ae;
    double scalars[MBX_NSCALARS + 14] = {0};
    int status = MBX_OK;
    bool done = false;
    size_t footprint = 0;
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

}  // namespace

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
                cv_work.wait(lk, [&] {
                    return stop || (!queue.empty() && in_use + queue.front()->footprint <= budget) ||
                           (!queue.empty() && in_use == 0);   // an oversized request runs alone
                });
                if (stop && queue.empty()) break;
                if (queue.empty()) continue;
                r = queue.front();
                queue.pop_front();
                in_use += r->footprint;
            }
            r->t_start = Clock::now();
            run(ctx, *r);
            r->t_done = Clock::now();
            {
                std::lock_guard<std::mutex> lk(mu);
                in_use -= r->footprint;
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
        // 1-body + MB-pol in one call; scalars: the MB-pol block, then the 1-body block
        double sc[MBX_NWATERSCALARS];
        r.status = mbx_water_forces(ctx, r.precision, r.imcon, r.cell, 3 * nw, lst.data(), nw, ang.data(), nullptr,
                                    nullptr, n, r.x.data(), r.y.data(), r.z.data(), r.fx.data(), r.fy.data(),
                                    r.fz.data(), r.heat ? r.vx.data() : nullptr, r.heat ? r.vy.data() : nullptr,
                                    r.heat ? r.vz.data() : nullptr, r.heat ? r.mass.data() : nullptr, r.ae.data(),
                                    sc);
        std::memcpy(r.scalars, sc, sizeof r.scalars);
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
        if (scalars) std::memcpy(scalars, r->scalars, sizeof r->scalars);
    }
    if (times) {
        times[0] = std::chrono::duration<double>(r->t_start - r->t_submit).count();   // queueing
        times[1] = std::chrono::duration<double>(r->t_done - r->t_start).count();     // on a slot
        times[2] = std::chrono::duration<double>(r->t_done - r->t_submit).count();    // latency
    }
    return r->status;
}

extern "C" const char* mbx_server_error(const mbx_server* s) { return s ? s->err : "no server"; }
