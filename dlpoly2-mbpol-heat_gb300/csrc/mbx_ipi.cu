// i-PI driver mode: the reference's IPI_INIT / IPI_STEP (SOURCE/ipi.f90:33-198) over its
// socket wrapper (SOURCE/sockets.c).  The client connects to an i-PI server and answers
// its messages:
//   STATUS   -> HAVEDATA (results waiting), READY (initialised), else NEEDINIT
//   INIT     <- replica index (int32), parameter length (int32), parameter string
//   POSDATA  <- cell h (9 doubles), its inverse (9), atoms (int32), positions (3 per atom),
//              in bohr; the configuration is evaluated before the next message is read
//   GETFORCE -> FORCEREADY, energy, atoms, forces (3 per atom), virial (9), then the water
//              dipoles as text (length, bytes), all in atomic units
//   EXIT     -> the loop ends (the reference stops on any other message).
// Unit factors are the reference's single-precision REAL parameters (SOURCE/ipi.f90:72-77),
// promoted to double where they multiply, as there.  The cell and virial are transposed as
// the reference's reshape/transpose pair does.  The dipole text holds, per water, the
// dipole of its DMS charges (hydrogens imaged next to the oxygen) plus its sites' induced
// dipoles, in Debye (SOURCE/dlpoly_cmd.f:2720-2752, SOURCE/qdetermine.f90:280-307), written
// as blank-separated numbers with 17 significant digits (the reference uses Fortran
// list-directed output, whose layout depends on the compiler).
#include "../../include/mbx.h"
#include "mbx_kernels.cuh"

#include <netdb.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <sys/socket.h>
#include <sys/un.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

using mbx::Cell;

namespace {

const double kBohrA = (double)0.52917721067f;                      // conv_length_a_au
const double kDlpolyHa = (double)3.8087989e-06f;                   // conv_energy_dlpoly_au
const double kKcalRatio = (double)(float)((double)418.6799938f / 418.4);   // cons_ratio
const double kEatd = 4.803239;                                     // Debye per e Angstrom

bool read_all(int fd, void* p, size_t n) {
    char* c = static_cast<char*>(p);
    while (n > 0) {
        const ssize_t r = ::read(fd, c, n);
        if (r <= 0) return false;
        c += r;
        n -= (size_t)r;
    }
    return true;
}

bool write_all(int fd, const void* p, size_t n) {
    const char* c = static_cast<const char*>(p);
    while (n > 0) {
        const ssize_t r = ::write(fd, c, n);
        if (r <= 0) return false;
        c += r;
        n -= (size_t)r;
    }
    return true;
}

// "inet:host:port" or "unix:name:port" as the reference parses it (host between the first
// and the last colon, port after the last; a unix socket is /tmp/ipi_<name>, or
// <dir>/ipi_<name> with the environment variable MBX_IPI_UNIX_DIR set), or "host:port"
// (inet).
int open_socket(const char* address, int* fd, std::string& err) {
    const std::string a = address ? address : "";
    const size_t first = a.find(':'), last = a.rfind(':');
    if (first == std::string::npos) {
        err = "i-PI address must be inet:host:port, unix:name:port or host:port";
        return MBX_ERR_ARG;
    }
    std::string kind = "inet", host, port;
    if (first == last) {
        host = a.substr(0, first);
        port = a.substr(last + 1);
    } else {
        kind = a.substr(0, first);
        host = a.substr(first + 1, last - first - 1);
        port = a.substr(last + 1);
    }
    if (kind == "unix") {
        sockaddr_un sa;
        std::memset(&sa, 0, sizeof sa);
        sa.sun_family = AF_UNIX;
        const char* dir = std::getenv("MBX_IPI_UNIX_DIR");
        const std::string path = std::string(dir && *dir ? dir : "/tmp") + "/ipi_" + host;
        if (path.size() >= sizeof sa.sun_path) {
            err = "unix socket path too long";
            return MBX_ERR_ARG;
        }
        std::memcpy(sa.sun_path, path.c_str(), path.size());
        const int s = ::socket(AF_UNIX, SOCK_STREAM, 0);
        if (s < 0 || ::connect(s, reinterpret_cast<sockaddr*>(&sa), sizeof sa) < 0) {
            if (s >= 0) ::close(s);
            err = "cannot connect to unix socket " + path;
            return MBX_ERR_ARG;
        }
        *fd = s;
        return MBX_OK;
    }
    addrinfo hints, *res = nullptr;
    std::memset(&hints, 0, sizeof hints);
    hints.ai_socktype = SOCK_STREAM;
    hints.ai_family = AF_UNSPEC;
    if (::getaddrinfo(host.c_str(), port.c_str(), &hints, &res) != 0 || !res) {
        err = "cannot resolve i-PI host " + host + ":" + port;
        return MBX_ERR_ARG;
    }
    int s = -1;
    for (addrinfo* r = res; r; r = r->ai_next) {
        s = ::socket(r->ai_family, r->ai_socktype, r->ai_protocol);
        if (s < 0) continue;
        if (::connect(s, r->ai_addr, r->ai_addrlen) == 0) {
            // replies are request-sized: no Nagle delay behind the peer's delayed ACKs
            const int one = 1;
            ::setsockopt(s, IPPROTO_TCP, TCP_NODELAY, &one, sizeof one);
            break;
        }
        ::close(s);
        s = -1;
    }
    ::freeaddrinfo(res);
    if (s < 0) {
        err = "cannot connect to i-PI server " + host + ":" + port;
        return MBX_ERR_ARG;
    }
    *fd = s;
    return MBX_OK;
}

std::string header_text(const char* h) {
    std::string t(h, 12);
    while (!t.empty() && (t.back() == ' ' || t.back() == '\0')) t.pop_back();
    return t;
}

bool send_header(int fd, const char* text) {
    char h[12];
    std::memset(h, ' ', sizeof h);
    std::memcpy(h, text, std::strlen(text));
    return write_all(fd, h, sizeof h);
}

// Inverse of the cell matrix (columns a, b, c in DL_POLY's cell(9)), stored as DL_POLY's
// invert does (rc[i + 3j]).
void cell_inverse(const double* a, double* b) {
    b[0] = a[4] * a[8] - a[5] * a[7];
    b[1] = a[2] * a[7] - a[1] * a[8];
    b[2] = a[1] * a[5] - a[2] * a[4];
    b[3] = a[5] * a[6] - a[3] * a[8];
    b[4] = a[0] * a[8] - a[2] * a[6];
    b[5] = a[2] * a[3] - a[0] * a[5];
    b[6] = a[3] * a[7] - a[4] * a[6];
    b[7] = a[1] * a[6] - a[0] * a[7];
    b[8] = a[0] * a[4] - a[1] * a[3];
    const double det = a[0] * b[0] + a[3] * b[1] + a[6] * b[2];
    const double r = det != 0.0 ? 1.0 / det : 0.0;
    for (int i = 0; i < 9; ++i) b[i] *= r;
}

// The minimum image of d through fractional coordinates rounded half away from zero
// (images with imcon 3; the same vector as imcon 1 and 2 for a diagonal cell).
void min_image_host(const Cell& cl, double* d) {
    const double* r = cl.rc;
    double s[3] = {r[0] * d[0] + r[3] * d[1] + r[6] * d[2], r[1] * d[0] + r[4] * d[1] + r[7] * d[2],
                   r[2] * d[0] + r[5] * d[1] + r[8] * d[2]};
    for (double& v : s) v -= std::round(v);
    for (int c = 0; c < 3; ++c) d[c] = cl.c[c] * s[0] + cl.c[3 + c] * s[1] + cl.c[6 + c] * s[2];
}

}  // namespace

extern "C" int mbx_ipi_run_callback(const char* address, mbx_ipi_force_fn fn, void* user, long max_steps,
                                    long* steps_done, char* err, int errlen) {
    auto fail = [&](int code, const std::string& msg) {
        if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", msg.c_str());
        return code;
    };
    if (steps_done) *steps_done = 0;
    if (!fn) return fail(MBX_ERR_ARG, "no force callback");
    int fd = -1;
    std::string msg;
    int rc = open_socket(address, &fd, msg);
    if (rc) return fail(rc, msg);
    bool hasdata = false, imginit = false;
    int replica = -1, nat = 0;
    double pot = 0.0;
    std::vector<double> forces, virial(9), dip;
    std::string diptext;
    long steps = 0;
    rc = MBX_OK;
    for (;;) {
        char h[12];
        if (!read_all(fd, h, sizeof h)) {
            rc = fail(MBX_ERR_ARG, "i-PI server closed the connection");
            break;
        }
        const std::string t = header_text(h);
        bool ok = true;
        if (t == "STATUS") {
            ok = send_header(fd, hasdata ? "HAVEDATA" : (imginit ? "READY" : "NEEDINIT"));
        } else if (t == "INIT") {
            int32_t rid = 0, len = 0;
            ok = read_all(fd, &rid, 4) && read_all(fd, &len, 4) && len >= 0 && len <= (1 << 24);
            std::vector<char> par(ok ? (size_t)len : 0);
            ok = ok && (len == 0 || read_all(fd, par.data(), (size_t)len));
            replica = rid;
            imginit = true;
        } else if (t == "POSDATA") {
            double hb[9], hi[9];
            int32_t n = 0;
            if (!(read_all(fd, hb, sizeof hb) && read_all(fd, hi, sizeof hi) && read_all(fd, &n, 4) && n > 0 &&
                  n <= 100000000)) {
                rc = fail(MBX_ERR_ARG, "i-PI POSDATA: bad cell or atom count");
                break;
            }
            nat = n;
            std::vector<double> pos(3 * (size_t)nat);
            if (!read_all(fd, pos.data(), pos.size() * sizeof(double))) {
                rc = fail(MBX_ERR_ARG, "i-PI POSDATA: positions cut short");
                break;
            }
            // cell = transpose(h) to Angstrom (DL_POLY's cell(9): a, b, c); positions to Angstrom
            double cell[9];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) cell[a + 3 * b] = hb[b + 3 * a] * kBohrA;
            for (double& x : pos) x *= kBohrA;
            forces.assign(3 * (size_t)nat, 0.0);
            dip.assign(3 * (size_t)(nat / 3), 0.0);
            double e = 0.0, st[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            const int frc = fn(user, replica, nat, cell, pos.data(), &e, forces.data(), st, dip.data());
            if (frc != MBX_OK && frc != MBX_ERR_CONVERGE) {
                rc = fail(frc, "force evaluation failed");
                break;
            }
            // energy, forces and virial in atomic units (the virial is the stress transposed)
            pot = e * kDlpolyHa * kKcalRatio;
            for (double& f : forces) f = f * kDlpolyHa * kBohrA * kKcalRatio;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) virial[a + 3 * b] = st[b + 3 * a] * kDlpolyHa * kKcalRatio;
            diptext.clear();
            char buf[40];
            for (double d : dip) {
                std::snprintf(buf, sizeof buf, " %.17g", d);
                diptext += buf;
            }
            hasdata = true;
        } else if (t == "GETFORCE") {
            if (hasdata) {
                // the whole reply in one write
                const int32_t n = nat, len = (int32_t)diptext.size();
                std::vector<char> msg;
                auto put = [&](const void* p, size_t b) {
                    const char* c = static_cast<const char*>(p);
                    msg.insert(msg.end(), c, c + b);
                };
                char hdr[12];
                std::memset(hdr, ' ', sizeof hdr);
                std::memcpy(hdr, "FORCEREADY", 10);
                put(hdr, sizeof hdr);
                put(&pot, sizeof pot);
                put(&n, 4);
                put(forces.data(), forces.size() * sizeof(double));
                put(virial.data(), 9 * sizeof(double));
                put(&len, 4);
                put(diptext.data(), diptext.size());
                ok = write_all(fd, msg.data(), msg.size());
                hasdata = false;
                imginit = false;
                ++steps;
                if (steps_done) *steps_done = steps;
                if (max_steps > 0 && steps >= max_steps) break;
            }
        } else if (t == "EXIT") {
            break;
        } else {
            rc = fail(MBX_ERR_ARG, "unexpected message from i-PI: " + t);
            break;
        }
        if (!ok) {
            rc = fail(MBX_ERR_ARG, "i-PI socket read or write failed");
            break;
        }
    }
    ::close(fd);
    return rc;
}

namespace {

// The whole force evaluation of a configuration of MB-pol water (3 atoms per water, O H H)
// through mbx_water_step, the dipoles of each replica kept as its next warm start.
struct WaterDriver {
    mbx_context* ctx;
    int precision;
    const double* prm;   // 15 Ewald / dipole settings, or null: mbx_polar_params_for_cell
    int dispersion;
    std::map<int, std::vector<double>> dip;   // per replica: 3 blocks of 4 nw site dipoles
    int last_replica = -1;
};

int water_driver_forces(void* user, int replica, int nat, const double* cell, const double* xyz, double* energy,
                        double* forces, double* stress, double* moldip) {
    WaterDriver& d = *static_cast<WaterDriver*>(user);
    if (nat % 3 != 0) return MBX_ERR_ARG;
    const int nw = nat / 3, n = 4 * nw;
    double prm[15];
    if (d.prm) std::memcpy(prm, d.prm, sizeof prm);
    else mbx_polar_params_for_cell(cell, prm);
    std::vector<double> x(n, 0.0), y(n, 0.0), z(n, 0.0), f(3 * (size_t)n, 0.0), q(n, 0.0), polr(n), polr2(n);
    for (int i = 0; i < nat; ++i) {
        x[i] = xyz[3 * i];
        y[i] = xyz[3 * i + 1];
        z[i] = xyz[3 * i + 2];
    }
    for (int i = 0; i < n; ++i) {   // MB-pol: O and M 1.310, H 0.294 A^3; the M site holds no dipole
        const bool m = i >= 3 * nw, o = !m && i % 3 == 0;
        polr[i] = (m || o) ? 1.310 : 0.294;
        polr2[i] = m ? 0.0 : polr[i];
    }
    std::vector<int> lt, mol;
    if (d.dispersion) {   // water types 1 (O), 2 (H), 3 (M) and one molecule per water
        lt.resize(n);
        mol.resize(n);
        for (int i = 0; i < n; ++i) {
            const bool m = i >= 3 * nw;
            lt[i] = m ? 3 : (i % 3 == 0 ? 1 : 2);
            mol[i] = (m ? i - 3 * nw : i / 3) + 1;
        }
    }
    // another replica than the last frame's: the ASPC step count restarts, as the reference's
    // imglock test does (SOURCE/dlpoly_cmd.f:1765-1768)
    if (replica != d.last_replica) {
        mbx_aspc_restart(d.ctx);
        d.last_replica = replica;
    }
    std::vector<double>& dp = d.dip[replica];
    if (dp.size() != 3 * (size_t)n) dp.assign(3 * (size_t)n, 0.0);
    const bool diag = cell[1] == 0.0 && cell[2] == 0.0 && cell[3] == 0.0 && cell[5] == 0.0 && cell[6] == 0.0 &&
                      cell[7] == 0.0;
    double sc[MBX_NSTEPSCALARS];
    const int rc = mbx_water_step(d.ctx, d.precision, diag ? 2 : 3, cell, nw, n, prm, polr.data(), polr2.data(),
                                  d.dispersion ? lt.data() : nullptr, d.dispersion ? mol.data() : nullptr, x.data(),
                                  y.data(), z.data(), dp.data(), dp.data() + n, dp.data() + 2 * (size_t)n, f.data(),
                                  f.data() + n, f.data() + 2 * (size_t)n, nullptr, nullptr, nullptr, nullptr, nullptr,
                                  q.data(), sc);
    if (rc != MBX_OK && rc != MBX_ERR_CONVERGE) return rc;
    // total potential energy and stress of the terms: MB-pol 2B + 3B, 1-body, dispersion,
    // electrostatics (the blocks of MBX_NSTEPSCALARS)
    const int nb = MBX_NSCALARS, b1 = nb, bd = nb + 14, be = MBX_NWATERSCALARS;
    *energy = sc[MBX_S_ENG2] + sc[MBX_S_ENG3] + sc[b1] + sc[bd] + sc[be];
    for (int c = 0; c < 9; ++c)
        stress[c] = sc[MBX_S_STRESS + c] + sc[b1 + 2 + c] + sc[bd + 2 + c] + sc[be + 2 + c];
    for (int i = 0; i < nat; ++i)
        for (int c = 0; c < 3; ++c) forces[3 * i + c] = f[(size_t)c * n + i];
    // per water: DMS charges times positions (hydrogens imaged next to the oxygen, the M
    // site as placed) plus the induced dipoles of its four sites, in Debye
    Cell cl;
    for (int c = 0; c < 9; ++c) cl.c[c] = cell[c];
    cell_inverse(cell, cl.rc);
    for (int w = 0; w < nw; ++w) {
        const int o = 3 * w, m = 3 * nw + w;
        const double ro[3] = {x[o], y[o], z[o]};
        double mu[3] = {q[m] * x[m], q[m] * y[m], q[m] * z[m]};
        for (int hh = 1; hh <= 2; ++hh) {
            const int h = o + hh;
            double dd[3] = {ro[0] - x[h], ro[1] - y[h], ro[2] - z[h]};
            min_image_host(cl, dd);
            for (int c = 0; c < 3; ++c) mu[c] += q[h] * (ro[c] - dd[c]);
        }
        const int site[4] = {o, o + 1, o + 2, m};
        for (int s = 0; s < 4; ++s)
            for (int c = 0; c < 3; ++c) mu[c] += dp[(size_t)c * n + site[s]];
        for (int c = 0; c < 3; ++c) moldip[3 * w + c] = mu[c] * kEatd;
    }
    return rc;
}

}  // namespace

extern "C" int mbx_ipi_run(mbx_context* ctx, const char* address, int precision, const double* polar_prm,
                           int dispersion, long max_steps, long* steps_done) {
    if (!ctx || (precision != MBX_FP64 && precision != MBX_MIXED)) return MBX_ERR_ARG;
    WaterDriver d{ctx, precision, polar_prm, dispersion, {}};
    char err[256] = {0};
    const int rc = mbx_ipi_run_callback(address, water_driver_forces, &d, max_steps, steps_done, err, sizeof err);
    if (rc && err[0]) mbx_set_error_text(ctx, err);
    return rc;
}
