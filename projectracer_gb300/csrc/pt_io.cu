// pt_io.cu -- the reference's output and restart files, written from the device state:
//   snapshots (main.f90:377-424): T<10000+fcount> with x, z, T, SF, u, w, the deviatoric stress
//     2 vis strain, vis, T_vis, nempty (and C, C_vis), one line per node, i outer, in the
//     reference's Fortran edit descriptors (G14.5E3, I6); P<10000+fcount> with the lateral
//     averages of T, the strain rate and the stress per row;
//   print_restart (main.f90:457-496): Trestart (xg, zg, T, [Cnew], SF) and restart_tracers
//     (rtr, str, [Ctr | Ttype], Ttr) as gfortran sequential unformatted records (4-byte length
//     markers; a record longer than the marker's range is split into sub-records whose markers
//     carry a negative sign where another sub-record follows or precedes);
//   the restart read (grid.f90:55-104, and the tracer record) into pt_upload_state.
// Writes are asynchronous: the device-to-host copies are queued on the library's stream, in
// order after the work that produced the state and before any later step, into pinned staging;
// a host thread then formats and writes the files while the caller keeps stepping.  pt_io_wait
// joins it and returns its status.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "pt_consts.cuh"

namespace pt {

namespace {

constexpr int64_t kMaxSubRecord = 2147483639;  // 2^31 - 9: gfortran's largest sub-record payload

struct IoState {
    std::thread th;
    bool active = false;
    int rc = 0;
    std::string msg;
    cudaEvent_t done = nullptr;
    unsigned char* stage = nullptr;  // pinned staging
    size_t stage_bytes = 0;
    int64_t rec_limit = kMaxSubRecord;
    bool consts = false;
};

IoState& io(Engine& E) {
    if (!E.io) E.io = new IoState();
    return *static_cast<IoState*>(E.io);
}

int io_join(Engine& E) {
    IoState& S = io(E);
    if (!S.active) return 0;
    S.th.join();
    S.active = false;
    if (S.rc) return fail(S.rc, S.msg);
    return 0;
}

int io_stage(Engine& E, size_t bytes) {
    IoState& S = io(E);
    if (S.stage_bytes >= bytes) return 0;
    if (S.stage) cudaFreeHost(S.stage);
    S.stage = nullptr;
    S.stage_bytes = 0;
    CK(cudaMallocHost(&S.stage, bytes));
    S.stage_bytes = bytes;
    if (!S.done) CK(cudaEventCreateWithFlags(&S.done, cudaEventDisableTiming));
    return 0;
}

// ---- Fortran edit descriptors
// Gw.dEe with w=14, d=5, e=3 (Fortran 2008, 13.7.2.3.8): after rounding to d significant digits,
// a magnitude in [0.1, 10^d) is written as F(w-e-2).(d-k) followed by e+2 blanks (k its decimal
// exponent, 0 <= k <= d), anything else as Ew.dEe; zero as F9.4 and five blanks
void put_g14_5e3(std::string& out, double x) {
    char buf[64];
    if (x == 0.0) {
        std::snprintf(buf, sizeof buf, "%9.4f     ", x);  // keeps the sign of -0
        out += buf;
        return;
    }
    std::snprintf(buf, sizeof buf, "%.4e", x);  // d significant digits: m.mmmme+pp
    const char* e = std::strchr(buf, 'e');
    const int p = std::atoi(e + 1);
    const int k = p + 1;  // x = 0.ddddd * 10^k
    if (k >= 0 && k <= 5) {
        std::snprintf(buf, sizeof buf, "%9.*f     ", 5 - k, x);
        out += buf;
        return;
    }
    // E14.5E3: [sign]0.ddddd E[sign]kkk, right-justified in 14
    std::snprintf(buf, sizeof buf, "%.4e", std::fabs(x));
    char digits[6] = {buf[0], buf[2], buf[3], buf[4], buf[5], 0};
    char field[32];
    std::snprintf(field, sizeof field, "%s0.%sE%c%03d", x < 0 ? "-" : "", digits, k < 0 ? '-' : '+', k < 0 ? -k : k);
    std::snprintf(buf, sizeof buf, "%14s", field);
    out += buf;
}

void put_i6(std::string& out, int v) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "%6d", v);
    out += buf;
}

// ---- gfortran sequential unformatted records
int write_record(FILE* f, const std::vector<std::pair<const void*, size_t>>& parts, int64_t limit) {
    size_t n = 0;
    for (auto& p : parts) n += p.second;
    auto marker = [&](int32_t m) { return std::fwrite(&m, 4, 1, f) == 1; };
    size_t part = 0, off = 0, done = 0;
    bool first = true;
    do {
        const size_t len = (n - done) > (size_t)limit ? (size_t)limit : (n - done);
        const bool last = done + len >= n;
        const int32_t head = last ? (int32_t)len : -(int32_t)len;
        const int32_t tail = first ? (int32_t)len : -(int32_t)len;
        if (!marker(head)) return -1;
        size_t left = len;
        while (left) {
            const size_t take = std::min(left, parts[part].second - off);
            if (take && std::fwrite(static_cast<const unsigned char*>(parts[part].first) + off, 1, take, f) != take)
                return -1;
            off += take;
            left -= take;
            if (off == parts[part].second) { part++; off = 0; }
        }
        if (!marker(tail)) return -1;
        done += len;
        first = false;
    } while (done < n);
    return 0;
}

int read_record(FILE* f, std::vector<unsigned char>& data) {
    data.clear();
    for (;;) {
        int32_t head = 0, tail = 0;
        if (std::fread(&head, 4, 1, f) != 1) return -1;
        const size_t len = (size_t)(head < 0 ? -(int64_t)head : head);
        const size_t at = data.size();
        data.resize(at + len);
        if (len && std::fread(data.data() + at, 1, len, f) != len) return -1;
        if (std::fread(&tail, 4, 1, f) != 1) return -1;
        if (head >= 0) return 0;
    }
}

}  // namespace

// strain(i,k,1) at every node: from the velocities for the direct solve
// (compute_strain_rate_invariant, momentum.f90:1-34), else from the multigrid's psi
// (compute_strain_rate_invariant_direct, momentum.f90:73-92); the same arithmetic as the statistics
__global__ void k_strain_field(double* out, const double* u, const double* w, const double* E1, Geo g, int direct) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i > cK.nx) return;
    double s;
    if (direct) {
        double ur = 0, us = 0, wr = 0, ws = 0;
        for (int j = -2; j <= 2; j++) ur = ur + cK.D1[3 + j] * u[g.at(i + j, k)];
        ur = ur / cK.dr;
        for (int j = -2; j <= 2; j++) us = us + cK.D1[3 + j] * u[g.at(i, k + j)];
        us = us / cK.ds;
        for (int j = -2; j <= 2; j++) wr = wr + cK.D1[3 + j] * w[g.at(i + j, k)];
        wr = wr / cK.dr;
        for (int j = -2; j <= 2; j++) ws = ws + cK.D1[3 + j] * w[g.at(i, k + j)];
        ws = ws / cK.ds;
        const double ux = ur / 1.0, uz = us / 1.0, wx = wr / 1.0, wz = ws / 1.0;
        s = pow(0.5 * (2.0 * (ux * ux + wz * wz) + (uz + wx) * (uz + wx)), 0.5);
    } else {
        double Sxx = 0, Szz = 0, Sxz = 0;
        for (int j = -2; j <= 2; j++) Sxx = Sxx + cK.D2[3 + j] * E1[g.at(i + j, k)];
        Sxx = qdiv(Sxx, cK.dr2, cK.inv_dr2);
        for (int j = -2; j <= 2; j++) Szz = Szz + cK.D2[3 + j] * E1[g.at(i, k + j)];
        Szz = qdiv(Szz, cK.ds2, cK.inv_ds2);
        for (int k2 = -2; k2 <= 2; k2++)
            for (int i2 = -2; i2 <= 2; i2++) Sxz = Sxz + cK.Drs[i2 + 2][k2 + 2] * E1[g.at(i + i2, k + k2)];
        Sxz = Sxz / (cK.dr * cK.ds);
        s = pow(2.0 * (Sxz * Sxz) + 0.5 * ((Szz - Sxx) * (Szz - Sxx)), 0.5);
    }
    out[g.at(i, k)] = s;
}

void io_release(Engine& E) {
    if (!E.io) return;
    IoState& S = io(E);
    if (S.active) {
        S.th.join();
        S.active = false;
    }
    if (S.stage) cudaFreeHost(S.stage);
    if (S.done) cudaEventDestroy(S.done);
    delete &S;
    E.io = nullptr;
}

// the uniform grid's xg(-6:nx+6) (grid.f90:44-54, 105-116); zg likewise with 1 for aspect
static void grid_line(std::vector<double>& x, int n, double len) {
    x.assign((size_t)n + 13, 0.0);
    const double h = len / (double)n;
    for (int i = 0; i <= n; i++) x[(size_t)i + 6] = h * (double)i;
    x[6] = 0.0;
    x[(size_t)n + 6] = len;
    for (int i = 1; i <= 6; i++) {
        x[(size_t)(6 - i)] = -x[(size_t)(6 + i)];
        x[(size_t)(6 + n + i)] = len - x[(size_t)(6 + n - i)] + len;
    }
}

// queue a 2-D device-to-host copy of field f (ghost gh) into staging at byte offset off
static int stage_field(Engine& E, const double* f, int gh, unsigned char* dst) {
    const size_t wdt = (size_t)(E.K.nx + 2 * gh + 1), h = (size_t)(E.K.nz + 2 * gh + 1);
    CK(cudaMemcpy2DAsync(dst, wdt * 8, f + E.g1.at(-gh, -gh), E.g1.pitch * 8, wdt * 8, h, cudaMemcpyDeviceToHost, E.st));
    return 0;
}

static std::string path_join(const char* dir, const char* name) {
    std::string p = dir && *dir ? dir : ".";
    if (p.back() != '/') p += '/';
    return p + name;
}

}  // namespace pt

using namespace pt;

extern "C" {

int pt_io_wait(void) {
    if (!g_eng) return fail(PT_ERR_STATE, "call pt_init first");
    return io_join(*g_eng);
}

int pt_prof_record_limit(int64_t bytes) {
    if (!g_eng) return fail(PT_ERR_STATE, "call pt_init first");
    if (bytes < 0 || bytes > kMaxSubRecord) return fail(PT_ERR_ARG, "record limit outside 1..2^31-9 (0: default)");
    io(*g_eng).rec_limit = bytes ? bytes : kMaxSubRecord;
    return 0;
}

int pt_write_restart(const char* dir) {
    if (!g_eng || !g_eng->uploaded) return fail(PT_ERR_STATE, "call pt_init and pt_upload_state first");
    Engine& E = *g_eng;
    if (int rc = io_join(E)) return rc;
    const int nx = E.K.nx, nz = E.K.nz, comp = E.cfg.comp, og = E.cfg.discrete_types;
    const size_t n3 = (size_t)(nx + 7) * (nz + 7), n5 = (size_t)(nx + 11) * (nz + 11), nt = (size_t)E.ntr;
    const size_t grid_b = 8 * (2 * n3 + (comp ? n5 : 0)), trc_b = 8 * 3 * nt + (comp ? (og ? 4 : 8) * nt : 0);
    if (int rc = io_stage(E, grid_b + trc_b)) return rc;
    IoState& S = io(E);
    unsigned char* g = S.stage;
    unsigned char* t = S.stage + grid_b;
    int rc;
    if ((rc = stage_field(E, E.T, 3, g))) return rc;
    if (comp && (rc = stage_field(E, E.Cnew, 5, g + 8 * n3))) return rc;
    if ((rc = stage_field(E, E.SF, 3, g + 8 * (n3 + (comp ? n5 : 0))))) return rc;
    // tracer records in the caller's order (the mixed path may hold them re-sorted): gathered into
    // the RK stage buffers, free between steps
    const double* arr[4] = {E.rtr, E.str, E.Ctr, E.Ttr};
    double* tmp[4] = {E.rtr1, E.str1, E.Ttr1, E.rtr2};
    const int na = 4;
    for (int a = 0; a < na; a++) {
        if (a == 2 && !comp) continue;
        const double* src = arr[a];
        if (E.perm_active) {
            if ((rc = tracer_user_order(E, const_cast<double*>(src), tmp[a], true))) return rc;
            src = tmp[a];
        }
        arr[a] = src;
    }
    size_t off = 0;
    for (int a = 0; a < na; a++) {
        if (a == 2 && !comp) continue;
        if (a == 2 && og) {  // Ttype (integer*4) instead of Ctr
            if ((rc = c_to_types(E, arr[2], E.tcell))) return rc;
            CK(cudaMemcpyAsync(t + off, E.tcell, 4 * nt, cudaMemcpyDeviceToHost, E.st));
            off += 4 * nt;
            continue;
        }
        CK(cudaMemcpyAsync(t + off, arr[a], 8 * nt, cudaMemcpyDeviceToHost, E.st));
        off += 8 * nt;
    }
    CK(cudaEventRecord(S.done, E.st));
    std::vector<double> xg, zg;
    grid_line(xg, nx, E.K.aspect);
    grid_line(zg, nz, 1.0);
    const std::string ft = path_join(dir, "Trestart"), fr = path_join(dir, "restart_tracers");
    const int64_t limit = S.rec_limit;
    const bool has_tr = true;  // comp = 1 or tracer = 1 (the engine always carries temperature tracers)
    S.rc = 0;
    S.msg.clear();
    S.active = true;
    S.th = std::thread([=, &S]() {
        if (cudaEventSynchronize(S.done) != cudaSuccess) {
            S.rc = PT_ERR_CUDA;
            S.msg = "restart writer: device-to-host copies failed";
            return;
        }
        FILE* f = std::fopen(ft.c_str(), "wb");
        std::vector<std::pair<const void*, size_t>> parts = {{xg.data(), 8 * xg.size()}, {zg.data(), 8 * zg.size()},
                                                             {g, 8 * n3}};
        if (comp) parts.push_back({g + 8 * n3, 8 * n5});
        parts.push_back({g + 8 * (n3 + (comp ? n5 : 0)), 8 * n3});
        int bad = !f || write_record(f, parts, limit) != 0;
        if (f && std::fclose(f) != 0) bad = 1;
        if (!bad && has_tr) {
            f = std::fopen(fr.c_str(), "wb");
            bad = !f || write_record(f, {{t, off}}, limit) != 0;
            if (f && std::fclose(f) != 0) bad = 1;
        }
        if (bad) {
            S.rc = PT_ERR_ARG;
            S.msg = "restart writer: cannot write " + ft + " / " + fr + ": " + std::strerror(errno);
        }
    });
    return 0;
}

int pt_write_snapshot(const char* dir, int fcount) {
    if (!g_eng || !g_eng->uploaded) return fail(PT_ERR_STATE, "call pt_init and pt_upload_state first");
    Engine& E = *g_eng;
    if (int rc = io_join(E)) return rc;
    IoState& S = io(E);
    if (!S.consts) {
        if (int rc = upload_tu_consts(E)) return rc;
        S.consts = true;
    }
    const int nx = E.K.nx, nz = E.K.nz, comp = E.cfg.comp;
    const size_t n3 = (size_t)(nx + 7) * (nz + 7), n5 = (size_t)(nx + 11) * (nz + 11), nn = (size_t)(nx + 1) * (nz + 1);
    const size_t bytes = 8 * (7 * n3 + 2 * n5) + 4 * nn;
    if (int rc = io_stage(E, bytes)) return rc;
    // strain(:,:,1) into the scratch field
    dim3 gg(nblk(nx + 1, 128), nz + 1);
    PT_COUNT(), k_strain_field<<<gg, 128, 0, E.st>>>(E.scratch, E.u, E.w, E.err[1], E.g1, E.cfg.direct);
    CKL("k_strain_field");
    unsigned char* b = S.stage;
    const double* f3[7] = {E.T, E.SF, E.u, E.w, E.scratch, E.vis[1], E.Tvis};
    int rc;
    for (int q = 0; q < 7; q++)
        if ((rc = stage_field(E, f3[q], 3, b + 8 * n3 * q))) return rc;
    if (comp) {
        if ((rc = stage_field(E, E.Cnew, 5, b + 8 * 7 * n3))) return rc;
        if ((rc = stage_field(E, E.Cvis, 5, b + 8 * (7 * n3 + n5)))) return rc;
    }
    int32_t* ne = reinterpret_cast<int32_t*>(b + 8 * (7 * n3 + 2 * n5));
    CK(cudaMemcpyAsync(ne, E.nempty, 4 * nn, cudaMemcpyDeviceToHost, E.st));
    CK(cudaEventRecord(S.done, E.st));
    char nm[16];
    std::snprintf(nm, sizeof nm, "T%5d", 10000 + fcount);
    const std::string ftn = path_join(dir, nm);
    std::snprintf(nm, sizeof nm, "P%5d", 10000 + fcount);
    const std::string fpn = path_join(dir, nm);
    std::vector<double> xg, zg;
    grid_line(xg, nx, E.K.aspect);
    grid_line(zg, nz, 1.0);
    const double dr = E.K.dr, aspect = E.K.aspect;
    S.rc = 0;
    S.msg.clear();
    S.active = true;
    S.th = std::thread([=, &S]() {
        if (cudaEventSynchronize(S.done) != cudaSuccess) {
            S.rc = PT_ERR_CUDA;
            S.msg = "snapshot writer: device-to-host copies failed";
            return;
        }
        const double* F = reinterpret_cast<const double*>(b);
        auto at3 = [&](int q, int i, int k) { return F[n3 * q + (size_t)(i + 3) + (size_t)(k + 3) * (nx + 7)]; };
        auto at5 = [&](int q, int i, int k) {
            return F[7 * n3 + n5 * q + (size_t)(i + 5) + (size_t)(k + 5) * (nx + 11)];
        };
        // the lines of columns i0 .. i1-1 (one block of lines per column, then a blank record)
        auto columns = [&](std::string& out, int i0, int i1) {
            out.reserve((size_t)(i1 - i0) * (nz + 2) * 200);
            for (int i = i0; i < i1; i++) {
                for (int k = 0; k <= nz; k++) {
                    put_g14_5e3(out, xg[(size_t)i + 6]);
                    put_g14_5e3(out, zg[(size_t)k + 6]);
                    put_g14_5e3(out, at3(0, i, k));
                    put_g14_5e3(out, at3(1, i, k));
                    put_g14_5e3(out, at3(2, i, k));
                    put_g14_5e3(out, at3(3, i, k));
                    put_g14_5e3(out, 2.0 * at3(5, i, k) * at3(4, i, k));
                    put_g14_5e3(out, at3(5, i, k));
                    put_g14_5e3(out, at3(6, i, k));
                    put_i6(out, ne[(size_t)i + (size_t)k * (nx + 1)]);
                    if (comp) {
                        put_g14_5e3(out, at5(0, i, k));
                        put_g14_5e3(out, at5(1, i, k));
                    }
                    out += '\n';
                }
                out += "  \n";  // write(101,*) " "
            }
        };
        // formatted by up to 16 host threads, column blocks in order
        const unsigned hc = std::thread::hardware_concurrency();
        const int nth = std::max(1, std::min({16, nx + 1, hc ? (int)hc : 1}));
        std::vector<std::string> parts((size_t)nth);
        {
            std::vector<std::thread> pool;
            for (int t = 1; t < nth; t++) {
                const int a = (int)((long long)(nx + 1) * t / nth), c = (int)((long long)(nx + 1) * (t + 1) / nth);
                try {
                    pool.emplace_back(columns, std::ref(parts[(size_t)t]), a, c);
                } catch (...) {  // no thread to be had: this one formats the block
                    columns(parts[(size_t)t], a, c);
                }
            }
            columns(parts[0], 0, (int)((long long)(nx + 1) / nth));
            for (std::thread& th : pool) th.join();
        }
        FILE* f = std::fopen(ftn.c_str(), "w");
        int bad = !f;
        for (const std::string& part : parts)
            if (!bad && std::fwrite(part.data(), 1, part.size(), f) != part.size()) bad = 1;
        if (f && std::fclose(f) != 0) bad = 1;
        std::string out;
        // lateral averages: integrate1Dx (basics.f90:494-515, trapezoids) over each row
        out.clear();
        auto lat = [&](auto fn, int k) {
            double s = 0.0, p = fn(0, k);
            for (int i = 0; i < nx; i++) {
                const double q = fn(i + 1, k);
                s = s + 0.5 * (p * 1.0 + q * 1.0) * dr;
                p = q;
            }
            return s / aspect;
        };
        for (int k = 0; k <= nz; k++) {
            put_g14_5e3(out, zg[(size_t)k + 6]);
            put_g14_5e3(out, lat([&](int i, int kk) { return at3(0, i, kk); }, k));
            put_g14_5e3(out, lat([&](int i, int kk) { return at3(4, i, kk); }, k));
            put_g14_5e3(out, lat([&](int i, int kk) { return 2.0 * at3(5, i, kk) * at3(4, i, kk); }, k));
            out += '\n';
        }
        if (!bad) {
            f = std::fopen(fpn.c_str(), "w");
            bad = !f || std::fwrite(out.data(), 1, out.size(), f) != out.size();
            if (f && std::fclose(f) != 0) bad = 1;
        }
        if (bad) {
            S.rc = PT_ERR_ARG;
            S.msg = "snapshot writer: cannot write " + ftn + " / " + fpn + ": " + std::strerror(errno);
        }
    });
    return 0;
}

int pt_read_restart(const char* dir) {
    if (!g_eng) return fail(PT_ERR_STATE, "call pt_init first");
    Engine& E = *g_eng;
    if (int rc = io_join(E)) return rc;
    const int nx = E.K.nx, nz = E.K.nz, comp = E.cfg.comp, og = E.cfg.discrete_types;
    const size_t n3 = (size_t)(nx + 7) * (nz + 7), n5 = (size_t)(nx + 11) * (nz + 11), nt = (size_t)E.ntr;
    std::vector<unsigned char> g, t;
    const std::string ft = path_join(dir, "Trestart"), fr = path_join(dir, "restart_tracers");
    FILE* f = std::fopen(ft.c_str(), "rb");
    if (!f) return fail(PT_ERR_ARG, "cannot open " + ft);
    int bad = read_record(f, g);
    std::fclose(f);
    if (bad) return fail(PT_ERR_ARG, "Trestart: truncated record");
    f = std::fopen(fr.c_str(), "rb");
    if (!f) return fail(PT_ERR_ARG, "cannot open " + fr);
    bad = read_record(f, t);
    std::fclose(f);
    if (bad) return fail(PT_ERR_ARG, "restart_tracers: truncated record");
    const size_t gx = (size_t)nx + 13, gz = (size_t)nz + 13;
    if (g.size() != 8 * (gx + gz + 2 * n3 + (comp ? n5 : 0)))
        return fail(PT_ERR_ARG, "Trestart: record size does not match the configuration");
    const size_t want = 8 * 3 * nt + (comp ? (og ? 4 : 8) * nt : 0);
    if (t.size() != want) return fail(PT_ERR_ARG, "restart_tracers: record size does not match the configuration");
    const double* G = reinterpret_cast<const double*>(g.data());
    const double *xg = G, *zg = G + gx, *T = zg + gz, *Cn = comp ? T + n3 : nullptr, *SF = T + n3 + (comp ? n5 : 0);
    const unsigned char* p = t.data();
    const double* r = reinterpret_cast<const double*>(p);
    const double* s = r + nt;
    const double* C = nullptr;
    const int32_t* ty = nullptr;
    size_t off = 16 * nt;
    if (comp) {
        if (og) ty = reinterpret_cast<const int32_t*>(p + off);
        else C = reinterpret_cast<const double*>(p + off);
        off += (og ? 4 : 8) * nt;
    }
    // tracer records are 8-byte aligned here only when the type record length is; copy to be safe
    std::vector<double> Tt(nt);
    std::memcpy(Tt.data(), p + off, 8 * nt);
    std::vector<double> Cz;
    if (!comp) Cn = nullptr;
    return pt_upload_state(xg, zg, T, Cn, SF, r, s, C, Tt.data(), ty);
}

}  // extern "C"
