// pt_api.cu -- the C ABI of include/ptgpu.h: context set-up, field exchange, the restart upload
// and the time-step orchestration (energy_time, energy.f90:181-556) on one CUDA stream.
#include <nvtx3/nvToolsExt.h>
#include <utility>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "pt_consts.cuh"
#include "../../include/ptgpu_prof.h"

namespace pt {

Engine* g_eng = nullptr;
std::atomic<int64_t> g_launches{0};
thread_local std::string g_err;

int upload_consts_fields(const Engine& E);
int upload_consts_tracers(const Engine& E);
int upload_consts_mg(const Engine& E);
int upload_consts_mixed(const Engine& E);

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return 0;
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return PT_ERR_CUDA;
}

static cudaEvent_t take_event(Engine& E) {
    cudaEvent_t ev = nullptr;
    if (!E.ev_pool.empty()) {
        ev = E.ev_pool.back();
        E.ev_pool.pop_back();
    } else if (cudaEventCreate(&ev) != cudaSuccess) {
        (void)cudaGetLastError();
        ev = nullptr;
    }
    return ev;
}

static void push_span(Engine& E, int slot, int kid, int n, cudaEvent_t a) {
    if (!a) return;
    cudaEvent_t b = take_event(E);
    if (!b) {
        E.ev_pool.push_back(a);
        return;
    }
    cudaEventRecord(b, E.st);
    E.spans.push_back({slot, kid, n, a, b});
    if (E.spans.size() > 8192) {  // bound the pending list
        cudaStreamSynchronize(E.st);
        harvest_spans(E);
    }
}

void harvest_spans(Engine& E) {
    size_t keep = 0;
    for (size_t q = 0; q < E.spans.size(); q++) {
        const Engine::Span s = E.spans[q];
        float ms = 0.f;
        const cudaError_t e = cudaEventElapsedTime(&ms, s.a, s.b);
        if (e == cudaErrorNotReady) {  // still running: keep for a later harvest
            (void)cudaGetLastError();
            E.spans[keep++] = s;
            continue;
        }
        if (e == cudaSuccess) {
            if (s.slot >= 0) {
                E.phase_ms[s.slot] += ms;
            } else {
                E.kms[s.kid] += ms;
                E.kcount[s.kid] += s.n;
            }
        } else {
            (void)cudaGetLastError();  // a timing miss must not surface as the next launch's error
        }
        E.ev_pool.push_back(s.a);
        E.ev_pool.push_back(s.b);
    }
    E.spans.resize(keep);
}

PhaseTimer::PhaseTimer(Engine& e, int s) : E(e), slot(s) {
    a = take_event(E);
    if (a) cudaEventRecord(a, E.st);
}
PhaseTimer::~PhaseTimer() { push_span(E, slot, 0, 0, a); }

// cudaEventRecordExternal makes the record a timing node of the captured graph (a plain record
// during capture only expresses a dependency)
GraphTimer::GraphTimer(Engine& e, int w, int count) : E(e), which(w), n(count) {
    if (n) cudaEventRecordWithFlags(E.gev[which][0], E.st, cudaEventRecordExternal);
}
GraphTimer::~GraphTimer() {
    if (!n) return;
    cudaEventRecordWithFlags(E.gev[which][1], E.st, cudaEventRecordExternal);
    E.gev_n[which] = n;
}
void harvest_graph_timer(Engine& E, int which) {
    if (!E.prof || !E.gev_n[which]) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, E.gev[which][0], E.gev[which][1]) == cudaSuccess) {
        const int id = which == 0 ? KT_RKC_FP64_L1 : KT_RKC_FP32_L1;
        E.kms[id] += ms;
        E.kcount[id] += E.gev_n[which];
    } else {
        (void)cudaGetLastError();  // a timing miss must not surface as the next launch's error
    }
}

KernelTimer::KernelTimer(Engine& e, int i, int count) : E(e), id(i), n(count) {
    if (!E.prof) return;
    a = take_event(E);
    if (a) cudaEventRecord(a, E.st);
}
KernelTimer::~KernelTimer() { push_span(E, -1, id, n, a); }

static int dalloc(Engine& E, double** p, size_t n) {
    CK(cudaMalloc(p, n * sizeof(double)));
    CK(cudaMemsetAsync(*p, 0, n * sizeof(double), E.st));
    E.bytes_allocated += n * sizeof(double);
    return 0;
}
static int ialloc(Engine& E, int32_t** p, size_t n) {
    CK(cudaMalloc(p, n * sizeof(int32_t)));
    CK(cudaMemsetAsync(*p, 0, n * sizeof(int32_t), E.st));
    E.bytes_allocated += n * sizeof(int32_t);
    return 0;
}

static int engine_alloc(Engine& E) {
    int rc;
    const size_t n1 = E.g1.elems();
    double** fine[] = {&E.T, &E.Tratio, &E.Tvis, &E.Tbuoy, &E.Cnew, &E.Cvis, &E.Cbuoy, &E.SF, &E.u, &E.w,
                       &E.cond, &E.cond_r, &E.cond_s, &E.tsa, &E.Text, &E.T0, &E.C0, &E.scratch, &E.psi_keep};
    for (auto p : fine)
        if ((rc = dalloc(E, p, n1))) return rc;
    for (int f = 0; f < 3; f++)
        for (int j = 0; j < 3; j++)
            if ((rc = dalloc(E, &E.der[f][j], n1))) return rc;
    const int ncell = (E.K.nx + 1) * (E.K.nz + 1);
    if ((rc = ialloc(E, &E.nempty, (size_t)ncell))) return rc;
    if (E.cfg.discrete_types && (rc = ialloc(E, &E.count1, (size_t)ncell))) return rc;
    if ((rc = dalloc(E, &E.red, (size_t)(4 * (E.K.nz + 1) + 64)))) return rc;
    if ((rc = dalloc(E, &E.dscal, 32))) return rc;
    CK(cudaMallocHost(&E.hscal, 64 * sizeof(double)));
    CK(cudaMalloc(&E.derr, sizeof(int)));
    CK(cudaMemsetAsync(E.derr, 0, sizeof(int), E.st));
    const size_t nt = (size_t)E.ntr;
    double** trc[] = {&E.rtr, &E.str, &E.Ttr, &E.Ctr, &E.rtr0, &E.str0, &E.Ttr0,
                      &E.rtr1, &E.str1, &E.Ttr1, &E.rtr2, &E.str2, &E.Ttr2};
    for (auto p : trc)
        if ((rc = dalloc(E, p, nt))) return rc;
    if (E.cfg.chebyshev)
        for (double** p : {&E.k0r, &E.k0s, &E.k0T})
            if ((rc = dalloc(E, p, nt))) return rc;
    if ((rc = ialloc(E, &E.tcell, nt))) return rc;
    if ((rc = ialloc(E, &E.clist, nt))) return rc;
    if ((rc = ialloc(E, &E.ccount, (size_t)ncell))) return rc;
    if ((rc = ialloc(E, &E.cstart, (size_t)ncell))) return rc;
    if ((rc = ialloc(E, &E.scan_tmp, (size_t)ncell + (size_t)ncell / 1024 + 64))) return rc;
    if ((rc = dalloc(E, &E.cpart, (size_t)27 * ncell))) return rc;
    if (E.cfg.precision == PT_PREC_MIXED) {  // tracer order (re-sorted by cell when locality is lost)
        if ((rc = ialloc(E, &E.perm, nt)) || (rc = ialloc(E, &E.perm2, nt))) return rc;
        const size_t nkey = resort_nkey(E.K.nx, E.K.nz);
        if (nkey <= (size_t)INT32_MAX &&  // int32 sort keys; larger grids keep the upload order
            ((rc = ialloc(E, &E.rs_count, nkey)) || (rc = ialloc(E, &E.rs_start, nkey)) ||
             (rc = ialloc(E, &E.rs_tot, nkey / 1024 + 64))))
            return rc;
        CK(cudaMalloc(&E.proj_runs, sizeof(unsigned long long)));
        if ((rc = tracer_order_reset(E))) return rc;
    }
    if ((rc = mg_alloc(E))) return rc;
    if (E.cfg.precision == PT_PREC_MIXED && (rc = mixed_alloc(E))) return rc;
    if (E.cfg.direct && (rc = direct_alloc(E))) return rc;
    return 0;
}

static void engine_free(Engine& E) {
    unet_engine_release(E);
    io_release(E);
    direct_free(E);
    if (E.psi_a) cudaFree(E.psi_a);
    if (E.psi_b) cudaFree(E.psi_b);
    double** fine[] = {&E.T, &E.Tratio, &E.Tvis, &E.Tbuoy, &E.Cnew, &E.Cvis, &E.Cbuoy, &E.SF, &E.u, &E.w,
                       &E.cond, &E.cond_r, &E.cond_s, &E.tsa, &E.Text, &E.T0, &E.C0, &E.scratch, &E.psi_keep,
                       &E.red, &E.dscal, &E.cpart, &E.rtr, &E.str, &E.Ttr, &E.Ctr, &E.rtr0, &E.str0,
                       &E.Ttr0, &E.rtr1, &E.str1, &E.Ttr1, &E.rtr2, &E.str2, &E.Ttr2, &E.Mc, &E.Bc, &E.RowB,
                       &E.k0r, &E.k0s, &E.k0T};
    for (auto p : fine)
        if (*p) { cudaFree(*p); *p = nullptr; }
    for (int f = 0; f < 3; f++)
        for (int j = 0; j < 3; j++)
            if (E.der[f][j]) cudaFree(E.der[f][j]);
    for (int f = 0; f < 3; f++) {
        if (E.ftab[f]) cudaFree(E.ftab[f]);
        if (E.facc[f]) cudaFree(E.facc[f]);
    }
    for (int l = 0; l < PT_MAXLEV; l++) {
        double* arrs[] = {E.err[l], E.S0[l], E.S1[l], E.S2[l], E.RHS[l], E.res[l], E.dtst[l], E.ratio[l],
                          E.vis[l], E.visst[l], E.vx[l], E.vz[l], E.vxx[l], E.vzz[l], E.vxz[l], E.vxxpzz[l],
                          E.vxxmzz[l], E.vsm[l]};
        for (auto a : arrs)
            if (a) cudaFree(a);
        float* farrs[] = {E.ferr[l], E.fS0[l], E.fS1[l], E.fS2[l], E.fRHS[l], E.fres[l],
                          E.fcoef[l][0], E.fcoef[l][1], E.fcoef[l][2], E.fcoef[l][3], E.fcoef[l][4], E.fcoef[l][5]};
        for (auto a : farrs)
            if (a) cudaFree(a);
    }
    for (int q = 0; q < 11; q++)
        if (E.visw[q]) cudaFree(E.visw[q]);
    if (E.proj_runs) cudaFree(E.proj_runs);
    int32_t* ia[] = {E.nempty, E.count1, E.tcell, E.clist, E.ccount, E.cstart, E.scan_tmp, E.perm, E.perm2, E.rs_count, E.rs_start, E.rs_tot};
    for (auto a : ia)
        if (a) cudaFree(a);
    if (E.ipiv) cudaFree(E.ipiv);
    if (E.job_active) {  // a coarse-level build may still be running on the worker thread
        E.coarse_job.join();
        E.job_active = false;
    }
    if (E.st2) cudaStreamSynchronize(E.st2);  // a factorisation may still be in flight
    for (int l = 1; l < PT_MAXLEV; l++) {
        double** sets[kVisArrays] = {E.vl2.vis, E.vl2.visst, E.vl2.vx, E.vl2.vz, E.vl2.vxx, E.vl2.vzz, E.vl2.vxz,
                                     E.vl2.vxxpzz, E.vl2.vxxmzz, E.vl2.vsm, E.vl2.ratio, E.vl2.dtst};
        for (double** s : sets)
            if (s[l]) cudaFree(s[l]);
    }
    for (double* p : E.visw2)
        if (p) cudaFree(p);
    if (E.dscal2) cudaFree(E.dscal2);
    if (E.hscal2) cudaFreeHost(E.hscal2);
    if (E.Ginv) cudaFree(E.Ginv);
    for (double* p : {E.Ginv2, E.Mc2, E.RowB2})
        if (p) cudaFree(p);
    if (E.ipiv2) cudaFree(E.ipiv2);
    if (E.derr2) cudaFree(E.derr2);
    if (E.hflag2) cudaFreeHost(E.hflag2);
    if (E.ev_in) cudaEventDestroy(E.ev_in);
    if (E.ev_fact) cudaEventDestroy(E.ev_fact);
    if (E.st2) cudaStreamDestroy(E.st2);
    if (E.derr) cudaFree(E.derr);
    if (E.hscal) cudaFreeHost(E.hscal);
    for (const Engine::Span& s : E.spans) {
        cudaEventDestroy(s.a);
        cudaEventDestroy(s.b);
    }
    E.spans.clear();
    for (cudaEvent_t ev : E.ev_pool) cudaEventDestroy(ev);
    E.ev_pool.clear();
    for (int q = 0; q < 2; q++)
        for (int j = 0; j < 2; j++)
            if (E.gev[q][j]) cudaEventDestroy(E.gev[q][j]);
    equalize_free(E);
    if (E.gM1) cudaGraphExecDestroy(E.gM1);
    if (E.gM2) cudaGraphExecDestroy(E.gM2);
    for (int j = 0; j < kGcrMax; j++) {
        if (E.gG0[j]) cudaGraphExecDestroy(E.gG0[j]);
        if (E.gG1[j]) cudaGraphExecDestroy(E.gG1[j]);
        if (E.gz[j]) cudaFree(E.gz[j]);
        if (E.gv[j]) cudaFree(E.gv[j]);
    }
    for (double* p : {E.gr1, E.gzero, E.gpart, E.gsc})
        if (p) cudaFree(p);
    if (E.gA) cudaGraphExecDestroy(E.gA);
    if (E.gB) cudaGraphExecDestroy(E.gB);
    if (E.rev0) cudaEventDestroy(E.rev0);
    if (E.rev1) cudaEventDestroy(E.rev1);
    if (E.st) cudaStreamDestroy(E.st);
}

static Geo make_geo(int nx, int nz) {
    Geo g;
    g.nx = nx;
    g.nz = nz;
    g.pitch = ((nx + 2 * GH + 1) + 15) / 16 * 16;
    return g;
}

bool trace_on() {
    static int on = -1;
    if (on < 0) on = getenv("PTGPU_TRACE") ? 1 : 0;
    return on == 1;
}
#define TRACE(msg)                                          \
    do {                                                    \
        if (trace_on()) fprintf(stderr, "[ptgpu] %s\n", msg); \
    } while (0)

static int need(int ok) { return ok ? 0 : fail(PT_ERR_STATE, "call pt_init (and pt_upload_state) first"); }

// host (Fortran layout, ghost gh) <-> device (ghost GH, pitch)
static int field_ghost(int id) {
    switch (id) {
        case PT_F_CNEW: case PT_F_CVIS: case PT_F_CBUOY: return 5;
        default: return 3;
    }
}
static double* field_ptr(Engine& E, int id) {
    switch (id) {
        case PT_F_T: return E.T;
        case PT_F_TRATIO: return E.Tratio;
        case PT_F_TVIS: return E.Tvis;
        case PT_F_TBUOY: return E.Tbuoy;
        case PT_F_CNEW: return E.Cnew;
        case PT_F_CVIS: return E.Cvis;
        case PT_F_CBUOY: return E.Cbuoy;
        case PT_F_SF: return E.SF;
        case PT_F_U: return E.u;
        case PT_F_W: return E.w;
        case PT_F_VIS: return E.vis[1];
        case PT_F_RHS: return E.RHS[1];
        case PT_F_TRACER_R: return E.rtr;
        case PT_F_TRACER_S: return E.str;
        case PT_F_TRACER_T: return E.Ttr;
        case PT_F_TRACER_C: return E.Ctr;
        default: return nullptr;
    }
}

static int copy_grid(Engine& E, int id, void* host, bool to_device) {
    double* d = field_ptr(E, id);
    if (!d) return fail(PT_ERR_ARG, "unknown field id");
    int gh = field_ghost(id), lo = -gh, hix = E.K.nx + gh, hiz = E.K.nz + gh;
    if (id == PT_F_RHS) { lo = 1; hix = E.K.nx - 1; hiz = E.K.nz - 1; }
    size_t w = (size_t)(hix - lo + 1), h = (size_t)(hiz - lo + 1);
    double* dp = d + E.g1.at(lo, lo);
    cudaError_t e;
    if (to_device)
        e = cudaMemcpy2DAsync(dp, E.g1.pitch * 8, host, w * 8, w * 8, h, cudaMemcpyHostToDevice, E.st);
    else
        e = cudaMemcpy2DAsync(host, w * 8, dp, E.g1.pitch * 8, w * 8, h, cudaMemcpyDeviceToHost, E.st);
    CK(e);
    CK(cudaStreamSynchronize(E.st));
    return 0;
}

}  // namespace pt

using namespace pt;

extern "C" {

const char* pt_last_error(void) { return g_err.c_str(); }

int pt_init(const pt_config* cfg) {
    if (!cfg) return fail(PT_ERR_ARG, "null config");
    if (g_eng) pt_finalize();
    TRACE("pt_init: constants");
    Engine* E = new Engine();
    E->cfg = *cfg;
    E->ntr = cfg->ntr;
    int rc = setup_constants(*E);
    if (rc) { delete E; return rc; }
    if (cfg->precision != PT_PREC_FP64 && cfg->precision != PT_PREC_MIXED) {
        delete E;
        return fail(PT_ERR_CONFIG, "precision must be PT_PREC_FP64 or PT_PREC_MIXED");
    }
    if ((int64_t)cfg->ntr > 2000000000LL) { delete E; return fail(PT_ERR_CONFIG, "ntr above 2e9 is not supported"); }
    if (cfg->direct != 0 && (cfg->direct != 1 || cfg->precision != PT_PREC_FP64 || cfg->ivis != 0)) {
        delete E;
        return fail(PT_ERR_CONFIG, "direct = 1 (banded direct solve) runs in PT_PREC_FP64 with ivis = 0");
    }
    if (cfg->reference_rounding != 0 && (cfg->reference_rounding != 1 || cfg->precision != PT_PREC_FP64)) {
        delete E;
        return fail(PT_ERR_CONFIG, "reference_rounding = 1 applies to PT_PREC_FP64 only");
    }
    if (cfg->discrete_types != 0 && (cfg->discrete_types != 1 || cfg->comp != 1)) {
        delete E;
        return fail(PT_ERR_CONFIG, "discrete_types = 1 needs comp = 1 (one dense type, ntype = 1)");
    }
    if (cfg->equalize != 0 && (cfg->equalize != 1 || (cfg->comp == 1 && cfg->discrete_types != 1) ||
                               cfg->dist_factor <= 0.0 || cfg->dist_factor >= 0.5 || (cfg->comp == 0 && cfg->tpc <= 0))) {
        delete E;
        return fail(PT_ERR_CONFIG, "equalize = 1 needs discrete_types = 1 (comp = 1) or tpc > 0 (comp = 0), "
                                   "and 0 < dist_factor < 0.5");
    }
    if (cfg->krylov != 0 && (cfg->krylov < 0 || cfg->krylov > kGcrMax || cfg->precision != PT_PREC_MIXED)) {
        delete E;
        return fail(PT_ERR_CONFIG, "krylov = 1..8 (GCR directions) applies to PT_PREC_MIXED only");
    }
    TRACE("pt_init: geometry and stream");
    E->g1 = make_geo(cfg->nx, cfg->nz);
    for (int l = 1; l <= E->grids; l++) E->gl[l] = make_geo(E->L[l].nx, E->L[l].nz);
    if ((rc = cuda_check(cudaStreamCreateWithFlags(&E->st, cudaStreamNonBlocking), "stream"))) { delete E; return rc; }
    for (int q = 0; q < 2; q++)
        for (int j = 0; j < 2; j++) cudaEventCreate(&E->gev[q][j]);
    g_eng = E;
    TRACE("pt_init: device allocations and constants");
    if ((rc = engine_alloc(*E)) || (rc = upload_consts_fields(*E)) || (rc = upload_consts_tracers(*E)) ||
        (rc = upload_consts_mg(*E)) || (rc = upload_consts_mixed(*E)) || (rc = noalloc_scratch_setup(nullptr))) {
        std::string msg = g_err;
        pt_finalize();
        g_err = msg;
        return rc;
    }
    rc = cuda_check(cudaStreamSynchronize(E->st), "init");
    TRACE("pt_init: done");
    return rc;
}

int pt_finalize(void) {
    if (!g_eng) return 0;
    engine_free(*g_eng);
    delete g_eng;
    g_eng = nullptr;
    return 0;
}

int pt_grids(void) { return g_eng ? g_eng->grids : 0; }

int pt_field_extent(int field, int32_t* lo_x, int32_t* hi_x, int32_t* lo_z, int32_t* hi_z, int32_t* elem_bytes) {
    if (int rc = need(g_eng != nullptr)) return rc;
    Engine& E = *g_eng;
    int32_t a = 0, b = 0, c = 0, d = 0, eb = 8;
    if (field >= PT_F_TRACER_R && field <= PT_F_TRACER_C) { a = 1; b = (int32_t)E.ntr; }
    else if (field == PT_F_NEMPTY || (field == PT_F_COUNT_TYPE && E.count1)) { a = 0; b = E.K.nx; c = 0; d = E.K.nz; eb = 4; }
    else if (field == PT_F_TRACER_TYPE && E.cfg.discrete_types) { a = 1; b = (int32_t)E.ntr; eb = 4; }
    else if (field == PT_F_RHS) { a = 1; b = E.K.nx - 1; c = 1; d = E.K.nz - 1; }
    else if (field_ptr(E, field)) { int g = field_ghost(field); a = -g; b = E.K.nx + g; c = -g; d = E.K.nz + g; }
    else return fail(PT_ERR_ARG, "unknown field id");
    if (lo_x) *lo_x = a;
    if (hi_x) *hi_x = b;
    if (lo_z) *lo_z = c;
    if (hi_z) *hi_z = d;
    if (elem_bytes) *elem_bytes = eb;
    return 0;
}

int pt_set_field(int field, const void* host) {
    if (g_eng) {
        // new temperature or composition fields change the viscosity, hence the operator: the
        // coarse levels and factorisation are rebuilt at the next solve.  Tracer arrays do not enter
        // the operator before the next projection (which the time level's own rebuild follows);
        // a new psi restarts the psi history.
        const bool tracers = field >= PT_F_TRACER_R && field <= PT_F_TRACER_C;
        if (!tracers && field != PT_F_SF && field != PT_F_U && field != PT_F_W) g_eng->coarse_ready = false;
        if (field == PT_F_SF) g_eng->hist_n = 0;
    }
    if (int rc = need(g_eng != nullptr)) return rc;
    if (!host) return fail(PT_ERR_ARG, "null pointer");
    Engine& E = *g_eng;
    if (field == PT_F_NEMPTY || field == PT_F_VIS || field == PT_F_RHS || field == PT_F_COUNT_TYPE)
        return fail(PT_ERR_ARG, "field is read-only");
    if (field == PT_F_TRACER_TYPE) {
        if (!E.cfg.discrete_types) return fail(PT_ERR_ARG, "tracer types exist with discrete_types = 1 only");
        CK(cudaMemcpyAsync(E.tcell, host, sizeof(int32_t) * (size_t)E.ntr, cudaMemcpyHostToDevice, E.st));
        if (!E.perm_active) return types_to_c(E, E.tcell, E.Ctr);
        if (int rc = types_to_c(E, E.tcell, E.str2)) return rc;  // user order, staged
        if (int rc = tracer_user_order(E, E.Ctr, E.str2, false)) return rc;
        CK(cudaStreamSynchronize(E.st));
        return 0;
    }
    if (field == PT_F_TRACER_C && E.cfg.discrete_types)
        return fail(PT_ERR_ARG, "discrete_types = 1: set the tracer types (PT_F_TRACER_TYPE), not C");
    if (field >= PT_F_TRACER_R && field <= PT_F_TRACER_C) {
        const size_t nb = sizeof(double) * (size_t)E.ntr;
        if (!E.perm_active) {
            CK(cudaMemcpy(field_ptr(E, field), host, nb, cudaMemcpyHostToDevice));
            return 0;
        }
        // re-sorted tracers: the host array is in the user's order (staged in an RK stage buffer)
        CK(cudaMemcpyAsync(E.str2, host, nb, cudaMemcpyHostToDevice, E.st));
        if (int rc = tracer_user_order(E, field_ptr(E, field), E.str2, false)) return rc;
        CK(cudaStreamSynchronize(E.st));
        return 0;
    }
    return copy_grid(E, field, const_cast<void*>(host), true);
}

int pt_get_field(int field, void* host) {
    if (int rc = need(g_eng != nullptr)) return rc;
    if (!host) return fail(PT_ERR_ARG, "null pointer");
    Engine& E = *g_eng;
    CK(cudaStreamSynchronize(E.st));
    if (field == PT_F_NEMPTY || field == PT_F_COUNT_TYPE) {
        const int32_t* src = field == PT_F_NEMPTY ? E.nempty : E.count1;
        if (!src) return fail(PT_ERR_ARG, "count_type exists with discrete_types = 1 only");
        CK(cudaMemcpy(host, src, sizeof(int32_t) * (size_t)(E.K.nx + 1) * (E.K.nz + 1), cudaMemcpyDeviceToHost));
        return 0;
    }
    if (field == PT_F_TRACER_TYPE) {
        if (!E.cfg.discrete_types) return fail(PT_ERR_ARG, "tracer types exist with discrete_types = 1 only");
        const double* c = E.Ctr;
        if (E.perm_active) {  // back to the user's order
            if (int rc = tracer_user_order(E, E.Ctr, E.str2, true)) return rc;
            c = E.str2;
        }
        if (int rc = c_to_types(E, c, E.tcell)) return rc;
        CK(cudaMemcpyAsync(host, E.tcell, sizeof(int32_t) * (size_t)E.ntr, cudaMemcpyDeviceToHost, E.st));
        CK(cudaStreamSynchronize(E.st));
        return 0;
    }
    if (field >= PT_F_TRACER_R && field <= PT_F_TRACER_C) {
        const size_t nb = sizeof(double) * (size_t)E.ntr;
        const double* src = field_ptr(E, field);
        if (E.perm_active) {  // back to the user's order
            if (int rc = tracer_user_order(E, const_cast<double*>(src), E.str2, true)) return rc;
            src = E.str2;
        }
        CK(cudaMemcpyAsync(host, src, nb, cudaMemcpyDeviceToHost, E.st));
        CK(cudaStreamSynchronize(E.st));
        return 0;
    }
    return copy_grid(E, field, host, false);
}

int pt_upload_state(const double* xg, const double* zg, const double* T, const double* Cnew, const double* SF,
                    const double* rtr, const double* str, const double* Ctr, const double* Ttr, const int32_t* Ttype) {
    if (int rc = need(g_eng != nullptr)) return rc;
    Engine& E = *g_eng;
    const bool og = E.cfg.discrete_types != 0;
    if (!xg || !zg || !T || !SF || !rtr || !str || !Ttr || (E.cfg.comp && !Cnew) || (E.cfg.comp && !og && !Ctr))
        return fail(PT_ERR_ARG, "null pointer in restart arrays");
    if (og != (Ttype != nullptr))
        return fail(PT_ERR_ARG, og ? "discrete_types = 1: Ttype is required" : "Ttype given without discrete_types = 1");
    const int nx = E.K.nx, nz = E.K.nz;
    for (int i = 0; i <= nx; i++)
        if (std::fabs(xg[i + 6] - E.K.dr * i) > 1e-12 * E.K.aspect)
            return fail(PT_ERR_CONFIG, "xg is not the uniform grid (stretched grids are not supported)");
    for (int k = 0; k <= nz; k++)
        if (std::fabs(zg[k + 6] - E.K.ds * k) > 1e-12) return fail(PT_ERR_CONFIG, "zg is not the uniform grid");
    int rc;
    double* zero_these[] = {E.T, E.Tratio, E.Tvis, E.Tbuoy, E.Cnew, E.Cvis, E.Cbuoy, E.SF, E.u, E.w};
    for (auto p : zero_these) CK(cudaMemsetAsync(p, 0, E.g1.elems() * 8, E.st));
    for (int l = 1; l <= E.grids; l++) CK(cudaMemsetAsync(E.err[l], 0, E.gl[l].elems() * 8, E.st));
    if ((rc = copy_grid(E, PT_F_T, const_cast<double*>(T), true))) return rc;
    if ((rc = copy_grid(E, PT_F_SF, const_cast<double*>(SF), true))) return rc;
    if (E.cfg.comp && (rc = copy_grid(E, PT_F_CNEW, const_cast<double*>(Cnew), true))) return rc;
    const size_t nb = sizeof(double) * (size_t)E.ntr;
    CK(cudaMemcpyAsync(E.rtr, rtr, nb, cudaMemcpyHostToDevice, E.st));
    CK(cudaMemcpyAsync(E.str, str, nb, cudaMemcpyHostToDevice, E.st));
    CK(cudaMemcpyAsync(E.Ttr, Ttr, nb, cudaMemcpyHostToDevice, E.st));
    if (og) {  // the types, held as 0.0 / 1.0 in the composition array
        CK(cudaMemcpyAsync(E.tcell, Ttype, sizeof(int32_t) * (size_t)E.ntr, cudaMemcpyHostToDevice, E.st));
        if ((rc = types_to_c(E, E.tcell, E.Ctr))) return rc;
    } else if (E.cfg.comp) {
        CK(cudaMemcpyAsync(E.Ctr, Ctr, nb, cudaMemcpyHostToDevice, E.st));
    }
    if ((rc = tracer_order_reset(E))) return rc;
    TRACE("upload: boundary conditions");
    // grid.f90:67-73: boundary conditions on the restart fields
    if ((rc = enforce_bcs_T(E, E.T))) return rc;
    if ((rc = enforce_bcs_stream(E, 1, E.SF))) return rc;
    if (E.cfg.comp && (rc = enforce_bcs_C(E, E.Cnew))) return rc;
    TRACE("upload: projection and smoothers");
    // grid.f90:93-95: projection without smoothing, then main.f90:205-209
    if ((rc = project(E, E.rtr, E.str, E.Ttr, E.T, 0))) return rc;
    if ((rc = smoother_time_T(E, E.T))) return rc;
    if (E.cfg.comp && (rc = smoother_time_C(E))) return rc;
    if ((rc = load_conductivity(E))) return rc;
    E.time = 0.0;
    E.have_mass = 0;
    E.uploaded = 1;
    E.coarse_ready = false;
    E.hist_n = 0;
    CK(cudaStreamSynchronize(E.st));
    return 0;
}

int pt_download_state(double* T, double* Cnew, double* SF, double* rtr, double* str, double* Ctr, double* Ttr,
                      int32_t* Ttype) {
    if (int rc = need(g_eng != nullptr && g_eng->uploaded)) return rc;
    int rc;
    if (T && (rc = pt_get_field(PT_F_T, T))) return rc;
    if (Cnew && (rc = pt_get_field(PT_F_CNEW, Cnew))) return rc;
    if (SF && (rc = pt_get_field(PT_F_SF, SF))) return rc;
    if (rtr && (rc = pt_get_field(PT_F_TRACER_R, rtr))) return rc;
    if (str && (rc = pt_get_field(PT_F_TRACER_S, str))) return rc;
    if (Ctr && (rc = pt_get_field(PT_F_TRACER_C, Ctr))) return rc;
    if (Ttr && (rc = pt_get_field(PT_F_TRACER_T, Ttr))) return rc;
    if (Ttype && (rc = pt_get_field(PT_F_TRACER_TYPE, Ttype))) return rc;
    return 0;
}

// x = a + c (a - b) over the whole padded array (boundary-consistent inputs stay consistent)
__global__ void k_extrapolate(double* x, const double* pa, const double* pb, double c, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) x[q] = pa[q] + c * (pa[q] - pb[q]);
}

static int extrapolated_guess(Engine& E) {
    if (E.hist_n < 2 || !(E.tau_a > E.tau_b) || E.solve_tau == E.tau_a) return 0;  // previous psi
    const double c = (E.solve_tau - E.tau_a) / (E.tau_a - E.tau_b);
    const size_t n = E.g1.elems();
    k_extrapolate<<<(unsigned)((n + 255) / 256), 256, 0, E.st>>>(E.SF, E.psi_a, E.psi_b, c, n);
    return cuda_check(cudaGetLastError(), "k_extrapolate");
}

static int record_psi(Engine& E) {
    const size_t bytes = E.g1.elems() * sizeof(double);
    if (!E.psi_a) {
        CK(cudaMalloc(&E.psi_a, bytes));
        CK(cudaMalloc(&E.psi_b, bytes));
    }
    if (E.hist_n > 0 && E.solve_tau == E.tau_a) {  // same solve time: the newer psi replaces a
        CK(cudaMemcpyAsync(E.psi_a, E.SF, bytes, cudaMemcpyDeviceToDevice, E.st));
        return 0;
    }
    std::swap(E.psi_a, E.psi_b);
    E.tau_b = E.tau_a;
    CK(cudaMemcpyAsync(E.psi_a, E.SF, bytes, cudaMemcpyDeviceToDevice, E.st));
    E.tau_a = E.solve_tau;
    E.hist_n = E.hist_n < 2 ? E.hist_n + 1 : 2;
    return 0;
}

static int solve_psi(Engine& E, pt_solve_info* info) {
    int rc;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, E.st);
    if (E.cfg.guess_mode == PT_GUESS_ZERO) CK(cudaMemsetAsync(E.SF, 0, E.g1.elems() * 8, E.st));
    if (E.cfg.guess_mode == PT_GUESS_EXTRAPOLATE && (rc = extrapolated_guess(E))) return rc;
    rc = E.cfg.direct ? direct_solve(E, info)
                      : (E.cfg.precision == PT_PREC_MIXED) ? multigrid_mixed(E, info) : multigrid(E, info);
    if (!rc && E.cfg.guess_mode == PT_GUESS_EXTRAPOLATE) rc = record_psi(E);
    if (!rc && E.pair_ring) rc = capture_pair(E);  // training pairs of a time-evolved run
    if (!rc) rc = compute_velocities(E);
    cudaEventRecord(b, E.st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    harvest_spans(E);
    if (info) {
        info->ms += ms;
        info->n_temp = E.n_temp;
        info->refinements += E.refinements;
    }
    return rc;
}

int pt_solve_psi(pt_solve_info* info) {
    if (int rc = need(g_eng != nullptr && g_eng->uploaded)) return rc;
    if (info) std::memset(info, 0, sizeof *info);
    g_eng->solve_tau = g_eng->time;
    return solve_psi(*g_eng, info);
}

static int stage_tables(Engine& E) {
    PhaseTimer tm(E, PH_GRID);
    int rc;
    if (use_tables_fx(E)) {
        if ((rc = tracer_space_fx(E))) return rc;
        return tables_fx(E, 2, E.tsa);
    }
    if ((rc = load_tracer_space(E))) return rc;
    if ((rc = compute_derivatives(E, E.tsa, 2))) return rc;
    return tables_to_f32(E, 2, E.tsa);
}
static int velocity_tables(Engine& E) {
    PhaseTimer tm(E, PH_GRID);
    int rc;
    if (use_tables_fx(E)) {
        if ((rc = tables_fx(E, 0, E.u))) return rc;
        return tables_fx(E, 1, E.w);
    }
    if ((rc = compute_derivatives(E, E.u, 0))) return rc;
    if ((rc = compute_derivatives(E, E.w, 1))) return rc;
    if ((rc = tables_to_f32(E, 0, E.u))) return rc;
    return tables_to_f32(E, 1, E.w);
}

// energy_time_Chebyshev (Chebyshev.f90:113-243): stage 1 from the step-start tracers (their slopes
// kept), stages 2..nstage each after a projection of the previous stage's tracers, a fresh psi
// (RK_update=1) and new tables; the last stage's tracers are the step's result
static int step_rkc2(Engine& E, double* dt_out, pt_solve_info* info) {
    int rc;
    if ((rc = stability_dt(E, &E.dt))) return rc;
    if (E.cfg.equalize && (rc = equalize_tracers(E, nullptr))) return rc;  // Chebyshev.f90:131-137
    const int comp = E.cfg.comp;
    if (comp && (rc = copy_field(E, E.C0, E.Cnew))) return rc;
    if ((rc = copy_field(E, E.T0, E.Tratio))) return rc;
    std::swap(E.rtr0, E.rtr);  // the step-start tracers (the stages write rtr/str/Ttr last)
    std::swap(E.str0, E.str);
    std::swap(E.Ttr0, E.Ttr);
    if ((rc = stage_tables(E)) || (rc = velocity_tables(E)) || (rc = rkc2_stage(E, 1))) return rc;
    double tstage = E.time + E.mewtCheb[1] * E.dt;
    for (int j = 2; j <= E.cfg.nstage; j++) {
        if (comp && (rc = copy_field(E, E.Cnew, E.C0))) return rc;
        if ((rc = project(E, E.rtr1, E.str1, E.Ttr1, E.T0, 1))) return rc;
        if ((rc = stage_tables(E))) return rc;
        E.solve_tau = tstage;
        if ((rc = solve_psi(E, info))) return rc;
        if ((rc = velocity_tables(E)) || (rc = rkc2_stage(E, j))) return rc;
        tstage = E.time + E.mewtCheb[j] * E.dt;
    }
    if (comp && (rc = copy_field(E, E.Cnew, E.C0))) return rc;
    if ((rc = project(E, E.rtr, E.str, E.Ttr, E.T0, 1))) return rc;
    if ((rc = copy_field(E, E.T, E.Tratio))) return rc;
    E.time = E.time + E.dt;
    if (dt_out) *dt_out = E.dt;
    if (info) info->n_temp = E.n_temp;
    CK(cudaStreamSynchronize(E.st));
    harvest_spans(E);
    return 0;
}

int pt_step(double* dt_out, pt_solve_info* info) {
    if (int rc = need(g_eng != nullptr && g_eng->uploaded)) return rc;
    Engine& E = *g_eng;
    if (info) std::memset(info, 0, sizeof *info);
    if (E.cfg.chebyshev) return step_rkc2(E, dt_out, info);
    int rc;
    if (E.want_resort && (rc = resort_tracers(E))) return rc;
    if ((rc = stability_dt(E, &E.dt))) return rc;
    if (E.cfg.equalize && (rc = equalize_tracers(E, nullptr))) return rc;  // energy.f90:198-204
    const int comp = E.cfg.comp;
    if (comp && (rc = copy_field(E, E.C0, E.Cnew))) return rc;
    if ((rc = copy_field(E, E.T0, E.Tratio))) return rc;
    // the step-start tracers (energy.f90:262-266) by exchanging buffers instead of copying them:
    // the RK stages write rtr/str/Ttr before reading them (stage 1 starts the FP64 path's slope
    // sums there; the mixed path writes them at stage 4)
    std::swap(E.rtr0, E.rtr);
    std::swap(E.str0, E.str);
    std::swap(E.Ttr0, E.Ttr);
    // stage 1
    if ((rc = stage_tables(E)) || (rc = velocity_tables(E)) || (rc = rk_stage(E, 1))) return rc;
    // stages 2-4: project the stage positions, re-solve psi, advance
    const double* sr[3] = {E.rtr1, E.rtr2, E.rtr1};
    const double* ss[3] = {E.str1, E.str2, E.str1};
    const double* sT[3] = {E.Ttr1, E.Ttr2, E.Ttr1};
    for (int st = 2; st <= 4; st++) {
        if (comp && st > 2 && (rc = copy_field(E, E.Cnew, E.C0))) return rc;
        if ((rc = project(E, sr[st - 2], ss[st - 2], sT[st - 2], E.T0, 1))) return rc;
        if ((rc = stage_tables(E))) return rc;
        E.solve_tau = E.time + (st == 4 ? E.dt : 0.5 * E.dt);  // stage time of this solve
        if ((rc = solve_psi(E, info))) return rc;
        if ((rc = velocity_tables(E)) || (rc = rk_stage(E, st))) return rc;
    }
    // wrap-up
    if (comp && (rc = copy_field(E, E.Cnew, E.C0))) return rc;
    if ((rc = project(E, E.rtr, E.str, E.Ttr, E.T0, 1))) return rc;
    if ((rc = copy_field(E, E.T, E.Tratio))) return rc;
    E.time = E.time + E.dt;
    if (dt_out) *dt_out = E.dt;
    if (info) info->n_temp = E.n_temp;
    CK(cudaStreamSynchronize(E.st));
    harvest_spans(E);
    return 0;
}

int pt_equalize_tracers(pt_equalize_info* info) {
    if (int rc = need(g_eng != nullptr && g_eng->uploaded)) return rc;
    Engine& E = *g_eng;
    if (E.cfg.comp == 1 && !E.cfg.discrete_types)
        return fail(PT_ERR_CONFIG, "tracer equalisation needs discrete tracer types (iC_continuous = 0)");
    if (E.cfg.comp == 0 && E.cfg.tpc <= 0) return fail(PT_ERR_CONFIG, "tracer equalisation needs tpc > 0 (comp = 0)");
    if (!(E.cfg.dist_factor > 0.0 && E.cfg.dist_factor < 0.5))
        return fail(PT_ERR_CONFIG, "tracer equalisation needs 0 < dist_factor < 0.5");
    int rc = equalize_tracers(E, info);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(E.st), "equalize");
    return rc;
}

int pt_stats(pt_stats_row* out) {
    if (int rc = need(g_eng != nullptr && g_eng->uploaded)) return rc;
    if (!out) return fail(PT_ERR_ARG, "null pointer");
    return stats(*g_eng, out);
}

int pt_tracers_to_corners(const double* T0, int smooth_vis) {
    if (int rc = need(g_eng != nullptr && g_eng->uploaded)) return rc;
    Engine& E = *g_eng;
    int rc;
    if (T0) {
        if ((rc = copy_grid(E, PT_F_TRATIO, const_cast<double*>(T0), true))) return rc;
    }
    rc = project(E, E.rtr, E.str, E.Ttr, E.Tratio, smooth_vis);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(E.st), "projection");
    return rc;
}

int pt_tracers_to_corners_noalloc(const double* T0, int smooth_vis) {
    if (int rc = need(g_eng != nullptr && g_eng->uploaded)) return rc;
    Engine& E = *g_eng;
    int rc;
    if (T0) {
        if ((rc = copy_grid(E, PT_F_TRATIO, const_cast<double*>(T0), true))) return rc;
    }
    rc = project_noalloc(E, E.Tratio, smooth_vis);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(E.st), "projection");
    return rc;
}

int pt_time(double* time, double* dt) {
    if (int rc = need(g_eng != nullptr)) return rc;
    if (time) *time = g_eng->time;
    if (dt) {
        int rc = stability_dt(*g_eng, &g_eng->dt);
        if (rc) return rc;
        *dt = g_eng->dt;
    }
    return 0;
}

int pt_set_guess_mode(int mode, const char* weights_path) {
    if (int rc = need(g_eng != nullptr)) return rc;
    if (mode != PT_GUESS_PREVIOUS && mode != PT_GUESS_ZERO && mode != PT_GUESS_UNET && mode != PT_GUESS_EXTRAPOLATE)
        return fail(PT_ERR_ARG, "unknown guess mode");
    if (mode == PT_GUESS_UNET) {
        if (int rc = unet_engine_load(*g_eng, weights_path)) return rc;
    }
    g_eng->cfg.guess_mode = mode;
    return 0;
}

int pt_prof_enable(int on) {
    if (int rc = need(g_eng != nullptr)) return rc;
    g_eng->prof = on ? 1 : 0;
    return 0;
}

int pt_prof_reset(void) {
    if (int rc = need(g_eng != nullptr)) return rc;
    CK(cudaStreamSynchronize(g_eng->st));
    harvest_spans(*g_eng);
    for (int q = 0; q < 8; q++) { g_eng->kcount[q] = 0; g_eng->kms[q] = 0.0; }
    g_launches = 0;
    return 0;
}

int pt_prof_kernel(int id, int64_t* launches, double* total_ms) {
    if (int rc = need(g_eng != nullptr)) return rc;
    if (id < 0 || id >= 8) return fail(PT_ERR_ARG, "kernel id out of range");
    CK(cudaStreamSynchronize(g_eng->st));
    harvest_spans(*g_eng);
    if (launches) *launches = g_eng->kcount[id];
    if (total_ms) *total_ms = g_eng->kms[id];
    return 0;
}

int64_t pt_prof_launches(void) { return g_launches.load(); }

int pt_prof_table(int which, float* host) {
    if (int rc = need(g_eng != nullptr)) return rc;
    Engine& E = *g_eng;
    if (which < 0 || which > 2 || !host) return fail(PT_ERR_ARG, "table id out of range or null pointer");
    if (!E.ftab[which]) return fail(PT_ERR_STATE, "the FP32 tables exist in mixed precision only");
    const size_t w = (size_t)(E.K.nx + 1) * sizeof(float4);
    CK(cudaMemcpy2DAsync(host, w, E.ftab[which] + E.g1.at(0, -3), E.g1.pitch * sizeof(float4), w,
                         (size_t)(E.K.nz + 7), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    return 0;
}

int pt_prof_tracer_order(int64_t* resorts, double* runs_per_thread) {
    if (int rc = need(g_eng != nullptr)) return rc;
    if (resorts) *resorts = g_eng->resorts;
    if (runs_per_thread) *runs_per_thread = g_eng->last_runs;
    return 0;
}

int pt_prof_residuals(double* out, int cap, int* count) {
    if (int rc = need(g_eng != nullptr)) return rc;
    const std::vector<double>& h = g_eng->res_hist;
    if (count) *count = (int)h.size();
    if (out)
        for (int q = 0; q < cap && q < (int)h.size(); q++) out[q] = h[(size_t)q];
    return 0;
}

int pt_prof_region(int end, double* ms) {
    if (int rc = need(g_eng != nullptr)) return rc;
    Engine& E = *g_eng;
    if (!E.rev0) {
        CK(cudaEventCreate(&E.rev0));
        CK(cudaEventCreate(&E.rev1));
    }
    if (!end) {
        nvtxRangePushA("pt_timed");
        CK(cudaEventRecord(E.rev0, E.st));
        return 0;
    }
    CK(cudaEventRecord(E.rev1, E.st));
    CK(cudaEventSynchronize(E.rev1));
    nvtxRangePop();
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, E.rev0, E.rev1));
    if (ms) *ms = f;
    return 0;
}

int pt_phase_times(double* ms8) {
    if (int rc = need(g_eng != nullptr)) return rc;
    if (!ms8) return fail(PT_ERR_ARG, "null pointer");
    CK(cudaStreamSynchronize(g_eng->st));
    harvest_spans(*g_eng);
    for (int q = 0; q < PT_NPHASE; q++) ms8[q] = g_eng->phase_ms[q];
    return 0;
}

}  // extern "C"
