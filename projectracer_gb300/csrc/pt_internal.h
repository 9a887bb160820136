// pt_internal.h -- device state and kernel interfaces of libptgpu (not part of the C ABI).
//
// Grid layout in HBM: every grid array (physical fields on the fine grid and the multigrid level
// arrays) stores node (i,k) at  p[(i+GH) + (k+GH)*pitch]  with a uniform ghost width GH=5 and a
// row pitch rounded up to 16 doubles (128 B), x fastest as in the reference's column-major
// arrays.  Ghost width 5 covers the widest reference extent (spanT=5 for C, conductivity and the
// extended T); fields with 3 ghosts simply leave the outer two unused.
// Tracers are structure-of-arrays FP64 vectors in tracer-ID order.
#pragma once

#include <cuda_runtime.h>
#include <cstdio>
#include <stdint.h>

#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ptgpu.h"

#define GH 5
#define PT_MAXLEV 8
constexpr int kGcrMax = 8;  // most GCR search directions of the mixed-precision solve (pt_config.krylov)

enum { PH_RK = 0, PH_PROJECT, PH_SOLVE, PH_SETUP, PH_CYCLE_L1, PH_CYCLE_COARSE, PH_GRID, PH_FACTOR, PT_NPHASE };

namespace pt {

struct Geo {
    int nx, nz, pitch;
    size_t elems() const { return (size_t)pitch * (size_t)(nz + 2 * GH + 1); }
    __host__ __device__ inline size_t at(int i, int k) const {
        return (size_t)(i + GH) + (size_t)(k + GH) * (size_t)pitch;
    }
};

// constants of one multigrid level (uniform grid: eigenvalue symbols are per-level scalars)
struct LevConst {
    int nx, nz;
    double dr, ds, dr2, ds2, dr3, ds3, dr4, ds4, drds, drds2, dr2ds, dr2ds2;
    // reciprocals of the above (exact for the power-of-two spacings of a multigrid hierarchy)
    double idr, ids, idr2, ids2, idr3, ids3, idr4, ids4, idrds, idrds2, idr2ds, idr2ds2;
    double SR1, SR2, SR4, SR5, SR6, SI1, SI2, SI4, SI5, SI6;
    double dt_vis;
};

// stencils and scalars shared by the kernels (copied to __constant__ memory)
struct Consts {
    double D1[7], D2[7], D3[7], D4[7];
    double Dm[5][7];  // D(1..4,-3:3)
    double Drs[5][5], Drss[5][5], Drrs[5][5], Drrss[5][5];  // [i+2][k+2]
    double D1so[3], D2so[3], Drsso[3][3];                    // [i+1][k+1]
    double SM1[7][7], SM2[7][7], SM4[7][7], SM5[7][7], SM6[7][7];  // [di+3][dk+3]
    double mewt[64], mew[64], vv[64], cc[64];
    double dr, ds, dr2, ds2, inv_dr, inv_ds, aspect;
    double dr_pow[4], ds_pow[4], fact[4];
    double inv_ds_pow[4], inv_dr_pow[4], inv_fact[4], inv_dr2, inv_ds2;
    int exact_div;  // dr and ds are powers of two: x/dr == x*inv_dr exactly
    int p_inv_dr, p_inv_ds;  // inv_dr = 2^p_inv_dr, inv_ds = 2^p_inv_ds when exact_div
    double two_over_D20;
    double Tbot_iso, Ttop_iso, H, Htype, conduct_factor;
    double RaT, RaC, lvisT, lvisP, lvisC;
    int nx, nz, comp, Tbot, Vbc, ivis;
};

// the per-level arrays a viscosity pass writes (compute_viscosity): the cycle's own, or the set
// the next time level's coarse levels are built into on the side stream (mixed precision)
struct VisLevels {
    double *vis[PT_MAXLEV], *visst[PT_MAXLEV], *vx[PT_MAXLEV], *vz[PT_MAXLEV], *vxx[PT_MAXLEV], *vzz[PT_MAXLEV],
        *vxz[PT_MAXLEV], *vxxpzz[PT_MAXLEV], *vxxmzz[PT_MAXLEV], *vsm[PT_MAXLEV], *ratio[PT_MAXLEV], *dtst[PT_MAXLEV];
};
constexpr int kVisArrays = 12;  // the members of VisLevels

// weights of the exact-sum stream operator of one level (pt_exact.cuh)
struct ResFxK {
    double k[10];  // per derivative group: the weight that turns its integer sum into the term
    int square;    // dr == ds: the derivatives are combined in integer arithmetic into 5 groups
};

struct Engine {
    pt_config cfg;
    Consts K;
    LevConst L[PT_MAXLEV];
    int grids = 0, nsteps = 0, multi[64];
    int mnsteps = 0, mmulti[64];  // schedule of the mixed-precision solve (PT_CYCLE_*)
    double RKC1_stability = 0, delta_T = 2, delta_C = 2, dts = 0;
    // the coarse-level RKC1 smoother of the mixed V-cycle (nstageC stages, same damping)
    int nstageC = 0;
    double RKC1_stability_c = 0, mew_c[64] = {}, vv_c[64] = {}, mewt_c[64] = {};
    // the RKC2 energy stepper (cfg.chebyshev): coefficients and the stage-1 slopes of each tracer
    double cCheb[64] = {}, mewCheb[64] = {}, vCheb[64] = {}, mewtCheb[64] = {}, gtCheb[64] = {};
    double *k0r = nullptr, *k0s = nullptr, *k0T = nullptr;
    double Tr_base = 0, Trr_base = 0, Trrr_base = 0, Trrrr_base = 0, Trs_base = 0, Trrs_base = 0,
           Trrss_base = 0, Tr_base_so = 0, Trr_base_so = 0;
    int kl = 0, ku = 0, ngc = 0, kent = 0;
    Geo g1;        // fine-grid geometry
    Geo gl[PT_MAXLEV];
    cudaStream_t st = nullptr;
    // physical fields (fine geometry)
    double *T = nullptr, *Tratio = nullptr, *Tvis = nullptr, *Tbuoy = nullptr, *Cnew = nullptr,
           *Cvis = nullptr, *Cbuoy = nullptr, *SF = nullptr, *u = nullptr, *w = nullptr,
           *cond = nullptr, *cond_r = nullptr, *cond_s = nullptr, *tsa = nullptr, *Text = nullptr,
           *T0 = nullptr, *C0 = nullptr, *scratch = nullptr;
    double* der[3][3] = {};  // derivative tables: [field u,w,tsa][order 1..3]
    float4* ftab[3] = {};    // mixed precision: per node (value, x-derivatives 1..3) in FP32, fields u, w, dT/dt
    float* facc[3] = {};     // mixed precision: per tracer FP32 sums of the RK slopes of r, s, T
    double* coef[3] = {};    // 16 Taylor coefficients per node per field (advection)
    int32_t* nempty = nullptr;
    int32_t* count1 = nullptr;  // discrete types: count_type(1, 0:nx, 0:nz) of the last projection
    // direct banded solve (cfg.direct, pt_direct.cu): band matrix and LU, row factors, right-hand
    // side, pivots, the LU kernel's barrier state and error words
    int dn = 0, dkl = 0, dku = 0, dahead = 8;  // dahead: the substitution kernel's column lookahead
    double *dMB = nullptr, *dRow = nullptr, *dB = nullptr;
    int *dipiv = nullptr, *dluerr = nullptr;
    void* dlu = nullptr;
    bool direct_ready = false;
    void* io = nullptr;  // snapshot / restart writer state (pt_io.cu)
    void* eq = nullptr;  // tracer equalisation scratch (pt_equalize.cu)
    int64_t eq_calls = 0;  // equalisations so far: the call index of the next one
    int32_t eq_done = 0;   // equalisations that moved tracers (the reference's nequalize)
    double eq_Cinit = -1;  // Cinit(1); < 0 until known
    // multigrid
    double *err[PT_MAXLEV] = {}, *S0[PT_MAXLEV] = {}, *S1[PT_MAXLEV] = {}, *S2[PT_MAXLEV] = {},
           *RHS[PT_MAXLEV] = {}, *res[PT_MAXLEV] = {}, *dtst[PT_MAXLEV] = {}, *ratio[PT_MAXLEV] = {},
           *vis[PT_MAXLEV] = {}, *visst[PT_MAXLEV] = {}, *vx[PT_MAXLEV] = {}, *vz[PT_MAXLEV] = {},
           *vxx[PT_MAXLEV] = {}, *vzz[PT_MAXLEV] = {}, *vxz[PT_MAXLEV] = {}, *vxxpzz[PT_MAXLEV] = {},
           *vxxmzz[PT_MAXLEV] = {}, *vsm[PT_MAXLEV] = {};
    double* visw[11] = {};  // work set for smoothing the finer level before restriction
    // mixed precision mirrors
    float *ferr[PT_MAXLEV] = {}, *fS0[PT_MAXLEV] = {}, *fS1[PT_MAXLEV] = {}, *fS2[PT_MAXLEV] = {},
          *fRHS[PT_MAXLEV] = {}, *fres[PT_MAXLEV] = {};
    float* fcoef[PT_MAXLEV][6] = {};  // vis, vx, vz, vxz, vxxmzz, dt_stream in FP32
    cudaGraphExec_t gM1 = nullptr, gM2 = nullptr;
    int64_t nM1 = 0, nM2 = 0;
    // GCR acceleration of the mixed solve (krylov > 0): search directions z_j (FP64, with their
    // ghost images) and v_j = -A z_j, the residual r - A P e_2 that the level-1 smoothing sees, a
    // zero right-hand side, per-row partial sums and the device scalars [|v_j|^2 (kGcrMax) | c_j
    // (kGcrMax) | alpha | sum |r| | last-CTA counter]; one pair of captured graphs per slot
    double *gz[kGcrMax] = {}, *gv[kGcrMax] = {};
    double *gr1 = nullptr, *gzero = nullptr, *gpart = nullptr, *gsc = nullptr;
    cudaGraphExec_t gG0[kGcrMax] = {}, gG1[kGcrMax] = {};
    int64_t nG0[kGcrMax] = {}, nG1[kGcrMax] = {};
    double* psi_keep = nullptr;
    // coarse band LU
    double *Mc = nullptr, *Bc = nullptr, *RowB = nullptr;
    double* Ginv = nullptr;  // explicit coarse inverse (row-major n x n), mixed precision
    bool res_int = false;     // stream operator with exact integer stencil sums (pt_exact.cuh)
    ResFxK resfx[PT_MAXLEV]{};  // per level (both precisions: the FP64 path's stages use them too)
    // mixed precision: the next time level's coarse factorisation, built on st2 while the
    // top-of-step solve runs with the previous one, then copied into Mc/RowB/ipiv/Ginv
    double *Mc2 = nullptr, *RowB2 = nullptr, *Ginv2 = nullptr;
    int *ipiv2 = nullptr, *derr2 = nullptr, *hflag2 = nullptr;
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_in = nullptr, ev_fact = nullptr;
    bool fact_pending = false;
    // mixed precision: levels 2..grids of the next time level (viscosity pipeline + coarse
    // factorisation) built by a host worker thread on st2 into vl2 while the top-of-step solve runs
    // with the previous ones; the first RK-stage solve joins it and copies them in
    VisLevels vl2{};
    double* visw2[11] = {};
    double *dscal2 = nullptr, *hscal2 = nullptr;
    std::thread coarse_job;
    bool job_active = false, coarse_fresh = false;
    std::atomic<bool> job_done{false};
    int job_rc = 0;
    std::string job_msg;
    int device = 0;
    // PT_GUESS_EXTRAPOLATE: the last converged psi (a) and the last one at an earlier solve time
    // (b), with their solve times; solve_tau is the time of the solve being set up
    double *psi_a = nullptr, *psi_b = nullptr;
    double tau_a = 0.0, tau_b = 0.0, solve_tau = 0.0;
    int hist_n = 0;
    void* unet = nullptr;        // pt_unet* of the learned guess (PT_GUESS_UNET)
    void* unet_core = nullptr;   // its network (pt::UNet*)
    float* pair_buf = nullptr;   // staging of pt_training_pair (5 planes of nz x nx)
    float* pair_ring = nullptr;  // captured pairs of converged solves (pt_pair_capture), 5 planes each
    int pair_cap = 0, pair_n = 0;
    int unet_used = 0;           // last solve started from the network's guess
    double unet_r_prev = 0.0, unet_r_net = 0.0;
    bool coarse_ready = false;  // coarse factorisation valid for coarse_time (mixed precision)
    bool levels_reused = false; // this solve reuses levels 2..grids (mixed precision)
    double coarse_time = -1.0;
    int* ipiv = nullptr;
    // reductions
    double* red = nullptr;       // partial sums scratch
    double* dscal = nullptr;     // device scalars
    double* hscal = nullptr;     // pinned host mirror
    int* derr = nullptr;         // device error word
    // tracers
    int64_t ntr = 0;
    double *rtr = nullptr, *str = nullptr, *Ttr = nullptr, *Ctr = nullptr, *rtr0 = nullptr,
           *str0 = nullptr, *Ttr0 = nullptr, *rtr1 = nullptr, *str1 = nullptr, *Ttr1 = nullptr,
           *rtr2 = nullptr, *str2 = nullptr, *Ttr2 = nullptr;
    int32_t *tcell = nullptr, *cstart = nullptr, *ccount = nullptr, *clist = nullptr;
    // mixed precision: tracer order (perm[p] = user index of the tracer at position p; perm2 the
    // re-sort's target), the projection's runs counter, and the re-sort state
    int32_t *perm = nullptr, *perm2 = nullptr;
    unsigned long long* proj_runs = nullptr;
    int32_t *rs_count = nullptr, *rs_start = nullptr, *rs_tot = nullptr;  // re-sort: per-key counts, starts
    bool perm_active = false, want_resort = false;
    int64_t resorts = 0;
    double last_runs = 0.0;  // average runs per thread of the last mixed projection
    double* cpart = nullptr;  // 27 partial sums per cell
    int32_t* scan_tmp = nullptr;
    // state
    double time = 0, dt = 0;
    int uploaded = 0;
    double mass = 0;
    int have_mass = 0;
    int n_eta = 0, n_temp = 0, cycles = 0, refinements = 0;
    double eig_fine = 0, resid_ratio = 0, res_ref[PT_MAXLEV] = {}, residual_mag1 = 0;
    double phase_ms[PT_NPHASE] = {};
    std::vector<double> res_hist;  // relative residual at each convergence test of the last solve
    // timed spans (phase slots, and kernel classes when profiling is on) whose events have been
    // recorded but not yet read: read at the library's existing synchronisation points
    // (harvest_spans), so that timing adds no host wait of its own
    struct Span {
        int slot, kid, n;  // slot >= 0: phase slot; else kernel class kid with n launches
        cudaEvent_t a, b;
    };
    std::vector<Span> spans;
    std::vector<cudaEvent_t> ev_pool;
    // events recorded inside the captured level-1 smoothing batch (graph nodes), read after the
    // graph's synchronisation when profiling is on: [0] FP64 batch, [1] FP32 batch
    cudaEvent_t gev[2][2] = {};
    int gev_n[2] = {0, 0};
    size_t bytes_allocated = 0;
    // measurement hooks (ptgpu_prof.h): kernel launch count and per-kernel event timing
    int64_t launches = 0;
    cudaGraphExec_t gA = nullptr, gB = nullptr;  // captured multigrid cycle (parts A and B)
    int64_t nA = 0, nB = 0;
    int prof = 0;
    cudaEvent_t rev0 = nullptr, rev1 = nullptr;  // pt_prof_region
    int64_t kcount[8] = {};
    double kms[8] = {};
};

extern Engine* g_eng;
extern std::atomic<int64_t> g_launches;
#define PT_COUNT() (++pt::g_launches)

// brackets a batch of n launches of kernel class `id` with events when profiling is on
struct KernelTimer {
    Engine& E;
    int id, n;
    cudaEvent_t a = nullptr;
    KernelTimer(Engine& e, int i, int count);
    ~KernelTimer();
};
// adds the completed spans to phase_ms / kms (call after a synchronisation of the stream)
void harvest_spans(Engine& E);
enum { KT_RKC_FP64_L1 = 0, KT_RKC_FP32_L1 = 1, KT_RK_STAGE = 2, KT_PROJECT = 3 };
// Event pair around the level-1 smoothing batch of a cycle; recorded into the CUDA graph when the
// batch is captured, read by harvest_graph_timer after the graph has run.
struct GraphTimer {
    Engine& E;
    int which, n;
    GraphTimer(Engine& e, int w, int count);
    ~GraphTimer();
};
void harvest_graph_timer(Engine& E, int which);
extern thread_local std::string g_err;

int fail(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);
#define CK(x)                                                \
    do {                                                     \
        int _rc = pt::cuda_check((x), #x);                   \
        if (_rc) return _rc;                                 \
    } while (0)
#define CKL(what)                                            \
    do {                                                     \
        int _rc = pt::cuda_check(cudaGetLastError(), what);  \
        if (_rc) return _rc;                                 \
    } while (0)

// host setup (pt_setup.cpp)
int setup_constants(Engine& E);

// constant upload (pt_fields.cu)
int upload_consts(const Engine& E);

// fine-grid field kernels (pt_fields.cu)
int enforce_bcs_T(Engine& E, double* f);             // enforceBCs, energy.f90:558-592
int enforce_bcs_C(Engine& E, double* f);             // enforceBCs_comp, composition.f90:1279-1292
int enforce_bcs_stream(Engine& E, int level, double* f);  // iterative_solver.f90:1616-1664
int smoother_time_T(Engine& E, const double* Tin);   // smoother.f90:638-672
int smoother_time_C(Engine& E);                      // smoother.f90:582-636
int load_conductivity(Engine& E);                    // energy.f90:59-86
int load_tracer_space(Engine& E);                    // energy.f90:154-179 (+extendT 595-630)
int noalloc_scratch_setup(unsigned char** base);  // static scratch of the current device (before any capture)
int project_noalloc(Engine& E, const double* T0f, int smooth);
int sort_tracers_by_node(Engine& E, const double* r, const double* s);
int exclusive_scan_i32(Engine& E, const int32_t* in, int32_t* out, int n);
int interp_T_at(Engine& E, const int32_t* ids, int64_t m);
int equalize_tracers(Engine& E, pt_equalize_info* info);  // pt_equalize.cu
int capture_pair(Engine& E);                               // pt_unet.cu: append the solve's pair
void equalize_free(Engine& E);
// learned initial psi (pt_unet.cu): after mg_setup_solve; fallback check after the first cycle
int unet_guess(Engine& E);
int unet_check_fallback(Engine& E, double ratio);
int coarse_scale_fit(Engine& E, double* alpha);   // pt_mg.cu
int unet_engine_release(Engine& E);
int unet_engine_load(Engine& E, const char* path);  // PT_GUESS_UNET weights
int tables_to_f32(Engine& E, int which, const double* f);  // FP32 copies for the mixed RK stage
// the mixed RK stage's FP32 table of f straight from exact integer stencil sums (no FP64 table)
bool use_tables_fx(const Engine& E);
int tables_fx(Engine& E, int which, const double* f);
int extend_T(Engine& E);              // Text from Tratio (extendT)
int tracer_space_fx(Engine& E);       // tsa from Text with exact integer stencil sums (mixed path)
int compute_derivatives(Engine& E, const double* f, int which);  // composition.f90:1457-1478
int compute_velocities(Engine& E);                   // momentum.f90:655-710
int stability_dt(Engine& E, double* dt);             // energy.f90:756-810
int stats(Engine& E, pt_stats_row* out);             // basics.f90:363-462
int copy_field(Engine& E, double* dst, const double* src);

// tracers (pt_tracers.cu)
// mixed precision tracer order: identity after an upload; re-sort by cell; exchange of one tracer
// array with a host-order staging buffer (to_user: staging = user order of internal)
int tracer_order_reset(Engine& E);
// sort keys of the re-sort: cells x 4x4 sub-cells
inline size_t resort_nkey(int nx, int nz) { return (size_t)(nx + 1) * (size_t)(nz + 1) * 16; }
int resort_tracers(Engine& E);
int tracer_user_order(Engine& E, double* internal, double* staging, bool to_user);
int project(Engine& E, const double* r, const double* s, const double* Tt, const double* T0f,
            int smooth);                              // composition.f90:923-1087
int rk_stage(Engine& E, int stage);                   // energy.f90:258-536 tracer loops
int rkc2_stage(Engine& E, int stage);                 // Chebyshev.f90:151-227 tracer loops
// discrete tracer types: int32 0/1 on the device <-> the type as 0.0 / 1.0 in a composition array
int types_to_c(Engine& E, const int32_t* dev_types, double* c);
int c_to_types(Engine& E, const double* c, int32_t* dev_types);

// output and restart files (pt_io.cu): joins a pending writer and frees its staging
void io_release(Engine& E);

// direct banded solve (pt_direct.cu)
int direct_alloc(Engine& E);
void direct_free(Engine& E);
int direct_solve(Engine& E, pt_solve_info* info);  // momentum.f90:258-317, 636-653

// multigrid (pt_mg.cu)
bool trace_on();  // PTGPU_TRACE set in the environment
int multigrid(Engine& E, pt_solve_info* info);        // iterative_solver.f90:124-341
int mg_alloc(Engine& E);

// mixed precision (pt_mixed.cu)
int multigrid_mixed(Engine& E, pt_solve_info* info);
int mixed_alloc(Engine& E);
int mg_setup_solve(Engine& E);
int coarse_apply(Engine& E, double* out64, float* out32, const double* rhs64, const float* rhs32);
int coarse_band_solve(Engine& E);
int residual_level1_nosum(Engine& E);  // res[1] = RHS - A err[1] (FP64)
int residual_level1(Engine& E);

// reductions (pt_fields.cu)
int reduce_sum_abs_interior(Engine& E, const double* f, int nx, int nz, int pitch, double* out);
int reduce_sum_abs_interior(Engine& E, const float* f, int nx, int nz, int pitch, double* out);
int reduce_max_smoothness(Engine& E, const double* f, double* out);

// device timing.  Phase slots (pt_phase_times): PH_RK tracer RK stages, PH_PROJECT projections,
// PH_SOLVE psi solves, PH_SETUP multigrid setup (viscosity pipeline, coarse matrix, LU, inverse),
// PH_CYCLE_L1 level-1 part of the cycles, PH_CYCLE_COARSE the coarser levels, PH_GRID grid work
// of a step (smoothers, conductivity, derivative tables, time step), PH_FACTOR the coarse matrix,
// its LU and explicit inverse (part of PH_SETUP).
struct PhaseTimer {
    Engine& E;
    int slot;
    cudaEvent_t a = nullptr;
    PhaseTimer(Engine& e, int s);
    ~PhaseTimer();
};

}  // namespace pt
