// pt_setup.cpp -- start-up constants of the engine (host side, run once in pt_init).
//
// Computes what the reference's start-up computes before the time loop (main.f90:168-198):
// finite-difference stencils (FD_coefficients, main.f90:499-642), Fourier-symbol maxima
// (derivative_eigenvalues, energy.f90:632-744), RKC1 coefficients (Chebyshev_prep_stream,
// Chebyshev.f90:82-110), the multigrid hierarchy and schedule (optimize_grid,
// iterative_solver.f90:1-61; multigrid_setup, multigrid_cycle.f90:1-99), per-level eigenvalue
// symbols (eigenvalue_prep, iterative_solver.f90:1232-1362), the coarse stencil matrices
// (stream_space_matrix_prep, 692-743) and the coarse band width (Compute_Matrix_coarse with
// analysis=1, 1723-1745).  Uniform grid only, so every metric term is 1 or 0.
#include <cmath>
#include <cstring>

#include "pt_internal.h"

namespace pt {

static const double kPi = 3.1415926535897932;  // basics.f90:32

// Fornberg weights for the node ordering 0, 1, -1, 2, -2, 3, -3 (main.f90:506-536).
static void fornberg(double w[6][7][7]) {
    const int M = 4, N = 6;
    double nodes[N + 1];
    nodes[0] = 0.0;
    for (int i = 1, k = 1; i <= N; i += 2, k++) {
        nodes[i] = (double)k;
        nodes[i + 1] = -(double)k;
    }
    // w[m+1][n][i]: m-th derivative weight of node i using the first n+1 nodes
    std::memset(w, 0, sizeof(double) * 6 * 7 * 7);
    w[1][0][0] = 1.0;
    double c1 = 1.0;
    for (int n = 1; n <= N; n++) {
        double c2 = 1.0;
        int mmax = n < M ? n : M;
        for (int i = 0; i < n; i++) {
            double c3 = nodes[n] - nodes[i];
            c2 = c2 * c3;
            if (n <= M) w[n + 1][n - 1][i] = 0.0;
            for (int m = 0; m <= mmax; m++)
                w[m + 1][n][i] = ((nodes[n] - 0.0) * w[m + 1][n - 1][i] - (double)m * w[m][n - 1][i]) / c3;
        }
        for (int m = 0; m <= mmax; m++)
            w[m + 1][n][n] = (c1 / c2) * ((double)m * w[m][n - 1][n - 1] - (nodes[n - 1] - 0.0) * w[m + 1][n - 1][n - 1]);
        c1 = c2;
    }
}

// Stencil with offsets -k..k taken from weights over nodes 0,1,-1,...: symmetric placement.
static void place(double out[7], double w[6][7][7], int m, int n) {
    for (int j = 0; j < 7; j++) out[j] = 0.0;
    out[3] = w[m + 1][n][0];
    for (int i = 1, k = 1; i <= n; i += 2, k++) {
        out[3 + k] = w[m + 1][n][i];
        out[3 - k] = w[m + 1][n][i + 1];
    }
}

static void fd_stencils(Consts& K) {
    static double w[6][7][7];
    fornberg(w);
    place(K.D1, w, 1, 4);
    place(K.D2, w, 2, 4);
    place(K.D3, w, 3, 6);
    place(K.D4, w, 4, 6);
    // D(1..4,-3:3) for interpolation and derivative tables (main.f90:552-571)
    for (int m = 0; m < 5; m++)
        for (int j = 0; j < 7; j++) K.Dm[m][j] = 0.0;
    place(K.Dm[1], w, 1, 4);
    place(K.Dm[2], w, 2, 4);
    place(K.Dm[3], w, 3, 6);
    place(K.Dm[4], w, 4, 6);
    for (int m = 1; m <= 3; m += 2) {
        K.Dm[m][3] = 0.0;
        for (int i = 1; i <= 3; i++) {
            K.Dm[m][3 + i] = -K.Dm[m][3 - i];
            K.Dm[m + 1][3 + i] = K.Dm[m + 1][3 - i];
        }
    }
    // exact (anti)symmetry of the derivative stencils (main.f90:588-595)
    K.D1[3] = 0.0;
    K.D3[3] = 0.0;
    for (int i = 1; i <= 3; i++) {
        K.D1[3 + i] = -K.D1[3 - i];
        K.D2[3 + i] = K.D2[3 - i];
        K.D3[3 + i] = -K.D3[3 - i];
        K.D4[3 + i] = K.D4[3 - i];
    }
    for (int i = -2; i <= 2; i++)
        for (int k = -2; k <= 2; k++) {
            K.Drs[i + 2][k + 2] = K.D1[3 + k] * K.D1[3 + i];
            K.Drss[i + 2][k + 2] = K.D2[3 + k] * K.D1[3 + i];
            K.Drrs[i + 2][k + 2] = K.D1[3 + k] * K.D2[3 + i];
            K.Drrss[i + 2][k + 2] = K.D2[3 + k] * K.D2[3 + i];
        }
    const double d1so[3] = {-0.5, 0.0, 0.5}, d2so[3] = {1.0, -2.0, 1.0};
    for (int j = 0; j < 3; j++) { K.D1so[j] = d1so[j]; K.D2so[j] = d2so[j]; }
    // Drs_so(i,k) (main.f90:615-617): [i+1][k+1]
    K.Drsso[0][2] = -0.25; K.Drsso[1][2] = 0.0; K.Drsso[2][2] = 0.25;
    K.Drsso[0][1] = 0.0;   K.Drsso[1][1] = 0.0; K.Drsso[2][1] = 0.0;
    K.Drsso[0][0] = 0.25;  K.Drsso[1][0] = 0.0; K.Drsso[2][0] = -0.25;
}

// Maxima of the stencils' Fourier symbols over 2049 wave numbers per direction.  The reference
// builds each test wave with the default-kind CMPLX intrinsic (energy.f90:753), i.e. both
// factors and their product are single precision; the same rounding is applied here so the
// maxima (and every quantity derived from them) carry identical bits.
static void fourier_bases(Engine& E) {
    const Consts& K = E.K;
    const int na = 2049;
    const double da = 2.0 * kPi / (double)(na - 1);
    std::vector<float> wr((size_t)na * 7), wi((size_t)na * 7);
    for (int a = 0; a < na; a++) {
        double kk = (double)a * da;
        for (int j = -3; j <= 3; j++) {
            wr[a * 7 + j + 3] = (float)std::cos(kk * (double)j);
            wi[a * 7 + j + 3] = (float)std::sin(kk * (double)j);
        }
    }
    double m1 = 0, m2 = 0, m3 = 0, m4 = 0, mrs = 0, mrrs = 0, mrrss = 0, m1so = 0, m2so = 0;
#pragma omp parallel for reduction(max : m1, m2, m3, m4, mrs, mrrs, mrrss, m1so, m2so) schedule(dynamic, 8)
    for (int a = 0; a < na; a++) {
        const float* ar = &wr[a * 7 + 3];
        const float* ai = &wi[a * 7 + 3];
        double s1i = 0, s2r = 0, s3i = 0, s4r = 0, so1i = 0, so2r = 0;
        for (int j = -2; j <= 2; j++) { s1i += K.D1[3 + j] * (double)ai[j]; s2r += K.D2[3 + j] * (double)ar[j]; }
        for (int j = -1; j <= 1; j++) { so1i += K.D1so[j + 1] * (double)ai[j]; so2r += K.D2so[j + 1] * (double)ar[j]; }
        for (int j = -3; j <= 3; j++) { s3i += K.D3[3 + j] * (double)ai[j]; s4r += K.D4[3 + j] * (double)ar[j]; }
        m1 = std::fmax(m1, std::fabs(s1i));
        m2 = std::fmax(m2, std::fabs(s2r));
        m3 = std::fmax(m3, std::fabs(s3i));
        m4 = std::fmax(m4, std::fabs(s4r));
        m1so = std::fmax(m1so, std::fabs(so1i));
        m2so = std::fmax(m2so, std::fabs(so2r));
        for (int b = 0; b < na; b++) {
            const float* br = &wr[b * 7 + 3];
            const float* bi = &wi[b * 7 + 3];
            double rs_r = 0, rrs_i = 0, rrss_r = 0;
            for (int j = -2; j <= 2; j++)
                for (int jj = -2; jj <= 2; jj++) {
                    volatile float pr1 = ar[j] * br[jj], pr2 = ai[j] * bi[jj];
                    volatile float pi1 = ar[j] * bi[jj], pi2 = ai[j] * br[jj];
                    float tr = pr1 - pr2, ti = pi1 + pi2;
                    rs_r += K.Drs[j + 2][jj + 2] * (double)tr;
                    rrs_i += K.Drrs[j + 2][jj + 2] * (double)ti;
                    rrss_r += K.Drrss[j + 2][jj + 2] * (double)tr;
                }
            mrs = std::fmax(mrs, std::fabs(rs_r));
            mrrs = std::fmax(mrrs, std::fabs(rrs_i));
            mrrss = std::fmax(mrrss, std::fabs(rrss_r));
        }
    }
    E.Tr_base = m1; E.Trr_base = m2; E.Trrr_base = m3; E.Trrrr_base = m4;
    E.Trs_base = mrs; E.Trrs_base = mrrs; E.Trrss_base = mrrss;
    E.Tr_base_so = m1so; E.Trr_base_so = m2so;
}

// RKC1 coefficients of an N-stage smoother with the configured damping (Chebyshev_prep_stream);
// returns the stability bound
static double rkc1_table(const Engine& E, int N, double* mew, double* vv, double* cc, double* mewt) {
    double T[64], Tx[64], b[64];
    const double w0 = 1.0 + E.cfg.dampingS / (double)(N * N);
    T[0] = 1.0; T[1] = w0; Tx[0] = 0.0; Tx[1] = 1.0;
    for (int j = 2; j <= N; j++) {
        T[j] = 2.0 * w0 * T[j - 1] - T[j - 2];
        Tx[j] = 2.0 * T[j - 1] + 2.0 * w0 * Tx[j - 1] - Tx[j - 2];
    }
    const double w1 = T[N] / Tx[N];
    for (int j = 0; j <= N; j++) b[j] = 1.0 / T[j];
    mewt[1] = b[1] * w1;
    for (int j = 2; j <= N; j++) {
        mew[j] = 2.0 * b[j] * w0 / b[j - 1];
        vv[j] = -b[j] / b[j - 2];
        if (cc) cc[j] = 1.0 - mew[j] - vv[j];
        mewt[j] = 2.0 * b[j] * w1 / b[j - 1];
    }
    return -2.0 * w0 / w1;
}

static void rkc1_coefficients_c(Engine& E) {
    const int N = E.cfg.nstageC > 0 ? E.cfg.nstageC : E.cfg.nstageS;
    E.nstageC = N;
    E.RKC1_stability_c = rkc1_table(E, N, E.mew_c, E.vv_c, nullptr, E.mewt_c);
}

static void rkc1_coefficients(Engine& E) {
    rkc1_coefficients_c(E);
    Consts& K = E.K;
    const int N = E.cfg.nstageS;
    double T[64], Tx[64], b[64];
    const double w0 = 1.0 + E.cfg.dampingS / (double)(N * N);
    T[0] = 1.0; T[1] = w0; Tx[0] = 0.0; Tx[1] = 1.0;
    for (int j = 2; j <= N; j++) {
        T[j] = 2.0 * w0 * T[j - 1] - T[j - 2];
        Tx[j] = 2.0 * T[j - 1] + 2.0 * w0 * Tx[j - 1] - Tx[j - 2];
    }
    const double w1 = T[N] / Tx[N];
    for (int j = 0; j <= N; j++) b[j] = 1.0 / T[j];
    K.mewt[1] = b[1] * w1;
    for (int j = 2; j <= N; j++) {
        K.mew[j] = 2.0 * b[j] * w0 / b[j - 1];
        K.vv[j] = -b[j] / b[j - 2];
        K.cc[j] = 1.0 - K.mew[j] - K.vv[j];
        K.mewt[j] = 2.0 * b[j] * w1 / b[j - 1];
    }
    E.RKC1_stability = -2.0 * w0 / w1;
}

// RKC2 coefficients of the nstage-stage Chebyshev energy stepper (Chebyshev_prep,
// Chebyshev.f90:38-80, with the recursions of Chebyshev_coefficients, 1-18); TCheb_x(j)**2 as a
// product
static void rkc2_coefficients(Engine& E) {
    const int N = E.cfg.nstage;
    double T[64], Tx[64], Txx[64], b[64], a[64];
    const double w0 = 1.0 + E.cfg.damping / (double)(N * N);
    T[0] = 1.0; T[1] = w0; Tx[0] = 0.0; Tx[1] = 1.0; Txx[0] = 0.0; Txx[1] = 0.0;
    for (int j = 2; j <= N; j++) {
        T[j] = 2.0 * w0 * T[j - 1] - T[j - 2];
        Tx[j] = 2.0 * T[j - 1] + 2.0 * w0 * Tx[j - 1] - Tx[j - 2];
        Txx[j] = 4.0 * Tx[j - 1] + 2.0 * w0 * Txx[j - 1] - Txx[j - 2];
    }
    const double w1 = Tx[N] / Txx[N];
    for (int j = 2; j <= N; j++) b[j] = Txx[j] / (Tx[j] * Tx[j]);
    b[0] = -b[2];
    b[1] = E.cfg.aRK2 / w1;
    a[0] = 1.0 - b[0];
    a[1] = 1.0 - b[1] * w0;
    for (int j = 2; j <= N; j++) a[j] = 1.0 - b[j] * T[j];
    E.mewtCheb[1] = b[1] * w1;
    for (int j = 2; j <= N; j++) {
        E.mewCheb[j] = 2.0 * b[j] * w0 / b[j - 1];
        E.vCheb[j] = -b[j] / b[j - 2];
        E.cCheb[j] = 1.0 - E.mewCheb[j] - E.vCheb[j];
    }
    for (int j = 2; j <= N; j++) {
        E.mewtCheb[j] = 2.0 * b[j] * w1 / b[j - 1];
        E.gtCheb[j] = -a[j - 1] * E.mewtCheb[j];
    }
}

static int choose_levels(Engine& E) {
    int nx = E.cfg.nx, nz = E.cfg.nz, grids = E.cfg.grids;
    const int small = nx < nz ? nx : nz;
    const int cmax = grids - 1;
    int best_n = small * (1 << cmax), best_c = 0;
    int n_in = (nz <= nx) ? nz : nx;
    for (int np = E.cfg.mingrid; np <= small; np++)
        for (int c = 1; c <= cmax; c++) {
            int n = np * (1 << c);
            if (n >= n_in && n < best_n) { best_n = n; best_c = c; }
        }
    int nx2 = nx, nz2 = nz;
    if (nz <= nx) nz2 = best_n; else nx2 = best_n;
    int big = (nz <= nx) ? nx : nz;
    int m = (int)std::lround((double)big / (double)(1 << best_c)) * (1 << best_c);
    if (nz <= nx) nx2 = m; else nz2 = m;
    if (nx2 != nx || nz2 != nz)
        return fail(PT_ERR_CONFIG, "grid is not multigrid-compatible: optimize_grid would change nx,nz to " +
                                       std::to_string(nx2) + "," + std::to_string(nz2));
    E.grids = best_c + 1;
    static const int c2[] = {1, 2};
    static const int c3[] = {1, 2, 3, 2, 3, 2};
    static const int c4[] = {1, 2, 3, 4, 3, 4, 3, 2, 3, 4, 3, 4, 3, 2};
    static const int c5[] = {1, 2, 3, 4, 5, 4, 5, 4, 3, 4, 5, 4, 3, 2, 3, 4, 5, 4, 3, 4, 5, 4, 5, 4, 3, 2};
    static const int c6[] = {1, 2, 3, 4, 5, 6, 5, 6, 5, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 3,
                             2, 3, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 5, 6, 5, 6, 5, 4, 3, 2};
    const int* sched[] = {nullptr, nullptr, c2, c3, c4, c5, c6};
    const int len[] = {0, 0, 2, 6, 14, 26, 42};
    if (E.grids < 2 || E.grids > 6) return fail(PT_ERR_CONFIG, "multigrid needs 2..6 levels");
    E.nsteps = len[E.grids];
    for (int p = 1; p <= E.nsteps; p++) E.multi[p] = sched[E.grids][p - 1];
    E.multi[0] = E.multi[E.nsteps];
    E.multi[E.nsteps + 1] = E.multi[1];
    // schedule of the mixed-precision solve: the reference's table or a V-cycle 1..g..2
    if (E.cfg.mg_cycle != PT_CYCLE_REFERENCE && E.cfg.mg_cycle != PT_CYCLE_V)
        return fail(PT_ERR_CONFIG, "mg_cycle must be PT_CYCLE_REFERENCE or PT_CYCLE_V");
    if (E.cfg.mg_cycle == PT_CYCLE_V) {
        int p = 0;
        for (int l = 1; l <= E.grids; l++) E.mmulti[++p] = l;
        for (int l = E.grids - 1; l >= 2; l--) E.mmulti[++p] = l;
        E.mnsteps = p;
    } else {
        E.mnsteps = E.nsteps;
        for (int p = 1; p <= E.nsteps; p++) E.mmulti[p] = E.multi[p];
    }
    E.mmulti[0] = E.mmulti[E.mnsteps];
    E.mmulti[E.mnsteps + 1] = E.mmulti[1];
    return 0;
}

int setup_constants(Engine& E) {
    const pt_config& c = E.cfg;
    Consts& K = E.K;
    std::memset(&K, 0, sizeof K);
    if (c.order != 4) return fail(PT_ERR_CONFIG, "order must be 4");
    if (c.iheattype != 0) return fail(PT_ERR_CONFIG, "iheattype must be 0 (constant heating)");
    if (c.nx < 8 || c.nz < 8) return fail(PT_ERR_CONFIG, "grid too small");
    if (c.nstageS < 2 || c.nstageS > 60) return fail(PT_ERR_CONFIG, "nstageS must be 2..60");
    if (c.nstageC != 0 && (c.nstageC < 2 || c.nstageC > 60)) return fail(PT_ERR_CONFIG, "nstageC must be 0 or 2..60");
    if (c.comp != 0 && c.comp != 1) return fail(PT_ERR_CONFIG, "comp must be 0 or 1");
    if (c.RaT == 0.0) return fail(PT_ERR_CONFIG, "RaT=0 (manual dt) is not supported");
    if (c.ntr <= 0) return fail(PT_ERR_CONFIG, "ntr must be positive");
    if (c.chebyshev != 0 && (c.chebyshev != 1 || c.precision != PT_PREC_FP64))
        return fail(PT_ERR_CONFIG, "chebyshev = 1 (RKC2 energy stepper) runs in PT_PREC_FP64");
    if (c.chebyshev && (c.nstage < 2 || c.nstage > 60)) return fail(PT_ERR_CONFIG, "nstage must be 2..60");
    if (c.chebyshev) rkc2_coefficients(E);
    int rc = choose_levels(E);
    if (rc) return rc;
    fd_stencils(K);
    rkc1_coefficients(E);
    fourier_bases(E);
    // smoothing thresholds, compute_smoothing_parameters (smoother.f90:31-73)
    E.delta_T = (c.ivis == 0 || c.RaT == 0.0) ? 2.0 : (c.visT != 1.0 ? std::log(c.delta_visT) / std::log(c.visT) : 2.0);
    E.delta_C = 2.0;
    if (c.comp == 1) {
        if (c.conduct_factor != 1.0) E.delta_C = std::fabs(std::log(c.delta_visC) / std::log(1.0 / c.conduct_factor));
        if (c.ivis >= 2 && c.visC != 1.0) E.delta_C = std::fabs(std::log(c.delta_visC) / std::log(c.visC));
    }
    if (c.comp == 1 && !(E.delta_C > 1.0))
        return fail(PT_ERR_CONFIG, "composition smoothing (delta_C<=1) is not supported");
    K.nx = c.nx; K.nz = c.nz; K.comp = c.comp; K.Tbot = c.Tbot; K.Vbc = c.Vbc; K.ivis = c.ivis;
    K.aspect = c.aspect;
    K.dr = c.aspect / (double)c.nx;
    K.ds = 1.0 / (double)c.nz;
    K.dr2 = K.dr * K.dr;
    K.ds2 = K.ds * K.ds;
    K.inv_dr = 1.0 / K.dr;
    K.inv_ds = 1.0 / K.ds;
    K.inv_dr2 = 1.0 / K.dr2;
    K.inv_ds2 = 1.0 / K.ds2;
    int ex;
    K.exact_div = (std::frexp(K.dr, &ex) == 0.5 && std::frexp(K.ds, &ex) == 0.5) ? 1 : 0;
    K.p_inv_dr = K.p_inv_ds = 0;
    if (K.exact_div) {
        std::frexp(K.inv_dr, &ex);
        K.p_inv_dr = ex - 1;
        std::frexp(K.inv_ds, &ex);
        K.p_inv_ds = ex - 1;
    }
    K.fact[0] = 1.0; K.dr_pow[0] = 1.0; K.ds_pow[0] = 1.0;
    for (int j = 1; j <= 3; j++) {
        K.fact[j] = (double)j * K.fact[j - 1];
        K.dr_pow[j] = std::pow(K.dr, (double)j);
        K.ds_pow[j] = std::pow(K.ds, (double)j);
    }
    for (int j = 0; j <= 3; j++) {
        K.inv_ds_pow[j] = 1.0 / K.ds_pow[j];
        K.inv_dr_pow[j] = 1.0 / K.dr_pow[j];
        K.inv_fact[j] = 1.0 / K.fact[j];
    }
    K.two_over_D20 = 2.0 / K.D2[3];
    K.Tbot_iso = c.Tbot_iso; K.Ttop_iso = c.Ttop_iso;
    K.H = c.H; K.Htype = c.Htype; K.conduct_factor = c.conduct_factor;
    K.RaT = c.RaT; K.RaC = c.RaC;
    K.lvisT = std::log(c.visT); K.lvisP = std::log(c.visP); K.lvisC = std::log(c.visC);
    // stability_RK4_smoother (smoother.f90:719-740): uniform grid, eI=0
    {
        double a = -E.Trr_base / K.dr2, b = -E.Trr_base / K.ds2;
        double eR = std::fabs(a / 1.0) + std::fabs(b / 1.0);
        E.dts = 2.0 * eR / (eR * eR + 0.0);
    }
    // multigrid levels
    for (int l = 1; l <= E.grids; l++) {
        LevConst& L = E.L[l];
        L.nx = c.nx >> (l - 1);
        L.nz = c.nz >> (l - 1);
        L.dr = c.aspect / (double)L.nx;
        L.ds = 1.0 / (double)L.nz;
        L.dr2 = L.dr * L.dr; L.ds2 = L.ds * L.ds;
        L.dr3 = std::pow(L.dr, 3.0); L.ds3 = std::pow(L.ds, 3.0);
        L.dr4 = std::pow(L.dr, 4.0); L.ds4 = std::pow(L.ds, 4.0);
        L.drds = L.dr * L.ds; L.drds2 = L.dr * L.ds2; L.dr2ds = L.dr2 * L.ds; L.dr2ds2 = L.dr2 * L.ds2;
        L.idr = 1.0 / L.dr; L.ids = 1.0 / L.ds;
        L.idr2 = 1.0 / L.dr2; L.ids2 = 1.0 / L.ds2; L.idr3 = 1.0 / L.dr3; L.ids3 = 1.0 / L.ds3;
        L.idr4 = 1.0 / L.dr4; L.ids4 = 1.0 / L.ds4; L.idrds = 1.0 / L.drds; L.idrds2 = 1.0 / L.drds2;
        L.idr2ds = 1.0 / L.dr2ds; L.idr2ds2 = 1.0 / L.dr2ds2;
        // symbols of the stream operator (real parts: even derivative counts, imaginary: odd)
        double Tss = -E.Trr_base / L.ds2, Tssss = E.Trrrr_base / L.ds4, Tsss = E.Trrr_base / L.ds3;
        double Trr = -E.Trr_base / L.dr2, Trrrr = E.Trrrr_base / L.dr4, Trrr = E.Trrr_base / L.dr3;
        double Trs = -E.Trs_base / L.drds, Trrss = E.Trrss_base / L.dr2ds2;
        double Trss = E.Trrs_base / L.drds2, Trrs = E.Trrs_base / L.dr2ds;
        L.SR1 = -(Trr - Tss);
        L.SR2 = -((Trrrr + Tssss) + 2.0 * Trrss);
        L.SR4 = -4.0 * Trs;
        L.SR5 = -2.0 * (0.0 + 0.0);
        L.SR6 = -2.0 * (0.0 + 0.0);
        L.SI1 = 0.0 + 0.0;
        L.SI2 = std::fabs(0.0 + 0.0) + std::fabs(2.0 * 0.0);
        L.SI4 = 4.0 * 0.0;
        L.SI5 = 2.0 * (Trrr + Trss);
        L.SI6 = 2.0 * (Tsss + Trrs);
        double a = -E.Trr_base_so / L.ds2, b = -E.Trr_base_so / L.dr2;
        double eR = std::fabs(b / 1.0) + std::fabs(a / 1.0);
        L.dt_vis = 2.0 * eR / (eR * eR + 0.0);
    }
    // coarse-level stencil matrices
    {
        const LevConst& L = E.L[E.grids];
        for (int dk = -3; dk <= 3; dk++)
            for (int di = -3; di <= 3; di++) {
                double Sxx = 0, Sxxx = 0, Sxxxx = 0, Szz = 0, Szzz = 0, Szzzz = 0;
                if (dk == 0) { Sxx = K.D2[3 + di] / L.dr2; Sxxx = K.D3[3 + di] / L.dr3; Sxxxx = K.D4[3 + di] / L.dr4; }
                if (di == 0) { Szz = K.D2[3 + dk] / L.ds2; Szzz = K.D3[3 + dk] / L.ds3; Szzzz = K.D4[3 + dk] / L.ds4; }
                double rs = 0, rss = 0, rrs = 0, rrss = 0;
                if (di >= -2 && di <= 2 && dk >= -2 && dk <= 2) {
                    rs = K.Drs[di + 2][dk + 2]; rss = K.Drss[di + 2][dk + 2];
                    rrs = K.Drrs[di + 2][dk + 2]; rrss = K.Drrss[di + 2][dk + 2];
                }
                double Sxz = rs / L.drds, Sxzz = rss / L.drds2, Sxxz = rrs / L.dr2ds, Sxxzz = rrss / L.dr2ds2;
                K.SM1[di + 3][dk + 3] = Sxx - Szz;
                K.SM2[di + 3][dk + 3] = Sxxxx + Szzzz + 2.0 * Sxxzz;
                K.SM4[di + 3][dk + 3] = 4.0 * Sxz;
                K.SM5[di + 3][dk + 3] = 2.0 * (Sxxx + Sxzz);
                K.SM6[di + 3][dk + 3] = 2.0 * (Szzz + Sxxz);
            }
    }
    // coarse band width for the node ordering p = (nz_c+1)*i + k + 1 (Database=2)
    {
        const int nxc = E.L[E.grids].nx, nzc = E.L[E.grids].nz, N = nzc + 1;
        const int reach[7] = {0, 2, 2, 3, 2, 2, 0};
        int kl = 0, ku = 0;
        E.ngc = (nxc + 1) * (nzc + 1);
        for (int p = 1; p <= E.ngc; p++) {
            int ip = (p - 1) / N, kp = (p - 1) % N;
            for (int j = -3; j <= 3; j++) {
                int iq = ip + j;
                if (iq <= 0 || iq >= nxc) continue;
                for (int kq = kp - reach[j + 3]; kq <= kp + reach[j + 3]; kq++) {
                    if (kq <= 0 || kq >= nzc) continue;
                    int d = N * iq + kq + 1 - p;
                    if (d > ku) ku = d;
                    if (-d > kl) kl = -d;
                }
            }
        }
        E.kl = kl;
        E.ku = ku;
    }
    // entrainment reference row (composition.f90:765-774)
    E.kent = 0;
    for (int k = 0; k <= c.nz; k++)
        if (K.ds * (double)k <= c.dent) E.kent = k;
    return 0;
}

}  // namespace pt
