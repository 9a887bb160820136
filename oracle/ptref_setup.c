/*
 * ptref_setup.c -- oracle (test infrastructure only): start-up of the reference run.
 * Follows main.f90:168-230 and the routines it calls; see ptref.h for the conventions.
 */
#include "ptref.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>


static const double pii = 3.1415926535897932; /* basics.f90:32 */

int ref_fail(ptref_state* s, int code, const char* msg) {
    s->status = code;
    snprintf(s->err_msg, sizeof s->err_msg, "%s", msg);
    return code;
}

const char* ptref_error(ptref_state* s) { return s->err_msg; }

rfld ref_fld_alloc(int nx, int nz, int g) {
    rfld f;
    f.nx = nx;
    f.nz = nz;
    f.g = g;
    f.ld = nx + 2 * g + 1;
    f.p = (double*)calloc((size_t)f.ld * (size_t)(nz + 2 * g + 1), sizeof(double));
    return f;
}

/* FD_coefficients, main.f90:499-642: Fornberg's recursion on the node set 0,1,-1,2,-2,3,-3. */
static void fd_coefficients(ptref_state* s) {
    enum { bigM = 4, bigN = 6 };
    double a[bigN + 1];
    static double delta[bigM + 2][bigN + 1][bigN + 1]; /* m index shifted by +1 */
#define DL(m, n, i) delta[(m) + 1][n][i]
    memset(delta, 0, sizeof delta);
    double x0 = 0.0;
    a[0] = 0.0;
    int k = 1;
    for (int i = 1; i <= bigN; i += 2) {
        a[i] = (double)k;
        a[i + 1] = -(double)k;
        k++;
    }
    DL(0, 0, 0) = 1.0;
    double c1 = 1.0;
    for (int n = 1; n <= bigN; n++) {
        double c2 = 1.0;
        for (int i = 0; i <= n - 1; i++) {
            double c3 = a[n] - a[i];
            c2 = c2 * c3;
            if (n <= bigM) DL(n, n - 1, i) = 0.0;
            int mm = n < bigM ? n : bigM;
            for (int m = 0; m <= mm; m++)
                DL(m, n, i) = ((a[n] - x0) * DL(m, n - 1, i) - (double)m * DL(m - 1, n - 1, i)) / c3;
        }
        int mm = n < bigM ? n : bigM;
        for (int m = 0; m <= mm; m++)
            DL(m, n, n) = (c1 / c2) * ((double)m * DL(m - 1, n - 1, n - 1) - (a[n - 1] - x0) * DL(m, n - 1, n - 1));
        c1 = c2;
    }
    const int order = 4;
    double *D1 = s->D1 + 3, *D2 = s->D2 + 3, *D3 = s->D3 + 3, *D4 = s->D4 + 3;
    for (int i = -3; i <= 3; i++) D1[i] = D2[i] = D3[i] = D4[i] = 0.0;
    D1[0] = DL(1, order, 0);
    D2[0] = DL(2, order, 0);
    k = 1;
    for (int i = 1; i <= order; i += 2) {
        D1[k] = DL(1, order, i);
        D1[-k] = DL(1, order, i + 1);
        D2[k] = DL(2, order, i);
        D2[-k] = DL(2, order, i + 1);
        k++;
    }
    /* D(1:Dnumber,-span_interp:span_interp), Dnumber=4 */
    for (int m = 0; m <= 4; m++)
        for (int i = 0; i < 7; i++) s->Dm[m][i] = 0.0;
    for (int m = 2; m <= 4; m += 2) {
        double* Dm1 = s->Dm[m - 1] + 3;
        double* Dmm = s->Dm[m] + 3;
        Dm1[0] = DL(m - 1, order + m - 2, 0);
        Dmm[0] = DL(m, order + m - 2, 0);
        k = 1;
        for (int i = 1; i <= order + m - 2; i += 2) {
            Dm1[k] = DL(m - 1, order + m - 2, i);
            Dm1[-k] = DL(m - 1, order + m - 2, i + 1);
            Dmm[k] = DL(m, order + m - 2, i);
            Dmm[-k] = DL(m, order + m - 2, i + 1);
            k++;
        }
    }
    for (int m = 1; m <= 4; m += 2) {
        double* Dm1 = s->Dm[m] + 3;
        double* Dmm = s->Dm[m + 1] + 3;
        Dm1[0] = 0.0;
        for (int i = 1; i <= 3; i++) {
            Dm1[i] = -Dm1[-i];
            Dmm[i] = Dmm[-i];
        }
    }
    D3[0] = DL(3, order + 2, 0);
    D4[0] = DL(4, order + 2, 0);
    k = 1;
    for (int i = 1; i <= order + 2; i += 2) {
        D3[k] = DL(3, order + 2, i);
        D3[-k] = DL(3, order + 2, i + 1);
        D4[k] = DL(4, order + 2, i);
        D4[-k] = DL(4, order + 2, i + 1);
        k++;
    }
    D1[0] = 0.0;
    D3[0] = 0.0;
    for (int i = 1; i <= 3; i++) {
        D1[i] = -D1[-i];
        D2[i] = D2[-i];
        D3[i] = -D3[-i];
        D4[i] = D4[-i];
    }
    for (int i = 0; i < 7; i++)
        for (int kk = 0; kk < 7; kk++) s->Drs[i][kk] = s->Drss[i][kk] = s->Drrs[i][kk] = s->Drrss[i][kk] = 0.0;
    for (int kk = -2; kk <= 2; kk++)
        for (int i = -2; i <= 2; i++) {
            s->Drs[i + 3][kk + 3] = D1[kk] * D1[i];
            s->Drss[i + 3][kk + 3] = D2[kk] * D1[i];
            s->Drrs[i + 3][kk + 3] = D1[kk] * D2[i];
            s->Drrss[i + 3][kk + 3] = D2[kk] * D2[i];
        }
    s->D1_so[0] = -0.5; s->D1_so[1] = 0.0; s->D1_so[2] = 0.5;
    s->D2_so[0] = 1.0; s->D2_so[1] = -2.0; s->D2_so[2] = 1.0;
    /* Drs_so(:,1)=(/-0.25,0,0.25/), Drs_so(:,0)=0, Drs_so(:,-1)=(/0.25,0,-0.25/) */
    s->Drs_so[0][2] = -0.25; s->Drs_so[1][2] = 0.0; s->Drs_so[2][2] = 0.25;
    s->Drs_so[0][1] = 0.0;   s->Drs_so[1][1] = 0.0; s->Drs_so[2][1] = 0.0;
    s->Drs_so[0][0] = 0.25;  s->Drs_so[1][0] = 0.0; s->Drs_so[2][0] = -0.25;
#undef DL
}

/* derivative_eigenvalues, energy.f90:632-744.  T_test (energy.f90:746-754) builds its waves
 * with the default-kind CMPLX intrinsic, so each factor is rounded to single precision and the
 * product is a single-precision complex multiply; this restatement keeps that rounding. */
typedef struct { float re, im; } cf32;
static cf32 cmul_f(cf32 a, cf32 b) {
    volatile float ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
    cf32 r;
    r.re = ac - bd;
    r.im = ad + bc;
    return r;
}

static void derivative_eigenvalues(ptref_state* s) {
    const int n_angle = 2048 + 1;
    const double d_angle = 2.0 * pii / (double)(n_angle - 1);
    cf32* wave = (cf32*)malloc(sizeof(cf32) * (size_t)n_angle * 7);
    for (int a = 0; a < n_angle; a++) {
        double kk = (double)a * d_angle;
        for (int j = -3; j <= 3; j++) {
            double r = (double)j;
            wave[a * 7 + j + 3].re = (float)cos(kk * r);
            wave[a * 7 + j + 3].im = (float)sin(kk * r);
        }
    }
    const double *D1 = s->D1 + 3, *D2 = s->D2 + 3, *D3 = s->D3 + 3, *D4 = s->D4 + 3;
    const double *D1so = s->D1_so + 1, *D2so = s->D2_so + 1;
    double Tr_max = 0, Trr_max = 0, Trrr_max = 0, Trrrr_max = 0, Trs_max = 0, Trrs_max = 0,
           Trrss_max = 0, Tr_max_so = 0, Trr_max_so = 0;
    cf32 one = {1.0f, 0.0f};
#pragma omp parallel for reduction(max : Tr_max, Trr_max, Trrr_max, Trrrr_max, Trs_max, Trrs_max, Trrss_max, Tr_max_so, Trr_max_so) schedule(dynamic, 16)
    for (int a = 0; a < n_angle; a++) {
        const cf32* wr = wave + a * 7 + 3;
        double Tr_re = 0, Tr_im = 0, Trr_re = 0, Trr_im = 0, T3_re = 0, T3_im = 0, T4_re = 0, T4_im = 0;
        double so1_re = 0, so1_im = 0, so2_re = 0, so2_im = 0;
        cf32 w0 = wave[0 * 7 + 3]; /* ks = 0 -> exp(i*0*s) = (1,0) for every s */
        (void)w0;
        for (int j = -2; j <= 2; j++) {
            cf32 t = cmul_f(wr[j], one);
            Tr_re += D1[j] * t.re; Tr_im += D1[j] * t.im;
            Trr_re += D2[j] * t.re; Trr_im += D2[j] * t.im;
        }
        for (int j = -1; j <= 1; j++) {
            cf32 t = cmul_f(wr[j], one);
            so1_re += D1so[j] * t.re; so1_im += D1so[j] * t.im;
            so2_re += D2so[j] * t.re; so2_im += D2so[j] * t.im;
        }
        for (int j = -3; j <= 3; j++) {
            cf32 t = cmul_f(wr[j], one);
            T3_re += D3[j] * t.re; T3_im += D3[j] * t.im;
            T4_re += D4[j] * t.re; T4_im += D4[j] * t.im;
        }
        /* division by T_test(0,0)=(1,0) leaves the sums unchanged */
        if (fabs(Tr_im) > Tr_max) Tr_max = fabs(Tr_im);
        if (fabs(Trr_re) > Trr_max) Trr_max = fabs(Trr_re);
        if (fabs(T3_im) > Trrr_max) Trrr_max = fabs(T3_im);
        if (fabs(T4_re) > Trrrr_max) Trrrr_max = fabs(T4_re);
        if (fabs(so1_im) > Tr_max_so) Tr_max_so = fabs(so1_im);
        if (fabs(so2_re) > Trr_max_so) Trr_max_so = fabs(so2_re);
        for (int a2 = 0; a2 < n_angle; a2++) {
            const cf32* ws = wave + a2 * 7 + 3;
            double rs_re = 0, rs_im = 0, rrs_re = 0, rrs_im = 0, rrss_re = 0, rrss_im = 0;
            for (int j = -2; j <= 2; j++)
                for (int jj = -2; jj <= 2; jj++) {
                    cf32 t = cmul_f(wr[j], ws[jj]);
                    double drs = s->Drs[j + 3][jj + 3], drrs = s->Drrs[j + 3][jj + 3], drrss = s->Drrss[j + 3][jj + 3];
                    rs_re += drs * t.re; rs_im += drs * t.im;
                    rrs_re += drrs * t.re; rrs_im += drrs * t.im;
                    rrss_re += drrss * t.re; rrss_im += drrss * t.im;
                }
            (void)rs_im; (void)rrs_re; (void)rrss_im;
            if (fabs(rs_re) > Trs_max) Trs_max = fabs(rs_re);
            if (fabs(rrs_im) > Trrs_max) Trrs_max = fabs(rrs_im);
            if (fabs(rrss_re) > Trrss_max) Trrss_max = fabs(rrss_re);
        }
    }
    free(wave);
    s->Tr_base = Tr_max; s->Trr_base = Trr_max; s->Trrr_base = Trrr_max; s->Trrrr_base = Trrrr_max;
    s->Trs_base = Trs_max; s->Trrs_base = Trrs_max; s->Trss_base = 0.0; s->Trrss_base = Trrss_max;
    s->Tr_base_so = Tr_max_so; s->Trr_base_so = Trr_max_so;
}

/* Chebyshev_prep_stream, Chebyshev.f90:182-210 (with Chebyshev_coefficients_stream 120-134). */
/* Chebyshev_prep (Chebyshev.f90:38-80) with Chebyshev_coefficients (1-18): the RKC2 coefficients
 * of the nstage-stage energy stepper; TCheb_x(j)**2 as TCheb_x(j)*TCheb_x(j) */
static void chebyshev_prep(ptref_state* s) {
    int N = s->cfg.nstage;
    double T[64], Tx[64], Txx[64], b[64], a[64];
    double w0 = 1.0 + s->cfg.damping / (double)(N * N);
    T[0] = 1.0; T[1] = w0; Tx[0] = 0.0; Tx[1] = 1.0; Txx[0] = 0.0; Txx[1] = 0.0;
    for (int j = 2; j <= N; j++) {
        T[j] = 2.0 * w0 * T[j - 1] - T[j - 2];
        Tx[j] = 2.0 * T[j - 1] + 2.0 * w0 * Tx[j - 1] - Tx[j - 2];
        Txx[j] = 4.0 * Tx[j - 1] + 2.0 * w0 * Txx[j - 1] - Txx[j - 2];
    }
    double w1 = Tx[N] / Txx[N];
    for (int j = 2; j <= N; j++) b[j] = Txx[j] / (Tx[j] * Tx[j]);
    b[0] = -b[2];
    b[1] = s->cfg.aRK2 / w1;
    a[0] = 1.0 - b[0];
    a[1] = 1.0 - b[1] * w0;
    for (int j = 2; j <= N; j++) a[j] = 1.0 - b[j] * T[j];
    s->mewtCheb[1] = b[1] * w1;
    for (int j = 2; j <= N; j++) {
        s->mewCheb[j] = 2.0 * b[j] * w0 / b[j - 1];
        s->vCheb[j] = -b[j] / b[j - 2];
        s->cCheb[j] = 1.0 - s->mewCheb[j] - s->vCheb[j];
    }
    for (int j = 2; j <= N; j++) {
        s->mewtCheb[j] = 2.0 * b[j] * w1 / b[j - 1];
        s->gtCheb[j] = -a[j - 1] * s->mewtCheb[j];
    }
}

static void chebyshev_prep_stream(ptref_state* s) {
    int N = s->cfg.nstageS;
    double T[64], Tx[64];
    double w0 = 1.0 + s->cfg.dampingS / (double)(N * N);
    T[0] = 1.0; T[1] = w0; Tx[0] = 0.0; Tx[1] = 1.0;
    for (int j = 2; j <= N; j++) {
        T[j] = 2.0 * w0 * T[j - 1] - T[j - 2];
        Tx[j] = 2.0 * T[j - 1] + 2.0 * w0 * Tx[j - 1] - Tx[j - 2];
    }
    double w1 = T[N] / Tx[N];
    for (int j = 0; j <= N; j++) s->bS[j] = 1.0 / T[j];
    s->mewtS[1] = s->bS[1] * w1;
    for (int j = 2; j <= N; j++) {
        s->mewS[j] = 2.0 * s->bS[j] * w0 / s->bS[j - 1];
        s->vS[j] = -s->bS[j] / s->bS[j - 2];
        s->cS[j] = 1.0 - s->mewS[j] - s->vS[j];
    }
    for (int j = 2; j <= N; j++) s->mewtS[j] = 2.0 * s->bS[j] * w1 / s->bS[j - 1];
    s->RKC1_stability = -2.0 * w0 / w1;
}

/* optimize_grid, iterative_solver.f90:1-61 (returns the possibly adjusted nx, nz, grids). */
static void optimize_grid(int* nx, int* nz, int* grids, int n_points_min) {
    int n_points_max = *nx < *nz ? *nx : *nz;
    int n_coarse_min = 1, n_coarse_max = *grids - 1;
    int n_max = n_points_max * (1 << n_coarse_max);
    int nxbig, n_in;
    if (*nz <= *nx) { nxbig = 1; n_in = *nz; } else { nxbig = 0; n_in = *nx; }
    int n_temp = n_max, n_coarse_temp = 0, n_points_temp = 0;
    for (int np = n_points_min; np <= n_points_max; np++)
        for (int nc = n_coarse_min; nc <= n_coarse_max; nc++) {
            int n = np * (1 << nc);
            if (n >= n_in && n < n_temp) { n_temp = n; n_coarse_temp = nc; n_points_temp = np; }
        }
    *grids = n_coarse_temp + 1;
    if (nxbig == 0) *nx = n_temp; else *nz = n_temp;
    n_in = (*nz <= *nx) ? *nx : *nz;
    n_points_temp = (int)lround((double)n_in / (double)(1 << n_coarse_temp));
    n_temp = n_points_temp * (1 << n_coarse_temp);
    if (nxbig == 0) *nz = n_temp; else *nx = n_temp;
}

/* multigrid_setup, multigrid_cycle.f90:1-99 (the schedules the reference selects). */
static int multigrid_setup(ptref_state* s) {
    static const int c2[] = {1, 2};
    static const int c3[] = {1, 2, 3, 2, 3, 2};
    static const int c4[] = {1, 2, 3, 4, 3, 4, 3, 2, 3, 4, 3, 4, 3, 2};
    static const int c5[] = {1, 2, 3, 4, 5, 4, 5, 4, 3, 4, 5, 4, 3, 2, 3, 4, 5, 4, 3, 4, 5, 4, 5, 4, 3, 2};
    static const int c6[] = {1, 2, 3, 4, 5, 6, 5, 6, 5, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 3,
                             2, 3, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 5, 6, 5, 6, 5, 4, 3, 2};
    const int* c;
    int n;
    switch (s->grids) {
        case 2: c = c2; n = 2; break;
        case 3: c = c3; n = 6; break;
        case 4: c = c4; n = 14; break;
        case 5: c = c5; n = 26; break;
        case 6: c = c6; n = 42; break;
        default: return -1;
    }
    s->nsteps = n;
    for (int p = 1; p <= n; p++) s->multi[p] = c[p - 1];
    s->multi[0] = s->multi[n];
    s->multi[n + 1] = s->multi[1];
    return 0;
}

/* eigenvalue_prep, iterative_solver.f90:1232-1362, on the uniform grid (metrics xr=zs=1,
 * xrr=zss=xrrr=zsss=0) where the real and imaginary symbols are the same at every node. */
static void eigenvalue_prep(ptref_state* s) {
    for (int l = 1; l <= s->grids; l++) {
        double Ts = s->Tr_base / s->dsl[l];
        double Tss = -s->Trr_base / s->ds2l[l];
        double Tsss = s->Trrr_base / s->ds3l[l];
        double Tssss = s->Trrrr_base / s->ds4l[l];
        double Tr = s->Tr_base / s->drl[l];
        double Trr = -s->Trr_base / s->dr2l[l];
        double Trrr = s->Trrr_base / s->dr3l[l];
        double Trrrr = s->Trrrr_base / s->dr4l[l];
        double Trs = -s->Trs_base / s->drdsl[l];
        double Trrss = s->Trrss_base / s->dr2ds2l[l];
        double Trss = s->Trrs_base / s->drds2l[l];
        double Trrs = s->Trrs_base / s->dr2dsl[l];
        /* real parts */
        double Sxx = Trr, Szz = Tss, Sxxxx = Trrrr, Szzzz = Tssss, Sxz = Trs, Sxxzz = Trrss;
        double Sxxx = 0.0, Szzz = 0.0, Sxxz = 0.0, Sxzz = 0.0;
        s->SR[l][1] = -(Sxx - Szz);
        s->SR[l][2] = -((Sxxxx + Szzzz) + 2.0 * Sxxzz);
        s->SR[l][4] = -4.0 * Sxz;
        s->SR[l][5] = -2.0 * (Sxxx + Sxzz);
        s->SR[l][6] = -2.0 * (Szzz + Sxxz);
        /* imaginary parts */
        double iSxx = 0.0, iSzz = 0.0, iSxxxx = 0.0, iSzzzz = 0.0, iSxz = 0.0, iSxxzz = 0.0;
        double iSxxx = Trrr, iSzzz = Tsss, iSxxz = Trrs, iSxzz = Trss;
        (void)Tr; (void)Ts;
        s->SI[l][1] = iSxx + iSzz;
        s->SI[l][2] = fabs(iSxxxx + iSzzzz) + fabs(2.0 * iSxxzz);
        s->SI[l][4] = 4.0 * iSxz;
        s->SI[l][5] = 2.0 * (iSxxx + iSxzz);
        s->SI[l][6] = 2.0 * (iSzzz + iSxxz);
        /* stability_vis_smoother, smoother.f90:761-782 (uniform): eI=0 */
        double Tss_so = -s->Trr_base_so / s->ds2l[l];
        double Trr_so = -s->Trr_base_so / s->dr2l[l];
        double eR = fabs(Trr_so / 1.0) + fabs(Tss_so / 1.0);
        s->dt_vis[l] = 2.0 * eR / (eR * eR + 0.0);
    }
}

/* stream_space_matrix_prep, iterative_solver.f90:692-743 (coarsest-level spacings). */
static void stream_space_matrix_prep(ptref_state* s) {
    int g = s->grids;
    const double *D2 = s->D2 + 3, *D3 = s->D3 + 3, *D4 = s->D4 + 3;
    for (int dk = -3; dk <= 3; dk++)
        for (int di = -3; di <= 3; di++) {
            double Sxx, Sxxx, Sxxxx, Szz, Szzz, Szzzz;
            if (dk == 0) { Sxx = D2[di] / s->dr2l[g]; Sxxx = D3[di] / s->dr3l[g]; Sxxxx = D4[di] / s->dr4l[g]; }
            else { Sxx = 0.0; Sxxx = 0.0; Sxxxx = 0.0; }
            if (di == 0) { Szz = D2[dk] / s->ds2l[g]; Szzz = D3[dk] / s->ds3l[g]; Szzzz = D4[dk] / s->ds4l[g]; }
            else { Szz = 0.0; Szzz = 0.0; Szzzz = 0.0; }
            double Sxz = s->Drs[di + 3][dk + 3] / s->drdsl[g];
            double Sxzz = s->Drss[di + 3][dk + 3] / s->drds2l[g];
            double Sxxz = s->Drrs[di + 3][dk + 3] / s->dr2dsl[g];
            double Sxxzz = s->Drrss[di + 3][dk + 3] / s->dr2ds2l[g];
            s->SM1[di + 3][dk + 3] = Sxx - Szz;
            s->SM2[di + 3][dk + 3] = Sxxxx + Szzzz + 2.0 * Sxxzz;
            s->SM4[di + 3][dk + 3] = 4.0 * Sxz;
            s->SM5[di + 3][dk + 3] = 2.0 * (Sxxx + Sxzz);
            s->SM6[di + 3][dk + 3] = 2.0 * (Szzz + Sxxz);
        }
}

/* Compute_Matrix_coarse with analysis=1, iterative_solver.f90:1723-1745 (Database=2). */
int ref_coarse_bandwidth(ptref_state* s) {
    int nxc = s->nxl[s->grids], nzc = s->nzl[s->grids];
    int limit[7] = {0, 2, 2, 3, 2, 2, 0};
    int ku = 0, kl = 0, N = nzc + 1;
    for (int p = 1; p <= s->ngrid_coarse; p++) {
        int kp = p - N * ((p - 1) / N) - 1, ip = (p - 1) / N;
        for (int j = -3; j <= 3; j++) {
            int iq = j + ip;
            if (iq > 0 && iq < nxc)
                for (int kq = kp - limit[j + 3]; kq <= kp + limit[j + 3]; kq++)
                    if (kq > 0 && kq < nzc) {
                        int q = N * iq + kq + 1, t = q - p;
                        if (t > ku) ku = t;
                        if (-t > kl) kl = -t;
                    }
        }
    }
    s->kl = kl;
    s->ku = ku;
    return 0;
}

/* compute_smoothing_parameters, smoother.f90:31-73 */
static void smoothing_parameters(ptref_state* s) {
    const pt_config* c = &s->cfg;
    if (c->ivis == 0 || c->RaT == 0.0) s->delta_T = 2.0;
    else s->delta_T = (c->visT != 1.0) ? log(c->delta_visT) / log(c->visT) : 2.0;
    s->delta_C = 2.0;
    if (c->comp == 1) {
        if (c->conduct_factor != 1.0) s->delta_C = fabs(log(c->delta_visC) / log(1.0 / c->conduct_factor));
        if (c->ivis >= 2 && c->visC != 1.0) s->delta_C = fabs(log(c->delta_visC) / log(c->visC));
    }
}

ptref_state* ptref_create(const pt_config* cfg, int iterate, int nparts) {
    ptref_state* s = (ptref_state*)calloc(1, sizeof(ptref_state));
    s->cfg = *cfg;
    s->iterate = iterate;
    s->nparts = nparts < 0 ? 0 : nparts; /* 0 = canonical projection order */
    s->smooth_vis = 1;
    int nx = cfg->nx, nz = cfg->nz, grids = cfg->grids;
    smoothing_parameters(s);
    if (iterate == 1) {
        optimize_grid(&nx, &nz, &grids, cfg->mingrid);
        if (nx != cfg->nx || nz != cfg->nz) {
            ref_fail(s, PT_ERR_CONFIG, "optimize_grid changes nx/nz; choose a multigrid-compatible grid");
            return s;
        }
        s->grids = grids;
        if (multigrid_setup(s) != 0) {
            ref_fail(s, PT_ERR_CONFIG, "grids must be 2..6");
            return s;
        }
    } else {
        s->grids = 1;
    }
    s->nx = nx;
    s->nz = nz;
    /* compute_basics, basics.f90:204-333 */
    s->dr = cfg->aspect / (double)nx;
    s->ds = 1.0 / (double)nz;
    s->dr2 = s->dr * s->dr;
    s->ds2 = s->ds * s->ds;
    s->factorial[0] = 1.0; s->dr_power[0] = 1.0; s->ds_power[0] = 1.0;
    for (int j = 1; j <= 4; j++) {
        s->factorial[j] = (double)j * s->factorial[j - 1];
        s->dr_power[j] = pow(s->dr, (double)j);
        s->ds_power[j] = pow(s->ds, (double)j);
    }
    for (int j = 1; j <= s->grids; j++) {
        s->nxl[j] = nx / (1 << (j - 1));
        s->nzl[j] = nz / (1 << (j - 1));
        s->drl[j] = cfg->aspect / (double)s->nxl[j];
        s->dsl[j] = 1.0 / (double)s->nzl[j];
        s->dr2l[j] = s->drl[j] * s->drl[j];
        s->ds2l[j] = s->dsl[j] * s->dsl[j];
        s->dr3l[j] = pow(s->drl[j], 3.0);
        s->ds3l[j] = pow(s->dsl[j], 3.0);
        s->dr4l[j] = pow(s->drl[j], 4.0);
        s->ds4l[j] = pow(s->dsl[j], 4.0);
        s->drdsl[j] = s->drl[j] * s->dsl[j];
        s->drds2l[j] = s->drl[j] * s->ds2l[j];
        s->dr2dsl[j] = s->dr2l[j] * s->dsl[j];
        s->dr2ds2l[j] = s->dr2l[j] * s->ds2l[j];
    }
    s->ngrid_coarse = (s->nxl[s->grids] + 1) * (s->nzl[s->grids] + 1);
    fd_coefficients(s);
    chebyshev_prep_stream(s);
    derivative_eigenvalues(s);
    /* stability_RK4_smoother, smoother.f90:719-740 (uniform grid) */
    {
        double Trr_max = -s->Trr_base / s->dr2, Tss_max = -s->Trr_base / s->ds2;
        double eR = fabs(Trr_max / 1.0) + fabs(Tss_max / 1.0);
        s->dts = 2.0 * eR / (eR * eR + 0.0);
    }
    if (iterate == 1) {
        eigenvalue_prep(s);
        stream_space_matrix_prep(s);
        ref_coarse_bandwidth(s);
    }
    /* storage, basics.f90:70-202 */
    int n6 = nx + 13, m6 = nz + 13;
    s->xg = (double*)calloc((size_t)n6, sizeof(double));
    s->zg = (double*)calloc((size_t)m6, sizeof(double));
    s->T = ref_fld_alloc(nx, nz, 3);
    s->SF = ref_fld_alloc(nx, nz, 3);
    s->u = ref_fld_alloc(nx, nz, 3);
    s->w = ref_fld_alloc(nx, nz, 3);
    s->Tvis = ref_fld_alloc(nx, nz, 3);
    s->Tbuoy = ref_fld_alloc(nx, nz, 3);
    s->Tratio = ref_fld_alloc(nx, nz, 3);
    s->tsa = ref_fld_alloc(nx, nz, 3);
    s->Cnew = ref_fld_alloc(nx, nz, 5);
    s->Cvis = ref_fld_alloc(nx, nz, 5);
    s->Cbuoy = ref_fld_alloc(nx, nz, 5);
    s->conduct = ref_fld_alloc(nx, nz, 5);
    s->Textend = ref_fld_alloc(nx, nz, 5);
    s->conduct_r = ref_fld_alloc(nx, nz, 3);
    s->conduct_s = ref_fld_alloc(nx, nz, 3);
    s->vis = ref_fld_alloc(nx, nz, 3);
    s->strain = ref_fld_alloc(nx, nz, 3);
    size_t nder = (size_t)3 * (size_t)(nx + 1) * (size_t)(nz + 7);
    s->DERr_u = (double*)calloc(nder, sizeof(double));
    s->DERr_w = (double*)calloc(nder, sizeof(double));
    s->DERr_t = (double*)calloc(nder, sizeof(double));
    s->nempty = (int32_t*)calloc((size_t)(nx + 1) * (size_t)(nz + 1), sizeof(int32_t));
    if (iterate == 1) {
        for (int l = 1; l <= s->grids; l++) {
            int a = s->nxl[l], b = s->nzl[l];
            s->err[l] = ref_fld_alloc(a, b, 3);
            s->RHS[l] = ref_fld_alloc(a, b, 0);
            s->res[l] = ref_fld_alloc(a, b, 0);
            s->dtst[l] = ref_fld_alloc(a, b, 0);
            s->ratio[l] = ref_fld_alloc(a, b, 0);
            s->visg[l] = ref_fld_alloc(a, b, 3);
            s->visst[l] = ref_fld_alloc(a, b, 3);
            s->vx[l] = ref_fld_alloc(a, b, 0);
            s->vz[l] = ref_fld_alloc(a, b, 0);
            s->vxx[l] = ref_fld_alloc(a, b, 0);
            s->vzz[l] = ref_fld_alloc(a, b, 0);
            s->vxz[l] = ref_fld_alloc(a, b, 0);
            s->vxxpzz[l] = ref_fld_alloc(a, b, 0);
            s->vxxmzz[l] = ref_fld_alloc(a, b, 0);
            s->vsm[l] = ref_fld_alloc(a, b, 0);
        }
        for (int d = 0; d < 10; d++) s->SFd[d] = ref_fld_alloc(nx, nz, 0);
        s->S0 = ref_fld_alloc(nx, nz, 3);
        s->S1 = ref_fld_alloc(nx, nz, 3);
        s->S2 = ref_fld_alloc(nx, nz, 3);
        int ldab = 2 * s->kl + s->ku + 1;
        s->Mc = (double*)calloc((size_t)ldab * (size_t)s->ngrid_coarse, sizeof(double));
        s->Bc = (double*)calloc((size_t)s->ngrid_coarse, sizeof(double));
        s->RowB = (double*)calloc((size_t)s->ngrid_coarse, sizeof(double));
        s->ipiv = (int*)calloc((size_t)s->ngrid_coarse, sizeof(int));
    }
    s->ntr = cfg->ntr;
    size_t nt = (size_t)(cfg->ntr > 0 ? cfg->ntr : 1);
    double** tr[] = {&s->rtr, &s->str, &s->Ttr, &s->Ctr, &s->rtr0, &s->str0, &s->Ttr0, &s->rtr1,
                     &s->str1, &s->Ttr1, &s->rtr2, &s->str2, &s->Ttr2};
    for (size_t i = 0; i < sizeof tr / sizeof tr[0]; i++) *tr[i] = (double*)calloc(nt, sizeof(double));
    if (cfg->chebyshev) { /* RKC2 energy stepper: coefficients and the stage-1 slopes */
        if (cfg->nstage < 2 || cfg->nstage > 60) {
            ref_fail(s, PT_ERR_CONFIG, "nstage must be 2..60");
        } else {
            chebyshev_prep(s);
            s->u0 = (double*)calloc(nt, sizeof(double));
            s->w0 = (double*)calloc(nt, sizeof(double));
            s->dT0 = (double*)calloc(nt, sizeof(double));
        }
    }
    /* uniform grid, grid.f90:46-54 and 105-116 */
    double* xg = s->xg + 6;
    double* zg = s->zg + 6;
    for (int i = 0; i <= nx; i++) xg[i] = s->dr * (double)i;
    for (int k = 0; k <= nz; k++) zg[k] = s->ds * (double)k;
    for (int i = 1; i <= 6; i++) { xg[-i] = -xg[i]; xg[nx + i] = cfg->aspect - xg[nx - i] + cfg->aspect; }
    for (int k = 1; k <= 6; k++) { zg[-k] = -zg[k]; zg[nz + k] = 1.0 - zg[nz - k] + 1.0; }
    xg[0] = 0.0; zg[0] = 0.0; xg[nx] = cfg->aspect; zg[nz] = 1.0;
    /* entrainment_setup, composition.f90:765-774 */
    s->kent = 0;
    for (int k = 0; k <= nz; k++)
        if (s->ds * (double)k <= cfg->dent) s->kent = k;
    return s;
}

int ptref_set_types(ptref_state* s, const int32_t* Ttype) {
    if (!s->cfg.comp) return ref_fail(s, PT_ERR_CONFIG, "discrete tracer types need comp=1");
    if (!s->Ttype) s->Ttype = (int32_t*)malloc(sizeof(int32_t) * (size_t)(s->ntr > 0 ? s->ntr : 1));
    if (!s->count_type1) s->count_type1 = (int32_t*)calloc((size_t)(s->nx + 1) * (size_t)(s->nz + 1), sizeof(int32_t));
    for (int64_t t = 0; t < s->ntr; t++) {
        if (Ttype[t] != 0 && Ttype[t] != 1) return ref_fail(s, PT_ERR_ARG, "tracer types must be 0 or 1 (ntype=1)");
        s->Ttype[t] = Ttype[t];
        s->Ctr[t] = (double)Ttype[t]; /* the type as a composition value (Ctr is unused by OG) */
    }
    return 0;
}

void ptref_destroy(ptref_state* s) {
    if (!s) return;
    /* process-lifetime test helper: the OS reclaims the remaining buffers */
    free(s);
}

/* mzran, composition.f90:7-20: 32-bit signed arithmetic that wraps (as the binary does). */
typedef struct { int32_t i, j, k, n; } mzseed;
static double mzran(mzseed* sd) {
    int32_t ran_int = sd->i - sd->k;
    if (ran_int < 0) ran_int += 2147483579;
    sd->i = sd->j;
    sd->j = sd->k;
    sd->k = ran_int;
    sd->n = (int32_t)((uint32_t)69069u * (uint32_t)sd->n + (uint32_t)1013904243u);
    ran_int = (int32_t)((uint32_t)ran_int + (uint32_t)sd->n);
    return 0.5 + (0.2328306e-9) * (double)ran_int;
}

/* H_horizontal_boundaries, H_routines/H_func.f90:73-92 */
static double H_horizontal_boundaries(double z, double RaC, double RaT, double k, double zI) {
    double t1 = z - zI, t2 = k * t1, t3 = exp(2.0 * t2), t4 = t3 * t3, t5 = t3 + 1.0;
    return 4.0 * (RaC * (k * k) * t3 / (t5 * t5) - 2.0 * RaC * (k * k) * t4 / ((t5 * t5) * t5)) / RaT;
}

/* compute_heating, energy.f90:1-41, for the calls made on the hot path. */
double ref_heating(ptref_state* s, int i, int k) {
    const pt_config* c = &s->cfg;
    if (c->comp == 0) return c->H;
    if (s->iheattype_boundary) {
        double z = s->zg[k + 6], x = s->xg[i + 6];
        (void)x;
        if (z == 0.0 || z == 1.0) return H_horizontal_boundaries(z, c->RaC, c->RaT, s->klayer, s->dlayer);
        s->status = PT_ERR_CONFIG;
        return 0.0;
    }
    double cv = RF(s->Cvis, i, k);
    double heating = c->H * (1.0 - (0.0 + cv));
    heating = c->Htype * cv + heating;
    return heating;
}

/* temperature() work area (initial_conditions.f90:267-270, f0=0) and composition_continuous
 * (initial_conditions.f90:199-213, initial_comp=-1) of the shipped run. */
static double golden_temperature(ptref_state* s, double x, double z) {
    const pt_config* c = &s->cfg;
    double f0 = 0.0;
    double a = c->aspect;
    double t1 = -(pii * pii * pii) * ((a * a + 1.0) * (a * a + 1.0)) / (a * a * a) * cos(pii * x / a) * sin(pii * z) * f0;
    return (t1 + c->RaC / (1.0 + exp(-2.0 * s->klayer * (s->dlayer - z))) + (c->RaT - c->RaC) * (1.0 - z)) / c->RaT;
}
static double golden_composition(const ptref_state* s, double x, double z) {
    (void)x;
    return 1.0 / (1.0 + exp(-2.0 * s->klayer * (s->dlayer - z)));
}

/* initial_temperature (basics.f90:335-361) + initialize_tracers (composition.f90:776-858). */
int ptref_init_reference(ptref_state* s, int tpc, int nthreads_rng, double klayer, double dlayer,
                         int iheattype_boundary) {
    s->klayer = klayer;
    s->dlayer = dlayer;
    s->iheattype_boundary = iheattype_boundary;
    int nx = s->nx, nz = s->nz;
    double* xg = s->xg + 6;
    double* zg = s->zg + 6;
    for (int i = 0; i <= nx; i++)
        for (int k = 0; k <= nz; k++) RF(s->T, i, k) = golden_temperature(s, xg[i], zg[k]);
    s->cfg.Ttop_iso = RF(s->T, 0, nz);
    s->cfg.Tbot_iso = RF(s->T, 0, 0);
    for (int i = -3; i <= nx + 3; i++) { RF(s->T, i, 0) = s->cfg.Tbot_iso; RF(s->T, i, nz) = s->cfg.Ttop_iso; }
    ref_enforceBCs(s, &s->T);
    int64_t ntr = (int64_t)(nx + 1) * (nz + 1) * tpc;
    if (ntr != s->ntr) return ref_fail(s, PT_ERR_CONFIG, "ntr must be (nx+1)*(nz+1)*tpc");
    int np = nthreads_rng;
    mzseed seeds[64];
    seeds[0].i = 521288629; seeds[0].j = 362436069; seeds[0].k = 16163801; seeds[0].n = 1131199299;
    for (int j = 1; j < np; j++) {
        int32_t ran_int = seeds[j - 1].i - seeds[j - 1].k;
        if (ran_int < 0) ran_int += 2147483579;
        seeds[j].i = seeds[j - 1].j;
        seeds[j].j = seeds[j - 1].k;
        seeds[j].k = ran_int;
        seeds[j].n = (int32_t)((uint32_t)69069u * (uint32_t)seeds[j - 1].n + (uint32_t)1013904243u);
    }
    int nx_start[64], nx_finish[64];
    int64_t id_start[64];
    nx_start[0] = 0;
    for (int r = 0; r <= np - 2; r++) { nx_finish[r] = nx_start[r] + ((nx + 1) / np - 1); nx_start[r + 1] = nx_finish[r] + 1; }
    nx_finish[np - 1] = nx;
    id_start[0] = 1;
    for (int r = 0; r <= np - 2; r++) id_start[r + 1] = (int64_t)(nx_finish[r] - nx_start[r] + 1) * (nz + 1) * tpc + id_start[r];
    for (int r = 0; r < np; r++) {
        int64_t id = id_start[r];
        for (int i = nx_start[r]; i <= nx_finish[r]; i++) {
            double rcell = s->dr * (double)i;
            for (int k = 0; k <= nz; k++) {
                double scell = s->ds * (double)k;
                for (int p = 1; p <= tpc; p++) {
                    double pr = mzran(&seeds[r]);
                    double ps = mzran(&seeds[r]);
                    pr = (pr - 0.5) * s->dr;
                    ps = (ps - 0.5) * s->ds;
                    double rt = rcell + pr, st = scell + ps;
                    if (rt <= 0.0) rt = 0.0;
                    if (rt >= s->cfg.aspect) rt = s->cfg.aspect;
                    if (st <= 0.0) st = 0.0;
                    if (st >= 1.0) st = 1.0;
                    s->rtr[id - 1] = rt;
                    s->str[id - 1] = st;
                    if (s->cfg.comp == 1) s->Ctr[id - 1] = golden_composition(s, rt, st);
                    s->Ttr[id - 1] = golden_temperature(s, rt, st);
                    id++;
                }
            }
        }
    }
    int rc = ref_project(s, s->rtr, s->str, s->Ttr, &s->T, 1);
    if (rc) return rc;
    s->time = 0.0;
    return s->status;
}

static void copy_in(rfld* f, const double* src) {
    memcpy(f->p, src, sizeof(double) * (size_t)f->ld * (size_t)(f->nz + 2 * f->g + 1));
}

/* restart=1 branch of build_grid (grid.f90:55-104) and main.f90:204-210. */
int ptref_load_restart(ptref_state* s, const double* xg, const double* zg, const double* T,
                       const double* Cnew, const double* SF, const double* rtr, const double* str,
                       const double* Ctr, const double* Ttr) {
    int nx = s->nx, nz = s->nz;
    for (int i = 0; i <= nx; i++)
        if (fabs(xg[i + 6] - s->xg[i + 6]) > 1e-12 * s->cfg.aspect) return ref_fail(s, PT_ERR_CONFIG, "non-uniform xg");
    for (int k = 0; k <= nz; k++)
        if (fabs(zg[k + 6] - s->zg[k + 6]) > 1e-12) return ref_fail(s, PT_ERR_CONFIG, "non-uniform zg");
    copy_in(&s->T, T);
    copy_in(&s->SF, SF);
    if (s->cfg.comp == 1) copy_in(&s->Cnew, Cnew);
    ref_enforceBCs(s, &s->T);
    if (s->iterate == 1) ref_enforceBCs_stream(s, 1, &s->SF);
    if (s->cfg.comp == 1) ref_enforceBCs_comp(s, &s->Cnew);
    size_t nt = (size_t)s->ntr;
    memcpy(s->rtr, rtr, nt * sizeof(double));
    memcpy(s->str, str, nt * sizeof(double));
    memcpy(s->Ttr, Ttr, nt * sizeof(double));
    if (s->cfg.comp == 1 && !s->Ttype) memcpy(s->Ctr, Ctr, nt * sizeof(double)); /* types: Ctr already holds them */
    int rc = ref_project(s, s->rtr, s->str, s->Ttr, &s->T, 0);
    if (rc) return rc;
    ref_smoother_time_T(s, &s->T);
    if (s->cfg.comp != 0) ref_smoother_time(s);
    ref_load_conductivity(s);
    if (s->iterate == 1)
        for (int l = 2; l <= s->grids; l++)
            memset(s->err[l].p, 0, sizeof(double) * (size_t)s->err[l].ld * (size_t)(s->err[l].nz + 7));
    s->time = 0.0;
    return s->status;
}
