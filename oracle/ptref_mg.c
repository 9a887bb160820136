/*
 * ptref_mg.c -- oracle (test infrastructure only): the variable-viscosity biharmonic
 * stream-function solve by multigrid, iterative_solver.f90:124-1887 (uniform grid, Newtonian,
 * RKC1 smoother, Database=2 coarse ordering).
 */
#include "ptref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double pii = 3.1415926535897932;

static rfld lview(rfld base, int nx, int nz, int g) {
    rfld f;
    f.p = base.p;
    f.nx = nx;
    f.nz = nz;
    f.g = g;
    f.ld = nx + 2 * g + 1;
    return f;
}

static void copy_lev(rfld* d, const rfld* s) {
    memcpy(d->p, s->p, sizeof(double) * (size_t)s->ld * (size_t)(s->nz + 2 * s->g + 1));
}

/* OpenMP static schedule of k=1..N over P threads: thread t's first k and count. */
static void part_range(int N, int P, int t, int* k0, int* cnt) {
    int q = N / P, r = N % P;
    *cnt = q + (t < r ? 1 : 0);
    *k0 = 1 + t * q + (t < r ? t : r);
}

/* enforceBCs_stream, iterative_solver.f90:1616-1664 */
void ref_enforceBCs_stream(ptref_state* s, int level, rfld* S0) {
    int nxl = s->nxl[level > 0 ? level : 1], nzl = s->nzl[level > 0 ? level : 1];
    if (s->iterate != 1) { nxl = s->nx; nzl = s->nz; }
    for (int k = -3; k <= nzl + 3; k++) { RF(*S0, 0, k) = 0.0; RF(*S0, nxl, k) = 0.0; }
    for (int i = -3; i <= nxl + 3; i++) { RF(*S0, i, 0) = 0.0; RF(*S0, i, nzl) = 0.0; }
    for (int k = 0; k <= nzl; k++)
        for (int i = 1; i <= 3; i++) RF(*S0, -i, k) = -RF(*S0, i, k);
    for (int k = 0; k <= nzl; k++)
        for (int i = 1; i <= 3; i++) RF(*S0, nxl + i, k) = -RF(*S0, nxl - i, k);
    double sg = (s->cfg.Vbc == 0) ? -1.0 : 1.0;
    for (int k = 1; k <= 3; k++)
        for (int i = -3; i <= nxl + 3; i++) RF(*S0, i, -k) = sg * RF(*S0, i, k);
    for (int k = 1; k <= 3; k++)
        for (int i = -3; i <= nxl + 3; i++) RF(*S0, i, nzl + k) = sg * RF(*S0, i, nzl - k);
}

/* compute_RHS, iterative_solver.f90:1075-1105 */
static void compute_RHS(ptref_state* s, int level) {
    rfld* R = &s->RHS[level];
    if (level == 1) {
        for (int k = 1; k <= s->nz - 1; k++)
            for (int i = 1; i <= s->nx - 1; i++) {
                double v = 0.0;
                if (s->cfg.RaT != 0.0) {
                    double Tr = 0.0;
                    for (int j = -2; j <= 2; j++) Tr += s->D1[j + 3] * RF(s->Tbuoy, i + j, k);
                    Tr = Tr / s->dr;
                    v = s->cfg.RaT * (Tr / 1.0);
                }
                if (s->cfg.comp == 1) {
                    double Cr = 0.0;
                    for (int j = -2; j <= 2; j++) Cr += s->D1[j + 3] * RF(s->Cbuoy, i + j, k);
                    Cr = Cr / s->dr;
                    v = v - s->cfg.RaC * (Cr / 1.0);
                }
                RF(*R, i, k) = v;
            }
    } else {
        /* restrict, iterative_solver.f90:1107-1125 */
        const rfld* in = &s->res[level - 1];
        for (int k = 1; k <= s->nzl[level] - 1; k++) {
            int kk = 2 * k;
            for (int i = 1; i <= s->nxl[level] - 1; i++) {
                int ii = 2 * i;
                double corners = (RF(*in, ii - 1, kk - 1) + RF(*in, ii - 1, kk + 1) + RF(*in, ii + 1, kk + 1) + RF(*in, ii + 1, kk - 1)) / 16.0;
                double sides = (RF(*in, ii - 1, kk) + RF(*in, ii, kk - 1) + RF(*in, ii + 1, kk) + RF(*in, ii, kk + 1)) / 8.0;
                double centre = RF(*in, ii, kk) / 4.0;
                RF(*R, i, k) = corners + sides + centre;
            }
        }
    }
}

/* compute_reference_residual, iterative_solver.f90:450-470 */
static void compute_reference_residual(ptref_state* s, int level) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    int P = s->nparts < 1 ? 1 : s->nparts;
    double total = 0.0;
    for (int t = 0; t < P; t++) {
        int k0, cnt;
        part_range(nzl - 1, P, t, &k0, &cnt);
        double part = 0.0;
        for (int k = k0; k < k0 + cnt; k++)
            for (int i = 1; i <= nxl - 1; i++) part = part + fabs(RF(s->RHS[level], i, k));
        total = total + part;
    }
    s->res_ref[level] = total / (double)(nxl - 2) / (double)(nzl - 2);
}

/* visf, rheology.f90:2-23 */
static double visf(ptref_state* s, int i, int k) {
    const pt_config* c = &s->cfg;
    double z = s->zg[k + 6];
    if (c->ivis == 1) return exp(-RF(s->Tvis, i, k) * log(c->visT) + (1.0 - z) * log(c->visP));
    if (c->ivis == 2 && c->comp == 1) {
        double dot = 0.0 + RF(s->Cvis, i, k) * log(c->visC);
        if (c->RaT != 0.0) return exp(-RF(s->Tvis, i, k) * log(c->visT) - dot + (1.0 - z) * log(c->visP));
        return exp(-dot + (1.0 - z) * log(c->visP));
    }
    return 1.0;
}

/* viscosityBCs, iterative_solver.f90:666-690 */
static void viscosityBCs(ptref_state* s, int level, rfld* v) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    for (int k = -3; k <= nzl + 3; k++)
        for (int i = 1; i <= 3; i++) RF(*v, -i, k) = RF(*v, i, k);
    for (int k = -3; k <= nzl + 3; k++)
        for (int i = 1; i <= 3; i++) RF(*v, nxl + i, k) = RF(*v, nxl - i, k);
    for (int k = 1; k <= 3; k++)
        for (int i = 0; i <= nxl; i++) {
            RF(*v, i, -k) = RF(*v, i, k);
            RF(*v, i, nzl + k) = RF(*v, i, nzl - k);
        }
}

/* viscosity_gradients, iterative_solver.f90:472-558 (uniform grid) */
static void viscosity_gradients(ptref_state* s, int level, int n) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    rfld *v = &s->visg[level];
    if (s->cfg.ivis == 0) {
        for (int k = 0; k <= nzl; k++)
            for (int i = 0; i <= nxl; i++) {
                RF(s->vx[level], i, k) = 0.0; RF(s->vz[level], i, k) = 0.0;
                RF(s->vxx[level], i, k) = 0.0; RF(s->vzz[level], i, k) = 0.0;
                RF(s->vxz[level], i, k) = 0.0; RF(s->vxxpzz[level], i, k) = 0.0;
                RF(s->vxxmzz[level], i, k) = 0.0;
            }
        return;
    }
    const double *D1so = s->D1_so + 1, *D2so = s->D2_so + 1;
    double dtv = s->dt_vis[level];
#pragma omp parallel for
    for (int k = 0; k <= nzl; k++)
        for (int i = 0; i <= nxl; i++) {
            double xx = 0.0, zz = 0.0;
            for (int j = -1; j <= 1; j++) xx += D2so[j] * RF(*v, i + j, k);
            xx = xx / s->dr2l[level];
            for (int j = -1; j <= 1; j++) zz += D2so[j] * RF(*v, i, k + j);
            zz = zz / s->ds2l[level];
            if (n != 0) {
                double xz = 0.0, x = 0.0, z = 0.0;
                for (int k2 = -1; k2 <= 1; k2++)
                    for (int i2 = -1; i2 <= 1; i2++) xz += s->Drs_so[i2 + 1][k2 + 1] * RF(*v, i + i2, k + k2);
                RF(s->vxz[level], i, k) = xz / s->drdsl[level];
                for (int j = -1; j <= 1; j++) x += D1so[j] * RF(*v, i + j, k);
                RF(s->vx[level], i, k) = x / s->drl[level];
                for (int j = -1; j <= 1; j++) z += D1so[j] * RF(*v, i, k + j);
                RF(s->vz[level], i, k) = z / s->dsl[level];
                RF(s->vxxmzz[level], i, k) = xx - zz;
            }
            RF(s->vxx[level], i, k) = xx;
            RF(s->vzz[level], i, k) = zz;
            RF(s->vxxpzz[level], i, k) = xx + zz;
            RF(s->vsm[level], i, k) = dtv * (xx + zz);
        }
}

/* test_eigenvalues, iterative_solver.f90:1187-1207 (RKC1=1, stream_tstep=1, diff_adv=1) */
static double test_eigenvalues(ptref_state* s, int level) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    double ae = -s->RKC1_stability / 2.0, be = (double)s->cfg.nstageS;
    double ctemp = s->cfg.courant_stream * (s->RKC1_stability / (ae * ae));
    const double* SR = s->SR[level];
    const double* SI = s->SI[level];
    double ratio_min = 1.0e100;
    for (int k = 1; k <= nzl - 1; k++)
        for (int i = 1; i <= nxl - 1; i++) {
            double vg = RF(s->visg[level], i, k);
            double eI = fabs(RF(s->vxxpzz[level], i, k) * SI[1]) + vg * SI[2] + fabs(RF(s->vxz[level], i, k) * SI[4]) +
                        fabs(RF(s->vx[level], i, k) * SI[5]) + fabs(RF(s->vz[level], i, k) * SI[6]);
            double eR = RF(s->vxxmzz[level], i, k) * SR[1] + vg * SR[2] + RF(s->vxz[level], i, k) * SR[4] +
                        RF(s->vx[level], i, k) * SR[5] + RF(s->vz[level], i, k) * SR[6];
            double ratio = fabs(eR / eI);
            RF(s->ratio[level], i, k) = ratio;
            double a = eR / ae, b = eI / be;
            RF(s->dtst[level], i, k) = ctemp * eR / (a * a + b * b);
            if (ratio < ratio_min) ratio_min = ratio;
        }
    return ratio_min;
}

/* smoother_vis, smoother.f90:454-580 */
static void smoother_vis(ptref_state* s, int level, int interpolate) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    rfld* v = &s->visg[level];
    viscosityBCs(s, level, v);
    int option, Niter;
    double lb, la;
    if (interpolate == 0) { option = 1; Niter = 3; lb = -3.0; la = -2.0; }
    else { option = 0; Niter = s->cfg.vis_iter; lb = -2.0; la = -1.0; }
    int Nvis_store = 0, nn_store = 1, n = 0, trigger = 0;
    double ratio_min = 1.0e100;
    int ivis = s->cfg.ivis;
    for (;;) {
        for (int nn = nn_store; nn <= Niter; nn++) {
            viscosity_gradients(s, level, Nvis_store);
            if (interpolate == 0 && (Nvis_store >= 1 || ivis == 0)) ratio_min = test_eigenvalues(s, level);
            if (option == 1) {
                if ((Nvis_store >= 1 && ratio_min > s->cfg.eig_ratio_min) || ivis == 0 || n > 20) {
                    if (level == 1) { s->eig_fine = ratio_min; s->n_eta = n; }
                    trigger = 1;
                    break;
                }
            } else {
                if (interpolate == 0) {
                    if (ratio_min > s->cfg.eig_ratio || ivis == 0) { trigger = 1; nn_store = nn; break; }
                } else if (Nvis_store >= 1 || ivis == 0) {
                    trigger = 1;
                    break;
                }
            }
            int ntemp = Niter - nn + 1;
            double c = 2.0 / (-lb - la + (lb - la) * cos((double)(2 * ntemp - 1) * pii / (double)(2 * Niter)));
            c = 0.99 * c;
            for (int k = 0; k <= nzl; k++)
                for (int i = 0; i <= nxl; i++) RF(*v, i, k) = RF(*v, i, k) + c * RF(s->vsm[level], i, k);
            viscosityBCs(s, level, v);
        }
        if (trigger) break;
        Nvis_store++;
        nn_store = 1;
        if (option == 1) { Niter = 6; lb = -2.0; la = -1.0; }
        n++;
    }
}

/* viscosityBCs_initialize, iterative_solver.f90:636-664 */
static void viscosityBCs_initialize(ptref_state* s, int level) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    rfld* v = &s->visg[level];
    const rfld* f = &s->visg[level - 1];
    for (int k = 1; k <= nzl - 1; k++) {
        RF(*v, 0, k) = RF(*f, 0, 2 * k);
        RF(*v, nxl, k) = RF(*f, s->nxl[level - 1], 2 * k);
    }
    for (int i = 0; i <= nxl; i++) {
        RF(*v, i, 0) = RF(*f, 2 * i, 0);
        RF(*v, i, nzl) = RF(*f, 2 * i, s->nzl[level - 1]);
    }
    for (int i = 1; i <= 3; i++)
        for (int k = 0; k <= nzl; k++) {
            RF(*v, -i, k) = RF(*v, i, k);
            RF(*v, nxl + i, k) = RF(*v, nxl - i, k);
        }
    for (int k = 1; k <= 3; k++)
        for (int i = -3; i <= nxl + 3; i++) {
            RF(*v, i, -k) = RF(*v, i, k);
            RF(*v, i, nzl + k) = RF(*v, i, nzl - k);
        }
}

/* compute_viscosity, iterative_solver.f90:560-634 (static=1, plastic=0, non_Newtonian=0) */
static void compute_viscosity(ptref_state* s, int level) {
    if (level == 1) {
        for (int k = 0; k <= s->nz; k++)
            for (int i = 0; i <= s->nx; i++) RF(s->visst[1], i, k) = visf(s, i, k);
        copy_lev(&s->visg[1], &s->visst[1]);
        smoother_vis(s, 1, 0);
        return;
    }
    int lf = level - 1;
    /* save the finer level's viscosity and gradients (vis_gridf ... vis_smoothf) */
    rfld* keep[] = {&s->visg[lf], &s->vx[lf], &s->vz[lf], &s->vxx[lf], &s->vzz[lf], &s->vxz[lf],
                    &s->vxxpzz[lf], &s->vxxmzz[lf], &s->vsm[lf]};
    double* saved[9];
    for (int q = 0; q < 9; q++) {
        size_t nb = sizeof(double) * (size_t)keep[q]->ld * (size_t)(keep[q]->nz + 2 * keep[q]->g + 1);
        saved[q] = (double*)malloc(nb);
        memcpy(saved[q], keep[q]->p, nb);
    }
    copy_lev(&s->visg[lf], &s->visst[lf]);
    smoother_vis(s, lf, 1);
    /* restrict_coefficients, iterative_solver.f90:1127-1145 */
    {
        const rfld* in = &s->visg[lf];
        rfld* out = &s->visg[level];
        for (int k = 1; k <= s->nzl[level] - 1; k++) {
            int kk = 2 * k;
            for (int i = 1; i <= s->nxl[level] - 1; i++) {
                int ii = 2 * i;
                double corners = (RF(*in, ii - 1, kk - 1) + RF(*in, ii - 1, kk + 1) + RF(*in, ii + 1, kk + 1) + RF(*in, ii + 1, kk - 1)) / 16.0;
                double sides = (RF(*in, ii - 1, kk) + RF(*in, ii, kk - 1) + RF(*in, ii + 1, kk) + RF(*in, ii, kk + 1)) / 8.0;
                double centre = RF(*in, ii, kk) / 4.0;
                RF(*out, i, k) = corners + sides + centre;
            }
        }
    }
    viscosityBCs_initialize(s, level);
    copy_lev(&s->visst[level], &s->visg[level]);
    smoother_vis(s, level, 0);
    for (int q = 0; q < 9; q++) {
        size_t nb = sizeof(double) * (size_t)keep[q]->ld * (size_t)(keep[q]->nz + 2 * keep[q]->g + 1);
        memcpy(keep[q]->p, saved[q], nb);
        free(saved[q]);
    }
}

/* stream_derivatives, iterative_solver.f90:973-1018 (uniform grid) */
static void stream_derivatives(ptref_state* s, int level, const rfld* S0) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    rfld d[10];
    for (int q = 0; q < 10; q++) d[q] = lview(s->SFd[q], nxl, nzl, 0);
    const double *D2 = s->D2 + 3, *D3 = s->D3 + 3, *D4 = s->D4 + 3;
#pragma omp parallel for
    for (int k = 0; k <= nzl; k++)
        for (int i = 0; i <= nxl; i++) {
            double a = 0, b = 0, c = 0;
            for (int j = -2; j <= 2; j++) a += D2[j] * RF(*S0, i + j, k);
            for (int j = -3; j <= 3; j++) b += D3[j] * RF(*S0, i + j, k);
            for (int j = -3; j <= 3; j++) c += D4[j] * RF(*S0, i + j, k);
            RF(d[0], i, k) = a / s->dr2l[level]; /* SFxx */
            RF(d[1], i, k) = b / s->dr3l[level]; /* SFxxx */
            RF(d[2], i, k) = c / s->dr4l[level]; /* SFxxxx */
            a = b = c = 0;
            for (int j = -2; j <= 2; j++) a += D2[j] * RF(*S0, i, k + j);
            for (int j = -3; j <= 3; j++) b += D3[j] * RF(*S0, i, k + j);
            for (int j = -3; j <= 3; j++) c += D4[j] * RF(*S0, i, k + j);
            RF(d[3], i, k) = a / s->ds2l[level]; /* SFzz */
            RF(d[4], i, k) = b / s->ds3l[level]; /* SFzzz */
            RF(d[5], i, k) = c / s->ds4l[level]; /* SFzzzz */
            double xz = 0, xxz = 0, xzz = 0, xxzz = 0;
            for (int k2 = -2; k2 <= 2; k2++)
                for (int i2 = -2; i2 <= 2; i2++) {
                    double v = RF(*S0, i + i2, k + k2);
                    xz += s->Drs[i2 + 3][k2 + 3] * v;
                    xxz += s->Drrs[i2 + 3][k2 + 3] * v;
                    xzz += s->Drss[i2 + 3][k2 + 3] * v;
                    xxzz += s->Drrss[i2 + 3][k2 + 3] * v;
                }
            RF(d[6], i, k) = xz / s->drdsl[level];
            RF(d[7], i, k) = xxz / s->dr2dsl[level];
            RF(d[8], i, k) = xzz / s->drds2l[level];
            RF(d[9], i, k) = xxzz / s->dr2ds2l[level];
        }
}

/* stream_space, iterative_solver.f90:890-911 (reads the derivative arrays at (i,k)) */
static inline double stream_space(ptref_state* s, int level, const rfld* d, int i, int k) {
    double r;
    double t2 = RF(s->visg[level], i, k) * (RF(d[2], i, k) + RF(d[5], i, k) + 2.0 * RF(d[9], i, k));
    if (s->cfg.ivis == 0) {
        r = t2 - RF(s->RHS[level], i, k);
    } else {
        double t1 = RF(s->vxxmzz[level], i, k) * (RF(d[0], i, k) - RF(d[3], i, k));
        double t4 = 4.0 * RF(s->vxz[level], i, k) * RF(d[6], i, k);
        double t5 = 2.0 * RF(s->vx[level], i, k) * (RF(d[1], i, k) + RF(d[8], i, k));
        double t6 = 2.0 * RF(s->vz[level], i, k) * (RF(d[4], i, k) + RF(d[7], i, k));
        r = t1 + t2 + t4 + t5 + t6 - RF(s->RHS[level], i, k);
    }
    return -r;
}

/* compute_residual, iterative_solver.f90:415-448 */
static int compute_residual(ptref_state* s, int level, int p) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    rfld d[10];
    for (int q = 0; q < 10; q++) d[q] = lview(s->SFd[q], nxl, nzl, 0);
    int P = s->nparts < 1 ? 1 : s->nparts;
    double total = 0.0;
    for (int t = 0; t < P; t++) {
        int k0, cnt;
        part_range(nzl - 1, P, t, &k0, &cnt);
        double part = 0.0;
        for (int k = k0; k < k0 + cnt; k++)
            for (int i = 1; i <= nxl - 1; i++) {
                double r = stream_space(s, level, d, i, k);
                RF(s->res[level], i, k) = r;
                part = part + fabs(r);
            }
        total = total + part;
    }
    s->residual_mag[p] = total / (double)(nxl - 2) / (double)(nzl - 2);
    if (!isfinite(s->residual_mag[p])) return ref_fail(s, PT_ERR_NOT_FINITE, "non-finite multigrid residual");
    if (level == 1 && s->residual_mag[p] > 1.0e10 * s->res_ref[level])
        return ref_fail(s, PT_ERR_MG_DIVERGED, "Multigrid Convergence Problem: Abnormally High Residual Detected");
    return 0;
}

/* iterate_stream, iterative_solver.f90:1418-1614 (RKC1=1, splitting=0) */
static int iterate_stream(ptref_state* s, int level, int Niter, int p) {
    int nxl = s->nxl[level], nzl = s->nzl[level];
    rfld E = s->err[level];
    rfld S0 = lview(s->S0, nxl, nzl, 3), S1 = lview(s->S1, nxl, nzl, 3), S2 = lview(s->S2, nxl, nzl, 3);
    rfld d[10];
    for (int q = 0; q < 10; q++) d[q] = lview(s->SFd[q], nxl, nzl, 0);
    int N = s->cfg.nstageS;
    for (int n = 1; n <= Niter; n++) {
        copy_lev(&S0, &E);
        stream_derivatives(s, level, &S0);
        int ntemp = Niter - n + 1;
        double temp = (s->cfg.Nmulti > 1) ? (s->cfg.c_2 - s->cfg.c_1) * (double)(ntemp - 1) / (double)(1 - Niter) : 0.0;
        double c = temp + s->cfg.c_2;
#pragma omp parallel for
        for (int k = 1; k <= nzl - 1; k++)
            for (int i = 1; i <= nxl - 1; i++) {
                RF(S1, i, k) = RF(S0, i, k) + s->mewtS[1] * c * RF(s->dtst[level], i, k) * stream_space(s, level, d, i, k);
                RF(S2, i, k) = RF(S0, i, k);
            }
        ref_enforceBCs_stream(s, level, &S1);
        for (int j = 2; j <= N; j++) {
            stream_derivatives(s, level, &S1);
#pragma omp parallel for
            for (int k = 1; k <= nzl - 1; k++)
                for (int i = 1; i <= nxl - 1; i++)
                    RF(E, i, k) = s->cS[j] * RF(S0, i, k) + s->mewS[j] * RF(S1, i, k) + s->vS[j] * RF(S2, i, k) +
                                  s->mewtS[j] * c * RF(s->dtst[level], i, k) * stream_space(s, level, d, i, k);
            ref_enforceBCs_stream(s, level, &E);
            if (j < N) {
                copy_lev(&S2, &S1);
                copy_lev(&S1, &E);
            }
        }
    }
    stream_derivatives(s, level, &E);
    return compute_residual(s, level, p);
}

/* prolong, iterative_solver.f90:343-396 */
static void prolong(ptref_state* s, int lc) {
    int lf = lc - 1;
    rfld* C = &s->err[lc];
    rfld* F = &s->err[lf];
    for (int k = 1; k <= s->nzl[lc] - 1; k++)
        for (int i = 1; i <= s->nxl[lc] - 1; i++) RF(*F, 2 * i, 2 * k) = RF(*F, 2 * i, 2 * k) + RF(*C, i, k);
    for (int k = 1; k <= s->nzl[lf] - 1; k += 2)
        for (int i = 2; i <= s->nxl[lf] - 2; i += 2)
            RF(*F, i, k) = RF(*F, i, k) + (RF(*C, i / 2, (k - 1) / 2) + RF(*C, i / 2, (k + 1) / 2)) / 2.0;
    for (int k = 2; k <= s->nzl[lf] - 2; k += 2)
        for (int i = 1; i <= s->nxl[lf] - 1; i += 2)
            RF(*F, i, k) = RF(*F, i, k) + (RF(*C, (i - 1) / 2, k / 2) + RF(*C, (i + 1) / 2, k / 2)) / 2.0;
    for (int k = 1; k <= s->nzl[lf] - 1; k += 2)
        for (int i = 1; i <= s->nxl[lf] - 1; i += 2)
            RF(*F, i, k) = RF(*F, i, k) + (RF(*C, (i - 1) / 2, (k - 1) / 2) + RF(*C, (i + 1) / 2, (k - 1) / 2) +
                                           RF(*C, (i + 1) / 2, (k + 1) / 2) + RF(*C, (i - 1) / 2, (k + 1) / 2)) / 4.0;
    ref_enforceBCs_stream(s, lf, F);
}

/* stream_space_matrix, iterative_solver.f90:745-825 (uniform grid) */
static double stream_space_matrix(ptref_state* s, int i, int k, int iq, int kq, int Sval) {
    int L = s->grids;
    int di = iq - i + 3, dk = kq - k + 3;
    double v;
    if (s->cfg.ivis == 0) v = RF(s->visg[L], i, k) * s->SM2[di][dk];
    else
        v = RF(s->vxxmzz[L], i, k) * s->SM1[di][dk] + RF(s->visg[L], i, k) * s->SM2[di][dk] +
            RF(s->vxz[L], i, k) * s->SM4[di][dk] + RF(s->vx[L], i, k) * s->SM5[di][dk] + RF(s->vz[L], i, k) * s->SM6[di][dk];
    return Sval == -1 ? -v : v;
}

/* Compute_Matrix_coarse (analysis=0), iterative_solver.f90:1747-1841 */
static int compute_matrix_coarse(ptref_state* s) {
    int nxc = s->nxl[s->grids], nzc = s->nzl[s->grids];
    int kl = s->kl, ku = s->ku, n = s->ngrid_coarse, ldab = 2 * kl + ku + 1, klku1 = kl + ku + 1;
    int N = nzc + 1;
    int limit[7] = {0, 2, 2, 3, 2, 2, 0};
    double* M = s->Mc;
    memset(M, 0, sizeof(double) * (size_t)ldab * (size_t)n);
#define MB(row, col) M[((row) - 1) + (size_t)((col) - 1) * (size_t)ldab]
    for (int p = 1; p <= n; p++) {
        int kp = p - N * ((p - 1) / N) - 1, ip = (p - 1) / N;
        if (ip > 0 && ip < nxc && kp > 0 && kp < nzc) {
            for (int j = -3; j <= 3; j++) {
                int iq = j + ip;
                if (iq >= 0 && iq <= nxc)
                    for (int kq = kp - limit[j + 3]; kq <= kp + limit[j + 3]; kq++)
                        if (kq >= 0 && kq <= nzc) {
                            int q = N * iq + kq + 1;
                            MB(klku1 + p - q, q) = stream_space_matrix(s, ip, kp, iq, kq, 1);
                        }
            }
            for (int j = -3; j <= 3; j++) {
                int iq = j + ip;
                for (int kq = kp - limit[j + 3]; kq <= kp + limit[j + 3]; kq++) {
                    if (iq < 0 || iq > nxc || kq < 0 || kq > nzc) {
                        int iiq, kkq, xval, zval;
                        if (iq < 0) { iiq = -iq; xval = -1; }
                        else if (iq > nxc) { iiq = 2 * nxc - iq; xval = -1; }
                        else { iiq = iq; xval = 1; }
                        if (kq < 0) { kkq = -kq; zval = (s->cfg.Vbc == 0) ? -1 : 1; }
                        else if (kq > nzc) { kkq = 2 * nzc - kq; zval = (s->cfg.Vbc == 0) ? -1 : 1; }
                        else { kkq = kq; zval = 1; }
                        int q = N * iiq + kkq + 1;
                        MB(klku1 + p - q, q) = MB(klku1 + p - q, q) + stream_space_matrix(s, ip, kp, iq, kq, xval * zval);
                    }
                }
            }
        }
    }
    for (int kp = 0; kp <= nzc; kp++) {
        MB(klku1, N * 0 + kp + 1) = 1.0;
        MB(klku1, N * nxc + kp + 1) = 1.0;
    }
    for (int ip = 0; ip <= nxc; ip++) {
        MB(klku1, N * ip + 0 + 1) = 1.0;
        MB(klku1, N * ip + nzc + 1) = 1.0;
    }
    /* DGBEQU on rows kl+1..2kl+ku+1 of the storage, then row scaling */
    if (ptref_band_equ(n, kl, ku, M + kl, ldab, s->RowB) != 0)
        return ref_fail(s, PT_ERR_SINGULAR_COARSE, "DGBEQU: zero row in the coarse matrix");
    for (int q = 1; q <= n; q++) {
        int p0 = q - ku > 1 ? q - ku : 1, p1 = q + kl < n ? q + kl : n;
        for (int p = p0; p <= p1; p++) MB(klku1 + p - q, q) = s->RowB[p - 1] * MB(klku1 + p - q, q);
    }
#undef MB
    return 0;
}

/* multigrid, iterative_solver.f90:124-341 (non_Newtonian=0) */
int ref_multigrid(ptref_state* s) {
    int grids = s->grids;
    copy_lev(&s->err[1], &s->SF);
    compute_RHS(s, 1);
    compute_reference_residual(s, 1);
    for (int level = 1; level <= grids; level++) compute_viscosity(s, level);
    if (s->time == 0.0 || s->cfg.ivis > 0) {
        if (compute_matrix_coarse(s)) return s->status;
        int info = ptref_band_lu(s->ngrid_coarse, s->kl, s->ku, s->Mc, 2 * s->kl + s->ku + 1, s->ipiv);
        if (info != 0) return ref_fail(s, PT_ERR_SINGULAR_COARSE, "DGBTRF: singular coarse matrix");
    }
    int q = 1, nsteps = s->nsteps;
    const int* multi = s->multi;
    int conv = 0;
    for (;;) {
        for (int p = 1; p <= nsteps; p++) {
            int level = multi[p];
            if (multi[p - 1] < multi[p]) {
                compute_RHS(s, level);
                if (s->cfg.mg_scheme == PT_MG_CORRECTION && level > 1)
                    memset(s->err[level].p, 0, sizeof(double) * (size_t)s->err[level].ld * (size_t)(s->err[level].nz + 7));
                if (p <= grids && q == 1) compute_reference_residual(s, level);
            }
            if (level < grids) {
                if (iterate_stream(s, level, s->cfg.Nmulti, p)) return s->status;
            } else {
                int nxc = s->nxl[grids], nzc = s->nzl[grids], N = nzc + 1;
                for (int t = 0; t < s->ngrid_coarse; t++) s->Bc[t] = 0.0;
                for (int k = 1; k <= nzc - 1; k++)
                    for (int i = 1; i <= nxc - 1; i++) {
                        int pp = N * i + k + 1;
                        s->Bc[pp - 1] = RF(s->RHS[grids], i, k) * s->RowB[pp - 1];
                    }
                ptref_band_solve(s->ngrid_coarse, s->kl, s->ku, s->Mc, 2 * s->kl + s->ku + 1, s->ipiv, s->Bc);
                for (int pp = 1; pp <= s->ngrid_coarse; pp++) {
                    int kp = pp - N * ((pp - 1) / N) - 1, ip = (pp - 1) / N;
                    RF(s->err[grids], ip, kp) = s->Bc[pp - 1];
                }
                ref_enforceBCs_stream(s, grids, &s->err[grids]);
            }
            if (level == 1 && s->residual_mag[1] / s->res_ref[1] <= s->cfg.tolerance) { conv = 1; break; }
            if (multi[p + 1] < multi[p]) prolong(s, level);
        }
        if (conv || s->residual_mag[1] / s->res_ref[1] <= s->cfg.tolerance) break;
        q++;
        if (q > s->cfg.max_cycles) return ref_fail(s, PT_ERR_MG_MAX_CYCLES, "Multigrid Convergence Problem: Too Many Multigrid Cycles Needed");
    }
    s->cycles = q;
    s->resid_ratio = s->residual_mag[1] / s->res_ref[1];
    copy_lev(&s->SF, &s->err[1]);
    return 0;
}
