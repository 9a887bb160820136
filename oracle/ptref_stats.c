/*
 * ptref_stats.c -- oracle (test infrastructure only): velocities, stats, and the solve driver.
 */
#include "ptref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* compute_velocities (momentum.f90:655-710, uniform grid) + velocityBCs (composition.f90:1295-1325) */
void ref_compute_velocities(ptref_state* s) {
    int nx = s->nx, nz = s->nz;
    for (int k = 0; k <= nz; k++)
        for (int i = 0; i <= nx; i++) {
            double a = 0.0, b = 0.0;
            for (int j = -2; j <= 2; j++) a += s->D1[j + 3] * RF(s->SF, i + j, k);
            RF(s->w, i, k) = -a / s->dr;
            for (int j = -2; j <= 2; j++) b += s->D1[j + 3] * RF(s->SF, i, k + j);
            RF(s->u, i, k) = b / s->ds;
        }
    int Vbc = s->cfg.Vbc;
    for (int i = 1; i <= 3; i++) {
        for (int k = 0; k <= nz; k++) {
            RF(s->w, -i, k) = RF(s->w, i, k);
            RF(s->w, nx + i, k) = RF(s->w, nx - i, k);
        }
        for (int ii = 0; ii <= nx; ii++) {
            if (Vbc == 0) {
                RF(s->u, ii, -i) = RF(s->u, ii, i);
                RF(s->u, ii, nz + i) = RF(s->u, ii, nz - i);
            } else {
                RF(s->u, ii, -i) = -RF(s->u, ii, i);
                RF(s->u, ii, nz + i) = -RF(s->u, ii, nz - i);
            }
        }
    }
    for (int k = 1; k <= 3; k++) {
        for (int i = -3; i <= nx + 3; i++) {
            RF(s->w, i, -k) = -RF(s->w, i, k);
            RF(s->w, i, nz + k) = -RF(s->w, i, nz - k);
        }
        for (int kk = -3; kk <= nz + 3; kk++) {
            RF(s->u, -k, kk) = -RF(s->u, k, kk);
            RF(s->u, nx + k, kk) = -RF(s->u, nx - k, kk);
        }
    }
    for (int kk = -3; kk <= nz + 3; kk++) { RF(s->u, 0, kk) = 0.0; RF(s->u, nx, kk) = 0.0; }
    for (int i = -3; i <= nx + 3; i++) { RF(s->w, i, 0) = 0.0; RF(s->w, i, nz) = 0.0; }
    if (Vbc == 1)
        for (int i = -3; i <= nx + 3; i++) { RF(s->u, i, 0) = 0.0; RF(s->u, i, nz) = 0.0; }
}

int ptref_velocities(ptref_state* s) {
    ref_compute_velocities(s);
    return 0;
}

int ptref_solve_psi(ptref_state* s) {
    s->status = 0;
    int rc = (s->iterate == 1) ? ref_multigrid(s) : ref_direct_solve(s, s->cfg.ivis >= 1 || s->time == 0.0);
    if (rc) return rc;
    ref_compute_velocities(s);
    return 0;
}

/* integrate1Dx / integrate1Dz / integrate2D, basics.f90:479-528 (xr=zs=1) */
static double int1x(ptref_state* s, const double* f) {
    double fint = 0.0;
    for (int i = 0; i <= s->nx - 1; i++) fint = fint + 0.5 * (f[i] * 1.0 + f[i + 1] * 1.0) * s->dr;
    return fint;
}
static double int1z(ptref_state* s, const double* f, int k0) {
    double fint = 0.0;
    for (int k = k0; k <= s->nz - 1; k++) fint = fint + 0.5 * (f[k] * 1.0 + f[k + 1] * 1.0) * s->ds;
    return fint;
}
typedef double (*nodefn)(ptref_state*, int, int);
static double int2d(ptref_state* s, nodefn fn, int k0) {
    int nx = s->nx, nz = s->nz;
    double* row = (double*)malloc(sizeof(double) * (size_t)(nx + 1));
    double* fx = (double*)malloc(sizeof(double) * (size_t)(nz + 1));
    for (int k = 0; k <= nz; k++) {
        for (int i = 0; i <= nx; i++) row[i] = fn(s, i, k);
        fx[k] = int1x(s, row);
    }
    double r = int1z(s, fx, k0);
    free(row);
    free(fx);
    return r;
}
static double f_T(ptref_state* s, int i, int k) { return RF(s->T, i, k); }
static double f_C(ptref_state* s, int i, int k) { return RF(s->Cnew, i, k); }
static double f_v2(ptref_state* s, int i, int k) {
    double u = RF(s->u, i, k), w = RF(s->w, i, k);
    return u * u + w * w;
}
static double f_ra(ptref_state* s, int i, int k) { return s->cfg.RaT / RF(s->conduct, i, k) / RF(s->vis, i, k); }

/* stats, basics.f90:363-462 (comp=1 or 0, tracer=1, local_time=0) */
int ptref_stats(ptref_state* s, pt_stats_row* o) {
    int nx = s->nx, nz = s->nz;
    memset(o, 0, sizeof *o);
    if (s->iterate == 1)
        memcpy(s->vis.p, s->visg[1].p, sizeof(double) * (size_t)s->vis.ld * (size_t)(nz + 7));
    /* strain: compute_strain_rate_invariant_direct(1) (momentum.f90:73-92) or
     * compute_strain_rate_invariant (momentum.f90:1-34) for the direct path */
    double strain_max = -HUGE_VAL;
    for (int i = 0; i <= nx; i++) {
        int k = nz;
        double st;
        if (s->iterate == 1) {
            double Sxx = 0, Szz = 0, Sxz = 0;
            for (int j = -2; j <= 2; j++) Sxx += s->D2[j + 3] * RF(s->err[1], i + j, k);
            Sxx /= s->dr2;
            for (int j = -2; j <= 2; j++) Szz += s->D2[j + 3] * RF(s->err[1], i, k + j);
            Szz /= s->ds2;
            for (int k2 = -2; k2 <= 2; k2++)
                for (int i2 = -2; i2 <= 2; i2++) Sxz += s->Drs[i2 + 3][k2 + 3] * RF(s->err[1], i + i2, k + k2);
            Sxz /= (s->dr * s->ds);
            st = pow(2.0 * (Sxz * Sxz) + 0.5 * ((Szz - Sxx) * (Szz - Sxx)), 0.5);
        } else {
            double ur = 0, us = 0, wr = 0, ws = 0;
            for (int j = -2; j <= 2; j++) ur += s->D1[j + 3] * RF(s->u, i + j, k);
            ur /= s->dr;
            for (int j = -2; j <= 2; j++) us += s->D1[j + 3] * RF(s->u, i, k + j);
            us /= s->ds;
            for (int j = -2; j <= 2; j++) wr += s->D1[j + 3] * RF(s->w, i + j, k);
            wr /= s->dr;
            for (int j = -2; j <= 2; j++) ws += s->D1[j + 3] * RF(s->w, i, k + j);
            ws /= s->ds;
            double ux = ur / 1.0, uz = us / 1.0, wx = wr / 1.0, wz = ws / 1.0;
            st = pow(0.5 * (2.0 * (ux * ux + wz * wz) + (uz + wx) * (uz + wx)), 0.5);
        }
        if (st > strain_max) strain_max = st;
    }
    o->strain_max = strain_max;
    if (s->cfg.comp == 1) {
        o->Cavg = int2d(s, f_C, 0) / s->cfg.aspect;
        if (!s->have_mass) { s->mass = o->Cavg; s->have_mass = 1; }
        o->entrainment = int2d(s, f_C, s->kent) / s->cfg.aspect / s->mass;
    }
    int empty = 0, tmin = 0x7fffffff, tmax = -0x7fffffff;
    for (int q = 0; q < (nx + 1) * (nz + 1); q++) {
        int n = s->nempty[q];
        if (n == 0) empty++;
        if (n < tmin) tmin = n;
        if (n > tmax) tmax = n;
    }
    o->empty_cells = empty;
    o->tracer_min = tmin;
    o->tracer_max = tmax;
    o->vrms = pow(int2d(s, f_v2, 0) / s->cfg.aspect, 0.5);
    {
        double* row = (double*)malloc(sizeof(double) * (size_t)(nx + 1));
        for (int i = 0; i <= nx; i++) {
            double u = RF(s->u, i, nz), w = RF(s->w, i, nz);
            row[i] = u * u + w * w;
        }
        o->mobility = pow(int1x(s, row) / s->cfg.aspect, 0.5) / o->vrms;
        free(row);
    }
    if (s->cfg.RaT != 0.0) {
        o->Tavg = int2d(s, f_T, 0) / s->cfg.aspect;
        o->RaT_avg = int2d(s, f_ra, 0) / s->cfg.aspect;
        double* tz_s = (double*)malloc(sizeof(double) * (size_t)(nx + 1));
        double* tz_b = (double*)malloc(sizeof(double) * (size_t)(nx + 1));
        double* a = (double*)malloc(sizeof(double) * (size_t)(nx + 1));
        double* b = (double*)malloc(sizeof(double) * (size_t)(nx + 1));
        for (int i = 0; i <= nx; i++) {
            double t1 = 0, t2 = 0;
            for (int j = -2; j <= 2; j++) t1 += s->D1[j + 3] * RF(s->T, i, nz + j);
            for (int j = -2; j <= 2; j++) t2 += s->D1[j + 3] * RF(s->T, i, j);
            tz_s[i] = t1 / s->ds / 1.0;
            tz_b[i] = t2 / s->ds / 1.0;
        }
        for (int i = 0; i <= nx; i++) { a[i] = -(RF(s->conduct, i, nz) * tz_s[i]); b[i] = RF(s->T, i, 0); }
        o->Nu = int1x(s, a) / int1x(s, b);
        for (int i = 0; i <= nx; i++) a[i] = -(RF(s->conduct, i, 0) * tz_b[i]);
        o->Nu_bot = int1x(s, a) / s->cfg.aspect;
        {
            /* q1..q4, basics.f90:410-413: -conduct*dot/ds/zs */
            double d;
            d = 0; for (int j = -2; j <= 2; j++) d += s->D1[j + 3] * RF(s->T, 0, nz + j);
            o->q1 = -(RF(s->conduct, 0, nz) * d / s->ds / 1.0);
            d = 0; for (int j = -2; j <= 2; j++) d += s->D1[j + 3] * RF(s->T, nx, nz + j);
            o->q2 = -(RF(s->conduct, nx, nz) * d / s->ds / 1.0);
            d = 0; for (int j = -2; j <= 2; j++) d += s->D1[j + 3] * RF(s->T, nx, j);
            o->q3 = -(RF(s->conduct, nx, 0) * d / s->ds / 1.0);
            d = 0; for (int j = -2; j <= 2; j++) d += s->D1[j + 3] * RF(s->T, 0, j);
            o->q4 = -(RF(s->conduct, 0, 0) * d / s->ds / 1.0);
        }
        free(tz_s); free(tz_b); free(a); free(b);
    }
    o->time = s->time;
    return 0;
}

static rfld* field_of(ptref_state* s, int id) {
    switch (id) {
        case PT_F_T: return &s->T;
        case PT_F_TRATIO: return &s->Tratio;
        case PT_F_TVIS: return &s->Tvis;
        case PT_F_TBUOY: return &s->Tbuoy;
        case PT_F_CNEW: return &s->Cnew;
        case PT_F_CVIS: return &s->Cvis;
        case PT_F_CBUOY: return &s->Cbuoy;
        case PT_F_SF: return &s->SF;
        case PT_F_U: return &s->u;
        case PT_F_W: return &s->w;
        case PT_F_VIS: return s->iterate == 1 ? &s->visg[1] : &s->vis;
        default: return NULL;
    }
}

int ptref_get_field(ptref_state* s, int id, void* out) {
    int nx = s->nx, nz = s->nz;
    if (id == PT_F_NEMPTY) { memcpy(out, s->nempty, sizeof(int32_t) * (size_t)(nx + 1) * (nz + 1)); return 0; }
    if (id == PT_F_COUNT_TYPE) {
        if (!s->count_type1) return PT_ERR_ARG;
        memcpy(out, s->count_type1, sizeof(int32_t) * (size_t)(nx + 1) * (nz + 1));
        return 0;
    }
    if (id == PT_F_TRACER_TYPE) {
        if (!s->Ttype) return PT_ERR_ARG;
        memcpy(out, s->Ttype, sizeof(int32_t) * (size_t)s->ntr);
        return 0;
    }
    if (id == PT_F_RHS) {
        double* o = (double*)out;
        for (int k = 1; k <= nz - 1; k++)
            for (int i = 1; i <= nx - 1; i++) o[(i - 1) + (size_t)(k - 1) * (nx - 1)] = RF(s->RHS[1], i, k);
        return 0;
    }
    double* tr = NULL;
    switch (id) {
        case PT_F_TRACER_R: tr = s->rtr; break;
        case PT_F_TRACER_S: tr = s->str; break;
        case PT_F_TRACER_T: tr = s->Ttr; break;
        case PT_F_TRACER_C: tr = s->Ctr; break;
    }
    if (tr) { memcpy(out, tr, sizeof(double) * (size_t)s->ntr); return 0; }
    rfld* f = field_of(s, id);
    if (!f) return PT_ERR_ARG;
    memcpy(out, f->p, sizeof(double) * (size_t)f->ld * (size_t)(f->nz + 2 * f->g + 1));
    return 0;
}

int ptref_set_field(ptref_state* s, int id, const void* in) {
    double* tr = NULL;
    switch (id) {
        case PT_F_TRACER_R: tr = s->rtr; break;
        case PT_F_TRACER_S: tr = s->str; break;
        case PT_F_TRACER_T: tr = s->Ttr; break;
        case PT_F_TRACER_C: tr = s->Ctr; break;
    }
    if (tr) { memcpy(tr, in, sizeof(double) * (size_t)s->ntr); return 0; }
    rfld* f = field_of(s, id);
    if (!f) return PT_ERR_ARG;
    memcpy(f->p, in, sizeof(double) * (size_t)f->ld * (size_t)(f->nz + 2 * f->g + 1));
    return 0;
}

int ptref_get_scalar(ptref_state* s, const char* name, double* out) {
#define S(nm, expr) if (!strcmp(name, nm)) { *out = (double)(expr); return 0; }
    S("dt", s->dt) S("time", s->time) S("dts", s->dts) S("RKC1_stability", s->RKC1_stability)
    S("Tr_base", s->Tr_base) S("Trr_base", s->Trr_base) S("Trrr_base", s->Trrr_base)
    S("Trrrr_base", s->Trrrr_base) S("Trs_base", s->Trs_base) S("Trrs_base", s->Trrs_base)
    S("Trrss_base", s->Trrss_base) S("Tr_base_so", s->Tr_base_so) S("Trr_base_so", s->Trr_base_so)
    S("kl", s->kl) S("ku", s->ku) S("subD", s->subD) S("supD", s->supD) S("grids", s->grids)
    S("cycles", s->cycles) S("resid_ratio", s->resid_ratio) S("n_eta", s->n_eta) S("n_temp", s->n_temp)
    S("eig_fine", s->eig_fine) S("delta_T", s->delta_T) S("delta_C", s->delta_C) S("Tbot_iso", s->cfg.Tbot_iso)
    S("Ttop_iso", s->cfg.Ttop_iso) S("res_ref1", s->res_ref[1]) S("kent", s->kent)
#undef S
    if (!strncmp(name, "D1_", 3)) { *out = s->D1[atoi(name + 3) + 3]; return 0; }
    if (!strncmp(name, "D2_", 3)) { *out = s->D2[atoi(name + 3) + 3]; return 0; }
    if (!strncmp(name, "D3_", 3)) { *out = s->D3[atoi(name + 3) + 3]; return 0; }
    if (!strncmp(name, "D4_", 3)) { *out = s->D4[atoi(name + 3) + 3]; return 0; }
    return PT_ERR_ARG;
}
