/*
 * ptref_tracers.c -- oracle (test infrastructure only): tracer advection, projection, field
 * boundary conditions and the T/C smoothers.  Follows energy.f90, composition.f90 and
 * smoother.f90 of ProjecTracer_Source (uniform grid, order=4, tracer=1, torder=4, RK_update=1).
 */
#include "ptref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define D1(j) (s->D1[(j) + 3])
#define D2(j) (s->D2[(j) + 3])

/* enforceBCs, energy.f90:558-592 */
void ref_enforceBCs(ptref_state* s, rfld* T0) {
    int nx = s->nx, nz = s->nz;
    const pt_config* c = &s->cfg;
    for (int i = 1; i <= 3; i++)
        for (int k = 0; k <= nz; k++) {
            RF(*T0, -i, k) = RF(*T0, i, k);
            RF(*T0, nx + i, k) = RF(*T0, nx - i, k);
        }
    for (int k = 1; k <= 3; k++) {
        if (c->Tbot == 0) {
            for (int i = -3; i <= nx + 3; i++) {
                double heating = ref_heating(s, i, 0);
                RF(*T0, i, -k) = 2.0 * c->Tbot_iso + 2.0 / D2(0) * heating * s->ds2 - RF(*T0, i, k);
            }
        } else {
            for (int i = -3; i <= nx + 3; i++) RF(*T0, i, -k) = RF(*T0, i, k);
        }
        for (int i = -3; i <= nx + 3; i++) {
            double heating = ref_heating(s, i, nz);
            RF(*T0, i, nz + k) = 2.0 * c->Ttop_iso + 2.0 / D2(0) * heating * s->ds2 - RF(*T0, i, nz - k);
        }
    }
    if (c->Tbot == 0)
        for (int i = -3; i <= nx + 3; i++) RF(*T0, i, 0) = c->Tbot_iso;
    for (int i = -3; i <= nx + 3; i++) RF(*T0, i, nz) = c->Ttop_iso;
}

/* extendT, energy.f90:595-630 */
static void extendT(ptref_state* s, const rfld* T0) {
    int nx = s->nx, nz = s->nz;
    const pt_config* c = &s->cfg;
    rfld* X = &s->Textend;
    for (int k = 0; k <= nz; k++)
        for (int i = 0; i <= nx; i++) RF(*X, i, k) = RF(*T0, i, k);
    for (int i = 1; i <= 5; i++)
        for (int k = 0; k <= nz; k++) {
            RF(*X, -i, k) = RF(*X, i, k);
            RF(*X, nx + i, k) = RF(*X, nx - i, k);
        }
    for (int k = 1; k <= 5; k++) {
        if (c->Tbot == 0) {
            for (int i = -5; i <= nx + 5; i++) {
                double heating = ref_heating(s, i, 0);
                RF(*X, i, -k) = 2.0 * c->Tbot_iso + 2.0 / D2(0) * heating * s->ds2 - RF(*X, i, k);
            }
        } else {
            for (int i = -5; i <= nx + 5; i++) RF(*X, i, -k) = RF(*X, i, k);
        }
        for (int i = -5; i <= nx + 5; i++) {
            double heating = ref_heating(s, i, nz);
            RF(*X, i, nz + k) = 2.0 * c->Ttop_iso + 2.0 / D2(0) * heating * s->ds2 - RF(*X, i, nz - k);
        }
    }
    if (c->Tbot == 0)
        for (int i = -5; i <= nx + 5; i++) RF(*X, i, 0) = c->Tbot_iso;
    for (int i = -5; i <= nx + 5; i++) RF(*X, i, nz) = c->Ttop_iso;
}

/* enforceBCs_comp, composition.f90:1279-1292 (spanT=5) */
void ref_enforceBCs_comp(ptref_state* s, rfld* C0) {
    int nx = s->nx, nz = s->nz;
    for (int i = 1; i <= 5; i++) {
        for (int k = 0; k <= nz; k++) {
            RF(*C0, -i, k) = RF(*C0, i, k);
            RF(*C0, nx + i, k) = RF(*C0, nx - i, k);
        }
        for (int ii = -5; ii <= nx + 5; ii++) {
            RF(*C0, ii, -i) = RF(*C0, ii, i);
            RF(*C0, ii, nz + i) = RF(*C0, ii, nz - i);
        }
    }
}

/* smoothness, smoother.f90:75-95 */
static double smoothness(ptref_state* s, const rfld* T0) {
    double diff = 0.0;
    int nx = s->nx, nz = s->nz;
#pragma omp parallel for reduction(max : diff)
    for (int i = 0; i <= nx - 1; i++)
        for (int k = 1; k <= nz - 1; k++) {
            double c = RF(*T0, i, k);
            double a1 = fabs(RF(*T0, i, k - 1) - c);
            double a2 = fabs(RF(*T0, i + 1, k - 1) - c);
            double a3 = fabs(RF(*T0, i + 1, k) - c);
            double a4 = fabs(RF(*T0, i, k + 1) - c);
            double a5 = fabs(RF(*T0, i + 1, k + 1) - c);
            double a = a1;
            if (a2 > a) a = a2;
            if (a3 > a) a = a3;
            if (a4 > a) a = a4;
            if (a5 > a) a = a5;
            if (a > diff) diff = a;
        }
    return diff;
}

static void copy_fld(rfld* d, const rfld* src) {
    memcpy(d->p, src->p, sizeof(double) * (size_t)src->ld * (size_t)(src->nz + 2 * src->g + 1));
}

/* smoother_time_T, smoother.f90:638-672 (smoother_space 121-139 on the uniform grid) */
void ref_smoother_time_T(ptref_state* s, const rfld* Tin) {
    copy_fld(&s->Tvis, Tin);
    copy_fld(&s->Tbuoy, Tin);
    s->n_temp = 0;
    if (s->cfg.RaT == 0.0 || s->cfg.ivis == 0) return;
    int nx = s->nx, nz = s->nz;
    rfld T0 = ref_fld_alloc(nx, nz, 3);
    int n = 0;
    for (;;) {
        double diff = smoothness(s, &s->Tvis);
        if (diff < s->delta_T) { s->n_temp = n; break; }
        if (n >= 1000000) { ref_fail(s, PT_ERR_ITER_CAP, "T smoother iteration cap"); break; }
        copy_fld(&T0, &s->Tvis);
        double dts = s->dts * s->cfg.courantT;
#pragma omp parallel for
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                double Trr = 0.0, Tss = 0.0;
                for (int j = -2; j <= 2; j++) Trr += D2(j) * RF(T0, i + j, k);
                for (int j = -2; j <= 2; j++) Tss += D2(j) * RF(T0, i, k + j);
                Trr = Trr / s->dr2;
                Tss = Tss / s->ds2;
                RF(s->Tvis, i, k) = RF(T0, i, k) + dts * (Trr + Tss);
            }
        ref_enforceBCs(s, &s->Tvis);
        n++;
    }
    free(T0.p);
}

/* smoother_time, smoother.f90:582-636.  With C in [0,1] the smoothness metric never reaches
 * delta_C>1, so the loop exits before the first pass; that is the only case on the hot path
 * (delta_C=2 when conduct_factor=1 and ivis<2).  Other settings are rejected. */
void ref_smoother_time(ptref_state* s) {
    copy_fld(&s->Cvis, &s->Cnew);
    copy_fld(&s->Cbuoy, &s->Cnew);
    if (!(s->delta_C > 1.0)) ref_fail(s, PT_ERR_CONFIG, "C smoother with delta_C<=1 not supported");
}

/* load_conductivity_array, energy.f90:59-86 (conductivity 43-57) */
void ref_load_conductivity(ptref_state* s) {
    int nx = s->nx, nz = s->nz;
    rfld* C = &s->conduct;
    for (int i = 0; i <= nx; i++)
        for (int k = 0; k <= nz; k++) {
            double cd = 1.0;
            if (s->cfg.comp == 1) cd = cd + RF(s->Cvis, i, k) * (s->cfg.conduct_factor - 1.0);
            RF(*C, i, k) = cd;
        }
    for (int i = 1; i <= 5; i++)
        for (int k = 0; k <= nz; k++) {
            RF(*C, -i, k) = RF(*C, i, k);
            RF(*C, nx + i, k) = RF(*C, nx - i, k);
        }
    for (int k = 1; k <= 5; k++)
        for (int i = -5; i <= nx + 5; i++) {
            RF(*C, i, -k) = RF(*C, i, k);
            RF(*C, i, nz + k) = RF(*C, i, nz - k);
        }
    for (int i = -3; i <= nx + 3; i++)
        for (int k = -3; k <= nz + 3; k++) {
            double a = 0.0, b = 0.0;
            for (int j = -2; j <= 2; j++) a += D1(j) * RF(*C, i + j, k);
            for (int j = -2; j <= 2; j++) b += D1(j) * RF(*C, i, k + j);
            RF(s->conduct_r, i, k) = a / s->dr;
            RF(s->conduct_s, i, k) = b / s->ds;
        }
}

/* load_tracer_space_array, energy.f90:154-179 (tracer_space_uniform 135-151) */
static void load_tracer_space(ptref_state* s) {
    extendT(s, &s->Tratio);
    int nx = s->nx, nz = s->nz;
    const rfld* X = &s->Textend;
#pragma omp parallel for
    for (int k = -3; k <= nz + 3; k++)
        for (int i = -3; i <= nx + 3; i++) {
            double Tx = 0, Tz = 0, Txx = 0, Tzz = 0;
            for (int j = -2; j <= 2; j++) Tx += D1(j) * RF(*X, i + j, k);
            Tx = Tx / s->dr;
            for (int j = -2; j <= 2; j++) Tz += D1(j) * RF(*X, i, k + j);
            Tz = Tz / s->ds;
            for (int j = -2; j <= 2; j++) Txx += D2(j) * RF(*X, i + j, k);
            Txx = Txx / s->dr2;
            for (int j = -2; j <= 2; j++) Tzz += D2(j) * RF(*X, i, k + j);
            Tzz = Tzz / s->ds2;
            double kx = RF(s->conduct_r, i, k), kz = RF(s->conduct_s, i, k);
            double heating = ref_heating(s, i, k);
            RF(s->tsa, i, k) = RF(s->conduct, i, k) * (Txx + Tzz) + (kx * Tx + kz * Tz) + heating;
        }
}

/* compute_derivatives, composition.f90:1457-1478.  DERr(1:3,0:nx,-3:nz+3). */
static void compute_derivatives(ptref_state* s, const rfld* f, double* DERr) {
    int nx = s->nx, nz = s->nz;
#pragma omp parallel for
    for (int k = -3; k <= nz + 3; k++)
        for (int i = 0; i <= nx; i++)
            for (int jj = 1; jj <= 3; jj++) {
                double a = 0.0;
                for (int j = -3; j <= 3; j++) a += s->Dm[jj][j + 3] * RF(*f, i + j, k);
                DERr[(jj - 1) + 3 * ((size_t)i + (size_t)(nx + 1) * (size_t)(k + 3))] = a / s->dr_power[jj];
            }
}

/* interpolate, composition.f90:1359-1393 */
static double interpolate(ptref_state* s, double r, double sv, const double* DERr, const rfld* f) {
    int nx = s->nx;
    int i = (int)lround(r / s->dr);
    int k = (int)lround(sv / s->ds);
    double hr = r - (double)i * s->dr;
    double fR[7];
    for (int jj = -3; jj <= 3; jj++) fR[jj + 3] = RF(*f, i, k + jj);
    for (int j = 1; j <= 3; j++) {
        double a1 = pow(hr, (double)j) / s->factorial[j];
        for (int jj = -3; jj <= 3; jj++)
            fR[jj + 3] = fR[jj + 3] + DERr[(j - 1) + 3 * ((size_t)i + (size_t)(nx + 1) * (size_t)(k + jj + 3))] * a1;
    }
    double hs = sv - (double)k * s->ds;
    double DERs[4];
    for (int jj = 1; jj <= 3; jj++) {
        double a = 0.0;
        for (int j = -3; j <= 3; j++) a += s->Dm[jj][j + 3] * fR[j + 3];
        DERs[jj] = a / s->ds_power[jj];
    }
    double fi = fR[3];
    for (int j = 1; j <= 3; j++) {
        double a1 = pow(hs, (double)j) / s->factorial[j];
        fi = fi + DERs[j] * a1;
    }
    return fi;
}

/* the three pieces the tracer equalisation uses to give moved tracers their temperature */
void ref_extendT(ptref_state* s, const rfld* T0) { extendT(s, T0); }
void ref_compute_derivatives(ptref_state* s, const rfld* f, double* DERr) { compute_derivatives(s, f, DERr); }
double ref_interpolate(ptref_state* s, double r, double sv, const double* DERr, const rfld* f) {
    return interpolate(s, r, sv, DERr, f);
}

/* shape_func, composition.f90:896-921 (bilinear): the x and z factors of one (i,k) pair. */
static inline double shape_1d(double x, int i, double h) {
    double a = 1.0 - fabs(x - (double)i * h) / h;
    return a > 0.0 ? a : 0.0;
}

/* tracers_to_corners_OG, composition.f90:1090-1276, with ntype=1 and the bilinear shape function
 * (shape_function=1; shape_fn, composition.f90:888-894): per node the shape-weighted sum of T
 * (T1), the shape sums of the type-0 and the type-1 tracers (count_type_real), and the per-type
 * counts of the tracers whose nearest node it is (count_type).  nempty_real is the sum over the
 * types (1221), C = count_type_real(1)/nempty_real and T = T1/nempty_real where nempty_real > 0
 * (1243-1258).  Summation orders as in ref_project: nparts >= 1 the reference's per-thread ranges
 * added in rank order (1110-1177); nparts == 0 the GPU's canonical order (per cell in ID order,
 * then the 9 cells of a node in a fixed order). */
static void project_og_sums(ptref_state* s, const double* r, const double* sv, const double* Tt, double* T1,
                            double* cr0, double* cr1, int32_t* cnt, int32_t* cnt1, size_t nn) {
    int nx = s->nx, nz = s->nz;
    int64_t ntr = s->ntr;
    const int32_t* ty = s->Ttype;
#define NI(i, k) ((size_t)((i) + 1) + (size_t)((k) + 1) * (size_t)(nx + 3))
    if (s->nparts >= 1) {
        int P = s->nparts;
        int64_t Nshare = ntr / P;
        double* tw = (double*)calloc(nn * (size_t)P, sizeof(double));
        double* w0 = (double*)calloc(nn * (size_t)P, sizeof(double));
        double* w1 = (double*)calloc(nn * (size_t)P, sizeof(double));
        int32_t* c0 = (int32_t*)calloc(nn * (size_t)P, sizeof(int32_t));
        int32_t* c1 = (int32_t*)calloc(nn * (size_t)P, sizeof(int32_t));
#pragma omp parallel for schedule(static, 1)
        for (int rank = 0; rank < P; rank++) {
            int64_t id_min = 1 + (int64_t)rank * Nshare;
            int64_t id_max = (rank == P - 1) ? ((rank + 1) * Nshare > ntr ? (rank + 1) * Nshare : ntr) : (rank + 1) * Nshare;
            size_t o = nn * (size_t)rank;
            for (int64_t id = id_min; id <= id_max; id++) {
                double rr = r[id - 1], ss = sv[id - 1];
                int i = (int)lround(rr / s->dr), k = (int)lround(ss / s->ds);
                int t1 = ty[id - 1] == 1;
                if (t1) c1[o + NI(i, k)]++;
                else c0[o + NI(i, k)]++;
                for (int di = -1; di <= 1; di++)
                    for (int dk = -1; dk <= 1; dk++) {
                        double S = shape_1d(rr, i + di, s->dr) * shape_1d(ss, k + dk, s->ds);
                        tw[o + NI(i + di, k + dk)] = tw[o + NI(i + di, k + dk)] + Tt[id - 1] * S;
                        double* w = t1 ? w1 : w0;
                        w[o + NI(i + di, k + dk)] = w[o + NI(i + di, k + dk)] + S;
                    }
            }
        }
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                double a = 0.0, b0 = 0.0, b1 = 0.0;
                int32_t n0 = 0, n1 = 0;
                for (int rank = 0; rank < P; rank++) {
                    size_t q = nn * (size_t)rank + NI(i, k);
                    a = a + tw[q];
                    b0 = b0 + w0[q];
                    b1 = b1 + w1[q];
                    n0 += c0[q];
                    n1 += c1[q];
                }
                T1[NI(i, k)] = a;
                cr0[NI(i, k)] = b0;
                cr1[NI(i, k)] = b1;
                cnt[NI(i, k)] = n0 + n1;
                cnt1[NI(i, k)] = n1;
            }
        free(tw); free(w0); free(w1); free(c0); free(c1);
    } else {
        size_t ncell = (size_t)(nx + 1) * (size_t)(nz + 1);
        int64_t* start = (int64_t*)calloc(ncell + 1, sizeof(int64_t));
        int64_t* list = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ntr > 0 ? ntr : 1));
        int32_t* cell = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ntr > 0 ? ntr : 1));
        for (int64_t id = 0; id < ntr; id++) {
            int i = (int)lround(r[id] / s->dr), k = (int)lround(sv[id] / s->ds);
            cell[id] = i + (nx + 1) * k;
            start[cell[id] + 1]++;
        }
        for (size_t q = 0; q < ncell; q++) start[q + 1] += start[q];
        int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (ncell + 1));
        memcpy(fill, start, sizeof(int64_t) * (ncell + 1));
        for (int64_t id = 0; id < ntr; id++) list[fill[cell[id]]++] = id;
        free(fill);
        double* Pc = (double*)calloc(ncell * 27, sizeof(double)); /* [cell][T, S type 1, S type 0][3x3] */
        int32_t* n1c = (int32_t*)calloc(ncell, sizeof(int32_t));
#pragma omp parallel for schedule(dynamic, 64)
        for (size_t q = 0; q < ncell; q++) {
            int ci = (int)(q % (size_t)(nx + 1)), ck = (int)(q / (size_t)(nx + 1));
            double* pc = Pc + q * 27;
            for (int64_t t = start[q]; t < start[q + 1]; t++) {
                int64_t id = list[t];
                double rr = r[id], ss = sv[id];
                int t1 = ty[id] == 1;
                n1c[q] += t1;
                double wx[3], wz[3];
                for (int d = 0; d < 3; d++) {
                    wx[d] = shape_1d(rr, ci + d - 1, s->dr);
                    wz[d] = shape_1d(ss, ck + d - 1, s->ds);
                }
                for (int dz = 0; dz < 3; dz++)
                    for (int dx = 0; dx < 3; dx++) {
                        double S = wx[dx] * wz[dz];
                        pc[0 * 9 + dz * 3 + dx] = pc[0 * 9 + dz * 3 + dx] + Tt[id] * S;
                        int plane = t1 ? 1 : 2;
                        pc[plane * 9 + dz * 3 + dx] = pc[plane * 9 + dz * 3 + dx] + S;
                    }
            }
        }
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                double a = 0.0, b1 = 0.0, b0 = 0.0;
                for (int ck = k - 1; ck <= k + 1; ck++)
                    for (int ci = i - 1; ci <= i + 1; ci++) {
                        if (ci < 0 || ci > nx || ck < 0 || ck > nz) continue;
                        const double* pc = Pc + ((size_t)ci + (size_t)(nx + 1) * (size_t)ck) * 27;
                        int dz = k - ck + 1, dx = i - ci + 1;
                        a = a + pc[0 * 9 + dz * 3 + dx];
                        b1 = b1 + pc[1 * 9 + dz * 3 + dx];
                        b0 = b0 + pc[2 * 9 + dz * 3 + dx];
                    }
                size_t q = (size_t)i + (size_t)(nx + 1) * (size_t)k;
                T1[NI(i, k)] = a;
                cr0[NI(i, k)] = b0;
                cr1[NI(i, k)] = b1;
                cnt[NI(i, k)] = (int32_t)(start[q + 1] - start[q]);
                cnt1[NI(i, k)] = n1c[q];
            }
        free(Pc); free(n1c); free(start); free(list); free(cell);
    }
#undef NI
}

/* tracers_to_corners_iC_continuous, composition.f90:942-1087.
 * nparts>=1: the reference's order -- tracer IDs split into nparts contiguous ranges (one per
 *            OpenMP thread), each summed in ID order, then the ranges added in rank order.
 * nparts==0: the GPU's canonical order -- per cell (nint of the position) a partial sum over its
 *            tracers in ID order for each of the 9 target nodes, then per node the 9 partials in
 *            the fixed order (k-1..k+1 outer, i-1..i+1 inner).  Same terms, fixed association. */
int ref_project(ptref_state* s, const double* r, const double* sv, const double* Tt, const rfld* T0,
                int smooth) {
    int nx = s->nx, nz = s->nz;
    const pt_config* c = &s->cfg;
    int64_t ntr = s->ntr;
    int comp = c->comp;
    copy_fld(&s->Tratio, T0);
    size_t nn = (size_t)(nx + 3) * (size_t)(nz + 3); /* nodes -1..nx+1 */
#define NI(i, k) ((size_t)((i) + 1) + (size_t)((k) + 1) * (size_t)(nx + 3))
    double* shape_sum = (double*)calloc(nn, sizeof(double));
    double* TxS = (double*)calloc(nn, sizeof(double));
    double* CxS = (double*)calloc(nn, sizeof(double));
    int32_t* cnt = (int32_t*)calloc(nn, sizeof(int32_t));
    for (int64_t id = 0; id < ntr; id++) {
        double rr = r[id], ss = sv[id];
        if (rr < 0.0 || rr > c->aspect || ss < 0.0 || ss > 1.0) {
            free(shape_sum); free(TxS); free(CxS); free(cnt);
            return ref_fail(s, PT_ERR_TRACER_OUT_OF_DOMAIN, "Tracer advected outside of domain");
        }
    }
    if (s->Ttype) { /* discrete types: tracers_to_corners_OG */
        double* cr0 = (double*)calloc(nn, sizeof(double));
        int32_t* cnt1 = (int32_t*)calloc(nn, sizeof(int32_t));
        project_og_sums(s, r, sv, Tt, TxS, cr0, CxS, cnt, cnt1, nn);
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                s->count_type1[i + (nx + 1) * k] = cnt1[NI(i, k)];
                shape_sum[NI(i, k)] = cr0[NI(i, k)] + CxS[NI(i, k)];
            }
        free(cr0); free(cnt1);
    } else if (s->nparts >= 1) {
        int P = s->nparts;
        int64_t Nshare = ntr / P;
        double* ssw = (double*)calloc(nn * (size_t)P, sizeof(double));
        double* tsw = (double*)calloc(nn * (size_t)P, sizeof(double));
        double* csw = (double*)calloc(nn * (size_t)P, sizeof(double));
        int32_t* cw = (int32_t*)calloc(nn * (size_t)P, sizeof(int32_t));
#pragma omp parallel for schedule(static, 1)
        for (int rank = 0; rank < P; rank++) {
            int64_t id_min = 1 + (int64_t)rank * Nshare;
            int64_t id_max = (rank == P - 1) ? ((rank + 1) * Nshare > ntr ? (rank + 1) * Nshare : ntr) : (rank + 1) * Nshare;
            double* sw = ssw + nn * rank;
            double* tw = tsw + nn * rank;
            double* cwk = csw + nn * rank;
            int32_t* cc = cw + nn * rank;
            for (int64_t id = id_min; id <= id_max; id++) {
                double rr = r[id - 1], ss = sv[id - 1];
                int i = (int)lround(rr / s->dr), k = (int)lround(ss / s->ds);
                cc[NI(i, k)]++;
                for (int di = -1; di <= 1; di++)
                    for (int dk = -1; dk <= 1; dk++) {
                        double S = shape_1d(rr, i + di, s->dr) * shape_1d(ss, k + dk, s->ds);
                        tw[NI(i + di, k + dk)] = tw[NI(i + di, k + dk)] + Tt[id - 1] * S;
                        if (comp) cwk[NI(i + di, k + dk)] = cwk[NI(i + di, k + dk)] + s->Ctr[id - 1] * S;
                    }
                for (int di = -1; di <= 1; di++)
                    for (int dk = -1; dk <= 1; dk++) {
                        double S = shape_1d(rr, i + di, s->dr) * shape_1d(ss, k + dk, s->ds);
                        sw[NI(i + di, k + dk)] = sw[NI(i + di, k + dk)] + S;
                    }
            }
        }
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                int32_t n = 0;
                double a = 0.0, b = 0.0, d = 0.0;
                for (int rank = 0; rank < P; rank++) {
                    n += cw[nn * rank + NI(i, k)];
                    a = a + ssw[nn * rank + NI(i, k)];
                    b = b + tsw[nn * rank + NI(i, k)];
                    d = d + csw[nn * rank + NI(i, k)];
                }
                cnt[NI(i, k)] = n;
                shape_sum[NI(i, k)] = a;
                TxS[NI(i, k)] = b;
                CxS[NI(i, k)] = d;
            }
        free(ssw); free(tsw); free(csw); free(cw);
    } else {
        /* canonical order: bucket tracers by cell (stable in ID), per-cell partial sums */
        size_t ncell = (size_t)(nx + 1) * (size_t)(nz + 1);
        int64_t* start = (int64_t*)calloc(ncell + 1, sizeof(int64_t));
        int64_t* list = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ntr > 0 ? ntr : 1));
        int32_t* cell = (int32_t*)malloc(sizeof(int32_t) * (size_t)(ntr > 0 ? ntr : 1));
        for (int64_t id = 0; id < ntr; id++) {
            int i = (int)lround(r[id] / s->dr), k = (int)lround(sv[id] / s->ds);
            cell[id] = i + (nx + 1) * k;
            start[cell[id] + 1]++;
        }
        for (size_t q = 0; q < ncell; q++) start[q + 1] += start[q];
        int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (ncell + 1));
        memcpy(fill, start, sizeof(int64_t) * (ncell + 1));
        for (int64_t id = 0; id < ntr; id++) list[fill[cell[id]]++] = id;
        free(fill);
        double* P = (double*)calloc(ncell * 27, sizeof(double)); /* [cell][3 quantities][3x3] */
#pragma omp parallel for schedule(dynamic, 64)
        for (size_t q = 0; q < ncell; q++) {
            int ci = (int)(q % (size_t)(nx + 1)), ck = (int)(q / (size_t)(nx + 1));
            double* pc = P + q * 27;
            for (int64_t t = start[q]; t < start[q + 1]; t++) {
                int64_t id = list[t];
                double rr = r[id], ss = sv[id];
                double wx[3], wz[3];
                for (int d = 0; d < 3; d++) {
                    wx[d] = shape_1d(rr, ci + d - 1, s->dr);
                    wz[d] = shape_1d(ss, ck + d - 1, s->ds);
                }
                for (int dz = 0; dz < 3; dz++)
                    for (int dx = 0; dx < 3; dx++) {
                        double S = wx[dx] * wz[dz];
                        pc[0 * 9 + dz * 3 + dx] = pc[0 * 9 + dz * 3 + dx] + Tt[id] * S;
                        if (comp) pc[1 * 9 + dz * 3 + dx] = pc[1 * 9 + dz * 3 + dx] + s->Ctr[id] * S;
                        pc[2 * 9 + dz * 3 + dx] = pc[2 * 9 + dz * 3 + dx] + S;
                    }
            }
        }
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                double a = 0.0, b = 0.0, d = 0.0;
                for (int ck = k - 1; ck <= k + 1; ck++)
                    for (int ci = i - 1; ci <= i + 1; ci++) {
                        if (ci < 0 || ci > nx || ck < 0 || ck > nz) continue;
                        const double* pc = P + ((size_t)ci + (size_t)(nx + 1) * (size_t)ck) * 27;
                        int dz = k - ck + 1, dx = i - ci + 1;
                        b = b + pc[0 * 9 + dz * 3 + dx];
                        d = d + pc[1 * 9 + dz * 3 + dx];
                        a = a + pc[2 * 9 + dz * 3 + dx];
                    }
                cnt[NI(i, k)] = (int32_t)(start[(size_t)i + (size_t)(nx + 1) * k + 1] - start[(size_t)i + (size_t)(nx + 1) * k]);
                shape_sum[NI(i, k)] = a;
                TxS[NI(i, k)] = b;
                CxS[NI(i, k)] = d;
            }
        free(P); free(start); free(list); free(cell);
    }
    for (int k = 0; k <= nz; k++)
        for (int i = 0; i <= nx; i++) {
            s->nempty[i + (nx + 1) * k] = cnt[NI(i, k)];
            if (shape_sum[NI(i, k)] > 0.0) {
                RF(s->Tratio, i, k) = TxS[NI(i, k)] / shape_sum[NI(i, k)];
                if (comp) RF(s->Cnew, i, k) = CxS[NI(i, k)] / shape_sum[NI(i, k)];
            }
        }
    free(shape_sum); free(TxS); free(CxS); free(cnt);
#undef NI
    if (comp) {
        ref_enforceBCs_comp(s, &s->Cnew);
        if (smooth) ref_smoother_time(s);
    }
    ref_enforceBCs(s, &s->Tratio);
    if (smooth) ref_smoother_time_T(s, &s->Tratio);
    ref_load_conductivity(s);
    return s->status;
}

/* stability_RK4, energy.f90:756-810 (eigA/eigD 850-875; tracer=1, torder=4, uniform grid: xr=zs=1,
 * xrr=zss=0).  CFL=1 adds the velocities to the advective eigenvalue (859-866) and caps dt at
 * 2/eigD_max (809). */
static double stability_RK4(ptref_state* s) {
    int nx = s->nx, nz = s->nz;
    double Ts_max = s->Tr_base / s->ds, Tr_max = s->Tr_base / s->dr;
    double Tss_max = -s->Trr_base / s->ds2, Trr_max = -s->Trr_base / s->dr2;
    double dt;
    if (s->cfg.RaT != 0.0) {
        double eigA_max = 0.0, eigD_max = 0.0;
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                double cd = RF(s->conduct, i, k);
                double uu = s->cfg.CFL == 1 ? RF(s->u, i, k) : 0.0, ww = s->cfg.CFL == 1 ? RF(s->w, i, k) : 0.0;
                double eA = fabs(-cd * 0.0 / 1.0 - uu / 1.0 + RF(s->conduct_r, i, k) / 1.0) * Tr_max +
                            fabs(-cd * 0.0 / 1.0 - ww / 1.0 + RF(s->conduct_s, i, k) / 1.0) * Ts_max;
                double eD = cd * (fabs(Trr_max / 1.0) + fabs(Tss_max / 1.0));
                if (eA > eigA_max) eigA_max = eA;
                if (eD > eigD_max) eigD_max = eD;
            }
        double dtA, dtD;
        if (s->cfg.chebyshev) { /* torder=2 (energy.f90:787-793), required by the RKC2 stepper */
            if (eigA_max >= eigD_max)
                return ref_fail(s, PT_ERR_CONFIG, "Advective Eigenvalues Exceed Diffusive Eigenvalues -- this does not work for RK2"), 0.0;
            dtA = 1.0 / eigA_max;
            dtD = 2.0 / eigD_max;
        } else {
            dtA = 2.8 / eigA_max;
            dtD = 2.8 / eigD_max;
        }
        dt = (eigA_max == 0.0) ? dtD : 1.0 / (1.0 / dtA + 1.0 / dtD);
        dt = s->cfg.courant * dt;
        if (s->cfg.CFL == 1 && 2.0 / eigD_max < dt) dt = 2.0 / eigD_max;
    } else {
        return ref_fail(s, PT_ERR_CONFIG, "RaT=0 (dt_manual) not supported"), 0.0;
    }
    return dt;
}

static rfld fld_view(ptref_state* s, double* p, int g) {
    rfld f;
    f.p = p;
    f.nx = s->nx;
    f.nz = s->nz;
    f.g = g;
    f.ld = s->nx + 2 * g + 1;
    return f;
}

int ptref_project(ptref_state* s, const double* r, const double* sv, const double* Tt,
                  const double* T0field, int smooth) {
    rfld T0 = ref_fld_alloc(s->nx, s->nz, 3);
    memcpy(T0.p, T0field ? T0field : s->Tratio.p, sizeof(double) * (size_t)T0.ld * (size_t)(s->nz + 7));
    int rc = ref_project(s, r, sv, Tt, &T0, smooth);
    free(T0.p);
    return rc;
}

int ptref_compute_derivatives(ptref_state* s, const double* f, double* DERr) {
    rfld F = fld_view(s, (double*)f, 3);
    compute_derivatives(s, &F, DERr);
    return 0;
}

double ptref_interpolate(ptref_state* s, double r, double sv, const double* DERr, const double* f) {
    rfld F = fld_view(s, (double*)f, 3);
    return interpolate(s, r, sv, DERr, &F);
}

int ptref_load_tracer_space(ptref_state* s, double* tsa_out) {
    load_tracer_space(s);
    if (tsa_out) memcpy(tsa_out, s->tsa.p, sizeof(double) * (size_t)s->tsa.ld * (size_t)(s->nz + 7));
    return s->status;
}

int ptref_smoother_T(ptref_state* s, const double* Tin) {
    rfld T = fld_view(s, (double*)Tin, 3);
    rfld Tc = ref_fld_alloc(s->nx, s->nz, 3);
    copy_fld(&Tc, &T);
    ref_smoother_time_T(s, &Tc);
    free(Tc.p);
    return s->status;
}

static int update_velocities(ptref_state* s) {
    int rc = (s->iterate == 1) ? ref_multigrid(s) : ref_direct_solve(s, s->cfg.ivis >= 1);
    if (rc) return rc;
    ref_compute_velocities(s);
    return 0;
}

/* energy_time_Chebyshev, Chebyshev.f90:113-243 (tracer=1, RK_update=1, equalize=0, uniform grid) */
static int step_chebyshev(ptref_state* s) {
    int nx = s->nx, nz = s->nz;
    int64_t ntr = s->ntr;
    int comp = s->cfg.comp, N = s->cfg.nstage;
    if (!s->u0) return ref_fail(s, PT_ERR_STATE, "RKC2 stepper not set up (chebyshev=1 at create)");
    double dt = stability_RK4(s);
    if (s->status) return s->status;
    s->dt = dt;
    if (s->cfg.equalize) { /* Chebyshev.f90:131-137, after the time step */
        int erc = ptref_equalize(s, -1, NULL);
        if (erc) return erc;
    }
    rfld C0 = ref_fld_alloc(nx, nz, 5);
    rfld T0 = ref_fld_alloc(nx, nz, 3);
    if (comp) copy_fld(&C0, &s->Cnew);
    copy_fld(&T0, &s->Tratio);
    size_t nb = sizeof(double) * (size_t)ntr;
    memcpy(s->Ttr0, s->Ttr, nb);
    memcpy(s->rtr0, s->rtr, nb);
    memcpy(s->str0, s->str, nb);
    int rc = 0;
    /* stage 1 */
    load_tracer_space(s);
    compute_derivatives(s, &s->tsa, s->DERr_t);
    compute_derivatives(s, &s->u, s->DERr_u);
    compute_derivatives(s, &s->w, s->DERr_w);
    double dtstage = s->mewtCheb[1] * dt;
#pragma omp parallel for
    for (int64_t id = 0; id < ntr; id++) {
        double tr = interpolate(s, s->rtr0[id], s->str0[id], s->DERr_u, &s->u);
        double ts = interpolate(s, s->rtr0[id], s->str0[id], s->DERr_w, &s->w);
        double tT = interpolate(s, s->rtr0[id], s->str0[id], s->DERr_t, &s->tsa);
        s->u0[id] = tr;
        s->w0[id] = ts;
        s->dT0[id] = tT;
        s->rtr1[id] = s->rtr0[id] + dtstage * tr;
        s->str1[id] = s->str0[id] + dtstage * ts;
        s->Ttr1[id] = s->Ttr0[id] + dtstage * tT;
        s->rtr2[id] = s->rtr0[id];
        s->str2[id] = s->str0[id];
        s->Ttr2[id] = s->Ttr0[id];
    }
    /* stages 2..nstage */
    for (int j = 2; j <= N; j++) {
        if (comp) copy_fld(&s->Cnew, &C0);
        if ((rc = ref_project(s, s->rtr1, s->str1, s->Ttr1, &T0, 1))) goto done;
        load_tracer_space(s);
        compute_derivatives(s, &s->tsa, s->DERr_t);
        if ((rc = update_velocities(s))) goto done;
        compute_derivatives(s, &s->u, s->DERr_u);
        compute_derivatives(s, &s->w, s->DERr_w);
        dtstage = s->mewtCheb[j] * dt;
        double dtstage2 = s->gtCheb[j] * dt;
        double cj = s->cCheb[j], mj = s->mewCheb[j], vj = s->vCheb[j];
#pragma omp parallel for
        for (int64_t id = 0; id < ntr; id++) {
            double tr = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_u, &s->u);
            double ts = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_w, &s->w);
            double tT = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_t, &s->tsa);
            s->rtr[id] = cj * s->rtr0[id] + mj * s->rtr1[id] + vj * s->rtr2[id] + dtstage * tr + dtstage2 * s->u0[id];
            s->str[id] = cj * s->str0[id] + mj * s->str1[id] + vj * s->str2[id] + dtstage * ts + dtstage2 * s->w0[id];
            s->Ttr[id] = cj * s->Ttr0[id] + mj * s->Ttr1[id] + vj * s->Ttr2[id] + dtstage * tT + dtstage2 * s->dT0[id];
            s->rtr2[id] = s->rtr1[id];
            s->str2[id] = s->str1[id];
            s->Ttr2[id] = s->Ttr1[id];
            s->rtr1[id] = s->rtr[id];
            s->str1[id] = s->str[id];
            s->Ttr1[id] = s->Ttr[id];
        }
    }
    /* wrap-up */
    if (comp) copy_fld(&s->Cnew, &C0);
    if ((rc = ref_project(s, s->rtr, s->str, s->Ttr, &T0, 1))) goto done;
    copy_fld(&s->T, &s->Tratio);
    s->time = s->time + dt;
done:
    free(C0.p);
    free(T0.p);
    return rc;
}

/* energy_time, energy.f90:181-556 (tracer=1, torder=4, RK_update=1, local_time=0) */
int ptref_step(ptref_state* s) {
    if (s->cfg.chebyshev) return step_chebyshev(s);
    int nx = s->nx, nz = s->nz;
    int64_t ntr = s->ntr;
    int comp = s->cfg.comp;
    double dt = stability_RK4(s);
    if (s->status) return s->status;
    s->dt = dt;
    if (s->cfg.equalize) { /* energy.f90:198-204, after the time step */
        int erc = ptref_equalize(s, -1, NULL);
        if (erc) return erc;
    }
    rfld C0 = ref_fld_alloc(nx, nz, 5);
    rfld T0 = ref_fld_alloc(nx, nz, 3);
    if (comp) copy_fld(&C0, &s->Cnew);
    copy_fld(&T0, &s->Tratio);
    size_t nb = sizeof(double) * (size_t)ntr;
    memcpy(s->Ttr0, s->Ttr, nb);
    memcpy(s->rtr0, s->rtr, nb);
    memcpy(s->str0, s->str, nb);
    int rc = 0;
    /* stage 1 */
    load_tracer_space(s);
    compute_derivatives(s, &s->tsa, s->DERr_t);
    compute_derivatives(s, &s->u, s->DERr_u);
    compute_derivatives(s, &s->w, s->DERr_w);
    {
        double dtstage = 0.5 * dt;
#pragma omp parallel for
        for (int64_t id = 0; id < ntr; id++) {
            double tr = interpolate(s, s->rtr0[id], s->str0[id], s->DERr_u, &s->u);
            double ts = interpolate(s, s->rtr0[id], s->str0[id], s->DERr_w, &s->w);
            double tT = interpolate(s, s->rtr0[id], s->str0[id], s->DERr_t, &s->tsa);
            s->rtr[id] = tr;
            s->str[id] = ts;
            s->Ttr[id] = tT;
            s->rtr1[id] = s->rtr0[id] + dtstage * tr;
            s->str1[id] = s->str0[id] + dtstage * ts;
            s->Ttr1[id] = s->Ttr0[id] + dtstage * tT;
        }
    }
    /* stage 2 */
    if ((rc = ref_project(s, s->rtr1, s->str1, s->Ttr1, &T0, 1))) goto done;
    load_tracer_space(s);
    compute_derivatives(s, &s->tsa, s->DERr_t);
    if ((rc = update_velocities(s))) goto done;
    compute_derivatives(s, &s->u, s->DERr_u);
    compute_derivatives(s, &s->w, s->DERr_w);
    {
        double dtstage = 0.5 * dt;
#pragma omp parallel for
        for (int64_t id = 0; id < ntr; id++) {
            double tr = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_u, &s->u);
            double ts = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_w, &s->w);
            s->rtr[id] = s->rtr[id] + 2.0 * tr;
            s->str[id] = s->str[id] + 2.0 * ts;
            double tT = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_t, &s->tsa);
            s->Ttr[id] = s->Ttr[id] + 2.0 * tT;
            s->rtr2[id] = s->rtr0[id] + dtstage * tr;
            s->str2[id] = s->str0[id] + dtstage * ts;
            s->Ttr2[id] = s->Ttr0[id] + dtstage * tT;
        }
    }
    /* stage 3 */
    if (comp) copy_fld(&s->Cnew, &C0);
    if ((rc = ref_project(s, s->rtr2, s->str2, s->Ttr2, &T0, 1))) goto done;
    load_tracer_space(s);
    compute_derivatives(s, &s->tsa, s->DERr_t);
    if ((rc = update_velocities(s))) goto done;
    compute_derivatives(s, &s->u, s->DERr_u);
    compute_derivatives(s, &s->w, s->DERr_w);
    {
        double dtt = dt;
#pragma omp parallel for
        for (int64_t id = 0; id < ntr; id++) {
            double tr = interpolate(s, s->rtr2[id], s->str2[id], s->DERr_u, &s->u);
            s->rtr[id] = s->rtr[id] + 2.0 * tr;
            s->rtr1[id] = s->rtr0[id] + dtt * tr;
            double ts = interpolate(s, s->rtr2[id], s->str2[id], s->DERr_w, &s->w);
            s->str[id] = s->str[id] + 2.0 * ts;
            s->str1[id] = s->str0[id] + dtt * ts;
            double tT = interpolate(s, s->rtr2[id], s->str2[id], s->DERr_t, &s->tsa);
            s->Ttr[id] = s->Ttr[id] + 2.0 * tT;
            s->Ttr1[id] = s->Ttr0[id] + dtt * tT;
        }
    }
    /* stage 4 */
    if (comp) copy_fld(&s->Cnew, &C0);
    if ((rc = ref_project(s, s->rtr1, s->str1, s->Ttr1, &T0, 1))) goto done;
    load_tracer_space(s);
    compute_derivatives(s, &s->tsa, s->DERr_t);
    if ((rc = update_velocities(s))) goto done;
    compute_derivatives(s, &s->u, s->DERr_u);
    compute_derivatives(s, &s->w, s->DERr_w);
    {
        double dto6 = dt / 6.0;
#pragma omp parallel for
        for (int64_t id = 0; id < ntr; id++) {
            double tr = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_u, &s->u);
            s->rtr[id] = s->rtr0[id] + dto6 * (s->rtr[id] + tr);
            double ts = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_w, &s->w);
            s->str[id] = s->str0[id] + dto6 * (s->str[id] + ts);
            double tT = interpolate(s, s->rtr1[id], s->str1[id], s->DERr_t, &s->tsa);
            s->Ttr[id] = s->Ttr0[id] + dto6 * (s->Ttr[id] + tT);
        }
    }
    /* wrap-up */
    if (comp) copy_fld(&s->Cnew, &C0);
    if ((rc = ref_project(s, s->rtr, s->str, s->Ttr, &T0, 1))) goto done;
    copy_fld(&s->T, &s->Tratio);
    s->time = s->time + dt;
done:
    free(C0.p);
    free(T0.p);
    return rc;
}
