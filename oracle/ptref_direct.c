/*
 * ptref_direct.c -- oracle (test infrastructure only): banded LU with partial pivoting and the
 * direct stream-function solve (iterate=0) of the reference's shipped run.
 *
 * The band routines restate the published unblocked LAPACK/BLAS algorithms that the reference
 * links (it does not vendor them): dgbequ.f (row equilibration), dgbtf2.f (band LU with partial
 * pivoting, IDAMAX pivot = first maximum), dgbtrs.f + dtbsv.f (solve).  Storage is LAPACK band
 * storage: A(i,j) at ab[(kl+ku+i-j) + (j-1)*ldab] (0-based row kl+ku+i-j), ldab >= 2kl+ku+1.
 */
#include "ptref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define AB(r, c) ab[((r) - 1) + (size_t)((c) - 1) * (size_t)ldab]

/* dgbequ.f row part: r(i) = 1/max_j |a(i,j)|, clamped to [smlnum, bignum].  ab points at the
 * rows that hold A (A(i,j) at AB(ku+1+i-j, j)).  Returns the first zero row (1-based) or 0. */
int ptref_band_equ(int n, int kl, int ku, const double* ab, int ldab, double* r) {
    const double smlnum = 2.2250738585072014e-308, bignum = 1.0 / smlnum;
    for (int i = 0; i < n; i++) r[i] = 0.0;
    for (int j = 1; j <= n; j++) {
        int i0 = j - ku > 1 ? j - ku : 1, i1 = j + kl < n ? j + kl : n;
        for (int i = i0; i <= i1; i++) {
            double a = fabs(AB(ku + 1 + i - j, j));
            if (a > r[i - 1]) r[i - 1] = a;
        }
    }
    for (int i = 0; i < n; i++)
        if (r[i] == 0.0) return i + 1;
    for (int i = 0; i < n; i++) {
        double v = r[i] > smlnum ? r[i] : smlnum;
        v = v < bignum ? v : bignum;
        r[i] = 1.0 / v;
    }
    return 0;
}

/* dgbtf2.f: returns INFO (0, or the first zero pivot column). */
int ptref_band_lu(int n, int kl, int ku, double* ab, int ldab, int* ipiv) {
    int kv = ku + kl, info = 0;
    for (int j = ku + 2; j <= (kv < n ? kv : n); j++)
        for (int i = kv - j + 2; i <= kl; i++) AB(i, j) = 0.0;
    int ju = 1;
    for (int j = 1; j <= n; j++) {
        if (j + kv <= n)
            for (int i = 1; i <= kl; i++) AB(i, j + kv) = 0.0;
        int km = kl < n - j ? kl : n - j;
        int jp = 1;
        double amax = fabs(AB(kv + 1, j));
        for (int i = 2; i <= km + 1; i++) {
            double a = fabs(AB(kv + i, j));
            if (a > amax) { amax = a; jp = i; }
        }
        ipiv[j - 1] = jp + j - 1;
        if (AB(kv + jp, j) != 0.0) {
            int jue = j + ku + jp - 1 < n ? j + ku + jp - 1 : n;
            if (jue > ju) ju = jue;
            if (jp != 1) {
                size_t a0 = (size_t)(kv + jp - 1) + (size_t)(j - 1) * ldab, b0 = (size_t)kv + (size_t)(j - 1) * ldab;
                for (int t = 0; t <= ju - j; t++) {
                    double tmp = ab[a0 + (size_t)t * (ldab - 1)];
                    ab[a0 + (size_t)t * (ldab - 1)] = ab[b0 + (size_t)t * (ldab - 1)];
                    ab[b0 + (size_t)t * (ldab - 1)] = tmp;
                }
            }
            if (km > 0) {
                double rp = 1.0 / AB(kv + 1, j);
                for (int i = 1; i <= km; i++) AB(kv + 1 + i, j) = AB(kv + 1 + i, j) * rp;
                if (ju > j) {
                    /* dger: A(kv+1.., j+1..) -= x * y', x = AB(kv+2..,j), y = row kv of the band */
                    for (int jj = 1; jj <= ju - j; jj++) {
                        double y = ab[(size_t)(kv - 1) + (size_t)j * ldab + (size_t)(jj - 1) * (ldab - 1)];
                        if (y != 0.0) {
                            double temp = -1.0 * y;
                            size_t a0 = (size_t)kv + (size_t)j * ldab + (size_t)(jj - 1) * (ldab - 1);
                            for (int i = 1; i <= km; i++)
                                ab[a0 + (size_t)(i - 1)] = ab[a0 + (size_t)(i - 1)] + AB(kv + 1 + i, j) * temp;
                        }
                    }
                }
            }
        } else if (info == 0) {
            info = j;
        }
    }
    return info;
}

/* dgbtrs.f (TRANS='N', one right-hand side) with dtbsv.f (upper, no transpose, non-unit).  Every
 * column is updated and every entry divided, zeros included, like the optimized BLAS that the
 * shipped run linked: its snapshot T10000 prints psi = -0 on every wall node that is not a corner
 * (0 divided by a negative pivot).  The reference dtbsv.f/dger.f skip zero entries, which leaves
 * those +0; nonzero results are the same either way. */
int ptref_band_solve(int n, int kl, int ku, const double* ab, int ldab, const int* ipiv, double* b) {
    int kd = ku + kl + 1;
    if (kl > 0)
        for (int j = 1; j <= n - 1; j++) {
            int lm = kl < n - j ? kl : n - j;
            int l = ipiv[j - 1];
            if (l != j) { double t = b[l - 1]; b[l - 1] = b[j - 1]; b[j - 1] = t; }
            double temp = -1.0 * b[j - 1];
            for (int i = 1; i <= lm; i++) b[j + i - 1] = b[j + i - 1] + AB(kd + i, j) * temp;
        }
    int k = kl + ku, kplus1 = k + 1;
    for (int j = n; j >= 1; j--) {
        int l = kplus1 - j;
        b[j - 1] = b[j - 1] / AB(kplus1, j);
        double temp = b[j - 1];
        int i0 = 1 > j - k ? 1 : j - k;
        for (int i = j - 1; i >= i0; i--) b[i - 1] = b[i - 1] - temp * AB(l + i, j);
    }
    return 0;
}
#undef AB

/* visf for the direct path (ivis=0 only: the golden run is isoviscous). */

/* Matrix_element, momentum.f90:495-621 (uniform metrics xr=zs=1, xrr=...=0 kept literally). */
static double matrix_element(ptref_state* s, int i, int k, int ip, int kp, int rsym, int ssym,
                             double visx, double visz, double visxx, double viszz, double visxz,
                             double visv, int* kind) {
    const double xr = 1.0, xrr = 0.0, xrrr = 0.0, xrrrr = 0.0, zs = 1.0, zss = 0.0, zsss = 0.0, zssss = 0.0;
    double dr = s->dr, ds = s->ds;
    double dr2 = dr * dr, ds2 = ds * ds, dr3 = pow(dr, 3.0), ds3 = pow(ds, 3.0), dr4 = pow(dr, 4.0), ds4 = pow(ds, 4.0);
    double drds = dr * ds, drds2 = dr * ds2, dr2ds = dr2 * ds, dr2ds2 = dr2 * ds2;
    double Ss, Sss, Ssss, Sssss, Sr, Srr, Srrr, Srrrr;
    if (i == 0) { Ss = s->D1[k + 3] / ds; Sss = s->D2[k + 3] / ds2; Ssss = s->D3[k + 3] / ds3; Sssss = s->D4[k + 3] / ds4; }
    else { Ss = 0.0; Sss = 0.0; Ssss = 0.0; Sssss = 0.0; }
    if (ssym == 1 && s->cfg.Vbc == 0) { Ss = -Ss; Sss = -Sss; Ssss = -Ssss; Sssss = -Sssss; }
    if (k == 0) { Sr = s->D1[i + 3] / dr; Srr = s->D2[i + 3] / dr2; Srrr = s->D3[i + 3] / dr3; Srrrr = s->D4[i + 3] / dr4; }
    else { Sr = 0.0; Srr = 0.0; Srrr = 0.0; Srrrr = 0.0; }
    if (rsym == 1) { Sr = -Sr; Srr = -Srr; Srrr = -Srrr; Srrrr = -Srrrr; }
    double Sx = Sr / xr;
    double Sxx = (Srr - Sx * xrr) / (xr * xr);
    double Sxxx = (Srrr - 3.0 * Sxx * xr * xrr - Sx * xrrr) / pow(xr, 3.0);
    double Sxxxx = (Srrrr - 6.0 * Sxxx * xrr * (xr * xr) - (3.0 * (xrr * xrr) + 4.0 * xr * xrrr) * Sxx - Sx * xrrrr) / pow(xr, 4.0);
    double Sz = Ss / zs;
    double Szz = (Sss - Sz * zss) / (zs * zs);
    double Szzz = (Ssss - 3.0 * Szz * zs * zss - Sz * zsss) / pow(zs, 3.0);
    double Szzzz = (Sssss - 6.0 * Szzz * zss * (zs * zs) - (3.0 * (zss * zss) + 4.0 * zs * zsss) * Szz - Sz * zssss) / pow(zs, 4.0);
    double Srs = 0, Srss = 0, Srrs = 0, Srrss = 0;
    if (i >= -2 && i <= 2 && k >= -2 && k <= 2) {
        Srs = s->Drs[i + 3][k + 3] / drds;
        Srss = s->Drss[i + 3][k + 3] / drds2;
        Srrs = s->Drrs[i + 3][k + 3] / dr2ds;
        Srrss = s->Drrss[i + 3][k + 3] / dr2ds2;
    } else {
        Srs = 0.0 / drds; Srss = 0.0 / drds2; Srrs = 0.0 / dr2ds; Srrss = 0.0 / dr2ds2;
    }
    if (s->cfg.Vbc == 0) {
        if ((rsym == 1) != (ssym == 1)) { Srs = -Srs; Srss = -Srss; Srrs = -Srrs; Srrss = -Srrss; }
    } else if (rsym == 1) { Srs = -Srs; Srss = -Srss; Srrs = -Srrs; Srrss = -Srrss; }
    double Sxz = Srs / xr / zs;
    double Sxxz = (Srrs - Sxz * zs * xrr) / zs / (xr * xr);
    double Sxzz = (Srss - Sxz * xr * zss) / xr / (zs * zs);
    double Sxxzz = (Srrss - Sxzz * xrr * (zs * zs) - Sxxz * zss * (xr * xr) - Sxz * xrr * zss) / ((xr * zs) * (xr * zs));
    if (ip == 0 || ip == s->nx) { *kind = 1; return Sxx; }
    if (kp == 0 || kp == s->nz) {
        if (s->cfg.Vbc == 0) { *kind = 1; return Szz; }
        *kind = 0;
        return 0.0;
    }
    double t1 = (visxx - viszz) * (Sxx - Szz);
    double t2 = visv * (Sxxxx + Szzzz);
    double t3 = 2.0 * visv * Sxxzz;
    double t4 = 4.0 * visxz * Sxz;
    double t5 = 2.0 * visx * (Sxxx + Sxzz);
    double t6 = 2.0 * visz * (Szzz + Sxxz);
    *kind = 1;
    return t1 + t2 + t3 + t4 + t5 + t6;
}

/* one (i,k) stencil point of build_SF_matrix (momentum.f90:397-470): reflect and accumulate */
static void add_point(ptref_state* s, int i, int k, int ip, int kp, int p, double* MBp, int ldab,
                      int subD, int supD, int* lo, int* hi, const double* vg) {
    int N = s->nz + 1, nx = s->nx, nz = s->nz;
    int rsym = 0, iq = ip + i;
    if (iq < 0) { iq = -iq; rsym = 1; }
    else if (iq > nx) { iq = nx - (iq - nx); rsym = 1; }
    int ssym = 0, kq = kp + k;
    if (kq < 0) { kq = -kq; ssym = 1; }
    else if (kq > nz) { kq = nz - (kq - nz); ssym = 1; }
    int q = N * iq + kq + 1;
    int kind = 0;
    double v = matrix_element(s, i, k, ip, kp, rsym, ssym, vg[0], vg[1], vg[2], vg[3], vg[4], vg[5], &kind);
    if (!kind) return;
    if (MBp == NULL) {
        int diff = q - p;
        if (diff < *lo) *lo = diff;
        else if (diff > *hi) *hi = diff;
        return;
    }
    size_t idx = (size_t)(subD + supD + p - q) + (size_t)(q - 1) * (size_t)ldab;
    MBp[idx] = MBp[idx] + v;
}

static void assemble(ptref_state* s, double* MBp, int ldab, int subD, int supD, int* lo, int* hi) {
    int nx = s->nx, nz = s->nz, N = nz + 1, ngrid = (nx + 1) * (nz + 1);
    for (int p = 1; p <= ngrid; p++) {
        int kp = p - N * ((p - 1) / N) - 1, ip = (p - 1) / N;
        int corner = (ip == 0 && kp == 0) || (ip == nx && kp == 0) || (ip == 0 && kp == nz) || (ip == nx && kp == nz);
        if (corner || (s->cfg.Vbc == 1 && (kp == 0 || kp == nz))) {
            if (MBp) MBp[(size_t)(subD + supD) + (size_t)(p - 1) * (size_t)ldab] = 1.0;
            continue;
        }
        double vg[6] = {0, 0, 0, 0, 0, RF(s->vis, ip, kp)};
        if (MBp && ip > 0 && ip < nx && kp > 0 && kp < nz) {
            const double *D1so = s->D1_so + 1, *D2so = s->D2_so + 1;
            double visr = 0, visrr = 0, viss = 0, visss = 0, visrs = 0;
            for (int j = -1; j <= 1; j++) visr += D1so[j] * RF(s->vis, ip + j, kp);
            visr /= s->dr;
            for (int j = -1; j <= 1; j++) visrr += D2so[j] * RF(s->vis, ip + j, kp);
            visrr /= s->dr2;
            for (int j = -1; j <= 1; j++) viss += D1so[j] * RF(s->vis, ip, kp + j);
            viss /= s->ds;
            for (int j = -1; j <= 1; j++) visss += D2so[j] * RF(s->vis, ip, kp + j);
            visss /= s->ds2;
            for (int k2 = -1; k2 <= 1; k2++)
                for (int i2 = -1; i2 <= 1; i2++) visrs += s->Drs_so[i2 + 1][k2 + 1] * RF(s->vis, ip + i2, kp + k2);
            visrs /= (s->dr * s->ds);
            vg[0] = visr / 1.0;
            vg[1] = viss / 1.0;
            vg[2] = (visrr - vg[0] * 0.0) / 1.0;
            vg[3] = (visss - vg[1] * 0.0) / 1.0;
            vg[4] = visrs / 1.0 / 1.0;
        }
        for (int i = -3; i <= 3; i += 6) add_point(s, i, 0, ip, kp, p, MBp, ldab, subD, supD, lo, hi, vg);
        for (int k = -3; k <= 3; k += 6) add_point(s, 0, k, ip, kp, p, MBp, ldab, subD, supD, lo, hi, vg);
        for (int i = -2; i <= 2; i++)
            for (int k = -2; k <= 2; k++) add_point(s, i, k, ip, kp, p, MBp, ldab, subD, supD, lo, hi, vg);
    }
}

/* build_SF_matrix (momentum.f90:319-492) + solve_SF_equation (636-653) with buoyancy (258-289)
 * and Stream_grid (291-317).  ivis=0 only (the golden run). */
int ref_direct_solve(ptref_state* s, int rebuild) {
    int nx = s->nx, nz = s->nz, N = nz + 1, ngrid = (nx + 1) * (nz + 1);
    if (s->cfg.ivis != 0) return ref_fail(s, PT_ERR_CONFIG, "direct solve restated for ivis=0 only");
    if (s->MB == NULL) {
        int lo = 0, hi = 0;
        assemble(s, NULL, 0, 0, 0, &lo, &hi);
        s->subD = -lo;
        s->supD = hi;
        int ldab = 2 * s->subD + s->supD + 1;
        s->MB = (double*)calloc((size_t)ldab * (size_t)ngrid, sizeof(double));
        s->Bvec = (double*)calloc((size_t)ngrid, sizeof(double));
        s->RowBd = (double*)calloc((size_t)ngrid, sizeof(double));
        s->ipivd = (int*)calloc((size_t)ngrid, sizeof(int));
        rebuild = 1;
    }
    int kl = s->subD, ku = s->supD, ldab = 2 * kl + ku + 1;
    if (rebuild || s->time == 0.0) {
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) RF(s->vis, i, k) = 1.0;
        memset(s->MB, 0, sizeof(double) * (size_t)ldab * (size_t)ngrid);
        assemble(s, s->MB, ldab, kl, ku, NULL, NULL);
        if (ptref_band_equ(ngrid, kl, ku, s->MB + kl, ldab, s->RowBd))
            return ref_fail(s, PT_ERR_SINGULAR_COARSE, "DGBEQU: zero row");
        for (int q = 1; q <= ngrid; q++) {
            int p0 = q - ku > 1 ? q - ku : 1, p1 = q + kl < ngrid ? q + kl : ngrid;
            for (int p = p0; p <= p1; p++) {
                size_t idx = (size_t)(kl + ku + p - q) + (size_t)(q - 1) * (size_t)ldab;
                s->MB[idx] = s->RowBd[p - 1] * s->MB[idx];
            }
        }
        if (ptref_band_lu(ngrid, kl, ku, s->MB, ldab, s->ipivd))
            return ref_fail(s, PT_ERR_SINGULAR_COARSE, "DGBTRF: singular matrix");
    }
    for (int p = 1; p <= ngrid; p++) {
        int kp = p - N * ((p - 1) / N) - 1, ip = (p - 1) / N;
        s->Bvec[p - 1] = 0.0;
        if (ip > 0 && ip < nx && kp > 0 && kp < nz) {
            double Tr = 0.0;
            for (int j = -2; j <= 2; j++) Tr += s->D1[j + 3] * RF(s->Tbuoy, ip + j, kp);
            double Tx = (Tr / s->dr) / 1.0;
            if (s->cfg.comp == 0) s->Bvec[p - 1] = s->cfg.RaT * Tx * s->RowBd[p - 1];
            else {
                double Cr = 0.0;
                for (int j = -2; j <= 2; j++) Cr += s->D1[j + 3] * RF(s->Cbuoy, ip + j, kp);
                double Cx = (Cr / s->dr) / 1.0;
                double dot = 0.0 + s->cfg.RaC * Cx;
                if (s->cfg.RaT != 0.0) s->Bvec[p - 1] = (s->cfg.RaT * Tx - dot) * s->RowBd[p - 1];
                else s->Bvec[p - 1] = (-dot) * s->RowBd[p - 1];
            }
        }
    }
    ptref_band_solve(ngrid, kl, ku, s->MB, ldab, s->ipivd, s->Bvec);
    for (int p = 1; p <= ngrid; p++) {
        int kp = p - N * ((p - 1) / N) - 1, ip = (p - 1) / N;
        RF(s->SF, ip, kp) = s->Bvec[p - 1];
    }
    for (int kp = 0; kp <= nz; kp++)
        for (int ip = 1; ip <= 3; ip++) {
            RF(s->SF, -ip, kp) = -RF(s->SF, ip, kp);
            RF(s->SF, nx + ip, kp) = -RF(s->SF, nx - ip, kp);
        }
    for (int kp = 1; kp <= 3; kp++)
        for (int ip = -3; ip <= nx + 3; ip++) {
            if (s->cfg.Vbc == 0) {
                RF(s->SF, ip, -kp) = -RF(s->SF, ip, kp);
                RF(s->SF, ip, nz + kp) = -RF(s->SF, ip, nz - kp);
            } else {
                RF(s->SF, ip, -kp) = RF(s->SF, ip, kp);
                RF(s->SF, ip, nz + kp) = RF(s->SF, ip, nz - kp);
            }
        }
    return 0;
}
