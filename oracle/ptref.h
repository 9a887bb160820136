/*
 * ptref -- CPU oracle: a plain-C restatement of the ProjecTracer hot path, used ONLY as test
 * infrastructure (the parity tests compare against it) and as the timed CPU baseline ("port").  The product library
 * never links, loads or calls anything in this directory.
 *
 * Every function cites the reference routine it follows (ProjecTracer_Source/<file>:<lines>).
 * Arrays keep the reference's index space: a field f(i,k) with ghost width g lives at
 * p[(i+g) + (k+g)*ld], ld = nx+2g+1, i.e. Fortran column-major with the reference's offsets.
 *
 * Parity pins: the t=0 state of the reference's shipped run (stats.dat row 1, T10000, P10000,
 * stdout KATs) is reproduced by ptref_init_reference() + ptref_solve_psi() with the direct
 * banded solver (see tests/test_oracle_golden.py).  The multigrid solve (iterate=1) has no
 * reference artefact: it is pinned only through the components it shares with the golden path.
 *
 * LAPACK is not vendored by the reference (compile_script.sh:12 links -llapack, version not
 * pinned); DGBEQU/DGBTRF/DGBTRS are restated here from their published unblocked algorithms
 * (LAPACK 3.x dgbequ.f, dgbtf2.f, dgbtrs.f, BLAS dtbsv.f) and cross-checked against scipy's
 * LAPACK in the tests.
 */
#ifndef PTREF_H
#define PTREF_H

#include <stdint.h>
#include <stddef.h>
#include "../include/ptgpu.h"

#define REF_MAXLEV 8

typedef struct {
    double* p;
    int nx, nz, g, ld;
} rfld;

#define RF(f, i, k) ((f).p[((i) + (f).g) + (size_t)((k) + (f).g) * (size_t)(f).ld])

typedef struct ptref_state {
    pt_config cfg;
    int iheattype_boundary; /* 1: comp=1 iheattype=1 boundary heating (the shipped run's start-up only) */
    double klayer, dlayer;  /* the shipped run's initial layer profile (initial_conditions.f90) */
    int nparts;        /* emulated OpenMP thread partitions (sum order of the reference) */
    int iterate;       /* 1 multigrid, 0 direct banded */
    int nx, nz, grids, nsteps;
    int multi[64];     /* multigrid schedule with multi[0]=multi[nsteps], multi[nsteps+1]=multi[1] */
    double dr, ds, dr2, ds2;
    double dr_power[5], ds_power[5], factorial[5];
    /* per-level spacings */
    int nxl[REF_MAXLEV], nzl[REF_MAXLEV];
    double drl[REF_MAXLEV], dsl[REF_MAXLEV], dr2l[REF_MAXLEV], ds2l[REF_MAXLEV], dr3l[REF_MAXLEV],
        ds3l[REF_MAXLEV], dr4l[REF_MAXLEV], ds4l[REF_MAXLEV], drdsl[REF_MAXLEV],
        drds2l[REF_MAXLEV], dr2dsl[REF_MAXLEV], dr2ds2l[REF_MAXLEV];
    /* FD stencils, index offset +3 */
    double D1[7], D2[7], D3[7], D4[7];
    double Dm[5][7];          /* D(1..4, -3:3) */
    double Drs[7][7], Drss[7][7], Drrs[7][7], Drrss[7][7]; /* [i+3][k+3] */
    double D1_so[3], D2_so[3], Drs_so[3][3];               /* [i+1][k+1] */
    /* Fourier bases (energy.f90:730-743) */
    double Tr_base, Trr_base, Trrr_base, Trrrr_base, Trs_base, Trrs_base, Trss_base, Trrss_base;
    double Tr_base_so, Trr_base_so;
    /* eigenvalue_prep per level (uniform grid: constants) */
    double SR[REF_MAXLEV][7], SI[REF_MAXLEV][7]; /* index 1,2,4,5,6 used */
    double dt_vis[REF_MAXLEV];                   /* stability_vis_smoother (uniform) */
    double dts;                                  /* stability_RK4_smoother (uniform) */
    double SM1[7][7], SM2[7][7], SM4[7][7], SM5[7][7], SM6[7][7]; /* [di+3][dk+3] */
    /* RKC1 coefficients (Chebyshev.f90:182-210) */
    double mewtS[64], mewS[64], vS[64], cS[64], bS[64];
    /* RKC2 energy stepper (Chebyshev_prep, Chebyshev.f90:38-80) */
    double cCheb[64], mewCheb[64], vCheb[64], mewtCheb[64], gtCheb[64];
    double* u0; double* w0; double* dT0; /* stage-1 slopes (1:ntr) */
    double RKC1_stability;
    double delta_T, delta_C;
    int kl, ku, ngrid_coarse;
    int subD, supD; /* direct solver bandwidth */
    /* grid */
    double* xg; double* zg; /* index -(6):nx+6 */
    /* fields */
    rfld T, SF, u, w, Tvis, Tbuoy, Tratio, tsa; /* g=3 */
    rfld Cnew, Cvis, Cbuoy, conduct, Textend;   /* g=5 */
    rfld conduct_r, conduct_s;                  /* g=3 */
    rfld vis;                                   /* g=3, stats/direct */
    rfld strain;                                /* g=3 */
    double* DERr_u; double* DERr_w; double* DERr_t; /* (3, 0:nx, -3:nz+3) */
    int32_t* nempty;                            /* (0:nx,0:nz) */
    /* multigrid per level */
    rfld err[REF_MAXLEV], RHS[REF_MAXLEV], res[REF_MAXLEV], dtst[REF_MAXLEV], ratio[REF_MAXLEV];
    rfld visg[REF_MAXLEV], visst[REF_MAXLEV], vx[REF_MAXLEV], vz[REF_MAXLEV], vxx[REF_MAXLEV],
        vzz[REF_MAXLEV], vxz[REF_MAXLEV], vxxpzz[REF_MAXLEV], vxxmzz[REF_MAXLEV], vsm[REF_MAXLEV];
    rfld SFd[10]; /* stream derivative scratch at the level in use */
    rfld S0, S1, S2;
    double res_ref[REF_MAXLEV];
    double residual_mag[64];
    double* Mc; double* Bc; double* RowB; int* ipiv; /* coarse band */
    double* MB; double* Bvec; double* RowBd; int* ipivd; /* direct band */
    int32_t n_eta, n_temp, cycles;
    double eig_fine, resid_ratio;
    /* tracers */
    int64_t ntr;
    double *rtr, *str, *Ttr, *Ctr;
    int32_t* Ttype;       /* discrete tracer types 0/1 (iC_continuous=0), NULL for continuous C */
    int32_t* count_type1; /* count_type(1, 0:nx, 0:nz) of the last discrete-type projection */
    double *rtr0, *str0, *Ttr0, *rtr1, *str1, *Ttr1, *rtr2, *str2, *Ttr2;
    double time, dt;
    double mass; int kent; int have_mass;
    int smooth_vis;
    int64_t eq_calls; /* equalisations so far (the call index of the next one) */
    int32_t eq_done;  /* equalisations that moved tracers (nequalize) */
    int status;
    char err_msg[256];
} ptref_state;

/* lifecycle */
ptref_state* ptref_create(const pt_config* cfg, int iterate, int nparts);
void ptref_destroy(ptref_state* s);
const char* ptref_error(ptref_state* s);

/* start-up of the shipped run (restart=0): initial_temperature + initialize_tracers with the
 * mzran stream partitioned over `nthreads_rng` OpenMP threads; tpc tracers per cell corner;
 * initial_temp=-1 / initial_comp=-1 work-area formulas with klayer, dlayer, f0=0. */
int ptref_init_reference(ptref_state* s, int tpc, int nthreads_rng, double klayer, double dlayer,
                         int iheattype_boundary);

/* restart=1 path (grid.f90:46-104 + main.f90:204-210). */
int ptref_load_restart(ptref_state* s, const double* xg, const double* zg, const double* T,
                       const double* Cnew, const double* SF, const double* rtr, const double* str,
                       const double* Ctr, const double* Ttr);

/* discrete tracer types (iC_continuous=0, ntype=1): the types 0/1 of the tracers, set before
 * ptref_load_restart; the projection is then tracers_to_corners_OG */
int ptref_set_types(ptref_state* s, const int32_t* Ttype);

int ptref_solve_psi(ptref_state* s);   /* update_velocities */
int ptref_step(ptref_state* s);        /* energy_time */
int ptref_stats(ptref_state* s, pt_stats_row* out);
int ptref_project(ptref_state* s, const double* r, const double* sv, const double* Tt,
                  const double* T0field, int smooth); /* tracers_to_corners */

/* tracer equalisation (equalize_tracers, composition.f90:266-763) as the GPU library defines it:
 * counter-based random numbers instead of mzran, see ptref_equalize.c.  call_index counts the
 * calls of the run (the random numbers of call n are independent of every other call's); a negative
 * call_index takes the next one of this state. */
int ptref_equalize(ptref_state* s, int64_t call_index, pt_equalize_info* info);

/* field exchange in the Fortran layout used by ptgpu.h */
int ptref_get_field(ptref_state* s, int id, void* out);
int ptref_set_field(ptref_state* s, int id, const void* in);
int ptref_get_scalar(ptref_state* s, const char* name, double* out);

/* component entry points used by kernel-level parity tests */
int ptref_compute_derivatives(ptref_state* s, const double* f, double* DERr); /* f g=3 */
double ptref_interpolate(ptref_state* s, double r, double sv, const double* DERr, const double* f);
int ptref_load_tracer_space(ptref_state* s, double* tsa_out);
int ptref_velocities(ptref_state* s);
int ptref_smoother_T(ptref_state* s, const double* Tin);
int ptref_band_lu(int n, int kl, int ku, double* ab, int ldab, int* ipiv);
int ptref_band_solve(int n, int kl, int ku, const double* ab, int ldab, const int* ipiv, double* b);
int ptref_band_equ(int n, int kl, int ku, const double* ab, int ldab, double* r);

/* internal helpers shared between translation units */
void ref_enforceBCs(ptref_state* s, rfld* f);
void ref_enforceBCs_comp(ptref_state* s, rfld* f);
void ref_smoother_time_T(ptref_state* s, const rfld* Tin);
void ref_smoother_time(ptref_state* s);
void ref_load_conductivity(ptref_state* s);
void ref_enforceBCs_stream(ptref_state* s, int level, rfld* f);
int ref_multigrid(ptref_state* s);
int ref_direct_solve(ptref_state* s, int rebuild);
void ref_compute_velocities(ptref_state* s);
int ref_project(ptref_state* s, const double* r, const double* sv, const double* Tt,
                const rfld* T0, int smooth);
void ref_extendT(ptref_state* s, const rfld* T0);
void ref_compute_derivatives(ptref_state* s, const rfld* f, double* DERr);
double ref_interpolate(ptref_state* s, double r, double sv, const double* DERr, const rfld* f);
double ref_heating(ptref_state* s, int i, int k);
int ref_coarse_bandwidth(ptref_state* s);
rfld ref_fld_alloc(int nx, int nz, int g);
int ref_fail(ptref_state* s, int code, const char* msg);



#endif
