/*
 * ptgpu.h -- C ABI of the GB300 timestep engine for ProjecTracer-style tracer convection.
 *
 * The reference (Fortran 90 + OpenMP) has no plugin interface: its hot-path subroutines take no
 * arguments and exchange data through the module globals of basics.f90 and arrays.f90.  The entry
 * points below replace the bodies of those subroutines; a Fortran driver binds them with
 * iso_c_binding.  Each declaration cites the reference routine it replaces (file:line inside
 * ProjecTracer_Source/).
 *
 * Conventions
 *  - Every function returns 0 (PT_OK) or a negative PT_ERR_* code; pt_last_error() describes it.
 *  - Grid arrays cross the boundary in Fortran column-major order (x index i fastest) with the
 *    reference's ghost extents; the pointer is the element at the lowest ghost index.  The extents
 *    of each array are given by pt_field_extent().
 *  - Tracer arrays are plain FP64 vectors of length ntr in tracer-ID order.
 *  - The library owns all device memory; no caller pointer is retained after a call returns.
 *  - One context per process; call from one host thread.
 */
#ifndef PTGPU_H
#define PTGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_OK 0
#define PT_ERR_CONFIG (-1)               /* unsupported or inconsistent configuration */
#define PT_ERR_TRACER_OUT_OF_DOMAIN (-2) /* composition.f90:1007-1010 ("Tracer advected outside of domain") */
#define PT_ERR_MG_DIVERGED (-3)          /* iterative_solver.f90:438-447 (residual > 1e10 x reference) */
#define PT_ERR_MG_MAX_CYCLES (-4)        /* iterative_solver.f90:325-334 (too many multigrid cycles) */
#define PT_ERR_SINGULAR_COARSE (-5)      /* DGBTRF INFO>0 on the coarsest grid (unchecked in the reference) */
#define PT_ERR_CUDA (-6)                 /* a CUDA runtime call failed */
#define PT_ERR_STATE (-7)                /* call out of order (e.g. pt_step before pt_upload_state) */
#define PT_ERR_ITER_CAP (-8)             /* a data-dependent smoother loop hit its iteration cap */
#define PT_ERR_ARG (-9)                  /* bad argument (null pointer, size, field id) */
#define PT_ERR_NOT_FINITE (-10)          /* NaN/Inf detected in a residual */

/* Precision of the stream-function solve (an extension; not in the reference). */
#define PT_PREC_FP64 0  /* plain FP64 multigrid: the reference algorithm on the GPU */
#define PT_PREC_MIXED 1 /* FP32 smoothing and transfers, FP64 residual and defect correction, FP64 coarse LU
                          and FP64 coarse solve; FP64 tracer positions and RK update, with the velocities
                          interpolated from FP32 tables; integer fixed-point (2^-28) projection sums */

/* Coarse-level initial guess inside a multigrid cycle.  The reference never resets
 * error(:,:,2:grids) (zeroed once, main.f90:229), so each coarse visit starts from the previous
 * coarse correction; PT_MG_CORRECTION starts each descent from zero (textbook correction scheme),
 * which converges in fewer cycles and keeps converging where the reference's variant stalls. */
#define PT_MG_REFERENCE 0
#define PT_MG_CORRECTION 1

/* Level schedule of the solve: PT_CYCLE_REFERENCE the reference's table for the level count (a
 * W-type cycle, multigrid_setup in multigrid_cycle.f90:1-99), PT_CYCLE_V one descent and one
 * ascent (no reference counterpart). */
#define PT_CYCLE_REFERENCE 0
#define PT_CYCLE_V 1

/* Initial-guess mode of the stream-function solve (an extension; not in the reference). */
#define PT_GUESS_PREVIOUS 0 /* previous psi (the reference's warm start, iterative_solver.f90:134) */
#define PT_GUESS_ZERO 1
#define PT_GUESS_UNET 2
/* Linear extrapolation in time from the last two converged psi at distinct solve times (no
 * reference counterpart): inside an RK4 step the stage solves at t+dt/2 and t+dt start from
 * 2 psi(latest) - psi(earlier) scaled to the stage time; solves at the time of the latest psi
 * start from it, as PT_GUESS_PREVIOUS does. */
#define PT_GUESS_EXTRAPOLATE 3

/*
 * Run configuration: the &inputs, &Rayleigh_numbers, &heating_conductivity and &viscosity namelist
 * values on the hot path (basics.f90:54-66), plus Tbot_iso/Ttop_iso (basics.f90:352-353; the
 * reference only sets them in initial_temperature, so a restart run must pass them explicitly) and
 * the &gpu extension group.  Supported subset: order=4, uniform grid (gridX=gridZ=0), Database=2,
 * ntype<=1 with continuous C (iC_continuous=1), temperature tracers (tracer=1), RK4 (torder=4) with
 * RK_update=1, multigrid with the RKC1 smoother (iterate=1, MG=1, RKC1=1, splitting=0), Newtonian
 * viscosity (non_Newtonian=0, plastic=0), constant internal heating (iheattype=0), CFL=0 or 1.
 */
typedef struct pt_config {
    /* grid (&inputs) */
    int32_t nx, nz;      /* cells in x and z; nodes are (nx+1)*(nz+1) */
    int32_t order;       /* must be 4 */
    int32_t grids;       /* max multigrid levels (2..6); optimize_grid may lower it */
    int32_t mingrid;     /* min coarse size for optimize_grid */
    int32_t Nmulti;      /* RKC1 passes per level visit */
    int32_t vis_iter;    /* Richardson passes before restricting viscosity */
    int32_t max_cycles;  /* multigrid cycle cap */
    int32_t nstageS;     /* RKC1 stages */
    int32_t comp;        /* 0 or 1: composition tracers */
    int32_t Tbot;        /* 0 isothermal, 1 insulating bottom */
    int32_t Vbc;         /* 0 free-slip, 1 rigid top/bottom */
    int32_t ivis;        /* 0 isoviscous, 1 eta(T,z), 2 eta(T,C,z) */
    int32_t iheattype;   /* must be 0 */
    int32_t precision;   /* PT_PREC_* (&gpu group) */
    int32_t guess_mode;  /* PT_GUESS_* (&gpu group) */
    int64_t ntr;         /* number of tracers */
    double aspect;
    double tolerance;      /* multigrid residual ratio target */
    double eig_ratio;      /* (kept for namelist fidelity; unused with RKC1) */
    double dampingS, c_2, c_1;
    double courant, courantT, courantC, courant_stream;
    double RaT, RaC;       /* RaC(1) */
    double H, Htype;       /* H and Htype(1) */
    double conduct_factor; /* conduct_factor(1) */
    double visP, visT, delta_visT, eig_ratio_min, visC, delta_visC;
    double Tbot_iso, Ttop_iso;
    double dent;           /* reference height for the entrainment statistic */
    int32_t mg_scheme;     /* PT_MG_* (&gpu group) */
    int32_t CFL;           /* &inputs CFL: 1 = velocity terms in the advective eigenvalue and
                              dt <= 2/eigD_max (energy.f90:809, 859-866) */
    int32_t mg_cycle;      /* PT_CYCLE_*: level schedule of the mixed-precision solve (&gpu group) */
    int32_t nstageC;       /* RKC1 stages on levels 2..grids of the mixed-precision V-cycle; 0 = nstageS
                              (&gpu group; the FP64 path always uses nstageS) */
    int32_t discrete_types; /* 1: tracers carry an integer type 0/1 instead of a continuous C
                              (iC_continuous=0, ntype=1, bilinear shape_function=1: the projection of
                              tracers_to_corners_OG, composition.f90:1090-1276); 0: continuous C */
    int32_t reference_rounding; /* FP64 precision only (&gpu group).  0: the RKC1 stages and residuals
                              form their stencil sums exactly in integer arithmetic and the coarsest
                              grid is solved through the explicit inverse of its LU (fast, and at
                              least as accurate as the reference's FP64 sums).  1: the reference's
                              FP64 operations in its order (stream_derivatives/stream_space,
                              iterative_solver.f90:890-1073; DGBTRS substitutions), no fused
                              multiply-adds, so that results follow the CPU reference to its own
                              rounding over many steps; slower */
    int32_t direct;        /* &inputs iterate=0: the psi solve is the direct banded solve of
                              build_SF_matrix/solve_SF_equation (momentum.f90:319-653): assembly,
                              row equilibration and band LU once (the operator of an isoviscous run
                              does not change), then per solve the banded substitutions.  FP64,
                              ivis=0 only; the substitutions keep a window of the right-hand side
                              and a ring of band columns (band width 3 (nz+1)) in one CTA's
                              shared memory (227 KB), which bounds nz at about 1,150 (pt_init
                              fails with PT_ERR_CONFIG past it).  0: multigrid (iterate=1, MG=1) */
    int32_t chebyshev;     /* &inputs Chebyshev=1: the energy step is the nstage-stage RKC2 Chebyshev
                              method of energy_time_Chebyshev (Chebyshev.f90:113-243) with the RK2
                              time step (torder=2, energy.f90:787-793); 0: RK4 (energy_time).  FP64
                              precision only */
    int32_t nstage;        /* RKC2 stages (2..60) */
    double damping, aRK2;  /* RKC2 damping and the free parameter b1 = aRK2/omega1 (Chebyshev.f90:55) */
    int32_t krylov;        /* mixed precision only (&gpu group).  0: each cycle adds its correction to
                              psi (defect correction).  m in 1..8: the cycle is the preconditioner of
                              a flexible GCR iteration that keeps the last m search directions
                              (restarted after m); same convergence test */
    int32_t equalize;      /* &inputs equalize=1: tracer equalisation (equalize_tracers, composition.f90:
                              266-763) at the start of every pt_step, as energy_time does
                              (energy.f90:198-204); needs discrete types (comp=1) or comp=0 */
    int32_t tpc;           /* &inputs tpc: tracers per cell corner (the comp=0 target count) */
    int32_t pad2_;
    double dist_factor;    /* &inputs dist_factor: dist_r = dist_factor dr, dist_s = dist_factor ds */
    double Cinit;          /* Cinit(1): the average composition at time 0 (basics.f90:461), which sets the
                              ideal tracer count per type, Nideal(1) = nint(Cinit ntr); < 0: taken from
                              the state at the first equalisation */
    uint64_t eq_seed;      /* seed of the equalisation's counter-based random numbers */
} pt_config;

/* Field identifiers for pt_set_field / pt_get_field / pt_field_extent. */
enum pt_field_id {
    PT_F_T = 0,       /* T(-3:nx+3,-3:nz+3)         grid temperature            arrays.f90:649 */
    PT_F_TRATIO = 1,  /* Tratio(-3:nx+3,-3:nz+3)    projected tracer T          arrays.f90:656 */
    PT_F_TVIS = 2,    /* Tvis(-3:nx+3,-3:nz+3)      smoothed T for viscosity    arrays.f90:655 */
    PT_F_TBUOY = 3,   /* Tbuoy(-3:nx+3,-3:nz+3)     T for buoyancy              arrays.f90:655 */
    PT_F_CNEW = 4,    /* Cnew(1,-5:nx+5,-5:nz+5)    projected composition       arrays.f90:658 */
    PT_F_CVIS = 5,    /* Cvis(1,-5:nx+5,-5:nz+5)                                arrays.f90:655 */
    PT_F_CBUOY = 6,   /* Cbuoy(1,-5:nx+5,-5:nz+5)                               arrays.f90:655 */
    PT_F_SF = 7,      /* SF(-3:nx+3,-3:nz+3)        stream function psi         arrays.f90:649 */
    PT_F_U = 8,       /* u(-3:nx+3,-3:nz+3)                                     arrays.f90:649 */
    PT_F_W = 9,       /* w(-3:nx+3,-3:nz+3)                                     arrays.f90:649 */
    PT_F_VIS = 10,    /* vis_grid(-3:nx+3,-3:nz+3,1) smoothed viscosity (get only) arrays.f90:665 */
    PT_F_NEMPTY = 11, /* nempty(0:nx,0:nz) int32 tracer count per dual cell (get only) */
    PT_F_RHS = 12,    /* RHS(1:nx-1,1:nz-1,1) buoyancy (get only)               arrays.f90:662 */
    PT_F_COUNT_TYPE = 13, /* count_type(1,0:nx,0:nz) int32 tracers of type 1 per dual cell (get only;
                             discrete types)                                   composition.f90:1141,1173 */
    PT_F_TRACER_R = 20, /* rtr(1:ntr) */
    PT_F_TRACER_S = 21, /* str(1:ntr) */
    PT_F_TRACER_T = 22, /* Ttr(1:ntr) */
    PT_F_TRACER_C = 23, /* Ctr(1:ntr) (with discrete types: the type as 0.0 / 1.0) */
    PT_F_TRACER_TYPE = 24 /* Ttype(1:ntr) int32, 0 or 1 (discrete types only)     basics.f90:110 */
};

/* Per-step solver telemetry (logged by the reference to stdout at iterative_solver.f90:197,338). */
typedef struct pt_solve_info {
    int32_t cycles;       /* multigrid cycles (FP64) or total inner cycles (mixed) */
    int32_t refinements;  /* defect-correction passes (mixed), 0 for FP64 */
    int32_t n_eta;        /* viscosity-smoother passes on level 1 (smoother.f90:521) */
    int32_t n_temp;       /* temperature-smoother iterations of the last projection (smoother.f90:654) */
    double resid_ratio;   /* final mean|r| / mean|RHS| on level 1 (FP64) */
    double eig_fine;      /* min eigenvalue ratio on level 1 (smoother.f90:520) */
    double ms;            /* device time of the solve in milliseconds */
} pt_solve_info;

/* Columns of stats.dat (basics.f90:427-428) for comp=1 / tracer=1, ntype=1. */
typedef struct pt_stats {
    double time, Tavg, vrms, Nu, Nu_bot, RaT_avg, mobility, strain_max, q1, q2, q3, q4;
    int32_t empty_cells, tracer_min, tracer_max, pad;
    double Cavg, entrainment;
} pt_stats_row;

/* Replaces the start-up part of main.f90:168-230 that sizes and allocates the arrays
 * (compute_basics basics.f90:204-333, storage basics.f90:70-202, multigrid_setup
 * multigrid_cycle.f90:1-99, FD_coefficients main.f90:499-642, derivative_eigenvalues
 * energy.f90:632-744, eigenvalue_prep iterative_solver.f90:1232-1362, Chebyshev_prep_stream
 * Chebyshev.f90:82-110).  Allocates all device buffers. */
int pt_init(const pt_config* cfg);

/* Releases everything pt_init allocated. */
int pt_finalize(void);

/* Text for the last non-zero return code of this thread. */
const char* pt_last_error(void);

/* Multigrid levels chosen by optimize_grid (iterative_solver.f90:1-61) after pt_init. */
int pt_grids(void);

/* Extents of a field: lo/hi index in x and z (for tracer fields, lo_x=1, hi_x=ntr, z unused).
 * Element size in bytes is returned in *elem_bytes (8, or 4 for PT_F_NEMPTY). */
int pt_field_extent(int field, int32_t* lo_x, int32_t* hi_x, int32_t* lo_z, int32_t* hi_z,
                    int32_t* elem_bytes);

/* Copy a host array in (Fortran layout as in pt_field_extent) / out of the device state. */
int pt_set_field(int field, const void* host);
int pt_get_field(int field, void* host);

/* Restart read (grid.f90:46-104 with restart=1, add_layer=0) plus the post-read steps of
 * main.f90:204-210: host arrays in the layout of the Trestart / restart_tracers records
 * (xg,zg,T,Cnew,SF and rtr,str,Ctr,Ttr).  Applies the T, psi and C boundary conditions, projects
 * the tracers (tracers_to_corners without smoothing), then runs smoother_time_T(T), smoother_time
 * and load_conductivity_array.  xg/zg are checked against the uniform grid.  Sets time=0.
 * Ttype: the tracer types 0/1 (restart_tracers with iC_continuous=0) when cfg.discrete_types is
 * 1, in which case Ctr may be NULL; must be NULL otherwise. */
int pt_upload_state(const double* xg, const double* zg, const double* T, const double* Cnew,
                    const double* SF, const double* rtr, const double* str, const double* Ctr,
                    const double* Ttr, const int32_t* Ttype);

/* Download of the restart records written by print_restart (main.f90:457-496); any pointer may
 * be NULL.  Ttype: the tracer types (discrete types only). */
int pt_download_state(double* T, double* Cnew, double* SF, double* rtr, double* str, double* Ctr,
                      double* Ttr, int32_t* Ttype);

/* Velocity solve at the top of a time step (main.f90:246-259): multigrid
 * (iterative_solver.f90:124-341) then compute_velocities (momentum.f90:655-710).
 * info may be NULL. */
int pt_solve_psi(pt_solve_info* info);

/* One call of energy_time (energy.f90:181-556): RK4 over the tracers with the velocity
 * re-solved at stages 2-4 (RK_update=1) and the tracer->grid projection after each stage.
 * Advances time by dt.  dt_out and info may be NULL; info accumulates the three inner solves. */
int pt_step(double* dt_out, pt_solve_info* info);

/* stats (basics.f90:363-462) on the current state: the stats.dat columns. */
int pt_stats(pt_stats_row* out);

/* tracers_to_corners (composition.f90:923-1087) on the current tracer state, with the given
 * empty-corner fallback field T0 (Fortran layout of PT_F_T; NULL = current Tratio) and
 * smoothing on/off (smooth_vis, basics.f90:315). */
int pt_tracers_to_corners(const double* T0, int smooth_vis);

/* pt_tracers_to_corners without any device allocation (no counterpart in the reference).  It is
 * for callers that cannot call cudaMalloc: a host program that hands all free device memory to its
 * own pool allocator at start-up, where any further allocation fails or fragments the pool, or one
 * that projects while other streams are busy, where cudaMalloc/cudaFree can synchronise the device
 * and stall them.  The sort and partial-sum scratch lives in one file-scope device
 * array of the library (about 12 MB) whose address pt_init resolves once per device, so no
 * symbol lookup happens inside a stream capture; calls on a thread with no prior pt_init on the
 * current device resolve it themselves and must not be made during a capture.  Limits: at most
 * PT_NOALLOC_MAX_TRACERS tracers and PT_NOALLOC_MAX_NODES grid nodes ((nx+1)*(nz+1)); larger
 * states return PT_ERR_ARG.  The scratch is shared: overlapping calls (other threads or
 * streams, or another engine on the same device) race on it and must be serialised by the
 * caller.  Results are identical to pt_tracers_to_corners. */
#define PT_NOALLOC_MAX_TRACERS 524288
#define PT_NOALLOC_MAX_NODES 33153
int pt_tracers_to_corners_noalloc(const double* T0, int smooth_vis);

/* Output and restart files of the current state, written asynchronously: the device-to-host copies
 * are queued in order after the work that produced the state (later calls may start at once and do
 * not change what is written), then a host thread formats and writes the files.  pt_io_wait waits
 * for that thread and returns its status; every writer and reader waits for the previous one.
 * pt_write_snapshot: snapshots (main.f90:377-424), the files T<10000+fcount> (x, z, T, SF, u, w,
 *   2 vis strain, vis, T_vis, nempty and, with composition, C and C_vis per node, i outer, edit
 *   descriptors G14.5E3 and I6) and P<10000+fcount> (lateral averages of T, strain rate and
 *   stress per row) in directory dir.
 * pt_write_restart: print_restart (main.f90:457-496), the records Trestart (xg, zg, T, [Cnew], SF)
 *   and restart_tracers (rtr, str, [Ctr or Ttype], Ttr) in gfortran's sequential unformatted form
 *   (4-byte length markers; records longer than 2^31-9 bytes split into sub-records).
 * pt_read_restart: the restart read (grid.f90:55-104) of those two files from dir, then
 *   pt_upload_state. */
/* Tracer equalisation (equalize_tracers, composition.f90:266-763): tracers from nodes with more
 * than their type's target count (donors; near-wall tracers of edge nodes first) are moved to the
 * nodes that lack the most (one per node and pass, the poorest level first), jittered around the
 * node, take the node's majority type and the temperature interpolated from Tratio; then the
 * projection (smooth_vis=0).  The reference's shuffles and lottery order (mzran per OpenMP thread)
 * are replaced by a counter-based hash of (eq_seed, call, tracer or node): the result does not
 * depend on the tracer order or the thread count.  The columns of the reference's equalize.dat
 * line are returned in info (nullable).  pt_step calls it first when cfg.equalize = 1.  A rich node
 * holding more than 8192 tracers is refused with PT_ERR_ARG (ranking its donors costs tracers x
 * donors on one thread). */
typedef struct pt_equalize_info {
    int32_t tpc_type[2];     /* target tracers per node, type 0 / type 1 */
    int32_t minexcess[2];    /* after the moves (composition.f90:738-745) */
    int64_t deficit;         /* sum of the negative excesses after the moves */
    int64_t moved;           /* tracers moved (sum index_save) */
    int64_t nfree;           /* donors found */
    int64_t count_type[2];   /* tracers per type after the moves (the reference's count_display) */
    int32_t passes, nequalize; /* lottery passes of this call; equalisations that moved tracers so far */
} pt_equalize_info;
int pt_equalize_tracers(pt_equalize_info* info);

int pt_write_snapshot(const char* dir, int fcount);
int pt_write_restart(const char* dir);
int pt_read_restart(const char* dir);
int pt_io_wait(void);

/* Current simulation time and the RK4 time step of stability_RK4 (energy.f90:756-810). */
int pt_time(double* time, double* dt);

/* Chooses the initial guess of the next solves (PT_GUESS_*).  weights_path names a U-Net
 * weight file for PT_GUESS_UNET (NULL otherwise). */
int pt_set_guess_mode(int mode, const char* weights_path);

/* Device time of each phase summed since pt_init, in milliseconds (8 entries): [0] tracer RK
 * stages, [1] projections, [2] psi solves, [3] multigrid setup (viscosity pipeline, coarse
 * matrix and factorisation), [4] level-1 part of the multigrid cycles, [5] coarser levels of the
 * cycles, [6] grid work of a step (smoothers, conductivity, derivative tables, time step), [7]
 * coarse matrix, banded LU and explicit inverse (included in [3]). */
int pt_phase_times(double* ms8);

#ifdef __cplusplus
}
#endif
#endif /* PTGPU_H */
