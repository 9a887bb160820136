// pt_fields.cu -- fine-grid field kernels: boundary conditions, T smoother, conductivity, the
// Lagrangian T rate, derivative tables, velocities, dt and statistics.
//
// Compiled with --fmad=false: every operation rounds exactly as the reference's Fortran
// expression (same association order), so these kernels reproduce the CPU oracle bit for bit and
// the data-dependent smoother loop counts match.  All are HBM-bound stencils or reductions.
#include <cmath>
#include <cstring>

#include "pt_consts.cuh"

namespace pt {

int upload_consts_fields(const Engine& E) { return upload_tu_consts(E); }

__device__ __forceinline__ double heating_at(const double* Cvis, const Geo g, int i, int k) {
    // compute_heating, energy.f90:19-40 (iheattype=0)
    if (cK.comp == 0) return cK.H;
    double cv = Cvis[g.at(i, k)];
    double h = cK.H * (1.0 - (0.0 + cv));
    return cK.Htype * cv + h;
}

// enforceBCs (energy.f90:558-592) when dst==src and span=3; extendT (595-630) when span=5 and
// src is the field to extend.  Every ghost value is built from interior values of src.
__global__ void k_bc_T(double* dst, const double* src, const double* Cvis, Geo g, int span, int full) {
    const int nx = cK.nx, nz = cK.nz;
    int w = nx + 2 * span + 1;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    int tot = w * (nz + 2 * span + 1);
    if (idx >= tot) return;
    int i = idx % w - span, k = idx / w - span;
    bool interior = (i >= 0 && i <= nx && k >= 1 && k <= nz - 1);
    if (interior) {
        if (full) dst[g.at(i, k)] = src[g.at(i, k)];
        return;
    }
    int mi = mirror_idx(i, nx);
    double v;
    if (k == 0) {
        if (cK.Tbot == 0) v = cK.Tbot_iso;
        else v = src[g.at(mi, 0)];
    } else if (k == nz) {
        v = cK.Ttop_iso;
    } else if (k < 0) {
        double Tm = src[g.at(mi, -k)];
        if (cK.Tbot == 0) {
            double h = heating_at(Cvis, g, i, 0);
            v = 2.0 * cK.Tbot_iso + cK.two_over_D20 * h * cK.ds2 - Tm;
        } else {
            v = Tm;
        }
    } else if (k > nz) {
        double Tm = src[g.at(mi, 2 * nz - k)];
        double h = heating_at(Cvis, g, i, nz);
        v = 2.0 * cK.Ttop_iso + cK.two_over_D20 * h * cK.ds2 - Tm;
    } else {
        v = src[g.at(mi, k)];
    }
    dst[g.at(i, k)] = v;
}

int enforce_bcs_T(Engine& E, double* f) {
    int tot = (E.K.nx + 7) * (E.K.nz + 7);
    PT_COUNT(), k_bc_T<<<nblk(tot, 256), 256, 0, E.st>>>(f, f, E.Cvis, E.g1, 3, 0);
    CKL("k_bc_T");
    return 0;
}

// enforceBCs_comp (composition.f90:1279-1292).  The reference interleaves the column and row
// ghost copies inside one loop over the ghost distance, so a corner ghost (-j,-i) with j>i takes
// the value that (-j,i) held before the call.  Phase 1 writes the row ghosts (reading the old
// column ghosts where the loop order implies it); phase 2 then writes the column ghosts.
__global__ void k_bc_C_rows(double* C, Geo g) {
    const int nx = cK.nx, nz = cK.nz;
    int w = nx + 11;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= w * 10) return;
    int c = idx % w - 5, r = idx / w;  // r 0..9: rows -5..-1 then nz+1..nz+5
    int i = (r < 5) ? (5 - r) : (r - 4);  // ghost distance 1..5
    int ksrc = (r < 5) ? i : nz - i;
    int kdst = (r < 5) ? -i : nz + i;
    double v;
    if (c >= 0 && c <= nx) {
        v = C[g.at(c, ksrc)];
    } else {
        int j = c < 0 ? -c : c - nx;  // column ghost distance
        int cm = c < 0 ? j : nx - j;
        v = (j <= i) ? C[g.at(cm, ksrc)] : C[g.at(c, ksrc)];
    }
    C[g.at(c, kdst)] = v;
}
__global__ void k_bc_C_cols(double* C, Geo g) {
    const int nx = cK.nx, nz = cK.nz;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 10 * (nz + 1)) return;
    int k = idx / 10, q = idx % 10;
    int j = (q < 5) ? q + 1 : q - 4;
    if (q < 5) C[g.at(-j, k)] = C[g.at(j, k)];
    else C[g.at(nx + j, k)] = C[g.at(nx - j, k)];
}

int enforce_bcs_C(Engine& E, double* f) {
    PT_COUNT(), k_bc_C_rows<<<nblk((E.K.nx + 11) * 10, 256), 256, 0, E.st>>>(f, E.g1);
    PT_COUNT(), k_bc_C_cols<<<nblk(10 * (E.K.nz + 1), 256), 256, 0, E.st>>>(f, E.g1);
    CKL("bc_C");
    return 0;
}

// smoothness (smoother.f90:75-95): max over the 5 forward neighbour jumps, as an atomic max on
// the bit pattern (non-negative doubles order like their bits), so the result is exact.
__global__ void k_smoothness(const double* T, Geo g, unsigned long long* out) {
    const int nx = cK.nx, nz = cK.nz;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int k = blockIdx.y + 1;
    double a = 0.0;
    if (i <= nx - 1 && k <= nz - 1) {
        double c = T[g.at(i, k)];
        double a1 = fabs(T[g.at(i, k - 1)] - c), a2 = fabs(T[g.at(i + 1, k - 1)] - c);
        double a3 = fabs(T[g.at(i + 1, k)] - c), a4 = fabs(T[g.at(i, k + 1)] - c);
        double a5 = fabs(T[g.at(i + 1, k + 1)] - c);
        a = fmax(fmax(fmax(a1, a2), fmax(a3, a4)), a5);
    }
    for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0 && a > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(a));
}

int reduce_max_smoothness(Engine& E, const double* f, double* out) {
    unsigned long long* d = (unsigned long long*)E.dscal;
    CK(cudaMemsetAsync(d, 0, 8, E.st));
    dim3 grid(nblk(E.K.nx, 128), E.K.nz - 1);
    PT_COUNT(), k_smoothness<<<grid, 128, 0, E.st>>>(f, E.g1, d);
    CKL("k_smoothness");
    CK(cudaMemcpyAsync(E.hscal, d, 8, cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    *out = E.hscal[0];
    return 0;
}

// one explicit diffusion pass of smoother_time_T (smoother.f90:659-668; smoother_space 121-139)
__global__ void k_smooth_T(double* out, const double* in, Geo g, double dts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i > cK.nx) return;
    double trr = 0.0, tss = 0.0;
#pragma unroll
    for (int j = -2; j <= 2; j++) trr = trr + cK.D2[3 + j] * in[g.at(i + j, k)];
#pragma unroll
    for (int j = -2; j <= 2; j++) tss = tss + cK.D2[3 + j] * in[g.at(i, k + j)];
    trr = qdiv(trr, cK.dr2, cK.inv_dr2);
    tss = qdiv(tss, cK.ds2, cK.inv_ds2);
    out[g.at(i, k)] = in[g.at(i, k)] + dts * (trr + tss);
}

int copy_field(Engine& E, double* dst, const double* src) {
    CK(cudaMemcpyAsync(dst, src, E.g1.elems() * sizeof(double), cudaMemcpyDeviceToDevice, E.st));
    return 0;
}

int smoother_time_T(Engine& E, const double* Tin) {
    int rc;
    if ((rc = copy_field(E, E.Tvis, Tin))) return rc;
    if ((rc = copy_field(E, E.Tbuoy, Tin))) return rc;
    E.n_temp = 0;
    if (E.cfg.RaT == 0.0 || E.cfg.ivis == 0) return 0;
    const double dts = E.dts * E.cfg.courantT;
    const int cap = 200000;
    for (int n = 0;; n++) {
        double diff;
        if ((rc = reduce_max_smoothness(E, E.Tvis, &diff))) return rc;
        if (diff < E.delta_T) { E.n_temp = n; return 0; }
        if (n >= cap) return fail(PT_ERR_ITER_CAP, "temperature smoother exceeded its iteration cap");
        dim3 grid(nblk(E.K.nx + 1, 128), E.K.nz + 1);
        PT_COUNT(), k_smooth_T<<<grid, 128, 0, E.st>>>(E.scratch, E.Tvis, E.g1, dts);
        CKL("k_smooth_T");
        std::swap(E.scratch, E.Tvis);
        if ((rc = enforce_bcs_T(E, E.Tvis))) return rc;
    }
}

// smoother_time (smoother.f90:582-636): with delta_C > 1 the C field (values in [0,1]) already
// satisfies the smoothness test, so Cvis = Cbuoy = Cnew (other settings are rejected in pt_init).
int smoother_time_C(Engine& E) {
    int rc;
    if ((rc = copy_field(E, E.Cvis, E.Cnew))) return rc;
    return copy_field(E, E.Cbuoy, E.Cnew);
}

// load_conductivity_array (energy.f90:59-86)
__global__ void k_cond(double* cd, const double* Cvis, Geo g) {
    const int nx = cK.nx, nz = cK.nz;
    int w = nx + 11;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= w * (nz + 11)) return;
    int i = idx % w - 5, k = idx / w - 5;
    int mi = mirror_idx(i, nx), mk = mirror_idx(k, nz);
    double v = 1.0;
    if (cK.comp == 1) v = v + Cvis[g.at(mi, mk)] * (cK.conduct_factor - 1.0);
    cd[g.at(i, k)] = v;
}
__global__ void k_cond_grad(double* cr, double* cs, const double* cd, Geo g) {
    const int nx = cK.nx, nz = cK.nz;
    int w = nx + 7;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= w * (nz + 7)) return;
    int i = idx % w - 3, k = idx / w - 3;
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int j = -2; j <= 2; j++) a = a + cK.D1[3 + j] * cd[g.at(i + j, k)];
#pragma unroll
    for (int j = -2; j <= 2; j++) b = b + cK.D1[3 + j] * cd[g.at(i, k + j)];
    cr[g.at(i, k)] = qdiv(a, cK.dr, cK.inv_dr);
    cs[g.at(i, k)] = qdiv(b, cK.ds, cK.inv_ds);
}

int load_conductivity(Engine& E) {
    int tot = (E.K.nx + 11) * (E.K.nz + 11);
    PT_COUNT(), k_cond<<<nblk(tot, 256), 256, 0, E.st>>>(E.cond, E.Cvis, E.g1);
    tot = (E.K.nx + 7) * (E.K.nz + 7);
    PT_COUNT(), k_cond_grad<<<nblk(tot, 256), 256, 0, E.st>>>(E.cond_r, E.cond_s, E.cond, E.g1);
    CKL("conductivity");
    return 0;
}

// tracer_space_uniform over (-3:nx+3,-3:nz+3), energy.f90:135-151
__global__ void k_tracer_space(double* tsa, const double* X, const double* cd, const double* cr,
                               const double* cs, const double* Cvis, Geo g) {
    const int nx = cK.nx, nz = cK.nz;
    int w = nx + 7;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= w * (nz + 7)) return;
    int i = idx % w - 3, k = idx / w - 3;
    double Tx = 0, Tz = 0, Txx = 0, Tzz = 0;
#pragma unroll
    for (int j = -2; j <= 2; j++) Tx = Tx + cK.D1[3 + j] * X[g.at(i + j, k)];
    Tx = qdiv(Tx, cK.dr, cK.inv_dr);
#pragma unroll
    for (int j = -2; j <= 2; j++) Tz = Tz + cK.D1[3 + j] * X[g.at(i, k + j)];
    Tz = qdiv(Tz, cK.ds, cK.inv_ds);
#pragma unroll
    for (int j = -2; j <= 2; j++) Txx = Txx + cK.D2[3 + j] * X[g.at(i + j, k)];
    Txx = qdiv(Txx, cK.dr2, cK.inv_dr2);
#pragma unroll
    for (int j = -2; j <= 2; j++) Tzz = Tzz + cK.D2[3 + j] * X[g.at(i, k + j)];
    Tzz = qdiv(Tzz, cK.ds2, cK.inv_ds2);
    double h = heating_at(Cvis, g, i, k);
    size_t a = g.at(i, k);
    tsa[a] = cd[a] * (Txx + Tzz) + (cr[a] * Tx + cs[a] * Tz) + h;
}

// extendT (energy.f90:595-630): Tratio with its span-5 ghosts into Text
int extend_T(Engine& E) {
    const int tot = (E.K.nx + 11) * (E.K.nz + 11);
    PT_COUNT(), k_bc_T<<<nblk(tot, 256), 256, 0, E.st>>>(E.Text, E.Tratio, E.Cvis, E.g1, 5, 1);
    CKL("extendT");
    return 0;
}

int load_tracer_space(Engine& E) {
    int tot = (E.K.nx + 11) * (E.K.nz + 11);
    PT_COUNT(), k_bc_T<<<nblk(tot, 256), 256, 0, E.st>>>(E.Text, E.Tratio, E.Cvis, E.g1, 5, 1);
    tot = (E.K.nx + 7) * (E.K.nz + 7);
    PT_COUNT(), k_tracer_space<<<nblk(tot, 256), 256, 0, E.st>>>(E.tsa, E.Text, E.cond, E.cond_r, E.cond_s, E.Cvis, E.g1);
    CKL("tracer_space");
    return 0;
}

// compute_derivatives (composition.f90:1457-1478): x-derivatives of order 1..3 at (0:nx,-3:nz+3)
__global__ void k_derivs(double* d1, double* d2, double* d3, const double* f, Geo g) {
    const int nx = cK.nx, nz = cK.nz;
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = (int)blockIdx.y - 3;
    if (i > nx || k > nz + 3) return;
    double v[7];
#pragma unroll
    for (int j = 0; j < 7; j++) v[j] = f[g.at(i + j - 3, k)];
    double a = 0, b = 0, c = 0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        a = a + cK.Dm[1][j] * v[j];
        b = b + cK.Dm[2][j] * v[j];
        c = c + cK.Dm[3][j] * v[j];
    }
    size_t o = g.at(i, k);
    d1[o] = qdiv(a, cK.dr_pow[1], cK.inv_dr_pow[1]);
    d2[o] = qdiv(b, cK.dr_pow[2], cK.inv_dr_pow[2]);
    d3[o] = qdiv(c, cK.dr_pow[3], cK.inv_dr_pow[3]);
}

int compute_derivatives(Engine& E, const double* f, int which) {
    dim3 grid(nblk(E.K.nx + 1, 128), E.K.nz + 7);
    PT_COUNT(), k_derivs<<<grid, 128, 0, E.st>>>(E.der[which][0], E.der[which][1], E.der[which][2], f, E.g1);
    CKL("k_derivs");
    return 0;
}

// compute_velocities (momentum.f90:655-710) with velocityBCs (composition.f90:1295-1325)
__global__ void k_vel_interior(double* u, double* w, const double* SF, Geo g) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i > cK.nx) return;
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int j = -2; j <= 2; j++) a = a + cK.D1[3 + j] * SF[g.at(i + j, k)];
#pragma unroll
    for (int j = -2; j <= 2; j++) b = b + cK.D1[3 + j] * SF[g.at(i, k + j)];
    w[g.at(i, k)] = qdiv(-a, cK.dr, cK.inv_dr);
    u[g.at(i, k)] = qdiv(b, cK.ds, cK.inv_ds);
}
__global__ void k_vel_bc(double* u, double* w, Geo g) {
    const int nx = cK.nx, nz = cK.nz;
    int W = nx + 7;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * (nz + 7)) return;
    int i = idx % W - 3, k = idx / W - 3;
    bool xin = (i >= 0 && i <= nx), zin = (k >= 0 && k <= nz);
    int mi = mirror_idx(i, nx), mk = mirror_idx(k, nz);
    // w: symmetric across the side walls, antisymmetric across top/bottom, zero on rows 0 and nz
    if (!(xin && zin) || k == 0 || k == nz) {
        double v = (k == 0 || k == nz) ? 0.0 : w[g.at(mi, mk)] * (zin ? 1.0 : -1.0);
        if (!zin && (mk == 0 || mk == nz)) v = 0.0;
        w[g.at(i, k)] = v;
    }
    // u: antisymmetric across the side walls, symmetric (free slip) or antisymmetric (rigid)
    // across top/bottom, zero on columns 0 and nx (and rows 0, nz when rigid)
    if (!(xin && zin) || i == 0 || i == nx || (cK.Vbc == 1 && (k == 0 || k == nz))) {
        double v;
        if (i == 0 || i == nx || mi == 0 || mi == nx) v = 0.0;
        else if (cK.Vbc == 1 && (k == 0 || k == nz || mk == 0 || mk == nz)) v = 0.0;
        else {
            double sx = xin ? 1.0 : -1.0, sz = zin ? 1.0 : (cK.Vbc == 0 ? 1.0 : -1.0);
            v = sx * (sz * u[g.at(mi, mk)]);
        }
        u[g.at(i, k)] = v;
    }
}

int compute_velocities(Engine& E) {
    dim3 grid(nblk(E.K.nx + 1, 128), E.K.nz + 1);
    PT_COUNT(), k_vel_interior<<<grid, 128, 0, E.st>>>(E.u, E.w, E.SF, E.g1);
    int tot = (E.K.nx + 7) * (E.K.nz + 7);
    PT_COUNT(), k_vel_bc<<<nblk(tot, 256), 256, 0, E.st>>>(E.u, E.w, E.g1);
    CKL("velocities");
    return 0;
}

// stability_RK4 (energy.f90:756-810): eigenvalue maxima over the nodes
// eigA/eigD of energy.f90:850-875 on the uniform grid (xr = zs = 1, xrr = zss = 0); u, w are
// nullptr unless CFL = 1
__global__ void k_eig_max(const double* cd, const double* cr, const double* cs, const double* u, const double* w,
                          Geo g, double Tr_max, double Ts_max, double Trr_max, double Tss_max,
                          unsigned long long* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    double eA = 0.0, eD = 0.0;
    if (i <= cK.nx) {
        size_t a = g.at(i, k);
        double c = cd[a];
        const double uu = u ? u[a] : 0.0, ww = w ? w[a] : 0.0;
        eA = fabs(-c * 0.0 / 1.0 - uu / 1.0 + cr[a] / 1.0) * Tr_max + fabs(-c * 0.0 / 1.0 - ww / 1.0 + cs[a] / 1.0) * Ts_max;
        eD = c * (fabs(Trr_max / 1.0) + fabs(Tss_max / 1.0));
    }
    for (int o = 16; o > 0; o >>= 1) {
        eA = fmax(eA, __shfl_xor_sync(0xffffffffu, eA, o));
        eD = fmax(eD, __shfl_xor_sync(0xffffffffu, eD, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (eA > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(eA));
        if (eD > 0.0) atomicMax(out + 1, (unsigned long long)__double_as_longlong(eD));
    }
}

int stability_dt(Engine& E, double* dt) {
    PhaseTimer tm(E, PH_GRID);
    const Consts& K = E.K;
    double Ts_max = E.Tr_base / K.ds, Tr_max = E.Tr_base / K.dr;
    double Tss_max = -E.Trr_base / K.ds2, Trr_max = -E.Trr_base / K.dr2;
    unsigned long long* d = (unsigned long long*)E.dscal;
    CK(cudaMemsetAsync(d, 0, 16, E.st));
    dim3 grid(nblk(K.nx + 1, 128), K.nz + 1);
    PT_COUNT(), k_eig_max<<<grid, 128, 0, E.st>>>(E.cond, E.cond_r, E.cond_s, E.cfg.CFL == 1 ? E.u : nullptr,
                                                   E.cfg.CFL == 1 ? E.w : nullptr, E.g1, Tr_max, Ts_max, Trr_max,
                                                   Tss_max, d);
    CKL("k_eig_max");
    CK(cudaMemcpyAsync(E.hscal, d, 16, cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    double eA = E.hscal[0], eD = E.hscal[1];
    double dtA = 2.8 / eA, dtD = 2.8 / eD;
    if (E.cfg.chebyshev) {  // torder=2 (energy.f90:787-793), which the RKC2 stepper requires
        if (eA >= eD)
            return fail(PT_ERR_CONFIG, "Advective Eigenvalues Exceed Diffusive Eigenvalues -- this does not work for RK2");
        dtA = 1.0 / eA;
        dtD = 2.0 / eD;
    }
    double v = (eA == 0.0) ? dtD : 1.0 / (1.0 / dtA + 1.0 / dtD);
    *dt = E.cfg.courant * v;
    if (E.cfg.CFL == 1 && 2.0 / eD < *dt) *dt = 2.0 / eD;  // energy.f90:809
    return 0;
}

// --- statistics (basics.f90:363-462), summed in the reference's serial order --------------
// per row k: trapezoid integrals in x of T, C, u^2+w^2, RaT/conduct/vis (integrate1Dx 494-515)
__global__ void k_stats_rows(const double* T, const double* C, const double* u, const double* w,
                             const double* cd, const double* vis, Geo g, double* rows) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = cK.nx, nz = cK.nz;
    if (k > nz) return;
    double fT = 0, fC = 0, fV = 0, fR = 0;
    double pT = T[g.at(0, k)], pC = C[g.at(0, k)];
    double pu = u[g.at(0, k)], pw = w[g.at(0, k)];
    double pV = pu * pu + pw * pw, pR = cK.RaT / cd[g.at(0, k)] / vis[g.at(0, k)];
    for (int i = 0; i < nx; i++) {
        double qT = T[g.at(i + 1, k)], qC = C[g.at(i + 1, k)];
        double qu = u[g.at(i + 1, k)], qw = w[g.at(i + 1, k)];
        double qV = qu * qu + qw * qw, qR = cK.RaT / cd[g.at(i + 1, k)] / vis[g.at(i + 1, k)];
        fT = fT + 0.5 * (pT * 1.0 + qT * 1.0) * cK.dr;
        fC = fC + 0.5 * (pC * 1.0 + qC * 1.0) * cK.dr;
        fV = fV + 0.5 * (pV * 1.0 + qV * 1.0) * cK.dr;
        fR = fR + 0.5 * (pR * 1.0 + qR * 1.0) * cK.dr;
        pT = qT; pC = qC; pV = qV; pR = qR;
    }
    rows[4 * k + 0] = fT;
    rows[4 * k + 1] = fC;
    rows[4 * k + 2] = fV;
    rows[4 * k + 3] = fR;
}

// single-thread tail: z integrals, fluxes, strain maximum, tracer counts
__global__ void k_stats_tail(const double* rows, const double* T, const double* u, const double* w,
                             const double* cd, const double* E1, const int32_t* nempty, Geo g,
                             double* out, int kent, int direct) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int nx = cK.nx, nz = cK.nz;
    double I[4] = {0, 0, 0, 0}, Ient = 0.0;
    for (int k = 0; k < nz; k++)
        for (int q = 0; q < 4; q++) I[q] = I[q] + 0.5 * (rows[4 * k + q] * 1.0 + rows[4 * (k + 1) + q] * 1.0) * cK.ds;
    for (int k = kent; k < nz; k++) Ient = Ient + 0.5 * (rows[4 * k + 1] * 1.0 + rows[4 * (k + 1) + 1] * 1.0) * cK.ds;
    // surface / bottom fluxes
    double Nu_top = 0.0, Tb = 0.0, Nu_b = 0.0, mob = 0.0;
    double pst = 0, psb = 0, pT0 = 0, pm = 0;
    for (int i = 0; i <= nx; i++) {
        double t1 = 0.0, t2 = 0.0;
        for (int j = -2; j <= 2; j++) t1 = t1 + cK.D1[3 + j] * T[g.at(i, nz + j)];
        for (int j = -2; j <= 2; j++) t2 = t2 + cK.D1[3 + j] * T[g.at(i, j)];
        double tzs = qdiv(t1, cK.ds, cK.inv_ds), tzb = qdiv(t2, cK.ds, cK.inv_ds);  // (the reference's / 1.0 is exact)
        double st = -(cd[g.at(i, nz)] * tzs), sb = -(cd[g.at(i, 0)] * tzb), t0 = T[g.at(i, 0)];
        double uu = u[g.at(i, nz)], ww = w[g.at(i, nz)];
        double m = uu * uu + ww * ww;
        if (i > 0) {
            Nu_top = Nu_top + 0.5 * (pst * 1.0 + st * 1.0) * cK.dr;
            Nu_b = Nu_b + 0.5 * (psb * 1.0 + sb * 1.0) * cK.dr;
            Tb = Tb + 0.5 * (pT0 * 1.0 + t0 * 1.0) * cK.dr;
            mob = mob + 0.5 * (pm * 1.0 + m * 1.0) * cK.dr;
        }
        pst = st; psb = sb; pT0 = t0; pm = m;
    }
    // strain-rate invariant on the top row: from the multigrid's psi (compute_strain_rate_invariant_direct,
    // momentum.f90:73-92), or for the direct solve from the velocities (compute_strain_rate_invariant,
    // momentum.f90:1-34)
    double smax = -1.0 / 0.0;
    for (int i = 0; i <= nx && direct; i++) {
        const int k = nz;
        double ur = 0, us = 0, wr = 0, ws = 0;
        for (int j = -2; j <= 2; j++) ur = ur + cK.D1[3 + j] * u[g.at(i + j, k)];
        ur = ur / cK.dr;
        for (int j = -2; j <= 2; j++) us = us + cK.D1[3 + j] * u[g.at(i, k + j)];
        us = us / cK.ds;
        for (int j = -2; j <= 2; j++) wr = wr + cK.D1[3 + j] * w[g.at(i + j, k)];
        wr = wr / cK.dr;
        for (int j = -2; j <= 2; j++) ws = ws + cK.D1[3 + j] * w[g.at(i, k + j)];
        ws = ws / cK.ds;
        const double ux = ur / 1.0, uz = us / 1.0, wx = wr / 1.0, wz = ws / 1.0;
        const double s = pow(0.5 * (2.0 * (ux * ux + wz * wz) + (uz + wx) * (uz + wx)), 0.5);
        if (s > smax) smax = s;
    }
    for (int i = 0; i <= nx && !direct; i++) {
        int k = nz;
        double Sxx = 0, Szz = 0, Sxz = 0;
        for (int j = -2; j <= 2; j++) Sxx = Sxx + cK.D2[3 + j] * E1[g.at(i + j, k)];
        Sxx = qdiv(Sxx, cK.dr2, cK.inv_dr2);
        for (int j = -2; j <= 2; j++) Szz = Szz + cK.D2[3 + j] * E1[g.at(i, k + j)];
        Szz = qdiv(Szz, cK.ds2, cK.inv_ds2);
        for (int k2 = -2; k2 <= 2; k2++)
            for (int i2 = -2; i2 <= 2; i2++) Sxz = Sxz + cK.Drs[i2 + 2][k2 + 2] * E1[g.at(i + i2, k + k2)];
        Sxz = Sxz / (cK.dr * cK.ds);
        double s = pow(2.0 * (Sxz * Sxz) + 0.5 * ((Szz - Sxx) * (Szz - Sxx)), 0.5);
        if (s > smax) smax = s;
    }
    int empty = 0, tmin = 0x7fffffff, tmax = -0x7fffffff;
    for (int q = 0; q < (nx + 1) * (nz + 1); q++) {
        int n = nempty[q];
        if (n == 0) empty++;
        if (n < tmin) tmin = n;
        if (n > tmax) tmax = n;
    }
    double q1, q2, q3, q4, d;
    d = 0; for (int j = -2; j <= 2; j++) d = d + cK.D1[3 + j] * T[g.at(0, nz + j)];
    q1 = -qdiv(cd[g.at(0, nz)] * d, cK.ds, cK.inv_ds);
    d = 0; for (int j = -2; j <= 2; j++) d = d + cK.D1[3 + j] * T[g.at(nx, nz + j)];
    q2 = -qdiv(cd[g.at(nx, nz)] * d, cK.ds, cK.inv_ds);
    d = 0; for (int j = -2; j <= 2; j++) d = d + cK.D1[3 + j] * T[g.at(nx, j)];
    q3 = -qdiv(cd[g.at(nx, 0)] * d, cK.ds, cK.inv_ds);
    d = 0; for (int j = -2; j <= 2; j++) d = d + cK.D1[3 + j] * T[g.at(0, j)];
    q4 = -qdiv(cd[g.at(0, 0)] * d, cK.ds, cK.inv_ds);
    out[0] = I[0];   // integral of T
    out[1] = I[1];   // integral of C
    out[2] = I[2];   // integral of u^2+w^2
    out[3] = I[3];   // integral of RaT/conduct/vis
    out[4] = Ient;
    out[5] = Nu_top; out[6] = Tb; out[7] = Nu_b; out[8] = mob; out[9] = smax;
    out[10] = q1; out[11] = q2; out[12] = q3; out[13] = q4;
    out[14] = (double)empty; out[15] = (double)tmin; out[16] = (double)tmax;
}

int stats(Engine& E, pt_stats_row* o) {
    double* rows = E.red;
    int nz = E.K.nz;
    const double* C = E.cfg.comp ? E.Cnew : E.T;
    PT_COUNT(), k_stats_rows<<<nblk(nz + 1, 64), 64, 0, E.st>>>(E.T, C, E.u, E.w, E.cond, E.vis[1], E.g1, rows);
    double* out = rows + 4 * (nz + 1) + 8;
    PT_COUNT(), k_stats_tail<<<1, 32, 0, E.st>>>(rows, E.T, E.u, E.w, E.cond, E.err[1], E.nempty, E.g1, out, E.kent,
                                                  E.cfg.direct);
    CKL("stats");
    CK(cudaMemcpyAsync(E.hscal, out, 17 * sizeof(double), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    const double* h = E.hscal;
    const double a = E.cfg.aspect;
    std::memset(o, 0, sizeof *o);
    o->time = E.time;
    o->Tavg = h[0] / a;
    o->RaT_avg = h[3] / a;
    o->vrms = std::pow(h[2] / a, 0.5);
    o->mobility = std::pow(h[8] / a, 0.5) / o->vrms;
    o->Nu = h[5] / h[6];
    o->Nu_bot = h[7] / a;
    o->strain_max = h[9];
    o->q1 = h[10]; o->q2 = h[11]; o->q3 = h[12]; o->q4 = h[13];
    o->empty_cells = (int32_t)h[14];
    o->tracer_min = (int32_t)h[15];
    o->tracer_max = (int32_t)h[16];
    if (E.cfg.comp == 1) {
        o->Cavg = h[1] / a;
        if (!E.have_mass) { E.mass = o->Cavg; E.have_mass = 1; }
        o->entrainment = h[4] / a / E.mass;
    }
    return 0;
}

// --- deterministic sum of |f| over the interior (1..nx-1, 1..nz-1) of a level array ----------
// pass 1: one block per row, fixed strided order + fixed tree; pass 2: one block over the rows.
template <typename R>
__global__ void k_rowsum_abs(const R* f, int nx, int pitch, double* part) {
    __shared__ double sh[256];
    int k = blockIdx.x + 1;
    double a = 0.0;
    for (int i = 1 + threadIdx.x; i <= nx - 1; i += blockDim.x) a += fabs((double)f[(size_t)(i + GH) + (size_t)(k + GH) * pitch]);
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_sum_parts(const double* part, int n, double* out) {
    __shared__ double sh[1024];
    double a = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) a += part[q];
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

template <typename R>
static int sum_abs_interior(Engine& E, const R* f, int nx, int nz, int pitch, double* dout) {
    PT_COUNT(), k_rowsum_abs<R><<<nz - 1, 256, 0, E.st>>>(f, nx, pitch, E.red);
    PT_COUNT(), k_sum_parts<<<1, 1024, 0, E.st>>>(E.red, nz - 1, dout);
    CKL("reduce_sum_abs");
    return 0;
}
int reduce_sum_abs_interior(Engine& E, const double* f, int nx, int nz, int pitch, double* dout) {
    return sum_abs_interior(E, f, nx, nz, pitch, dout);
}
int reduce_sum_abs_interior(Engine& E, const float* f, int nx, int nz, int pitch, double* dout) {
    return sum_abs_interior(E, f, nx, nz, pitch, dout);
}

}  // namespace pt
