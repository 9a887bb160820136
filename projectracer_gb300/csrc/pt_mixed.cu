// pt_mixed.cu -- mixed-precision stream-function solve (no reference counterpart): FP32
// multigrid cycles on the correction inside FP64 defect correction.
//
//   x = psi (FP64 warm start)
//   repeat:  r = RHS - A x (FP64);  FP32 RKC1 smoothing of A e = r on level 1 from e = 0
//            (increment form, see k_rkc_first_f);  x += e;  r = RHS - A x (FP64)
//            stop when mean|r| / mean|RHS| <= tolerance: the reference's test, taken at the same
//            point as in the FP64 cycle (after the level-1 smoothing), on the FP64 residual
//            the rest of the reference's level schedule on a correction that restarts from zero
//            on every descent (correction scheme), FP32 restriction/prolongation, the coarsest
//            level through the FP64 banded LU;  x += P e_2 (FP64)
// The viscosity pipeline and the coarse LU factors are the FP64 ones (mg_setup_solve); the
// coefficient fields are rounded to FP32 once per solve.  Residuals that feed a coarser level use
// FP64 arithmetic on the FP32 correction: for smooth modes the biharmonic stencil cancels by many
// orders of magnitude on the fine levels.  Each iteration is two captured CUDA graphs.
#include <cmath>
#include <cstdlib>
#include <utility>

#include "pt_consts.cuh"
#include "pt_exact.cuh"

namespace pt {

// Programmatic dependent launch: every kernel of the mixed cycle starts by waiting for its
// predecessor grid (griddepcontrol.wait returns once that grid has completed and its writes are
// visible; it is a no-op for a kernel launched without the attribute) and then lets its own
// successor be scheduled.  The successor's launch latency hides behind this kernel's run, which
// matters on the coarse levels where each stage kernel lasts a couple of microseconds.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
static int launch_pdl(const char* what, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                      Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PT_COUNT();
    return cuda_check(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...), what);
}

// Per-level stencils with the grid spacing folded in (FP32 and FP64 copies): no division and no
// FP64->FP32 conversion in the kernels (both run on the FP64 pipe of this part).
//   Sxx = sum x2[j] S(i+j-2), Sxxx = sum x3[j] S(i+j-3), Sxxxx = sum x4[j] S(i+j-3), same in z;
//   cross terms: d1_kk = sum_ii D1[ii] S(i+ii,k+kk), d2_kk = sum_ii D2[ii] S(i+ii,k+kk), then
//   Sxz = sum o_xz[kk] d1_kk, Sxzz = sum o_xzz[kk] d1_kk, Sxxz = sum o_xxz[kk] d2_kk,
//   Sxxzz = sum o_xxzz[kk] d2_kk  (the reference's stream_derivatives, folded)
template <typename T>
struct Stencil {
    T x2[5], x3[7], x4[7], z2[5], z3[7], z4[7], i1[5], i2[5], o_xz[5], o_xzz[5], o_xxz[5], o_xxzz[5];
};
static __constant__ Stencil<float> cSF[PT_MAXLEV];
static __constant__ Stencil<double> cSD[PT_MAXLEV];

template <typename T>
static void make_stencil(const Engine& E, int l, Stencil<T>& c) {
    const Consts& K = E.K;
    const LevConst& L = E.L[l];
    for (int j = 0; j < 5; j++) {
        c.x2[j] = (T)(K.D2[j + 1] / L.dr2);
        c.z2[j] = (T)(K.D2[j + 1] / L.ds2);
        c.i1[j] = (T)K.D1[j + 1];
        c.i2[j] = (T)K.D2[j + 1];
        c.o_xz[j] = (T)(K.D1[j + 1] / L.drds);
        c.o_xzz[j] = (T)(K.D2[j + 1] / L.drds2);
        c.o_xxz[j] = (T)(K.D1[j + 1] / L.dr2ds);
        c.o_xxzz[j] = (T)(K.D2[j + 1] / L.dr2ds2);
    }
    for (int j = 0; j < 7; j++) {
        c.x3[j] = (T)(K.D3[j] / L.dr3);
        c.x4[j] = (T)(K.D4[j] / L.dr4);
        c.z3[j] = (T)(K.D3[j] / L.ds3);
        c.z4[j] = (T)(K.D4[j] / L.ds4);
    }
}

int upload_consts_mixed(const Engine& E) {
    if (int rc = upload_tu_consts(E)) return rc;
    Stencil<float> sf[PT_MAXLEV] = {};
    Stencil<double> sd[PT_MAXLEV] = {};
    for (int l = 1; l <= E.grids && l < PT_MAXLEV; l++) {
        make_stencil(E, l, sf[l]);
        make_stencil(E, l, sd[l]);
    }
    CK(cudaMemcpyToSymbol(cSF, sf, sizeof sf));
    CK(cudaMemcpyToSymbol(cSD, sd, sizeof sd));
    return 0;
}

struct FOp {
    const float *vis, *vx, *vz, *vxz, *vxxmzz, *rhs, *dtst;
};
struct DOp {
    const double *vis, *vx, *vz, *vxz, *vxxmzz, *rhs;
};


__device__ __forceinline__ void store_ghosts_f(float* out, Geo g, int i, int k, int nx, int nz, float v, float sz) {
    int xs[3], zs[3];
    float xf[3], zf[3];
    int nxp = 0, nzp = 0;
    xs[nxp] = i; xf[nxp++] = 1.0f;
    if (i <= 3) { xs[nxp] = -i; xf[nxp++] = -1.0f; }
    if (i >= nx - 3) { xs[nxp] = 2 * nx - i; xf[nxp++] = -1.0f; }
    zs[nzp] = k; zf[nzp++] = 1.0f;
    if (k <= 3) { zs[nzp] = -k; zf[nzp++] = sz; }
    if (k >= nz - 3) { zs[nzp] = 2 * nz - k; zf[nzp++] = sz; }
    for (int a = 0; a < nxp; a++)
        for (int b = 0; b < nzp; b++) out[g.at(xs[a], zs[b])] = (xf[a] * zf[b]) * v;
}

template <typename T>
__device__ __forceinline__ const Stencil<T>& stencil(int l);
template <>
__device__ __forceinline__ const Stencil<float>& stencil<float>(int l) { return cSF[l]; }
template <>
__device__ __forceinline__ const Stencil<double>& stencil<double>(int l) { return cSD[l]; }

// A S (no right-hand side) at a node, in arithmetic T with the folded stencils of level l
// (FP32: the smoother stages; FP64: residuals); ld(dx, dz) returns S at offset (dx, dz) from the
// node (global memory or values held in registers: the same operations in the same order either
// way), o is the node's index into the coefficient fields
template <typename T, typename Ld, typename Op>
__device__ __forceinline__ T apply_A_ld(const Ld& ld, int l, const Op& op, size_t o, int ivis) {
    const Stencil<T>& C = stencil<T>(l);
    T sx[7], sz[7];
#pragma unroll
    for (int j = 0; j < 7; j++) {
        sx[j] = (T)ld(j - 3, 0);
        sz[j] = (T)ld(0, j - 3);
    }
    T Sxx = 0, Sxxx = 0, Sxxxx = 0, Szz = 0, Szzz = 0, Szzzz = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) { Sxx += C.x2[j] * sx[j + 1]; Szz += C.z2[j] * sz[j + 1]; }
#pragma unroll
    for (int j = 0; j < 7; j++) {
        Sxxx += C.x3[j] * sx[j]; Sxxxx += C.x4[j] * sx[j];
        Szzz += C.z3[j] * sz[j]; Szzzz += C.z4[j] * sz[j];
    }
    T Sxz = 0, Sxxz = 0, Sxzz = 0, Sxxzz = 0;
#pragma unroll
    for (int kk = 0; kk < 5; kk++) {
        T d1 = 0, d2 = 0;
#pragma unroll
        for (int ii = 0; ii < 5; ii++) {
            T v = (kk == 2) ? sx[ii + 1] : (T)ld(ii - 2, kk - 2);
            d1 += C.i1[ii] * v;
            d2 += C.i2[ii] * v;
        }
        Sxz += C.o_xz[kk] * d1;
        Sxzz += C.o_xzz[kk] * d1;
        Sxxz += C.o_xxz[kk] * d2;
        Sxxzz += C.o_xxzz[kk] * d2;
    }
    T r = (T)op.vis[o] * (Sxxxx + Szzzz + (T)2 * Sxxzz);
    if (ivis != 0)
        r += (T)op.vxxmzz[o] * (Sxx - Szz) + (T)4 * (T)op.vxz[o] * Sxz + (T)2 * (T)op.vx[o] * (Sxxx + Sxzz) +
             (T)2 * (T)op.vz[o] * (Szzz + Sxxz);
    return r;
}

// A S at node (i,k) of the array S in global memory
template <typename T, typename SIn = float, typename Op = FOp>
__device__ __forceinline__ T apply_A(const SIn* __restrict__ S, Geo g, int l, const Op& op, int i, int k, int ivis) {
    return apply_A_ld<T>([&](int dx, int dz) { return S[g.at(i + dx, k + dz)]; }, l, op, g.at(i, k), ivis);
}

// RKC1 in increment form.  With Y_0 = e and D_j = Y_j - Y_0 the reference's recurrence
//   Y_j = cc_j Y_0 + mew_j Y_{j-1} + vv_j Y_{j-2} + mewt_j c dt F(Y_{j-1}),  cc_j = 1 - mew_j - vv_j
// becomes  D_j = mew_j D_{j-1} + vv_j D_{j-2} + mewt_j c dt (F0 - A D_{j-1}),  F0 = F(Y_0).
// Stored in FP32, the increments carry rounding relative to |D| instead of |Y|: a 35-stage
// Chebyshev recurrence amplifies per-stage rounding by O(s^2), which on the stored stage values
// themselves swamps the correction after a prolongation.  F0 = F(Y_0) is evaluated in FP32: for
// a smooth Y_0 the stencil cancels and the rounding of A Y_0 is large next to A Y_0 itself, but it
// is node-to-node noise, i.e. high-frequency forcing, which the correction equation maps to
// errors of size noise / lambda_max (the biharmonic's largest eigenvalue, ~h^-4): negligible,
// and measured to leave the cycle count unchanged.  After a descent Y_0 = 0 and F0 is the
// right-hand side itself (the ZERO variant also clears Y_0's interior node, so no separate
// clearing pass is needed).
template <bool ZERO>
__device__ __forceinline__ void rkc_first_node(float* D1, float* F0, float* Y0, const FOp& op, Geo g, int l, int nx,
                                               int nz, float mewtc, int ivis, float sz, int i, int k) {
    const size_t o = g.at(i, k);
    float F;
    if (ZERO) {
        F = op.rhs[o];
        Y0[o] = 0.0f;  // the correction restarts from zero (its ghosts are written by the last stage)
    } else {
        F = op.rhs[o] - apply_A<float>(Y0, g, l, op, i, k, ivis);
    }
    F0[o] = F;
    store_ghosts_f(D1, g, i, k, nx, nz, mewtc * op.dtst[o] * F, sz);
}

template <bool ZERO>
__global__ void __launch_bounds__(256) k_rkc_first_f(float* __restrict__ D1, float* __restrict__ F0,
                                                     float* __restrict__ Y0, FOp op, Geo g, int l, int nx,
                                                     int nz, float mewtc, int ivis, float sz) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    rkc_first_node<ZERO>(D1, F0, Y0, op, g, l, nx, nz, mewtc, ivis, sz, i, k);
}

template <typename R>
__device__ __forceinline__ float restrict_node(const R* in, Geo gf, int i, int k);

// the restriction of the finer level's residual (full weighting) fused into the zero-start first
// stage of the level it lands on: writes that level's RHS and runs rkc_first_node<true>
template <typename R>
__global__ void __launch_bounds__(256) k_restrict_first_f(float* __restrict__ D1, float* __restrict__ F0,
                                                          float* __restrict__ Y0, float* __restrict__ rhs, const R* fine,
                                                          Geo gf, FOp op, Geo g, int l, int nx, int nz, float mewtc,
                                                          int ivis, float sz) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    rhs[g.at(i, k)] = restrict_node(fine, gf, i, k);
    rkc_first_node<true>(D1, F0, Y0, op, g, l, nx, nz, mewtc, ivis, sz, i, k);
}

// stage j >= 2: out may alias Dm2 (each thread reads Dm2 only at its own interior node).
// The last stage (Y0out != nullptr) writes Y0 + D_s into Y0out instead.
__global__ void __launch_bounds__(256) k_rkc_stage_f(float* out, const float* __restrict__ Dm1, const float* Dm2,
                                                     const float* __restrict__ F0, float* Y0out, FOp op, Geo g,
                                                     int l, int nx, int nz, float mew, float vv, float mewtc,
                                                     int ivis, float sz) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    size_t o = g.at(i, k);
    float F = F0[o] - apply_A<float>(Dm1, g, l, op, i, k, ivis);
    float d = mew * Dm1[o] + mewtc * op.dtst[o] * F;
    if (Dm2) d += vv * Dm2[o];
    if (Y0out) store_ghosts_f(Y0out, g, i, k, nx, nz, Y0out[o] + d, sz);
    else store_ghosts_f(out, g, i, k, nx, nz, d, sz);
}

// k_rkc_stage_f for two vertically adjacent nodes per thread: the union of their stencils (36
// values of D_{j-1}: rows k-3..k+4 of column i, rows k-2..k+3 of columns i-2..i+2, rows k and k+1
// of columns i-3 and i+3) is loaded once into registers, about half the loads per node of the
// one-node kernel.  Same arithmetic per node.
__global__ void __launch_bounds__(128) k_rkc_stage_f2(float* out, const float* __restrict__ Dm1, const float* Dm2,
                                                      const float* __restrict__ F0, float* Y0out, FOp op, Geo g,
                                                      int l, int nx, int nz, float mew, float vv, float mewtc,
                                                      int ivis, float sz) {
    pdl_begin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = 2 * (blockIdx.y * blockDim.y + threadIdx.y) + 1;
    if (i > nx - 1 || k > nz - 1) return;
    // w[r + 3][c + 3] = D_{j-1}(i + c, k + r), r = -3..4 (the rows of both nodes' stencils)
    float w[8][7];
#pragma unroll
    for (int r = -3; r <= 4; r++)
#pragma unroll
        for (int c = -3; c <= 3; c++) {
            const bool need = c == 0 || ((r >= -2 && r <= 3) && (c >= -2 && c <= 2)) || r == 0 || r == 1;
            w[r + 3][c + 3] = need ? Dm1[g.at(i + c, k + r)] : 0.0f;
        }
#pragma unroll
    for (int n = 0; n < 2; n++) {
        const int kn = k + n;
        if (kn > nz - 1) break;
        const size_t o = g.at(i, kn);
        const float A = apply_A_ld<float>([&](int dx, int dz) { return w[n + dz + 3][dx + 3]; }, l, op, o, ivis);
        const float F = F0[o] - A;
        float d = mew * w[n + 3][3] + mewtc * op.dtst[o] * F;
        if (Dm2) d += vv * Dm2[o];
        if (Y0out) store_ghosts_f(Y0out, g, i, kn, nx, nz, Y0out[o] + d, sz);
        else store_ghosts_f(out, g, i, kn, nx, nz, d, sz);
    }
}

// Residual of the correction equation, the RHS the next coarser level sees.  T = double when the
// correction holds a prolongated coarse correction: for smooth modes the biharmonic stencil
// cancels by orders of magnitude, which FP32 cannot resolve on the fine levels.  T = float after a
// smoothing pass that started from zero: the correction was built from this RHS, so FP32 rounding
// stays a small fraction of |RHS|.
template <typename T>
__global__ void __launch_bounds__(256) k_residual_f(float* __restrict__ res, const float* __restrict__ S, FOp op, Geo g,
                                                    int l, int nx, int nz, int ivis) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    size_t o = g.at(i, k);
    res[o] = (float)((T)op.rhs[o] - apply_A<T>(S, g, l, op, i, k, ivis));
}

// FP64 residual of the level-1 iterate, r = RHS - A x, with the folded FP64 stencil
__global__ void __launch_bounds__(128) k_residual64(double* __restrict__ res, const double* __restrict__ x, DOp op, Geo g,
                                                    int nx, int nz, int ivis) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    size_t o = g.at(i, k);
    res[o] = op.rhs[o] - apply_A<double, double, DOp>(x, g, 1, op, i, k, ivis);
}

// ---------------------------------------------------------------- level-1 residual, exact sums
// r = RHS - A x with the stencil sums of A formed exactly in integer arithmetic (pt_exact.cuh):
// about 16 FP64 operations per node instead of about 120, at least as accurate as the FP64 stencil.
template <bool SQUARE>
__global__ void __launch_bounds__(256) k_residual_fx(double* __restrict__ res, float* __restrict__ res32,
                                                     const double* __restrict__ x, DOp op, Geo g, int nx, int nz,
                                                     int ivis, ResFxK K) {
    __shared__ int2 X[kRfHt][kRfW];
    __shared__ int emax_s;
    pdl_begin();
    const int i0 = blockIdx.x * kRfTX + 1, k0 = blockIdx.y * kRfTZ + 1;
    const int emax = load_tile_fx<TileBig>(X, &emax_s, x, g, i0, k0, nx, nz);
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
        const int lz = threadIdx.y + 8 * r, lx = threadIdx.x;
        const int i = i0 + lx, k = k0 + lz;
        if (i > nx - 1 || k > nz - 1) continue;
        const size_t o = g.at(i, k);
        const double acc = tile_apply_A<SQUARE>(X, lx + kRfH, lz + kRfH, emax, op.vis, op.vx, op.vz, op.vxz, op.vxxmzz,
                                                o, ivis, K);
        const double rv = op.rhs[o] - acc;
        res[o] = rv;
        if (res32) res32[o] = (float)rv;  // the FP32 right-hand side of the level-1 correction
    }
}

// Residual after the level-1 pre-smoothing, updated instead of recomputed: r -= A e with the
// FP32 stencil on the FP32 correction.  e was built from r, so its rounding error is a fraction
// ~1e-5 of |r| (not of |x|, which is what forces FP64 when A is applied to the iterate itself);
// the solve's final convergence test recomputes the FP64 residual from x.
__global__ void __launch_bounds__(128) k_residual_update(double* __restrict__ res, const float* __restrict__ e, FOp op,
                                                         Geo g, int nx, int nz, int ivis) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    const size_t o = g.at(i, k);
    res[o] -= (double)apply_A<float>(e, g, 1, op, i, k, ivis);
}

// full weighting (restrict, iterative_solver.f90:398-418) into FP32; R = double restricts the
// FP64 level-1 residual directly
template <typename R>
__device__ __forceinline__ float restrict_node(const R* in, Geo gf, int i, int k) {
    const int ii = 2 * i, kk = 2 * k;
    R corners = (in[gf.at(ii - 1, kk - 1)] + in[gf.at(ii - 1, kk + 1)] + in[gf.at(ii + 1, kk + 1)] + in[gf.at(ii + 1, kk - 1)]) * (R)0.0625;
    R sides = (in[gf.at(ii - 1, kk)] + in[gf.at(ii, kk - 1)] + in[gf.at(ii + 1, kk)] + in[gf.at(ii, kk + 1)]) * (R)0.125;
    return (float)(corners + sides + in[gf.at(ii, kk)] * (R)0.25);
}

template <typename R>
__global__ void k_restrict_f(float* out, const R* in, Geo gc, Geo gf, int nxc, int nzc) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nxc - 1) return;
    out[gc.at(i, k)] = restrict_node(in, gf, i, k);
}

// bilinear prolongation of the coarse correction C at fine node (i,k)
__device__ __forceinline__ float prolong_value(const float* C, Geo gc, int i, int k) {
    if (!(i & 1) && !(k & 1)) return C[gc.at(i / 2, k / 2)];
    if (!(i & 1)) return (C[gc.at(i / 2, (k - 1) / 2)] + C[gc.at(i / 2, (k + 1) / 2)]) * 0.5f;
    if (!(k & 1)) return (C[gc.at((i - 1) / 2, k / 2)] + C[gc.at((i + 1) / 2, k / 2)]) * 0.5f;
    return (C[gc.at((i - 1) / 2, (k - 1) / 2)] + C[gc.at((i + 1) / 2, (k - 1) / 2)] + C[gc.at((i + 1) / 2, (k + 1) / 2)] +
            C[gc.at((i - 1) / 2, (k + 1) / 2)]) * 0.25f;
}

// the prolongation added to F followed by F's boundary values (k_stream_bcs_f), in one pass: each
// interior node writes its mirror images; the wall nodes and the images of wall nodes are zero
// (nothing else writes them), which is what the boundary pass would set
__global__ void k_prolong_bc_f(float* F, const float* C, Geo gf, Geo gc, int nxf, int nzf, float sz) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nxf - 1) return;
    store_ghosts_f(F, gf, i, k, nxf, nzf, F[gf.at(i, k)] + prolong_value(C, gc, i, k), sz);
}

__global__ void k_stream_bcs_f(float* S, Geo g, int nx, int nz, float sz) {
    pdl_begin();
    int W = nx + 7;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * (nz + 7)) return;
    int i = idx % W - 3, k = idx / W - 3;
    if (i > 0 && i < nx && k > 0 && k < nz) return;
    int mi = mirror_idx(i, nx), mk = mirror_idx(k, nz);
    float v = 0.0f;
    if (!(mi == 0 || mi == nx || mk == 0 || mk == nz)) {
        float s = 1.0f;
        if (i < 0 || i > nx) s = -s;
        if (k < 0 || k > nz) s *= sz;
        v = s * S[g.at(mi, mk)];
    }
    S[g.at(i, k)] = v;
}

// FP64 coefficient fields -> FP32 (whole arrays, ghosts included)
__global__ void k_coef_to_f32(float* v0, float* v1, float* v2, float* v3, float* v4, float* v5, const double* a0,
                              const double* a1, const double* a2, const double* a3, const double* a4,
                              const double* a5, size_t n) {
    size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    v0[q] = (float)a0[q]; v1[q] = (float)a1[q]; v2[q] = (float)a2[q];
    v3[q] = (float)a3[q]; v4[q] = (float)a4[q]; v5[q] = (float)a5[q];
}

__global__ void k_res_to_f32(float* out, const double* in, size_t n) {
    pdl_begin();
    size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) out[q] = (float)in[q];
}

// writes value v of interior node (i,k) of the FP64 iterate and its free-slip ghost images (the
// per-node form of enforceBCs_stream: antisymmetric across the side walls, sign sz across top and
// bottom; wall nodes and their images are zero and are not written)
__device__ __forceinline__ void store_ghosts_d(double* out, Geo g, int i, int k, int nx, int nz, double v, double sz) {
    int xs[3], zs[3];
    double xf[3], zf[3];
    int nxp = 0, nzp = 0;
    xs[nxp] = i; xf[nxp++] = 1.0;
    if (i <= 3) { xs[nxp] = -i; xf[nxp++] = -1.0; }
    if (i >= nx - 3) { xs[nxp] = 2 * nx - i; xf[nxp++] = -1.0; }
    zs[nzp] = k; zf[nzp++] = 1.0;
    if (k <= 3) { zs[nzp] = -k; zf[nzp++] = sz; }
    if (k >= nz - 3) { zs[nzp] = 2 * nz - k; zf[nzp++] = sz; }
    for (int a = 0; a < nxp; a++)
        for (int b = 0; b < nzp; b++) out[g.at(xs[a], zs[b])] = (xf[a] * zf[b]) * v;
}

// x += P e2 on the interior in FP64: the closing prolongation of a cycle (level 2 -> 1) fused
// with the update, so the level-1 correction is never rounded to FP32.  SET: x = P e2 (the GCR
// direction), with the ghost images; wall nodes are not written
template <bool SET>
__global__ void k_prolong_add(double* x, const float* C, Geo gf, Geo gc, int nxf, int nzf, double sz) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nxf - 1) return;
    double add;
    if (!(i & 1) && !(k & 1)) add = (double)C[gc.at(i / 2, k / 2)];
    else if (!(i & 1)) add = ((double)C[gc.at(i / 2, (k - 1) / 2)] + (double)C[gc.at(i / 2, (k + 1) / 2)]) * 0.5;
    else if (!(k & 1)) add = ((double)C[gc.at((i - 1) / 2, k / 2)] + (double)C[gc.at((i + 1) / 2, k / 2)]) * 0.5;
    else
        add = ((double)C[gc.at((i - 1) / 2, (k - 1) / 2)] + (double)C[gc.at((i + 1) / 2, (k - 1) / 2)] +
               (double)C[gc.at((i + 1) / 2, (k + 1) / 2)] + (double)C[gc.at((i - 1) / 2, (k + 1) / 2)]) * 0.25;
    size_t o = gf.at(i, k);
    store_ghosts_d(x, gf, i, k, nxf, nzf, SET ? add : x[o] + add, sz);
}

// x += e on the interior (FP64 accumulate of the FP32 correction), with the ghost images
__global__ void k_add_correction(double* x, const float* e, Geo g, int nx, int nz, double sz) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nx - 1) return;
    size_t o = g.at(i, k);
    store_ghosts_d(x, g, i, k, nx, nz, x[o] + (double)e[o], sz);
}

__global__ void k_coarse_rhs_f(double* B, const float* R, const double* RowB, Geo g, int nxc, int nzc) {
    int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int N = nzc + 1, n = (nxc + 1) * N;
    if (p > n) return;
    int ip = (p - 1) / N, kp = (p - 1) % N;
    B[p - 1] = (ip > 0 && ip < nxc && kp > 0 && kp < nzc) ? (double)R[g.at(ip, kp)] * RowB[p - 1] : 0.0;
}
__global__ void k_coarse_scatter_f(float* e, const double* B, Geo g, int nxc, int nzc) {
    int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int N = nzc + 1, n = (nxc + 1) * N;
    if (p > n) return;
    e[g.at((p - 1) / N, (p - 1) % N)] = (float)B[p - 1];
}

// ---------------------------------------------------------------- GCR acceleration (krylov > 0)
// Flexible GCR with the mixed cycle as its preconditioner: per iteration j (direction slot j
// since the last restart)
//   z_j = M r        the V-cycle below level 1 on r, prolongated: z_0 = P e_2 (FP64); then the
//                    FP32 level-1 smoothing e_3 of A e = r_2, r_2 = r - A z_0 (FP64, exact
//                    integer stencil sums), from zero: z_j = z_0 + e_3.  The smoothing comes last
//                    because A applied to an unsmoothed prolongation is dominated by its grid-scale
//                    interpolation error (the plain cycle, too, tests its residual after the level-1
//                    smoothing, never right after a prolongation)
//   v_j = -A z_j     FP64, exact integer stencil sums on z_j: v_j must be exact to FP64 rounding,
//                    since r is only ever updated through it (an FP32 A e_3 makes r drift from the
//                    true residual by ~1e-4 of the starting residual over a solve at 1024x512)
//   v_j -= sum_i c_i v_i,  z_j -= sum_i c_i z_i,  c_i = (v_j, v_i) / (v_i, v_i)    (i < j)
//   alpha = -(r, v_j) / (v_j, v_j);   x += alpha z_j;   r += alpha v_j
// so that r stays the residual of x (up to FP64 rounding) and |r| is minimised over the span of
// the directions.  After the smoothing: k_gcr_zadd (z_j), the exact residual kernel (v_j), then
// one CTA per padded grid row: k_gcr_dots (the dots (v_j, v_i)), k_gcr_orth (the
// orthogonalisation, (v_j, v_j), (r, v_j)) and k_gcr_update (x, r, sum |r|).  Each writes per-row partial sums over the interior nodes, and its
// last CTA to finish (a counter, reset by that CTA) reduces them in row order into the device
// scalars gsc = [|v_i|^2 (kGcrMax) | c_i (kGcrMax) | alpha | sum |r|]: the iteration is
// deterministic and the scalars never leave the device.
struct GcrSet {
    const double* v[kGcrMax];
    double* z[kGcrMax];
};
constexpr int kGcrThreads = 256;
constexpr int kGcrScAlpha = 2 * kGcrMax, kGcrScRes = 2 * kGcrMax + 1, kGcrSc = 2 * kGcrMax + 2;

// block sum of nq (<= kGcrMax) per-thread values, in a fixed order; thread 0 writes
// out[q * stride]
__device__ __forceinline__ void gcr_block_sums(const double* a, int nq, double* out, int stride) {
    __shared__ double sh[kGcrThreads / 32][kGcrMax];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kGcrMax; q++) {
        if (q >= nq) break;
        double v = a[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int q = 0; q < nq; q++) {
            double t = 0.0;
            for (int w = 0; w < kGcrThreads / 32; w++) t += sh[w][q];
            out[(size_t)q * stride] = t;
        }
}

// After the CTA's partials are written: true in the last CTA of the grid to get here (it then
// sees every CTA's partials); that CTA resets the counter for the next launch.
__device__ __forceinline__ bool gcr_last_block(unsigned* count) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        __threadfence();
        if (threadIdx.x == 0) *count = 0u;
    }
    return last;
}

// the totals of nq partial planes part[q * R + b] (b < R) in row order into tot[q] (all threads)
__device__ __forceinline__ void gcr_totals(const double* part, int R, int nq, double* tot) {
    double a[kGcrMax] = {};
#pragma unroll
    for (int q = 0; q < kGcrMax; q++)
        if (q < nq)
            for (int b = threadIdx.x; b < R; b += kGcrThreads) a[q] += __ldcg(part + (size_t)q * R + b);
    gcr_block_sums(a, nq, tot, 1);
    __syncthreads();
}

// alpha from the totals (v_j, v_j), (r, v_j): |v_j|^2 -> sc[j], alpha -> sc[kGcrScAlpha] (0 for a
// vanishing or non-finite direction)
__device__ __forceinline__ void gcr_alpha(const double* tot, int j, double* sc) {
    if (threadIdx.x == 0) {
        const double n2 = tot[0];
        const bool ok = n2 > 0.0 && isfinite(n2) && isfinite(tot[1]);
        sc[j] = ok ? n2 : 0.0;
        sc[kGcrScAlpha] = ok ? -tot[1] / n2 : 0.0;
    }
}

// z += e (FP64, with the ghost images): the end of z_j = M r
__global__ void __launch_bounds__(128) k_gcr_zadd(double* __restrict__ z, const float* __restrict__ e, Geo g, int nx,
                                                  int nz, double sz) {
    pdl_begin();
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    const size_t o = g.at(i, k);
    store_ghosts_d(z, g, i, k, nx, nz, z[o] + (double)e[o], sz);
}

// nk > 0: partial dots (v, v_i), i < nk, then (last CTA) c_i = (v, v_i) / |v_i|^2;
// nk = 0: partial (v, v) and (r, v), then (last CTA) alpha.
__global__ void __launch_bounds__(kGcrThreads) k_gcr_dots(const double* __restrict__ v, const double* __restrict__ r,
                                                          GcrSet S, int nk, Geo g, int nx, int nz, double* part,
                                                          double* sc, unsigned* count) {
    pdl_begin();
    const int R = gridDim.x, b = blockIdx.x, k = b - GH;
    double a[kGcrMax] = {};
    if (k >= 1 && k <= nz - 1)
        for (int i = 1 + threadIdx.x; i <= nx - 1; i += kGcrThreads) {
            const size_t o = g.at(i, k);
            const double vv = v[o];
            if (nk == 0) {
                a[0] += vv * vv;
                a[1] += r[o] * vv;
            } else {
#pragma unroll
                for (int q = 0; q < kGcrMax; q++)
                    if (q < nk) a[q] += vv * S.v[q][o];
            }
        }
    const int nq = nk == 0 ? 2 : nk;
    gcr_block_sums(a, nq, part + b, R);
    if (!gcr_last_block(count)) return;
    __shared__ double tot[kGcrMax];
    gcr_totals(part, R, nq, tot);
    if (nk == 0) {
        gcr_alpha(tot, 0, sc);
    } else if (threadIdx.x < (unsigned)nk) {
        const double n2 = sc[threadIdx.x];
        sc[kGcrMax + threadIdx.x] = n2 > 0.0 ? tot[threadIdx.x] / n2 : 0.0;
    }
}

// vn -= sum c_i v_i, zn -= sum c_i z_i over the whole padded row (ghost images stay images);
// partial (vn, vn) and (r, vn) over the interior, then (last CTA) alpha for slot nk
__global__ void __launch_bounds__(kGcrThreads) k_gcr_orth(double* __restrict__ vn, double* __restrict__ zn, GcrSet S,
                                                          int nk, double* sc, const double* __restrict__ r, Geo g,
                                                          int nx, int nz, double* part, unsigned* count) {
    pdl_begin();
    const int R = gridDim.x, b = blockIdx.x, k = b - GH;
    double c[kGcrMax];
#pragma unroll
    for (int q = 0; q < kGcrMax; q++) c[q] = q < nk ? sc[kGcrMax + q] : 0.0;
    double a[2] = {0.0, 0.0};
    const size_t row = (size_t)b * g.pitch;
    for (int col = threadIdx.x; col < g.pitch; col += kGcrThreads) {
        const size_t o = row + col;
        double v = vn[o], z = zn[o];
#pragma unroll
        for (int q = 0; q < kGcrMax; q++)
            if (q < nk) {
                v -= c[q] * S.v[q][o];
                z -= c[q] * S.z[q][o];
            }
        vn[o] = v;
        zn[o] = z;
        const int i = col - GH;
        if (k >= 1 && k <= nz - 1 && i >= 1 && i <= nx - 1) {
            a[0] += v * v;
            a[1] += r[o] * v;
        }
    }
    gcr_block_sums(a, 2, part + b, R);
    if (!gcr_last_block(count)) return;
    __shared__ double tot[2];
    gcr_totals(part, R, 2, tot);
    gcr_alpha(tot, nk, sc);
}

// x += alpha z (whole padded row), r += alpha v (interior); partial sum |r|, then (last CTA) the
// total into sc[kGcrScRes]
__global__ void __launch_bounds__(kGcrThreads) k_gcr_update(double* __restrict__ x, double* __restrict__ r,
                                                            const double* __restrict__ zn,
                                                            const double* __restrict__ vn, double* sc, Geo g, int nx,
                                                            int nz, double* part, unsigned* count) {
    pdl_begin();
    const int R = gridDim.x, b = blockIdx.x, k = b - GH;
    const double al = sc[kGcrScAlpha];
    double a[1] = {0.0};
    const size_t row = (size_t)b * g.pitch;
    for (int col = threadIdx.x; col < g.pitch; col += kGcrThreads) {
        const size_t o = row + col;
        x[o] += al * zn[o];
        const int i = col - GH;
        if (k >= 1 && k <= nz - 1 && i >= 1 && i <= nx - 1) {
            const double rv = r[o] + al * vn[o];
            r[o] = rv;
            a[0] += fabs(rv);
        }
    }
    gcr_block_sums(a, 1, part + b, R);
    if (!gcr_last_block(count)) return;
    __shared__ double tot[1];
    gcr_totals(part, R, 1, tot);
    if (threadIdx.x == 0) sc[kGcrScRes] = tot[0];
}

// FP64 level-1 residual (and optionally the sum of |r| into dscal[8])
static int residual64(Engine& E, bool want_sum, float* res32 = nullptr) {
    const Geo& g = E.gl[1];
    DOp op{E.vis[1], E.vx[1], E.vz[1], E.vxz[1], E.vxxmzz[1], E.RHS[1]};
    if (E.res_int) {
        dim3 blk(kRfTX, 8), grd(nblk(g.nx - 1, kRfTX), nblk(g.nz - 1, kRfTZ));
        auto kern = E.resfx[1].square ? k_residual_fx<true> : k_residual_fx<false>;
        if (int rc = launch_pdl("k_residual_fx", kern, grd, blk, 0, E.st, E.res[1], res32, (const double*)E.err[1], op, g,
                                g.nx, g.nz, E.cfg.ivis, E.resfx[1]))
            return rc;
    } else {
        dim3 blk(32, 4), grd(nblk(g.nx - 1, 32), nblk(g.nz - 1, 4));
        if (int rc = launch_pdl("k_residual64", k_residual64, grd, blk, 0, E.st, E.res[1], (const double*)E.err[1], op, g,
                                g.nx, g.nz, E.cfg.ivis))
            return rc;
        if (res32) {
            const size_t n1 = g.elems();
            if (int rc = launch_pdl("k_res_to_f32", k_res_to_f32, dim3(nblk(n1, 256)), dim3(256), 0, E.st, res32,
                                    (const double*)E.res[1], n1))
                return rc;
        }
    }
    if (want_sum) return reduce_sum_abs_interior(E, E.res[1], g.nx, g.nz, g.pitch, E.dscal + 8);
    return 0;
}

static int add_correction(Engine& E) {
    const Geo& g1 = E.gl[1];
    return launch_pdl("k_add_correction", k_add_correction, dim3(nblk(g1.nx - 1, 128), g1.nz - 1), dim3(128), 0, E.st,
                      E.err[1], (const float*)E.ferr[1], g1, g1.nx, g1.nz, E.cfg.Vbc == 0 ? -1.0 : 1.0);
}

static FOp fop(Engine& E, int l) {
    float* const* c = E.fcoef[l];
    return FOp{c[0], c[1], c[2], c[3], c[4], E.fRHS[l], c[5]};
}

static int bcs_f(Engine& E, int l, float* f) {
    const Geo& g = E.gl[l];
    return launch_pdl("k_stream_bcs_f", k_stream_bcs_f, dim3(nblk((size_t)(g.nx + 7) * (g.nz + 7), 256)), dim3(256), 0,
                      E.st, f, g, g.nx, g.nz, E.cfg.Vbc == 0 ? -1.f : 1.f);
}

// FP32 iterate_stream on the correction of level l, RKC1 in increment form (k_rkc_first_f).
// zero: the correction is zero on entry (first visit after a descent); want_res: the residual is
// needed (the next step descends).
static int smooth_f(Engine& E, int l, bool zero, bool want_res, bool restrict_in = false,
                    const double* res1 = nullptr) {
    const Geo& g = E.gl[l];
    // level 1: the nstageS-stage smoother; levels 2..grids: the nstageC-stage one
    const bool coarse = l >= 2;
    const int N = coarse ? E.nstageC : E.cfg.nstageS, ivis = E.cfg.ivis;
    const double* kmew = coarse ? E.mew_c : E.K.mew;
    const double* kvv = coarse ? E.vv_c : E.K.vv;
    const double* kmewt = coarse ? E.mewt_c : E.K.mewt;
    const float sz = E.cfg.Vbc == 0 ? -1.f : 1.f;
    FOp op = fop(E, l);
    dim3 blk(32, 8), grd(nblk(g.nx - 1, 32), nblk(g.nz - 1, 8));
    const dim3 blk2(32, 4), grd2(nblk(g.nx - 1, 32), nblk(g.nz - 1, 8));  // two nodes per thread in z
    const bool two = (size_t)(g.nx - 1) * (size_t)(g.nz - 1) >= 262144;
    // FP64-arithmetic residual in 64-thread blocks: this part issues about two FP64 FMAs per
    // clock per SM, so the coarse levels need every SM they can get
    dim3 blk64(32, 2), grd64(nblk(g.nx - 1, 32), nblk(g.nz - 1, 2));
    float* e = E.ferr[l];
    float* F0 = E.fS0[l];
    const double c = E.cfg.c_2;  // Nmulti = 1: one pass with c = c_2
    for (int n = 1; n <= E.cfg.Nmulti; n++) {
        GraphTimer gt(E, 1, (l == 1 && zero) ? N : 0);
        float* Dm1 = E.fS1[l];
        float* Dm2 = E.fS2[l];
        const float mewtc1 = (float)(kmewt[1] * c);
        if (restrict_in && zero && n == 1) {  // restriction of the finer residual fused in
            const Geo& gf = E.gl[l - 1];
            int rc;
            if (l == 2)
                rc = launch_pdl("k_restrict_first_f", k_restrict_first_f<double>, grd, blk, 0, E.st, Dm1, F0, e,
                                E.fRHS[l], res1 ? res1 : (const double*)E.res[1], gf, op, g, l, g.nx, g.nz, mewtc1,
                                ivis, sz);
            else
                rc = launch_pdl("k_restrict_first_f", k_restrict_first_f<float>, grd, blk, 0, E.st, Dm1, F0, e,
                                E.fRHS[l], (const float*)E.fres[l - 1], gf, op, g, l, g.nx, g.nz, mewtc1, ivis, sz);
            if (rc) return rc;
        } else {
            auto first = (zero && n == 1) ? k_rkc_first_f<true> : k_rkc_first_f<false>;
            if (int rc = launch_pdl("k_rkc_first_f", first, grd, blk, 0, E.st, Dm1, F0, e, op, g, l, g.nx, g.nz, mewtc1,
                                    ivis, sz))
                return rc;
        }
        for (int j = 2; j <= N; j++) {
            const bool last = (j == N);
            // D_{j-2} = D_0 = 0 at j = 2; the output overwrites D_{j-2}
            // large levels: two nodes per thread (half the loads); small ones: one (twice the threads)
            auto kst = two ? k_rkc_stage_f2 : k_rkc_stage_f;
            if (int rc = launch_pdl(two ? "k_rkc_stage_f2" : "k_rkc_stage_f", kst, two ? grd2 : grd, two ? blk2 : blk, 0,
                                    E.st, Dm2, (const float*)Dm1, (const float*)(j == 2 ? nullptr : Dm2),
                                    (const float*)F0, last ? e : nullptr, op, g, l, g.nx, g.nz, (float)kmew[j],
                                    (float)kvv[j], (float)(kmewt[j] * c), ivis, sz))
                return rc;
            float* t = Dm1;
            Dm1 = Dm2;
            Dm2 = t;
        }
        CKL("k_rkc_stage_f");
    }
    if (want_res) {
        auto kres = zero ? k_residual_f<float> : k_residual_f<double>;
        if (int rc = launch_pdl("k_residual_f", kres, zero ? grd : grd64, zero ? blk : blk64, 0, E.st, E.fres[l],
                                (const float*)e, op, g, l, g.nx, g.nz, ivis))
            return rc;
    }
    return 0;
}

static int coarse_solve_f(Engine& E) {
    const int L = E.grids, n = E.ngc;
    const Geo& g = E.gl[L];
    if (E.Ginv) return coarse_apply(E, nullptr, E.ferr[L], nullptr, E.fRHS[L]);  // with the boundary values
    PT_COUNT(), k_coarse_rhs_f<<<nblk(n, 128), 128, 0, E.st>>>(E.Bc, E.fRHS[L], E.RowB, g, g.nx, g.nz);
    int rc = coarse_band_solve(E);
    if (rc) return rc;
    PT_COUNT(), k_coarse_scatter_f<<<nblk(n, 128), 128, 0, E.st>>>(E.ferr[L], E.Bc, g, g.nx, g.nz);
    CKL("coarse_solve_f");
    return bcs_f(E, L, E.ferr[L]);
}

// part 0: r = RHS - A x (FP64); FP32 pre-smoothing of A e = r on level 1 from e = 0; x += e;
//         r = RHS - A x (FP64) and the sum of |r| for the convergence test -- the same test, at
//         the same point (after the level-1 smoothing), as in the FP64 cycle;
// part 1: the rest of the schedule on the correction, from the restriction of that FP64
//         residual onwards; the closing prolongation (level 2 -> 1) is added to x in FP64.
static int gcr_tail(Engine& E, int slot);

// slot >= 0: the GCR form (krylov > 0) for direction slot `slot` (part 1 runs first): part 1 is
// the V-cycle below level 1 on the current residual, prolongated into z_slot = P e_2; part 0 the
// level-1 smoothing of r - A z_slot added to z_slot, v_slot, and the GCR update of x and r
// (gcr_tail)
static int mixed_part(Engine& E, int part, int slot = -1) {
    int rc;
    const Geo& g1 = E.gl[1];
    const bool gcr = slot >= 0;
    if (part == 0 && gcr) return gcr_tail(E, slot);
    // the level-1 residual the levels below see (after the pre-smoothing of part 0, or the GCR
    // residual) and where the closing prolongation goes
    const double* r1 = E.res[1];
    double* xdst = gcr ? E.gz[slot] : E.err[1];
    if (part == 0) {
        if ((rc = residual64(E, false, E.fRHS[1]))) return rc;
        if ((rc = smooth_f(E, 1, true, false))) return rc;
        if ((rc = add_correction(E))) return rc;
        dim3 blk(32, 4), grd(nblk(g1.nx - 1, 32), nblk(g1.nz - 1, 4));
        if ((rc = launch_pdl("k_residual_update", k_residual_update, grd, blk, 0, E.st, E.res[1], (const float*)E.ferr[1],
                             fop(E, 1), g1, g1.nx, g1.nz, E.cfg.ivis)))
            return rc;
        return reduce_sum_abs_interior(E, E.res[1], g1.nx, g1.nz, g1.pitch, E.dscal + 8);
    }
    const int grids = E.grids, nsteps = E.mnsteps;
    const int* multi = E.mmulti;
    for (int p = 2; p <= nsteps; p++) {
        const int l = multi[p];
        const Geo& g = E.gl[l];
        // the reference's schedules visit level 1 only at their first step; the pre-smoothing of
        // part 0 is already in x, so the cycle's level-1 correction is the closing prolongation
        if (l == 1) return fail(PT_ERR_CONFIG, "mixed-precision cycle: schedule revisits level 1");
        const bool descend = multi[p - 1] < multi[p];
        if (descend && l == grids) {  // (above the coarsest level the restriction is fused into smooth_f)
            const Geo& gf = E.gl[l - 1];
            dim3 gr(nblk(g.nx - 1, 128), g.nz - 1);
            // the correction of level l restarts from zero: cleared by the first smoothing stage
            // (or overwritten whole by the coarse solve)
            if (l == 2)
                rc = launch_pdl("k_restrict_f", k_restrict_f<double>, gr, dim3(128), 0, E.st, E.fRHS[l], r1, g, gf,
                                g.nx, g.nz);
            else
                rc = launch_pdl("k_restrict_f", k_restrict_f<float>, gr, dim3(128), 0, E.st, E.fRHS[l],
                                (const float*)E.fres[l - 1], g, gf, g.nx, g.nz);
            if (rc) return rc;
        }
        if (l < grids) {
            if ((rc = smooth_f(E, l, descend, multi[p + 1] > multi[p], descend, r1))) return rc;
        } else if ((rc = coarse_solve_f(E))) {
            return rc;
        }
        if (multi[p + 1] < multi[p]) {
            if (l == 2) {  // closing prolongation, added to x (or to z_slot) in FP64
                // GCR: z_slot = P e_2 is written, not added (its wall nodes are zero in every direction)
                return launch_pdl("k_prolong_add", gcr ? k_prolong_add<true> : k_prolong_add<false>,
                                  dim3(nblk(g1.nx - 1, 128), g1.nz - 1), dim3(128), 0, E.st, xdst,
                                  (const float*)E.ferr[2], g1, g, g1.nx, g1.nz, E.cfg.Vbc == 0 ? -1.0 : 1.0);
            }
            const Geo& gf = E.gl[l - 1];
            if ((rc = launch_pdl("k_prolong_bc_f", k_prolong_bc_f, dim3(nblk(gf.nx - 1, 128), gf.nz - 1), dim3(128), 0,
                                 E.st, E.ferr[l - 1], (const float*)E.ferr[l], gf, g, gf.nx, gf.nz,
                                 E.cfg.Vbc == 0 ? -1.f : 1.f)))
                return rc;
        }
    }
    return fail(PT_ERR_CONFIG, "mixed-precision cycle: schedule does not return to level 1");
}

// v_j = -A z_j (FP64), orthogonalisation against the slot's predecessors, then x += alpha z_j,
// r += alpha v_j and the sum of |r| into dscal[8]
static int gcr_tail(Engine& E, int slot) {
    const Geo& g = E.gl[1];
    int rc;
    // r2 = r - A z_0 in FP64 (and its FP32 copy, the right-hand side of the level-1 smoothing)
    DOp opr{E.vis[1], E.vx[1], E.vz[1], E.vxz[1], E.vxxmzz[1], E.res[1]};
    if (E.res_int) {
        dim3 blk(kRfTX, 8), grd(nblk(g.nx - 1, kRfTX), nblk(g.nz - 1, kRfTZ));
        auto kern = E.resfx[1].square ? k_residual_fx<true> : k_residual_fx<false>;
        rc = launch_pdl("k_residual_fx", kern, grd, blk, 0, E.st, E.gr1, E.fRHS[1], (const double*)E.gz[slot], opr, g,
                        g.nx, g.nz, E.cfg.ivis, E.resfx[1]);
    } else {
        dim3 blk(32, 4), grd(nblk(g.nx - 1, 32), nblk(g.nz - 1, 4));
        rc = launch_pdl("k_residual64", k_residual64, grd, blk, 0, E.st, E.gr1, (const double*)E.gz[slot], opr, g,
                        g.nx, g.nz, E.cfg.ivis);
        const size_t n1 = g.elems();
        if (!rc)
            rc = launch_pdl("k_res_to_f32", k_res_to_f32, dim3(nblk(n1, 256)), dim3(256), 0, E.st, E.fRHS[1],
                            (const double*)E.gr1, n1);
    }
    if (rc) return rc;
    if ((rc = smooth_f(E, 1, true, false))) return rc;
    {
        dim3 blk(32, 4), grd(nblk(g.nx - 1, 32), nblk(g.nz - 1, 4));
        if ((rc = launch_pdl("k_gcr_zadd", k_gcr_zadd, grd, blk, 0, E.st, E.gz[slot], (const float*)E.ferr[1], g, g.nx,
                             g.nz, E.cfg.Vbc == 0 ? -1.0 : 1.0)))
            return rc;
    }
    // v_j = 0 - A z_j
    DOp op0{E.vis[1], E.vx[1], E.vz[1], E.vxz[1], E.vxxmzz[1], E.gzero};
    if (E.res_int) {
        dim3 blk(kRfTX, 8), grd(nblk(g.nx - 1, kRfTX), nblk(g.nz - 1, kRfTZ));
        auto kern = E.resfx[1].square ? k_residual_fx<true> : k_residual_fx<false>;
        rc = launch_pdl("k_residual_fx", kern, grd, blk, 0, E.st, E.gv[slot], (float*)nullptr,
                        (const double*)E.gz[slot], op0, g, g.nx, g.nz, E.cfg.ivis, E.resfx[1]);
    } else {
        dim3 blk(32, 4), grd(nblk(g.nx - 1, 32), nblk(g.nz - 1, 4));
        rc = launch_pdl("k_residual64", k_residual64, grd, blk, 0, E.st, E.gv[slot], (const double*)E.gz[slot], op0, g,
                        g.nx, g.nz, E.cfg.ivis);
    }
    if (rc) return rc;
    GcrSet S{};
    for (int q = 0; q < slot; q++) {
        S.v[q] = E.gv[q];
        S.z[q] = E.gz[q];
    }
    const int R = g.nz + 2 * GH + 1;
    unsigned* cnt = reinterpret_cast<unsigned*>(E.gsc + kGcrSc);
    if ((rc = launch_pdl("k_gcr_dots", k_gcr_dots, dim3(R), dim3(kGcrThreads), 0, E.st, (const double*)E.gv[slot],
                         (const double*)E.res[1], S, slot, g, g.nx, g.nz, E.gpart, E.gsc, cnt)))
        return rc;
    if (slot > 0 && (rc = launch_pdl("k_gcr_orth", k_gcr_orth, dim3(R), dim3(kGcrThreads), 0, E.st, E.gv[slot],
                                     E.gz[slot], S, slot, E.gsc, (const double*)E.res[1], g, g.nx, g.nz, E.gpart, cnt)))
        return rc;
    return launch_pdl("k_gcr_update", k_gcr_update, dim3(R), dim3(kGcrThreads), 0, E.st, E.err[1], E.res[1],
                      (const double*)E.gz[slot], (const double*)E.gv[slot], E.gsc, g, g.nx, g.nz, E.gpart, cnt);
}

static int run_gcr(Engine& E, int part, int slot) {
    cudaGraphExec_t& ex = part == 0 ? E.gG0[slot] : E.gG1[slot];
    int64_t& n = part == 0 ? E.nG0[slot] : E.nG1[slot];
    if (!ex) {
        cudaGraph_t graph = nullptr;
        int64_t before = g_launches.load();
        CK(cudaStreamBeginCapture(E.st, cudaStreamCaptureModeThreadLocal));
        int rc = mixed_part(E, part, slot);
        cudaError_t e = cudaStreamEndCapture(E.st, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        CK(e);
        CK(cudaGraphInstantiate(&ex, graph, 0));
        cudaGraphDestroy(graph);
        n = g_launches - before;
        g_launches = before;
    }
    CK(cudaGraphLaunch(ex, E.st));
    g_launches += n;
    return 0;
}

static int run_mixed(Engine& E, int part) {
    cudaGraphExec_t& ex = part == 0 ? E.gM1 : E.gM2;
    int64_t& n = part == 0 ? E.nM1 : E.nM2;
    if (!ex) {
        cudaGraph_t graph = nullptr;
        int64_t before = g_launches.load();
        CK(cudaStreamBeginCapture(E.st, cudaStreamCaptureModeThreadLocal));
        int rc = mixed_part(E, part);
        cudaError_t e = cudaStreamEndCapture(E.st, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        CK(e);
        CK(cudaGraphInstantiate(&ex, graph, 0));
        cudaGraphDestroy(graph);
        n = g_launches - before;
        g_launches = before;
    }
    CK(cudaGraphLaunch(ex, E.st));
    g_launches += n;
    return 0;
}

// |r| / |RHS| of the current residual: the sum written to dscal[8], read back
static int read_ratio(Engine& E, double norm, double* ratio, const double* sum = nullptr) {
    CK(cudaMemcpyAsync(E.hscal, sum ? sum : E.dscal + 8, 8, cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    *ratio = E.hscal[0] / norm / E.res_ref[1];
    if (E.res_hist.size() < 100000) E.res_hist.push_back(*ratio);
    if (!std::isfinite(*ratio)) return fail(PT_ERR_NOT_FINITE, "non-finite residual in the mixed-precision solve");
    if (*ratio > 1.0e10) return fail(PT_ERR_MG_DIVERGED, "mixed-precision solve: abnormally high residual");
    return 0;
}

// The GCR-accelerated solve (krylov = m > 0): the FP64 residual of the start, then per iteration
// the preconditioning cycle (the levels below 1, then level 1) and the GCR update (two captured
// graphs per slot j = iterations since the last restart, restarted after m).  The updated residual is tested after every iteration;
// when it passes, the residual is recomputed from x and tested again (a failed confirmation
// restarts the directions from that residual).
static int gcr_solve(Engine& E, pt_solve_info* info, double norm) {
    int rc, cycles = 0, slot = 0;
    double ratio = 0.0;
    if ((rc = residual64(E, true)) || (rc = read_ratio(E, norm, &ratio))) return rc;
    bool confirmed = ratio <= E.cfg.tolerance;
    while (!confirmed) {
        if (cycles >= E.cfg.max_cycles) return fail(PT_ERR_MG_MAX_CYCLES, "mixed-precision solve: too many cycles");
        {
            PhaseTimer tp(E, PH_CYCLE_COARSE);
            if ((rc = run_gcr(E, 1, slot))) return rc;
        }
        {
            PhaseTimer tp(E, PH_CYCLE_L1);
            if ((rc = run_gcr(E, 0, slot))) return rc;
        }
        if ((rc = read_ratio(E, norm, &ratio, E.gsc + kGcrScRes))) return rc;
        harvest_graph_timer(E, 1);
        cycles++;
        if (trace_on()) fprintf(stderr, "[ptgpu] gcr iteration %d residual ratio %.4e\n", cycles, ratio);
        slot = (slot + 1) % E.cfg.krylov;
        if (cycles == 1) {  // one iteration from a learned guess: keep it or restart from the previous psi
            const int fb = unet_check_fallback(E, ratio);
            if (fb < 0) return fail(PT_ERR_CUDA, "learned-guess fallback copy");
            if (fb) {
                if ((rc = residual64(E, true)) || (rc = read_ratio(E, norm, &ratio))) return rc;
                slot = 0;
                confirmed = ratio <= E.cfg.tolerance;
                continue;
            }
        }
        if (ratio <= E.cfg.tolerance) {  // confirm with the FP64 residual of x
            if ((rc = residual64(E, true)) || (rc = read_ratio(E, norm, &ratio))) return rc;
            confirmed = ratio <= E.cfg.tolerance;
            slot = 0;
        }
    }
    E.cycles = cycles;
    E.refinements = cycles;
    E.resid_ratio = ratio;
    CK(cudaMemcpyAsync(E.SF, E.err[1], E.g1.elems() * 8, cudaMemcpyDeviceToDevice, E.st));
    if (info) {
        info->cycles += cycles;
        info->resid_ratio = ratio;
        info->n_eta = E.n_eta;
        info->eig_fine = E.eig_fine;
    }
    return 0;
}

int multigrid_mixed(Engine& E, pt_solve_info* info) {
    int rc;
    PhaseTimer tm(E, PH_SOLVE);
    {
        PhaseTimer ts(E, PH_SETUP);
        if ((rc = mg_setup_solve(E))) return rc;
        if (E.cfg.guess_mode == PT_GUESS_UNET && (rc = unet_guess(E))) return rc;
        // FP32 coefficients: level 1 every solve, the coarse levels when they were rebuilt (here, or
        // by the worker thread of this time level, joined in mg_setup_solve)
        const int lmax = (E.levels_reused && !E.coarse_fresh) ? 2 : E.grids;
        E.coarse_fresh = false;
        for (int l = 1; l < lmax; l++) {
            size_t n = E.gl[l].elems();
            float* const* f = E.fcoef[l];
            PT_COUNT(), k_coef_to_f32<<<nblk(n, 256), 256, 0, E.st>>>(f[0], f[1], f[2], f[3], f[4], f[5], E.vis[l], E.vx[l],
                                                                      E.vz[l], E.vxz[l], E.vxxmzz[l], E.dtst[l], n);
        }
        CKL("k_coef_to_f32");
    }
    // the level-1 updates write each node's ghost images and never the wall nodes: start from an
    // iterate whose walls and images are consistent (a restart's psi may not be)
    if ((rc = enforce_bcs_stream(E, 1, E.err[1]))) return rc;
    const double norm = (double)(E.gl[1].nx - 2) * (double)(E.gl[1].nz - 2);
    int cycles = 0;
    double mag1 = 0.0;
    E.res_hist.clear();
    if (E.cfg.krylov > 0) return gcr_solve(E, info, norm);
    for (;;) {
        {
            PhaseTimer tp(E, PH_CYCLE_L1);
            if ((rc = run_mixed(E, 0))) return rc;
            CK(cudaMemcpyAsync(E.hscal, E.dscal + 8, 8, cudaMemcpyDeviceToHost, E.st));
        }
        CK(cudaStreamSynchronize(E.st));
        harvest_graph_timer(E, 1);
        mag1 = E.hscal[0] / norm;
        if (E.res_hist.size() < 100000) E.res_hist.push_back(mag1 / E.res_ref[1]);
        if (!std::isfinite(mag1)) return fail(PT_ERR_NOT_FINITE, "non-finite residual in the mixed-precision solve");
        if (mag1 > 1.0e10 * E.res_ref[1])
            return fail(PT_ERR_MG_DIVERGED, "mixed-precision solve: abnormally high residual");
        if (trace_on()) fprintf(stderr, "[ptgpu] mixed cycle %d residual ratio %.4e\n", cycles, mag1 / E.res_ref[1]);
        if (cycles == 1) {  // one full cycle from a learned guess: keep it or restart from the previous psi
            const int fb = unet_check_fallback(E, mag1 / E.res_ref[1]);
            if (fb < 0) return fail(PT_ERR_CUDA, "learned-guess fallback copy");
            if (fb) {
                cycles++;
                continue;
            }
        }
        if (mag1 / E.res_ref[1] <= E.cfg.tolerance) {
            // the updated residual says converged: confirm with the FP64 residual of x
            if ((rc = residual64(E, true))) return rc;
            CK(cudaMemcpyAsync(E.hscal, E.dscal + 8, 8, cudaMemcpyDeviceToHost, E.st));
            CK(cudaStreamSynchronize(E.st));
            mag1 = E.hscal[0] / norm;
            if (E.res_hist.size() < 100000) E.res_hist.push_back(mag1 / E.res_ref[1]);
            if (mag1 / E.res_ref[1] <= E.cfg.tolerance) break;
        }
        if (cycles >= E.cfg.max_cycles)
            return fail(PT_ERR_MG_MAX_CYCLES, "mixed-precision solve: too many cycles");
        {
            PhaseTimer tp(E, PH_CYCLE_COARSE);
            if ((rc = run_mixed(E, 1))) return rc;
        }
        cycles++;
    }
    E.cycles = cycles + 1;  // level-1 smoothings, counted as in the FP64 cycle
    E.refinements = cycles;
    E.resid_ratio = mag1 / E.res_ref[1];
    CK(cudaMemcpyAsync(E.SF, E.err[1], E.g1.elems() * 8, cudaMemcpyDeviceToDevice, E.st));
    if (info) {
        info->cycles += cycles + 1;
        info->resid_ratio = E.resid_ratio;
        info->n_eta = E.n_eta;
        info->eig_fine = E.eig_fine;
    }
    return 0;
}

int mixed_alloc(Engine& E) {
    if (E.res_int && !exact_stencils_setup(E)) return fail(PT_ERR_CUDA, "exact-stencil constants (mixed kernels)");
    if (E.cfg.krylov > 0) {
        const size_t n = E.g1.elems(), R = (size_t)E.g1.nz + 2 * GH + 1;
        auto get = [&](double** p, size_t cnt) {
            CK(cudaMalloc(p, cnt * sizeof(double)));
            CK(cudaMemsetAsync(*p, 0, cnt * sizeof(double), E.st));
            E.bytes_allocated += cnt * sizeof(double);
            return 0;
        };
        int rc;
        for (int j = 0; j < E.cfg.krylov; j++)
            if ((rc = get(&E.gz[j], n)) || (rc = get(&E.gv[j], n))) return rc;
        if ((rc = get(&E.gr1, n)) || (rc = get(&E.gzero, n)) || (rc = get(&E.gpart, (size_t)(kGcrMax + 2) * R)) ||
            (rc = get(&E.gsc, kGcrSc + 1)))  // the scalars, then the last-CTA counter
            return rc;
    }
    for (int f = 0; f < 3; f++) {
        const size_t n = E.g1.elems();
        CK(cudaMalloc(&E.ftab[f], n * sizeof(float4)));
        CK(cudaMemsetAsync(E.ftab[f], 0, n * sizeof(float4), E.st));
        CK(cudaMalloc(&E.facc[f], (size_t)E.ntr * sizeof(float)));
        E.bytes_allocated += (size_t)E.ntr * sizeof(float);
        E.bytes_allocated += n * sizeof(float4);
    }
    for (int l = 1; l <= E.grids; l++) {
        const size_t n = E.gl[l].elems();
        float** arrs[] = {&E.ferr[l], &E.fS0[l], &E.fS1[l], &E.fS2[l], &E.fRHS[l], &E.fres[l], &E.fcoef[l][0],
                          &E.fcoef[l][1], &E.fcoef[l][2], &E.fcoef[l][3], &E.fcoef[l][4], &E.fcoef[l][5]};
        for (auto a : arrs) {
            CK(cudaMalloc(a, n * sizeof(float)));
            CK(cudaMemsetAsync(*a, 0, n * sizeof(float), E.st));
            E.bytes_allocated += n * sizeof(float);
        }
    }
    return 0;
}

}  // namespace pt
