// pt_mixed.cu -- mixed-precision stream-function solve (spec extension, no reference
// counterpart): FP64 residual and defect correction around FP32 multigrid cycles.
//
//   x = psi (FP64 warm start);  r = RHS - A x (FP64, the reference's stream_space residual)
//   until mean|r| / mean|RHS| <= tolerance (the reference's convergence test, unchanged):
//     one FP32 cycle of the reference's level schedule on A e = r, e = 0 on entry and at every
//     descent (correction scheme): FP32 RKC1 smoothing with the FP64 pipeline's viscosity
//     coefficients and local pseudo-time steps rounded to FP32, FP32 restriction/prolongation,
//     coarsest level through the FP64 banded LU;  x += e (FP64);  r = RHS - A x (FP64).
// The viscosity pipeline and the coarse LU are the FP64 ones (mg_setup_solve).  Each cycle is
// two captured CUDA graphs: the FP64 residual + |r| sum, and the FP32 cycle + update.
#include <cmath>

#include "pt_consts.cuh"

namespace pt {

int upload_consts_mixed(const Engine& E) { return upload_tu_consts(E); }

struct FOp {
    const float *vis, *vx, *vz, *vxz, *vxxmzz, *rhs, *dtst;
};

struct FLev {
    float dr2, dr3, dr4, ds2, ds3, ds4, drds, dr2ds, drds2, dr2ds2;
};

// -(A S - rhs) in FP32 at node (i,k)
__device__ __forceinline__ float stream_F_f(const float* __restrict__ S, Geo g, const FLev& L, const FOp& op, int i,
                                            int k, int ivis) {
    float sx[7], sz[7];
#pragma unroll
    for (int j = 0; j < 7; j++) {
        sx[j] = S[g.at(i + j - 3, k)];
        sz[j] = S[g.at(i, k + j - 3)];
    }
    float Sxx = 0, Sxxx = 0, Sxxxx = 0, Szz = 0, Szzz = 0, Szzzz = 0;
#pragma unroll
    for (int j = 1; j <= 5; j++) { Sxx += (float)cK.D2[j] * sx[j]; Szz += (float)cK.D2[j] * sz[j]; }
#pragma unroll
    for (int j = 0; j < 7; j++) {
        Sxxx += (float)cK.D3[j] * sx[j]; Sxxxx += (float)cK.D4[j] * sx[j];
        Szzz += (float)cK.D3[j] * sz[j]; Szzzz += (float)cK.D4[j] * sz[j];
    }
    Sxx /= L.dr2; Sxxx /= L.dr3; Sxxxx /= L.dr4;
    Szz /= L.ds2; Szzz /= L.ds3; Szzzz /= L.ds4;
    float Sxz = 0, Sxxz = 0, Sxzz = 0, Sxxzz = 0;
#pragma unroll
    for (int kk = -2; kk <= 2; kk++) {
        float d1 = 0, d2 = 0;
#pragma unroll
        for (int ii = -2; ii <= 2; ii++) {
            float v = (kk == 0) ? sx[ii + 3] : S[g.at(i + ii, k + kk)];
            d1 += (float)cK.D1[3 + ii] * v;
            d2 += (float)cK.D2[3 + ii] * v;
        }
        Sxz += (float)cK.D1[3 + kk] * d1;
        Sxzz += (float)cK.D2[3 + kk] * d1;
        Sxxz += (float)cK.D1[3 + kk] * d2;
        Sxxzz += (float)cK.D2[3 + kk] * d2;
    }
    Sxz /= L.drds; Sxxz /= L.dr2ds; Sxzz /= L.drds2; Sxxzz /= L.dr2ds2;
    size_t o = g.at(i, k);
    float r = op.vis[o] * (Sxxxx + Szzzz + 2.0f * Sxxzz);
    if (ivis != 0) {
        r += op.vxxmzz[o] * (Sxx - Szz) + 4.0f * op.vxz[o] * Sxz + 2.0f * op.vx[o] * (Sxxx + Sxzz) +
             2.0f * op.vz[o] * (Szzz + Sxxz);
    }
    return -(r - op.rhs[o]);
}

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

// one FP32 RKC1 stage; 2-D blocks so the 7x7 stencil reuses neighbours from L1
__global__ void __launch_bounds__(256) k_rkc_stage_f(float* __restrict__ out, const float* __restrict__ S1,
                                                     const float* __restrict__ S2, const float* __restrict__ S0,
                                                     FOp op, Geo g, FLev L, int nx, int nz, float cS0, float mew,
                                                     float vv, float mewtc, int first, int ivis, float sz) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    float F = stream_F_f(S1, g, L, op, i, k, ivis);
    size_t o = g.at(i, k);
    float v;
    if (first) v = S1[o] + mewtc * op.dtst[o] * F;
    else v = cS0 * S0[o] + mew * S1[o] + vv * S2[o] + mewtc * op.dtst[o] * F;
    store_ghosts_f(out, g, i, k, nx, nz, v, sz);
}

// Residual of the correction equation with FP64 arithmetic on the FP32 correction: for smooth
// modes the biharmonic stencil cancels by orders of magnitude, which FP32 cannot resolve on the
// fine levels; this residual is what the coarser levels see.
__global__ void k_residual_f(float* __restrict__ res, const float* __restrict__ S, FOp op, Geo g, int l, int nx, int nz,
                             int ivis) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (i > nx - 1 || k > nz - 1) return;
    const LevConst& L = cL[l];
    double sx[7], sz[7];
#pragma unroll
    for (int j = 0; j < 7; j++) {
        sx[j] = (double)S[g.at(i + j - 3, k)];
        sz[j] = (double)S[g.at(i, k + j - 3)];
    }
    double Sxx = 0, Sxxx = 0, Sxxxx = 0, Szz = 0, Szzz = 0, Szzzz = 0;
#pragma unroll
    for (int j = 1; j <= 5; j++) { Sxx += cK.D2[j] * sx[j]; Szz += cK.D2[j] * sz[j]; }
#pragma unroll
    for (int j = 0; j < 7; j++) {
        Sxxx += cK.D3[j] * sx[j]; Sxxxx += cK.D4[j] * sx[j];
        Szzz += cK.D3[j] * sz[j]; Szzzz += cK.D4[j] * sz[j];
    }
    Sxx /= L.dr2; Sxxx /= L.dr3; Sxxxx /= L.dr4;
    Szz /= L.ds2; Szzz /= L.ds3; Szzzz /= L.ds4;
    double Sxz = 0, Sxxz = 0, Sxzz = 0, Sxxzz = 0;
#pragma unroll
    for (int kk = -2; kk <= 2; kk++) {
        double d1 = 0, d2 = 0;
#pragma unroll
        for (int ii = -2; ii <= 2; ii++) {
            double v = (kk == 0) ? sx[ii + 3] : (double)S[g.at(i + ii, k + kk)];
            d1 += cK.D1[3 + ii] * v;
            d2 += cK.D2[3 + ii] * v;
        }
        Sxz += cK.D1[3 + kk] * d1;
        Sxzz += cK.D2[3 + kk] * d1;
        Sxxz += cK.D1[3 + kk] * d2;
        Sxxzz += cK.D2[3 + kk] * d2;
    }
    Sxz /= L.drds; Sxxz /= L.dr2ds; Sxzz /= L.drds2; Sxxzz /= L.dr2ds2;
    size_t o = g.at(i, k);
    double r = (double)op.vis[o] * (Sxxxx + Szzzz + 2.0 * Sxxzz);
    if (ivis != 0)
        r += (double)op.vxxmzz[o] * (Sxx - Szz) + 4.0 * (double)op.vxz[o] * Sxz + 2.0 * (double)op.vx[o] * (Sxxx + Sxzz) +
             2.0 * (double)op.vz[o] * (Szzz + Sxxz);
    res[o] = (float)((double)op.rhs[o] - r);
}

__global__ void k_restrict_f(float* out, const float* in, Geo gc, Geo gf, int nxc, int nzc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nxc - 1) return;
    int ii = 2 * i, kk = 2 * k;
    float corners = (in[gf.at(ii - 1, kk - 1)] + in[gf.at(ii - 1, kk + 1)] + in[gf.at(ii + 1, kk + 1)] + in[gf.at(ii + 1, kk - 1)]) * 0.0625f;
    float sides = (in[gf.at(ii - 1, kk)] + in[gf.at(ii, kk - 1)] + in[gf.at(ii + 1, kk)] + in[gf.at(ii, kk + 1)]) * 0.125f;
    out[gc.at(i, k)] = corners + sides + in[gf.at(ii, kk)] * 0.25f;
}

__global__ void k_prolong_f(float* F, const float* C, Geo gf, Geo gc, int nxf, int nzf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nxf - 1) return;
    float add;
    if (!(i & 1) && !(k & 1)) add = C[gc.at(i / 2, k / 2)];
    else if (!(i & 1)) add = (C[gc.at(i / 2, (k - 1) / 2)] + C[gc.at(i / 2, (k + 1) / 2)]) * 0.5f;
    else if (!(k & 1)) add = (C[gc.at((i - 1) / 2, k / 2)] + C[gc.at((i + 1) / 2, k / 2)]) * 0.5f;
    else
        add = (C[gc.at((i - 1) / 2, (k - 1) / 2)] + C[gc.at((i + 1) / 2, (k - 1) / 2)] + C[gc.at((i + 1) / 2, (k + 1) / 2)] +
               C[gc.at((i - 1) / 2, (k + 1) / 2)]) * 0.25f;
    F[gf.at(i, k)] += add;
}

__global__ void k_stream_bcs_f(float* S, Geo g, int nx, int nz, float sz) {
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
    size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) out[q] = (float)in[q];
}

// x += e on the interior (FP64 accumulate of the FP32 correction)
__global__ void k_add_correction(double* x, const float* e, Geo g, int nx, int nz) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nx - 1) return;
    size_t o = g.at(i, k);
    x[o] += (double)e[o];
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

static FLev flev(const LevConst& L) {
    return FLev{(float)L.dr2, (float)L.dr3, (float)L.dr4, (float)L.ds2, (float)L.ds3, (float)L.ds4,
                (float)L.drds, (float)L.dr2ds, (float)L.drds2, (float)L.dr2ds2};
}
static FOp fop(Engine& E, int l) {
    float* const* c = E.fcoef[l];
    return FOp{c[0], c[1], c[2], c[3], c[4], E.fRHS[l], c[5]};
}

static int bcs_f(Engine& E, int l, float* f) {
    const Geo& g = E.gl[l];
    PT_COUNT(), k_stream_bcs_f<<<nblk((size_t)(g.nx + 7) * (g.nz + 7), 256), 256, 0, E.st>>>(f, g, g.nx, g.nz,
                                                                                             E.cfg.Vbc == 0 ? -1.f : 1.f);
    CKL("k_stream_bcs_f");
    return 0;
}

// FP32 iterate_stream on the correction of level l (e starts at zero: correction scheme)
static int smooth_f(Engine& E, int l) {
    const Geo& g = E.gl[l];
    const int N = E.cfg.nstageS, ivis = E.cfg.ivis;
    const float sz = E.cfg.Vbc == 0 ? -1.f : 1.f;
    FOp op = fop(E, l);
    FLev L = flev(E.L[l]);
    dim3 blk(32, 8), grd(nblk(g.nx - 1, 32), nblk(g.nz - 1, 8));
    float* buf[3] = {E.fS0[l], E.fS1[l], E.fS2[l]};
    float* e = E.ferr[l];
    const double c = E.cfg.c_2;  // Nmulti passes: one pass with c = c_2 (Nmulti=1)
    for (int n = 1; n <= E.cfg.Nmulti; n++) {
        KernelTimer kt(E, KT_RKC_FP32_L1, l == 1 ? N : 0);
        int cur = 0;
        PT_COUNT(), k_rkc_stage_f<<<grd, blk, 0, E.st>>>(buf[cur], e, nullptr, nullptr, op, g, L, g.nx, g.nz, 0.f, 0.f, 0.f,
                                                          (float)(E.K.mewt[1] * c), 1, ivis, sz);
        const float* Sm1 = buf[cur];
        const float* Sm2 = e;
        for (int j = 2; j <= N; j++) {
            int nxt = (cur + 1) % 3;
            if (buf[nxt] == Sm2) nxt = (nxt + 1) % 3;
            float* out = (j == N) ? e : buf[nxt];
            PT_COUNT(), k_rkc_stage_f<<<grd, blk, 0, E.st>>>(out, Sm1, Sm2, e, op, g, L, g.nx, g.nz, (float)E.K.cc[j],
                                                              (float)E.K.mew[j], (float)E.K.vv[j],
                                                              (float)(E.K.mewt[j] * c), 0, ivis, sz);
            Sm2 = Sm1;
            Sm1 = out;
            cur = nxt;
        }
        CKL("k_rkc_stage_f");
    }
    PT_COUNT(), k_residual_f<<<grd, blk, 0, E.st>>>(E.fres[l], e, op, g, l, g.nx, g.nz, ivis);
    CKL("k_residual_f");
    return 0;
}

static int coarse_solve_f(Engine& E) {
    const int L = E.grids, n = E.ngc;
    const Geo& g = E.gl[L];
    PT_COUNT(), k_coarse_rhs_f<<<nblk(n, 128), 128, 0, E.st>>>(E.Bc, E.fRHS[L], E.RowB, g, g.nx, g.nz);
    int rc = coarse_band_solve(E);
    if (rc) return rc;
    PT_COUNT(), k_coarse_scatter_f<<<nblk(n, 128), 128, 0, E.st>>>(E.ferr[L], E.Bc, g, g.nx, g.nz);
    CKL("coarse_solve_f");
    return bcs_f(E, L, E.ferr[L]);
}

// part 0: FP64 residual + sum; part 1: FP32 cycle on the correction + FP64 update
static int mixed_part(Engine& E, int part) {
    int rc;
    if (part == 0) return residual_level1(E);
    const Geo& g1 = E.gl[1];
    const size_t n1 = g1.elems();
    PT_COUNT(), k_res_to_f32<<<nblk(n1, 256), 256, 0, E.st>>>(E.fRHS[1], E.res[1], n1);
    const int grids = E.grids, nsteps = E.nsteps;
    const int* multi = E.multi;
    for (int p = 1; p <= nsteps; p++) {
        const int l = multi[p];
        const Geo& g = E.gl[l];
        const bool descend = (p == 1) || multi[p - 1] < multi[p];
        if (descend) {
            if (l > 1) {
                const Geo& gf = E.gl[l - 1];
                PT_COUNT(), k_restrict_f<<<dim3(nblk(g.nx - 1, 128), g.nz - 1), 128, 0, E.st>>>(E.fRHS[l], E.fres[l - 1], g, gf,
                                                                                                 g.nx, g.nz);
            }
            CK(cudaMemsetAsync(E.ferr[l], 0, g.elems() * sizeof(float), E.st));
        }
        if (l < grids) {
            if ((rc = smooth_f(E, l))) return rc;
        } else if ((rc = coarse_solve_f(E))) {
            return rc;
        }
        if (multi[p + 1] < multi[p]) {
            const Geo& gf = E.gl[l - 1];
            PT_COUNT(), k_prolong_f<<<dim3(nblk(gf.nx - 1, 128), gf.nz - 1), 128, 0, E.st>>>(E.ferr[l - 1], E.ferr[l], gf, g,
                                                                                             gf.nx, gf.nz);
            if ((rc = bcs_f(E, l - 1, E.ferr[l - 1]))) return rc;
        }
    }
    PT_COUNT(), k_add_correction<<<dim3(nblk(g1.nx - 1, 128), g1.nz - 1), 128, 0, E.st>>>(E.err[1], E.ferr[1], g1, g1.nx,
                                                                                           g1.nz);
    CKL("mixed cycle");
    return enforce_bcs_stream(E, 1, E.err[1]);
}

static int run_mixed(Engine& E, int part) {
    if (E.prof) return mixed_part(E, part);
    cudaGraphExec_t& ex = part == 0 ? E.gM1 : E.gM2;
    int64_t& n = part == 0 ? E.nM1 : E.nM2;
    if (!ex) {
        cudaGraph_t graph = nullptr;
        int64_t before = g_launches;
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

int multigrid_mixed(Engine& E, pt_solve_info* info) {
    int rc;
    PhaseTimer tm(E, 2);
    if ((rc = mg_setup_solve(E))) return rc;
    for (int l = 1; l < E.grids; l++) {
        size_t n = E.gl[l].elems();
        float* const* f = E.fcoef[l];
        PT_COUNT(), k_coef_to_f32<<<nblk(n, 256), 256, 0, E.st>>>(f[0], f[1], f[2], f[3], f[4], f[5], E.vis[l], E.vx[l],
                                                                  E.vz[l], E.vxz[l], E.vxxmzz[l], E.dtst[l], n);
    }
    CKL("k_coef_to_f32");
    const double norm = (double)(E.gl[1].nx - 2) * (double)(E.gl[1].nz - 2);
    int cycles = 0;
    double mag1 = 0.0;
    for (;;) {
        if ((rc = run_mixed(E, 0))) return rc;
        CK(cudaMemcpyAsync(E.hscal, E.dscal + 8, 8, cudaMemcpyDeviceToHost, E.st));
        CK(cudaStreamSynchronize(E.st));
        mag1 = E.hscal[0] / norm;
        if (!std::isfinite(mag1)) return fail(PT_ERR_NOT_FINITE, "non-finite residual in the mixed-precision solve");
        if (mag1 > 1.0e10 * E.res_ref[1])
            return fail(PT_ERR_MG_DIVERGED, "mixed-precision solve: abnormally high residual");
        if (mag1 / E.res_ref[1] <= E.cfg.tolerance) break;
        if (cycles >= E.cfg.max_cycles)
            return fail(PT_ERR_MG_MAX_CYCLES, "mixed-precision solve: too many cycles");
        if ((rc = run_mixed(E, 1))) return rc;
        cycles++;
    }
    E.cycles = cycles;
    E.refinements = cycles;
    E.resid_ratio = mag1 / E.res_ref[1];
    CK(cudaMemcpyAsync(E.SF, E.err[1], E.g1.elems() * 8, cudaMemcpyDeviceToDevice, E.st));
    if (info) {
        info->cycles += cycles;
        info->resid_ratio = E.resid_ratio;
        info->n_eta = E.n_eta;
        info->eig_fine = E.eig_fine;
    }
    return 0;
}

int mixed_alloc(Engine& E) {
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
