// pt_mg.cu -- the variable-viscosity biharmonic stream-function solve (FP64): multigrid driver
// (iterative_solver.f90:124-341) with the reference's level schedule, the viscosity pipeline
// (compute_viscosity 560-634, smoother_vis smoother.f90:454-580, viscosity_gradients 472-558,
// test_eigenvalues 1147-1211), the RKC1 smoother (iterate_stream 1418-1614), residual (415-470),
// transfers (restrict 1107-1125, prolong 343-396) and the coarsest-grid banded LU
// (Compute_Matrix_coarse 1701-1844 + DGBEQU/DGBTRF/DGBTRS) -- all on the device.
//
// The RKC1 stage kernel fuses stream_derivatives + stream_space + the three-term recurrence +
// enforceBCs_stream: each thread evaluates the 10 stencil derivatives of S_{j-1} at its node
// (separable 5x5/7-point stencils), writes S_j and the antisymmetric ghost images of S_j, so one
// launch is one stage.  Error arrays keep the reference's quirk: error(:,:,2:grids) is never
// reset, so a coarse visit starts from the previous coarse correction.
#include <cmath>
#include <cstring>
#include <vector>

#include "pt_consts.cuh"
#include "pt_exact.cuh"

namespace pt {

int upload_consts_mg(const Engine& E) { return upload_tu_consts(E); }

struct VisSet {
    double *vis, *vx, *vz, *vxx, *vzz, *vxz, *vxxpzz, *vxxmzz, *vsm, *ratio, *dtst;
};

// where a viscosity pass runs and writes: the stream, the test_eig scalars, the work arrays and
// the level arrays (the cycle's own, or the side set of the next time level)
struct VisCtx {
    cudaStream_t st;
    double *dscal, *hscal;
    double* const* visw;
    VisLevels V;
};

static VisLevels primary_levels(Engine& E) {
    VisLevels V{};
    for (int l = 0; l < PT_MAXLEV; l++) {
        V.vis[l] = E.vis[l]; V.visst[l] = E.visst[l]; V.vx[l] = E.vx[l]; V.vz[l] = E.vz[l]; V.vxx[l] = E.vxx[l];
        V.vzz[l] = E.vzz[l]; V.vxz[l] = E.vxz[l]; V.vxxpzz[l] = E.vxxpzz[l]; V.vxxmzz[l] = E.vxxmzz[l];
        V.vsm[l] = E.vsm[l]; V.ratio[l] = E.ratio[l]; V.dtst[l] = E.dtst[l];
    }
    return V;
}
static VisCtx primary_ctx(Engine& E) { return VisCtx{E.st, E.dscal, E.hscal, E.visw, primary_levels(E)}; }
static VisCtx side_ctx(Engine& E) { return VisCtx{E.st2, E.dscal2, E.hscal2, E.visw2, E.vl2}; }

static VisSet level_set(const VisLevels& V, int l) {
    return VisSet{V.vis[l], V.vx[l], V.vz[l], V.vxx[l], V.vzz[l], V.vxz[l], V.vxxpzz[l], V.vxxmzz[l],
                  V.vsm[l], V.ratio[l], V.dtst[l]};
}

// ------------------------------------------------------------------ viscosity pipeline
// visf, rheology.f90:2-23
__global__ void k_visf(double* visst, const double* Tvis, const double* Cvis, Geo g) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i > cK.nx) return;
    double z = (double)k * cK.ds;
    if (k == 0) z = 0.0;
    if (k == cK.nz) z = 1.0;
    double v;
    if (cK.ivis == 1) v = exp(-Tvis[g.at(i, k)] * cK.lvisT + (1.0 - z) * cK.lvisP);
    else if (cK.ivis == 2 && cK.comp == 1) {
        double dot = 0.0 + Cvis[g.at(i, k)] * cK.lvisC;
        v = exp(-Tvis[g.at(i, k)] * cK.lvisT - dot + (1.0 - z) * cK.lvisP);
    } else v = 1.0;
    visst[g.at(i, k)] = v;
}

// viscosityBCs (iterative_solver.f90:666-690): phase 1 column ghosts over all rows (the row
// ghosts still hold the previous values there), phase 2 row ghosts for columns 0..nx.
__global__ void k_visbc_cols(double* v, Geo g, int nx, int nz) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 6 * (nz + 7)) return;
    int k = idx / 6 - 3, q = idx % 6;
    int j = q % 3 + 1;
    if (q < 3) v[g.at(-j, k)] = v[g.at(j, k)];
    else v[g.at(nx + j, k)] = v[g.at(nx - j, k)];
}
__global__ void k_visbc_rows(double* v, Geo g, int nx, int nz) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 6 * (nx + 1)) return;
    int i = idx / 6, q = idx % 6;
    int j = q % 3 + 1;
    if (q < 3) v[g.at(i, -j)] = v[g.at(i, j)];
    else v[g.at(i, nz + j)] = v[g.at(i, nz - j)];
}
static int vis_bcs(Engine& E, double* v, int l, cudaStream_t st) {
    const Geo& g = E.gl[l];
    PT_COUNT(), k_visbc_cols<<<nblk(6 * (g.nz + 7), 128), 128, 0, st>>>(v, g, g.nx, g.nz);
    PT_COUNT(), k_visbc_rows<<<nblk(6 * (g.nx + 1), 128), 128, 0, st>>>(v, g, g.nx, g.nz);
    CKL("vis_bcs");
    return 0;
}

// c + a b: fused (fma) for the fast paths, two roundings in the reference's order for the FP64
// path with reference_rounding (this file is compiled with --fmad=false, so only fma() fuses)
template <bool FUSED>
__device__ __forceinline__ double madd(double a, double b, double c) {
    return FUSED ? fma(a, b, c) : c + a * b;
}

// viscosity_gradients, second-order stencils (uniform grid)
template <bool FUSED>
__global__ void k_vis_grad(VisSet S, Geo g, int l, int full, int ivis) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    const LevConst& L = cL[l];
    if (i > L.nx) return;
    size_t o = g.at(i, k);
    if (ivis == 0) {
        S.vx[o] = 0; S.vz[o] = 0; S.vxx[o] = 0; S.vzz[o] = 0; S.vxz[o] = 0; S.vxxpzz[o] = 0; S.vxxmzz[o] = 0;
        return;
    }
    const double* v = S.vis;
    double xx = 0.0, zz = 0.0;
    for (int j = -1; j <= 1; j++) xx = madd<FUSED>(cK.D2so[j + 1], v[g.at(i + j, k)], xx);
    xx = qdiv(xx, L.dr2, L.idr2);
    for (int j = -1; j <= 1; j++) zz = madd<FUSED>(cK.D2so[j + 1], v[g.at(i, k + j)], zz);
    zz = qdiv(zz, L.ds2, L.ids2);
    if (full) {
        double xz = 0.0, x = 0.0, z = 0.0;
        for (int k2 = -1; k2 <= 1; k2++)
            for (int i2 = -1; i2 <= 1; i2++) xz = madd<FUSED>(cK.Drsso[i2 + 1][k2 + 1], v[g.at(i + i2, k + k2)], xz);
        for (int j = -1; j <= 1; j++) x = madd<FUSED>(cK.D1so[j + 1], v[g.at(i + j, k)], x);
        for (int j = -1; j <= 1; j++) z = madd<FUSED>(cK.D1so[j + 1], v[g.at(i, k + j)], z);
        S.vxz[o] = qdiv(xz, L.drds, L.idrds);
        S.vx[o] = qdiv(x, L.dr, L.idr);
        S.vz[o] = qdiv(z, L.ds, L.ids);
        S.vxxmzz[o] = xx - zz;
    }
    S.vxx[o] = xx;
    S.vzz[o] = zz;
    S.vxxpzz[o] = xx + zz;
    S.vsm[o] = L.dt_vis * (xx + zz);
}

// test_eigenvalues (RKC1 branch): ratio, local pseudo-time step, min ratio
// FEW (mixed precision): the pseudo-time step with two divisions instead of four, by the
// reciprocals of ae and be (the step feeds an FP32 smoother there); the ratio keeps its division.
// FUSED: the sums as fused multiply-adds (not with reference_rounding).
template <bool FEW, bool FUSED>
__global__ void k_test_eig(VisSet S, Geo g, int l, double ae, double be, double ctemp, unsigned long long* rmin) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    const LevConst& L = cL[l];
    double ratio = 1.0e100;
    if (i <= L.nx - 1) {
        size_t o = g.at(i, k);
        double vg = S.vis[o];
        double eI = madd<FUSED>(vg, L.SI2, fabs(S.vxxpzz[o] * L.SI1)) + fabs(S.vxz[o] * L.SI4) + fabs(S.vx[o] * L.SI5) +
                    fabs(S.vz[o] * L.SI6);
        double eR = madd<FUSED>(vg, L.SR2, S.vxxmzz[o] * L.SR1);
        eR = madd<FUSED>(S.vxz[o], L.SR4, eR);
        eR = madd<FUSED>(S.vx[o], L.SR5, eR);
        eR = madd<FUSED>(S.vz[o], L.SR6, eR);
        ratio = fabs(eR / eI);
        S.ratio[o] = ratio;
        const double a = FEW ? eR * ae : eR / ae, b = FEW ? eI * be : eI / be;  // FEW: ae, be are 1/ae, 1/be
        S.dtst[o] = ctemp * eR / madd<FUSED>(a, a, b * b);
    }
    double m = fmin(ratio, 1.0e100);
    for (int off = 16; off > 0; off >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMin(rmin, (unsigned long long)__double_as_longlong(m));
}

// The smoothing update v += c vsm (smoother_vis) followed by viscosityBCs, in one pass.  Every node writes its own mirror images:
// the column and row ghosts take the updated value; a corner ghost is what viscosityBCs' column
// phase copies from the row ghost of the mirrored column, which still holds what the previous
// call wrote there: the mirrored node's value before this update.  (The first call of a smoothing
// pass is a plain vis_bcs, so that previous call always exists.)
template <bool FUSED>
__global__ void k_vis_update_bc(double* v, const double* vsm, Geo g, int nx, int nz, double c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i > nx) return;
    const size_t o = g.at(i, k);
    const double old = v[o];
    const double nv = madd<FUSED>(c, vsm[o], old);
    v[o] = nv;
    int xs[2], zs[2], nxm = 0, nzm = 0;
    if (i >= 1 && i <= 3) xs[nxm++] = -i;
    if (i >= nx - 3 && i <= nx - 1) xs[nxm++] = 2 * nx - i;
    if (k >= 1 && k <= 3) zs[nzm++] = -k;
    if (k >= nz - 3 && k <= nz - 1) zs[nzm++] = 2 * nz - k;
    for (int a = 0; a < nxm; a++) v[g.at(xs[a], k)] = nv;
    for (int b = 0; b < nzm; b++) v[g.at(i, zs[b])] = nv;
    for (int a = 0; a < nxm; a++)
        for (int b = 0; b < nzm; b++) v[g.at(xs[a], zs[b])] = old;
}

static const double kPi = 3.1415926535897932;

// smoother_vis (smoother.f90:454-580) on the arrays of set S at level l
static int smoother_vis(Engine& E, const VisCtx& C, int l, int interpolate, VisSet S, int record) {
    const Geo& g = E.gl[l];
    const int nx = g.nx, nz = g.nz, ivis = E.cfg.ivis;
    int rc;
    if ((rc = vis_bcs(E, S.vis, l, C.st))) return rc;
    int option, Niter;
    double lb, la;
    if (interpolate == 0) { option = 1; Niter = 3; lb = -3.0; la = -2.0; }
    else { option = 0; Niter = E.cfg.vis_iter; lb = -2.0; la = -1.0; }
    int Nvis_store = 0, nn_store = 1, n = 0, trigger = 0;
    double ratio_min = 1.0e100;
    // the pseudo-time step (test_eigenvalues) matches the smoother that will run on level l: the
    // mixed V-cycle's coarse-level smoother has its own stage count
    const bool coarse_smoother = E.cfg.precision == PT_PREC_MIXED && l >= 2;
    const double stab = coarse_smoother ? E.RKC1_stability_c : E.RKC1_stability;
    const double ae = -stab / 2.0, be = (double)(coarse_smoother ? E.nstageC : E.cfg.nstageS);
    const double ctemp = E.cfg.courant_stream * (stab / (ae * ae));
    const bool fused = !E.cfg.reference_rounding;
    dim3 gg(nblk(nx + 1, 128), nz + 1);
    for (int guard = 0; guard < 100000; guard++) {
        for (int nn = nn_store; nn <= Niter; nn++) {
            PT_COUNT(), (fused ? k_vis_grad<true> : k_vis_grad<false>)<<<gg, 128, 0, C.st>>>(S, g, l, Nvis_store != 0,
                                                                                        ivis);
            CKL("k_vis_grad");
            if (interpolate == 0 && (Nvis_store >= 1 || ivis == 0)) {
                unsigned long long* d = (unsigned long long*)C.dscal;
                unsigned long long init = (unsigned long long)__builtin_bit_cast(long long, 1.0e100);
                CK(cudaMemcpyAsync(d, &init, 8, cudaMemcpyHostToDevice, C.st));
                dim3 ge(nblk(nx - 1, 128), nz - 1);
                if (E.cfg.precision == PT_PREC_MIXED)
                    PT_COUNT(), k_test_eig<true, true><<<ge, 128, 0, C.st>>>(S, g, l, 1.0 / ae, 1.0 / be, ctemp, d);
                else if (fused)
                    PT_COUNT(), k_test_eig<false, true><<<ge, 128, 0, C.st>>>(S, g, l, ae, be, ctemp, d);
                else
                    PT_COUNT(), k_test_eig<false, false><<<ge, 128, 0, C.st>>>(S, g, l, ae, be, ctemp, d);
                CKL("k_test_eig");
                CK(cudaMemcpyAsync(C.hscal, d, 8, cudaMemcpyDeviceToHost, C.st));
                CK(cudaStreamSynchronize(C.st));
                ratio_min = C.hscal[0];
            }
            if (option == 1) {
                if ((Nvis_store >= 1 && ratio_min > E.cfg.eig_ratio_min) || ivis == 0 || n > 20) {
                    if (record) { E.eig_fine = ratio_min; E.n_eta = n; }
                    trigger = 1;
                    break;
                }
            } else if (interpolate == 0) {
                if (ratio_min > E.cfg.eig_ratio || ivis == 0) { trigger = 1; nn_store = nn; break; }
            } else if (Nvis_store >= 1 || ivis == 0) {
                trigger = 1;
                break;
            }
            int ntemp = Niter - nn + 1;
            double c = 2.0 / (-lb - la + (lb - la) * std::cos((double)(2 * ntemp - 1) * kPi / (double)(2 * Niter)));
            c = 0.99 * c;
            PT_COUNT(), (fused ? k_vis_update_bc<true> : k_vis_update_bc<false>)<<<gg, 128, 0, C.st>>>(S.vis, S.vsm, g, nx,
                                                                                                  nz, c);
            CKL("k_vis_update_bc");
        }
        if (trigger) return 0;
        Nvis_store++;
        nn_store = 1;
        if (option == 1) { Niter = 6; lb = -2.0; la = -1.0; }
        n++;
    }
    return fail(PT_ERR_ITER_CAP, "viscosity smoother exceeded its iteration cap");
}

// restrict_coefficients / restrict: full weighting onto coarse interior nodes
__global__ void k_restrict(double* out, const double* in, Geo gc, Geo gf, int nxc, int nzc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nxc - 1) return;
    int ii = 2 * i, kk = 2 * k;
    double corners = (in[gf.at(ii - 1, kk - 1)] + in[gf.at(ii - 1, kk + 1)] + in[gf.at(ii + 1, kk + 1)] + in[gf.at(ii + 1, kk - 1)]) / 16.0;
    double sides = (in[gf.at(ii - 1, kk)] + in[gf.at(ii, kk - 1)] + in[gf.at(ii + 1, kk)] + in[gf.at(ii, kk + 1)]) / 8.0;
    double centre = in[gf.at(ii, kk)] / 4.0;
    out[gc.at(i, k)] = corners + sides + centre;
}

// viscosityBCs_initialize (iterative_solver.f90:636-664)
__global__ void k_visbc_init(double* v, const double* vf, Geo g, Geo gf, int nx, int nz, int nxf, int nzf) {
    int W = nx + 7;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * (nz + 7)) return;
    int i = idx % W - 3, k = idx / W - 3;
    bool xin = (i >= 0 && i <= nx), zin = (k >= 0 && k <= nz);
    if (xin && zin && i > 0 && i < nx && k > 0 && k < nz) return;  // interior: restricted values
    int mi = mirror_idx(i, nx), mk = mirror_idx(k, nz);
    // boundary value of the mirrored boundary node, taken from the finer level by injection
    double val;
    if (mk == 0) val = vf[gf.at(2 * mi, 0)];
    else if (mk == nz) val = vf[gf.at(2 * mi, nzf)];
    else if (mi == 0) val = vf[gf.at(0, 2 * mk)];
    else if (mi == nx) val = vf[gf.at(nxf, 2 * mk)];
    else val = v[g.at(mi, mk)];  // ghost of an interior node
    v[g.at(i, k)] = val;
}

static int compute_viscosity(Engine& E, const VisCtx& C, int level) {
    int rc;
    const Geo& g = E.gl[level];
    const VisLevels& V = C.V;
    if (level == 1) {
        dim3 gg(nblk(g.nx + 1, 128), g.nz + 1);
        PT_COUNT(), k_visf<<<gg, 128, 0, C.st>>>(V.visst[1], E.Tvis, E.Cvis, g);
        CKL("k_visf");
        CK(cudaMemcpyAsync(V.vis[1], V.visst[1], g.elems() * 8, cudaMemcpyDeviceToDevice, C.st));
        return smoother_vis(E, C, 1, 0, level_set(V, 1), 1);
    }
    const int lf = level - 1;
    const Geo& gf = E.gl[lf];
    // smooth a work copy of the finer static viscosity (the reference smooths in place and
    // restores the finer level's arrays afterwards)
    VisSet W{C.visw[0], C.visw[1], C.visw[2], C.visw[3], C.visw[4], C.visw[5], C.visw[6], C.visw[7],
             C.visw[8], C.visw[9], C.visw[10]};
    CK(cudaMemcpyAsync(W.vis, V.visst[lf], gf.elems() * 8, cudaMemcpyDeviceToDevice, C.st));
    if ((rc = smoother_vis(E, C, lf, 1, W, 0))) return rc;
    dim3 gr(nblk(g.nx - 1, 128), g.nz - 1);
    PT_COUNT(), k_restrict<<<gr, 128, 0, C.st>>>(V.vis[level], W.vis, g, gf, g.nx, g.nz);
    int tot = (g.nx + 7) * (g.nz + 7);
    PT_COUNT(), k_visbc_init<<<nblk(tot, 128), 128, 0, C.st>>>(V.vis[level], W.vis, g, gf, g.nx, g.nz, gf.nx, gf.nz);
    CKL("restrict_coefficients");
    CK(cudaMemcpyAsync(V.visst[level], V.vis[level], g.elems() * 8, cudaMemcpyDeviceToDevice, C.st));
    return smoother_vis(E, C, level, 0, level_set(V, level), 0);
}

// ------------------------------------------------------------------ RHS and residual norms
__global__ void k_rhs1(double* RHS, const double* Tb, const double* Cb, Geo g, int comp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > cK.nx - 1) return;
    double v = 0.0;
    if (cK.RaT != 0.0) {
        double tr = 0.0;
        for (int j = -2; j <= 2; j++) tr = tr + cK.D1[3 + j] * Tb[g.at(i + j, k)];
        v = cK.RaT * qdiv(tr, cK.dr, cK.inv_dr);  // (the reference's / 1.0 is exact)
    }
    if (comp) {
        double cr = 0.0;
        for (int j = -2; j <= 2; j++) cr = cr + cK.D1[3 + j] * Cb[g.at(i + j, k)];
        v = v - cK.RaC * qdiv(cr, cK.dr, cK.inv_dr);
    }
    RHS[g.at(i, k)] = v;
}

static int compute_RHS(Engine& E, int level) {
    const Geo& g = E.gl[level];
    dim3 gr(nblk(g.nx - 1, 128), g.nz - 1);
    if (level == 1) PT_COUNT(), k_rhs1<<<gr, 128, 0, E.st>>>(E.RHS[1], E.Tbuoy, E.Cbuoy, g, E.cfg.comp);
    else PT_COUNT(), k_restrict<<<gr, 128, 0, E.st>>>(E.RHS[level], E.res[level - 1], g, E.gl[level - 1], g.nx, g.nz);
    CKL("compute_RHS");
    return 0;
}

static int mean_abs(Engine& E, const double* f, int level, double* host_out) {
    const Geo& g = E.gl[level];
    int rc = reduce_sum_abs_interior(E, f, g.nx, g.nz, g.pitch, E.dscal + 8);
    if (rc) return rc;
    CK(cudaMemcpyAsync(E.hscal, E.dscal + 8, 8, cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    *host_out = E.hscal[0] / (double)(g.nx - 2) / (double)(g.nz - 2);
    return 0;
}

// ------------------------------------------------------------------ RKC1 stage kernel
struct StreamOp {
    const double *vis, *vx, *vz, *vxz, *vxxmzz, *rhs, *dtst;
};

// -(stream operator - RHS) at node (i,k) of S: stream_derivatives (iterative_solver.f90:973-1073)
// and stream_space (890-911) with the reference's operations in the reference's order -- each
// derivative a sum over its full stencil (zero weights included) divided by the spacing power,
// the cross derivatives as 25-point sums, no fused multiply-adds (this file is compiled with
// --fmad=false) -- so that the FP64 path with reference_rounding rounds like the reference.
__device__ __forceinline__ double stream_F(const double* __restrict__ S, Geo g, const LevConst& L,
                                           const StreamOp& op, int i, int k, int ivis) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (int j = -2; j <= 2; j++) a += cK.D2[j + 3] * S[g.at(i + j, k)];
    for (int j = -3; j <= 3; j++) b += cK.D3[j + 3] * S[g.at(i + j, k)];
    for (int j = -3; j <= 3; j++) c += cK.D4[j + 3] * S[g.at(i + j, k)];
    const double Sxx = a / L.dr2, Sxxx = b / L.dr3, Sxxxx = c / L.dr4;
    a = 0.0; b = 0.0; c = 0.0;
    for (int j = -2; j <= 2; j++) a += cK.D2[j + 3] * S[g.at(i, k + j)];
    for (int j = -3; j <= 3; j++) b += cK.D3[j + 3] * S[g.at(i, k + j)];
    for (int j = -3; j <= 3; j++) c += cK.D4[j + 3] * S[g.at(i, k + j)];
    const double Szz = a / L.ds2, Szzz = b / L.ds3, Szzzz = c / L.ds4;
    double xz = 0.0, xxz = 0.0, xzz = 0.0, xxzz = 0.0;
    for (int k2 = -2; k2 <= 2; k2++)
        for (int i2 = -2; i2 <= 2; i2++) {
            const double v = S[g.at(i + i2, k + k2)];
            xz += cK.Drs[i2 + 2][k2 + 2] * v;
            xxz += cK.Drrs[i2 + 2][k2 + 2] * v;
            xzz += cK.Drss[i2 + 2][k2 + 2] * v;
            xxzz += cK.Drrss[i2 + 2][k2 + 2] * v;
        }
    const double Sxz = xz / L.drds, Sxxz = xxz / L.dr2ds, Sxzz = xzz / L.drds2, Sxxzz = xxzz / L.dr2ds2;
    size_t o = g.at(i, k);
    double r;
    double t2 = op.vis[o] * (Sxxxx + Szzzz + 2.0 * Sxxzz);
    if (ivis == 0) r = t2 - op.rhs[o];
    else {
        double t1 = op.vxxmzz[o] * (Sxx - Szz);
        double t4 = 4.0 * op.vxz[o] * Sxz;
        double t5 = 2.0 * op.vx[o] * (Sxxx + Sxzz);
        double t6 = 2.0 * op.vz[o] * (Szzz + Sxxz);
        r = t1 + t2 + t4 + t5 + t6 - op.rhs[o];
    }
    return -r;
}

// writes value v of interior node (i,k) of out and its free-slip ghost images: the mirror
// across a side wall flips the sign, across top/bottom it multiplies by sz (-1 free slip, +1 rigid)
__device__ __forceinline__ void store_with_ghosts(double* out, Geo g, int i, int k, int nx, int nz, double v,
                                                  double sz) {
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

// zero the boundary lines and their ghost images (done once per buffer per pass)
__global__ void k_stream_zero_bnd(double* out, Geo g, int nx, int nz) {
    int W = nx + 7;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * (nz + 7)) return;
    int i = idx % W - 3, k = idx / W - 3;
    if (i == 0 || i == nx || k == 0 || k == nz) out[g.at(i, k)] = 0.0;
    else if ((i < 0 || i > nx) && (k == 0 || k == nz)) out[g.at(i, k)] = 0.0;
}

// one RKC1 stage: out = cS0*S0 + mew*S1 + v*S2 + (mewt*c)*dt*F(S1)   (stage 1: S0 + (mewt*c)*dt*F(S0))
__global__ void __launch_bounds__(128) k_rkc_stage(double* __restrict__ out, const double* __restrict__ S1,
                                                   const double* __restrict__ S2, const double* __restrict__ S0,
                                                   StreamOp op, Geo g, int l, double cS0, double mew, double vv,
                                                   double mewtc, int first, int ivis, double sz) {
    const LevConst& L = cL[l];
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > L.nx - 1) return;
    double F = stream_F(S1, g, L, op, i, k, ivis);
    size_t o = g.at(i, k);
    double v;
    if (first) v = S1[o] + mewtc * op.dtst[o] * F;
    else v = cS0 * S0[o] + mew * S1[o] + vv * S2[o] + mewtc * op.dtst[o] * F;
    store_with_ghosts(out, g, i, k, L.nx, L.nz, v, sz);
}

// k_rkc_stage with the stream operator's stencil sums formed exactly (pt_exact.cuh); a CTA owns a
// TG::TX x TG::TZ tile of nodes.
template <bool SQUARE, class TG>
__global__ void __launch_bounds__(TG::NT) k_rkc_stage_fx(double* __restrict__ out, const double* __restrict__ S1,
                                                         const double* __restrict__ S2, const double* __restrict__ S0,
                                                         StreamOp op, Geo g, int l, double cS0, double mew, double vv,
                                                         double mewtc, int first, int ivis, double sz, ResFxK K) {
    __shared__ int2 X[TG::HT][TG::W];
    __shared__ int emax_s;
    const LevConst& L = cL[l];
    const int i0 = blockIdx.x * TG::TX + 1, k0 = blockIdx.y * TG::TZ + 1;
    const int emax = load_tile_fx<TG>(X, &emax_s, S1, g, i0, k0, L.nx, L.nz);
#pragma unroll 1
    for (int r = 0; r < TG::RPT; r++) {
        const int lx = threadIdx.x, lz = threadIdx.y + TG::TY * r;
        const int i = i0 + lx, k = k0 + lz;
        if (i > L.nx - 1 || k > L.nz - 1) continue;
        const size_t o = g.at(i, k);
        const double F = op.rhs[o] - tile_apply_A<SQUARE>(X, lx + TG::H, lz + TG::H, emax, op.vis, op.vx, op.vz, op.vxz,
                                                          op.vxxmzz, o, ivis, K);
        double v;
        if (first) v = S1[o] + mewtc * op.dtst[o] * F;
        else v = cS0 * S0[o] + mew * S1[o] + vv * S2[o] + mewtc * op.dtst[o] * F;
        store_with_ghosts(out, g, i, k, L.nx, L.nz, v, sz);
    }
}

// k_residual with exact stencil sums
template <bool SQUARE, class TG>
__global__ void __launch_bounds__(TG::NT) k_residual_fx64(double* __restrict__ res, const double* __restrict__ S,
                                                          StreamOp op, Geo g, int l, int ivis, ResFxK K) {
    __shared__ int2 X[TG::HT][TG::W];
    __shared__ int emax_s;
    const LevConst& L = cL[l];
    const int i0 = blockIdx.x * TG::TX + 1, k0 = blockIdx.y * TG::TZ + 1;
    const int emax = load_tile_fx<TG>(X, &emax_s, S, g, i0, k0, L.nx, L.nz);
#pragma unroll 1
    for (int r = 0; r < TG::RPT; r++) {
        const int lx = threadIdx.x, lz = threadIdx.y + TG::TY * r;
        const int i = i0 + lx, k = k0 + lz;
        if (i > L.nx - 1 || k > L.nz - 1) continue;
        const size_t o = g.at(i, k);
        res[o] = op.rhs[o] - tile_apply_A<SQUARE>(X, lx + TG::H, lz + TG::H, emax, op.vis, op.vx, op.vz, op.vxz,
                                                  op.vxxmzz, o, ivis, K);
    }
}

// residual = -(L S - RHS) on the interior (compute_residual)
__global__ void k_residual(double* __restrict__ res, const double* __restrict__ S, StreamOp op, Geo g, int l, int ivis) {
    const LevConst& L = cL[l];
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > L.nx - 1) return;
    res[g.at(i, k)] = stream_F(S, g, L, op, i, k, ivis);
}

// full free-slip ghost/boundary fill of a level array (enforceBCs_stream)
__global__ void k_stream_bcs(double* S, Geo g, int nx, int nz, double sz) {
    int W = nx + 7;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * (nz + 7)) return;
    int i = idx % W - 3, k = idx / W - 3;
    bool xin = (i > 0 && i < nx), zin = (k > 0 && k < nz);
    if (xin && zin) return;
    int mi = mirror_idx(i, nx), mk = mirror_idx(k, nz);
    double v;
    if (mi == 0 || mi == nx || mk == 0 || mk == nz) v = 0.0;
    else {
        double s = 1.0;
        if (i < 0 || i > nx) s = -s;
        if (k < 0 || k > nz) s = s * sz;
        v = s * S[g.at(mi, mk)];
    }
    S[g.at(i, k)] = v;
}

int enforce_bcs_stream(Engine& E, int level, double* f) {
    const Geo& g = E.gl[level];
    int tot = (g.nx + 7) * (g.nz + 7);
    PT_COUNT(), k_stream_bcs<<<nblk(tot, 256), 256, 0, E.st>>>(f, g, g.nx, g.nz, E.cfg.Vbc == 0 ? -1.0 : 1.0);
    CKL("k_stream_bcs");
    return 0;
}

static StreamOp stream_op(Engine& E, int l) {
    return StreamOp{E.vis[l], E.vx[l], E.vz[l], E.vxz[l], E.vxxmzz[l], E.RHS[l], E.dtst[l]};
}

// one RKC1 stage / one residual on level l: the exact-sum kernels when the stencils allow them
static void launch_stage(Engine& E, int l, double* out, const double* S1, const double* S2, const double* S0,
                         const StreamOp& op, double cS0, double mew, double vv, double mewtc, int first, double sz) {
    const Geo& g = E.gl[l];
    const int ivis = E.cfg.ivis;
    if (E.res_int) {
        const bool sq = E.resfx[l].square;
        if (use_big_tiles(g.nx, g.nz)) {
            dim3 blk(TileBig::TX, TileBig::TY), grd(nblk(g.nx - 1, TileBig::TX), nblk(g.nz - 1, TileBig::TZ));
            auto kern = sq ? k_rkc_stage_fx<true, TileBig> : k_rkc_stage_fx<false, TileBig>;
            PT_COUNT(), kern<<<grd, blk, 0, E.st>>>(out, S1, S2, S0, op, g, l, cS0, mew, vv, mewtc, first, ivis, sz,
                                                    E.resfx[l]);
        } else {
            dim3 blk(TileSmall::TX, TileSmall::TY), grd(nblk(g.nx - 1, TileSmall::TX), nblk(g.nz - 1, TileSmall::TZ));
            auto kern = sq ? k_rkc_stage_fx<true, TileSmall> : k_rkc_stage_fx<false, TileSmall>;
            PT_COUNT(), kern<<<grd, blk, 0, E.st>>>(out, S1, S2, S0, op, g, l, cS0, mew, vv, mewtc, first, ivis, sz,
                                                    E.resfx[l]);
        }
    } else {
        dim3 gs(nblk(g.nx - 1, 128), g.nz - 1);
        PT_COUNT(), k_rkc_stage<<<gs, 128, 0, E.st>>>(out, S1, S2, S0, op, g, l, cS0, mew, vv, mewtc, first, ivis, sz);
    }
}
static void launch_residual(Engine& E, int l, double* res, const double* S, const StreamOp& op) {
    const Geo& g = E.gl[l];
    if (E.res_int) {
        const bool sq = E.resfx[l].square;
        if (use_big_tiles(g.nx, g.nz)) {
            dim3 blk(TileBig::TX, TileBig::TY), grd(nblk(g.nx - 1, TileBig::TX), nblk(g.nz - 1, TileBig::TZ));
            auto kern = sq ? k_residual_fx64<true, TileBig> : k_residual_fx64<false, TileBig>;
            PT_COUNT(), kern<<<grd, blk, 0, E.st>>>(res, S, op, g, l, E.cfg.ivis, E.resfx[l]);
        } else {
            dim3 blk(TileSmall::TX, TileSmall::TY), grd(nblk(g.nx - 1, TileSmall::TX), nblk(g.nz - 1, TileSmall::TZ));
            auto kern = sq ? k_residual_fx64<true, TileSmall> : k_residual_fx64<false, TileSmall>;
            PT_COUNT(), kern<<<grd, blk, 0, E.st>>>(res, S, op, g, l, E.cfg.ivis, E.resfx[l]);
        }
    } else {
        PT_COUNT(), k_residual<<<dim3(nblk(g.nx - 1, 128), g.nz - 1), 128, 0, E.st>>>(res, S, op, g, l, E.cfg.ivis);
    }
}

// iterate_stream (RKC1 = 1, splitting = 0) + compute_residual.  The last stage writes straight
// into error(:,:,level): a stage reads S0 only at its own node, so the update is safe in place.
// With want_sum the sum of |residual| is left in dscal[8] (no host synchronisation, so the
// sequence can be captured in a CUDA graph).  The boundary lines of the stage buffers are zero
// from allocation and are never written by the stage kernel.
static int iterate_stream(Engine& E, int l, int want_sum) {
    const Geo& g = E.gl[l];
    const int N = E.cfg.nstageS, Niter = E.cfg.Nmulti;
    const double sz = E.cfg.Vbc == 0 ? -1.0 : 1.0;
    StreamOp op = stream_op(E, l);
    double* buf[3] = {E.S0[l], E.S1[l], E.S2[l]};
    for (int n = 1; n <= Niter; n++) {
        int ntemp = Niter - n + 1;
        double temp = (E.cfg.Nmulti > 1) ? (E.cfg.c_2 - E.cfg.c_1) * (double)(ntemp - 1) / (double)(1 - Niter) : 0.0;
        double c = temp + E.cfg.c_2;
        const double* S0 = E.err[l];
        GraphTimer gt(E, 0, (l == 1 && want_sum) ? N : 0);
        int cur = 0;
        launch_stage(E, l, buf[cur], S0, nullptr, nullptr, op, 0, 0, 0, E.K.mewt[1] * c, 1, sz);
        const double* Sm1 = buf[cur];
        const double* Sm2 = S0;
        for (int j = 2; j <= N; j++) {
            int nxt = (cur + 1) % 3;
            if (buf[nxt] == Sm2) nxt = (nxt + 1) % 3;
            double* out = (j == N) ? E.err[l] : buf[nxt];
            launch_stage(E, l, out, Sm1, Sm2, S0, op, E.K.cc[j], E.K.mew[j], E.K.vv[j], E.K.mewt[j] * c, 0, sz);
            Sm2 = Sm1;
            Sm1 = out;
            cur = nxt;
        }
        CKL("k_rkc_stage");
    }
    launch_residual(E, l, E.res[l], E.err[l], op);
    CKL("k_residual");
    if (want_sum) return reduce_sum_abs_interior(E, E.res[l], g.nx, g.nz, g.pitch, E.dscal + 8);
    return 0;
}

// prolong (iterative_solver.f90:343-396): bilinear coarse correction added to the finer level
__global__ void k_prolong(double* F, const double* C, Geo gf, Geo gc, int nxf, int nzf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y + 1;
    if (i > nxf - 1) return;
    double add;
    if (!(i & 1) && !(k & 1)) add = C[gc.at(i / 2, k / 2)];
    else if (!(i & 1)) add = (C[gc.at(i / 2, (k - 1) / 2)] + C[gc.at(i / 2, (k + 1) / 2)]) / 2.0;
    else if (!(k & 1)) add = (C[gc.at((i - 1) / 2, k / 2)] + C[gc.at((i + 1) / 2, k / 2)]) / 2.0;
    else
        add = (C[gc.at((i - 1) / 2, (k - 1) / 2)] + C[gc.at((i + 1) / 2, (k - 1) / 2)] +
               C[gc.at((i + 1) / 2, (k + 1) / 2)] + C[gc.at((i - 1) / 2, (k + 1) / 2)]) / 4.0;
    size_t o = gf.at(i, k);
    F[o] = F[o] + add;
}

static int prolong(Engine& E, int lc) {
    const int lf = lc - 1;
    const Geo &gf = E.gl[lf], &gc = E.gl[lc];
    dim3 gp(nblk(gf.nx - 1, 128), gf.nz - 1);
    PT_COUNT(), k_prolong<<<gp, 128, 0, E.st>>>(E.err[lf], E.err[lc], gf, gc, gf.nx, gf.nz);
    CKL("k_prolong");
    return enforce_bcs_stream(E, lf, E.err[lf]);
}

// ------------------------------------------------------------------ coarsest level
// Compute_Matrix_coarse (analysis=0) rows in LAPACK band storage, one thread per row
__global__ void k_coarse_matrix(double* M, Geo g, int l, int kl, int ku, int n, double* RowB, int Vbc, int ivis,
                                const double* vis, const double* vx, const double* vz, const double* vxz,
                                const double* vxxmzz, int* err) {
    int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (p > n) return;
    const LevConst& L = cL[l];
    const int nxc = L.nx, nzc = L.nz, N = nzc + 1, ldab = 2 * kl + ku + 1, kk1 = kl + ku + 1;
    const int reach[7] = {0, 2, 2, 3, 2, 2, 0};
    int ip = (p - 1) / N, kp = (p - 1) % N;
#define MB(row, col) M[(size_t)((row) - 1) + (size_t)((col) - 1) * (size_t)ldab]
    for (int q = (p - kl > 1 ? p - kl : 1); q <= (p + ku < n ? p + ku : n); q++) MB(kk1 + p - q, q) = 0.0;
    if (ip > 0 && ip < nxc && kp > 0 && kp < nzc) {
        size_t o = g.at(ip, kp);
        double a1 = vxxmzz[o], a2 = vis[o], a4 = vxz[o], a5 = vx[o], a6 = vz[o];
        for (int pass = 0; pass < 2; pass++)
            for (int j = -3; j <= 3; j++) {
                int iq = j + ip;
                for (int kq = kp - reach[j + 3]; kq <= kp + reach[j + 3]; kq++) {
                    bool inside = (iq >= 0 && iq <= nxc && kq >= 0 && kq <= nzc);
                    if ((pass == 0) != inside) continue;
                    int di = iq - ip + 3, dk = kq - kp + 3;
                    double v = (ivis == 0) ? a2 * cK.SM2[di][dk]
                                           : a1 * cK.SM1[di][dk] + a2 * cK.SM2[di][dk] + a4 * cK.SM4[di][dk] +
                                                 a5 * cK.SM5[di][dk] + a6 * cK.SM6[di][dk];
                    if (pass == 0) {
                        int q = N * iq + kq + 1;
                        MB(kk1 + p - q, q) = v;
                    } else {
                        int iiq = iq, kkq = kq, sv = 1;
                        if (iq < 0) { iiq = -iq; sv = -sv; }
                        else if (iq > nxc) { iiq = 2 * nxc - iq; sv = -sv; }
                        if (kq < 0) { kkq = -kq; if (Vbc == 0) sv = -sv; }
                        else if (kq > nzc) { kkq = 2 * nzc - kq; if (Vbc == 0) sv = -sv; }
                        int q = N * iiq + kkq + 1;
                        MB(kk1 + p - q, q) = MB(kk1 + p - q, q) + (sv == -1 ? -v : v);
                    }
                }
            }
    } else {
        MB(kk1, p) = 1.0;
    }
    // row equilibration (DGBEQU row factors) and scaling
    double rmax = 0.0;
    for (int q = (p - kl > 1 ? p - kl : 1); q <= (p + ku < n ? p + ku : n); q++) rmax = fmax(rmax, fabs(MB(kk1 + p - q, q)));
    if (rmax == 0.0) { atomicOr(err, 2); rmax = 1.0; }
    const double smlnum = 2.2250738585072014e-308;
    double rf = 1.0 / fmin(fmax(rmax, smlnum), 1.0 / smlnum);
    RowB[p - 1] = rf;
    for (int q = (p - kl > 1 ? p - kl : 1); q <= (p + ku < n ? p + ku : n); q++) MB(kk1 + p - q, q) = rf * MB(kk1 + p - q, q);
#undef MB
}

// DGBTF2: unblocked band LU with partial pivoting, one CTA (band in global memory / L2)
__global__ void __launch_bounds__(1024) k_band_lu(double* ab, int* ipiv, int n, int kl, int ku, int* err) {
    const int ldab = 2 * kl + ku + 1, kv = ku + kl;
    __shared__ int s_jp, s_ju, s_nz;
    const int tid = threadIdx.x, nt = blockDim.x;
#define AB(r, c) ab[(size_t)((r) - 1) + (size_t)((c) - 1) * (size_t)ldab]
    for (int j = ku + 2; j <= (kv < n ? kv : n); j++)
        for (int i = kv - j + 2 + tid; i <= kl; i += nt) AB(i, j) = 0.0;
    if (tid == 0) s_ju = 1;
    __syncthreads();
    for (int j = 1; j <= n; j++) {
        if (j + kv <= n)
            for (int i = 1 + tid; i <= kl; i += nt) AB(i, j + kv) = 0.0;
        const int km = kl < n - j ? kl : n - j;
        // pivot: first index of the maximum |a| in AB(kv+1..kv+1+km, j).  A NaN never wins the
        // comparison; the search starts from row 1 so the index stays inside the band even for a
        // column of NaNs, which is then reported like a zero pivot.
        if (tid < 32) {
            double best = -1.0;
            int bi = 1 << 30;
            for (int i = 1 + tid; i <= km + 1; i += 32) {
                double a = fabs(AB(kv + i, j));
                if (a > best) { best = a; bi = i; }
            }
            if (bi > km + 1) bi = 1;
            for (int o = 16; o > 0; o >>= 1) {
                double ob = __shfl_xor_sync(0xffffffffu, best, o);
                int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (tid == 0) {
                s_jp = bi;
                ipiv[j - 1] = bi + j - 1;
                const double piv = AB(kv + bi, j);
                s_nz = (piv != 0.0 && piv == piv);
                if (s_nz) {
                    int jue = j + ku + bi - 1 < n ? j + ku + bi - 1 : n;
                    if (jue > s_ju) s_ju = jue;
                } else {
                    atomicCAS(err, 0, j);
                }
            }
        }
        __syncthreads();
        const int jp = s_jp, ju = s_ju;
        if (s_nz) {
            if (jp != 1) {
                for (int t = tid; t <= ju - j; t += nt) {
                    size_t a0 = (size_t)(kv + jp - 1) + (size_t)(j - 1) * ldab + (size_t)t * (ldab - 1);
                    size_t b0 = (size_t)kv + (size_t)(j - 1) * ldab + (size_t)t * (ldab - 1);
                    double x = ab[a0];
                    ab[a0] = ab[b0];
                    ab[b0] = x;
                }
                __syncthreads();
            }
            if (km > 0) {
                const double rp = 1.0 / AB(kv + 1, j);
                for (int i = 1 + tid; i <= km; i += nt) AB(kv + 1 + i, j) = AB(kv + 1 + i, j) * rp;
                __syncthreads();
                const int ncol = ju - j;
                for (int e = tid; e < ncol * km; e += nt) {
                    int jj = e / km + 1, i = e % km + 1;
                    double y = ab[(size_t)(kv - 1) + (size_t)j * ldab + (size_t)(jj - 1) * (ldab - 1)];
                    if (y != 0.0) {
                        size_t a0 = (size_t)kv + (size_t)j * ldab + (size_t)(jj - 1) * (ldab - 1) + (size_t)(i - 1);
                        ab[a0] = ab[a0] + AB(kv + 1 + i, j) * (-1.0 * y);
                    }
                }
            }
        }
        __syncthreads();
    }
#undef AB
}

// DGBTRS (forward substitution with the row interchanges and L, back substitution with U) on one
// right-hand side.  The substitutions are sequential over the n columns, so one warp carries
// them, its lanes splitting each column's band update; the band columns (and pivots) a chunk of
// steps needs are staged in shared memory by the whole CTA beforehand, so each step works from
// shared memory instead of waiting on a global load.  Same operations in the same order as the
// column-by-column DGBTRS, zero entries divided and propagated too (the optimized-BLAS behaviour
// of the shipped run, which only decides the sign of exact zeros).
constexpr int kBsChunk = 32, kBsThreads = 128;
__host__ __device__ constexpr size_t band_solve_smem(int n, int kl, int ku) {
    return sizeof(double) * ((size_t)n + (size_t)kBsChunk * (kl + ku + 1)) + sizeof(int) * kBsChunk;
}
__global__ void __launch_bounds__(kBsThreads) k_band_solve(const double* ab, const int* ipiv, double* bg, int n, int kl,
                                                         int ku) {
    extern __shared__ double b[];
    const int ldab = 2 * kl + ku + 1, kd = ku + kl + 1, kp1 = kl + ku + 1, k = kl + ku;
    double* cb = b + n;
    int* cp = reinterpret_cast<int*>(cb + (size_t)kBsChunk * kp1);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int q = tid; q < n; q += kBsThreads) b[q] = bg[q];
#define AB(r, c) ab[(size_t)((r) - 1) + (size_t)((c) - 1) * (size_t)ldab]
    // forward: columns 1..n-1, rows kd+1..kd+kl of each (the multipliers of L)
    for (int c0 = 1; c0 <= n - 1; c0 += kBsChunk) {
        const int cn = min(kBsChunk, n - c0);
        __syncthreads();
        for (int q = tid; q < cn * kl; q += kBsThreads) cb[q] = AB(kd + 1 + q % kl, c0 + q / kl);
        for (int q = tid; q < cn; q += kBsThreads) cp[q] = ipiv[c0 + q - 1];
        __syncthreads();
        if (warp == 0) {
            for (int jj = 0; jj < cn; jj++) {
                const int j = c0 + jj;
                const int lm = kl < n - j ? kl : n - j;
                const int l = cp[jj];
                if (l != j && lane == 0) { double t = b[l - 1]; b[l - 1] = b[j - 1]; b[j - 1] = t; }
                __syncwarp();
                const double temp = -1.0 * b[j - 1];
                for (int i = 1 + lane; i <= lm; i += 32) b[j + i - 1] = b[j + i - 1] + cb[jj * kl + i - 1] * temp;
                __syncwarp();
            }
        }
    }
    // back substitution: columns n..1, rows 1..kp1 of each (U, diagonal in row kp1)
    for (int c1 = n; c1 >= 1; c1 -= kBsChunk) {
        const int cn = min(kBsChunk, c1);
        __syncthreads();
        for (int q = tid; q < cn * kp1; q += kBsThreads) cb[q] = AB(1 + q % kp1, c1 - q / kp1);
        __syncthreads();
        if (warp == 0) {
            for (int jj = 0; jj < cn; jj++) {
                const int j = c1 - jj;
                const double* col = cb + (size_t)jj * kp1;  // col[r - 1] = AB(r, j)
                const double x = b[j - 1] / col[kp1 - 1];
                __syncwarp();
                if (lane == 0) b[j - 1] = x;
                const int l = kp1 - j, i0 = 1 > j - k ? 1 : j - k;
                for (int i = j - 1 - lane; i >= i0; i -= 32) b[i - 1] = b[i - 1] - x * col[l + i - 1];
                __syncwarp();
            }
        }
    }
#undef AB
    __syncthreads();
    for (int q = tid; q < n; q += kBsThreads) bg[q] = b[q];
}

// Explicit inverse of the factored coarse matrix, G = (P L U)^{-1}.  Warp w of a block carries
// column c = 4 blockIdx.x + w through the forward/back substitution of k_band_solve (DGBTRS
// restated) on the unit vector e_c, its lanes splitting each step's band update.  The four warps
// share the band columns, staged through shared memory kInvChunk at a time; each column vector
// lives in shared memory.  G is row-major, so the per-cycle coarse solve is a coalesced GEMV.
constexpr int kInvWarps = 4, kInvChunk = 16;
__host__ __device__ constexpr size_t inv_smem(int n, int kl, int ku) {
    return sizeof(double) * ((size_t)kInvChunk * (kl + ku + 1) + (size_t)kInvWarps * n) + sizeof(int) * kInvChunk;
}
__global__ void __launch_bounds__(32 * kInvWarps) k_band_inverse(const double* ab, const int* ipiv, double* G, int n,
                                                                 int kl, int ku) {
    extern __shared__ double sm[];
    const int ldab = 2 * kl + ku + 1, kd = ku + kl + 1, k = kl + ku, kp1 = k + 1;
    double* band = sm;                                           // kInvChunk x kp1
    double* y = band + (size_t)kInvChunk * kp1 + (size_t)(threadIdx.x >> 5) * n;
    int* piv = reinterpret_cast<int*>(sm + (size_t)kInvChunk * kp1 + (size_t)kInvWarps * n);
    const int lane = threadIdx.x & 31, c = blockIdx.x * kInvWarps + (threadIdx.x >> 5);
    const bool active = c < n;  // inactive warps still join every __syncthreads
#define AB(r, cc) ab[(size_t)((r) - 1) + (size_t)((cc) - 1) * (size_t)ldab]
    if (active)
        for (int q = lane; q < n; q += 32) y[q] = (q == c) ? 1.0 : 0.0;
    // forward: L with the row interchanges
    for (int j0 = 1; j0 <= n - 1; j0 += kInvChunk) {
        __syncthreads();
        for (int t = threadIdx.x; t < kInvChunk * kl; t += blockDim.x) {
            const int jj = j0 + t / kl, i = t % kl + 1;
            band[(size_t)(t / kl) * kl + (i - 1)] = (jj <= n - 1 && i <= n - jj) ? AB(kd + i, jj) : 0.0;
        }
        for (int t = threadIdx.x; t < kInvChunk; t += blockDim.x) piv[t] = (j0 + t <= n - 1) ? ipiv[j0 + t - 1] : 0;
        __syncthreads();
        if (!active) continue;
        const int jend = min(n - 1, j0 + kInvChunk - 1);
        for (int j = j0; j <= jend; j++) {
            const int lm = kl < n - j ? kl : n - j, l = piv[j - j0];
            if (l != j && lane == 0) {
                const double tt = y[l - 1];
                y[l - 1] = y[j - 1];
                y[j - 1] = tt;
            }
            __syncwarp();
            const double bj = y[j - 1];
            if (bj != 0.0) {
                const double temp = -1.0 * bj;
                const double* bc = band + (size_t)(j - j0) * kl;
                for (int i = 1 + lane; i <= lm; i += 32) y[j + i - 1] = y[j + i - 1] + bc[i - 1] * temp;
            }
            __syncwarp();
        }
    }
    // backward: U (band rows 1..kp1 of each column), columns n..1
    for (int j1 = n; j1 >= 1; j1 -= kInvChunk) {
        __syncthreads();
        for (int t = threadIdx.x; t < kInvChunk * kp1; t += blockDim.x) {
            const int jj = j1 - t / kp1, r = t % kp1 + 1;
            band[(size_t)(t / kp1) * kp1 + (r - 1)] = (jj >= 1) ? AB(r, jj) : 0.0;
        }
        __syncthreads();
        if (!active) continue;
        const int jend = max(1, j1 - kInvChunk + 1);
        for (int j = j1; j >= jend; j--) {
            const double* bc = band + (size_t)(j1 - j) * kp1;  // bc[r - 1] = AB(r, j)
            const double bj = y[j - 1];
            if (bj != 0.0) {
                const double x = bj / bc[kp1 - 1];
                __syncwarp();
                if (lane == 0) y[j - 1] = x;
                const int l = kp1 - j, i0 = 1 > j - k ? 1 : j - k;
                for (int i = j - 1 - lane; i >= i0; i -= 32) y[i - 1] = y[i - 1] - x * bc[l + i - 1];
            }
            __syncwarp();
        }
    }
#undef AB
    if (active)
        for (int q = lane; q < n; q += 32) G[(size_t)q * n + c] = y[q];
}

// coarse solve through the explicit inverse: b = RowB * RHS on interior nodes (0 on the
// boundary), x = G b (one warp per row, lanes stride the row, fixed-order shuffle reduction),
// scattered into the level array.
template <typename R>
__global__ void __launch_bounds__(256) k_coarse_apply(R* Eout, const R* RHS, const double* G, const double* RowB, Geo g,
                                                      int nxc, int nzc) {
    extern __shared__ double bsh[];
    const int N = nzc + 1, n = (nxc + 1) * N;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        int ip = q / N, kp = q % N;
        bsh[q] = (ip > 0 && ip < nxc && kp > 0 && kp < nzc) ? (double)RHS[g.at(ip, kp)] * RowB[q] : 0.0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + warp;
    if (p >= n) return;
    const double* row = G + (size_t)p * n;
    double a = 0.0;
    for (int q = lane; q < n; q += 32) a += row[q] * bsh[q];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) Eout[g.at(p / N, p % N)] = (R)a;
}

// The mixed-precision V-cycle's coarse solve: x = G b with the FP64 inverse and FP64 sums (the
// coarsest level stays FP64), from the FP32 restricted residual, into the FP32 correction with
// its boundary values.  A GEMV of n^2 FMAs (n = 561 at 1024x512) spread over n warps costs a few
// microseconds on the FP64 pipe.
__global__ void __launch_bounds__(256) k_coarse_apply_mixed(float* Eout, const float* RHS, const double* G,
                                                            const double* RowB, Geo g, int nxc, int nzc, float sz) {
    extern __shared__ double bsm[];
    const int N = nzc + 1, n = (nxc + 1) * N;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        int ip = q / N, kp = q % N;
        bsm[q] = (ip > 0 && ip < nxc && kp > 0 && kp < nzc) ? (double)RHS[g.at(ip, kp)] * RowB[q] : 0.0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + warp;
    if (p >= n) return;
    const double* row = G + (size_t)p * n;
    double a = 0.0;
    for (int q = lane; q < n; q += 32) a = fma(row[q], bsm[q], a);
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane != 0) return;
    // the correction with its boundary values: wall nodes zero, interior nodes with their free-slip
    // images (antisymmetric across the side walls, sign sz across top and bottom)
    const int ip = p / N, kp = p % N;
    if (ip == 0 || ip == nxc || kp == 0 || kp == nzc) {
        Eout[g.at(ip, kp)] = 0.0f;
        return;
    }
    const float v = (float)a;
    int xs[3], zs[3];
    float xf[3], zf[3];
    int nxp = 0, nzp = 0;
    xs[nxp] = ip; xf[nxp++] = 1.0f;
    if (ip <= 3) { xs[nxp] = -ip; xf[nxp++] = -1.0f; }
    if (ip >= nxc - 3) { xs[nxp] = 2 * nxc - ip; xf[nxp++] = -1.0f; }
    zs[nzp] = kp; zf[nzp++] = 1.0f;
    if (kp <= 3) { zs[nzp] = -kp; zf[nzp++] = sz; }
    if (kp >= nzc - 3) { zs[nzp] = 2 * nzc - kp; zf[nzp++] = sz; }
    for (int u = 0; u < nxp; u++)
        for (int w = 0; w < nzp; w++) Eout[g.at(xs[u], zs[w])] = (xf[u] * zf[w]) * v;
}

__global__ void k_coarse_rhs(double* B, const double* RHS, const double* RowB, Geo g, int nxc, int nzc) {
    int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int N = nzc + 1, n = (nxc + 1) * N;
    if (p > n) return;
    int ip = (p - 1) / N, kp = (p - 1) % N;
    B[p - 1] = (ip > 0 && ip < nxc && kp > 0 && kp < nzc) ? RHS[g.at(ip, kp)] * RowB[p - 1] : 0.0;
}
__global__ void k_coarse_scatter(double* E, const double* B, Geo g, int nxc, int nzc) {
    int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    int N = nzc + 1, n = (nxc + 1) * N;
    if (p > n) return;
    E[g.at((p - 1) / N, (p - 1) % N)] = B[p - 1];
}

static int coarse_factor(Engine& E) {
    PhaseTimer tf(E, PH_FACTOR);
    const int L = E.grids, n = E.ngc;
    CK(cudaMemsetAsync(E.derr, 0, sizeof(int), E.st));
    PT_COUNT(), k_coarse_matrix<<<nblk(n, 128), 128, 0, E.st>>>(E.Mc, E.gl[L], L, E.kl, E.ku, n, E.RowB, E.cfg.Vbc,
                                                    E.cfg.ivis, E.vis[L], E.vx[L], E.vz[L], E.vxz[L], E.vxxmzz[L], E.derr);
    PT_COUNT(), k_band_lu<<<1, 1024, 0, E.st>>>(E.Mc, E.ipiv, n, E.kl, E.ku, E.derr);
    CKL("coarse LU");
    int h = 0;
    CK(cudaMemcpyAsync(&h, E.derr, sizeof(int), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    if (h) return fail(PT_ERR_SINGULAR_COARSE, "coarse banded LU: zero row or pivot");
    if (E.Ginv) {
        PT_COUNT(), k_band_inverse<<<nblk(n, kInvWarps), 32 * kInvWarps, inv_smem(n, E.kl, E.ku), E.st>>>(
            E.Mc, E.ipiv, E.Ginv, n, E.kl, E.ku);
        CKL("k_band_inverse");
    }
    return 0;
}

// Mixed precision: build the coarse matrix, its LU and inverse for the viscosity just computed
// on st into the second buffer set on st2, overlapped with the solve that follows on st (the LU
// runs on one SM).  coarse_resolve copies the result into the live buffers.
static int coarse_factor_async(Engine& E, const VisLevels& V) {
    const int L = E.grids, n = E.ngc;
    CK(cudaMemsetAsync(E.derr2, 0, sizeof(int), E.st2));
    PT_COUNT(), k_coarse_matrix<<<nblk(n, 128), 128, 0, E.st2>>>(E.Mc2, E.gl[L], L, E.kl, E.ku, n, E.RowB2, E.cfg.Vbc,
                                                     E.cfg.ivis, V.vis[L], V.vx[L], V.vz[L], V.vxz[L], V.vxxmzz[L],
                                                     E.derr2);
    PT_COUNT(), k_band_lu<<<1, 1024, 0, E.st2>>>(E.Mc2, E.ipiv2, n, E.kl, E.ku, E.derr2);
    PT_COUNT(), k_band_inverse<<<nblk(n, kInvWarps), 32 * kInvWarps, inv_smem(n, E.kl, E.ku), E.st2>>>(
        E.Mc2, E.ipiv2, E.Ginv2, n, E.kl, E.ku);
    CKL("async coarse factorisation");
    CK(cudaMemcpyAsync(E.hflag2, E.derr2, sizeof(int), cudaMemcpyDeviceToHost, E.st2));
    E.fact_pending = true;
    return 0;
}

// The worker thread of a new time level (mixed precision): the viscosity pipeline of levels
// 2..grids into the side set vl2 (from the snapshot of level 1's static viscosity in
// vl2.visst[1]) and the coarse factorisation from it, all on st2; ev_fact marks the end.  Reads
// only its own arrays and the engine's constant configuration; its status goes to job_rc.
static void coarse_levels_worker(Engine* Ep) {
    Engine& E = *Ep;
    int rc = 0;
    if (cudaSetDevice(E.device) != cudaSuccess || cudaStreamWaitEvent(E.st2, E.ev_in, 0) != cudaSuccess)
        rc = fail(PT_ERR_CUDA, "coarse-level worker: device or event");
    const VisCtx C = side_ctx(E);
    for (int level = 2; level <= E.grids && !rc; level++) rc = compute_viscosity(E, C, level);
    if (!rc && E.cfg.ivis > 0) rc = coarse_factor_async(E, E.vl2);
    if (!rc && cudaEventRecord(E.ev_fact, E.st2) != cudaSuccess) rc = fail(PT_ERR_CUDA, "coarse-level worker: event");
    E.job_rc = rc;
    if (rc) E.job_msg = g_err;
    E.job_done = true;
}

// Joins the worker and moves its levels into the cycle's arrays (after st2's work, in stream
// order); the factorisation follows in coarse_resolve.  Unless `wait`, only a worker whose work
// has completed on the device is joined: the solves of this time level keep the previous coarse
// levels until then (a preconditioner, O(dt) older), so the worker never delays a solve.
static int coarse_join(Engine& E, bool wait) {
    if (!E.job_active) return 0;
    if (!wait && !(E.job_done.load() && cudaEventQuery(E.ev_fact) == cudaSuccess)) {
        cudaGetLastError();  // a not-ready query is not an error
        return 0;
    }
    E.coarse_job.join();
    E.job_active = false;
    if (E.job_rc) return fail(E.job_rc, E.job_msg);
    CK(cudaStreamWaitEvent(E.st, E.ev_fact, 0));
    const VisLevels P = primary_levels(E);
    double* const* dst[kVisArrays] = {P.vis, P.visst, P.vx, P.vz, P.vxx, P.vzz, P.vxz, P.vxxpzz, P.vxxmzz, P.vsm, P.ratio, P.dtst};
    double* const* src[kVisArrays] = {E.vl2.vis, E.vl2.visst, E.vl2.vx, E.vl2.vz, E.vl2.vxx, E.vl2.vzz, E.vl2.vxz,
                                      E.vl2.vxxpzz, E.vl2.vxxmzz, E.vl2.vsm, E.vl2.ratio, E.vl2.dtst};
    for (int l = 2; l <= E.grids; l++)
        for (int a = 0; a < kVisArrays; a++)
            CK(cudaMemcpyAsync(dst[a][l], src[a][l], E.gl[l].elems() * 8, cudaMemcpyDeviceToDevice, E.st));
    E.coarse_fresh = true;
    return 0;
}

int coarse_resolve(Engine& E) {
    if (!E.fact_pending) return 0;
    E.fact_pending = false;
    CK(cudaEventSynchronize(E.ev_fact));
    if (*E.hflag2) return fail(PT_ERR_SINGULAR_COARSE, "coarse banded LU: zero row or pivot");
    const int n = E.ngc, ldab = 2 * E.kl + E.ku + 1;
    CK(cudaMemcpyAsync(E.Mc, E.Mc2, sizeof(double) * (size_t)ldab * n, cudaMemcpyDeviceToDevice, E.st));
    CK(cudaMemcpyAsync(E.RowB, E.RowB2, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, E.st));
    CK(cudaMemcpyAsync(E.ipiv, E.ipiv2, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, E.st));
    CK(cudaMemcpyAsync(E.Ginv, E.Ginv2, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, E.st));
    return 0;
}

// x = G b into err[L] (FP64) or ferr[L] (FP32); needs E.Ginv
int coarse_apply(Engine& E, double* out64, float* out32, const double* rhs64, const float* rhs32) {
    const int L = E.grids, n = E.ngc;
    const Geo& g = E.gl[L];
    const unsigned blocks = nblk(n, 8);
    const size_t smem = sizeof(double) * (size_t)n;
    if (out64) PT_COUNT(), k_coarse_apply<double><<<blocks, 256, smem, E.st>>>(out64, rhs64, E.Ginv, E.RowB, g, g.nx, g.nz);
    else PT_COUNT(), k_coarse_apply_mixed<<<blocks, 256, smem, E.st>>>(out32, rhs32, E.Ginv, E.RowB, g, g.nx, g.nz,
                                                                       E.cfg.Vbc == 0 ? -1.f : 1.f);
    CKL("k_coarse_apply");
    return 0;
}

static int coarse_solve(Engine& E) {
    const int L = E.grids, n = E.ngc;
    const Geo& g = E.gl[L];
    if (E.Ginv) {
        if (int rc = coarse_apply(E, E.err[L], nullptr, E.RHS[L], nullptr)) return rc;
        return enforce_bcs_stream(E, L, E.err[L]);
    }
    PT_COUNT(), k_coarse_rhs<<<nblk(n, 128), 128, 0, E.st>>>(E.Bc, E.RHS[L], E.RowB, g, g.nx, g.nz);
    PT_COUNT(), k_band_solve<<<1, kBsThreads, band_solve_smem(n, E.kl, E.ku), E.st>>>(E.Mc, E.ipiv, E.Bc, n, E.kl, E.ku);
    PT_COUNT(), k_coarse_scatter<<<nblk(n, 128), 128, 0, E.st>>>(E.err[L], E.Bc, g, g.nx, g.nz);
    CKL("coarse solve");
    return enforce_bcs_stream(E, L, E.err[L]);
}

// helpers shared with the mixed-precision solver (pt_mixed.cu)
int coarse_band_solve(Engine& E) {
    const int n = E.ngc;
    PT_COUNT(), k_band_solve<<<1, kBsThreads, band_solve_smem(n, E.kl, E.ku), E.st>>>(E.Mc, E.ipiv, E.Bc, n, E.kl, E.ku);
    CKL("k_band_solve");
    return 0;
}

int residual_level1_nosum(Engine& E) {
    launch_residual(E, 1, E.res[1], E.err[1], stream_op(E, 1));
    CKL("k_residual");
    return 0;
}

int residual_level1(Engine& E) {
    const Geo& g = E.gl[1];
    launch_residual(E, 1, E.res[1], E.err[1], stream_op(E, 1));
    CKL("k_residual");
    return reduce_sum_abs_interior(E, E.res[1], g.nx, g.nz, g.pitch, E.dscal + 8);
}

// ------------------------------------------------------------------ driver
int mg_setup_solve(Engine& E) {
    int rc;
    // coarse levels and factorisation built by the worker of this time level, once they are done
    // (at a new time level: always, before the next worker starts)
    const bool new_level = !(E.coarse_ready && E.coarse_time == E.time);
    if ((rc = coarse_join(E, new_level))) return rc;
    if (!E.job_active && (rc = coarse_resolve(E))) return rc;
    CK(cudaMemcpyAsync(E.err[1], E.SF, E.g1.elems() * 8, cudaMemcpyDeviceToDevice, E.st));
    if ((rc = compute_RHS(E, 1))) return rc;
    if ((rc = mean_abs(E, E.RHS[1], 1, &E.res_ref[1]))) return rc;
    // The mixed-precision cycle uses levels 2..grids only as a preconditioner inside FP64 defect
    // correction on level 1: their viscosity pipeline and the coarse factorisation are refreshed
    // once per time level (the top-of-step solve) and reused by the RK-stage solves of the step,
    // whose viscosity differs by O(dt).  Level 1, which defines the residual, is rebuilt every
    // solve.  The FP64 cycle rebuilds every level every solve, as the reference does.
    const bool mixed = E.cfg.precision == PT_PREC_MIXED;
    const bool reuse = mixed && E.coarse_ready && E.coarse_time == E.time;
    // a new time level with coarse levels in place (mixed precision): build the new ones on the
    // worker thread, off the critical path; this solve keeps the previous time level's (a
    // preconditioner, O(dt) older)
    const bool async = mixed && E.coarse_ready && !reuse && E.Ginv2 && E.vl2.vis[2];
    E.levels_reused = reuse || async;
    const VisCtx C = primary_ctx(E);
    for (int level = 1; level <= (E.levels_reused ? 1 : E.grids); level++)
        if ((rc = compute_viscosity(E, C, level))) return rc;
    if (async) {
        CK(cudaMemcpyAsync(E.vl2.visst[1], E.visst[1], E.g1.elems() * 8, cudaMemcpyDeviceToDevice, E.st));
        CK(cudaEventRecord(E.ev_in, E.st));
        E.job_rc = 0;
        E.job_done = false;
        E.coarse_job = std::thread(coarse_levels_worker, &E);
        E.job_active = true;
        E.coarse_time = E.time;
    } else if (!reuse && (E.time == 0.0 || E.cfg.ivis > 0)) {
        if ((rc = coarse_factor(E))) return rc;
        E.coarse_ready = true;
        E.coarse_time = E.time;
    }
    return 0;
}

// One multigrid cycle of the reference's schedule, split where the reference tests convergence
// (after the level-1 smoothing pass, iterative_solver.f90:313-315).  Part A: level-1 smoothing,
// residual and sum|r|.  Part B: the rest of the schedule (restrict, coarse visits, coarse solve,
// prolong back to level 1).  Neither part synchronises, so both are captured as CUDA graphs.
static int cycle_part(Engine& E, int part) {
    int rc;
    // the reference's schedule, or a V-cycle when asked for (mg_cycle); the parity path keeps the
    // reference's
    const bool v = E.cfg.mg_cycle == PT_CYCLE_V;
    const int grids = E.grids, nsteps = v ? E.mnsteps : E.nsteps;
    const int* multi = v ? E.mmulti : E.multi;
    if (part == 0) return iterate_stream(E, 1, 1);
    for (int p = 2; p <= nsteps; p++) {
        const int level = multi[p];
        if (multi[p - 1] < multi[p]) {
            if ((rc = compute_RHS(E, level))) return rc;
            if (E.cfg.mg_scheme == PT_MG_CORRECTION && level > 1)
                CK(cudaMemsetAsync(E.err[level], 0, E.gl[level].elems() * sizeof(double), E.st));
        }
        if (level < grids) {
            if ((rc = iterate_stream(E, level, 0))) return rc;
        } else if ((rc = coarse_solve(E))) {
            return rc;
        }
        if (multi[p + 1] < multi[p] && (rc = prolong(E, level))) return rc;
    }
    return 0;
}

static int capture_part(Engine& E, int part, cudaGraphExec_t* exec, int64_t* nlaunch) {
    cudaGraph_t graph = nullptr;
    int64_t before = g_launches.load();
    CK(cudaStreamBeginCapture(E.st, cudaStreamCaptureModeThreadLocal));
    int rc = cycle_part(E, part);
    cudaError_t e = cudaStreamEndCapture(E.st, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    CK(e);
    CK(cudaGraphInstantiate(exec, graph, 0));
    cudaGraphDestroy(graph);
    *nlaunch = g_launches - before;
    g_launches = before;
    return 0;
}

static int run_part(Engine& E, int part) {
    cudaGraphExec_t& ex = part == 0 ? E.gA : E.gB;
    int64_t& n = part == 0 ? E.nA : E.nB;
    if (!ex) {
        int rc = capture_part(E, part, &ex, &n);
        if (rc) return rc;
    }
    CK(cudaGraphLaunch(ex, E.st));
    g_launches += n;
    return 0;
}

int multigrid(Engine& E, pt_solve_info* info) {
    int rc;
    PhaseTimer tm(E, PH_SOLVE);
    {
        PhaseTimer ts(E, PH_SETUP);
        if ((rc = mg_setup_solve(E))) return rc;
        if (E.cfg.guess_mode == PT_GUESS_UNET && (rc = unet_guess(E))) return rc;
    }
    const double norm = (double)(E.gl[1].nx - 2) * (double)(E.gl[1].nz - 2);
    int q = 1;
    double mag1 = 0.0;
    E.res_hist.clear();
    for (;;) {
        {
            PhaseTimer tp(E, PH_CYCLE_L1);
            if ((rc = run_part(E, 0))) return rc;
            CK(cudaMemcpyAsync(E.hscal, E.dscal + 8, 8, cudaMemcpyDeviceToHost, E.st));
        }
        CK(cudaStreamSynchronize(E.st));
        harvest_graph_timer(E, 0);
        mag1 = E.hscal[0] / (double)(E.gl[1].nx - 2) / (double)(E.gl[1].nz - 2);
        (void)norm;
        if (E.res_hist.size() < 100000) E.res_hist.push_back(mag1 / E.res_ref[1]);
        if (!std::isfinite(mag1)) return fail(PT_ERR_NOT_FINITE, "non-finite multigrid residual");
        if (mag1 > 1.0e10 * E.res_ref[1])
            return fail(PT_ERR_MG_DIVERGED, "Multigrid Convergence Problem: Abnormally High Residual Detected");
        if (trace_on()) fprintf(stderr, "[ptgpu] cycle %d residual ratio %.4e\n", q, mag1 / E.res_ref[1]);
        if (q == 2) {  // one full cycle from a learned guess: keep it or restart from the previous psi
            const int fb = unet_check_fallback(E, mag1 / E.res_ref[1]);
            if (fb < 0) return fail(PT_ERR_CUDA, "learned-guess fallback copy");
            if (fb) {
                q++;  // the cycle spent on the dropped guess counts
                continue;
            }
        }
        if (mag1 / E.res_ref[1] <= E.cfg.tolerance) break;
        {
            PhaseTimer tp(E, PH_CYCLE_COARSE);
            if ((rc = run_part(E, 1))) return rc;
        }
        q++;
        if (q > E.cfg.max_cycles) return fail(PT_ERR_MG_MAX_CYCLES, "Multigrid Convergence Problem: Too Many Multigrid Cycles Needed");
    }
    E.cycles = q;
    E.residual_mag1 = mag1;
    E.resid_ratio = mag1 / E.res_ref[1];
    CK(cudaMemcpyAsync(E.SF, E.err[1], E.g1.elems() * 8, cudaMemcpyDeviceToDevice, E.st));
    if (info) {
        info->cycles += q;
        info->resid_ratio = E.resid_ratio;
        info->n_eta = E.n_eta;
        info->eig_fine = E.eig_fine;
    }
    return 0;
}

int mg_alloc(Engine& E) {
    auto alloc = [&](double** p, size_t n) -> int {
        CK(cudaMalloc(p, n * sizeof(double)));
        CK(cudaMemsetAsync(*p, 0, n * sizeof(double), E.st));
        E.bytes_allocated += n * sizeof(double);
        return 0;
    };
    for (int l = 1; l <= E.grids; l++) {
        size_t n = E.gl[l].elems();
        double** arrs[] = {&E.err[l], &E.S0[l], &E.S1[l], &E.S2[l], &E.RHS[l], &E.res[l], &E.dtst[l], &E.ratio[l],
                           &E.vis[l], &E.visst[l], &E.vx[l], &E.vz[l], &E.vxx[l], &E.vzz[l], &E.vxz[l],
                           &E.vxxpzz[l], &E.vxxmzz[l], &E.vsm[l]};
        for (auto a : arrs)
            if (int rc = alloc(a, n)) return rc;
    }
    for (int q = 0; q < 11; q++)
        if (int rc = alloc(&E.visw[q], E.gl[1].elems())) return rc;
    // exact integer stencil sums unless the FP64 path is asked to round like the reference
    E.res_int = !E.cfg.reference_rounding && exact_stencils_setup(E);
    int ldab = 2 * E.kl + E.ku + 1;
    if (int rc = alloc(&E.Mc, (size_t)ldab * E.ngc)) return rc;
    if (int rc = alloc(&E.Bc, E.ngc)) return rc;
    if (int rc = alloc(&E.RowB, E.ngc)) return rc;
    CK(cudaMalloc(&E.ipiv, sizeof(int) * E.ngc));
    const size_t smem = sizeof(double) * (size_t)E.ngc;
    if (smem > 220 * 1024) return fail(PT_ERR_CONFIG, "coarsest grid too large for the banded solve");
    if (band_solve_smem(E.ngc, E.kl, E.ku) > 220 * 1024)
        return fail(PT_ERR_CONFIG, "coarsest grid too large for the banded solve");
    CK(cudaFuncSetAttribute(k_band_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)band_solve_smem(E.ngc, E.kl, E.ku)));
    CK(cudaFuncSetAttribute(k_coarse_apply<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(k_coarse_apply_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // explicit coarse inverse (both precisions): the coarse solve becomes a GEMV spread over the
    // SMs instead of two sequential banded substitutions on one warp of this part's narrow FP64
    // pipe; n^2 doubles, kept while it is small next to the level arrays (n <= 4096: <= 134 MB)
    if (!E.cfg.reference_rounding && E.ngc <= 4096 && inv_smem(E.ngc, E.kl, E.ku) <= 200 * 1024) {
        CK(cudaMalloc(&E.Ginv, sizeof(double) * (size_t)E.ngc * E.ngc));
        E.bytes_allocated += sizeof(double) * (size_t)E.ngc * E.ngc;
        CK(cudaMalloc(&E.Ginv2, sizeof(double) * (size_t)E.ngc * E.ngc));
        CK(cudaMalloc(&E.Mc2, sizeof(double) * (size_t)ldab * E.ngc));
        CK(cudaMalloc(&E.RowB2, sizeof(double) * (size_t)E.ngc));
        CK(cudaMalloc(&E.ipiv2, sizeof(int) * (size_t)E.ngc));
        CK(cudaMalloc(&E.derr2, sizeof(int)));
        CK(cudaMallocHost(&E.hflag2, sizeof(int)));
        *E.hflag2 = 0;
        CK(cudaStreamCreateWithFlags(&E.st2, cudaStreamNonBlocking));
        CK(cudaGetDevice(&E.device));
        // the side set of the coarse levels (and level 1's static viscosity snapshot), its work
        // arrays and scalars
        for (int l = 1; l <= E.grids; l++) {
            double** sets[kVisArrays] = {E.vl2.vis, E.vl2.visst, E.vl2.vx, E.vl2.vz, E.vl2.vxx, E.vl2.vzz, E.vl2.vxz,
                                         E.vl2.vxxpzz, E.vl2.vxxmzz, E.vl2.vsm, E.vl2.ratio, E.vl2.dtst};
            for (int a = 0; a < kVisArrays; a++) {
                if (l == 1 && a != 1) continue;  // level 1: only visst (the snapshot)
                if (int rc = alloc(&sets[a][l], E.gl[l].elems())) return rc;
            }
        }
        for (int q = 0; q < 11; q++)
            if (int rc = alloc(&E.visw2[q], E.gl[1].elems())) return rc;
        CK(cudaMalloc(&E.dscal2, 32 * sizeof(double)));
        CK(cudaMallocHost(&E.hscal2, 64 * sizeof(double)));
        CK(cudaEventCreateWithFlags(&E.ev_in, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&E.ev_fact, cudaEventDisableTiming));
        E.bytes_allocated += sizeof(double) * ((size_t)E.ngc * E.ngc + (size_t)ldab * E.ngc + E.ngc);
        CK(cudaFuncSetAttribute(k_band_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_smem(E.ngc, E.kl, E.ku)));
    }
    return 0;
}

// ------------------------------------------------------------------ learned-guess support
// level-1 values at the nodes of level L (every s-th node), boundary included
__global__ void k_inject(double* c, const double* f, Geo gc, Geo gf, int nxc, int nzc, int s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i > nxc || k > nzc) return;
    c[gc.at(i, k)] = f[gf.at(i * s, k * s)];
}
// per interior row of a level: sum RHS*(RHS - r) and (RHS - r)^2  (r = RHS - A g, so RHS - r = A g)
__global__ void k_fit_rows(const double* rhs, const double* r, Geo g, int nx, double* part) {
    __shared__ double s1[128], s2[128];
    const int k = blockIdx.x + 1;
    double a = 0.0, b = 0.0;
    for (int i = 1 + threadIdx.x; i <= nx - 1; i += blockDim.x) {
        const size_t o = g.at(i, k);
        const double ag = rhs[o] - r[o];
        a += rhs[o] * ag;
        b += ag * ag;
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s1[0];
        part[2 * blockIdx.x + 1] = s2[0];
    }
}

// Scale of a psi shape held in err[1], fitted on the coarsest level where the shape's
// grid-scale noise is averaged away: RHS restricted by full weighting (as at a descent), the shape
// injected, alpha = <RHS_L, A_L g> / <A_L g, A_L g> with the level-L operator.  Uses the level
// arrays of levels 2..L, which the cycles overwrite anyway.
int coarse_scale_fit(Engine& E, double* alpha) {
    const int L = E.grids;
    for (int l = 2; l <= L; l++) {
        const Geo& g = E.gl[l];
        PT_COUNT(), k_restrict<<<dim3(nblk(g.nx - 1, 128), g.nz - 1), 128, 0, E.st>>>(E.RHS[l], E.RHS[l - 1], g,
                                                                                       E.gl[l - 1], g.nx, g.nz);
    }
    const Geo& gc = E.gl[L];
    PT_COUNT(), k_inject<<<dim3(nblk(gc.nx + 1, 128), gc.nz + 1), 128, 0, E.st>>>(E.err[L], E.err[1], gc, E.gl[1], gc.nx,
                                                                                   gc.nz, 1 << (L - 1));
    CKL("k_inject");
    if (int rc = enforce_bcs_stream(E, L, E.err[L])) return rc;
    launch_residual(E, L, E.res[L], E.err[L], stream_op(E, L));
    PT_COUNT(), k_fit_rows<<<gc.nz - 1, 128, 0, E.st>>>(E.RHS[L], E.res[L], gc, gc.nx, E.red);
    CKL("coarse_scale_fit");
    std::vector<double> part(2 * (size_t)(gc.nz - 1));
    CK(cudaMemcpyAsync(part.data(), E.red, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    double a = 0.0, b = 0.0;
    for (size_t k = 0; k + 1 < part.size(); k += 2) {
        a += part[k];
        b += part[k + 1];
    }
    *alpha = b > 0.0 ? a / b : 0.0;
    return 0;
}

}  // namespace pt
