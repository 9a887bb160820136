// pt_direct.cu -- the direct stream-function solve (iterate=0, the reference's shipped default):
// build_SF_matrix (momentum.f90:319-492) with Matrix_element (495-621), row equilibration (DGBEQU),
// banded LU with partial pivoting (DGBTRF), and per solve the buoyancy right-hand side (258-289),
// the banded substitutions (DGBTRS, solve_SF_equation 636-653) and Stream_grid (291-317).
//
// The matrix has one row per grid node, p = (nz+1) i + k + 1 (Database=2), with the 29-point
// biharmonic stencil folded at the walls (free-slip images carry a sign) and identity rows at the
// corners; its band is kl = ku = 3 (nz+1) wide.  For an isoviscous run (ivis=0, the only case the
// reference builds once) every stencil value depends only on the stencil offset, the two image
// signs and the row's kind (interior, side wall, top/bottom wall), so the host evaluates
// Matrix_element once per combination -- with the host's pow, like the reference -- and the
// assembly kernel only places and sums them, in the reference's stencil order.
//
// The band LU is the reference's unblocked algorithm (the LAPACK DGBTF2 that its DGBTRF call runs
// at these band widths): for each column, a pivot search, a row interchange over the columns the
// pivot reaches, the column scaled by the pivot's reciprocal, and a rank-1 update of the trailing
// kl x (ju - j) block.  The update is spread over the whole GPU: one cooperative kernel, one CTA per
// SM, the column steps separated by grid barriers (bounded spins that report a timeout instead of
// waiting forever).  Every element sees the same operations in the same order as in DGBTF2 and this
// file is compiled with --fmad=false, so the factors round exactly like the reference's.
#include <cmath>
#include <cstring>

#include "pt_consts.cuh"

namespace pt {

namespace {

// the 29 stencil points of build_SF_matrix in the reference's order (momentum.f90:397-470): the
// x and z arms at distance 3, then the 5 x 5 block
constexpr int kStencilPts = 29;
struct StencilPts {
    int n = 0;
    int di[kStencilPts], dk[kStencilPts];
    StencilPts() {
        for (int i = -3; i <= 3; i += 6) { di[n] = i; dk[n++] = 0; }
        for (int k = -3; k <= 3; k += 6) { di[n] = 0; dk[n++] = k; }
        for (int i = -2; i <= 2; i++)
            for (int k = -2; k <= 2; k++) { di[n] = i; dk[n++] = k; }
    }
};

// Matrix_element (momentum.f90:495-621) on the uniform grid (xr = zs = 1, higher metric terms 0)
// for the isoviscous operator (vis = 1, its derivatives 0): the value and whether it enters.
// row: 0 interior, 1 side wall (ip = 0 or nx), 2 top/bottom wall (kp = 0 or nz).
static double matrix_element(const Engine& E, int i, int k, int rsym, int ssym, int row, int* kind) {
    const Consts& K = E.K;
    const double xr = 1.0, xrr = 0.0, xrrr = 0.0, xrrrr = 0.0, zs = 1.0, zss = 0.0, zsss = 0.0, zssss = 0.0;
    const double dr = K.dr, ds = K.ds;
    const double dr2 = dr * dr, ds2 = ds * ds, dr3 = std::pow(dr, 3.0), ds3 = std::pow(ds, 3.0),
                 dr4 = std::pow(dr, 4.0), ds4 = std::pow(ds, 4.0);
    const double drds = dr * ds, drds2 = dr * ds2, dr2ds = dr2 * ds, dr2ds2 = dr2 * ds2;
    double Ss, Sss, Ssss, Sssss, Sr, Srr, Srrr, Srrrr;
    if (i == 0) { Ss = K.D1[k + 3] / ds; Sss = K.D2[k + 3] / ds2; Ssss = K.D3[k + 3] / ds3; Sssss = K.D4[k + 3] / ds4; }
    else { Ss = 0.0; Sss = 0.0; Ssss = 0.0; Sssss = 0.0; }
    if (ssym == 1 && E.cfg.Vbc == 0) { Ss = -Ss; Sss = -Sss; Ssss = -Ssss; Sssss = -Sssss; }
    if (k == 0) { Sr = K.D1[i + 3] / dr; Srr = K.D2[i + 3] / dr2; Srrr = K.D3[i + 3] / dr3; Srrrr = K.D4[i + 3] / dr4; }
    else { Sr = 0.0; Srr = 0.0; Srrr = 0.0; Srrrr = 0.0; }
    if (rsym == 1) { Sr = -Sr; Srr = -Srr; Srrr = -Srrr; Srrrr = -Srrrr; }
    const double Sx = Sr / xr;
    const double Sxx = (Srr - Sx * xrr) / (xr * xr);
    const double Sxxx = (Srrr - 3.0 * Sxx * xr * xrr - Sx * xrrr) / std::pow(xr, 3.0);
    const double Sxxxx =
        (Srrrr - 6.0 * Sxxx * xrr * (xr * xr) - (3.0 * (xrr * xrr) + 4.0 * xr * xrrr) * Sxx - Sx * xrrrr) / std::pow(xr, 4.0);
    const double Sz = Ss / zs;
    const double Szz = (Sss - Sz * zss) / (zs * zs);
    const double Szzz = (Ssss - 3.0 * Szz * zs * zss - Sz * zsss) / std::pow(zs, 3.0);
    const double Szzzz =
        (Sssss - 6.0 * Szzz * zss * (zs * zs) - (3.0 * (zss * zss) + 4.0 * zs * zsss) * Szz - Sz * zssss) / std::pow(zs, 4.0);
    double Srs, Srss, Srrs, Srrss;
    if (i >= -2 && i <= 2 && k >= -2 && k <= 2) {
        Srs = K.Drs[i + 2][k + 2] / drds;
        Srss = K.Drss[i + 2][k + 2] / drds2;
        Srrs = K.Drrs[i + 2][k + 2] / dr2ds;
        Srrss = K.Drrss[i + 2][k + 2] / dr2ds2;
    } else {
        Srs = 0.0 / drds; Srss = 0.0 / drds2; Srrs = 0.0 / dr2ds; Srrss = 0.0 / dr2ds2;
    }
    if (E.cfg.Vbc == 0) {
        if ((rsym == 1) != (ssym == 1)) { Srs = -Srs; Srss = -Srss; Srrs = -Srrs; Srrss = -Srrss; }
    } else if (rsym == 1) {
        Srs = -Srs; Srss = -Srss; Srrs = -Srrs; Srrss = -Srrss;
    }
    const double Sxz = Srs / xr / zs;
    const double Sxxz = (Srrs - Sxz * zs * xrr) / zs / (xr * xr);
    const double Sxzz = (Srss - Sxz * xr * zss) / xr / (zs * zs);
    const double Sxxzz = (Srrss - Sxzz * xrr * (zs * zs) - Sxxz * zss * (xr * xr) - Sxz * xrr * zss) / ((xr * zs) * (xr * zs));
    if (row == 1) { *kind = 1; return Sxx; }
    if (row == 2) {
        if (E.cfg.Vbc == 0) { *kind = 1; return Szz; }
        *kind = 0;
        return 0.0;
    }
    const double visx = 0.0, visz = 0.0, visxx = 0.0, viszz = 0.0, visxz = 0.0, visv = 1.0;
    const double t1 = (visxx - viszz) * (Sxx - Szz);
    const double t2 = visv * (Sxxxx + Szzzz);
    const double t3 = 2.0 * visv * Sxxzz;
    const double t4 = 4.0 * visxz * Sxz;
    const double t5 = 2.0 * visx * (Sxxx + Sxzz);
    const double t6 = 2.0 * visz * (Szzz + Sxxz);
    *kind = 1;
    return t1 + t2 + t3 + t4 + t5 + t6;
}

// element table [point][rsym][ssym][row]; kind 0 entries carry NaN and are skipped
struct ElemTable {
    double v[kStencilPts][2][2][3];
    int di[kStencilPts], dk[kStencilPts];
};
__constant__ ElemTable cET;

}  // namespace

// Row p's entries (momentum.f90:397-470): each stencil point (i,k) of the node (ip,kp), folded into
// the domain, adds its value to A(p, q), in the reference's order.  Corners (and, for rigid top
// and bottom, those rows) are identity rows.
__global__ void k_direct_assemble(double* MB, int n, int ldab, int kl, int ku, int nx, int nz, int Vbc) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (p > n) return;
    const int N = nz + 1, ip = (p - 1) / N, kp = (p - 1) % N;
    const bool corner = (ip == 0 || ip == nx) && (kp == 0 || kp == nz);
    if (corner || (Vbc == 1 && (kp == 0 || kp == nz))) {
        MB[(size_t)(kl + ku) + (size_t)(p - 1) * (size_t)ldab] = 1.0;
        return;
    }
    const int row = (ip == 0 || ip == nx) ? 1 : ((kp == 0 || kp == nz) ? 2 : 0);
    for (int q0 = 0; q0 < kStencilPts; q0++) {
        int iq = ip + cET.di[q0], rsym = 0;
        if (iq < 0) { iq = -iq; rsym = 1; }
        else if (iq > nx) { iq = nx - (iq - nx); rsym = 1; }
        int kq = kp + cET.dk[q0], ssym = 0;
        if (kq < 0) { kq = -kq; ssym = 1; }
        else if (kq > nz) { kq = nz - (kq - nz); ssym = 1; }
        const double v = cET.v[q0][rsym][ssym][row];
        if (v != v) continue;  // kind 0: not an entry
        const int q = N * iq + kq + 1;
        const size_t idx = (size_t)(kl + ku + p - q) + (size_t)(q - 1) * (size_t)ldab;
        MB[idx] = MB[idx] + v;
    }
}

// DGBEQU row factors r(p) = 1 / max_q |A(p,q)| (clamped to the normal range) and the row scaling
// MB(p, :) = r(p) MB(p, :); a zero row is flagged
__global__ void k_direct_equ(double* MB, double* RowB, int n, int ldab, int kl, int ku, int* err) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (p > n) return;
    const int q0 = p - kl > 1 ? p - kl : 1, q1 = p + ku < n ? p + ku : n;
    double m = 0.0;
    for (int q = q0; q <= q1; q++) {
        const double a = fabs(MB[(size_t)(kl + ku + p - q) + (size_t)(q - 1) * (size_t)ldab]);
        if (a > m) m = a;
    }
    if (m == 0.0) {
        atomicOr(err, 2);
        m = 1.0;
    }
    const double smlnum = 2.2250738585072014e-308, bignum = 1.0 / smlnum;
    double v = m > smlnum ? m : smlnum;
    v = v < bignum ? v : bignum;
    const double r = 1.0 / v;
    RowB[p - 1] = r;
    for (int q = q0; q <= q1; q++) {
        const size_t idx = (size_t)(kl + ku + p - q) + (size_t)(q - 1) * (size_t)ldab;
        MB[idx] = r * MB[idx];
    }
}

__global__ void k_fill(double* a, double v, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) a[q] = v;
}

// ---- band LU over the whole GPU
struct LuShared {
    unsigned count, gen;  // grid barrier
    int jp, ju, nz;       // this column's pivot offset, reach and pivot-is-usable flag
};

// Grid barrier for a cooperative launch (every CTA is resident, so every CTA arrives).  The wait
// is bounded: after about a second it flags err (bit 8) and returns false, and every CTA then
// leaves the kernel at its next check.
__device__ __forceinline__ bool grid_barrier(LuShared* sh, unsigned nblocks, int* err) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* vgen = &sh->gen;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&sh->count, 1u) == nblocks - 1) {
            atomicExch(&sh->count, 0u);
            __threadfence();
            atomicAdd(&sh->gen, 1u);
        } else {
            unsigned it = 0;
            while (*vgen == g) {
                if (++it > (1u << 24)) {
                    atomicOr(err, 8);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        if (*(volatile int*)err & 8) ok = 0;
    }
    __syncthreads();
    return ok != 0;
}

constexpr int kLuThreads = 256;

// err[0]: barrier timeout (bit 8); err[1]: DGBTF2's INFO, the first zero pivot column
__global__ void __launch_bounds__(kLuThreads) k_direct_lu(double* ab, int* ipiv, int n, int kl, int ku, int* err,
                                                        LuShared* sh) {
    const int ldab = 2 * kl + ku + 1, kv = ku + kl;
    const unsigned nb = gridDim.x;
    const int tid = threadIdx.x;
    const size_t gtid = (size_t)blockIdx.x * kLuThreads + tid, gstride = (size_t)nb * kLuThreads;
    __shared__ int s_jp, s_nz, s_ju;
#define AB(r, c) ab[(size_t)((r) - 1) + (size_t)((c) - 1) * (size_t)ldab]
    // fill-in rows above the band of the first kv columns
    for (int j = ku + 2; j <= (kv < n ? kv : n); j++)
        for (size_t i = kv - j + 2 + gtid; i <= (size_t)kl; i += gstride) AB((int)i, j) = 0.0;
    if (gtid == 0) sh->ju = 1;
    if (!grid_barrier(sh, nb, err)) return;
    for (int j = 1; j <= n; j++) {
        const int km = kl < n - j ? kl : n - j;
        if (blockIdx.x == 0) {
            // CTA 0: fill-in column, pivot, interchange, scaling.  Loads bypass L1 (ld.global.cg):
            // other CTAs wrote these elements in earlier steps.
            if (j + kv <= n)
                for (int i = 1 + tid; i <= kl; i += kLuThreads) AB(i, j + kv) = 0.0;
            if (tid < 32) {
                double best = -1.0;
                int bi = 1 << 30;
                for (int i = 1 + tid; i <= km + 1; i += 32) {
                    const double a = fabs(__ldcg(&AB(kv + i, j)));
                    if (a > best) { best = a; bi = i; }
                }
                if (bi > km + 1) bi = 1;  // a column of NaNs: stay inside the band (reported below)
                for (int o = 16; o > 0; o >>= 1) {
                    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
                }
                if (tid == 0) {
                    const double piv = __ldcg(&AB(kv + bi, j));
                    ipiv[j - 1] = bi + j - 1;
                    s_jp = bi;
                    s_nz = (piv != 0.0 && piv == piv);
                    int ju = *(volatile int*)&sh->ju;
                    if (s_nz) {
                        const int jue = j + ku + bi - 1 < n ? j + ku + bi - 1 : n;
                        if (jue > ju) ju = jue;
                    } else {
                        atomicCAS(err + 1, 0, j);
                    }
                    s_ju = ju;
                }
            }
            __syncthreads();
            const int jp = s_jp, ju = s_ju;
            if (s_nz) {
                if (jp != 1)
                    for (int t = tid; t <= ju - j; t += kLuThreads) {
                        const size_t a0 = (size_t)(kv + jp - 1) + (size_t)(j - 1) * ldab + (size_t)t * (ldab - 1);
                        const size_t b0 = (size_t)kv + (size_t)(j - 1) * ldab + (size_t)t * (ldab - 1);
                        const double x = __ldcg(ab + a0);
                        ab[a0] = __ldcg(ab + b0);
                        ab[b0] = x;
                    }
                __syncthreads();
                if (km > 0) {
                    const double rp = 1.0 / __ldcg(&AB(kv + 1, j));
                    for (int i = 1 + tid; i <= km; i += kLuThreads) AB(kv + 1 + i, j) = __ldcg(&AB(kv + 1 + i, j)) * rp;
                }
            }
            if (tid == 0) {
                sh->jp = jp;
                sh->ju = ju;
                sh->nz = s_nz;
            }
        }
        if (!grid_barrier(sh, nb, err)) return;
        // all CTAs: A(kv+1+i, j+jj) -= A(kv+1+i, j) * A(kv, j+jj) over the trailing block (dger)
        const int ju = *(volatile int*)&sh->ju, nzp = *(volatile int*)&sh->nz;
        if (nzp && km > 0) {
            const int tot = (ju - j) * km;  // <= kl (kl + ku): far below 2^31 for any band that fits
            for (int e = (int)gtid; e < tot; e += (int)gstride) {
                const int jj = e / km + 1, i = e % km + 1;
                const double y = __ldcg(ab + (size_t)(kv - 1) + (size_t)j * ldab + (size_t)(jj - 1) * (ldab - 1));
                if (y != 0.0) {
                    const double temp = -1.0 * y;
                    const size_t a0 = (size_t)kv + (size_t)j * ldab + (size_t)(jj - 1) * (ldab - 1) + (size_t)(i - 1);
                    ab[a0] = __ldcg(ab + a0) + __ldcg(&AB(kv + 1 + i, j)) * temp;
                }
            }
        }
        if (!grid_barrier(sh, nb, err)) return;
    }
#undef AB
}

// DGBTRS (TRANS='N', one right-hand side): forward substitution with the interchanges and L,
// back substitution with U (dtbsv).  Same operations in the same order for every element as the
// column-by-column DGBTRS; zero entries are divided and propagated too, like the optimized BLAS of
// the shipped run (psi = -0 on the non-corner wall nodes of its snapshots).
//
// The column steps are sequential, so one CTA carries them.  Every element of b has one owner
// thread (element i: thread (i - 1) mod kDsThreads), which alone writes it: in a column step each
// thread applies the column to the elements it owns, and the value the next step needs first (the
// pivot row's b for the forward step, the next x = b / U_jj for the back substitution) is
// published by its owner, so a step needs one barrier.
//   * b stays in global memory; the elements a step touches (j .. j+kl forward, j-k .. j back)
//     live in a window of W shared-memory slots (W a power of two >= k + 4, element i in slot
//     (i - 1) mod W).  An element enters two steps before its first use: its owner loads it into
//     a register one step, stores it into its slot the next.  An element is written back by its
//     owner in the step it becomes final (forward: when swapped into b(j); back: as x).
//   * The band columns stream through a ring of AHEAD + 1 shared-memory slots, filled by
//     cp.async AHEAD columns ahead of their step (16-byte copies from the 16-byte boundary at or
//     below the column's first entry; the column sits at offset s0 & 1 in its slot).
// On this part a step is bound by the SM's FP64 pipe: forward kl, backward kl + ku
// multiply-subtract pairs.  AHEAD = 8 where that ring fits, else 2.
constexpr int kDsThreads = 256;
static __host__ __device__ int direct_slot_len(int kl, int ku) { return (kl + ku + 3) & ~1; }
static int direct_window(int kl, int ku) {
    int w = 64;
    while (w < kl + ku + 4) w *= 2;
    return w;
}
static size_t direct_solve_smem(int kl, int ku, int ahead) {
    return sizeof(double) * ((size_t)(ahead + 1) * (size_t)direct_slot_len(kl, ku) + (size_t)direct_window(kl, ku) + 4) +
           sizeof(int) * (size_t)(ahead + 1);
}

__device__ __forceinline__ void ds_cp16(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void ds_cp4(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void ds_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void ds_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// copies band entries [s0, s0 + len) into a slot from the even index at or below s0 (the slot
// then holds entry s0 at position s0 & 1); every thread commits one group, empty or not
__device__ __forceinline__ void ds_issue(double* slot, const double* ab, size_t s0, int len, bool live, int tid) {
    if (live) {
        const size_t a0 = s0 & ~(size_t)1;
        const int pairs = (int)((s0 - a0) + (size_t)len + 1) >> 1;
        for (int q = tid; q < pairs; q += kDsThreads) ds_cp16(slot + 2 * q, ab + a0 + 2 * (size_t)q);
    }
    ds_commit();
}

template <int kDsAhead>
__global__ void __launch_bounds__(kDsThreads, 1) k_direct_solve(const double* __restrict__ ab, const int* __restrict__ ipiv,
                                                               double* __restrict__ bg, int n, int kl, int ku, int W) {
    constexpr int kDsRing = kDsAhead + 1;
    extern __shared__ __align__(16) double dsm[];
    const int SL = direct_slot_len(kl, ku), mask = W - 1;
    double* ring = dsm;                                  // kDsRing slots of SL doubles
    double* win = ring + (size_t)kDsRing * SL;           // W: the window of b
    double* pub = win + W;                               // [4]: published values, by step parity
    int* ipr = reinterpret_cast<int*>(pub + 4);          // pivots of the columns in the ring
    const int ldab = 2 * kl + ku + 1, kd = kl + ku + 1, kp1 = kl + ku + 1, k = kl + ku;
    const int tid = threadIdx.x;
    auto B = [&](int i) -> double& { return win[(i - 1) & mask]; };
    // the first element >= a that this thread owns
    auto first_owned = [&](int a) {
        int r = (tid - (a - 1)) % kDsThreads;
        if (r < 0) r += kDsThreads;
        return a + r;
    };
    auto owns = [&](int i) { return (i - 1) % kDsThreads == tid; };
    double pend = 0.0;  // the element this thread loaded for the window, stored the next step
    int pend_i = 0;

    // ---- forward: for j = 1 .. n-1, b(j) <-> b(ipiv(j)), then b(j+1 .. j+lm) += L(., j) * (-b(j));
    // the window holds b(j .. j+kl) at step j
    auto issue_fwd = [&](int c) {  // column c's multipliers AB(kd+1 .. kd+kl, c) and its pivot
        const bool live = c <= n - 1;
        double* slot = ring + (size_t)(c % kDsRing) * SL;
        if (live && tid == 0) ds_cp4(ipr + c % kDsRing, ipiv + (c - 1));
        ds_issue(slot, ab, (size_t)kd + (size_t)(c - 1) * (size_t)ldab, kl, live, tid);
    };
    for (int c = 1; c <= kDsAhead; c++) issue_fwd(c);
    for (int i = 1 + tid; i <= n && i <= kl + 1; i += kDsThreads) B(i) = bg[i - 1];
    if (kl + 2 <= n && owns(kl + 2)) {  // needed from step 2
        pend = bg[kl + 1];
        pend_i = kl + 2;
    }
    ds_wait<kDsAhead - 1>();  // column 1
    __syncthreads();
    if (n >= 2 && tid == 0) {
        pub[1] = B(ipr[1 % kDsRing]);  // the value the first step swaps into b(1)
        pub[3] = B(1);
    }
    for (int j = 1; j <= n - 1; j++) {
        ds_wait<kDsAhead - 2>();  // columns j and j + 1
        __syncthreads();
        if (pend_i) {  // b(j + kl + 1), first used in step j + 1
            B(pend_i) = pend;
            pend_i = 0;
        }
        const int sl = j % kDsRing;
        const double* L = ring + (size_t)sl * SL + (((size_t)kd + (size_t)(j - 1) * (size_t)ldab) & 1);
        const int l = ipr[sl];
        const double T = pub[j & 1], S = pub[2 + (j & 1)];
        if (owns(j)) {
            B(j) = T;
            bg[j - 1] = T;  // final for the forward substitution
        }
        if (l != j && owns(l)) B(l) = S;
        const double temp = -T;  // -1.0 * T, exactly
        const int lm = kl < n - j ? kl : n - j;
        for (int i = first_owned(j + 1); i <= j + lm; i += kDsThreads) B(i) = B(i) + L[i - j - 1] * temp;
        if (j + 1 <= n - 1) {
            const int l1 = ipr[(j + 1) % kDsRing];
            if (owns(l1)) pub[(j + 1) & 1] = B(l1);
            if (owns(j + 1)) pub[2 + ((j + 1) & 1)] = B(j + 1);
        }
        const int f = j + kl + 2;  // first used in step j + 2
        if (f <= n && owns(f)) {
            pend = bg[f - 1];
            pend_i = f;
        }
        issue_fwd(j + kDsAhead);
    }
    if (owns(n)) bg[n - 1] = B(n);
    __syncthreads();  // the forward results in bg are visible to the whole CTA

    // ---- back substitution: for j = n .. 1, x = b(j) / U(j,j), b(j) = x, b(i0 .. j-1) -= x U(., j)
    // (step m handles column j = n - m + 1); the window holds b(j-k .. j) at step j
    auto issue_bwd = [&](int m) {  // column n - m + 1: AB(1 .. kp1, j)
        const int c = n - m + 1;
        ds_issue(ring + (size_t)(m % kDsRing) * SL, ab, (size_t)(c - 1) * (size_t)ldab, kp1, c >= 1, tid);
    };
    auto ucol = [&](int m) {
        const int c = n - m + 1;
        return ring + (size_t)(m % kDsRing) * SL + (((size_t)(c - 1) * (size_t)ldab) & 1);
    };
    for (int m = 1; m <= kDsAhead; m++) issue_bwd(m);
    pend_i = 0;
    for (int i = n - tid; i >= 1 && i >= n - k; i -= kDsThreads) B(i) = bg[i - 1];
    if (n - k - 1 >= 1 && owns(n - k - 1)) {  // needed from step j = n - 1
        pend = bg[n - k - 2];
        pend_i = n - k - 1;
    }
    ds_wait<kDsAhead - 1>();  // column n
    __syncthreads();
    if (owns(n)) {
        const double x = B(n) / ucol(1)[kp1 - 1];
        B(n) = x;
        bg[n - 1] = x;
        pub[1] = x;
    }
    for (int m = 1; m <= n; m++) {
        const int j = n - m + 1;
        ds_wait<kDsAhead - 2>();  // columns j and j - 1
        __syncthreads();
        if (pend_i) {  // b(j - k - 1), first used in step j - 1
            B(pend_i) = pend;
            pend_i = 0;
        }
        const double* U = ucol(m);
        const double x = pub[m & 1];
        const int lo = kp1 - j, i0 = 1 > j - k ? 1 : j - k;
        for (int i = first_owned(i0); i <= j - 1; i += kDsThreads) B(i) = B(i) - x * U[lo + i - 1];
        if (j >= 2 && owns(j - 1)) {
            const double x1 = B(j - 1) / ucol(m + 1)[kp1 - 1];
            B(j - 1) = x1;
            bg[j - 2] = x1;
            pub[(m + 1) & 1] = x1;
        }
        const int f = j - k - 2;  // first used in step j - 2
        if (f >= 1 && owns(f)) {
            pend = bg[f - 1];
            pend_i = f;
        }
        issue_bwd(m + kDsAhead);
    }
    ds_wait<0>();
}

// buoyancy (momentum.f90:258-289): Bvec(p) = (Ra_T T_x - Ra_C C_x) r(p) on interior nodes, 0 on
// the boundary rows
__global__ void k_direct_rhs(double* B, const double* Tb, const double* Cb, const double* RowB, Geo g, int n, int comp,
                             double RaT, double RaC) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (p > n) return;
    const int N = cK.nz + 1, ip = (p - 1) / N, kp = (p - 1) % N;
    double v = 0.0;
    if (ip > 0 && ip < cK.nx && kp > 0 && kp < cK.nz) {
        double Tr = 0.0;
        for (int j = -2; j <= 2; j++) Tr += cK.D1[j + 3] * Tb[g.at(ip + j, kp)];
        const double Tx = (Tr / cK.dr) / 1.0;
        if (comp == 0) {
            v = RaT * Tx * RowB[p - 1];
        } else {
            double Cr = 0.0;
            for (int j = -2; j <= 2; j++) Cr += cK.D1[j + 3] * Cb[g.at(ip + j, kp)];
            const double Cx = (Cr / cK.dr) / 1.0;
            const double dot = 0.0 + RaC * Cx;
            v = (RaT != 0.0) ? (RaT * Tx - dot) * RowB[p - 1] : (-dot) * RowB[p - 1];
        }
    }
    B[p - 1] = v;
}

// Stream_grid (momentum.f90:291-317): the solution into SF(0:nx,0:nz), then the side-wall images
// (antisymmetric) for every row, then the top/bottom images (antisymmetric for free slip) for
// every column including the side images
__global__ void k_direct_scatter(double* SF, const double* B, Geo g, int nx, int nz) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int N = nz + 1;
    if (p > (nx + 1) * N) return;
    SF[g.at((p - 1) / N, (p - 1) % N)] = B[p - 1];
}
__global__ void k_direct_images_x(double* SF, Geo g, int nx, int nz) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * (nz + 1)) return;
    const int kp = idx / 3, ip = idx % 3 + 1;
    SF[g.at(-ip, kp)] = -SF[g.at(ip, kp)];
    SF[g.at(nx + ip, kp)] = -SF[g.at(nx - ip, kp)];
}
__global__ void k_direct_images_z(double* SF, Geo g, int nx, int nz, int Vbc) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * (nx + 7)) return;
    const int ip = idx / 3 - 3, kp = idx % 3 + 1;
    if (Vbc == 0) {
        SF[g.at(ip, -kp)] = -SF[g.at(ip, kp)];
        SF[g.at(ip, nz + kp)] = -SF[g.at(ip, nz - kp)];
    } else {
        SF[g.at(ip, -kp)] = SF[g.at(ip, kp)];
        SF[g.at(ip, nz + kp)] = SF[g.at(ip, nz - kp)];
    }
}

// band widths of build_SF_matrix's dry pass (momentum.f90:330-395): the extreme column offsets
// q - p of the folded stencil over all non-identity rows
static void direct_bandwidth(const Engine& E, int* kl, int* ku) {
    static const StencilPts P;
    const int nx = E.K.nx, nz = E.K.nz, N = nz + 1, n = (nx + 1) * N;
    int lo = 0, hi = 0;
    for (int p = 1; p <= n; p++) {
        const int ip = (p - 1) / N, kp = (p - 1) % N;
        const bool corner = (ip == 0 || ip == nx) && (kp == 0 || kp == nz);
        if (corner || (E.cfg.Vbc == 1 && (kp == 0 || kp == nz))) continue;
        for (int q0 = 0; q0 < P.n; q0++) {
            int iq = ip + P.di[q0];
            if (iq < 0) iq = -iq;
            else if (iq > nx) iq = nx - (iq - nx);
            int kq = kp + P.dk[q0];
            if (kq < 0) kq = -kq;
            else if (kq > nz) kq = nz - (kq - nz);
            const int q = N * iq + kq + 1, diff = q - p;
            if (diff < lo) lo = diff;
            else if (diff > hi) hi = diff;
        }
    }
    *kl = -lo;
    *ku = hi;
}

int direct_alloc(Engine& E) {
    if (E.cfg.ivis != 0) return fail(PT_ERR_CONFIG, "the direct solve (direct = 1) is built for ivis = 0 (isoviscous)");
    if (E.cfg.precision != PT_PREC_FP64) return fail(PT_ERR_CONFIG, "the direct solve runs in PT_PREC_FP64");
    if (int rc = upload_tu_consts(E)) return rc;  // this file's copy of the grid constants
    int kl = 0, ku = 0;
    direct_bandwidth(E, &kl, &ku);
    const int n = (E.K.nx + 1) * (E.K.nz + 1), ldab = 2 * kl + ku + 1;
    E.dkl = kl;
    E.dku = ku;
    E.dn = n;
    // the substitution kernel keeps its window of b and its column ring in shared memory
    E.dahead = direct_solve_smem(kl, ku, 8) <= 227 * 1024 ? 8 : 2;
    if (direct_solve_smem(kl, ku, E.dahead) > 227 * 1024)
        return fail(PT_ERR_CONFIG, "direct solve: the band is too wide for the banded substitution kernel");
    const int smem = (int)direct_solve_smem(kl, ku, E.dahead);
    if (E.dahead == 8) CK(cudaFuncSetAttribute(k_direct_solve<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    else CK(cudaFuncSetAttribute(k_direct_solve<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    CK(cudaMalloc(&E.dMB, sizeof(double) * (size_t)ldab * (size_t)n));
    CK(cudaMalloc(&E.dRow, sizeof(double) * (size_t)n));
    CK(cudaMalloc(&E.dB, sizeof(double) * (size_t)n));
    CK(cudaMalloc(&E.dipiv, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&E.dlu, sizeof(LuShared)));
    CK(cudaMalloc(&E.dluerr, 2 * sizeof(int)));
    E.bytes_allocated += sizeof(double) * ((size_t)ldab + 2) * (size_t)n + sizeof(int) * (size_t)n;
    // Matrix_element for every (stencil point, image signs, row kind)
    static const StencilPts P;
    ElemTable T;
    for (int q = 0; q < kStencilPts; q++) {
        T.di[q] = P.di[q];
        T.dk[q] = P.dk[q];
        for (int rs = 0; rs < 2; rs++)
            for (int ss = 0; ss < 2; ss++)
                for (int row = 0; row < 3; row++) {
                    int kind = 0;
                    const double v = matrix_element(E, P.di[q], P.dk[q], rs, ss, row, &kind);
                    T.v[q][rs][ss][row] = kind ? v : std::nan("");
                }
    }
    CK(cudaMemcpyToSymbol(cET, &T, sizeof T));
    E.direct_ready = false;
    return 0;
}

void direct_free(Engine& E) {
    for (void* p : {(void*)E.dMB, (void*)E.dRow, (void*)E.dB, (void*)E.dipiv, (void*)E.dlu, (void*)E.dluerr})
        if (p) cudaFree(p);
    E.dMB = E.dRow = E.dB = nullptr;
    E.dipiv = E.dluerr = nullptr;
    E.dlu = nullptr;
}

// build_SF_matrix: assembly, equilibration and factorisation (once: the isoviscous operator does
// not change)
static int direct_factor(Engine& E) {
    const int n = E.dn, kl = E.dkl, ku = E.dku, ldab = 2 * kl + ku + 1;
    CK(cudaMemsetAsync(E.dMB, 0, sizeof(double) * (size_t)ldab * (size_t)n, E.st));
    CK(cudaMemsetAsync(E.derr, 0, sizeof(int), E.st));
    CK(cudaMemsetAsync(E.dlu, 0, sizeof(LuShared), E.st));
    CK(cudaMemsetAsync(E.dluerr, 0, 2 * sizeof(int), E.st));
    PT_COUNT(), k_direct_assemble<<<nblk(n, 128), 128, 0, E.st>>>(E.dMB, n, ldab, kl, ku, E.K.nx, E.K.nz, E.cfg.Vbc);
    PT_COUNT(), k_direct_equ<<<nblk(n, 128), 128, 0, E.st>>>(E.dMB, E.dRow, n, ldab, kl, ku, E.derr);
    CKL("direct assembly");
    int h = 0;
    CK(cudaMemcpyAsync(&h, E.derr, sizeof(int), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    if (h) return fail(PT_ERR_SINGULAR_COARSE, "direct solve: DGBEQU found a zero row");
    // one CTA per SM, all resident (cooperative launch)
    int dev = 0, sms = 0, per = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_direct_lu, kLuThreads, 0));
    if (per < 1) return fail(PT_ERR_CUDA, "direct solve: the LU kernel cannot be resident");
    double* ab = E.dMB;
    int* ipiv = E.dipiv;
    int* lu_err = E.dluerr;
    int nn = n, kkl = kl, kku = ku;
    LuShared* sh = reinterpret_cast<LuShared*>(E.dlu);
    void* args[] = {&ab, &ipiv, &nn, &kkl, &kku, &lu_err, &sh};
    PT_COUNT();
    CK(cudaLaunchCooperativeKernel((void*)k_direct_lu, dim3(sms), dim3(kLuThreads), args, 0, E.st));
    int hl[2] = {0, 0};
    CK(cudaMemcpyAsync(hl, lu_err, 2 * sizeof(int), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    if (hl[0] & 8) return fail(PT_ERR_ITER_CAP, "direct solve: LU grid barrier timed out");
    if (hl[1]) return fail(PT_ERR_SINGULAR_COARSE, "direct solve: DGBTRF found a zero pivot");
    // the isoviscous viscosity the statistics read (vis = 1, as the reference's direct path sets it)
    PT_COUNT(), k_fill<<<nblk(E.g1.elems(), 256), 256, 0, E.st>>>(E.vis[1], 1.0, E.g1.elems());
    CKL("direct solve: viscosity");
    E.direct_ready = true;
    return 0;
}

// solve_SF_equation: buoyancy right-hand side, banded substitutions, Stream_grid
int direct_solve(Engine& E, pt_solve_info* info) {
    PhaseTimer tm(E, PH_SOLVE);
    if (!E.direct_ready) {
        PhaseTimer tf(E, PH_FACTOR);
        if (int rc = direct_factor(E)) return rc;
    }
    const int n = E.dn, kl = E.dkl, ku = E.dku;
    PT_COUNT(), k_direct_rhs<<<nblk(n, 128), 128, 0, E.st>>>(E.dB, E.Tbuoy, E.Cbuoy, E.dRow, E.g1, n, E.cfg.comp,
                                                            E.cfg.RaT, E.cfg.RaC);
    const size_t smem = direct_solve_smem(kl, ku, E.dahead);
    const int W = direct_window(kl, ku);
    if (E.dahead == 8) PT_COUNT(), k_direct_solve<8><<<1, kDsThreads, smem, E.st>>>(E.dMB, E.dipiv, E.dB, n, kl, ku, W);
    else PT_COUNT(), k_direct_solve<2><<<1, kDsThreads, smem, E.st>>>(E.dMB, E.dipiv, E.dB, n, kl, ku, W);
    PT_COUNT(), k_direct_scatter<<<nblk(n, 128), 128, 0, E.st>>>(E.SF, E.dB, E.g1, E.K.nx, E.K.nz);
    PT_COUNT(), k_direct_images_x<<<nblk(3 * (E.K.nz + 1), 128), 128, 0, E.st>>>(E.SF, E.g1, E.K.nx, E.K.nz);
    PT_COUNT(), k_direct_images_z<<<nblk(3 * (E.K.nx + 7), 128), 128, 0, E.st>>>(E.SF, E.g1, E.K.nx, E.K.nz,
                                                                                E.cfg.Vbc);
    CKL("direct solve");
    E.cycles = 0;
    E.resid_ratio = 0.0;
    if (info) {
        info->resid_ratio = 0.0;
        info->n_eta = 0;
    }
    return 0;
}

}  // namespace pt
