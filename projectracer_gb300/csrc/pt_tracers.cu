// pt_tracers.cu -- tracer kernels: the RK4 stage loops of energy_time (energy.f90:258-536)
// with the Taylor interpolation of interpolate (composition.f90:1359-1393), and the tracer->grid
// projection tracers_to_corners_iC_continuous (composition.f90:942-1087).
//
// Projection, GB300 form.  FP64 precision: a counting sort of tracer IDs by cell (cell = nint of
// the position), a per-cell sort of the IDs, per-cell partial sums of T*S, C*S and S for the 3x3
// target nodes in ascending ID order, then per node a fixed-order sum of the 9 partials.  Counts
// and cell indices are integers (bit-exact); every floating-point sum has a fixed association, so
// the result is deterministic and equals the oracle's canonical order bit for bit (the arithmetic
// uses explicit round-to-nearest intrinsics, no contraction).  Mixed precision: one pass with
// per-tracer fixed-point contributions and integer sums (k_project_fx), deterministic without a
// sort and independent of the tracer order; counts bit-exact, sums to 2^-28.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>

#include "pt_consts.cuh"

namespace pt {

// z-direction interpolation stencils with 1/ds^j folded in, FP32 (mixed-precision stage)
static __constant__ float cDmf[4][7];
// dr / 2^28 and ds / 2^28 in FP32 (exact for power-of-two spacings): 28-bit fixed-point offsets
// to lengths
static __constant__ float cH28[2];

int upload_consts_tracers(const Engine& E) {
    if (int rc = upload_tu_consts(E)) return rc;
    float d[4][7] = {};
    for (int m = 1; m <= 3; m++)
        for (int j = 0; j < 7; j++) d[m][j] = (float)(E.K.Dm[m][j] * E.K.inv_ds_pow[m]);
    CK(cudaMemcpyToSymbol(cDmf, d, sizeof d));
    const float h28[2] = {(float)(E.K.dr / 268435456.0), (float)(E.K.ds / 268435456.0)};
    CK(cudaMemcpyToSymbol(cH28, h28, sizeof h28));
    return 0;
}

// nint(x * 2^p) (round half away from zero, as llround), exactly, from the bit pattern with
// integer operations (this part's FP64 pipe is its scarcest resource).  |x * 2^p| >= 2^30
// (and NaN) saturate to +-2^30; zero and subnormal x give 0.
__device__ __forceinline__ int nint_pow2(double x, int p) {
    const unsigned long long raw = (unsigned long long)__double_as_longlong(x);
    const bool neg = (raw >> 63) != 0;
    const unsigned long long b = raw & 0x7FFFFFFFFFFFFFFFull;
    const int be = (int)(b >> 52);
    const int e = be - 1023 + p;  // exponent of |x| * 2^p
    if (be == 0 || e < -1) return 0;
    if (e >= 30) return neg ? -(1 << 30) : (1 << 30);
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;  // m * 2^(e-52)
    const int sh = 52 - e;  // 23..53
    const int v = (int)((m + (1ull << (sh - 1))) >> sh);
    return neg ? -v : v;
}

__device__ __forceinline__ int cell_index(double x, double inv, double h, int exact, int p) {
    if (exact) return nint_pow2(x, p);
    return (int)llround(x / h);
}

// 0 <= x <= hi (hi > 0) by comparing bit patterns: non-negative doubles order like their bits,
// negative values and NaN compare above hi, -0 counts as 0
__device__ __forceinline__ bool in_range(double x, double hi) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return b <= (unsigned long long)__double_as_longlong(hi) || b == 0x8000000000000000ull;
}

// ---------------------------------------------------------------- projection
// Cell of each tracer and the per-cell counts.  Tracer IDs are spatially grouped (seeding order),
// so the lanes of a warp mostly share a cell: one atomic per distinct cell of the warp
// (__match_any_sync) instead of one per tracer.  Integer counts: the result does not depend on
// the grouping.  The grid is a whole number of warps; lanes past n carry cell -1.
__global__ void k_cells(const double* __restrict__ r, const double* __restrict__ s, int64_t n,
                        int32_t* __restrict__ cell, int32_t* __restrict__ count, int* err) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1;
    if (t < n) {
        const double rr = r[t], ss = s[t];
        if (!(in_range(rr, cK.aspect) && in_range(ss, 1.0))) {
            atomicOr(err, 1);  // composition.f90:1007-1010
        } else {
            const int i = cell_index(rr, cK.inv_dr, cK.dr, cK.exact_div, cK.p_inv_dr);
            const int k = cell_index(ss, cK.inv_ds, cK.ds, cK.exact_div, cK.p_inv_ds);
            c = i + (cK.nx + 1) * k;
        }
        cell[t] = c;
    }
    const unsigned group = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && (int)(threadIdx.x & 31) == __ffs(group) - 1) atomicAdd(&count[c], __popc(group));
}

// exclusive scan of int32 counts: block scan, scan of block totals, add offsets
__global__ void k_scan_block(const int32_t* in, int32_t* out, int32_t* totals, int n) {
    __shared__ int32_t ws[32];
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    int v = gid < n ? in[gid] : 0;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int y = (lane < (int)(blockDim.x >> 5)) ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += z;
        }
        ws[lane] = y;
    }
    __syncthreads();
    int base = wid > 0 ? ws[wid - 1] : 0;
    if (gid < n) out[gid] = base + x - v;
    if (threadIdx.x == blockDim.x - 1) totals[blockIdx.x] = base + x;
}
// exclusive scan of the nb block totals in place: one CTA of 1024 threads, a contiguous chunk per
// thread (chunk sums scanned across the CTA, then each chunk written serially)
constexpr int kScanTotThreads = 1024;
__global__ void __launch_bounds__(kScanTotThreads) k_scan_totals(int32_t* totals, int nb) {
    __shared__ int32_t ws[32];
    const int per = (nb + kScanTotThreads - 1) / kScanTotThreads;
    const int b0 = (int)threadIdx.x * per, b1 = min(b0 + per, nb);
    int v = 0;
    for (int b = b0; b < b1; b++) v += totals[b];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int y = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += z;
        }
        ws[lane] = y;
    }
    __syncthreads();
    int acc = (wid > 0 ? ws[wid - 1] : 0) + x - v;
    for (int b = b0; b < b1; b++) {
        const int t = totals[b];
        totals[b] = acc;
        acc += t;
    }
}
__global__ void k_scan_add(int32_t* out, const int32_t* totals, int n) {
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid < n) out[gid] += totals[blockIdx.x];
}

// Tracer IDs into their cell's segment: one atomic per distinct cell of a warp, lanes placed by
// rank, so IDs of one warp keep ascending order inside a cell and the per-cell sort that follows
// mostly sees sorted input.
__global__ void k_scatter(const int32_t* __restrict__ cell, int64_t n, const int32_t* __restrict__ start,
                          int32_t* cursor, int32_t* __restrict__ list) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = t < n ? cell[t] : -1;
    const unsigned group = __match_any_sync(0xffffffffu, c);
    const int lane = (int)(threadIdx.x & 31), leader = __ffs(group) - 1;
    int base = 0;
    if (c >= 0 && lane == leader) base = atomicAdd(&cursor[c], __popc(group));
    base = __shfl_sync(group, base, leader);
    if (c >= 0) list[start[c] + base + __popc(group & ((1u << lane) - 1u))] = (int32_t)t;
}

// ascending tracer IDs inside each cell (insertion sort: cells hold a few dozen tracers)
__global__ void k_sort_cells(int32_t* list, const int32_t* start, const int32_t* count, int ncell) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int b = start[c], n = count[c];
    for (int a = 1; a < n; a++) {
        int32_t key = list[b + a];
        int j = a - 1;
        while (j >= 0 && list[b + j] > key) {
            list[b + j + 1] = list[b + j];
            j--;
        }
        list[b + j + 1] = key;
    }
}

__device__ __forceinline__ double shape1(double x, int i, double h, double inv, int exact) {
    double d = fabs(__dsub_rn(x, __dmul_rn((double)i, h)));
    double q = exact ? __dmul_rn(d, inv) : __ddiv_rn(d, h);
    double a = __dsub_rn(1.0, q);
    return a > 0.0 ? a : 0.0;
}

// per-cell partial sums for the 3x3 nodes around the cell; planes of ncell: [q*9 + dz*3 + dx]
// Continuous C (tracers_to_corners_iC_continuous): T*S, C*S, S.  Discrete types (OG,
// tracers_to_corners_OG, composition.f90:1139-1166, the type held in Ct as 0.0 / 1.0): T*S, the
// shape sum of the type-1 tracers (count_type_real(1)) and that of the type-0 tracers
// (count_type_real(0)); a tracer of the other type leaves a plane's partial unchanged (+0.0 and
// x 1.0 are exact), so the sums are those of the reference's per-type loops in ID order.
template <bool OG>
__global__ void k_cell_partials(const double* __restrict__ r, const double* __restrict__ s,
                                const double* __restrict__ Tt, const double* __restrict__ Ct,
                                const int32_t* __restrict__ list, const int32_t* __restrict__ start,
                                const int32_t* __restrict__ count, int ncell, double* __restrict__ P,
                                int comp) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int nx1 = cK.nx + 1;
    int ci = c % nx1, ck = c / nx1;
    double aT[9], aC[9], aS[9];
#pragma unroll
    for (int q = 0; q < 9; q++) { aT[q] = 0.0; aC[q] = 0.0; aS[q] = 0.0; }
    int b = start[c], n = count[c];
    for (int a = 0; a < n; a++) {
        int32_t t = list[b + a];
        double rr = r[t], ss = s[t], tv = Tt[t], cv = comp ? Ct[t] : 0.0;
        const bool type1 = OG && cv != 0.0;
        double wx[3], wz[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            wx[d] = shape1(rr, ci + d - 1, cK.dr, cK.inv_dr, cK.exact_div);
            wz[d] = shape1(ss, ck + d - 1, cK.ds, cK.inv_ds, cK.exact_div);
        }
#pragma unroll
        for (int dz = 0; dz < 3; dz++)
#pragma unroll
            for (int dx = 0; dx < 3; dx++) {
                double S = __dmul_rn(wx[dx], wz[dz]);
                int q = dz * 3 + dx;
                aT[q] = __dadd_rn(aT[q], __dmul_rn(tv, S));
                if (OG) {
                    if (type1) aC[q] = __dadd_rn(aC[q], S);
                    else aS[q] = __dadd_rn(aS[q], S);
                } else {
                    aC[q] = __dadd_rn(aC[q], __dmul_rn(cv, S));
                    aS[q] = __dadd_rn(aS[q], S);
                }
            }
    }
#pragma unroll
    for (int q = 0; q < 9; q++) {
        P[(size_t)q * ncell + c] = aT[q];
        P[(size_t)(9 + q) * ncell + c] = aC[q];
        P[(size_t)(18 + q) * ncell + c] = aS[q];
    }
}

// per node: fixed-order sum of the partials of the 3x3 surrounding cells, then the ratio.
// OG: the shape sum is nempty_real = count_type_real(0) + count_type_real(1)
// (composition.f90:1221), C = count_type_real(1) / nempty_real, T = T1 / nempty_real (1253-1256).
template <bool OG>
__global__ void k_node_sums(const double* __restrict__ P, const int32_t* __restrict__ count, int ncell,
                            double* Tratio, double* Cnew, int32_t* nempty, Geo g, int comp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    const int nx = cK.nx, nz = cK.nz;
    if (i > nx) return;
    double sT = 0.0, sC = 0.0, sS = 0.0;
    for (int ck = k - 1; ck <= k + 1; ck++)
        for (int ci = i - 1; ci <= i + 1; ci++) {
            if (ci < 0 || ci > nx || ck < 0 || ck > nz) continue;
            int c = ci + (nx + 1) * ck;
            int q = (k - ck + 1) * 3 + (i - ci + 1);
            sT = __dadd_rn(sT, P[(size_t)q * ncell + c]);
            sC = __dadd_rn(sC, P[(size_t)(9 + q) * ncell + c]);
            sS = __dadd_rn(sS, P[(size_t)(18 + q) * ncell + c]);
        }
    if (OG) sS = __dadd_rn(sS, sC);
    int c = i + (nx + 1) * k;
    nempty[c] = count[c];
    if (sS > 0.0) {
        Tratio[g.at(i, k)] = __ddiv_rn(sT, sS);
        if (comp) Cnew[g.at(i, k)] = __ddiv_rn(sC, sS);
    }
}

// count_type(1, i, k) of tracers_to_corners_OG (composition.f90:1141, 1173): type-1 tracers
// (Ct != 0) per nearest node, one atomic per distinct node of a warp.  Positions were checked by
// the projection that runs before it; a tracer outside the domain is skipped.
__global__ void k_count_type1(const double* __restrict__ r, const double* __restrict__ s,
                              const double* __restrict__ Ct, int64_t n, int32_t* __restrict__ count1) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1;
    if (t < n && Ct[t] != 0.0) {
        const double rr = r[t], ss = s[t];
        if (in_range(rr, cK.aspect) && in_range(ss, 1.0)) {
            const int i = cell_index(rr, cK.inv_dr, cK.dr, cK.exact_div, cK.p_inv_dr);
            const int k = cell_index(ss, cK.inv_ds, cK.ds, cK.exact_div, cK.p_inv_ds);
            c = i + (cK.nx + 1) * k;
        }
    }
    const unsigned group = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && (int)(threadIdx.x & 31) == __ffs(group) - 1) atomicAdd(&count1[c], __popc(group));
}

// tracer types (int32 0/1) <-> the type as 0.0 / 1.0 in the composition array; a type other
// than 0 and 1 sets bad (ntype = 1)
__global__ void k_types_to_c(const int32_t* __restrict__ ty, double* __restrict__ c, int64_t n, int* bad) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int32_t v = ty[t];
    if (v != 0 && v != 1) atomicOr(bad, 4);
    c[t] = v == 1 ? 1.0 : 0.0;
}
__global__ void k_c_to_types(const double* __restrict__ c, int32_t* __restrict__ ty, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) ty[t] = c[t] != 0.0 ? 1 : 0;
}

int types_to_c(Engine& E, const int32_t* dev_types, double* c) {
    CK(cudaMemsetAsync(E.derr, 0, sizeof(int), E.st));
    PT_COUNT(), k_types_to_c<<<nblk(E.ntr, 256), 256, 0, E.st>>>(dev_types, c, E.ntr, E.derr);
    CKL("k_types_to_c");
    int h = 0;
    CK(cudaMemcpyAsync(&h, E.derr, sizeof(int), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    if (h) return fail(PT_ERR_ARG, "tracer types must be 0 or 1 (ntype = 1)");
    return 0;
}
int c_to_types(Engine& E, const double* c, int32_t* dev_types) {
    PT_COUNT(), k_c_to_types<<<nblk(E.ntr, 256), 256, 0, E.st>>>(c, dev_types, E.ntr);
    CKL("k_c_to_types");
    return 0;
}

// ---------------------------------------------------------------- projection, mixed precision
// The same sums as k_cell_partials, in fixed point (scale 2^28) with integer arithmetic only, so
// that each node's totals are exact integer sums: the result does not depend on the tracer order
// or on the scheduling, it is bit-deterministic, and oracle/project_fx.py restates it exactly.
//   position  u = x / dr (x * 2^p for dr = 2^-p, from the bit pattern); cell i0 = floor(u),
//             fraction fx = floor((u - i0) * 2^28); a tracer on the right (top) wall goes to the
//             last cell with fx = 2^28;
//   counts    per nearest node (the reference's nint cell): i0 + (fx >= 2^27);
//   weights   wx = (2^28 - fx, fx) for the nodes i0, i0+1 (the reference's hat functions: the
//             third node of its 3x3 neighbourhood has weight 0), wz likewise,
//             S = (wx_a wz_b + 2^27) >> 28;
//   values    T28 = round(T 2^28) (half away from zero, |T| < 4), TS = (T28 S + 2^27) >> 28, CS.
constexpr int kFixOne = 1 << 28;

// floor(x * 2^p) and the first 28 bits of its fraction for x >= 0 (domain-checked), from the bit
// pattern with 32-bit operations: x * 2^(p+28) = m * 2^-sh with m the 53-bit significand (high
// word mh, low word lo).  Zero and subnormal x give sh >= 64, hence 0; x * 2^p >= 2^24 saturates.
__device__ __forceinline__ int floor_fix_pow2(double x, int p, uint32_t& frac) {
    const uint32_t hw = (uint32_t)__double2hiint(x) & 0x7FFFFFFFu, lo = (uint32_t)__double2loint(x);
    const int sh = 1047 - p - (int)(hw >> 20);
    if (sh <= 4) {
        frac = 0;
        return 1 << 24;
    }
    const uint32_t mh = (hw & 0xFFFFFu) | 0x100000u;
    const uint32_t xl = sh < 32 ? __funnelshift_r(lo, mh, sh) : (sh < 64 ? mh >> (sh - 32) : 0u);
    frac = xl & (uint32_t)(kFixOne - 1);
    return sh - 4 < 32 ? (int)(mh >> (sh - 4)) : 0;  // m >> (sh + 28)
}

template <bool EXACT>
__device__ __forceinline__ int floor_fix(double x, double h, int p, uint32_t& frac) {
    if (EXACT) return floor_fix_pow2(x, p, frac);
    const double u = x / h;
    const double fl = floor(u);
    frac = (uint32_t)((u - fl) * 268435456.0);
    return (int)fl;
}

// round(v * 2^28), half away from zero, from the bit pattern: |v| * 2^28 = m * 2^-sh, and with
// q = floor(2 |v| 2^28) = m >> (sh - 1) (below 2^31 for |v| < 4) the result is (q + 1) >> 1.
// |v| >= 4 (and NaN/Inf) set bad.
__device__ __forceinline__ int fix28(double v, int& bad) {
    const uint32_t hw = (uint32_t)__double2hiint(v), lo = (uint32_t)__double2loint(v);
    const int k = 1046 - (int)((hw >> 20) & 0x7FFu);  // sh - 1
    if (k < 22) {
        bad |= 2;
        return 0;
    }
    const uint32_t mh = (hw & 0xFFFFFu) | 0x100000u;
    const uint32_t q = k < 32 ? __funnelshift_r(lo, mh, k) : (k < 64 ? mh >> (k - 32) : 0u);
    const int a = (int)((q + 1u) >> 1);
    return (hw >> 31) ? -a : a;
}

// Re-sort threshold of the mixed path, as a fraction of the way from cell order to a random order
// in runs (cells) per 16 consecutive tracers.  Measured at 1024x512 with 32 tracers per cell:
// the seeding order loses about half of its locality within ten steps; a random order costs the RK
// stage 1.25 ms instead of 0.42 ms and the projection 0.93 ms instead of about 0.5 ms, and a
// re-sort costs about 0.35 ms.
constexpr double kResortFrac = 0.5;

// cell and fractions of a tracer; false outside the domain (composition.f90:1007-1010).  EXACT:
// dr and ds are powers of two (integer decoding only, no FP64 arithmetic)
struct TracerCell {
    int i0, k0, near;  // cell, nearest corner (a + 2 b)
    uint32_t fx, fz;
};
template <bool EXACT>
__device__ __forceinline__ bool locate(double rr, double ss, TracerCell& c) {
    if (!(in_range(rr, cK.aspect) && in_range(ss, 1.0))) return false;
    c.i0 = floor_fix<EXACT>(rr, cK.dr, cK.p_inv_dr, c.fx);
    c.k0 = floor_fix<EXACT>(ss, cK.ds, cK.p_inv_ds, c.fz);
    int ni = c.i0 + (int)(c.fx >> 27), nk = c.k0 + (int)(c.fz >> 27);
    if (c.i0 >= cK.nx) { c.i0 = cK.nx - 1; c.fx = kFixOne; }  // on the right wall
    if (c.k0 >= cK.nz) { c.k0 = cK.nz - 1; c.fz = kFixOne; }  // on the top wall
    c.near = (ni - c.i0) + 2 * (nk - c.k0);
    return true;
}

// One CTA per chunk of kPjChunk consecutive tracers, kPjPer consecutive tracers per lane.  The
// tracers are kept in cell order, so a lane's tracers mostly share a cell: it keeps the running
// sums of its current cell (a run) in registers.  A lane that finishes a run adds it at once to a
// shared-memory window of the grid (64-bit integer shared atomics; 8% faster than queueing the
// runs of a warp and draining them together, which moved every run through shared memory twice).
// At the end the window is added to the global sums with one integer atomic per non-zero value.
// The window is the box of the cells of every lane's first and last tracer plus one cell of
// margin; runs outside it (and every run when the box is too large for the window) go to the
// global sums directly.
// acc: [node][TS, CS, S, count] int64; window planes [TS | CS | S + (count << 44)] (a chunk's S
// stays below 2^44, its counts below 2^20).  runs (optional): the number of runs.
constexpr int kPjThreads = 256, kPjPer = 16, kPjChunk = kPjThreads * kPjPer, kPjWin = 1280;
constexpr int kPjCountShift = 44;


template <bool EXACT, bool COMP>
__global__ void __launch_bounds__(kPjThreads, 3) k_project_fx(const double* __restrict__ r, const double* __restrict__ s,
                                                              const double* __restrict__ Tt,
                                                              const double* __restrict__ Ct, int64_t n,
                                                              unsigned long long* __restrict__ acc, int* err,
                                                              unsigned long long* runs) {
    __shared__ unsigned long long win[3 * kPjWin];  // planes [TS | CS | S + count << 44] of the window
    __shared__ int box[4];
    const int nx1 = cK.nx + 1;
    const int lane = threadIdx.x & 31;
    const int64_t t0 = (int64_t)blockIdx.x * kPjChunk + (int64_t)threadIdx.x * kPjPer;
    const int64_t t1 = t0 + kPjPer < n ? t0 + kPjPer : n;
    int bad = 0;
    if (threadIdx.x == 0) { box[0] = INT_MAX; box[1] = -1; box[2] = INT_MAX; box[3] = -1; }
    __syncthreads();
    for (int q = 0; q < 2 && t0 < t1; q++) {
        const int64_t t = q ? t1 - 1 : t0;
        TracerCell c;
        if (locate<EXACT>(r[t], s[t], c)) {
            atomicMin(&box[0], c.i0); atomicMax(&box[1], c.i0);
            atomicMin(&box[2], c.k0); atomicMax(&box[3], c.k0);
        }
    }
    __syncthreads();
    // window: cells box +- 1, i.e. nodes [imin-1, imax+2] x [kmin-1, kmax+2], odd row pitch; its
    // geometry is re-derived from box[] where a run is flushed (fewer live registers in the tracer loop)
    auto geometry = [&](int& wi, int& wk, int& W, int& H, int& P) {
        wi = box[0] - 1; wk = box[2] - 1;
        W = box[1] - box[0] + 4; H = box[3] - box[2] + 4; P = W | 1;
        return box[1] >= 0 && P * H <= kPjWin;
    };
    {
        int wi, wk, W, H, P;
        if (geometry(wi, wk, W, H, P)) {
            for (int q = threadIdx.x; q < 3 * kPjWin; q += kPjThreads) win[q] = 0ull;
            __syncthreads();
        }
    }
    unsigned nruns = 0;      // runs of this lane
    long long aT[4], aC[4], aS[4];
    uint32_t cnt = 0;  // four 8-bit counters, one per corner (a run holds at most kPjPer tracers)
    int ri = -1, rk = -1;
    // one warp-synchronous step: lane tracer (valid: a tracer to add, fin: the lane's last call)
    auto step = [&](bool valid, double rr, double ss, double tv, double cv, bool fin) {
        TracerCell c;
        bool inside = false;
        if (valid) {
            inside = locate<EXACT>(rr, ss, c);
            if (!inside) bad |= 1;
        }
        const bool close = ri >= 0 && (fin || (inside && (c.i0 != ri || c.k0 != rk)));
        if (close) {  // the run's sums into the window (or the global sums)
            int wi, wk, W, H, P;
            const bool use_win = geometry(wi, wk, W, H, P);
            const int li = ri - wi, lk = rk - wk;
            if (use_win && li >= 0 && lk >= 0 && li + 1 < W && lk + 1 < H) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int o = (li + (j & 1)) + P * (lk + (j >> 1));
                    const unsigned long long vT = (unsigned long long)aT[j], vC = (unsigned long long)aC[j];
                    const unsigned long long vS = (unsigned long long)aS[j] +
                                                  ((unsigned long long)((cnt >> (8 * j)) & 255u) << kPjCountShift);
                    if (vT) atomicAdd(&win[o], vT);
                    if (vC) atomicAdd(&win[kPjWin + o], vC);
                    if (vS) atomicAdd(&win[2 * kPjWin + o], vS);
                }
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const size_t node = (size_t)(ri + (j & 1)) + (size_t)nx1 * (size_t)(rk + (j >> 1));
                    const unsigned long long v4[4] = {(unsigned long long)aT[j], (unsigned long long)aC[j],
                                                      (unsigned long long)aS[j], (cnt >> (8 * j)) & 255u};
#pragma unroll
                    for (int p = 0; p < 4; p++)
                        if (v4[p]) atomicAdd(&acc[4 * node + p], v4[p]);
                }
            }
            nruns++;
            ri = -1;
        }
        if (!inside) return;
        if (ri < 0) {
            ri = c.i0;
            rk = c.k0;
#pragma unroll
            for (int j = 0; j < 4; j++) aT[j] = aC[j] = aS[j] = 0;
            cnt = 0;
        }
        const int T28 = fix28(tv, bad), C28 = COMP ? fix28(cv, bad) : 0;
        const uint32_t wx[2] = {(uint32_t)kFixOne - c.fx, c.fx}, wz[2] = {(uint32_t)kFixOne - c.fz, c.fz};
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int S = (int)(((unsigned long long)wx[j & 1] * wz[j >> 1] + (1ull << 27)) >> 28);
            aS[j] += S;
            aT[j] += (int)(((long long)T28 * S + (1ll << 27)) >> 28);  // |.| <= |T28|: fits
            if (COMP) aC[j] += (int)(((long long)C28 * S + (1ll << 27)) >> 28);
        }
        cnt += 1u << (8 * c.near);
    };
    // consecutive pairs with 16-byte loads (t0 is even; the arrays are 16-byte aligned); every
    // lane runs the same number of steps (the warp's last lanes may hold fewer tracers)
    auto ld2 = [](const double* a, int64_t i) { return __ldg(reinterpret_cast<const double2*>(a + i)); };
    for (int q = 0; q < kPjPer; q += 2) {
        const int64_t t = t0 + q;
        if (t + 1 < t1) {
            const double2 r2 = ld2(r, t), s2 = ld2(s, t), T2 = ld2(Tt, t);
            const double2 C2 = COMP ? ld2(Ct, t) : make_double2(0.0, 0.0);
            step(true, r2.x, s2.x, T2.x, C2.x, false);
            step(true, r2.y, s2.y, T2.y, C2.y, false);
        } else {
            const bool v = t < t1;
            step(v, v ? r[t] : 0.0, v ? s[t] : 0.0, v ? Tt[t] : 0.0, v && COMP ? Ct[t] : 0.0, false);
            step(false, 0.0, 0.0, 0.0, 0.0, false);
        }
    }
    step(false, 0.0, 0.0, 0.0, 0.0, true);  // close the open runs
    if (bad) atomicOr(err, bad);
    if (runs) {
        const unsigned wr = __reduce_add_sync(0xffffffffu, nruns);
        if (lane == 0 && wr) atomicAdd(runs, (unsigned long long)wr);
    }
    int wi, wk, W, H, P;
    if (!geometry(wi, wk, W, H, P)) return;
    __syncthreads();
    const int nw = W * H;
    const unsigned long long smask = (1ull << kPjCountShift) - 1ull;
    for (int q = threadIdx.x; q < 3 * nw; q += kPjThreads) {
        const int p = q % 3, cell = q / 3;
        const int row = cell / W, col = cell - row * W;
        const unsigned long long v = win[p * kPjWin + row * P + col];
        if (!v) continue;
        unsigned long long* a = &acc[4 * ((size_t)(wi + col) + (size_t)nx1 * (size_t)(wk + row))];
        if (p < 2) {
            atomicAdd(&a[p], v);
        } else {
            if (v & smask) atomicAdd(&a[2], v & smask);
            if (v >> kPjCountShift) atomicAdd(&a[3], v >> kPjCountShift);
        }
    }
}

// per node: the ratios of the fixed-point sums (the 2^28 scale cancels exactly) and the count
__global__ void k_node_fx(const unsigned long long* __restrict__ acc, double* Tratio, double* Cnew, int32_t* nempty,
                          Geo g, int comp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    const int nx = cK.nx;
    if (i > nx) return;
    const size_t c = (size_t)i + (size_t)(nx + 1) * (size_t)k;
    nempty[c] = (int32_t)acc[4 * c + 3];
    const long long sS = (long long)acc[4 * c + 2];
    if (sS > 0) {
        const double dS = (double)sS;
        Tratio[g.at(i, k)] = __ddiv_rn((double)(long long)acc[4 * c], dS);
        if (comp) Cnew[g.at(i, k)] = __ddiv_rn((double)(long long)acc[4 * c + 1], dS);
    }
}

// scratch of one projection: cell of each tracer, per-cell counts/starts/list, scan blocks,
// the 27 partial planes and the out-of-domain flag
struct ProjScratch {
    int32_t *tcell, *clist, *ccount, *cstart, *scan_tmp;
    double* cpart;
    int* derr;
    unsigned long long* runs;  // runs counter of the mixed projection (nullptr: not counted)
};

static int project_with(Engine& E, const ProjScratch& W, const double* r, const double* s, const double* Tt,
                        const double* T0f, int smooth) {
    const int nx = E.K.nx, nz = E.K.nz;
    const int ncell = (nx + 1) * (nz + 1);
    const int64_t n = E.ntr;
    int rc;
    PhaseTimer tm(E, PH_PROJECT);
    if (T0f && T0f != E.Tratio) {
        if ((rc = copy_field(E, E.Tratio, T0f))) return rc;
    }
    {
        // the kernel timer brackets k_project_fx alone on the mixed path (the roofline's dominant
        // kernel), the whole sort-based sequence on the FP64 path
        CK(cudaMemsetAsync(W.ccount, 0, sizeof(int32_t) * (size_t)ncell, E.st));
        CK(cudaMemsetAsync(W.derr, 0, sizeof(int), E.st));
        dim3 grid(nblk(nx + 1, 128), nz + 1);
        if (E.cfg.precision == PT_PREC_MIXED) {  // one pass, order-independent fixed-point sums
            for (const void* p : {(const void*)r, (const void*)s, (const void*)Tt, (const void*)E.Ctr})
                if (reinterpret_cast<uintptr_t>(p) % 16)
                    return fail(PT_ERR_ARG, "mixed-precision projection: tracer arrays must be 16-byte aligned");
            unsigned long long* acc = reinterpret_cast<unsigned long long*>(W.cpart);
            CK(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 4 * (size_t)ncell, E.st));
            auto kern = E.K.exact_div ? (E.cfg.comp ? k_project_fx<true, true> : k_project_fx<true, false>)
                                      : (E.cfg.comp ? k_project_fx<false, true> : k_project_fx<false, false>);
            if (W.runs) CK(cudaMemsetAsync(W.runs, 0, sizeof(unsigned long long), E.st));
            {
                KernelTimer kt(E, KT_PROJECT, 1);
                PT_COUNT(), kern<<<nblk(n, kPjChunk), kPjThreads, 0, E.st>>>(r, s, Tt, E.Ctr, n, acc, W.derr,
                                                                             W.runs);
            }
            PT_COUNT(), k_node_fx<<<grid, 128, 0, E.st>>>(acc, E.Tratio, E.Cnew, E.nempty, E.g1, E.cfg.comp);
        } else {  // the reference's association: ascending tracer ID per cell, FP64
            KernelTimer kt(E, KT_PROJECT, 1);
            PT_COUNT(), k_cells<<<nblk(n, 256), 256, 0, E.st>>>(r, s, n, W.tcell, W.ccount, W.derr);
            int nb = (int)nblk(ncell, 1024);
            PT_COUNT(), k_scan_block<<<nb, 1024, 0, E.st>>>(W.ccount, W.cstart, W.scan_tmp, ncell);
            PT_COUNT(), k_scan_totals<<<1, kScanTotThreads, 0, E.st>>>(W.scan_tmp, nb);
            PT_COUNT(), k_scan_add<<<nb, 1024, 0, E.st>>>(W.cstart, W.scan_tmp, ncell);
            int32_t* cursor = W.scan_tmp + nb + 32;
            CK(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)ncell, E.st));
            PT_COUNT(), k_scatter<<<nblk(n, 256), 256, 0, E.st>>>(W.tcell, n, W.cstart, cursor, W.clist);
            PT_COUNT(), k_sort_cells<<<nblk(ncell, 128), 128, 0, E.st>>>(W.clist, W.cstart, W.ccount, ncell);
            const bool og = E.cfg.discrete_types != 0;
            PT_COUNT(), (og ? k_cell_partials<true> : k_cell_partials<false>)<<<nblk(ncell, 128), 128, 0, E.st>>>(
                r, s, Tt, E.Ctr, W.clist, W.cstart, W.ccount, ncell, W.cpart, E.cfg.comp);
            PT_COUNT(), (og ? k_node_sums<true> : k_node_sums<false>)<<<grid, 128, 0, E.st>>>(
                W.cpart, W.ccount, ncell, E.Tratio, E.Cnew, E.nempty, E.g1, E.cfg.comp);
        }
        CKL("projection");
        if (E.cfg.discrete_types && E.count1) {  // count_type(1, :, :) of the same projection
            CK(cudaMemsetAsync(E.count1, 0, sizeof(int32_t) * (size_t)ncell, E.st));
            PT_COUNT(), k_count_type1<<<nblk(n, 256), 256, 0, E.st>>>(r, s, E.Ctr, n, E.count1);
            CKL("k_count_type1");
        }
    }
    int herr = 0;
    unsigned long long hruns = 0;
    CK(cudaMemcpyAsync(&herr, W.derr, sizeof(int), cudaMemcpyDeviceToHost, E.st));
    const bool counted = W.runs && E.cfg.precision == PT_PREC_MIXED;
    if (counted) CK(cudaMemcpyAsync(&hruns, W.runs, sizeof hruns, cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    if (herr & 1) return fail(PT_ERR_TRACER_OUT_OF_DOMAIN, "Tracer advected outside of domain");
    // runs per kPjPer consecutive tracers: from about kPjPer / (tracers per cell) in cell order to
    // kPjPer in a random order; past kResortFrac of the way the tracers are re-sorted by cell
    // before the next step (mixed precision, where the order does not enter any result)
    if (counted) {
        E.last_runs = (double)hruns * (double)kPjPer / (double)E.ntr;
        const double per_cell = (double)E.ntr / ((double)E.K.nx * (double)E.K.nz);
        const double sorted = std::max(1.0, (double)kPjPer / std::max(per_cell, 1.0));
        if (E.last_runs > sorted + kResortFrac * ((double)kPjPer - sorted)) E.want_resort = true;
    }
    if (herr & 2)
        return fail(PT_ERR_CONFIG, "mixed-precision projection: a tracer's T or C is outside (-4, 4) (FP64 precision "
                                   "has no such limit)");
    if (E.cfg.comp) {
        if ((rc = enforce_bcs_C(E, E.Cnew))) return rc;
        if (smooth && (rc = smoother_time_C(E))) return rc;
    }
    if ((rc = enforce_bcs_T(E, E.Tratio))) return rc;
    if (smooth && (rc = smoother_time_T(E, E.Tratio))) return rc;
    return load_conductivity(E);
}

int project(Engine& E, const double* r, const double* s, const double* Tt, const double* T0f, int smooth) {
    ProjScratch W{E.tcell, E.clist, E.ccount, E.cstart, E.scan_tmp, E.cpart, E.derr, E.proj_runs};
    return project_with(E, W, r, s, Tt, T0f, smooth);
}

// ---------------------------------------------------------------- projection without allocation
// Scratch of pt_tracers_to_corners_noalloc: one file-scope device array, carved as
// [partials 27 x nodes doubles | tcell | clist | ccount | cstart | scan | flag], each part
// 256-byte aligned.  Sized for PT_NOALLOC_MAX_TRACERS and PT_NOALLOC_MAX_NODES.
static constexpr size_t na_round(size_t b) { return (b + 255) / 256 * 256; }
static constexpr size_t kNaNodes = PT_NOALLOC_MAX_NODES, kNaTracers = PT_NOALLOC_MAX_TRACERS;
static constexpr size_t kNaScan = kNaNodes + kNaNodes / 1024 + 64;
static constexpr size_t kNaOffPart = 0;
static constexpr size_t kNaOffCell = kNaOffPart + na_round(27 * kNaNodes * sizeof(double));
static constexpr size_t kNaOffList = kNaOffCell + na_round(kNaTracers * sizeof(int32_t));
static constexpr size_t kNaOffCount = kNaOffList + na_round(kNaTracers * sizeof(int32_t));
static constexpr size_t kNaOffStart = kNaOffCount + na_round(kNaNodes * sizeof(int32_t));
static constexpr size_t kNaOffScan = kNaOffStart + na_round(kNaNodes * sizeof(int32_t));
static constexpr size_t kNaOffFlag = kNaOffScan + na_round(kNaScan * sizeof(int32_t));
static constexpr size_t kNaBytes = kNaOffFlag + 256;
static_assert(kNaBytes <= 16u * 1024u * 1024u, "no-alloc projection scratch stays below 16 MB");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];
// per device, from cudaGetSymbolAddress; threads that resolve the same device at once store the
// same address
static std::atomic<unsigned char*> s_noalloc_base[64];

// Resolves (once per device) and returns the scratch address of the current device.  pt_init
// calls it, so the lookup (which may load the module) never happens inside a stream capture.
int noalloc_scratch_setup(unsigned char** base) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(PT_ERR_CUDA, "device index out of range for the no-alloc scratch table");
    unsigned char* b = s_noalloc_base[dev].load(std::memory_order_acquire);
    if (!b) {
        void* p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        b = static_cast<unsigned char*>(p);
        s_noalloc_base[dev].store(b, std::memory_order_release);
    }
    if (base) *base = b;
    return 0;
}

int project_noalloc(Engine& E, const double* T0f, int smooth) {
    const size_t ncell = (size_t)(E.K.nx + 1) * (size_t)(E.K.nz + 1);
    if ((size_t)E.ntr > kNaTracers || ncell > kNaNodes)
        return fail(PT_ERR_ARG, "pt_tracers_to_corners_noalloc: more than " + std::to_string(kNaTracers) +
                                    " tracers or " + std::to_string(kNaNodes) + " grid nodes");
    unsigned char* b = nullptr;
    if (int rc = noalloc_scratch_setup(&b)) return rc;
    ProjScratch W{reinterpret_cast<int32_t*>(b + kNaOffCell), reinterpret_cast<int32_t*>(b + kNaOffList),
                  reinterpret_cast<int32_t*>(b + kNaOffCount), reinterpret_cast<int32_t*>(b + kNaOffStart),
                  reinterpret_cast<int32_t*>(b + kNaOffScan), reinterpret_cast<double*>(b + kNaOffPart),
                  reinterpret_cast<int*>(b + kNaOffFlag), nullptr};
    // project_with clears the counts, the scatter cursors and the flag before use; every other
    // part is fully written before it is read
    return project_with(E, W, E.rtr, E.str, E.Ttr, T0f, smooth);
}

// ---------------------------------------------------------------- tracer locality (mixed precision)
// The mixed path's results do not depend on the order of the tracers (integer projection sums,
// per-tracer RK stages), but its speed does: k_project_fx keeps per-cell runs in registers and the
// RK stage's table gathers hit L1 when neighbouring tracers share cells.  Advection scatters the
// seeding order, so when the projection reports lost locality the tracers are re-sorted by cell
// and sub-cell (counting sort) at the start of the next step.  perm[p] is the user's index of the
// tracer held at position p; tracer fields are exchanged in the user's order (tracer_user_order).

// sort key of each tracer: its cell, column by column (k fastest: the RK stage's 7-row stencils
// then overlap from one warp to the next), times 16 plus its 4x4 sub-cell (row-major), so that
// tracers of one cell stay together and, inside the cell, close tracers stay close.  0 for a
// tracer outside the domain (the projection reports it).  Per-key counts.
constexpr int kSubKeys = 16;
template <bool EXACT>
__global__ void k_tracer_keys(const double* __restrict__ r, const double* __restrict__ s, int64_t n,
                              int32_t* __restrict__ key, int32_t* __restrict__ count) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1;
    if (t < n) {
        TracerCell tc;
        c = 0;
        if (locate<EXACT>(r[t], s[t], tc)) {
            const int sx = min((int)(tc.fx >> 26), 3), sz = min((int)(tc.fz >> 26), 3);
            c = (tc.k0 + (cK.nz + 1) * tc.i0) * kSubKeys + 4 * sz + sx;
        }
        key[t] = c;
    }
    const unsigned group = __match_any_sync(0xffffffffu, c);
    if (c >= 0 && (int)(threadIdx.x & 31) == __ffs(group) - 1) atomicAdd(&count[c], __popc(group));
}

// out_q[p] = in_q[src[p]] for the four tracer arrays, and the user index with them
__global__ void k_permute_tracers(const int32_t* __restrict__ src, int64_t n, const double* __restrict__ a0,
                                  const double* __restrict__ a1, const double* __restrict__ a2,
                                  const double* __restrict__ a3, double* __restrict__ b0, double* __restrict__ b1,
                                  double* __restrict__ b2, double* __restrict__ b3, const int32_t* __restrict__ pin,
                                  int32_t* __restrict__ pout) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t t = src[p];
    b0[p] = a0[t]; b1[p] = a1[t]; b2[p] = a2[t]; b3[p] = a3[t];
    pout[p] = pin[t];
}

__global__ void k_iota(int32_t* p, int64_t n) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) p[q] = (int32_t)q;
}

int tracer_order_reset(Engine& E) {
    E.perm_active = false;
    E.want_resort = false;
    E.resorts = 0;
    if (!E.perm) return 0;
    PT_COUNT(), k_iota<<<nblk(E.ntr, 256), 256, 0, E.st>>>(E.perm, E.ntr);
    CKL("k_iota");
    return 0;
}

// counting sort of the tracers by key; the four tracer arrays and perm move together (into the
// RK stage buffers, then the pointers swap)
int resort_tracers(Engine& E) {
    E.want_resort = false;
    if (!E.perm || !E.rs_count) return 0;
    const int nkey = (int)resort_nkey(E.K.nx, E.K.nz);
    const int64_t n = E.ntr;
    CK(cudaMemsetAsync(E.rs_count, 0, sizeof(int32_t) * (size_t)nkey, E.st));
    auto kk = E.K.exact_div ? k_tracer_keys<true> : k_tracer_keys<false>;
    PT_COUNT(), kk<<<nblk(n, 256), 256, 0, E.st>>>(E.rtr, E.str, n, E.tcell, E.rs_count);
    const int nb = (int)nblk(nkey, 1024);
    PT_COUNT(), k_scan_block<<<nb, 1024, 0, E.st>>>(E.rs_count, E.rs_start, E.rs_tot, nkey);
    PT_COUNT(), k_scan_totals<<<1, kScanTotThreads, 0, E.st>>>(E.rs_tot, nb);
    PT_COUNT(), k_scan_add<<<nb, 1024, 0, E.st>>>(E.rs_start, E.rs_tot, nkey);
    CK(cudaMemsetAsync(E.rs_count, 0, sizeof(int32_t) * (size_t)nkey, E.st));  // now the cursors
    PT_COUNT(), k_scatter<<<nblk(n, 256), 256, 0, E.st>>>(E.tcell, n, E.rs_start, E.rs_count, E.clist);
    PT_COUNT(), k_permute_tracers<<<nblk(n, 256), 256, 0, E.st>>>(E.clist, n, E.rtr, E.str, E.Ttr, E.Ctr, E.rtr1,
                                                                   E.str1, E.Ttr1, E.rtr2, E.perm, E.perm2);
    CKL("resort_tracers");
    std::swap(E.rtr, E.rtr1);
    std::swap(E.str, E.str1);
    std::swap(E.Ttr, E.Ttr1);
    std::swap(E.Ctr, E.rtr2);
    std::swap(E.perm, E.perm2);
    E.perm_active = true;
    E.resorts++;
    return 0;
}

// user-order exchange of one tracer array: to_user: user[perm[p]] = in[p]; else in[p] = user[perm[p]]
__global__ void k_perm_scatter(const int32_t* __restrict__ perm, const double* __restrict__ in, double* __restrict__ out,
                               int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) out[perm[p]] = in[p];
}
__global__ void k_perm_gather(const int32_t* __restrict__ perm, const double* __restrict__ in, double* __restrict__ out,
                              int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) out[p] = in[perm[p]];
}
int tracer_user_order(Engine& E, double* internal, double* staging, bool to_user) {
    if (to_user) PT_COUNT(), k_perm_scatter<<<nblk(E.ntr, 256), 256, 0, E.st>>>(E.perm, internal, staging, E.ntr);
    else PT_COUNT(), k_perm_gather<<<nblk(E.ntr, 256), 256, 0, E.st>>>(E.perm, staging, internal, E.ntr);
    CKL("tracer_user_order");
    return 0;
}

// ---------------------------------------------------------------- RK4 stage loops
// interpolate (composition.f90:1359-1393): x-Taylor series (order 3) on the 7 rows around the
// nearest node, z-derivatives of those values with the 7-point stencils, z-Taylor series.
struct Tables {
    const double *f, *d1, *d2, *d3;
};

__device__ __forceinline__ double interp(const Tables& tb, Geo g, int i, int k, double a1, double a2,
                                         double a3, double b1, double b2, double b3) {
    double fR[7];
#pragma unroll
    for (int jj = 0; jj < 7; jj++) {
        size_t o = g.at(i, k + jj - 3);
        double v = tb.f[o];
        v = v + tb.d1[o] * a1;
        v = v + tb.d2[o] * a2;
        v = v + tb.d3[o] * a3;
        fR[jj] = v;
    }
    double s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        s1 = s1 + cK.Dm[1][j] * fR[j];
        s2 = s2 + cK.Dm[2][j] * fR[j];
        s3 = s3 + cK.Dm[3][j] * fR[j];
    }
    // reciprocal multiplies: this part issues about two FP64 operations per clock per SM and a
    // division costs many; with power-of-two spacings the reciprocals are exact
    s1 = s1 * cK.inv_ds_pow[1];
    s2 = s2 * cK.inv_ds_pow[2];
    s3 = s3 * cK.inv_ds_pow[3];
    double fi = fR[3];
    fi = fi + s1 * b1;
    fi = fi + s2 * b2;
    fi = fi + s3 * b3;
    return fi;
}

struct StageArgs {
    Tables u, w, t;
    const double *xr, *xs;      // interpolation positions
    double *rtr, *str, *Ttr;    // accumulators k1 + 2k2 + 2k3 (+k4)
    const double *r0, *s0, *T0; // step-start state
    double *rn, *sn, *Tn;       // next stage position/temperature
    double dtstage;
    int stage;
    int64_t n;
};

__global__ void __launch_bounds__(256) k_rk_stage(StageArgs A, Geo g) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.n) return;
    double r = A.xr[t], s = A.xs[t];
    int i = cell_index(r, cK.inv_dr, cK.dr, cK.exact_div, cK.p_inv_dr);
    int k = cell_index(s, cK.inv_ds, cK.ds, cK.exact_div, cK.p_inv_ds);
    i = min(max(i, 0), cK.nx);  // positions were validated by the projection; clamp keeps reads in bounds
    k = min(max(k, 0), cK.nz);
    double hr = r - (double)i * cK.dr, hs = s - (double)k * cK.ds;
    double a1 = hr * cK.inv_fact[1], a2 = hr * hr * cK.inv_fact[2], a3 = hr * hr * hr * cK.inv_fact[3];
    double b1 = hs * cK.inv_fact[1], b2 = hs * hs * cK.inv_fact[2], b3 = hs * hs * hs * cK.inv_fact[3];
    double tr = interp(A.u, g, i, k, a1, a2, a3, b1, b2, b3);
    double ts = interp(A.w, g, i, k, a1, a2, a3, b1, b2, b3);
    double tT = interp(A.t, g, i, k, a1, a2, a3, b1, b2, b3);
    double r0 = A.r0[t], s0 = A.s0[t], T0 = A.T0[t];
    switch (A.stage) {
        case 1:  // energy.f90:288-299
            A.rtr[t] = tr; A.str[t] = ts; A.Ttr[t] = tT;
            A.rn[t] = r0 + A.dtstage * tr; A.sn[t] = s0 + A.dtstage * ts; A.Tn[t] = T0 + A.dtstage * tT;
            break;
        case 2:  // energy.f90:376-399
        case 3:  // energy.f90:458-470
            A.rtr[t] = A.rtr[t] + 2.0 * tr; A.str[t] = A.str[t] + 2.0 * ts; A.Ttr[t] = A.Ttr[t] + 2.0 * tT;
            A.rn[t] = r0 + A.dtstage * tr; A.sn[t] = s0 + A.dtstage * ts; A.Tn[t] = T0 + A.dtstage * tT;
            break;
        default:  // stage 4, energy.f90:525-534
            A.rtr[t] = r0 + A.dtstage * (A.rtr[t] + tr);
            A.str[t] = s0 + A.dtstage * (A.str[t] + ts);
            A.Ttr[t] = T0 + A.dtstage * (A.Ttr[t] + tT);
            break;
    }
}

// One stage of the RKC2 energy stepper (Chebyshev.f90:151-227), FP64 interpolation as in
// k_rk_stage.  Stage 1 at the step-start position x0: keeps the slopes k0, x1 = x0 + mewt_1 dt k,
// x2 = x0.  Stage j at x1: x = c_j x0 + mew_j x1 + v_j x2 + mewt_j dt k + gt_j dt k0, then x2 = x1,
// x1 = x (the last stage's x is the step's result).
struct Rkc2Args {
    Tables u, w, t;
    const double *r0, *s0, *T0;      // step start
    double *r1, *s1, *T1, *r2, *s2, *T2;
    double *r, *s, *T;               // this stage's result
    double *kr, *ks, *kT;            // stage-1 slopes
    double c, mew, v, dtst, dtst2;
    int stage;
    int64_t n;
};
__global__ void __launch_bounds__(256) k_rkc2_stage(Rkc2Args A, Geo g) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.n) return;
    const double r = A.stage == 1 ? A.r0[t] : A.r1[t], s = A.stage == 1 ? A.s0[t] : A.s1[t];
    int i = cell_index(r, cK.inv_dr, cK.dr, cK.exact_div, cK.p_inv_dr);
    int k = cell_index(s, cK.inv_ds, cK.ds, cK.exact_div, cK.p_inv_ds);
    i = min(max(i, 0), cK.nx);  // positions were validated by the projection; clamp keeps reads in bounds
    k = min(max(k, 0), cK.nz);
    const double hr = r - (double)i * cK.dr, hs = s - (double)k * cK.ds;
    const double a1 = hr * cK.inv_fact[1], a2 = hr * hr * cK.inv_fact[2], a3 = hr * hr * hr * cK.inv_fact[3];
    const double b1 = hs * cK.inv_fact[1], b2 = hs * hs * cK.inv_fact[2], b3 = hs * hs * hs * cK.inv_fact[3];
    const double tr = interp(A.u, g, i, k, a1, a2, a3, b1, b2, b3);
    const double ts = interp(A.w, g, i, k, a1, a2, a3, b1, b2, b3);
    const double tT = interp(A.t, g, i, k, a1, a2, a3, b1, b2, b3);
    const double r0 = A.r0[t], s0 = A.s0[t], T0 = A.T0[t];
    if (A.stage == 1) {
        A.kr[t] = tr; A.ks[t] = ts; A.kT[t] = tT;
        A.r1[t] = r0 + A.dtst * tr; A.s1[t] = s0 + A.dtst * ts; A.T1[t] = T0 + A.dtst * tT;
        A.r2[t] = r0; A.s2[t] = s0; A.T2[t] = T0;
        return;
    }
    const double r1 = A.r1[t], s1 = A.s1[t], T1 = A.T1[t];
    const double x = A.c * r0 + A.mew * r1 + A.v * A.r2[t] + A.dtst * tr + A.dtst2 * A.kr[t];
    const double z = A.c * s0 + A.mew * s1 + A.v * A.s2[t] + A.dtst * ts + A.dtst2 * A.ks[t];
    const double y = A.c * T0 + A.mew * T1 + A.v * A.T2[t] + A.dtst * tT + A.dtst2 * A.kT[t];
    A.r[t] = x; A.s[t] = z; A.T[t] = y;
    A.r2[t] = r1; A.s2[t] = s1; A.T2[t] = T1;
    A.r1[t] = x; A.s1[t] = z; A.T1[t] = y;
}

// ---------------------------------------------------------------- mixed-precision stage
// The same stage with the Taylor interpolation in FP32 from FP32 copies of the velocity and
// dT/dt tables: positions, step-start values and the RK accumulators stay FP64.  Interpolated
// velocities carry a relative error of order 1e-7, below the psi solve's tolerance; the FP64
// stage (k_rk_stage) is the reference-order path.
// one 16-byte load per table row: (value, x-derivatives of order 1..3) interleaved per node
__device__ __forceinline__ float interp_f(const float4* __restrict__ tb, Geo g, int i, int k, float a1, float a2,
                                          float a3, float b1, float b2, float b3) {
    float fR[7];
#pragma unroll
    for (int jj = 0; jj < 7; jj++) {
        const float4 q = __ldg(tb + g.at(i, k + jj - 3));
        fR[jj] = q.x + q.y * a1 + q.z * a2 + q.w * a3;
    }
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        s1 += cDmf[1][j] * fR[j];
        s2 += cDmf[2][j] * fR[j];
        s3 += cDmf[3][j] * fR[j];
    }
    return fR[3] + s1 * b1 + s2 * b2 + s3 * b3;
}

struct StageArgsF {
    const float4 *u, *w, *t;
    const double *xr, *xs;
    double *rtr, *str, *Ttr;  // the step's result (stage 4)
    float *ar, *as, *aT;      // FP32 sums of the RK slopes, k1 + 2 k2 + 2 k3 (stages 1-3)
    const double *r0, *s0, *T0;
    double *rn, *sn, *Tn;
    double dtstage;
    float dtf;  // dtstage in FP32
    int stage;
    int64_t n;
};

// nearest node of x (spacing 2^-p, x >= 0) and the offset x - i h as a multiple of h 2^-28, from
// the bit pattern (floor_fix_pow2): no FP64 arithmetic
__device__ __forceinline__ int nearest_off_pow2(double x, int p, int& off28) {
    uint32_t f;
    const int fl = floor_fix_pow2(x, p, f);
    if (f >= (1u << 27)) {
        off28 = (int)f - (1 << 28);
        return fl + 1;
    }
    off28 = (int)f;
    return fl;
}

// The slopes (dr/dt, ds/dt, dT/dt) of energy.f90:258-536 at (r, s) by FP32 interpolation: the cell
// and the offsets come from the position's bit pattern.
__device__ __forceinline__ void rk_slopes(const StageArgsF& A, Geo g, double r, double s, float& tr, float& ts,
                                          float& tT) {
    int i, k;
    float hr, hs;
    if (cK.exact_div) {
        int qr, qs;
        i = nearest_off_pow2(r, cK.p_inv_dr, qr);
        k = nearest_off_pow2(s, cK.p_inv_ds, qs);
        hr = (float)qr * cH28[0];
        hs = (float)qs * cH28[1];
    } else {
        i = cell_index(r, cK.inv_dr, cK.dr, 0, 0);
        k = cell_index(s, cK.inv_ds, cK.ds, 0, 0);
        hr = (float)(r - (double)i * cK.dr);
        hs = (float)(s - (double)k * cK.ds);
    }
    if (i < 0 || i > cK.nx || k < 0 || k > cK.nz) {  // validated by the projection; keep reads in bounds
        i = min(max(i, 0), cK.nx);
        k = min(max(k, 0), cK.nz);
        hr = (float)(r - (double)i * cK.dr);
        hs = (float)(s - (double)k * cK.ds);
    }
    const float a1 = hr, a2 = 0.5f * hr * hr, a3 = hr * hr * hr * (1.0f / 6.0f);
    const float b1 = hs, b2 = 0.5f * hs * hs, b3 = hs * hs * hs * (1.0f / 6.0f);
    tr = interp_f(A.u, g, i, k, a1, a2, a3, b1, b2, b3);
    ts = interp_f(A.w, g, i, k, a1, a2, a3, b1, b2, b3);
    tT = interp_f(A.t, g, i, k, a1, a2, a3, b1, b2, b3);
}

// One RK4 stage (energy.f90:258-536) with FP32 interpolation and FP32 slope sums; only the
// position/value updates (FP64 state + an FP32 increment) use the FP64 pipe.  Every load that does
// not depend on the position (step-start values, slope sums) is issued before the table gathers,
// so that its latency overlaps theirs.
__global__ void __launch_bounds__(256) k_rk_stage_f(StageArgsF A, Geo g) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.n) return;
    const double r = A.xr[t], s = A.xs[t];
    const double r0 = A.r0[t], s0 = A.s0[t], T0 = A.T0[t];
    float pr = 0.f, ps = 0.f, pT = 0.f;
    if (A.stage > 1) { pr = A.ar[t]; ps = A.as[t]; pT = A.aT[t]; }
    float tr, ts, tT;
    rk_slopes(A, g, r, s, tr, ts, tT);
    switch (A.stage) {
        case 1:
            A.ar[t] = tr; A.as[t] = ts; A.aT[t] = tT;
            A.rn[t] = r0 + (double)(A.dtf * tr); A.sn[t] = s0 + (double)(A.dtf * ts); A.Tn[t] = T0 + (double)(A.dtf * tT);
            break;
        case 2:
        case 3:
            A.ar[t] = pr + 2.0f * tr; A.as[t] = ps + 2.0f * ts; A.aT[t] = pT + 2.0f * tT;
            A.rn[t] = r0 + (double)(A.dtf * tr); A.sn[t] = s0 + (double)(A.dtf * ts); A.Tn[t] = T0 + (double)(A.dtf * tT);
            break;
        default:
            A.rtr[t] = r0 + (double)(A.dtf * (pr + tr));
            A.str[t] = s0 + (double)(A.dtf * (ps + ts));
            A.Ttr[t] = T0 + (double)(A.dtf * (pT + tT));
            break;
    }
}

// FP32 copy of one interpolation table set, interleaved per node (value, x-derivatives 1..3)
__global__ void k_tables_to_f32(float4* out, const double* F, const double* D1, const double* D2, const double* D3,
                                size_t n) {
    size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    out[q] = make_float4((float)F[q], (float)D1[q], (float)D2[q], (float)D3[q]);
}

// ---- the same table from exact integer stencil sums (mixed path)
// The x-derivative stencils are small rationals (D1 = [1,-8,0,8,-1]/12, D2 = [-1,16,-30,16,-1]/12,
// D3 = [1,-8,13,0,-13,8,-1]/8, checked on the host), so with a row segment of f in fixed point
// (X = round(f 2^s), |X| < 2^62 from the segment's largest exponent, split as Xh 2^31 + Xl) each
// derivative is an exact integer sum; only its conversion to FP32 rounds.  The conversions are
// integer operations, so the table costs no FP64 arithmetic (the FP64 path's k_derivs takes 45
// FP64 operations per node and its FP32 copy four more).
constexpr int kTbX = 128;

// v 2^e2 as a double from integer operations: the leading 53 bits of |v| (truncated; the callers'
// sums already carry 2^-54 of their scale), 0 below the normal range
__device__ __forceinline__ double i64_to_double_trunc(long long v, int e2) {
    if (v == 0) return 0.0;
    const unsigned long long sgn = (unsigned long long)v & 0x8000000000000000ull;
    const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    const int lz = __clzll(a);
    const unsigned long long mant = (a << lz) >> 11;  // leading one at bit 52
    const long long ex = (long long)(1023 + 63 - lz + e2);
    if (ex <= 0) return 0.0;
    return __longlong_as_double((long long)(sgn | ((unsigned long long)ex << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// v 2^e2 rounded to FP32 (to nearest, ties away from zero; below the normal range: 0)
__device__ __forceinline__ float i64_to_float_scaled(long long v, int e2) {
    if (v == 0) return 0.f;
    const unsigned sgn = v < 0 ? 0x80000000u : 0u;
    unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    const int lz = __clzll(a);
    a <<= lz;                                             // leading one at bit 63
    unsigned long long m = (a >> 39) + 1;                 // 25 bits, rounding bit added
    int ex = 127 + 63 - lz + e2;
    if (m >> 25) { m >>= 1; ex++; }                       // the rounding carried into bit 25
    m >>= 1;                                              // 24 bits, leading one at bit 23
    if (ex <= 0) return 0.f;
    if (ex >= 255) return __uint_as_float(sgn | 0x7F800000u);
    return __uint_as_float(sgn | ((unsigned)ex << 23) | ((unsigned)m & 0x7FFFFFu));
}
// FP64 to FP32 from the bit pattern (to nearest, ties to even, as the conversion instruction;
// FP32-subnormal results: 0)
__device__ __forceinline__ float d2f_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0x7FF) return __uint_as_float(sgn | 0x7F800000u | (unsigned)((b & 0xFFFFFFFFFFFFFull) != 0) << 22);
    unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    m += (1ull << 28) - 1 + ((m >> 29) & 1);  // round at bit 29, ties to the even result
    int ex = e - 1023 + 127;
    if (m >> 53) { m >>= 1; ex++; }
    if (e == 0 || ex <= 0) return __uint_as_float(sgn);
    if (ex >= 255) return __uint_as_float(sgn | 0x7F800000u);
    return __uint_as_float(sgn | ((unsigned)ex << 23) | ((unsigned)(m >> 29) & 0x7FFFFFu));
}

// one CTA per kTbX nodes of a row k in [-3, nz+3]; nodes i in [0, nx]
__global__ void __launch_bounds__(kTbX) k_tables_fx(float4* __restrict__ out, const double* __restrict__ f, Geo g,
                                                    float c1, float c2, float c3) {
    __shared__ int2 X[kTbX + 6];
    __shared__ int emax_s;
    const int nx = cK.nx;
    const int i0 = blockIdx.x * kTbX, k = (int)blockIdx.y - 3;
    if (threadIdx.x == 0) emax_s = 0;
    __syncthreads();
    unsigned long long raw[2];
    int em = 0;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int idx = threadIdx.x + kTbX * q;
        unsigned long long b = 0;
        if (idx < kTbX + 6) {
            const int i = i0 - 3 + idx;
            if (i <= nx + 3) b = (unsigned long long)__double_as_longlong(f[g.at(i, k)]);
        }
        raw[q] = b;
        em = max(em, (int)((b >> 52) & 0x7FF));
    }
    em = __reduce_max_sync(0xffffffffu, em);
    if ((threadIdx.x & 31) == 0) atomicMax(&emax_s, em);
    __syncthreads();
    const int emax = emax_s;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int idx = threadIdx.x + kTbX * q;
        if (idx >= kTbX + 6) break;
        const unsigned long long b = raw[q];
        const int e = (int)((b >> 52) & 0x7FF);
        long long v = 0;
        if (e != 0 && emax != 0x7FF) {
            const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
            const int sh = emax - 9 - e;  // X = m 2^-sh, |X| < 2^62
            unsigned long long a;
            if (sh <= 0) a = m << (-sh);
            else if (sh < 64) a = (m + (1ull << (sh - 1))) >> sh;
            else a = 0;
            v = (b >> 63) ? -(long long)a : (long long)a;
        }
        const long long h = v >> 31;  // floor
        X[idx] = make_int2((int)h, (int)(v - (h << 31)));
    }
    __syncthreads();
    const int i = i0 + (int)threadIdx.x;
    if (i > nx) return;
    const double fv = f[g.at(i, k)];
    if (emax == 0x7FF) {  // Inf/NaN in the segment: NaN derivatives, as the FP64 stencil gives
        const float nan = __uint_as_float(0x7FC00000u);
        out[g.at(i, k)] = make_float4(d2f_bits(fv), nan, nan, nan);
        return;
    }
    constexpr int w1[7] = {0, 1, -8, 0, 8, -1, 0}, w2[7] = {0, -1, 16, -30, 16, -1, 0},
                  w3[7] = {1, -8, 13, 0, -13, 8, -1};
    long long h1 = 0, l1 = 0, h2 = 0, l2 = 0, h3 = 0, l3 = 0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        const int2 x = X[threadIdx.x + j];
        if (w1[j]) { h1 += (long long)w1[j] * x.x; l1 += (long long)w1[j] * x.y; }
        if (w2[j]) { h2 += (long long)w2[j] * x.x; l2 += (long long)w2[j] * x.y; }
        if (w3[j]) { h3 += (long long)w3[j] * x.x; l3 += (long long)w3[j] * x.y; }
    }
    // sum = (h 2^31 + l) 2^-s with s = 1084 - emax; h 2^23 + (l >> 8) keeps 2^-54 of the
    // segment's scale and fits 64 bits
    const int e2 = 8 - (1084 - emax);
    const float d1 = i64_to_float_scaled((h1 << 23) + (l1 >> 8), e2) * c1;
    const float d2 = i64_to_float_scaled((h2 << 23) + (l2 >> 8), e2) * c2;
    const float d3 = i64_to_float_scaled((h3 << 23) + (l3 >> 8), e2) * c3;
    out[g.at(i, k)] = make_float4(d2f_bits(fv), d1, d2, d3);
}

// load_tracer_space (energy.f90:59-179) for the mixed path: Tx, Tz, Txx, Tzz of Text as exact
// integer sums (D1 = [1,-8,0,8,-1]/12, D2 = [-1,16,-30,16,-1]/12) on a tile in 62-bit fixed point,
// so that only the combination with the conductivity fields is FP64 arithmetic (about 10
// operations per node instead of about 50).  Nodes i in [-3, nx+3], k in [-3, nz+3].
constexpr int kTsX = 32, kTsZ = 8, kTsW = kTsX + 4, kTsH = kTsZ + 4;
__global__ void __launch_bounds__(kTsX * kTsZ) k_tracer_space_fx(double* __restrict__ tsa, const double* __restrict__ X,
                                                                 const double* __restrict__ cd,
                                                                 const double* __restrict__ cr,
                                                                 const double* __restrict__ cs,
                                                                 const double* __restrict__ Cvis, Geo g, double sx,
                                                                 double sxx, double sz, double szz) {
    __shared__ int2 Xf[kTsH][kTsW];
    __shared__ int emax_s;
    const int nx = cK.nx, nz = cK.nz;
    const int tid = threadIdx.y * kTsX + threadIdx.x;
    const int i0 = -3 + (int)blockIdx.x * kTsX, k0 = -3 + (int)blockIdx.y * kTsZ;
    if (tid == 0) emax_s = 0;
    __syncthreads();
    constexpr int NT = kTsW * kTsH, PER = (NT + kTsX * kTsZ - 1) / (kTsX * kTsZ);
    unsigned long long raw[PER];
    int em = 0;
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int idx = tid + kTsX * kTsZ * q;
        unsigned long long b = 0;
        if (idx < NT) {
            const int i = i0 - 2 + idx % kTsW, k = k0 - 2 + idx / kTsW;  // i, k >= -5
            if (i <= nx + 5 && k <= nz + 5) b = (unsigned long long)__double_as_longlong(X[g.at(i, k)]);
        }
        raw[q] = b;
        em = max(em, (int)((b >> 52) & 0x7FF));
    }
    em = __reduce_max_sync(0xffffffffu, em);
    if ((tid & 31) == 0) atomicMax(&emax_s, em);
    __syncthreads();
    const int emax = emax_s;
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int idx = tid + kTsX * kTsZ * q;
        if (idx >= NT) break;
        const unsigned long long b = raw[q];
        const int e = (int)((b >> 52) & 0x7FF);
        long long v = 0;
        if (e != 0 && emax != 0x7FF) {
            const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
            const int sh = emax - 9 - e;  // X = m 2^-sh, |X| < 2^62
            unsigned long long a;
            if (sh <= 0) a = m << (-sh);
            else if (sh < 64) a = (m + (1ull << (sh - 1))) >> sh;
            else a = 0;
            v = (b >> 63) ? -(long long)a : (long long)a;
        }
        const long long h = v >> 31;
        Xf[idx / kTsW][idx % kTsW] = make_int2((int)h, (int)(v - (h << 31)));
    }
    __syncthreads();
    const int i = i0 + (int)threadIdx.x, k = k0 + (int)threadIdx.y;
    if (i > nx + 3 || k > nz + 3) return;
    const size_t o = g.at(i, k);
    double Tx, Tz, Txx, Tzz;
    if (emax == 0x7FF) {
        Tx = Tz = Txx = Tzz = __longlong_as_double(0x7FF8000000000000ll);
    } else {
        constexpr int w1[5] = {1, -8, 0, 8, -1}, w2[5] = {-1, 16, -30, 16, -1};
        long long h1 = 0, l1 = 0, h2 = 0, l2 = 0, h3 = 0, l3 = 0, h4 = 0, l4 = 0;
        const int cx = threadIdx.x + 2, cz = threadIdx.y + 2;
#pragma unroll
        for (int j = 0; j < 5; j++) {
            const int2 ax = Xf[cz][cx + j - 2], az = Xf[cz + j - 2][cx];
            if (w1[j]) {
                h1 += (long long)w1[j] * ax.x; l1 += (long long)w1[j] * ax.y;
                h3 += (long long)w1[j] * az.x; l3 += (long long)w1[j] * az.y;
            }
            h2 += (long long)w2[j] * ax.x; l2 += (long long)w2[j] * ax.y;
            h4 += (long long)w2[j] * az.x; l4 += (long long)w2[j] * az.y;
        }
        // (h 2^31 + l) 2^-s, s = 1084 - emax, as h 2^23 + (l >> 8) at 2^(8-s) (|.| < 2^60)
        const int e2 = 8 - (1084 - emax);
        Tx = i64_to_double_trunc((h1 << 23) + (l1 >> 8), e2) * sx;
        Txx = i64_to_double_trunc((h2 << 23) + (l2 >> 8), e2) * sxx;
        Tz = i64_to_double_trunc((h3 << 23) + (l3 >> 8), e2) * sz;
        Tzz = i64_to_double_trunc((h4 << 23) + (l4 >> 8), e2) * szz;
    }
    double h = cK.H;  // compute_heating, energy.f90:19-40 (iheattype=0)
    if (cK.comp != 0) {
        const double cv = Cvis[o];
        h = cK.Htype * cv + cK.H * (1.0 - cv);
    }
    tsa[o] = cd[o] * (Txx + Tzz) + (cr[o] * Tx + cs[o] * Tz) + h;
}

int tracer_space_fx(Engine& E) {
    if (int rc = extend_T(E)) return rc;
    const Consts& K = E.K;
    dim3 grid(nblk(K.nx + 7, kTsX), nblk(K.nz + 7, kTsZ)), block(kTsX, kTsZ);
    PT_COUNT(), k_tracer_space_fx<<<grid, block, 0, E.st>>>(E.tsa, E.Text, E.cond, E.cond_r, E.cond_s, E.Cvis, E.g1,
                                                            1.0 / (12.0 * K.dr), 1.0 / (12.0 * K.dr2),
                                                            1.0 / (12.0 * K.ds), 1.0 / (12.0 * K.ds2));
    CKL("k_tracer_space_fx");
    return 0;
}

// the integer stencils above are the run's derivative stencils (checked on the host at every
// call: 35 comparisons)
static bool tables_exact_ok(const Consts& K) {
    const int w[4][7] = {{}, {0, 1, -8, 0, 8, -1, 0}, {0, -1, 16, -30, 16, -1, 0}, {1, -8, 13, 0, -13, 8, -1}};
    const double den[4] = {1.0, 12.0, 12.0, 8.0};
    for (int m = 1; m <= 3; m++)
        for (int j = 0; j < 7; j++)
            if (std::fabs(K.Dm[m][j] * den[m] - w[m][j]) > 1e-12) return false;
    // the first and second derivatives of the tracer-space term (k_tracer_space_fx)
    for (int j = 0; j < 7; j++)
        if (std::fabs(12.0 * K.D1[j] - w[1][j]) > 1e-12 || std::fabs(12.0 * K.D2[j] - w[2][j]) > 1e-12) return false;
    return true;
}

int tables_fx(Engine& E, int which, const double* f) {
    const Consts& K = E.K;
    const float c1 = (float)(1.0 / (12.0 * K.dr_pow[1])), c2 = (float)(1.0 / (12.0 * K.dr_pow[2])),
                c3 = (float)(1.0 / (8.0 * K.dr_pow[3]));
    dim3 grid(nblk(K.nx + 1, kTbX), K.nz + 7);
    PT_COUNT(), k_tables_fx<<<grid, kTbX, 0, E.st>>>(E.ftab[which], f, E.g1, c1, c2, c3);
    CKL("k_tables_fx");
    return 0;
}

bool use_tables_fx(const Engine& E) { return E.ftab[0] != nullptr && tables_exact_ok(E.K); }

int tables_to_f32(Engine& E, int which, const double* f) {
    if (!E.ftab[which]) return 0;
    const size_t n = E.g1.elems();
    PT_COUNT(), k_tables_to_f32<<<nblk(n, 256), 256, 0, E.st>>>(E.ftab[which], f, E.der[which][0], E.der[which][1],
                                                                E.der[which][2], n);
    CKL("k_tables_to_f32");
    return 0;
}

int rkc2_stage(Engine& E, int stage) {
    PhaseTimer tm(E, PH_RK);
    Rkc2Args A;
    A.u = {E.u, E.der[0][0], E.der[0][1], E.der[0][2]};
    A.w = {E.w, E.der[1][0], E.der[1][1], E.der[1][2]};
    A.t = {E.tsa, E.der[2][0], E.der[2][1], E.der[2][2]};
    A.r0 = E.rtr0; A.s0 = E.str0; A.T0 = E.Ttr0;
    A.r1 = E.rtr1; A.s1 = E.str1; A.T1 = E.Ttr1;
    A.r2 = E.rtr2; A.s2 = E.str2; A.T2 = E.Ttr2;
    A.r = E.rtr; A.s = E.str; A.T = E.Ttr;
    A.kr = E.k0r; A.ks = E.k0s; A.kT = E.k0T;
    A.stage = stage;
    A.n = E.ntr;
    A.c = stage > 1 ? E.cCheb[stage] : 0.0;
    A.mew = stage > 1 ? E.mewCheb[stage] : 0.0;
    A.v = stage > 1 ? E.vCheb[stage] : 0.0;
    A.dtst = E.mewtCheb[stage] * E.dt;
    A.dtst2 = stage > 1 ? E.gtCheb[stage] * E.dt : 0.0;
    KernelTimer kt(E, KT_RK_STAGE, 1);
    PT_COUNT(), k_rkc2_stage<<<nblk(E.ntr, 256), 256, 0, E.st>>>(A, E.g1);
    CKL("k_rkc2_stage");
    return 0;
}

int rk_stage(Engine& E, int stage) {
    PhaseTimer tm(E, PH_RK);
    StageArgs A;
    A.u = {E.u, E.der[0][0], E.der[0][1], E.der[0][2]};
    A.w = {E.w, E.der[1][0], E.der[1][1], E.der[1][2]};
    A.t = {E.tsa, E.der[2][0], E.der[2][1], E.der[2][2]};
    A.rtr = E.rtr; A.str = E.str; A.Ttr = E.Ttr;
    A.r0 = E.rtr0; A.s0 = E.str0; A.T0 = E.Ttr0;
    A.n = E.ntr;
    A.stage = stage;
    switch (stage) {
        case 1: A.xr = E.rtr0; A.xs = E.str0; A.rn = E.rtr1; A.sn = E.str1; A.Tn = E.Ttr1; A.dtstage = 0.5 * E.dt; break;
        case 2: A.xr = E.rtr1; A.xs = E.str1; A.rn = E.rtr2; A.sn = E.str2; A.Tn = E.Ttr2; A.dtstage = 0.5 * E.dt; break;
        case 3: A.xr = E.rtr2; A.xs = E.str2; A.rn = E.rtr1; A.sn = E.str1; A.Tn = E.Ttr1; A.dtstage = E.dt; break;
        default: A.xr = E.rtr1; A.xs = E.str1; A.rn = nullptr; A.sn = nullptr; A.Tn = nullptr; A.dtstage = E.dt / 6.0; break;
    }
    if (E.ftab[0]) {  // mixed precision: FP32 interpolation
        StageArgsF F{E.ftab[0], E.ftab[1], E.ftab[2], A.xr, A.xs, A.rtr, A.str, A.Ttr, E.facc[0], E.facc[1], E.facc[2],
                     A.r0, A.s0, A.T0, A.rn, A.sn, A.Tn, A.dtstage, (float)A.dtstage, A.stage, A.n};
        KernelTimer kt(E, KT_RK_STAGE, 1);
        PT_COUNT(), k_rk_stage_f<<<nblk(E.ntr, 256), 256, 0, E.st>>>(F, E.g1);
    } else {
        KernelTimer kt(E, KT_RK_STAGE, 1);
        PT_COUNT(), k_rk_stage<<<nblk(E.ntr, 256), 256, 0, E.st>>>(A, E.g1);
    }
    CKL("k_rk_stage");
    return 0;
}

// ---------------------------------------------------------------- helpers of the tracer equalisation
// Tracers grouped by their nearest node (the reference's nint cell): tcell, ccount (= nempty),
// cstart (exclusive scan) and clist (tracer positions per node).  Out-of-domain tracers fail.
int sort_tracers_by_node(Engine& E, const double* r, const double* s) {
    const int ncell = (E.K.nx + 1) * (E.K.nz + 1);
    const int64_t n = E.ntr;
    CK(cudaMemsetAsync(E.ccount, 0, sizeof(int32_t) * (size_t)ncell, E.st));
    CK(cudaMemsetAsync(E.derr, 0, sizeof(int), E.st));
    PT_COUNT(), k_cells<<<nblk(n, 256), 256, 0, E.st>>>(r, s, n, E.tcell, E.ccount, E.derr);
    if (int rc = exclusive_scan_i32(E, E.ccount, E.cstart, ncell)) return rc;
    const int nb = (int)nblk(ncell, 1024);
    int32_t* cursor = E.scan_tmp + nb + 32;
    CK(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)ncell, E.st));
    PT_COUNT(), k_scatter<<<nblk(n, 256), 256, 0, E.st>>>(E.tcell, n, E.cstart, cursor, E.clist);
    CKL("sort_tracers_by_node");
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, E.derr, sizeof(int), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    if (herr & 1) return fail(PT_ERR_TRACER_OUT_OF_DOMAIN, "Tracer advected outside of domain");
    return 0;
}

// exclusive scan of n <= (nx+1)(nz+1) int32 values (block totals in E.scan_tmp)
int exclusive_scan_i32(Engine& E, const int32_t* in, int32_t* out, int n) {
    const int nb = (int)nblk(n, 1024);
    PT_COUNT(), k_scan_block<<<nb, 1024, 0, E.st>>>(in, out, E.scan_tmp, n);
    PT_COUNT(), k_scan_totals<<<1, kScanTotThreads, 0, E.st>>>(E.scan_tmp, nb);
    PT_COUNT(), k_scan_add<<<nb, 1024, 0, E.st>>>(out, E.scan_tmp, n);
    CKL("exclusive_scan_i32");
    return 0;
}

// Ttr(p) = interpolate(rtr(p), str(p)) of Tratio (extendT, compute_derivatives, interpolate:
// composition.f90:726-737) for the m tracers ids[0..m)
__global__ void __launch_bounds__(256) k_interp_T_at(const int32_t* __restrict__ ids, int64_t m, Tables tb,
                                                     const double* __restrict__ r, const double* __restrict__ s,
                                                     double* __restrict__ Tt, Geo g) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const int32_t p = ids[j];
    const double rr = r[p], ss = s[p];
    int i = cell_index(rr, cK.inv_dr, cK.dr, cK.exact_div, cK.p_inv_dr);
    int k = cell_index(ss, cK.inv_ds, cK.ds, cK.exact_div, cK.p_inv_ds);
    i = min(max(i, 0), cK.nx);
    k = min(max(k, 0), cK.nz);
    const double hr = rr - (double)i * cK.dr, hs = ss - (double)k * cK.ds;
    const double a1 = hr * cK.inv_fact[1], a2 = hr * hr * cK.inv_fact[2], a3 = hr * hr * hr * cK.inv_fact[3];
    const double b1 = hs * cK.inv_fact[1], b2 = hs * hs * cK.inv_fact[2], b3 = hs * hs * hs * cK.inv_fact[3];
    Tt[p] = interp(tb, g, i, k, a1, a2, a3, b1, b2, b3);
}
int interp_T_at(Engine& E, const int32_t* ids, int64_t m) {
    if (m <= 0) return 0;
    if (int rc = extend_T(E)) return rc;
    if (int rc = compute_derivatives(E, E.Text, 2)) return rc;
    const Tables tb{E.Text, E.der[2][0], E.der[2][1], E.der[2][2]};
    PT_COUNT(), k_interp_T_at<<<nblk(m, 256), 256, 0, E.st>>>(ids, m, tb, E.rtr, E.str, E.Ttr, E.g1);
    CKL("k_interp_T_at");
    return 0;
}

}  // namespace pt
