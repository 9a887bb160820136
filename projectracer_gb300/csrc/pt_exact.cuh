// pt_exact.cuh -- the biharmonic stream operator A S with its stencil sums formed exactly in
// integer arithmetic, for the kernels whose FP64 stencil would otherwise run on this part's
// narrow FP64 pipe (the mixed path's level-1 residual, the FP64 path's RKC stages and residuals).
//
// The reference's finite-difference weights are small rationals: D1 = [1,-8,0,8,-1]/12,
// D2 = [-1,16,-30,16,-1]/12, D3 = [1,-8,13,0,-13,8,-1]/8, D4 = [-1,12,-39,56,-39,12,-1]/6
// (checked against the FP64 weights at setup; the kernels are used only when they match), so
// with S in fixed point every derivative sum (stream_derivatives) is an integer.  A CTA stages its
// tile of S (plus the 3-node halo) in shared memory as X = round(S 2^s), s chosen from the tile's
// largest exponent so that |X| < 2^62, split as X = Xh 2^31 + Xl with Xl in [0, 2^31); each sum
// is accumulated exactly on both halves in 64-bit integers (|sum| < 2^46).  Only the combination
// with the viscosity fields is FP64 arithmetic: about 16 operations per node instead of about
// 120.  The sums are exact and the rounding of S to fixed point is 2^-62 of the tile's largest
// value, so the result is at least as accurate as the FP64 stencil (which rounds at every one of
// its ~120 operations).
#pragma once
#include <cmath>

#include "pt_consts.cuh"

namespace pt {

static __constant__ int cD1i[5], cD2i[5], cD3i[7], cD4i[7];

// Tile geometry: TX x TZ nodes, a CTA of TX x TY threads (TZ / TY rows of nodes per thread), halo 3.
// Large tiles amortise the halo on the fine levels; small ones keep enough CTAs in flight on the
// coarse levels, where a kernel's time is its CTAs' critical path.
template <int TX_, int TZ_, int TY_>
struct TileGeo {
    static constexpr int TX = TX_, TZ = TZ_, TY = TY_, H = 3;
    static constexpr int W = TX + 2 * H, HT = TZ + 2 * H, NT = TX * TY, RPT = TZ / TY;
};
using TileBig = TileGeo<32, 16, 8>;   // 256 threads, 2 nodes each
using TileSmall = TileGeo<16, 8, 8>;  // 128 threads, 1 node each
constexpr int kRfTX = TileBig::TX, kRfTZ = TileBig::TZ, kRfH = TileBig::H;
constexpr int kRfW = TileBig::W, kRfHt = TileBig::HT;
// the tiling for a level of (nx-1) x (nz-1) interior nodes: large tiles while they give at least
// two CTAs per SM of this part (152 SMs)
__host__ __forceinline__ bool use_big_tiles(int nx, int nz) {
    return (size_t)((nx - 2) / TileBig::TX + 1) * (size_t)((nz - 2) / TileBig::TZ + 1) >= 304;
}

// v * 2^e2 as a double, exactly (|v| < 2^53, result normal), from integer operations only
__device__ __forceinline__ double i64_to_double_scaled(long long v, int e2) {
    if (v == 0) return 0.0;
    const unsigned long long sgn = (unsigned long long)v & 0x8000000000000000ull;
    const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    const int lz = __clzll(a);                      // a < 2^53: lz >= 11
    const unsigned long long mant = a << (lz - 11);  // leading one at bit 52
    const unsigned long long ex = (unsigned long long)(1023 + 63 - lz + e2);
    if ((long long)ex <= 0) return 0.0;  // below the normal range (S itself near underflow)
    return __longlong_as_double((long long)(sgn | (ex << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

struct HL {
    long long h, l;
};
__device__ __forceinline__ void mac(HL& a, int c, int2 v) {
    a.h += (long long)c * v.x;
    a.l += (long long)c * v.y;
}
__device__ __forceinline__ void mac64(HL& a, int c, const HL& v) {
    a.h += (long long)c * v.h;
    a.l += (long long)c * v.l;
}
// (h 2^31 + l) 2^-s, rounded once; s = 1084 - emax
__device__ __forceinline__ double hl_value(const HL& a, int emax) {
    const int s = 1084 - emax;
    return i64_to_double_scaled(a.h, 31 - s) + i64_to_double_scaled(a.l, -s);
}

// Stages the tile of S with first interior node (i0, k0) (nodes i0-3 .. i0+TX+2, k0-3 .. k0+TZ+2;
// zero beyond nx+3 / nz+3) as fixed point in X; returns the tile's largest biased exponent (0x7FF
// when the tile holds Inf/NaN).  Called by all TG::NT threads of the CTA (blockDim TX x TY).
template <class TG>
__device__ __forceinline__ int load_tile_fx(int2 (*X)[TG::W], int* emax_s, const double* __restrict__ S, Geo g, int i0,
                                            int k0, int nx, int nz) {
    constexpr int kRfW = TG::W, kRfH = TG::H;
    constexpr int NT = TG::W * TG::HT, PER = (NT + TG::NT - 1) / TG::NT;
    const int tid = threadIdx.y * TG::TX + threadIdx.x;
    if (tid == 0) *emax_s = 0;
    __syncthreads();
    unsigned long long raw[PER];
    int em = 0;
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int idx = tid + TG::NT * q;
        unsigned long long b = 0;
        if (idx < NT) {
            const int i = i0 - kRfH + idx % kRfW, k = k0 - kRfH + idx / kRfW;
            if (i <= nx + kRfH && k <= nz + kRfH) b = (unsigned long long)__double_as_longlong(S[g.at(i, k)]);
        }
        raw[q] = b;
        em = max(em, (int)((b >> 52) & 0x7FF));
    }
    atomicMax(emax_s, em);
    __syncthreads();
    const int emax = *emax_s;
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int idx = tid + TG::NT * q;
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
        const long long h = v >> 31;  // floor
        X[idx / kRfW][idx % kRfW] = make_int2((int)h, (int)(v - (h << 31)));
    }
    __syncthreads();
    return emax;
}

// A S at the node at tile position (cx, cz) (stream_derivatives + the viscosity terms of
// stream_space, without the right-hand side); NaN when the tile holds Inf/NaN.
template <bool SQUARE, int W>
__device__ __forceinline__ double tile_apply_A(const int2 (*X)[W], int cx, int cz, int emax,
                                               const double* __restrict__ vis, const double* __restrict__ vx,
                                               const double* __restrict__ vz, const double* __restrict__ vxz,
                                               const double* __restrict__ vxxmzz, size_t o, int ivis,
                                               const ResFxK& K) {
    if (emax == 0x7FF) return __longlong_as_double(0x7FF8000000000000ll);
    HL I2x{0, 0}, I3x{0, 0}, I4x{0, 0}, I2z{0, 0}, I3z{0, 0}, I4z{0, 0};
#pragma unroll
    for (int j = 0; j < 7; j++) {
        const int2 ax = X[cz][cx + j - 3], az = X[cz + j - 3][cx];
        if (j >= 1 && j <= 5) { mac(I2x, cD2i[j - 1], ax); mac(I2z, cD2i[j - 1], az); }
        if (j != 3) { mac(I3x, cD3i[j], ax); mac(I3z, cD3i[j], az); }
        mac(I4x, cD4i[j], ax);
        mac(I4z, cD4i[j], az);
    }
    HL I11{0, 0}, I12{0, 0}, I21{0, 0}, I22{0, 0};  // I<x order><z order>
#pragma unroll
    for (int kk = 0; kk < 5; kk++) {
        HL d1{0, 0}, d2{0, 0};
#pragma unroll
        for (int ii = 0; ii < 5; ii++) {
            const int2 v = X[cz + kk - 2][cx + ii - 2];
            if (ii != 2) mac(d1, cD1i[ii], v);
            mac(d2, cD2i[ii], v);
        }
        if (kk != 2) { mac64(I11, cD1i[kk], d1); mac64(I21, cD1i[kk], d2); }
        mac64(I12, cD2i[kk], d1);
        mac64(I22, cD2i[kk], d2);
    }
    double acc;
    if (SQUARE) {
        // vis (Sxxxx + Szzzz + 2 Sxxzz) = vis (24 I4x + 24 I4z + 2 I22) / (144 h^4), and so on
        const HL ga{24 * (I4x.h + I4z.h) + 2 * I22.h, 24 * (I4x.l + I4z.l) + 2 * I22.l};
        acc = K.k[0] * vis[o] * hl_value(ga, emax);
        if (ivis != 0) {
            const HL gb{I2x.h - I2z.h, I2x.l - I2z.l};
            const HL gd{18 * I3x.h + I12.h, 18 * I3x.l + I12.l};
            const HL ge{18 * I3z.h + I21.h, 18 * I3z.l + I21.l};
            acc = fma(K.k[1] * vxxmzz[o], hl_value(gb, emax), acc);
            acc = fma(K.k[2] * vxz[o], hl_value(I11, emax), acc);
            acc = fma(K.k[3] * vx[o], hl_value(gd, emax), acc);
            acc = fma(K.k[4] * vz[o], hl_value(ge, emax), acc);
        }
    } else {
        // k: weights of [Sxxxx, Szzzz, Sxxzz, Sxx, Szz, Sxz, Sxxx, Sxzz, Szzz, Sxxz]
        const double Sxxxx = K.k[0] * hl_value(I4x, emax), Szzzz = K.k[1] * hl_value(I4z, emax);
        const double Sxxzz = K.k[2] * hl_value(I22, emax);
        acc = vis[o] * (Sxxxx + Szzzz + 2.0 * Sxxzz);
        if (ivis != 0) {
            const double Sxx = K.k[3] * hl_value(I2x, emax), Szz = K.k[4] * hl_value(I2z, emax);
            const double Sxz = K.k[5] * hl_value(I11, emax);
            const double Sxxx = K.k[6] * hl_value(I3x, emax), Sxzz = K.k[7] * hl_value(I12, emax);
            const double Szzz = K.k[8] * hl_value(I3z, emax), Sxxz = K.k[9] * hl_value(I21, emax);
            acc += vxxmzz[o] * (Sxx - Szz) + 4.0 * vxz[o] * Sxz + 2.0 * vx[o] * (Sxxx + Sxzz) + 2.0 * vz[o] * (Szzz + Sxxz);
        }
    }
    return acc;
}

// Integer forms of the stencils (uploaded into this translation unit) and the per-level weights;
// false (and the FP64 stencils are used) when the weights are not the rationals above.
static inline bool exact_stencils_setup(Engine& E) {
    const Consts& K = E.K;
    const int d1[5] = {1, -8, 0, 8, -1}, d2[5] = {-1, 16, -30, 16, -1};
    const int d3[7] = {1, -8, 13, 0, -13, 8, -1}, d4[7] = {-1, 12, -39, 56, -39, 12, -1};
    for (int j = 0; j < 5; j++)
        if (std::fabs(12.0 * K.D1[j + 1] - d1[j]) > 1e-9 || std::fabs(12.0 * K.D2[j + 1] - d2[j]) > 1e-9) return false;
    for (int j = 0; j < 7; j++)
        if (std::fabs(8.0 * K.D3[j] - d3[j]) > 1e-9 || std::fabs(6.0 * K.D4[j] - d4[j]) > 1e-9) return false;
    if (cudaMemcpyToSymbol(cD1i, d1, sizeof d1) != cudaSuccess || cudaMemcpyToSymbol(cD2i, d2, sizeof d2) != cudaSuccess ||
        cudaMemcpyToSymbol(cD3i, d3, sizeof d3) != cudaSuccess || cudaMemcpyToSymbol(cD4i, d4, sizeof d4) != cudaSuccess)
        return false;
    for (int l = 1; l <= E.grids && l < PT_MAXLEV; l++) {
        const LevConst& L = E.L[l];
        ResFxK& R = E.resfx[l];
        R.square = L.dr == L.ds ? 1 : 0;
        for (double& k : R.k) k = 0.0;
        if (R.square) {
            const double h = L.dr;
            R.k[0] = 1.0 / (144.0 * h * h * h * h);
            R.k[1] = 1.0 / (12.0 * h * h);
            R.k[2] = 4.0 / (144.0 * h * h);
            R.k[3] = 2.0 / (144.0 * h * h * h);
            R.k[4] = 2.0 / (144.0 * h * h * h);
        } else {
            R.k[0] = 1.0 / (6.0 * L.dr4);
            R.k[1] = 1.0 / (6.0 * L.ds4);
            R.k[2] = 1.0 / (144.0 * L.dr2ds2);
            R.k[3] = 1.0 / (12.0 * L.dr2);
            R.k[4] = 1.0 / (12.0 * L.ds2);
            R.k[5] = 1.0 / (144.0 * L.drds);
            R.k[6] = 1.0 / (8.0 * L.dr3);
            R.k[7] = 1.0 / (144.0 * L.drds2);
            R.k[8] = 1.0 / (8.0 * L.ds3);
            R.k[9] = 1.0 / (144.0 * L.dr2ds);
        }
    }
    return true;
}

}  // namespace pt
