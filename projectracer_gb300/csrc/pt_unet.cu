// pt_unet.cu -- learned psi guess (no reference counterpart): BF16 implicit-GEMM convolutions
// on the tcgen05 tensor cores (pt_tc.cuh), their self-check entry point, and the U-Net built on
// them.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pt_internal.h"
#include "../../include/ptgpu_unet.h"
#include "pt_tc.cuh"
#include <cuda_bf16.h>

namespace pt {

// plain GEMM problem: C (M x N, FP32) = A (M x K) * B (N x K)^T, BF16 row-major operands
struct GemmProb {
    static constexpr int kGather = tc::kGatherElem;
    int M, N, K, Ntile, kc_split;
    const uint16_t* A;
    const uint16_t* B;
    float* C;
    __device__ __forceinline__ uint16_t gather_a(int r, int k) const {
        return (r < M && k < K) ? A[(size_t)r * K + k] : (uint16_t)0;
    }
    __device__ __forceinline__ uint16_t gather_b(int c, int k) const { return k < K ? B[(size_t)c * K + k] : (uint16_t)0; }
    __device__ __forceinline__ void store(int r, int c, int, float v) const { C[(size_t)r * N + c] = v; }
};


static inline unsigned nblk(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

// ============================================================================ U-Net kernels
__device__ __forceinline__ uint16_t f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }
__device__ __forceinline__ float bf2f(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// The input of a convolution as seen by its im2col gather, at the convolution's resolution
// (B x H x W): mode 0 one BF16 NHWC tensor; mode 1 a tensor at 2H x 2W averaged over 2x2 (pooling);
// mode 2 the concatenation of a tensor at H/2 x W/2 read nearest-neighbour (upsampling, channels
// 0..C0-1) and a skip tensor at H x W (channels C0..C0+C1-1).
struct InView {
    const uint16_t* t0;
    const uint16_t* t1;
    int B, H, W, C0, C1, mode;
    __host__ __device__ int C() const { return C0 + C1; }
    __device__ __forceinline__ float get(int b, int y, int x, int c) const {
        if (mode == 0) return bf2f(t0[(((size_t)b * H + y) * W + x) * C0 + c]);
        if (mode == 1) {
            const size_t W2 = 2 * (size_t)W;
            const uint16_t* q = t0 + (((size_t)b * 2 * H + 2 * y) * W2 + 2 * x) * C0 + c;
            const float s = ((bf2f(q[0]) + bf2f(q[C0])) + bf2f(q[W2 * C0])) + bf2f(q[W2 * C0 + C0]);
            return s * 0.25f;
        }
        if (c < C0) return bf2f(t0[(((size_t)b * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)) * C0 + c]);
        return bf2f(t1[(((size_t)b * H + y) * W + x) * C1 + (c - C0)]);
    }
};

// pixel p of a B x H x W grid shifted by tap (3x3, row-major taps); false outside the grid
__device__ __forceinline__ bool tap_pixel(int p, int tap, int H, int W, int& b, int& y, int& x) {
    x = p % W;
    const int r = p / W;
    y = r % H;
    b = r / H;
    y += tap / 3 - 1;
    x += tap % 3 - 1;
    return y >= 0 && y < H && x >= 0 && x < W;
}

// 8 BF16 values from one 16-byte-aligned address
__device__ __forceinline__ uint4 ld8(const uint16_t* p) { return *reinterpret_cast<const uint4*>(p); }
__device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }

// channels c..c+7 of a view at pixel (b, y, x) as 8 BF16 values (c, C0 and C1 multiples of 8):
// one 16-byte load, or four averaged in the order of InView::get for a pooled view
__device__ __forceinline__ uint4 view_load8(const InView& in, int b, int y, int x, int c) {
    if (in.mode == 0) return ld8(in.t0 + (((size_t)b * in.H + y) * in.W + x) * in.C0 + c);
    if (in.mode == 2) {
        if (c < in.C0) return ld8(in.t0 + (((size_t)b * (in.H >> 1) + (y >> 1)) * (in.W >> 1) + (x >> 1)) * in.C0 + c);
        return ld8(in.t1 + (((size_t)b * in.H + y) * in.W + x) * in.C1 + (c - in.C0));
    }
    const size_t W2 = 2 * (size_t)in.W;
    const uint16_t* q = in.t0 + (((size_t)b * 2 * in.H + 2 * y) * W2 + 2 * x) * in.C0 + c;
    const uint4 a = ld8(q), bq = ld8(q + in.C0), cq = ld8(q + W2 * in.C0), d = ld8(q + W2 * in.C0 + in.C0);
    const uint32_t* pa = &a.x;
    const uint32_t* pb = &bq.x;
    const uint32_t* pc = &cq.x;
    const uint32_t* pd = &d.x;
    uint32_t o[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        uint16_t h[2];
#pragma unroll
        for (int e = 0; e < 2; e++) {
            const int sh = 16 * e;
            const float sum = ((bf2f((uint16_t)(pa[j] >> sh)) + bf2f((uint16_t)(pb[j] >> sh))) +
                               bf2f((uint16_t)(pc[j] >> sh))) + bf2f((uint16_t)(pd[j] >> sh));
            h[e] = f2bf(sum * 0.25f);
        }
        o[j] = pack2(h[0], h[1]);
    }
    return make_uint4(o[0], o[1], o[2], o[3]);
}

// channels c..c+7 of dZ (the ReLU-masked gradient, BF16) at flat index idx = pixel * C + c
__device__ __forceinline__ uint4 dz_load8(const float* dY, const uint16_t* Y, size_t idx) {
    const float4 g0 = *reinterpret_cast<const float4*>(dY + idx), g1 = *reinterpret_cast<const float4*>(dY + idx + 4);
    const float g[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
    uint16_t h[8];
    if (Y) {
        const uint4 m = ld8(Y + idx);
        const uint32_t mm[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const uint16_t yb = (uint16_t)(mm[j >> 1] >> (16 * (j & 1)));
            h[j] = bf2f(yb) > 0.f ? f2bf(g[j]) : (uint16_t)0;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 8; j++) h[j] = f2bf(g[j]);
    }
    return make_uint4(pack2(h[0], h[1]), pack2(h[2], h[3]), pack2(h[4], h[5]), pack2(h[6], h[7]));
}

// forward: out[p][co] = relu(sum_{tap,ci} in(p+tap)[ci] w[co][tap][ci] + bias[co]) in BF16.
// K = 9 cin, ordered (tap, ci): with cin a multiple of 8 the 8 values of a gather_a8 are 8
// consecutive channels of one pixel (one 16-byte load of an NHWC tensor, four for a pooled view),
// and those of a gather_b8 8 consecutive weights; the first layer (cin = 4) gathers element-wise.
struct ConvFwd {
    static constexpr int kGather = tc::kGatherRow;
    int M, N, K, Ntile, kc_split;
    InView in;
    const uint16_t* w;
    const float* bias;
    uint16_t* out;
    int relu;
    __device__ __forceinline__ uint16_t gather_a(int p, int k) const {
        if (p >= M || k >= K) return 0;
        const int cin = in.C(), tap = k / cin, ci = k - tap * cin;
        int b, y, x;
        if (!tap_pixel(p, tap, in.H, in.W, b, y, x)) return 0;
        return f2bf(in.get(b, y, x, ci));
    }
    __device__ __forceinline__ uint16_t gather_b(int co, int k) const {
        return (co < N && k < K) ? w[(size_t)co * K + k] : (uint16_t)0;
    }
    __device__ __forceinline__ uint4 gather_a8(int p, int k0) const {
        const int cin = in.C();
        if ((cin & 7) || (in.C0 & 7) || k0 + 8 > K) {
            uint16_t v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = gather_a(p, k0 + j);
            return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
        }
        if (p >= M) return make_uint4(0u, 0u, 0u, 0u);
        const int tap = k0 / cin, ci = k0 - tap * cin;
        int b, y, x;
        if (!tap_pixel(p, tap, in.H, in.W, b, y, x)) return make_uint4(0u, 0u, 0u, 0u);
        return view_load8(in, b, y, x, ci);
    }
    __device__ __forceinline__ uint4 gather_b8(int co, int k0) const {
        if ((K & 7) || co >= N || k0 + 8 > K) {
            uint16_t v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = gather_b(co, k0 + j);
            return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
        }
        return ld8(w + (size_t)co * K + k0);
    }
    __device__ __forceinline__ void store(int p, int co, int, float v) const {
        v += bias[co];
        if (relu) v = fmaxf(v, 0.f);
        out[(size_t)p * N + co] = f2bf(v);
    }
};

// gradient w.r.t. the pre-activation of a layer, as a BF16 GEMM operand: dY masked by Y > 0
__device__ __forceinline__ uint16_t dz_bf(const float* dY, const uint16_t* Y, size_t idx) {
    const float g = dY[idx];
    if (Y && !(bf2f(Y[idx]) > 0.f)) return 0;
    return f2bf(g);
}

// backward data: dX[q][ci] = sum_{t,co} dZ[q + tap t][co] w[co][8 - t][ci]  (FP32 out).  K is
// ordered (t, co): a gather_a8 takes 8 consecutive channels of dZ at one shifted pixel (two 16-byte
// loads of dY, one of the ReLU mask), a gather_b8 8 consecutive weights of wbd[ci][t][co] =
// w[co][8 - t][ci], the layout k_w_bwd_layout writes before the GEMM.
struct ConvBwdData {
    static constexpr int kGather = tc::kGatherRow;
    int M, N, K, Ntile, kc_split;  // M pixels, N = Cin, K = 9 Cout
    int H, W, Cout;
    const float* dY;
    const uint16_t* Y;
    const uint16_t* w;
    const uint16_t* wbd;
    float* dX;
    __device__ __forceinline__ uint4 gather_a8(int q, int k0) const {
        if ((Cout & 7) || k0 + 8 > K) {
            uint16_t v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = gather_a(q, k0 + j);
            return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
        }
        if (q >= M) return make_uint4(0u, 0u, 0u, 0u);
        const int t = k0 / Cout, co = k0 - t * Cout;
        int b, y, x;
        if (!tap_pixel(q, t, H, W, b, y, x)) return make_uint4(0u, 0u, 0u, 0u);
        return dz_load8(dY, Y, (((size_t)b * H + y) * W + x) * Cout + co);
    }
    __device__ __forceinline__ uint4 gather_b8(int ci, int k0) const {
        if ((K & 7) || ci >= N || k0 + 8 > K) {
            uint16_t v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = gather_b(ci, k0 + j);
            return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
        }
        return ld8(wbd + (size_t)ci * K + k0);
    }
    __device__ __forceinline__ uint16_t gather_a(int q, int k) const {
        if (q >= M || k >= K) return 0;
        const int t = k / Cout, co = k - t * Cout;
        int b, y, x;
        if (!tap_pixel(q, t, H, W, b, y, x)) return 0;
        return dz_bf(dY, Y, (((size_t)b * H + y) * W + x) * Cout + co);
    }
    __device__ __forceinline__ uint16_t gather_b(int ci, int k) const {
        if (ci >= N || k >= K) return 0;
        const int t = k / Cout, co = k - t * Cout;
        return w[((size_t)co * 9 + (8 - t)) * N + ci];
    }
    __device__ __forceinline__ void store(int q, int ci, int, float v) const { dX[(size_t)q * N + ci] = v; }
};

// backward weights (split over pixels): part[z][tap*Cin + ci][co] = sum_{p in split z} in(p+tap)[ci] dZ[p][co]
struct ConvBwdW {
    static constexpr int kGather = tc::kGatherCol;
    int M, N, K, Ntile, kc_split;  // M = 9 Cin, N = Cout, K = pixels
    InView in;
    const float* dY;
    const uint16_t* Y;
    float* part;
    __device__ __forceinline__ uint16_t gather_a(int kk, int p) const {
        if (kk >= M || p >= K) return 0;
        const int cin = in.C(), tap = kk / cin, ci = kk - tap * cin;
        int b, y, x;
        if (!tap_pixel(p, tap, in.H, in.W, b, y, x)) return 0;
        return f2bf(in.get(b, y, x, ci));
    }
    __device__ __forceinline__ uint16_t gather_b(int co, int p) const {
        return (co < N && p < K) ? dz_bf(dY, Y, (size_t)p * N + co) : (uint16_t)0;
    }
    // A[kk0..kk0+7][p]: channels ci..ci+7 of the input at pixel p shifted by the rows' tap
    __device__ __forceinline__ uint4 gather_col_a(int kk0, int p) const {
        const int cin = in.C();
        if ((cin & 7) || (in.C0 & 7)) {
            uint16_t v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = gather_a(kk0 + j, p);
            return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
        }
        if (kk0 >= M || p >= K) return make_uint4(0u, 0u, 0u, 0u);
        const int tap = kk0 / cin, ci = kk0 - tap * cin;
        int b, y, x;
        if (!tap_pixel(p, tap, in.H, in.W, b, y, x)) return make_uint4(0u, 0u, 0u, 0u);
        return view_load8(in, b, y, x, ci);
    }
    // B[co0..co0+7][p]: channels co0..co0+7 of dZ at pixel p
    __device__ __forceinline__ uint4 gather_col_b(int co0, int p) const {
        if (N & 7) {
            uint16_t v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = gather_b(co0 + j, p);
            return make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
        }
        if (co0 >= N || p >= K) return make_uint4(0u, 0u, 0u, 0u);
        return dz_load8(dY, Y, (size_t)p * N + co0);
    }
    __device__ __forceinline__ void store(int kk, int co, int z, float v) const {
        part[((size_t)z * M + kk) * N + co] = v;
    }
};

// wbd[ci][t][co] = w[co][8 - t][ci]: the weights in the K order of the backward-data GEMM
__global__ void k_w_bwd_layout(uint16_t* __restrict__ wbd, const uint16_t* __restrict__ w, int cin, int cout) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (size_t)cin * 9 * cout) return;
    const int co = (int)(q % cout);
    const int t = (int)((q / cout) % 9);
    const int ci = (int)(q / ((size_t)cout * 9));
    wbd[q] = w[((size_t)co * 9 + (8 - t)) * cin + ci];
}

// dW[co][kk] = sum_z part[z][kk][co], z ascending
__global__ void k_wgrad_reduce(float* dW, const float* part, int nsplit, int M, int N) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M * N) return;
    const int kk = q / N, co = q % N;
    float s = 0.f;
    for (int z = 0; z < nsplit; z++) s += part[((size_t)z * M + kk) * N + co];
    dW[(size_t)co * M + kk] = s;
}

// db[co] = sum_p dZ[p][co] (block per channel, fixed-order tree)
__global__ void k_bias_grad(float* db, const float* dY, const uint16_t* Y, int P, int C) {
    __shared__ float sh[256];
    const int co = blockIdx.x;
    float s = 0.f;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        const size_t idx = (size_t)p * C + co;
        if (!Y || bf2f(Y[idx]) > 0.f) s += dY[idx];
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[co] = sh[0];
}

// adjoints of the input views: add dXg (P x C at the view's resolution) into the sources' grads
__global__ void k_adj_plain(float* g0, const float* dX, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) g0[q] += dX[q];
}
__global__ void k_adj_pool(float* g0, const float* dX, int B, int H, int W, int C) {  // g0 at 2H x 2W
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)B * 4 * H * W * C;
    if (q >= n) return;
    const int c = (int)(q % C);
    size_t r = q / C;
    const int x2 = (int)(r % (2 * W));
    r /= (2 * W);
    const int y2 = (int)(r % (2 * H));
    const int b = (int)(r / (2 * H));
    g0[q] += 0.25f * dX[(((size_t)b * H + (y2 >> 1)) * W + (x2 >> 1)) * C + c];
}
__global__ void k_adj_upcat(float* g0, float* g1, const float* dX, int B, int H, int W, int C0, int C1) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n0 = (size_t)B * (H / 2) * (W / 2) * C0, n1 = (size_t)B * H * W * C1;
    const int C = C0 + C1;
    if (q < n0) {  // coarse source: sum of its 2x2 fine pixels, fixed order
        const int c = (int)(q % C0);
        size_t r = q / C0;
        const int x = (int)(r % (W / 2));
        r /= (W / 2);
        const int y = (int)(r % (H / 2));
        const int b = (int)(r / (H / 2));
        const size_t f = (((size_t)b * H + 2 * y) * W + 2 * x) * C + c;
        g0[q] += ((dX[f] + dX[f + C]) + dX[f + (size_t)W * C]) + dX[f + (size_t)W * C + C];
    } else if (q < n0 + n1) {
        const size_t u = q - n0;
        const int c = (int)(u % C1);
        const size_t p = u / C1;
        g1[u] += dX[p * C + C0 + c];
    }
}

// 1x1 output convolution (linear, FP32 out) and its backward
__global__ void k_out_fwd(float* y, const uint16_t* d, const float* w, const float* b, int P, int C) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    float s = b[0];
    for (int c = 0; c < C; c++) s += bf2f(d[(size_t)p * C + c]) * w[c];
    y[p] = s;
}
// loss = mean (y - t)^2; dy = 2 (y - t) / P; per-block partial sums of (y - t)^2
__global__ void k_mse(float* dy, float* lpart, const float* y, const float* t, int P) {
    __shared__ float sh[256];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.f;
    if (p < P) {
        const float d = y[p] - t[p];
        dy[p] = 2.f * d / (float)P;
        e = d * d;
    }
    sh[threadIdx.x] = e;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) lpart[blockIdx.x] = sh[0];
}
__global__ void k_out_bwd_data(float* gd, const float* dy, const float* w, int P, int C) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (size_t)P * C) return;
    gd[q] = dy[q / C] * w[q % C];
}
// dw[c] = sum_p dy[p] d[p][c] (block per c), db = sum_p dy[p] (block C)
__global__ void k_out_bwd_w(float* dw, float* db, const float* dy, const uint16_t* d, int P, int C) {
    __shared__ float sh[256];
    const int c = blockIdx.x;
    float s = 0.f;
    for (int p = threadIdx.x; p < P; p += blockDim.x) s += c < C ? dy[p] * bf2f(d[(size_t)p * C + c]) : dy[p];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (c < C) dw[c] = sh[0];
        else db[0] = sh[0];
    }
}

// Adam on FP32 master weights, with the BF16 copy used by the convolution GEMMs
__global__ void k_adam(float* w, float* m, float* v, uint16_t* wbf, const float* g, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float gg = g[q];
    const float mm = b1 * m[q] + (1.f - b1) * gg;
    const float vv = b2 * v[q] + (1.f - b2) * gg * gg;
    m[q] = mm;
    v[q] = vv;
    const float wn = w[q] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    w[q] = wn;
    wbf[q] = f2bf(wn);
}
__global__ void k_to_bf16(uint16_t* o, const float* i, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) o[q] = f2bf(i[q]);
}
// NCHW FP32 -> NHWC BF16
__global__ void k_input_nhwc(uint16_t* o, const float* i, int B, int C, int H, int W) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)B * C * H * W;
    if (q >= n) return;
    const int c = (int)(q % C);
    size_t r = q / C;
    const int x = (int)(r % W);
    r /= W;
    const int y = (int)(r % H);
    const int b = (int)(r / H);
    o[q] = f2bf(i[(((size_t)b * C + c) * H + y) * W + x]);
}

// ============================================================================ U-Net host side
// 4 levels, base width 32, 3x3 convolutions with ReLU, 2x2 average pooling, nearest upsampling
// with skip concatenation, 1x1 linear output.  Activations BF16 NHWC; FP32 master weights with
// BF16 copies for the tensor-core GEMMs; FP32 gradients; Adam.
struct UConv {
    int src0, src1, mode, cin, cout, level, out;  // src -1 = network input
    size_t woff, boff;                             // in the flat parameter vector
};

struct UNet {
    int H = 0, W = 0, maxB = 0;
    std::vector<UConv> L;
    int tch[14] = {}, tlev[14] = {};
    size_t nparams = 0, out_w = 0, out_b = 0;
    float *w32 = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
    uint16_t* wbf = nullptr;
    uint16_t* wbd = nullptr;  // one layer's weights in the backward-data K order (k_w_bwd_layout)
    int step = 0;
    uint16_t* act[14] = {};
    float* grad[14] = {};
    uint16_t* x0 = nullptr;
    float *xin = nullptr, *y = nullptr, *dy = nullptr, *tgt = nullptr, *lpart = nullptr, *dXg = nullptr,
          *part = nullptr;
    size_t part_cap = 0, dxg_cap = 0;
    int* derr = nullptr;
    cudaStream_t st = nullptr;
    std::vector<void*> owned;
};

static uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double unit_open(uint64_t& s) { return ((double)(splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
static double normal01(uint64_t& s) {  // Box-Muller
    const double u1 = unit_open(s), u2 = unit_open(s);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

template <class T>
static int ualloc(UNet& U, T** p, size_t n) {
    CK(cudaMalloc(p, sizeof(T) * (n ? n : 1)));
    U.owned.push_back(*p);
    CK(cudaMemsetAsync(*p, 0, sizeof(T) * (n ? n : 1), U.st));
    return 0;
}

// split of a weight-gradient GEMM over pixels: about two CTAs per SM in total
static void wsplit(int Mw, int P, int* per, int* ns) {
    const int gx = (Mw + 127) / 128, chunks = (P + 63) / 64;
    const int n0 = std::max(1, std::min(chunks, 304 / gx));
    *per = (chunks + n0 - 1) / n0;
    *ns = (chunks + *per - 1) / *per;
}

static int unet_build(UNet& U, int H, int W, int maxB, uint64_t seed) {
    U.H = H;
    U.W = W;
    U.maxB = maxB;
    // tensor ids: 0 e1a 1 e1 2 e2a 3 e2 4 e3a 5 e3 6 b1 7 b2 8 d3a 9 d3 10 d2a 11 d2 12 d1a 13 d1
    const int spec[14][7] = {{-1, -1, 0, 4, 32, 0, 0},   {0, -1, 0, 32, 32, 0, 1},   {1, -1, 1, 32, 64, 1, 2},
                             {2, -1, 0, 64, 64, 1, 3},   {3, -1, 1, 64, 128, 2, 4},  {4, -1, 0, 128, 128, 2, 5},
                             {5, -1, 1, 128, 256, 3, 6}, {6, -1, 0, 256, 256, 3, 7}, {7, 5, 2, 384, 128, 2, 8},
                             {8, -1, 0, 128, 128, 2, 9}, {9, 3, 2, 192, 64, 1, 10},  {10, -1, 0, 64, 64, 1, 11},
                             {11, 1, 2, 96, 32, 0, 12},  {12, -1, 0, 32, 32, 0, 13}};
    size_t off = 0;
    for (auto& r : spec) {
        UConv c{r[0], r[1], r[2], r[3], r[4], r[5], r[6], 0, 0};
        c.woff = off;
        off += (size_t)c.cout * 9 * c.cin;
        c.boff = off;
        off += c.cout;
        U.L.push_back(c);
        U.tch[c.out] = c.cout;
        U.tlev[c.out] = c.level;
    }
    for (auto& c : U.L)  // ConvFwd::gather_b8 reads 16-byte-aligned rows of the BF16 weights
        if (c.woff % 8) return fail(PT_ERR_CONFIG, "U-Net: weight offsets must be multiples of 8");
    U.out_w = off;
    off += 32;
    U.out_b = off;
    off += 1;
    U.nparams = off;
    int rc;
    size_t wmax = 0;
    for (auto& c : U.L) wmax = std::max(wmax, (size_t)c.cout * 9 * c.cin);
    if ((rc = ualloc(U, &U.w32, off)) || (rc = ualloc(U, &U.m, off)) || (rc = ualloc(U, &U.v, off)) ||
        (rc = ualloc(U, &U.g, off)) || (rc = ualloc(U, &U.wbf, off)) || (rc = ualloc(U, &U.wbd, wmax)) ||
        (rc = ualloc(U, &U.derr, 1)))
        return rc;
    // He-normal initialisation from a portable generator; biases zero
    std::vector<float> h(off, 0.f);
    uint64_t sd = seed;
    for (auto& c : U.L) {
        const double sdev = std::sqrt(2.0 / (9.0 * c.cin));
        for (size_t q = 0; q < (size_t)c.cout * 9 * c.cin; q++) h[c.woff + q] = (float)(sdev * normal01(sd));
    }
    for (int q = 0; q < 32; q++) h[U.out_w + q] = (float)(std::sqrt(1.0 / 32.0) * normal01(sd));
    CK(cudaMemcpyAsync(U.w32, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice, U.st));
    k_to_bf16<<<nblk(off, 256), 256, 0, U.st>>>(U.wbf, U.w32, off);
    CK(cudaGetLastError());
    // activations and gradients for maxB samples
    const size_t P0 = (size_t)maxB * H * W;
    for (int t = 0; t < 14; t++) {
        const size_t n = (P0 >> (2 * U.tlev[t])) * U.tch[t];
        if ((rc = ualloc(U, &U.act[t], n)) || (rc = ualloc(U, &U.grad[t], n))) return rc;
    }
    if ((rc = ualloc(U, &U.x0, P0 * 4)) || (rc = ualloc(U, &U.xin, P0 * 4)) || (rc = ualloc(U, &U.y, P0)) ||
        (rc = ualloc(U, &U.dy, P0)) || (rc = ualloc(U, &U.tgt, P0)) || (rc = ualloc(U, &U.lpart, P0 / 256 + 1)))
        return rc;
    // workspaces: the largest view gradient, and the largest split-K partial buffer
    size_t dxg = 0, part = 0;
    for (auto& c : U.L) {
        const size_t P = P0 >> (2 * c.level);
        dxg = std::max(dxg, P * (size_t)c.cin);
        int per, ns;
        wsplit(9 * c.cin, (int)P, &per, &ns);
        part = std::max(part, (size_t)ns * 9 * c.cin * c.cout);
    }
    U.dxg_cap = dxg;
    U.part_cap = part;
    if ((rc = ualloc(U, &U.dXg, dxg)) || (rc = ualloc(U, &U.part, part))) return rc;
    const int smax = (int)tc::smem_bytes(256);
    CK(cudaFuncSetAttribute(tc::k_tc_gemm<ConvFwd>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    CK(cudaFuncSetAttribute(tc::k_tc_gemm<ConvBwdData>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    CK(cudaFuncSetAttribute(tc::k_tc_gemm<ConvBwdW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    return 0;
}

static int ntile_for(int n) {
    const int tiles = (n + 255) / 256;
    const int t = (n + tiles - 1) / tiles;
    return (t + 15) / 16 * 16;
}

template <class Prob>
static int run_gemm(UNet& U, Prob p, int nsplit) {
    dim3 grid((p.M + tc::kTileM - 1) / tc::kTileM, (p.N + p.Ntile - 1) / p.Ntile, nsplit);
    tc::k_tc_gemm<Prob><<<grid, tc::kThreads, tc::smem_bytes(p.Ntile), U.st>>>(p, U.derr);
    CK(cudaGetLastError());
    return 0;
}

static InView view_of(const UNet& U, const UConv& c, int B) {
    InView v{};
    v.B = B;
    v.H = U.H >> c.level;
    v.W = U.W >> c.level;
    v.mode = c.mode;
    if (c.src0 < 0) {
        v.t0 = U.x0;
        v.C0 = 4;
    } else {
        v.t0 = U.act[c.src0];
        v.C0 = U.tch[c.src0];
    }
    if (c.mode == 2) {
        v.t1 = U.act[c.src1];
        v.C1 = U.tch[c.src1];
    }
    return v;
}

// network input already in U.xin (device, NCHW FP32); output in U.y ([B][H][W] FP32).
// ev (optional): 15 CUDA events recorded around the 14 convolution GEMMs
static int unet_forward(UNet& U, int B, cudaEvent_t* ev = nullptr) {
    const size_t P0 = (size_t)B * U.H * U.W;
    k_input_nhwc<<<nblk(P0 * 4, 256), 256, 0, U.st>>>(U.x0, U.xin, B, 4, U.H, U.W);
    CK(cudaGetLastError());
    int li = 0;
    if (ev) CK(cudaEventRecord(ev[0], U.st));
    for (auto& c : U.L) {
        const InView v = view_of(U, c, B);
        const int P = B * v.H * v.W;
        ConvFwd f{P, c.cout, 9 * c.cin, ntile_for(c.cout), 0, v, U.wbf + c.woff, U.w32 + c.boff, U.act[c.out], 1};
        if (int rc = run_gemm(U, f, 1)) return rc;
        if (ev) CK(cudaEventRecord(ev[++li], U.st));
    }
    k_out_fwd<<<nblk(P0, 256), 256, 0, U.st>>>(U.y, U.act[13], U.w32 + U.out_w, U.w32 + U.out_b, (int)P0, 32);
    CK(cudaGetLastError());
    return 0;
}

static int gemm_error(UNet& U) {
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, U.derr, sizeof(int), cudaMemcpyDeviceToHost, U.st));
    CK(cudaStreamSynchronize(U.st));
    if (herr) return fail(PT_ERR_ITER_CAP, "U-Net tensor-core GEMM: mbarrier wait gave up");
    return 0;
}

// gradients of the MSE loss against U.tgt into U.g; loss on the host
static int unet_backward(UNet& U, int B, float* loss) {
    const int P0 = B * U.H * U.W;
    const int nb = (int)nblk(P0, 256);
    k_mse<<<nb, 256, 0, U.st>>>(U.dy, U.lpart, U.y, U.tgt, P0);
    for (int t = 0; t < 14; t++)
        CK(cudaMemsetAsync(U.grad[t], 0, sizeof(float) * ((size_t)P0 >> (2 * U.tlev[t])) * U.tch[t], U.st));
    k_out_bwd_data<<<nblk((size_t)P0 * 32, 256), 256, 0, U.st>>>(U.grad[13], U.dy, U.w32 + U.out_w, P0, 32);
    k_out_bwd_w<<<33, 256, 0, U.st>>>(U.g + U.out_w, U.g + U.out_b, U.dy, U.act[13], P0, 32);
    CK(cudaGetLastError());
    for (int li = (int)U.L.size() - 1; li >= 0; li--) {
        const UConv& c = U.L[li];
        const InView v = view_of(U, c, B);
        const int P = B * v.H * v.W;
        const float* dY = U.grad[c.out];
        const uint16_t* Y = U.act[c.out];
        // weights: split over pixels, then a fixed-order reduction of the splits
        const int Mw = 9 * c.cin;
        int per, ns;
        wsplit(Mw, P, &per, &ns);
        if ((size_t)ns * Mw * c.cout > U.part_cap) return fail(PT_ERR_STATE, "U-Net: split workspace too small");
        ConvBwdW bw{Mw, c.cout, P, ntile_for(c.cout), per, v, dY, Y, U.part};
        if (int rc = run_gemm(U, bw, ns)) return rc;
        k_wgrad_reduce<<<nblk((size_t)Mw * c.cout, 256), 256, 0, U.st>>>(U.g + c.woff, U.part, ns, Mw, c.cout);
        k_bias_grad<<<c.cout, 256, 0, U.st>>>(U.g + c.boff, dY, Y, P, c.cout);
        CK(cudaGetLastError());
        if (c.src0 < 0) continue;  // the network input needs no gradient
        if ((size_t)P * c.cin > U.dxg_cap) return fail(PT_ERR_STATE, "U-Net: view-gradient workspace too small");
        const size_t nw = (size_t)c.cin * 9 * c.cout;
        k_w_bwd_layout<<<nblk(nw, 256), 256, 0, U.st>>>(U.wbd, U.wbf + c.woff, c.cin, c.cout);
        ConvBwdData bd{P, c.cin, 9 * c.cout, ntile_for(c.cin), 0, v.H, v.W, c.cout, dY, Y, U.wbf + c.woff, U.wbd,
                       U.dXg};
        if (int rc = run_gemm(U, bd, 1)) return rc;
        if (c.mode == 0) {
            const size_t n = (size_t)P * c.cin;
            k_adj_plain<<<nblk(n, 256), 256, 0, U.st>>>(U.grad[c.src0], U.dXg, n);
        } else if (c.mode == 1) {
            const size_t n = (size_t)B * 4 * v.H * v.W * c.cin;
            k_adj_pool<<<nblk(n, 256), 256, 0, U.st>>>(U.grad[c.src0], U.dXg, B, v.H, v.W, c.cin);
        } else {
            const size_t n = (size_t)B * (v.H / 2) * (v.W / 2) * v.C0 + (size_t)P * v.C1;
            k_adj_upcat<<<nblk(n, 256), 256, 0, U.st>>>(U.grad[c.src0], U.grad[c.src1], U.dXg, B, v.H, v.W, v.C0, v.C1);
        }
        CK(cudaGetLastError());
    }
    std::vector<float> lp(nb);
    CK(cudaMemcpyAsync(lp.data(), U.lpart, sizeof(float) * nb, cudaMemcpyDeviceToHost, U.st));
    if (int rc = gemm_error(U)) return rc;
    double sum = 0.0;
    for (float a : lp) sum += a;
    if (loss) *loss = (float)(sum / P0);
    return 0;
}

static int unet_adam(UNet& U, float lr) {
    U.step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)U.step), c2 = 1.f - std::pow(b2, (float)U.step);
    k_adam<<<nblk(U.nparams, 256), 256, 0, U.st>>>(U.w32, U.m, U.v, U.wbf, U.g, U.nparams, lr, b1, b2, 1e-8f, c1, c2);
    CK(cudaGetLastError());
    return 0;
}

// ============================================================================ engine side
// features of node (i, k), i < nx, k < nz, as the network's input planes [4][nz][nx]:
// T, C, log10(eta)/5, RHS/max|RHS| (0 on the boundary rows), and psi/max|psi| (training target)
__global__ void k_absmax_grid(const double* f, Geo g, int nx, int nz, unsigned long long* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    double a = 0.0;
    if (i <= nx && k <= nz) a = fabs(f[g.at(i, k)]);
    for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0 && a > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(a));
}
__global__ void k_features(float* x4, float* psi, const double* Tb, const double* Cb, const double* vis,
                           const double* rhs, const double* sf, Geo g, int nx, int nz, const unsigned long long* scal,
                           int comp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i >= nx || k >= nz) return;
    const size_t o = g.at(i, k), plane = (size_t)nx * nz, q = (size_t)k * nx + i;
    const double rmax = __longlong_as_double((long long)scal[0]), smax = __longlong_as_double((long long)scal[1]);
    x4[q] = (float)Tb[o];
    x4[plane + q] = comp ? (float)Cb[o] : 0.f;
    x4[2 * plane + q] = (float)(log10(vis[o]) * 0.2);
    x4[3 * plane + q] = (i > 0 && k > 0 && rmax > 0.0) ? (float)(rhs[o] / rmax) : 0.f;
    if (psi) psi[q] = smax > 0.0 ? (float)(sf[o] / smax) : 0.f;
}
// network output (psi shape, [nz][nx]) into the level-1 iterate: interior nodes, boundary 0
__global__ void k_guess_scatter(double* x, const float* y, Geo g, int nx, int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
    if (i > nx || k > nz) return;
    x[g.at(i, k)] = (i > 0 && k > 0 && i < nx && k < nz) ? (double)y[(size_t)k * nx + i] : 0.0;
}
__global__ void k_scale_all(double* x, double a, size_t n) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) x[q] *= a;
}

static int engine_features(Engine& E, float* x4, float* psi) {
    const Geo& g = E.g1;
    const int nx = E.cfg.nx, nz = E.cfg.nz;
    unsigned long long* scal = reinterpret_cast<unsigned long long*>(E.dscal);
    CK(cudaMemsetAsync(scal, 0, 16, E.st));
    dim3 gm(nblk(nx + 1, 128), nz + 1);
    k_absmax_grid<<<gm, 128, 0, E.st>>>(E.RHS[1], g, nx, nz, scal);
    if (psi) k_absmax_grid<<<gm, 128, 0, E.st>>>(E.SF, g, nx, nz, scal + 1);
    k_features<<<dim3(nblk(nx, 128), nz), 128, 0, E.st>>>(x4, psi, E.Tbuoy, E.Cbuoy, E.vis[1], E.RHS[1], E.SF, g, nx, nz,
                                                           scal, E.cfg.comp);
    CK(cudaGetLastError());
    return 0;
}

static int mean_resid(Engine& E, double* ratio) {
    if (int rc = residual_level1(E)) return rc;
    CK(cudaMemcpyAsync(E.hscal, E.dscal + 8, 8, cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    *ratio = E.hscal[0] / (double)(E.gl[1].nx - 2) / (double)(E.gl[1].nz - 2) / E.res_ref[1];
    return 0;
}

// Learned initial guess.  The network's psi shape g (BF16 output, grid-scale noise of order 1e-3)
// is scaled by the least-squares factor fitted on the coarsest level (coarse_scale_fit) and
// starts the solve.  The residual of the previous psi (the reference's warm start) is kept: if the
// residual after the first full cycle is not below it, the solver falls back to the previous psi
// (unet_check_fallback), so a poor guess costs one cycle.
int unet_guess(Engine& E) {
    E.unet_used = 0;
    if (!E.unet) return 0;
    UNet& U = *static_cast<UNet*>(E.unet_core);
    const Geo& g = E.g1;
    const int nx = E.cfg.nx, nz = E.cfg.nz;
    int rc;
    double r_prev = 0.0, alpha = 0.0;
    if ((rc = mean_resid(E, &r_prev))) return rc;  // err[1] holds the previous psi
    if ((rc = engine_features(E, U.xin, nullptr))) return rc;
    CK(cudaStreamSynchronize(E.st));
    if ((rc = unet_forward(U, 1)) || (rc = gemm_error(U))) return rc;
    k_guess_scatter<<<dim3(nblk(nx + 1, 128), nz + 1), 128, 0, E.st>>>(E.err[1], U.y, g, nx, nz);
    CK(cudaGetLastError());
    if ((rc = enforce_bcs_stream(E, 1, E.err[1])) || (rc = coarse_scale_fit(E, &alpha))) return rc;
    k_scale_all<<<nblk(g.elems(), 256), 256, 0, E.st>>>(E.err[1], alpha, g.elems());
    CK(cudaGetLastError());
    E.unet_r_prev = r_prev;
    E.unet_r_net = 0.0;
    E.unet_used = 1;
    return 0;
}

// Called with the residual ratio measured after the first full cycle from the network's guess:
// falls back to the previous psi when the guess did not lower the residual.  Returns 1 when the
// solve restarts from the previous psi.
int unet_check_fallback(Engine& E, double ratio) {
    if (E.unet_used != 1) return 0;
    E.unet_r_net = ratio;
    if (ratio < E.unet_r_prev) {
        E.unet_used = 2;  // kept; checked
        return 0;
    }
    E.unet_used = 0;
    if (cudaMemcpyAsync(E.err[1], E.SF, E.g1.elems() * sizeof(double), cudaMemcpyDeviceToDevice, E.st) != cudaSuccess)
        return -1;
    return 1;
}

}  // namespace pt

using namespace pt;

extern "C" {

int pt_tc_gemm_check(const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K) {
    if (!A || !B || !C) return fail(PT_ERR_ARG, "null pointer");
    if (M <= 0 || K <= 0 || N < 16 || N > 256 || N % 16) return fail(PT_ERR_ARG, "pt_tc_gemm_check: N must be 16..256, a multiple of 16");
    uint16_t *dA = nullptr, *dB = nullptr;
    float* dC = nullptr;
    int* derr = nullptr;
    int rc = 0, herr = 0;
    const size_t smem = tc::smem_bytes(N);
    auto cleanup = [&]() {
        if (dA) cudaFree(dA);
        if (dB) cudaFree(dB);
        if (dC) cudaFree(dC);
        if (derr) cudaFree(derr);
    };
    if ((rc = cuda_check(cudaMalloc(&dA, sizeof(uint16_t) * (size_t)M * K), "gemm check")) ||
        (rc = cuda_check(cudaMalloc(&dB, sizeof(uint16_t) * (size_t)N * K), "gemm check")) ||
        (rc = cuda_check(cudaMalloc(&dC, sizeof(float) * (size_t)M * N), "gemm check")) ||
        (rc = cuda_check(cudaMalloc(&derr, sizeof(int)), "gemm check")) ||
        (rc = cuda_check(cudaMemcpy(dA, A, sizeof(uint16_t) * (size_t)M * K, cudaMemcpyHostToDevice), "gemm check")) ||
        (rc = cuda_check(cudaMemcpy(dB, B, sizeof(uint16_t) * (size_t)N * K, cudaMemcpyHostToDevice), "gemm check")) ||
        (rc = cuda_check(cudaMemset(derr, 0, sizeof(int)), "gemm check")) ||
        (rc = cuda_check(cudaFuncSetAttribute(tc::k_tc_gemm<GemmProb>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "gemm check"))) {
        cleanup();
        return rc;
    }
    GemmProb p{M, N, K, N, 0, dA, dB, dC};
    tc::k_tc_gemm<GemmProb><<<dim3((M + tc::kTileM - 1) / tc::kTileM, 1, 1), tc::kThreads, smem>>>(p, derr);
    rc = cuda_check(cudaGetLastError(), "k_tc_gemm launch");
    if (!rc) rc = cuda_check(cudaDeviceSynchronize(), "k_tc_gemm");
    if (!rc) rc = cuda_check(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost), "gemm check");
    if (!rc) rc = cuda_check(cudaMemcpy(C, dC, sizeof(float) * (size_t)M * N, cudaMemcpyDeviceToHost), "gemm check");
    cleanup();
    if (!rc && herr) rc = fail(PT_ERR_ITER_CAP, "tensor-core GEMM: mbarrier wait gave up");
    return rc;
}

struct pt_unet {
    UNet u;
};

static void unet_release(pt_unet* n) {
    for (void* p : n->u.owned) cudaFree(p);
    if (n->u.st) cudaStreamDestroy(n->u.st);
    delete n;
}

int pt_unet_create(int nz, int nx, int max_batch, uint64_t seed, pt_unet** out) {
    if (!out) return fail(PT_ERR_ARG, "null pointer");
    *out = nullptr;
    if (nz < 8 || nx < 8 || nz % 8 || nx % 8 || max_batch < 1)
        return fail(PT_ERR_ARG, "pt_unet_create: nz and nx must be positive multiples of 8, max_batch >= 1");
    pt_unet* n = new pt_unet();
    int rc = cuda_check(cudaStreamCreateWithFlags(&n->u.st, cudaStreamNonBlocking), "U-Net stream");
    if (!rc) rc = unet_build(n->u, nz, nx, max_batch, seed);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(n->u.st), "U-Net init");
    if (rc) {
        std::string msg = g_err;
        unet_release(n);
        g_err = msg;
        return rc;
    }
    *out = n;
    return 0;
}

int pt_unet_destroy(pt_unet* net) {
    if (net) unet_release(net);
    return 0;
}

int pt_unet_num_params(pt_unet* net, int64_t* n) {
    if (!net || !n) return fail(PT_ERR_ARG, "null pointer");
    *n = (int64_t)net->u.nparams;
    return 0;
}

int pt_unet_get_params(pt_unet* net, float* host) {
    if (!net || !host) return fail(PT_ERR_ARG, "null pointer");
    UNet& U = net->u;
    CK(cudaMemcpyAsync(host, U.w32, sizeof(float) * U.nparams, cudaMemcpyDeviceToHost, U.st));
    CK(cudaStreamSynchronize(U.st));
    return 0;
}

int pt_unet_set_params(pt_unet* net, const float* host) {
    if (!net || !host) return fail(PT_ERR_ARG, "null pointer");
    UNet& U = net->u;
    CK(cudaMemcpyAsync(U.w32, host, sizeof(float) * U.nparams, cudaMemcpyHostToDevice, U.st));
    k_to_bf16<<<nblk(U.nparams, 256), 256, 0, U.st>>>(U.wbf, U.w32, U.nparams);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(U.st));
    return 0;
}

static int unet_input(UNet& U, const float* x, int batch) {
    if (batch < 1 || batch > U.maxB) return fail(PT_ERR_ARG, "U-Net: batch outside 1..max_batch");
    CK(cudaMemcpyAsync(U.xin, x, sizeof(float) * (size_t)batch * 4 * U.H * U.W, cudaMemcpyHostToDevice, U.st));
    return 0;
}

int pt_unet_forward(pt_unet* net, const float* x, int batch, float* y) {
    if (!net || !x || !y) return fail(PT_ERR_ARG, "null pointer");
    UNet& U = net->u;
    int rc;
    if ((rc = unet_input(U, x, batch)) || (rc = unet_forward(U, batch))) return rc;
    CK(cudaMemcpyAsync(y, U.y, sizeof(float) * (size_t)batch * U.H * U.W, cudaMemcpyDeviceToHost, U.st));
    return gemm_error(U);
}

int pt_unet_gradients(pt_unet* net, const float* x, const float* target, int batch, float* grads, float* loss) {
    if (!net || !x || !target || !grads) return fail(PT_ERR_ARG, "null pointer");
    UNet& U = net->u;
    int rc;
    if ((rc = unet_input(U, x, batch)) || (rc = unet_forward(U, batch))) return rc;
    CK(cudaMemcpyAsync(U.tgt, target, sizeof(float) * (size_t)batch * U.H * U.W, cudaMemcpyHostToDevice, U.st));
    if ((rc = unet_backward(U, batch, loss))) return rc;
    CK(cudaMemcpyAsync(grads, U.g, sizeof(float) * U.nparams, cudaMemcpyDeviceToHost, U.st));
    CK(cudaStreamSynchronize(U.st));
    return 0;
}

int pt_unet_train_step(pt_unet* net, const float* x, const float* target, int batch, float lr, float* loss) {
    if (!net || !x || !target) return fail(PT_ERR_ARG, "null pointer");
    UNet& U = net->u;
    int rc;
    if ((rc = unet_input(U, x, batch)) || (rc = unet_forward(U, batch))) return rc;
    CK(cudaMemcpyAsync(U.tgt, target, sizeof(float) * (size_t)batch * U.H * U.W, cudaMemcpyHostToDevice, U.st));
    if ((rc = unet_backward(U, batch, loss)) || (rc = unet_adam(U, lr))) return rc;
    CK(cudaStreamSynchronize(U.st));
    return 0;
}

int pt_unet_save(pt_unet* net, const char* path) {
    if (!net || !path) return fail(PT_ERR_ARG, "null pointer");
    UNet& U = net->u;
    std::vector<float> h(U.nparams);
    if (int rc = pt_unet_get_params(net, h.data())) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(PT_ERR_ARG, std::string("cannot write ") + path);
    const int32_t dims[2] = {U.H, U.W};
    const int64_t n = (int64_t)U.nparams;
    bool ok = std::fwrite("PTUNET01", 1, 8, f) == 8 && std::fwrite(dims, 4, 2, f) == 2 && std::fwrite(&n, 8, 1, f) == 1 &&
              std::fwrite(h.data(), 4, h.size(), f) == h.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? 0 : fail(PT_ERR_ARG, std::string("short write to ") + path);
}

int pt_unet_load(const char* path, int nz, int nx, int max_batch, pt_unet** out) {
    if (!path || !out) return fail(PT_ERR_ARG, "null pointer");
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(PT_ERR_ARG, std::string("cannot read ") + path);
    char magic[8];
    int32_t dims[2];
    int64_t n = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "PTUNET01", 8) == 0 && std::fread(dims, 4, 2, f) == 2 &&
              std::fread(&n, 8, 1, f) == 1 && n > 0 && n < ((int64_t)1 << 30);
    std::vector<float> h(ok ? (size_t)n : 0);
    ok = ok && std::fread(h.data(), 4, h.size(), f) == h.size();
    std::fclose(f);
    if (!ok) return fail(PT_ERR_ARG, std::string("not a U-Net weight file: ") + path);
    int rc = pt_unet_create(nz, nx, max_batch, 0, out);
    if (rc) return rc;
    if ((int64_t)(*out)->u.nparams != n) {
        pt_unet_destroy(*out);
        *out = nullptr;
        return fail(PT_ERR_ARG, "U-Net weight file has a different parameter count");
    }
    return pt_unet_set_params(*out, h.data());
}

int pt_unet_profile_forward(pt_unet* net, const float* x, int batch, float* ms) {
    if (!net || !x || !ms) return fail(PT_ERR_ARG, "null pointer");
    UNet& U = net->u;
    if (batch < 1 || batch > U.maxB) return fail(PT_ERR_ARG, "batch out of range");
    const size_t P0 = (size_t)batch * U.H * U.W;
    CK(cudaMemcpyAsync(U.xin, x, sizeof(float) * P0 * 4, cudaMemcpyHostToDevice, U.st));
    if (int rc = unet_forward(U, batch)) return rc;  // warm-up
    cudaEvent_t ev[15];
    for (auto& e : ev) CK(cudaEventCreate(&e));
    int rc = unet_forward(U, batch, ev);
    if (!rc) rc = cuda_check(cudaStreamSynchronize(U.st), "pt_unet_profile_forward");
    for (int l = 0; l < 14 && !rc; l++) cudaEventElapsedTime(&ms[l], ev[l], ev[l + 1]);
    for (auto& e : ev) cudaEventDestroy(e);
    if (!rc) rc = gemm_error(U);
    return rc;
}

int pt_training_pair(float* x4, float* psi) {
    if (!x4 || !psi) return fail(PT_ERR_ARG, "null pointer");
    if (!g_eng) return fail(PT_ERR_STATE, "call pt_init, pt_upload_state and pt_solve_psi first");
    Engine& E = *g_eng;
    if (!E.uploaded) return fail(PT_ERR_STATE, "call pt_upload_state and pt_solve_psi first");
    const size_t plane = (size_t)E.cfg.nx * E.cfg.nz;
    if (!E.pair_buf) CK(cudaMalloc(&E.pair_buf, sizeof(float) * 5 * plane));
    if (int rc = engine_features(E, E.pair_buf, E.pair_buf + 4 * plane)) return rc;
    CK(cudaMemcpyAsync(x4, E.pair_buf, sizeof(float) * 4 * plane, cudaMemcpyDeviceToHost, E.st));
    CK(cudaMemcpyAsync(psi, E.pair_buf + 4 * plane, sizeof(float) * plane, cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    return 0;
}

int pt_pair_capture(int capacity) {
    if (!g_eng) return fail(PT_ERR_STATE, "call pt_init first");
    if (capacity < 0 || capacity > 100000) return fail(PT_ERR_ARG, "pt_pair_capture: capacity must be 0..100000");
    Engine& E = *g_eng;
    if (E.pair_ring) cudaFree(E.pair_ring);
    E.pair_ring = nullptr;
    E.pair_cap = E.pair_n = 0;
    if (capacity == 0) return 0;
    const size_t plane = (size_t)E.cfg.nx * E.cfg.nz;
    CK(cudaMalloc(&E.pair_ring, sizeof(float) * 5 * plane * (size_t)capacity));
    E.pair_cap = capacity;
    return 0;
}

int pt_pair_take(float* x4, float* psi, int max_pairs, int* taken) {
    if (!g_eng) return fail(PT_ERR_STATE, "call pt_init first");
    if ((!x4 || !psi) && max_pairs > 0) return fail(PT_ERR_ARG, "null pointer");
    Engine& E = *g_eng;
    const size_t plane = (size_t)E.cfg.nx * E.cfg.nz;
    const int n = E.pair_n < max_pairs ? E.pair_n : (max_pairs > 0 ? max_pairs : 0);
    for (int j = 0; j < n; j++) {
        const float* src = E.pair_ring + (size_t)j * 5 * plane;
        CK(cudaMemcpyAsync(x4 + (size_t)j * 4 * plane, src, sizeof(float) * 4 * plane, cudaMemcpyDeviceToHost, E.st));
        CK(cudaMemcpyAsync(psi + (size_t)j * plane, src + 4 * plane, sizeof(float) * plane, cudaMemcpyDeviceToHost,
                           E.st));
    }
    CK(cudaStreamSynchronize(E.st));
    if (taken) *taken = n;
    E.pair_n = 0;
    return 0;
}

int pt_unet_guess_info(int* used, double* resid_prev, double* resid_net) {
    if (!g_eng) return fail(PT_ERR_STATE, "call pt_init first");
    Engine& E = *g_eng;
    if (used) *used = E.unet_used;
    if (resid_prev) *resid_prev = E.unet_r_prev;
    if (resid_net) *resid_net = E.unet_r_net;
    return 0;
}

}  // extern "C"

namespace pt {
int capture_pair(Engine& E) {
    if (!E.pair_ring || E.pair_n >= E.pair_cap) return 0;
    const size_t plane = (size_t)E.cfg.nx * E.cfg.nz;
    float* slot = E.pair_ring + (size_t)E.pair_n * 5 * plane;
    if (int rc = engine_features(E, slot, slot + 4 * plane)) return rc;
    E.pair_n++;
    return 0;
}

int unet_engine_load(Engine& E, const char* path) {
    if (!path) return fail(PT_ERR_ARG, "PT_GUESS_UNET needs a weight file");
    pt_unet* net = nullptr;
    if (int rc = pt_unet_load(path, E.cfg.nz, E.cfg.nx, 1, &net)) return rc;
    unet_engine_release(E);
    E.unet = net;
    E.unet_core = &net->u;
    return 0;
}
int unet_engine_release(Engine& E) {
    if (E.unet) pt_unet_destroy(static_cast<pt_unet*>(E.unet));
    E.unet = nullptr;
    E.unet_core = nullptr;
    if (E.pair_buf) cudaFree(E.pair_buf);
    E.pair_buf = nullptr;
    if (E.pair_ring) cudaFree(E.pair_ring);
    E.pair_ring = nullptr;
    E.pair_cap = E.pair_n = 0;
    return 0;
}
}  // namespace pt
