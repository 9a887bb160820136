// pt_tc.cuh -- 5th-generation tensor-core (tcgen05) GEMM tile for sm_103a, hand-written PTX.
//
// One CTA of 128 threads computes a 128 x N tile of D = A * B^T (A: M x K, B: N x K, BF16, FP32
// accumulation in tensor memory):
//   * the operand tiles of one K chunk (64) are gathered into shared memory by all threads, in
//     the canonical no-swizzle K-major layout: 8x8 "core matrices" of 128 contiguous bytes (8 rows
//     of 16 bytes), LBO = 128 B between core matrices adjacent in K, SBO = 1024 B between the
//     8-row groups (8 core matrices per 64-wide chunk);
//   * two stages: while the MMAs of chunk c read one stage, the threads gather chunk c+1 into the
//     other; a stage is overwritten only after the MMAs of the chunk two back have completed;
//   * P::kGather says how a problem fills the tiles: kGatherElem one element per call;
//     kGatherRow 8 consecutive K elements (one 16-byte core-matrix row) per call (gather_a8 /
//     gather_b8), the threads spread over rows first so that a warp's 16-byte stores hit all 32
//     banks; kGatherCol 8 consecutive rows at one K index per call (gather_col_a / gather_col_b,
//     for operands whose K is strided in memory): 8 lanes load the 8 columns of a core matrix and
//     transpose it among themselves with three shuffle stages, each lane then storing one row;
//   * one thread issues the four K=16 MMAs of a chunk (tcgen05.mma.cta_group::1.kind::f16) and
//     commits them to the stage's mbarrier; waits on it are bounded spins;
//   * the epilogue reads the accumulator with tcgen05.ld.32x32b (warp w owns TMEM lanes
//     32w..32w+31 = tile rows) and hands each row's values to the problem's store functor.
// A problem type supplies M, N, K, gather_a / gather_b (element (row, k) of A or B as BF16 bits,
// zero outside the matrix) and store(row, col, value).  Waits on the mbarrier give up after a
// fixed number of polls, set an error flag and skip the rest of the tile (TMEM is still freed).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pt {
namespace tc {

constexpr int kTileM = 128;
constexpr int kChunkK = 64;
constexpr int kThreads = 128;
constexpr int kWaitPolls = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (tcgen05 format: start, LBO, SBO in 16-byte units, version 1,
// no swizzle)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, M = 128, N
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

// byte offset of element (r, k) of a chunk tile (k < 64) in the core-matrix layout
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
    return (uint32_t)((r >> 3) * 1024 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// bounded wait for the given phase parity; returns false when the poll budget ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (int it = 0; it < kWaitPolls; it++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.u32 %0, 1, 0, P;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 8 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = __uint_as_float(r[j]);
}

__host__ __device__ constexpr uint32_t tmem_cols(int n) {
    return n <= 32 ? 32u : n <= 64 ? 64u : n <= 128 ? 128u : 256u;
}

// Dynamic shared memory: two stages of [A tile (128 x 64 BF16 = 16 KB) | B tile (N x 64 BF16)] |
// two mbarriers | tmem addr | 16 KB of slack, so that every core-matrix offset a descriptor can
// form from the tile bases stays inside the allocation.  Each stage starts on a 1024-byte boundary
// (N is a multiple of 16).
__host__ __device__ constexpr size_t stage_bytes(int n) { return 16384 + (size_t)n * 128; }
__host__ __device__ constexpr size_t smem_bytes(int n) { return 2 * stage_bytes(n) + 64 + 16384; }

constexpr int kGatherElem = 0, kGatherRow = 1, kGatherCol = 2;

// 8 x 8 transpose of 16-bit values among the 8 lanes of an aligned lane group: lane j holds
// column j (v = M[0..7][j], two values per word) on entry and row j (M[j][0..7]) on return
// (butterfly stages exchanging 4-, 2- and 1-element blocks with lanes j^4, j^2, j^1)
__device__ __forceinline__ uint4 transpose8(uint4 v, int j) {
    uint32_t w0 = v.x, w1 = v.y, w2 = v.z, w3 = v.w;
    {
        const bool b = j & 4;
        const uint32_t r0 = __shfl_xor_sync(0xffffffffu, b ? w0 : w2, 4);
        const uint32_t r1 = __shfl_xor_sync(0xffffffffu, b ? w1 : w3, 4);
        if (b) { w0 = r0; w1 = r1; } else { w2 = r0; w3 = r1; }
    }
    {
        const bool b = j & 2;
        const uint32_t r0 = __shfl_xor_sync(0xffffffffu, b ? w0 : w1, 2);
        const uint32_t r1 = __shfl_xor_sync(0xffffffffu, b ? w2 : w3, 2);
        if (b) { w0 = r0; w2 = r1; } else { w1 = r0; w3 = r1; }
    }
    {
        const bool b = j & 1;
        const uint32_t s0 = b ? __byte_perm(w0, w1, 0x5410) : __byte_perm(w0, w1, 0x7632);
        const uint32_t s1 = b ? __byte_perm(w2, w3, 0x5410) : __byte_perm(w2, w3, 0x7632);
        const uint32_t r0 = __shfl_xor_sync(0xffffffffu, s0, 1);
        const uint32_t r1 = __shfl_xor_sync(0xffffffffu, s1, 1);
        if (b) {
            w0 = __byte_perm(w0, r0, 0x3254); w1 = __byte_perm(w1, r0, 0x3276);
            w2 = __byte_perm(w2, r1, 0x3254); w3 = __byte_perm(w3, r1, 0x3276);
        } else {
            w0 = __byte_perm(w0, r0, 0x5410); w1 = __byte_perm(w1, r0, 0x7610);
            w2 = __byte_perm(w2, r1, 0x5410); w3 = __byte_perm(w3, r1, 0x7610);
        }
    }
    return make_uint4(w0, w1, w2, w3);
}

template <class P>
__device__ __forceinline__ void gather_chunk(const P& prob, unsigned char* sa, unsigned char* sb, int m0, int col0,
                                             int n, int k0, int tid) {
    if constexpr (P::kGather == kGatherCol) {
        // core matrix cm = (row block cm / 8, K group cm % 8): 4 per warp at a time, 8 lanes each
        const int lane = tid & 31, j = lane & 7, g = (tid >> 3);
        for (int cm = g; cm < (kTileM / 8) * (kChunkK / 8); cm += kThreads / 8) {
            const int rb = cm >> 3, kg = cm & 7;
            const uint4 v = transpose8(prob.gather_col_a(m0 + rb * 8, k0 + kg * 8 + j), j);
            *reinterpret_cast<uint4*>(sa + tile_off(rb * 8 + j, kg * 8)) = v;
        }
        for (int cm = g; cm < (n / 8) * (kChunkK / 8); cm += kThreads / 8) {
            const int rb = cm >> 3, kg = cm & 7;
            const uint4 v = transpose8(prob.gather_col_b(col0 + rb * 8, k0 + kg * 8 + j), j);
            *reinterpret_cast<uint4*>(sb + tile_off(rb * 8 + j, kg * 8)) = v;
        }
    } else if constexpr (P::kGather == kGatherRow) {
        for (int q = tid; q < kTileM * (kChunkK / 8); q += kThreads) {
            const int r = q % kTileM, kg = q / kTileM;
            *reinterpret_cast<uint4*>(sa + tile_off(r, kg * 8)) = prob.gather_a8(m0 + r, k0 + kg * 8);
        }
        for (int q = tid; q < n * (kChunkK / 8); q += kThreads) {
            const int r = q % n, kg = q / n;
            *reinterpret_cast<uint4*>(sb + tile_off(r, kg * 8)) = prob.gather_b8(col0 + r, k0 + kg * 8);
        }
    } else {
        for (int q = tid; q < kTileM * kChunkK; q += kThreads) {
            const int r = q / kChunkK, k = q % kChunkK;
            *reinterpret_cast<uint16_t*>(sa + tile_off(r, k)) = prob.gather_a(m0 + r, k0 + k);
        }
        for (int q = tid; q < n * kChunkK; q += kThreads) {
            const int r = q / kChunkK, k = q % kChunkK;
            *reinterpret_cast<uint16_t*>(sb + tile_off(r, k)) = prob.gather_b(col0 + r, k0 + k);
        }
    }
}

// The GEMM tile.  Problem P: int M, N, K (matrix sizes), int Ntile (columns per CTA, a multiple
// of 16 in [16, 256]), int kc_split (K chunks per CTA along grid z; 0 = all);
// uint16_t gather_a(int row, int k) const; uint16_t gather_b(int col, int k) const (zero outside
// the matrices); void store(int row, int col, int split, float v) const.
// Grid: (ceil(M/128), ceil(N/Ntile), number of K splits).
template <class P>
__global__ void __launch_bounds__(kThreads) k_tc_gemm(P prob, int* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int n = prob.Ntile, col0 = blockIdx.y * prob.Ntile;
    const size_t sbytes = stage_bytes(n);
    unsigned char* sa[2] = {smem, smem + sbytes};
    unsigned char* sb[2] = {smem + 16384, smem + sbytes + 16384};
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * sbytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * kTileM;
    const uint32_t ncols = tmem_cols(n);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
    }
    if (warp == 0) tmem_alloc(tslot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tslot;
    const uint32_t idesc = idesc_bf16(n);
    const int nall = (prob.K + kChunkK - 1) / kChunkK;
    const int per = prob.kc_split > 0 ? prob.kc_split : nall;
    const int cbeg = blockIdx.z * per, cend = min(nall, cbeg + per);
    uint32_t phase[2] = {0u, 0u};
    bool pending[2] = {false, false};
    bool ok = true;
    for (int c = cbeg; c < cend && ok; c++) {
        const int st = (c - cbeg) & 1;
        if (pending[st]) {  // the MMAs of chunk c - 2 read this stage: wait for them before overwriting
            const int timed_out = __syncthreads_or(mbar_wait(bar + st, phase[st]) ? 0 : 1);
            if (timed_out) {
                if (tid == 0) atomicOr(err, 1);
                ok = false;
                break;
            }
            phase[st] ^= 1u;
            pending[st] = false;
        }
        gather_chunk(prob, sa[st], sb[st], m0, col0, n, c * kChunkK, tid);
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_u32(sa[st]), b0 = smem_u32(sb[st]);
#pragma unroll
            for (int s = 0; s < kChunkK / 16; s++)
                mma_bf16(taddr, smem_desc(a0 + s * 256, 128, 1024), smem_desc(b0 + s * 256, 128, 1024), idesc,
                         (c > cbeg || s > 0) ? 1u : 0u);
            mma_commit(bar + st);
        }
        pending[st] = true;
    }
    // the outstanding commits, oldest first (each commit tracks every MMA issued before it)
    for (int q = 0; q < 2 && ok; q++) {
        const int st = ((cend - cbeg) + q) & 1;  // the stage of chunk cend - 2 first, then cend - 1
        if (!pending[st]) continue;
        const int timed_out = __syncthreads_or(mbar_wait(bar + st, phase[st]) ? 0 : 1);
        if (timed_out) {
            if (tid == 0) atomicOr(err, 1);
            ok = false;
        }
        phase[st] ^= 1u;
        pending[st] = false;
    }
    tc_fence_after();
    if (ok) {
        const int row = m0 + warp * 32 + (tid & 31);
        const uint32_t lane_base = taddr + ((uint32_t)(warp * 32) << 16);
        const bool empty = cbeg >= cend;  // a K split past the end: the accumulator was never written
        for (int c0 = 0; c0 < n; c0 += 8) {
            float v[8];
            tmem_ld8(lane_base + (uint32_t)c0, v);
            if (row < prob.M)
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (col0 + c0 + j < prob.N) prob.store(row, col0 + c0 + j, (int)blockIdx.z, empty ? 0.f : v[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(taddr, ncols);
}

}  // namespace tc
}  // namespace pt
