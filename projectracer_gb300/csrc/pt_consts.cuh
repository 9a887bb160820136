// pt_consts.cuh -- per-translation-unit copies of the engine constants in __constant__ memory.
#pragma once
#include "pt_internal.h"

namespace pt {
static __constant__ Consts cK;
static __constant__ LevConst cL[PT_MAXLEV];

static inline int upload_tu_consts(const Engine& E) {
    CK(cudaMemcpyToSymbol(cK, &E.K, sizeof(Consts)));
    CK(cudaMemcpyToSymbol(cL, E.L, sizeof(LevConst) * PT_MAXLEV));
    return 0;
}

__device__ __forceinline__ int mirror_idx(int i, int n) { return i < 0 ? -i : (i > n ? 2 * n - i : i); }

// x / d for a grid constant d with reciprocal inv.  When the spacings are powers of two (so are d
// and inv) the product is exact, hence equal to the correctly rounded quotient bit for bit, and
// it avoids the division, a long sequence on this part's FP64 pipe.
__device__ __forceinline__ double qdiv(double x, double d, double inv) { return cK.exact_div ? x * inv : x / d; }

static inline unsigned nblk(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }
}  // namespace pt
