// pt_equalize.cu -- tracer equalisation (equalize_tracers, composition.f90:266-763) on the GPU.
//
// Tracers from nodes that hold more than their type's target count are moved to the nodes that
// lack the most.  The reference draws its shuffles and lottery order from one mzran stream per
// OpenMP thread; here every random choice is a counter-based hash of (seed, call, tracer or node),
// so the result is deterministic and does not depend on the tracer order:
//   key(tag, a, b) = mix(mix(mix(seed ^ tag << 56) ^ a) ^ b) (mix: the SplitMix64 finaliser),
//   uniform(h) = (h >> 11) 2^-53;
//   tag 1: a donor's rank among its node's tracers; tag 2: a node's place in a pass's lottery;
//   tags 3, 4: a moved tracer's offsets in x and z.
// Steps (one kernel or a few per step, the host deciding between passes):
//   1. tracers grouped by nearest node (nint cell), per-node type counts (count_type, 1127-1176);
//   2. target per type tpc_type (comp=0: tpc; comp=1: the mean count over the pure nodes,
//      300-321) and each node's excess (nempty - target where the whole 3x3 neighbourhood holds one
//      type, 322-340);
//   3. donors: each rich node gives its excess, near-wall tracers of edge nodes first, otherwise in
//      key order (412-534); per type, the donors are listed by node;
//   4. lottery passes (566-722): the nodes whose excess is the least of their type's nodes (and
//      negative) each draw one donor; when a type's donors run short, the nodes with the smallest
//      keys win (an exact radix select on the 64-bit keys); winners take donors in node order; a
//      moved tracer lands at its node jittered by half a cell, with the node's majority type;
//   5. the moved tracers' temperature interpolated from Tratio (726-737), then the projection with
//      smooth_vis = 0.
// The same algorithm, restated in C, is the oracle's ptref_equalize; tests compare the two bit for
// bit.  This file is compiled without fused multiply-adds (positions are formed as in the oracle).
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "pt_consts.cuh"

namespace pt {

namespace {

struct EqState {
    int32_t *cnt0 = nullptr, *cnt1 = nullptr, *nexc = nullptr, *cand = nullptr, *win = nullptr, *widx = nullptr,
            *d0 = nullptr, *d1 = nullptr, *off0 = nullptr, *off1 = nullptr, *hist = nullptr;
    int32_t* don[2] = {nullptr, nullptr};
    int64_t dcap = 0;
    unsigned long long* acc = nullptr;  // device reduction slots
    unsigned long long* hacc = nullptr; // pinned host mirror
    int32_t* hhist = nullptr;           // pinned host histogram
};

constexpr int kEqAcc = 16;
constexpr int kEqBins = 1 << 16;

EqState& eqs(Engine& E) {
    if (!E.eq) E.eq = new EqState();
    return *static_cast<EqState*>(E.eq);
}

__device__ __host__ __forceinline__ uint64_t eq_mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __host__ __forceinline__ uint64_t eq_key(uint64_t seed, uint64_t tag, uint64_t a, uint64_t b) {
    return eq_mix(eq_mix(eq_mix(seed ^ (tag << 56)) ^ a) ^ b);
}
__device__ __forceinline__ double eq_uniform(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }

// warp-aggregated 64-bit atomic add
__device__ __forceinline__ void warp_add(unsigned long long* a, long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(a, (unsigned long long)v);
}

}  // namespace

// per node: tracers of type 1 (C = 1.0) and type 0 among the node's list
__global__ void k_eq_node_counts(const int32_t* __restrict__ clist, const int32_t* __restrict__ cstart,
                                 const int32_t* __restrict__ ccount, const double* __restrict__ Ct, int comp,
                                 int32_t* __restrict__ cnt0, int32_t* __restrict__ cnt1, int nn) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nn) return;
    const int m = ccount[q], b = cstart[q];
    int c1 = 0;
    if (comp)
        for (int j = 0; j < m; j++) c1 += Ct[clist[b + j]] != 0.0;
    cnt1[q] = c1;
    cnt0[q] = m - c1;
}

// sums of the type counts over the pure nodes: acc[0..3] = sum cnt0 | #(C=0) | sum cnt1 | #(C=1)
__global__ void k_eq_tpc(const double* __restrict__ Cnew, Geo g, const int32_t* __restrict__ cnt0,
                         const int32_t* __restrict__ cnt1, int nx, int nz, unsigned long long* acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int nn = (nx + 1) * (nz + 1);
    long long a0 = 0, m0 = 0, a1 = 0, m1 = 0;
    if (q < nn) {
        const double c = Cnew[g.at(q % (nx + 1), q / (nx + 1))];
        if (c == 0.0) { a0 = cnt0[q]; m0 = 1; }
        if (c == 1.0) { a1 = cnt1[q]; m1 = 1; }
    }
    warp_add(acc + 0, a0);
    warp_add(acc + 1, m0);
    warp_add(acc + 2, a1);
    warp_add(acc + 3, m1);
}

// count of type tt at (i, k) with the mirrored ghosts of the projection; corner ghosts 0
__device__ __forceinline__ void eq_counts_at(const int32_t* cnt0, const int32_t* cnt1, int nx, int nz, int i, int k,
                                             int& c0, int& c1) {
    const bool outx = i < 0 || i > nx, outz = k < 0 || k > nz;
    if (outx && outz) { c0 = 0; c1 = 0; return; }
    if (i < 0) i = -i;
    if (i > nx) i = 2 * nx - i;
    if (k < 0) k = -k;
    if (k > nz) k = 2 * nz - k;
    const int q = i + (nx + 1) * k;
    c0 = cnt0[q];
    c1 = cnt1[q];
}

// excess per node; acc[4] += positive excess, acc[5] += #(excess != 0)
__global__ void k_eq_excess(const int32_t* __restrict__ cnt0, const int32_t* __restrict__ cnt1,
                            int32_t* __restrict__ nexc, int nx, int nz, int comp, int tpc, int tpc0, int tpc1,
                            unsigned long long* acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int nn = (nx + 1) * (nz + 1);
    int e = 0;
    if (q < nn) {
        const int i = q % (nx + 1), k = q / (nx + 1);
        const int ne = cnt0[q] + cnt1[q];
        if (!comp) {
            if (ne > 0) e = ne - tpc;
        } else if (ne > 0) {
            for (int tt = 0; tt < 2; tt++) {
                bool all = true;
                for (int dk = -1; dk <= 1 && all; dk++)
                    for (int di = -1; di <= 1 && all; di++) {
                        int c0, c1;
                        eq_counts_at(cnt0, cnt1, nx, nz, i + di, k + dk, c0, c1);
                        if ((tt ? c1 : c0) != c0 + c1) all = false;
                    }
                if (all) {
                    e = ne - (tt ? tpc1 : tpc0);
                    break;
                }
            }
        }
        nexc[q] = e;
    }
    warp_add(acc + 4, e > 0 ? e : 0);
    warp_add(acc + 5, e != 0 ? 1 : 0);
}

// donations per node and type (a rich node's tracers are all of one type); acc[6], acc[7] totals;
// acc[15] = the most tracers on one rich node (the donor ranking costs tracers x donors per node)
__global__ void k_eq_donations(const int32_t* __restrict__ nexc, const int32_t* __restrict__ cnt0,
                               const int32_t* __restrict__ cnt1, int32_t* __restrict__ d0,
                               int32_t* __restrict__ d1, int nn, unsigned long long* acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    int a = 0, b = 0;
    unsigned long long m = 0;
    if (q < nn) {
        const int e = nexc[q] > 0 ? nexc[q] : 0;
        if (cnt1[q] > 0) b = e;
        else a = e;
        d0[q] = a;
        d1[q] = b;
        if (e > 0) m = (unsigned long long)(cnt0[q] + cnt1[q]);
    }
    warp_add(acc + 6, a);
    warp_add(acc + 7, b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(acc + 15, m);
}

// a rich node holding more tracers than this is refused (its donor ranking would take seconds)
constexpr int kEqMaxNode = 8192;

// a rich node's donors: its nexc tracers of smallest (near-wall class, key(1, call, id), id), in
// that order, into the donor list of their type at the node's offset; its excess becomes 0
__global__ void k_eq_donors(const int32_t* __restrict__ clist, const int32_t* __restrict__ cstart,
                            const int32_t* __restrict__ ccount, int32_t* __restrict__ nexc,
                            const int32_t* __restrict__ cnt1, const int32_t* __restrict__ off0,
                            const int32_t* __restrict__ off1, int32_t* __restrict__ don0, int32_t* __restrict__ don1,
                            const double* __restrict__ r, const double* __restrict__ s,
                            const int32_t* __restrict__ perm, int nx, int nz, double dist_r, double dist_s,
                            double aspect, uint64_t seed, uint64_t call) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (nx + 1) * (nz + 1)) return;
    const int e = nexc[q];
    if (e <= 0) return;
    const int i = q % (nx + 1), k = q / (nx + 1);
    const bool edge = i == 0 || i == nx || k == 0 || k == nz;
    const int m = ccount[q], b = cstart[q];
    int32_t* out = cnt1[q] > 0 ? don1 + off1[q] : don0 + off0[q];
    // selection in increasing (class, key, id): each round takes the least triple above the last
    int lc = -1;
    uint64_t lk = 0;
    long long lid = -1;
    for (int j = 0; j < e && j < m; j++) {
        int bc = 2, bp = -1;
        uint64_t bk = 0;
        long long bid = 0;
        for (int t = 0; t < m; t++) {
            const int32_t p = clist[b + t];
            const long long id = perm ? (long long)perm[p] : (long long)p;
            const double rr = r[p], ss = s[p];
            const bool near = ss < dist_s || ss > 1.0 - dist_s || rr < dist_r || rr > aspect - dist_r;
            const int cl = (edge && near) ? 0 : 1;
            const uint64_t ky = eq_key(seed, 1, call, (uint64_t)id);
            const bool above = cl > lc || (cl == lc && (ky > lk || (ky == lk && id > lid)));
            const bool less = cl < bc || (cl == bc && (ky < bk || (ky == bk && id < bid)));
            if (above && (bp < 0 || less)) {
                bc = cl; bk = ky; bid = id; bp = p;
            }
        }
        out[j] = bp;
        lc = bc; lk = bk; lid = bid;
    }
    nexc[q] = 0;
}

// the pass's reductions: acc[8], acc[9] = sum cnt0, sum cnt1; acc[10], acc[11] = least excess
// <= 0 over the nodes of type 0 / 1 (C = 0 / 1; comp=0: every node, type 0); stored as
// excess + 2^31 so that an unsigned minimum orders them
__device__ __forceinline__ void eq_pass_reduce(const int32_t* __restrict__ cnt0, const int32_t* __restrict__ cnt1,
                                               const int32_t* __restrict__ nexc, const double* __restrict__ Cnew,
                                               Geo g, int nx, int nz, int comp, unsigned long long* acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int nn = (nx + 1) * (nz + 1);
    long long a0 = 0, a1 = 0;
    unsigned long long m0 = ULLONG_MAX, m1 = ULLONG_MAX;
    if (q < nn) {
        a0 = cnt0[q];
        a1 = cnt1[q];
        const int e = nexc[q];
        if (e <= 0) {
            const unsigned long long v = (unsigned long long)((long long)e + 2147483648LL);
            if (!comp) {
                m0 = v;
            } else {
                const double c = Cnew[g.at(q % (nx + 1), q / (nx + 1))];
                if (c == 0.0) m0 = v;
                if (c == 1.0) m1 = v;
            }
        }
    }
    warp_add(acc + 8, a0);
    warp_add(acc + 9, a1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m0 = min(m0, __shfl_down_sync(0xffffffffu, m0, o));
        m1 = min(m1, __shfl_down_sync(0xffffffffu, m1, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (m0 != ULLONG_MAX) atomicMin(acc + 10, m0);
        if (m1 != ULLONG_MAX) atomicMin(acc + 11, m1);
    }
}
__global__ void k_eq_pass_reduce(const int32_t* __restrict__ cnt0, const int32_t* __restrict__ cnt1,
                                 const int32_t* __restrict__ nexc, const double* __restrict__ Cnew, Geo g, int nx,
                                 int nz, int comp, unsigned long long* acc) {
    eq_pass_reduce(cnt0, cnt1, nexc, Cnew, g, nx, nz, comp, acc);
}

// the pass's candidates: cand[q] = 1 + donor type of a qualifying node, else 0; acc[12 + tt]
// counts them.  td = -1: each node draws its majority type, else every node draws type td.
__global__ void k_eq_qualify(const int32_t* __restrict__ cnt0, const int32_t* __restrict__ cnt1,
                             const int32_t* __restrict__ nexc, int32_t* __restrict__ cand, int nn, int minex0,
                             int minex1, int td, unsigned long long* acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    int c = 0;
    if (q < nn) {
        const int ts = cnt1[q] > cnt0[q] ? 1 : 0;
        const int e = nexc[q];
        if (e < 0 && e == (ts ? minex1 : minex0)) c = 1 + (td < 0 ? ts : td);
        cand[q] = c;
    }
    warp_add(acc + 12, c == 1 ? 1 : 0);
    warp_add(acc + 13, c == 2 ? 1 : 0);
}

// histogram of the 16-bit digit at `shift` of the lottery keys of type-tt candidates whose higher
// digits equal `prefix`
__global__ void k_eq_hist(const int32_t* __restrict__ cand, int nn, int tt, uint64_t seed, uint64_t a,
                          uint64_t prefix, int shift, int32_t* __restrict__ hist) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nn || cand[q] != 1 + tt) return;
    const uint64_t key = eq_key(seed, 2, a, (uint64_t)q);
    if (shift < 48 && (key >> (shift + 16)) != prefix) return;
    atomicAdd(&hist[(key >> shift) & 0xFFFFu], 1);
}

// winners of type tt: all candidates (all = 1), or those with key < kstar plus the key == kstar
// ties (win = 2, thinned by the caller when more tie than are needed)
__global__ void k_eq_win(const int32_t* __restrict__ cand, int32_t* __restrict__ win, int nn, int tt, int all,
                         uint64_t seed, uint64_t a, uint64_t kstar, unsigned long long* acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    int w = 0;
    if (q < nn && cand[q] == 1 + tt) {
        if (all) {
            w = 1;
        } else {
            const uint64_t key = eq_key(seed, 2, a, (uint64_t)q);
            w = key < kstar ? 1 : (key == kstar ? 2 : 0);
        }
    }
    if (q < nn) win[q] = w;
    warp_add(acc + 14, w == 2 ? 1 : 0);
}
// keep the first `need` ties (node order; tidx = exclusive scan of the tie flags)
__global__ void k_eq_thin_ties(int32_t* __restrict__ win, const int32_t* __restrict__ tidx, int nn, int need) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nn) return;
    if (win[q] == 2) win[q] = tidx[q] < need ? 1 : 0;
}
__global__ void k_eq_flags(const int32_t* __restrict__ win, int32_t* __restrict__ out, int nn, int value) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nn) out[q] = win[q] == value ? 1 : 0;
}

// each winner (in node order, widx = its rank) takes donor don[used + widx]: new position at the
// node jittered by up to half a cell, clamped inside the walls; type = the node's majority type;
// first phase: the node's counts move one tracer from the donor type to that type; excess + 1
__global__ void k_eq_assign(const int32_t* __restrict__ win, const int32_t* __restrict__ widx,
                            const int32_t* __restrict__ don, int64_t used, int tt, int phase,
                            int32_t* __restrict__ cnt0, int32_t* __restrict__ cnt1, int32_t* __restrict__ nexc,
                            double* __restrict__ r, double* __restrict__ s, double* __restrict__ Ct,
                            const int32_t* __restrict__ perm, int nx, int nz, int comp, double dr, double ds,
                            double dist_r, double dist_s, double aspect, uint64_t seed, uint64_t call) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (nx + 1) * (nz + 1) || win[q] != 1) return;
    const int i = q % (nx + 1), k = q / (nx + 1);
    const int ts = cnt1[q] > cnt0[q] ? 1 : 0;
    const int32_t p = don[used + widx[q]];
    const uint64_t id = perm ? (uint64_t)perm[p] : (uint64_t)p;
    double rr = dr * (double)i, ss = ds * (double)k;
    const double pr = (eq_uniform(eq_key(seed, 3, call, id)) - 0.5) * dr;
    const double ps = (eq_uniform(eq_key(seed, 4, call, id)) - 0.5) * ds;
    rr = rr + pr;
    ss = ss + ps;
    if (rr <= 0.0) rr = dist_r;
    if (rr >= aspect) rr = aspect - dist_r;
    if (ss <= 0.0) ss = dist_s;
    if (ss >= 1.0) ss = 1.0 - dist_s;
    r[p] = rr;
    s[p] = ss;
    if (comp) Ct[p] = ts ? 1.0 : 0.0;
    if (phase == 1) {
        if (tt) cnt1[q]--;
        else cnt0[q]--;
        if (ts) cnt1[q]++;
        else cnt0[q]++;
    }
    nexc[q]++;
}

// after the moves: acc[0], acc[1] = sum cnt0, sum cnt1; acc[2] = sum of the excesses <= 0 (as a
// signed value); acc[10], acc[11] = least excess <= 0 per type (+2^31)
__global__ void k_eq_final(const int32_t* __restrict__ cnt0, const int32_t* __restrict__ cnt1,
                           const int32_t* __restrict__ nexc, const double* __restrict__ Cnew, Geo g, int nx, int nz,
                           int comp, unsigned long long* acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int nn = (nx + 1) * (nz + 1);
    long long d = 0;
    if (q < nn && nexc[q] <= 0) d = nexc[q];
    warp_add(acc + 2, d);
    eq_pass_reduce(cnt0, cnt1, nexc, Cnew, g, nx, nz, comp, acc);
}

static int eq_alloc(Engine& E, EqState& S) {
    if (S.cnt0) return 0;
    const size_t nn = (size_t)(E.K.nx + 1) * (size_t)(E.K.nz + 1);
    int32_t** a[] = {&S.cnt0, &S.cnt1, &S.nexc, &S.cand, &S.win, &S.widx, &S.d0, &S.d1, &S.off0, &S.off1};
    for (auto p : a) {
        CK(cudaMalloc(p, nn * sizeof(int32_t)));
        E.bytes_allocated += nn * sizeof(int32_t);
    }
    CK(cudaMalloc(&S.hist, kEqBins * sizeof(int32_t)));
    CK(cudaMalloc(&S.acc, kEqAcc * sizeof(unsigned long long)));
    CK(cudaMallocHost(&S.hacc, kEqAcc * sizeof(unsigned long long)));
    CK(cudaMallocHost(&S.hhist, kEqBins * sizeof(int32_t)));
    return 0;
}

void equalize_free(Engine& E) {
    if (!E.eq) return;
    EqState& S = eqs(E);
    for (int32_t* p : {S.cnt0, S.cnt1, S.nexc, S.cand, S.win, S.widx, S.d0, S.d1, S.off0, S.off1, S.hist, S.don[0], S.don[1]})
        if (p) cudaFree(p);
    if (S.acc) cudaFree(S.acc);
    if (S.hacc) cudaFreeHost(S.hacc);
    if (S.hhist) cudaFreeHost(S.hhist);
    delete &S;
    E.eq = nullptr;
}

// device reduction slots -> host (after the work queued so far)
static int read_acc(Engine& E, EqState& S) {
    CK(cudaMemcpyAsync(S.hacc, S.acc, kEqAcc * sizeof(unsigned long long), cudaMemcpyDeviceToHost, E.st));
    CK(cudaStreamSynchronize(E.st));
    return 0;
}
static int reset_acc(Engine& E, EqState& S) {
    CK(cudaMemsetAsync(S.acc, 0, kEqAcc * sizeof(unsigned long long), E.st));
    // the two minimum slots start at the largest value
    static const unsigned long long big[2] = {ULLONG_MAX, ULLONG_MAX};
    CK(cudaMemcpyAsync(S.acc + 10, big, sizeof big, cudaMemcpyHostToDevice, E.st));
    return 0;
}

int equalize_tracers(Engine& E, pt_equalize_info* info) {
    EqState& S = eqs(E);
    if (int rc = eq_alloc(E, S)) return rc;
    const int nx = E.K.nx, nz = E.K.nz, nn = (nx + 1) * (nz + 1), comp = E.cfg.comp;
    const int64_t ntr = E.ntr;
    const uint64_t seed = E.cfg.eq_seed, call = (uint64_t)E.eq_calls++;
    const double dr = E.K.dr, ds = E.K.ds, aspect = E.K.aspect;
    const double dist_r = E.cfg.dist_factor * dr, dist_s = E.cfg.dist_factor * ds;
    const int32_t* perm = E.perm_active ? E.perm : nullptr;
    const unsigned nb = (unsigned)nblk(nn, 256);
    pt_equalize_info out;
    std::memset(&out, 0, sizeof out);
    int rc;
    if (comp && E.eq_Cinit < 0.0) {  // Cinit = Cavg of the state (basics.f90:461)
        if (E.cfg.Cinit >= 0.0) {
            E.eq_Cinit = E.cfg.Cinit;
        } else {
            pt_stats_row row;
            if ((rc = stats(E, &row))) return rc;
            E.eq_Cinit = row.Cavg;
        }
    }
    // 1. nodes and type counts
    if ((rc = sort_tracers_by_node(E, E.rtr, E.str))) return rc;
    PT_COUNT(), k_eq_node_counts<<<nb, 256, 0, E.st>>>(E.clist, E.cstart, E.ccount, E.Ctr, comp, S.cnt0, S.cnt1, nn);
    // 2. targets and excess
    if ((rc = reset_acc(E, S))) return rc;
    int tpc[2] = {E.cfg.tpc, 0};
    if (comp) {
        PT_COUNT(), k_eq_tpc<<<nb, 256, 0, E.st>>>(E.Cnew, E.g1, S.cnt0, S.cnt1, nx, nz, S.acc);
        if ((rc = read_acc(E, S))) return rc;
        for (int tt = 0; tt < 2; tt++) {
            const long long sum = (long long)S.hacc[2 * tt], m = (long long)S.hacc[2 * tt + 1];
            tpc[tt] = m > 0 ? (int)std::llround((double)sum / (double)m) : 0;
        }
    }
    PT_COUNT(), k_eq_excess<<<nb, 256, 0, E.st>>>(S.cnt0, S.cnt1, S.nexc, nx, nz, comp, E.cfg.tpc, tpc[0], tpc[1],
                                                  S.acc);
    if ((rc = read_acc(E, S))) return rc;
    const int64_t nfree = (int64_t)S.hacc[4];
    const bool any = S.hacc[5] != 0;
    out.tpc_type[0] = tpc[0];
    out.tpc_type[1] = tpc[1];
    out.nfree = nfree;
    if (!any) {
        out.nequalize = E.eq_done;
        if (info) *info = out;
        return 0;
    }
    E.eq_done++;
    // 3. donors
    PT_COUNT(), k_eq_donations<<<nb, 256, 0, E.st>>>(S.nexc, S.cnt0, S.cnt1, S.d0, S.d1, nn, S.acc);
    if ((rc = exclusive_scan_i32(E, S.d0, S.off0, nn)) || (rc = exclusive_scan_i32(E, S.d1, S.off1, nn))) return rc;
    if ((rc = read_acc(E, S))) return rc;
    if (S.hacc[15] > (unsigned long long)kEqMaxNode)
        return fail(PT_ERR_ARG, "tracer equalisation: a node holds more than 8192 tracers");
    const int64_t ndon[2] = {(int64_t)S.hacc[6], (int64_t)S.hacc[7]};
    const int64_t need_cap = ndon[0] > ndon[1] ? ndon[0] : ndon[1];
    if (need_cap > S.dcap) {
        for (int t = 0; t < 2; t++) {
            if (S.don[t]) cudaFree(S.don[t]);
            S.don[t] = nullptr;
            CK(cudaMalloc(&S.don[t], (size_t)need_cap * sizeof(int32_t)));
        }
        S.dcap = need_cap;
    }
    PT_COUNT(), k_eq_donors<<<nblk(nn, 128), 128, 0, E.st>>>(E.clist, E.cstart, E.ccount, S.nexc, S.cnt1, S.off0, S.off1, S.don[0],
                                                  S.don[1], E.rtr, E.str, perm, nx, nz, dist_r, dist_s, aspect, seed,
                                                  call);
    CKL("equalize donors");
    // 4. lottery
    int64_t Nideal[2] = {ntr, 0};
    if (comp) {
        Nideal[1] = (int64_t)std::llround(E.eq_Cinit * (double)ntr);
        Nideal[0] = ntr - Nideal[1];
    }
    int64_t used[2] = {0, 0};
    bool escape = false;
    int pass = 0;
    for (int phase = 1; phase <= 2; phase++) {
        for (int guard = 0; guard < 4 * (nx + nz + 64) + 1000000; guard++) {
            if ((rc = reset_acc(E, S))) return rc;
            PT_COUNT(), k_eq_pass_reduce<<<nb, 256, 0, E.st>>>(S.cnt0, S.cnt1, S.nexc, E.Cnew, E.g1, nx, nz, comp, S.acc);
            if ((rc = read_acc(E, S))) return rc;
            const int64_t tcount[2] = {(int64_t)S.hacc[8], (int64_t)S.hacc[9]};
            if (!escape && tcount[0] == Nideal[0] && tcount[1] == Nideal[1]) escape = true;
            int minex[2] = {0, 0};
            for (int tt = 0; tt < 2; tt++) {
                if (tt == 1 && !comp) continue;
                const int gate = (phase == 2 && tt == 1) ? tpc[0] : tpc[tt];
                if (gate <= 0) continue;
                const unsigned long long v = S.hacc[10 + tt];
                minex[tt] = v == ULLONG_MAX ? INT_MAX : (int)((long long)v - 2147483648LL);
            }
            if (minex[0] == 0 && minex[1] == 0) break;
            if (used[0] + used[1] >= nfree) break;
            // escape is decided at the first pass of the first phase too (before the loop in the
            // reference); the second phase always draws the node's own type
            const int td = (phase == 2 || escape) ? -1 : (tcount[0] > Nideal[0] ? 0 : 1);
            if ((rc = reset_acc(E, S))) return rc;
            PT_COUNT(), k_eq_qualify<<<nb, 256, 0, E.st>>>(S.cnt0, S.cnt1, S.nexc, S.cand, nn, minex[0], minex[1], td,
                                                          S.acc);
            if ((rc = read_acc(E, S))) return rc;
            const int64_t ncand[2] = {(int64_t)S.hacc[12], (int64_t)S.hacc[13]};
            const uint64_t a = (call << 24) | (uint64_t)pass;
            int64_t moved = 0;
            for (int tt = 0; tt < 2; tt++) {
                if (ncand[tt] == 0) continue;
                const int64_t avail = ndon[tt] - used[tt];
                if (avail <= 0) continue;
                int64_t nwin = ncand[tt];
                if (ncand[tt] > avail) {
                    // exact select of the `avail` smallest (key, node): 16-bit digits from the top
                    uint64_t prefix = 0;
                    int64_t rank = avail;  // still to take among the keys matching prefix
                    for (int shift = 48; shift >= 0; shift -= 16) {
                        CK(cudaMemsetAsync(S.hist, 0, kEqBins * sizeof(int32_t), E.st));
                        PT_COUNT(), k_eq_hist<<<nb, 256, 0, E.st>>>(S.cand, nn, tt, seed, a, prefix, shift, S.hist);
                        CK(cudaMemcpyAsync(S.hhist, S.hist, kEqBins * sizeof(int32_t), cudaMemcpyDeviceToHost, E.st));
                        CK(cudaStreamSynchronize(E.st));
                        int64_t below = 0;
                        int d = 0;
                        for (; d < kEqBins; d++) {
                            if (below + S.hhist[d] >= rank) break;
                            below += S.hhist[d];
                        }
                        if (d >= kEqBins) return fail(PT_ERR_CUDA, "equalize: lottery selection out of range");
                        rank -= below;
                        prefix = (prefix << 16) | (uint64_t)d;
                    }
                    if ((rc = reset_acc(E, S))) return rc;
                    PT_COUNT(), k_eq_win<<<nb, 256, 0, E.st>>>(S.cand, S.win, nn, tt, 0, seed, a, prefix, S.acc);
                    if ((rc = read_acc(E, S))) return rc;
                    if ((int64_t)S.hacc[14] > rank) {  // more ties at the threshold key than needed
                        PT_COUNT(), k_eq_flags<<<nb, 256, 0, E.st>>>(S.win, S.d0, nn, 2);
                        if ((rc = exclusive_scan_i32(E, S.d0, S.widx, nn))) return rc;
                        PT_COUNT(), k_eq_thin_ties<<<nb, 256, 0, E.st>>>(S.win, S.widx, nn, (int)rank);
                    } else {
                        PT_COUNT(), k_eq_thin_ties<<<nb, 256, 0, E.st>>>(S.win, S.widx, nn, INT_MAX);
                    }
                    nwin = avail;
                } else {
                    PT_COUNT(), k_eq_win<<<nb, 256, 0, E.st>>>(S.cand, S.win, nn, tt, 1, seed, a, 0, S.acc);
                }
                PT_COUNT(), k_eq_flags<<<nb, 256, 0, E.st>>>(S.win, S.d1, nn, 1);
                if ((rc = exclusive_scan_i32(E, S.d1, S.widx, nn))) return rc;
                PT_COUNT(), k_eq_assign<<<nb, 256, 0, E.st>>>(S.win, S.widx, S.don[tt], used[tt], tt, phase, S.cnt0, S.cnt1,
                                                             S.nexc, E.rtr, E.str, E.Ctr, perm, nx, nz, comp, dr, ds,
                                                             dist_r, dist_s, aspect, seed, call);
                CKL("equalize lottery");
                used[tt] += nwin;
                moved += nwin;
            }
            pass++;
            if (moved == 0) break;
        }
    }
    // 5. temperatures of the moved tracers, the equalize.dat columns, the projection
    for (int tt = 0; tt < 2; tt++)
        if ((rc = interp_T_at(E, S.don[tt], used[tt]))) return rc;
    if ((rc = reset_acc(E, S))) return rc;
    PT_COUNT(), k_eq_final<<<nb, 256, 0, E.st>>>(S.cnt0, S.cnt1, S.nexc, E.Cnew, E.g1, nx, nz, comp, S.acc);
    if ((rc = read_acc(E, S))) return rc;
    out.count_type[0] = (int64_t)S.hacc[8];
    out.count_type[1] = (int64_t)S.hacc[9];
    out.deficit = (int64_t)(long long)S.hacc[2];
    for (int tt = 0; tt < 2; tt++) {
        if (tt == 1 && !comp) continue;
        const unsigned long long v = S.hacc[10 + tt];
        out.minexcess[tt] = v == ULLONG_MAX ? INT_MAX : (int)((long long)v - 2147483648LL);
    }
    out.moved = used[0] + used[1];
    out.passes = pass;
    out.nequalize = E.eq_done;
    if (info) *info = out;
    return project(E, E.rtr, E.str, E.Ttr, E.T, 0);
}

}  // namespace pt
