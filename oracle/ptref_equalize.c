/*
 * ptref_equalize.c -- oracle (test infrastructure only): tracer equalisation, equalize_tracers
 * (ProjecTracer_Source/composition.f90:266-763), in the deterministic form the GPU library runs.
 *
 * The reference draws its shuffles and its lottery order from mzran streams, one per OpenMP thread,
 * over a thread partition of the grid, so its result depends on the thread count.  Here every
 * random choice is a counter-based hash of (seed, call, what is drawn), which both the GPU and this
 * restatement evaluate identically:
 *   key(tag, a, b) = mix(mix(mix(seed ^ tag << 56) ^ a) ^ b), mix = the SplitMix64 finaliser;
 *   uniform(h) = (h >> 11) 2^-53.
 *
 * The steps, with the reference lines they follow:
 *  1. nodes and counts (1127-1176, 1220): each tracer's node is (nint(r/dr), nint(s/ds)); per node
 *     the tracers of type 0 and 1 (comp=0: all type 0); nempty = their sum.  Outside 0..nx x 0..nz a
 *     count is the mirror image across the wall (1184-1191); the corner ghosts are 0.
 *  2. target per type (300-321): comp=0: tpc; comp=1: tpc_type(tt) = nint(mean count of type tt
 *     over the nodes with Cnew = 0 (tt=0) or Cnew = 1 (tt=1)), 0 if there is no such node.
 *  3. excess (297-340): comp=0: nempty - tpc where nempty > 0; comp=1: nempty - tpc_type(tt) for
 *     the first tt whose count equals nempty on the whole 3x3 neighbourhood (nempty > 0), else 0.
 *     nfree = the sum of the positive excesses; no excess anywhere: nothing to do (348-355).
 *  4. donors (412-534): a node with excess e > 0 gives e of its tracers: on an edge node (i = 0
 *     or nx, or k = 0 or nz) first those within dist_r / dist_s of a wall, then the others, each
 *     group in the order of key(1, call, id) (the reference's shuffled cell list); on interior
 *     nodes all in that order.  Its excess becomes 0.  Donors of type tt are listed by node, then
 *     by that order (the reference's per-thread shuffled donor lists: which donor goes where does
 *     not change the result's physics, since a moved tracer takes a new position, type and T).
 *  5. lottery, first phase (566-662): passes until nothing moves, all minexcess are 0, or every
 *     donor is used.  At the start of a pass: tracer_count(tt) = the sum of the type counts;
 *     escape once they equal Nideal (Nideal(1) = nint(Cinit ntr), Nideal(0) = ntr - Nideal(1));
 *     minexcess(tt) = the least excess <= 0 over the nodes with Cnew = 0 / 1 (comp=0: all nodes;
 *     2147483647 for none; 0 where tpc_type(tt) = 0).  A node qualifies if its excess equals
 *     minexcess(type_save) and is negative, type_save = its majority type (ties: type 0); it
 *     draws a donor of type tt = type_save after escape, else the first type with tracer_count >
 *     Nideal.  When a type's qualifying nodes outnumber its unused donors, the nodes with the
 *     smallest key(2, call << 24 | pass, node) win (the reference: its random loop order); winners
 *     take the next donors in node order.  A winner's donor moves to (i dr + (u - 1/2) dr,
 *     k ds + (v - 1/2) ds), u = uniform(key(3, call, id)), v = uniform(key(4, call, id)), clamped
 *     to dist_r / dist_s inside the walls, takes type type_save, and the node's counts move one
 *     tracer from type tt to type_save; its excess grows by one.
 *  6. second phase (664-722): the same passes with tt = type_save, without the count update, and
 *     minexcess(1) gated on tpc_type(0) as the reference writes it.
 *  7. the moved tracers' T interpolated from Tratio (extendT + compute_derivatives + interpolate,
 *     726-737), the equalize.dat columns (739-759), then tracers_to_corners with smooth_vis = 0.
 * The random draws use the caller's tracer index (its ID), so the result does not depend on how a
 * library orders its copy of the tracers.
 */
#include "ptref.h"

#include <limits.h>
#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

static uint64_t eq_mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static uint64_t eq_key(uint64_t seed, uint64_t tag, uint64_t a, uint64_t b) {
    return eq_mix(eq_mix(eq_mix(seed ^ (tag << 56)) ^ a) ^ b);
}
static double eq_uniform(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }

typedef struct {
    uint64_t key;
    int32_t id, cls;
} eq_cand;
static int cmp_cand(const void* a, const void* b) {
    const eq_cand *x = a, *y = b;
    if (x->cls != y->cls) return x->cls < y->cls ? -1 : 1;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->id < y->id ? -1 : (x->id > y->id);
}
typedef struct {
    uint64_t key;
    int32_t node;
} eq_node;
static int cmp_node(const void* a, const void* b) {
    const eq_node *x = a, *y = b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->node < y->node ? -1 : (x->node > y->node);
}
static int cmp_int(const void* a, const void* b) {
    const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return x < y ? -1 : (x > y);
}

int ptref_equalize(ptref_state* s, int64_t call, pt_equalize_info* info) {
    if (call < 0) call = s->eq_calls;
    s->eq_calls = call + 1;
    const pt_config* c = &s->cfg;
    const int nx = s->nx, nz = s->nz, nn = (nx + 1) * (nz + 1), comp = c->comp;
    const int64_t ntr = s->ntr;
    const uint64_t seed = c->eq_seed;
    const double dist_r = c->dist_factor * s->dr, dist_s = c->dist_factor * s->ds, aspect = c->aspect;
    pt_equalize_info out;
    memset(&out, 0, sizeof out);
    if (comp && (!s->Ttype || c->Cinit < 0.0)) {
        s->status = -1;
        snprintf(s->err_msg, sizeof s->err_msg, "equalize: comp=1 needs discrete tracer types and Cinit >= 0");
        return -1;
    }
    int32_t* node = malloc(sizeof(int32_t) * (size_t)ntr);
    int32_t* cnt = calloc((size_t)2 * nn, sizeof(int32_t)); /* [type][node] */
    int32_t* nexc = calloc((size_t)nn, sizeof(int32_t));
    int32_t* start = calloc((size_t)nn + 1, sizeof(int32_t));
    int32_t* list = malloc(sizeof(int32_t) * (size_t)(ntr > 0 ? ntr : 1));
    /* 1. nodes and counts */
    for (int64_t t = 0; t < ntr; t++) {
        const int i = (int)lround(s->rtr[t] / s->dr), k = (int)lround(s->str[t] / s->ds);
        node[t] = i + (nx + 1) * k;
        const int ty = comp ? s->Ttype[t] : 0;
        cnt[(size_t)ty * nn + node[t]]++;
    }
#define NEMPTY(q) (cnt[q] + cnt[(size_t)nn + (q)])
    /* 2. targets */
    int tpc_type[2] = {0, 0};
    if (!comp) {
        tpc_type[0] = c->tpc;
    } else {
        for (int tt = 0; tt < 2; tt++) {
            const double want = tt ? 1.0 : 0.0;
            long long sum = 0, m = 0;
            for (int k = 0; k <= nz; k++)
                for (int i = 0; i <= nx; i++)
                    if (RF(s->Cnew, i, k) == want) {
                        sum += cnt[(size_t)tt * nn + i + (nx + 1) * k];
                        m++;
                    }
            tpc_type[tt] = m > 0 ? (int)lround((double)sum / (double)m) : 0;
        }
    }
    /* 3. excess */
    int64_t nfree = 0;
    int any = 0;
    for (int k = 0; k <= nz; k++)
        for (int i = 0; i <= nx; i++) {
            const int q = i + (nx + 1) * k;
            int e = 0;
            if (!comp) {
                if (NEMPTY(q) > 0) e = NEMPTY(q) - c->tpc;
            } else if (NEMPTY(q) > 0) {
                for (int tt = 0; tt < 2; tt++) {
                    int all = 1;
                    for (int dk = -1; dk <= 1 && all; dk++)
                        for (int di = -1; di <= 1 && all; di++) {
                            int ii = i + di, kk = k + dk;
                            const int outx = ii < 0 || ii > nx, outz = kk < 0 || kk > nz;
                            int ct = 0, ne = 0;
                            if (!(outx && outz)) {
                                if (ii < 0) ii = -ii;
                                if (ii > nx) ii = 2 * nx - ii;
                                if (kk < 0) kk = -kk;
                                if (kk > nz) kk = 2 * nz - kk;
                                const int qq = ii + (nx + 1) * kk;
                                ct = cnt[(size_t)tt * nn + qq];
                                ne = NEMPTY(qq);
                            }
                            if (ct != ne) all = 0;
                        }
                    if (all) {
                        e = NEMPTY(q) - tpc_type[tt];
                        break;
                    }
                }
            }
            nexc[q] = e;
            if (e > 0) nfree += e;
            if (e != 0) any = 1;
        }
    out.tpc_type[0] = tpc_type[0];
    out.tpc_type[1] = tpc_type[1];
    out.nfree = nfree;
    if (!any) goto done;
    /* 4. donors: tracers grouped by node (ascending id), ranked by (class, key, id) */
    for (int64_t t = 0; t < ntr; t++) start[node[t] + 1]++;
    for (int q = 0; q < nn; q++) start[q + 1] += start[q];
    {
        int32_t* cur = calloc((size_t)nn, sizeof(int32_t));
        for (int64_t t = 0; t < ntr; t++) list[start[node[t]] + cur[node[t]]++] = (int32_t)t;
        free(cur);
    }
    int32_t* donors[2];
    int64_t ndon[2] = {0, 0};
    donors[0] = malloc(sizeof(int32_t) * (size_t)(nfree > 0 ? nfree : 1));
    donors[1] = malloc(sizeof(int32_t) * (size_t)(nfree > 0 ? nfree : 1));
    for (int q = 0; q < nn; q++) {
        if (nexc[q] <= 0) continue;
        const int i = q % (nx + 1), k = q / (nx + 1), m = start[q + 1] - start[q];
        const int edge = i == 0 || i == nx || k == 0 || k == nz;
        eq_cand* cand = malloc(sizeof(eq_cand) * (size_t)m);
        for (int j = 0; j < m; j++) {
            const int32_t id = list[start[q] + j];
            const double r = s->rtr[id], sv = s->str[id];
            const int near = sv < dist_s || sv > 1.0 - dist_s || r < dist_r || r > aspect - dist_r;
            cand[j].key = eq_key(seed, 1, (uint64_t)call, (uint64_t)id);
            cand[j].id = id;
            cand[j].cls = (edge && near) ? 0 : 1;
        }
        qsort(cand, (size_t)m, sizeof(eq_cand), cmp_cand);
        for (int j = 0; j < nexc[q]; j++) {
            const int32_t id = cand[j].id;
            const int ty = comp ? s->Ttype[id] : 0;
            donors[ty][ndon[ty]++] = id;
        }
        free(cand);
        nexc[q] = 0;
    }
    /* 5./6. lottery */
    int64_t Nideal[2];
    if (comp) {
        Nideal[1] = (int64_t)llround(c->Cinit * (double)ntr);
        Nideal[0] = ntr - Nideal[1];
    } else {
        Nideal[0] = ntr;
        Nideal[1] = 0;
    }
    int64_t used[2] = {0, 0};
    eq_node* qn = malloc(sizeof(eq_node) * (size_t)nn);
    int32_t* win = malloc(sizeof(int32_t) * (size_t)nn);
    int32_t* tsave = malloc(sizeof(int32_t) * (size_t)nn);
    int escape = 0;
    {
        int64_t tc0 = 0, tc1 = 0;
        for (int q = 0; q < nn; q++) { tc0 += cnt[q]; tc1 += cnt[(size_t)nn + q]; }
        if (tc0 == Nideal[0] && tc1 == Nideal[1]) escape = 1;
    }
    int pass = 0;
    for (int phase = 1; phase <= 2; phase++) {
        for (;;) {
            int64_t tcount[2] = {0, 0};
            for (int q = 0; q < nn; q++) { tcount[0] += cnt[q]; tcount[1] += cnt[(size_t)nn + q]; }
            if (phase == 1 && !escape && tcount[0] == Nideal[0] && tcount[1] == Nideal[1]) escape = 1;
            int minex[2] = {0, 0};
            for (int tt = 0; tt < 2; tt++) {
                const int gate = (phase == 2 && tt == 1) ? tpc_type[0] : tpc_type[tt];
                if (tt == 1 && !comp) continue;
                if (gate <= 0) continue;
                int mn = INT_MAX;
                for (int k = 0; k <= nz; k++)
                    for (int i = 0; i <= nx; i++) {
                        const int q = i + (nx + 1) * k;
                        if (nexc[q] > 0) continue;
                        if (comp && RF(s->Cnew, i, k) != (tt ? 1.0 : 0.0)) continue;
                        if (nexc[q] < mn) mn = nexc[q];
                    }
                minex[tt] = mn;
            }
            if (minex[0] == 0 && minex[1] == 0) break;
            if (used[0] + used[1] >= nfree) break;
            int swap = 0;
            if (phase == 1 && !escape) swap = tcount[0] > Nideal[0] ? 0 : 1;
            /* qualifying nodes per donor type */
            int64_t moved_pass = 0;
            for (int tt = 0; tt < 2; tt++) {
                int nq = 0;
                for (int q = 0; q < nn; q++) {
                    const int ts = cnt[(size_t)nn + q] > cnt[q] ? 1 : 0;
                    const int td = (phase == 1 && !escape) ? swap : ts;
                    if (td != tt) continue;
                    if (nexc[q] == minex[ts] && nexc[q] < 0) {
                        qn[nq].key = eq_key(seed, 2, ((uint64_t)call << 24) | (uint64_t)pass, (uint64_t)q);
                        qn[nq].node = q;
                        tsave[q] = ts;
                        nq++;
                    }
                }
                const int64_t avail = ndon[tt] - used[tt];
                int nw = nq;
                if ((int64_t)nq > avail) {
                    qsort(qn, (size_t)nq, sizeof(eq_node), cmp_node);
                    nw = (int)avail;
                }
                for (int j = 0; j < nw; j++) win[j] = qn[j].node;
                qsort(win, (size_t)nw, sizeof(int32_t), cmp_int);
                for (int j = 0; j < nw; j++) {
                    const int q = win[j], i = q % (nx + 1), k = q / (nx + 1), ts = tsave[q];
                    const int32_t id = donors[tt][used[tt] + j];
                    double r = s->dr * (double)i, sv = s->ds * (double)k;
                    const double pr = (eq_uniform(eq_key(seed, 3, (uint64_t)call, (uint64_t)id)) - 0.5) * s->dr;
                    const double ps = (eq_uniform(eq_key(seed, 4, (uint64_t)call, (uint64_t)id)) - 0.5) * s->ds;
                    r = r + pr;
                    sv = sv + ps;
                    if (r <= 0.0) r = dist_r;
                    if (r >= aspect) r = aspect - dist_r;
                    if (sv <= 0.0) sv = dist_s;
                    if (sv >= 1.0) sv = 1.0 - dist_s;
                    s->rtr[id] = r;
                    s->str[id] = sv;
                    if (comp) s->Ttype[id] = ts;
                    if (phase == 1) {
                        cnt[(size_t)tt * nn + q]--;
                        cnt[(size_t)ts * nn + q]++;
                    }
                    nexc[q]++;
                }
                used[tt] += nw;
                moved_pass += nw;
            }
            pass++;
            if (moved_pass == 0) break;
        }
    }
    /* 7. temperatures of the moved tracers */
    ref_extendT(s, &s->Tratio);
    ref_compute_derivatives(s, &s->Textend, s->DERr_t);
    for (int tt = 0; tt < 2; tt++)
        for (int64_t j = 0; j < used[tt]; j++) {
            const int32_t id = donors[tt][j];
            s->Ttr[id] = ref_interpolate(s, s->rtr[id], s->str[id], s->DERr_t, &s->Textend);
        }
    if (comp)
        for (int64_t t = 0; t < ntr; t++) s->Ctr[t] = s->Ttype[t] ? 1.0 : 0.0;
    /* equalize.dat columns */
    for (int tt = 0; tt < 2; tt++) {
        if (tt == 1 && !comp) continue;
        int mn = INT_MAX;
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                const int q = i + (nx + 1) * k;
                if (nexc[q] > 0) continue;
                if (comp && RF(s->Cnew, i, k) != (tt ? 1.0 : 0.0)) continue;
                if (nexc[q] < mn) mn = nexc[q];
            }
        out.minexcess[tt] = mn;
    }
    for (int q = 0; q < nn; q++) {
        if (nexc[q] <= 0) out.deficit += nexc[q];
        out.count_type[0] += cnt[q];
        out.count_type[1] += cnt[(size_t)nn + q];
    }
    out.moved = used[0] + used[1];
    out.passes = pass;
    s->eq_done++;
    free(qn);
    free(win);
    free(tsave);
    free(donors[0]);
    free(donors[1]);
done:
    out.nequalize = (int32_t)s->eq_done;
    free(node);
    free(cnt);
    free(nexc);
    free(start);
    free(list);
    if (info) *info = out;
    if (!any) return 0;
    /* tracers_to_corners with smooth_vis = 0 */
    return ref_project(s, s->rtr, s->str, s->Ttr, &s->T, 0);
}
