/*
 * CPU oracle for HiQ's greedy gate clustering ("greedy fusion k <= K").
 *
 * TEST INFRASTRUCTURE ONLY (see sv_oracle.c). Restates the reference
 * ClusterScheduler (src/scheduler/cluster_scheduler.h:25-162,
 * src/scheduler/cluster_scheduler.cpp:23-99, src/scheduler/convertors.cpp:34-89)
 * driven the way GreedyScheduler drives it
 * (hiq/projectq/cengines/_greedyscheduler.py:119-137, with every gate treated
 * as non-diagonal per _greedyscheduler.py:28): repeatedly pick the cluster of
 * at most K local qubits that lets the most gates run in order, emit those
 * gates, flush, drop them, and repeat. Pinned against the reference
 * _sched_cpp module in tests/test_oracle_pin.py.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef uint64_t msk_t;

typedef struct {
    msk_t* keys;
    msk_t* vals;
    uint8_t* used;
    size_t cap, count;
} umap; /* open-addressing map msk -> msk, absent == 0 */

static size_t h64(msk_t k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdULL; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ULL; k ^= k >> 33;
    return (size_t)k;
}
static void umap_init(umap* m, size_t cap) {
    m->cap = cap;
    m->count = 0;
    m->keys = (msk_t*)calloc(cap, sizeof(msk_t));
    m->vals = (msk_t*)calloc(cap, sizeof(msk_t));
    m->used = (uint8_t*)calloc(cap, 1);
}
static void umap_free(umap* m) { free(m->keys); free(m->vals); free(m->used); }
static msk_t* umap_ref(umap* m, msk_t k);
static void umap_grow(umap* m) {
    umap n;
    umap_init(&n, m->cap * 2);
    for (size_t i = 0; i < m->cap; ++i)
        if (m->used[i]) *umap_ref(&n, m->keys[i]) = m->vals[i];
    umap_free(m);
    *m = n;
}
/* Inserts 0 when absent, like std::map::operator[]. The returned pointer stays
 * valid until the next umap_ref call (which may grow the table). */
static msk_t* umap_ref(umap* m, msk_t k) {
    if (2 * (m->count + 1) > m->cap) umap_grow(m);
    size_t i = h64(k) & (m->cap - 1);
    while (m->used[i]) {
        if (m->keys[i] == k) return &m->vals[i];
        i = (i + 1) & (m->cap - 1);
    }
    m->used[i] = 1; m->keys[i] = k; m->vals[i] = 0;
    ++m->count;
    return &m->vals[i];
}

typedef struct {
    int K, ngates;
    const msk_t* gate; const msk_t* ctrl;
    msk_t locals, all;
    int best_ans; msk_t best;
    umap used;
} sched;

static int can_take(const sched* s, int i, msk_t cluster, msk_t bad) {
    msk_t ga = s->gate[i] | s->ctrl[i];
    if ((ga & bad) || ((ga & s->locals) & ~cluster)) return 0;
    return (s->gate[i] & ~s->locals) == 0; /* non-diagonal gate: targets must be local */
}

static void calc_combination(sched* s, msk_t cur) {
    if (*umap_ref(&s->used, cur) != 0) return;
    msk_t bad = 0;
    int ans = 0;
    for (int i = 0; i < s->ngates; ++i) {
        if (can_take(s, i, cur, bad)) ++ans;
        else {
            bad |= s->gate[i] | s->ctrl[i];
            /* once every qubit is blocked no later gate can be taken */
            if ((bad & s->all) == s->all) break;
        }
    }
    if (ans > s->best_ans ||
        (ans == s->best_ans && __builtin_popcountll(cur) < __builtin_popcountll(s->best))) {
        s->best_ans = ans;
        s->best = cur;
    }
}

static void rec(sched* s, msk_t cur, msk_t bit) {
    calc_combination(s, cur);
    if (bit > s->locals) return;
    msk_t* u = umap_ref(&s->used, cur);
    if (*u & bit) return;
    *u |= bit;
    if (!(bit & ~s->locals) && !(bit & cur) && __builtin_popcountll(cur) < s->K)
        rec(s, cur | bit, bit << 1);
    rec(s, cur, bit << 1);
}

static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

/*
 * ngates gates; gate g has targets tgt[toff[g]..toff[g+1]) and controls
 * ctl[coff[g]..coff[g+1]) (qubit ids). locals: the simulator's local ids.
 * Output: order[] = gate indices in emission order, cluster_end[c] = index in
 * order[] one past the end of cluster c. Returns the number of clusters, or -1
 * when more than 63 distinct qubits are involved.
 */
int orc_greedy_schedule(int ngates, const int64_t* tgt, const int* toff, const int64_t* ctl,
                        const int* coff, int nlocals, const int64_t* locals, int K, int* order,
                        int* cluster_end) {
    int nid = toff[ngates] + coff[ngates] + nlocals;
    int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * (nid + 1));
    int c = 0;
    for (int i = 0; i < toff[ngates]; ++i) ids[c++] = tgt[i];
    for (int i = 0; i < coff[ngates]; ++i) ids[c++] = ctl[i];
    for (int i = 0; i < nlocals; ++i) ids[c++] = locals[i];
    qsort(ids, c, sizeof(int64_t), cmp_i64);
    int u = 0;
    for (int i = 0; i < c; ++i)
        if (u == 0 || ids[u - 1] != ids[i]) ids[u++] = ids[i];
    if (u >= 64) { free(ids); return -1; }
#define POS(id) ((int)(((int64_t*)bsearch(&(id), ids, u, sizeof(int64_t), cmp_i64)) - ids))
    msk_t* gm = (msk_t*)malloc(sizeof(msk_t) * (ngates + 1));
    msk_t* cm = (msk_t*)malloc(sizeof(msk_t) * (ngates + 1));
    int* idx = (int*)malloc(sizeof(int) * (ngates + 1));
    msk_t locm = 0, all = 0;
    for (int i = 0; i < nlocals; ++i) locm |= 1ULL << POS(locals[i]);
    for (int g = 0; g < ngates; ++g) {
        gm[g] = cm[g] = 0;
        for (int j = toff[g]; j < toff[g + 1]; ++j) gm[g] |= 1ULL << POS(tgt[j]);
        for (int j = coff[g]; j < coff[g + 1]; ++j) cm[g] |= 1ULL << POS(ctl[j]);
        all |= gm[g] | cm[g];
        idx[g] = g;
    }
#undef POS
    int remaining = ngates, emitted = 0, nclusters = 0;
    msk_t* sg = (msk_t*)malloc(sizeof(msk_t) * (ngates + 1));
    msk_t* sc = (msk_t*)malloc(sizeof(msk_t) * (ngates + 1));
    int* take = (int*)malloc(sizeof(int) * (ngates + 1));
    while (remaining > 0) {
        /* the reference recomputes bit positions over the remaining gates each
         * round; positions are the rank of the id among those present */
        int nid2 = 0;
        msk_t present = locm;
        for (int r = 0; r < remaining; ++r) present |= gm[idx[r]] | cm[idx[r]];
        int remap[64];
        for (int b = 0; b < u; ++b) remap[b] = ((present >> b) & 1) ? nid2++ : -1;
        msk_t loc2 = 0, all2 = 0;
        for (int b = 0; b < u; ++b)
            if ((locm >> b) & 1) loc2 |= 1ULL << remap[b];
        for (int r = 0; r < remaining; ++r) {
            msk_t a = 0, b2 = 0;
            for (int b = 0; b < u; ++b) {
                if ((gm[idx[r]] >> b) & 1) a |= 1ULL << remap[b];
                if ((cm[idx[r]] >> b) & 1) b2 |= 1ULL << remap[b];
            }
            sg[r] = a; sc[r] = b2;
            all2 |= a | b2;
        }
        sched s;
        s.K = K; s.ngates = remaining; s.gate = sg; s.ctrl = sc; s.locals = loc2; s.all = all2 | loc2;
        s.best_ans = 0; s.best = 0;
        umap_init(&s.used, 1024);
        for (int i = 0; i < remaining; ++i) {
            msk_t cl = loc2 & (sg[i] | sc[i]);
            if (__builtin_popcountll(cl) <= K) rec(&s, cl, 1);
        }
        int ntake = 0;
        if (s.best_ans != 0) {
            msk_t bad = 0;
            for (int i = 0; i < remaining; ++i) {
                if (can_take(&s, i, s.best, bad)) take[ntake++] = i;
                else bad |= sg[i] | sc[i];
            }
        } else {
            msk_t bad = 0;
            for (int i = 0; i < remaining; ++i) {
                if (can_take(&s, i, loc2, bad)) { take[ntake++] = i; break; }
                bad |= sg[i] | sc[i];
            }
        }
        umap_free(&s.used);
        if (ntake == 0) break;
        for (int t = 0; t < ntake; ++t) order[emitted++] = idx[take[t]];
        cluster_end[nclusters++] = emitted;
        /* drop the taken gates, keeping the rest in order */
        int w = 0, t = 0;
        for (int r = 0; r < remaining; ++r) {
            if (t < ntake && take[t] == r) { ++t; continue; }
            idx[w++] = idx[r];
        }
        remaining = w;
    }
    free(ids); free(gm); free(cm); free(idx); free(sg); free(sc); free(take);
    return nclusters;
}
