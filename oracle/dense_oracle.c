/*
 * Dense FP64 statevector oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/ may load this library. It is an independent textbook check of the engine's
 * gates, sharing no code or operand order with it: every gate is a complex matrix (2x2 for
 * one target qubit, 4x4 for two) applied to every index pair (or quadruple) of a full
 * 2^nq-amplitude vector, with no pruning. The matrices are built by the caller (oracle/dense.py)
 * from their textbook definitions.
 *
 * Storage: the vector is split into pages of 2^P amplitudes; a page that has only ever held
 * zeros is not allocated and reads as zeros. Applying a matrix to a group of all-zero
 * amplitudes gives zeros, so skipping such groups changes no value: the result is the dense
 * statevector's, bit for bit, at a cost proportional to the pages the state reaches. That makes
 * 30-qubit registers affordable for states that occupy a small part of the space.
 *
 * Conventions (the reference's, emulator/src/QLib.cpp:15-28): qubit t is bit t of the basis
 * index, qubit 0 the least significant. A controlled gate acts iff every control bit is 1.
 * Products are complex multiplications written out as (ar*br - ai*bi, ar*bi + ai*br), compiled
 * with -ffp-contract=off.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int nq, P;            /* qubits; log2 amplitudes per page */
    uint64_t npages;
    double** pages;       /* page i holds amplitudes [i << P, (i + 1) << P) as (re, im) pairs */
    uint64_t* live;       /* indices of the allocated pages, in no particular order */
    uint64_t nlive, cap_live;
    int nthreads;
} dno_state;

/* The page directory of a 40-qubit register has 2^26 entries: gates walk the list of allocated
 * pages, never the directory. */
static double* page_alloc(dno_state* st, uint64_t p) {
    if (st->pages[p]) return st->pages[p];
    if (st->nlive == st->cap_live) {
        const uint64_t cap = st->cap_live ? 2 * st->cap_live : 64;
        uint64_t* l = (uint64_t*)realloc(st->live, cap * sizeof(uint64_t));
        if (!l) return NULL;
        st->live = l;
        st->cap_live = cap;
    }
    st->pages[p] = (double*)calloc((size_t)2 << st->P, sizeof(double));
    if (st->pages[p]) st->live[st->nlive++] = p;
    return st->pages[p];
}

/* Drop freed pages from the live list. */
static void live_compact(dno_state* st) {
    uint64_t n = 0;
    for (uint64_t i = 0; i < st->nlive; ++i)
        if (st->pages[st->live[i]]) st->live[n++] = st->live[i];
    st->nlive = n;
}

static int cmp_u64(const void* a, const void* b) {
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

static void free_pages(dno_state* st) {
    for (uint64_t i = 0; i < st->nlive; ++i) {
        free(st->pages[st->live[i]]);
        st->pages[st->live[i]] = NULL;
    }
    st->nlive = 0;
}

dno_state* dno_create(int nq) {
    if (nq < 1 || nq > 40) return NULL;
    dno_state* st = (dno_state*)calloc(1, sizeof(dno_state));
    if (!st) return NULL;
    st->nq = nq;
    st->P = nq < 14 ? nq : 14;
    st->npages = 1ULL << (nq - st->P);
    st->pages = (double**)calloc(st->npages, sizeof(double*));
    st->nthreads = 1;
    if (!st->pages || !page_alloc(st, 0)) { free(st->pages); free(st->live); free(st); return NULL; }
    st->pages[0][0] = 1.0;
    return st;
}

void dno_destroy(dno_state* st) {
    if (!st) return;
    free_pages(st);
    free(st->pages);
    free(st->live);
    free(st);
}

void dno_set_threads(dno_state* st, int n) { st->nthreads = n > 0 ? n : 1; }

/* Replace the state by the given entries (keys < 2^nq). Returns -1 on a bad key. */
int dno_set_state(dno_state* st, const uint64_t* keys, const double* re, const double* im, uint64_t n) {
    free_pages(st);
    for (uint64_t i = 0; i < n; ++i) {
        if (st->nq < 64 && (keys[i] >> st->nq)) return -1;
        double* pg = page_alloc(st, keys[i] >> st->P);
        if (!pg) return -2;
        const uint64_t o = keys[i] & ((1ULL << st->P) - 1);
        pg[2 * o] = re[i];
        pg[2 * o + 1] = im[i];
    }
    return 0;
}

/* out = sum_k m[row][k] * v[k] for a 2^w-square complex matrix m (row-major (re, im) pairs). */
static inline void matvec(int dim, const double* m, const double* vr, const double* vi, double* orr, double* oi) {
    for (int r = 0; r < dim; ++r) {
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < dim; ++k) {
            const double mr = m[2 * (r * dim + k)], mi = m[2 * (r * dim + k) + 1];
            sr = sr + (mr * vr[k] - mi * vi[k]);
            si = si + (mr * vi[k] + mi * vr[k]);
        }
        orr[r] = sr;
        oi[r] = si;
    }
}

/* Apply a (2^w)x(2^w) matrix to target qubits t[0..w-1] (t[0] the least significant bit of
 * the matrix index) under controls. Index groups whose members all lie in unallocated pages
 * are skipped; pages a group writes to are allocated first. Returns 0, or -1 on bad arguments. */
static int apply_w(dno_state* st, int w, const uint32_t* t, uint64_t controls, const double* m) {
    const int dim = 1 << w;
    uint64_t tmask = 0;
    for (int a = 0; a < w; ++a) {
        if ((int)t[a] >= st->nq || (tmask >> t[a]) & 1ULL) return -1;
        tmask |= 1ULL << t[a];
    }
    if (controls & tmask) return -1;
    if (st->nq < 64 && (controls >> st->nq)) return -1;
    const int P = st->P;
    const uint64_t in_mask = (1ULL << P) - 1;
    const uint64_t pt_mask = tmask >> P;             /* target bits above the page offset */
    const uint64_t pc_mask = controls >> P, c_in = controls & in_mask;
    /* the base pages (page-level target bits clear, page-level controls set) of the groups
     * that hold an allocated page; then every page of those groups is allocated, before the
     * parallel update */
    uint64_t* base = (uint64_t*)malloc((st->nlive ? st->nlive : 1) * sizeof(uint64_t));
    if (!base) return -2;
    uint64_t nb = 0;
    for (uint64_t i = 0; i < st->nlive; ++i) {
        const uint64_t b = st->live[i] & ~pt_mask;
        if ((b & pc_mask) == pc_mask) base[nb++] = b;
    }
    qsort(base, nb, sizeof(uint64_t), cmp_u64);
    uint64_t nu = 0;
    for (uint64_t i = 0; i < nb; ++i)
        if (!nu || base[nu - 1] != base[i]) base[nu++] = base[i];
    for (uint64_t i = 0; i < nu; ++i) {
        for (uint64_t s = pt_mask;; s = (s - 1) & pt_mask) {
            if (!page_alloc(st, base[i] | s)) { free(base); return -2; }
            if (!s) break;
        }
    }
    const uint64_t in_tmask = tmask & in_mask;
    const int64_t np = (int64_t)nu;
#pragma omp parallel for schedule(dynamic, 1) num_threads(st->nthreads)
    for (int64_t pi = 0; pi < np; ++pi) {
        const uint64_t p = base[pi];
        for (uint64_t o = 0; o <= in_mask; ++o) {
            if ((o & in_tmask) || (o & c_in) != c_in) continue;
            double vr[16], vi[16], orr[16], oi[16];
            double* ptr[16];
            for (int k = 0; k < dim; ++k) {
                uint64_t idx = (p << P) | o;
                for (int a = 0; a < w; ++a)
                    if ((k >> a) & 1) idx |= 1ULL << t[a];
                double* pg = st->pages[idx >> P];
                ptr[k] = pg + 2 * (idx & in_mask);
                vr[k] = ptr[k][0];
                vi[k] = ptr[k][1];
            }
            matvec(dim, m, vr, vi, orr, oi);
            for (int k = 0; k < dim; ++k) {
                ptr[k][0] = orr[k];
                ptr[k][1] = oi[k];
            }
        }
        /* a member page left holding only zeros goes back to the implicit zero page (these
         * pages belong to this base page alone, so no other thread touches them) */
        for (uint64_t s = pt_mask;; s = (s - 1) & pt_mask) {
            double* pg = st->pages[p | s];
            int any = 0;
            for (uint64_t o = 0; o < 2 * (in_mask + 1) && !any; ++o) any = pg[o] != 0.0;
            if (!any && (p | s) != 0) { free(pg); st->pages[p | s] = NULL; }
            if (!s) break;
        }
    }
    free(base);
    live_compact(st);
    return 0;
}

/* One-qubit gate: m = 2x2 complex matrix, row-major, (re, im) pairs. */
int dno_apply1(dno_state* st, uint32_t target, uint64_t controls, const double* m) {
    return apply_w(st, 1, &target, controls, m);
}

/* Two-qubit gate on (a, b): m = 4x4 complex matrix over the index i_a + 2*i_b. */
int dno_apply2(dno_state* st, uint32_t a, uint32_t b, uint64_t controls, const double* m) {
    const uint32_t t[2] = {a, b};
    return apply_w(st, 2, t, controls, m);
}

/* Entries with !(|re| < thr && |im| < thr), key-sorted, into caller arrays. Returns the count
 * (entries beyond cap are counted, not written). */
uint64_t dno_get_state(dno_state* st, uint64_t* keys, double* re, double* im, uint64_t cap, double thr) {
    uint64_t n = 0;
    const uint64_t per = 1ULL << st->P;
    qsort(st->live, st->nlive, sizeof(uint64_t), cmp_u64);   /* key order */
    for (uint64_t i = 0; i < st->nlive; ++i) {
        const uint64_t p = st->live[i];
        const double* pg = st->pages[p];
        for (uint64_t o = 0; o < per; ++o) {
            const double r = pg[2 * o], i = pg[2 * o + 1];
            const double ar = r < 0 ? -r : r, ai = i < 0 ? -i : i;
            if (ar < thr && ai < thr) continue;
            if (n < cap) { keys[n] = (p << st->P) | o; re[n] = r; im[n] = i; }
            ++n;
        }
    }
    return n;
}

int dno_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
