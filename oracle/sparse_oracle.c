/*
 * Sparse CPU oracle for the gate path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
 * library. It is the checker and the timed CPU baseline, never part of the product.
 *
 * It restates the reference's FC gate algorithm (ivanNovikau/SparQC) on the CPU:
 *   - pair rule: the key with target bit 0 owns the pair; the key with bit 1 owns it only
 *     when its bit-0 partner is absent; a missing partner counts as amplitude 0
 *     (emulator/device/device_table_FC.cuh:62-110);
 *   - 2x2 updates, operand order as written in emulator/device/device_data.cuh:159-319
 *     (H: f*(a+b) with f = 1./sqrt(2.), emulator/device/device_data.cuh:199-209 and
 *     emulator/include/data_t.h:63-80);
 *   - Rz/Rx/Ry receive theta/2, Phase receives theta unchanged
 *     (emulator/device/table_manager.cuh:333-336), and the coefficients are cos/sin of that
 *     argument (emulator/device/device_table_FC.cuh:182) -- computed here on the host;
 *   - pruning after branching gates only: a key survives iff !(|re|<thr && |im|<thr)
 *     (emulator/device/device_data.cuh:134-156, emulator/include/data_t.h:50-60);
 *     swap gates (X, Y) move keys and diagonal gates keep every key
 *     (emulator/device/device_data.cuh:108-131).
 * Gates the reference lacks (controls, S, Sdg, T, Tdg, U) follow the engine's documented
 * definitions: a gate applies iff (key & controls) == controls; S/Sdg multiply the bit-1
 * amplitude by +-i exactly; T/Tdg are Phase with cos = +-sin = sqrt(1/2); U is the u3
 * matrix applied with an explicit fused-multiply-add chain, self term first.
 *
 * Arithmetic: compiled with -ffp-contract=off so that every product and sum rounds
 * exactly as written; fma() is used only where the definition says so (U).
 * FP32 mode runs the same formulas in float with float-rounded coefficients; its prune
 * comparison is done in double after exact promotion.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { K_X = 0, K_Y, K_Z, K_H, K_PHASE, K_RZ, K_RX, K_RY, K_S, K_SDG, K_T, K_TDG, K_U, K_COUNT };
enum { C_SWAP = 0, C_DIAG = 1, C_BRANCH = 2 };

typedef struct {
    uint32_t kind, target;
    uint64_t controls;
    double theta, phi, lambda;
} orc_gate;

typedef struct {
    int prec;           /* 64 or 32 */
    double thr;         /* prune threshold */
    uint64_t n, cap;    /* entries, allocated entries */
    uint64_t *keys;
    double *re, *im;    /* in FP32 mode every stored value is exactly a float */
    uint64_t icap;      /* index capacity (power of two) */
    uint64_t *idx;      /* position+1, 0 = empty */
    int nthreads;
    uint64_t amp_updates;  /* sum over applied gates of the input key count */
    uint64_t scap;         /* scratch entries allocated */
    uint64_t *sk;          /* scratch: output keys, values and validity of a key-changing gate */
    double *sr, *si;
    unsigned char *sv;
} orc_state;

typedef struct { double c, s; double m[8]; } coef_t;

static int gate_class(uint32_t kind) {
    switch (kind) {
    case K_X: case K_Y: return C_SWAP;
    case K_H: case K_RX: case K_RY: case K_U: return C_BRANCH;
    default: return C_DIAG;
    }
}

static void resolve(const orc_gate* g, coef_t* k) {
    memset(k, 0, sizeof *k);
    switch (g->kind) {
    case K_PHASE: k->c = cos(g->theta); k->s = sin(g->theta); break;
    case K_RZ: case K_RX: case K_RY: { double h = g->theta / 2.; k->c = cos(h); k->s = sin(h); break; }
    case K_T: k->c = 0.70710678118654752440; k->s = 0.70710678118654752440; break;
    case K_TDG: k->c = 0.70710678118654752440; k->s = -0.70710678118654752440; break;
    case K_H: k->c = 1. / sqrt(2.); break;
    case K_U: {
        double c = cos(g->theta / 2.), s = sin(g->theta / 2.);
        double cl = cos(g->lambda), sl = sin(g->lambda);
        double cp = cos(g->phi), sp = sin(g->phi);
        double cpl = cos(g->phi + g->lambda), spl = sin(g->phi + g->lambda);
        k->m[0] = c;          k->m[1] = 0.;          /* m00 */
        k->m[2] = -(cl * s);  k->m[3] = -(sl * s);   /* m01 */
        k->m[4] = cp * s;     k->m[5] = sp * s;      /* m10 */
        k->m[6] = cpl * c;    k->m[7] = spl * c;     /* m11 */
        break;
    }
    default: break;
    }
}

/* 2x2 update of one pair in double. v0 = amplitude of the bit-0 key, v1 = bit-1 key. */
static void pair64(uint32_t kind, const coef_t* k, double v0r, double v0i, double v1r, double v1i,
                   double* o0r, double* o0i, double* o1r, double* o1i) {
    const double c = k->c, s = k->s;
    switch (kind) {
    case K_X: *o0r = v1r; *o0i = v1i; *o1r = v0r; *o1i = v0i; break;
    case K_Y: *o0r = v1i; *o0i = -v1r; *o1r = -v0i; *o1i = v0r; break;
    case K_Z: *o0r = v0r; *o0i = v0i; *o1r = -v1r; *o1i = -v1i; break;
    case K_S: *o0r = v0r; *o0i = v0i; *o1r = -v1i; *o1i = v1r; break;
    case K_SDG: *o0r = v0r; *o0i = v0i; *o1r = v1i; *o1i = -v1r; break;
    case K_PHASE: case K_T: case K_TDG:
        *o0r = v0r; *o0i = v0i; *o1r = c * v1r - s * v1i; *o1i = c * v1i + s * v1r; break;
    case K_RZ:
        *o0r = c * v0r + s * v0i; *o0i = c * v0i - s * v0r;
        *o1r = c * v1r - s * v1i; *o1i = c * v1i + s * v1r; break;
    case K_H:
        *o0r = c * (v0r + v1r); *o0i = c * (v0i + v1i);
        *o1r = c * (v0r - v1r); *o1i = c * (v0i - v1i); break;
    case K_RX:
        *o0r = c * v0r + s * v1i; *o0i = c * v0i - s * v1r;
        *o1r = c * v1r + s * v0i; *o1i = c * v1i - s * v0r; break;
    case K_RY:
        *o0r = c * v0r - s * v1r; *o0i = c * v0i - s * v1i;
        *o1r = c * v1r + s * v0r; *o1i = c * v1i + s * v0i; break;
    case K_U: {
        const double* m = k->m;
        *o0r = fma(-m[3], v1i, fma(m[2], v1r, fma(-m[1], v0i, m[0] * v0r)));
        *o0i = fma(m[3], v1r, fma(m[2], v1i, fma(m[1], v0r, m[0] * v0i)));
        *o1r = fma(-m[5], v0i, fma(m[4], v0r, fma(-m[7], v1i, m[6] * v1r)));
        *o1i = fma(m[5], v0r, fma(m[4], v0i, fma(m[7], v1r, m[6] * v1i)));
        break;
    }
    default: *o0r = v0r; *o0i = v0i; *o1r = v1r; *o1i = v1i; break;
    }
}

/* The same formulas in float with float-rounded coefficients. */
static void pair32(uint32_t kind, const coef_t* k, float v0r, float v0i, float v1r, float v1i,
                   float* o0r, float* o0i, float* o1r, float* o1i) {
    const float c = (float)k->c, s = (float)k->s;
    switch (kind) {
    case K_X: *o0r = v1r; *o0i = v1i; *o1r = v0r; *o1i = v0i; break;
    case K_Y: *o0r = v1i; *o0i = -v1r; *o1r = -v0i; *o1i = v0r; break;
    case K_Z: *o0r = v0r; *o0i = v0i; *o1r = -v1r; *o1i = -v1i; break;
    case K_S: *o0r = v0r; *o0i = v0i; *o1r = -v1i; *o1i = v1r; break;
    case K_SDG: *o0r = v0r; *o0i = v0i; *o1r = v1i; *o1i = -v1r; break;
    case K_PHASE: case K_T: case K_TDG:
        *o0r = v0r; *o0i = v0i; *o1r = c * v1r - s * v1i; *o1i = c * v1i + s * v1r; break;
    case K_RZ:
        *o0r = c * v0r + s * v0i; *o0i = c * v0i - s * v0r;
        *o1r = c * v1r - s * v1i; *o1i = c * v1i + s * v1r; break;
    case K_H:
        *o0r = c * (v0r + v1r); *o0i = c * (v0i + v1i);
        *o1r = c * (v0r - v1r); *o1i = c * (v0i - v1i); break;
    case K_RX:
        *o0r = c * v0r + s * v1i; *o0i = c * v0i - s * v1r;
        *o1r = c * v1r + s * v0i; *o1i = c * v1i - s * v0r; break;
    case K_RY:
        *o0r = c * v0r - s * v1r; *o0i = c * v0i - s * v1i;
        *o1r = c * v1r + s * v0r; *o1i = c * v1i + s * v0i; break;
    case K_U: {
        float m[8];
        for (int i = 0; i < 8; ++i) m[i] = (float)k->m[i];
        *o0r = fmaf(-m[3], v1i, fmaf(m[2], v1r, fmaf(-m[1], v0i, m[0] * v0r)));
        *o0i = fmaf(m[3], v1r, fmaf(m[2], v1i, fmaf(m[1], v0r, m[0] * v0i)));
        *o1r = fmaf(-m[5], v0i, fmaf(m[4], v0r, fmaf(-m[7], v1i, m[6] * v1r)));
        *o1i = fmaf(m[5], v0r, fmaf(m[4], v0i, fmaf(m[7], v1r, m[6] * v1i)));
        break;
    }
    default: *o0r = v0r; *o0i = v0i; *o1r = v1r; *o1i = v1i; break;
    }
}

static inline int negligible(double r, double i, double thr) { return fabs(r) < thr && fabs(i) < thr; }

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27; x *= 0x94d049bb133111ebULL;
    x ^= x >> 31; return x;
}

static int build_index(orc_state* st) {
    uint64_t want = 16;
    while (want < 2 * st->n + 2) want <<= 1;
    if (want != st->icap) {
        free(st->idx);
        st->idx = (uint64_t*)malloc(want * sizeof(uint64_t));
        if (!st->idx) { st->icap = 0; return -1; }
        st->icap = want;
    }
    const int64_t ic = (int64_t)st->icap;
#pragma omp parallel for schedule(static) num_threads(st->nthreads)
    for (int64_t i = 0; i < ic; ++i) st->idx[i] = 0;
    const uint64_t mask = st->icap - 1;
    const int64_t n = (int64_t)st->n;
#pragma omp parallel for schedule(static) num_threads(st->nthreads)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t h = mix64(st->keys[i]) & mask;
        for (;;) {
            uint64_t expect = 0;
            if (__atomic_compare_exchange_n(&st->idx[h], &expect, (uint64_t)i + 1, 0,
                                            __ATOMIC_RELAXED, __ATOMIC_RELAXED))
                break;
            h = (h + 1) & mask;
        }
    }
    return 0;
}

static inline int64_t lookup(const orc_state* st, uint64_t key) {
    const uint64_t mask = st->icap - 1;
    uint64_t h = mix64(key) & mask;
    for (;;) {
        uint64_t p = st->idx[h];
        if (p == 0) return -1;
        if (st->keys[p - 1] == key) return (int64_t)(p - 1);
        h = (h + 1) & mask;
    }
}

static int reserve(orc_state* st, uint64_t cap) {
    if (cap <= st->cap) return 0;
    uint64_t* k = (uint64_t*)realloc(st->keys, cap * sizeof(uint64_t));
    if (!k) return -1;
    st->keys = k;
    double* r = (double*)realloc(st->re, cap * sizeof(double));
    if (!r) return -1;
    st->re = r;
    double* i = (double*)realloc(st->im, cap * sizeof(double));
    if (!i) return -1;
    st->im = i;
    st->cap = cap;
    return 0;
}

orc_state* orc_create(int precision, double prune_threshold) {
    orc_state* st = (orc_state*)calloc(1, sizeof(orc_state));
    if (!st) return NULL;
    st->prec = precision == 32 ? 32 : 64;
    st->thr = prune_threshold;
    st->nthreads = 1;
    if (reserve(st, 16)) { free(st); return NULL; }
    st->n = 1; st->keys[0] = 0; st->re[0] = 1.; st->im[0] = 0.;
    build_index(st);
    return st;
}

void orc_destroy(orc_state* st) {
    if (!st) return;
    free(st->keys); free(st->re); free(st->im); free(st->idx);
    free(st->sk); free(st->sr); free(st->si); free(st->sv); free(st);
}

void orc_set_threads(orc_state* st, int nthreads) { st->nthreads = nthreads > 0 ? nthreads : 1; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Replace the state; keys must be distinct. In FP32 mode values are rounded to float. */
int orc_set_state(orc_state* st, const uint64_t* keys, const double* re, const double* im, uint64_t n) {
    if (reserve(st, n > 16 ? n : 16)) return -1;
    for (uint64_t i = 0; i < n; ++i) {
        st->keys[i] = keys[i];
        st->re[i] = st->prec == 32 ? (double)(float)re[i] : re[i];
        st->im[i] = st->prec == 32 ? (double)(float)im[i] : im[i];
    }
    st->n = n;
    if (build_index(st)) return -1;
    for (uint64_t i = 0; i < n; ++i)
        if (lookup(st, keys[i]) != (int64_t)i) return -2; /* duplicate key */
    return 0;
}

/* Output scratch of a key-changing gate, kept between gates (2n entries). */
static int scratch(orc_state* st, uint64_t n2) {
    if (n2 <= st->scap) return 0;
    free(st->sk); free(st->sr); free(st->si); free(st->sv);
    st->sk = (uint64_t*)malloc(n2 * sizeof(uint64_t));
    st->sr = (double*)malloc(n2 * sizeof(double));
    st->si = (double*)malloc(n2 * sizeof(double));
    st->sv = (unsigned char*)malloc(n2);
    if (!st->sk || !st->sr || !st->si || !st->sv) { st->scap = 0; return -1; }
    st->scap = n2;
    return 0;
}

/* The 2x2 update of one pair at the state's precision. */
static inline void pair_any(const orc_state* st, uint32_t kind, const coef_t* k, double v0r, double v0i,
                            double v1r, double v1i, double* o0r, double* o0i, double* o1r, double* o1i) {
    if (st->prec == 32) {
        float a, b, c2, d;
        pair32(kind, k, (float)v0r, (float)v0i, (float)v1r, (float)v1i, &a, &b, &c2, &d);
        *o0r = a; *o0i = b; *o1r = c2; *o1i = d;
    } else {
        pair64(kind, k, v0r, v0i, v1r, v1i, o0r, o0i, o1r, o1i);
    }
}

/* Apply one gate: every pair with at least one present member is updated once.
 * A diagonal gate's outputs each depend on their own input only and it keeps every key
 * (emulator/device/device_data.cuh:108-131), so it is applied in place, key by key, with the
 * same pair formula and no index rebuild. */
static int apply_one(orc_state* st, const orc_gate* g) {
    if (g->kind >= K_COUNT || g->target > 63) return -3;
    const uint64_t bq = 1ULL << g->target;
    if (g->controls & bq) return -3;
    coef_t k;
    resolve(g, &k);
    const int cls = gate_class(g->kind);
    const uint64_t C = g->controls;
    const int64_t n = (int64_t)st->n;
    if (cls == C_DIAG) {
#pragma omp parallel for schedule(static) num_threads(st->nthreads)
        for (int64_t i = 0; i < n; ++i) {
            const uint64_t key = st->keys[i];
            if ((key & C) != C) continue;
            double o0r, o0i, o1r, o1i;
            if (key & bq) {
                pair_any(st, g->kind, &k, 0., 0., st->re[i], st->im[i], &o0r, &o0i, &o1r, &o1i);
                st->re[i] = o1r; st->im[i] = o1i;
            } else {
                pair_any(st, g->kind, &k, st->re[i], st->im[i], 0., 0., &o0r, &o0i, &o1r, &o1i);
                st->re[i] = o0r; st->im[i] = o0i;
            }
        }
        return 0;
    }
    if (scratch(st, 2 * (uint64_t)n + 1)) return -1;
    uint64_t* ok = st->sk;
    double* orr = st->sr;
    double* oi = st->si;
    unsigned char* valid = st->sv;

#pragma omp parallel for schedule(static) num_threads(st->nthreads)
    for (int64_t i = 0; i < n; ++i) {
        const uint64_t key = st->keys[i];
        valid[2 * i] = valid[2 * i + 1] = 0;
        if ((key & C) != C) {            /* control not satisfied: the key passes unchanged */
            ok[2 * i] = key; orr[2 * i] = st->re[i]; oi[2 * i] = st->im[i]; valid[2 * i] = 1;
            continue;
        }
        const int bit = (key & bq) != 0;
        const int64_t j = lookup(st, key ^ bq);
        if (bit && j >= 0) continue;      /* the bit-0 partner is present and owns the pair */
        const uint64_t k0 = key & ~bq, k1 = key | bq;
        int have0, have1;
        double v0r, v0i, v1r, v1i;
        if (!bit) {
            have0 = 1; v0r = st->re[i]; v0i = st->im[i];
            have1 = j >= 0; v1r = have1 ? st->re[j] : 0.; v1i = have1 ? st->im[j] : 0.;
        } else {
            have0 = 0; v0r = 0.; v0i = 0.;
            have1 = 1; v1r = st->re[i]; v1i = st->im[i];
        }
        double o0r, o0i, o1r, o1i;
        pair_any(st, g->kind, &k, v0r, v0i, v1r, v1i, &o0r, &o0i, &o1r, &o1i);
        int e0, e1;
        if (cls == C_SWAP) { e0 = have1; e1 = have0; }
        else { e0 = !negligible(o0r, o0i, st->thr); e1 = !negligible(o1r, o1i, st->thr); }
        if (e0) { ok[2 * i] = k0; orr[2 * i] = o0r; oi[2 * i] = o0i; valid[2 * i] = 1; }
        if (e1) { ok[2 * i + 1] = k1; orr[2 * i + 1] = o1r; oi[2 * i + 1] = o1i; valid[2 * i + 1] = 1; }
    }
    /* stable compaction of the valid outputs: per-thread counts over fixed ranges, a prefix sum,
     * then each range copies its entries to its offset (the same order as one serial sweep) */
    enum { kParts = 256 };
    uint64_t cnt[kParts + 1];
    const int64_t m2 = 2 * n;
    const int64_t per = (m2 + kParts - 1) / kParts;
#pragma omp parallel for schedule(static) num_threads(st->nthreads)
    for (int p = 0; p < kParts; ++p) {
        uint64_t c = 0;
        const int64_t lo = (int64_t)p * per, hi = lo + per < m2 ? lo + per : m2;
        for (int64_t i = lo; i < hi; ++i) c += valid[i];
        cnt[p + 1] = c;
    }
    cnt[0] = 0;
    for (int p = 0; p < kParts; ++p) cnt[p + 1] += cnt[p];
    const uint64_t m = cnt[kParts];
    if (reserve(st, m > 16 ? m : 16)) return -1;
#pragma omp parallel for schedule(static) num_threads(st->nthreads)
    for (int p = 0; p < kParts; ++p) {
        uint64_t w = cnt[p];
        const int64_t lo = (int64_t)p * per, hi = lo + per < m2 ? lo + per : m2;
        for (int64_t i = lo; i < hi; ++i)
            if (valid[i]) { st->keys[w] = ok[i]; st->re[w] = orr[i]; st->im[w] = oi[i]; ++w; }
    }
    st->n = m;
    return build_index(st);
}

int orc_apply(orc_state* st, const orc_gate* gates, uint64_t ngates) {
    for (uint64_t g = 0; g < ngates; ++g) {
        st->amp_updates += st->n;
        int rc = apply_one(st, &gates[g]);
        if (rc) return rc;
    }
    return 0;
}

uint64_t orc_nnz(const orc_state* st) { return st->n; }

uint64_t orc_amp_updates(const orc_state* st) { return st->amp_updates; }

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

/* Copy the state out. sorted != 0 orders by key. Returns the entry count, or -1 when cap is short. */
int64_t orc_get_state(const orc_state* st, uint64_t* keys, double* re, double* im, uint64_t cap, int sorted) {
    if (cap < st->n) return -1;
    if (!sorted) {
        memcpy(keys, st->keys, st->n * sizeof(uint64_t));
        memcpy(re, st->re, st->n * sizeof(double));
        memcpy(im, st->im, st->n * sizeof(double));
        return (int64_t)st->n;
    }
    memcpy(keys, st->keys, st->n * sizeof(uint64_t));
    qsort(keys, st->n, sizeof(uint64_t), cmp_u64);
    for (uint64_t i = 0; i < st->n; ++i) {
        int64_t p = lookup(st, keys[i]);
        re[i] = st->re[p]; im[i] = st->im[p];
    }
    return (int64_t)st->n;
}

/* Sum of |amp|^2 in double. */
double orc_norm2(const orc_state* st) {
    double acc = 0.;
    for (uint64_t i = 0; i < st->n; ++i) acc += st->re[i] * st->re[i] + st->im[i] * st->im[i];
    return acc;
}
