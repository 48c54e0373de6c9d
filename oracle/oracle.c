/*
 * oracle.c -- CPU restatement of MP-sort's single-node sort path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it, and only as the checker.
 *
 * It restates, in plain C written for this project, what these reference
 * functions compute (file:line within the MP-sort tree):
 *
 *   a1  radix_func_{u8,i8,u4,i4}          mpsort/binding.pyx:81-121
 *   a2  compare / bisect of radix bytes   radixsort.c:47-195
 *   a3  radix_sort (stable merge sort)    radixsort.c:35-44, stdlib/msort.c:52-314
 *   a4  mpsort_omp driver                 mpsort-omp.c:47-108, 220-395
 *   a6  global min/max radix              mpsort-omp.c:251-265
 *   a7  piter_init/bisect/accept/done     internal-parallel.h:128-248
 *   a8  _histogram, _bsearch_last_lt/le   internal-parallel.h:8-126
 *   a9  reduce / gather of counts         mpsort-omp.c:110-127
 *   a10 _solve_for_layout                 mpsort-omp.c:143-218
 *   a11 exchange + second local sort      mpsort-omp.c:336-389
 *
 * The tasks of mpsort_omp run on OpenMP threads when this file is built with
 * -fopenmp (oracle/Makefile does), else one after another; the result is the
 * same either way.  Errors are returned, never abort().
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stddef.h>

#include "../include/gbsort_key.h"

typedef void (*oracle_radix_fn)(const void *ptr, void *radix, void *arg);

/* ------------------------------------------------------------------ a1 */

/* Order-preserving 64-bit word of one key field (binding.pyx:81-121). */
static uint64_t key_word(const unsigned char *rec, const gbsort_key_word *w)
{
    if (w->width == 8) {
        uint64_t v;
        memcpy(&v, rec + w->offset, 8);
        return w->is_signed ? v + 0x8000000000000000ull : v;
    } else {
        uint32_t v;
        memcpy(&v, rec + w->offset, 4);
        if (w->is_signed) {
            int64_t s = (int64_t)(int32_t)v;
            return (uint64_t)s + 0x8000000000000000ull;
        }
        return (uint64_t)v;
    }
}

/* radix() callback driven by a gbsort_key_desc passed as `arg`. */
void oracle_radix_desc(const void *ptr, void *radix, void *arg)
{
    const gbsort_key_desc *d = (const gbsort_key_desc *)arg;
    unsigned char *out = (unsigned char *)radix;
    uint32_t i;
    for (i = 0; i < d->nwords; i++) {
        uint64_t v = key_word((const unsigned char *)ptr, &d->word[i]);
        memcpy(out + 8 * i, &v, 8);
    }
}

/* ------------------------------------------------------------------ a2 */

/* On a little-endian host every compare that radixsort.c:47-194 selects
 * (native u16/u32/u64, word-wise u64 from the last word, byte-wise from the
 * last byte) orders the rsize bytes as one little-endian unsigned integer. */
int oracle_compar(const void *r1, const void *r2, size_t rsize)
{
    const unsigned char *a = (const unsigned char *)r1;
    const unsigned char *b = (const unsigned char *)r2;
    size_t i = rsize;
    while (i > 0) {
        i--;
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    }
    return 0;
}

/* floor((r1 + r2) / 2) of two rsize-byte little-endian integers; for
 * r1 <= r2 this equals r1 + ((r2 - r1) >> 1) (radixsort.c:59, 111-138). */
void oracle_bisect(void *r, const void *r1, const void *r2, size_t rsize)
{
    const unsigned char *a = (const unsigned char *)r1;
    const unsigned char *b = (const unsigned char *)r2;
    unsigned char *o = (unsigned char *)r;
    unsigned carry = 0;
    size_t i;
    for (i = 0; i < rsize; i++) {          /* sum, least significant first */
        unsigned t = (unsigned)a[i] + b[i] + carry;
        o[i] = (unsigned char)(t & 0xff);
        carry = t >> 8;
    }
    for (i = rsize; i > 0; i--) {          /* shift right by one, top first */
        unsigned t = (unsigned)o[i - 1] | (carry << 8);
        carry = t & 1;
        o[i - 1] = (unsigned char)(t >> 1);
    }
}

/* ------------------------------------------------------------------ a3 */

struct keyed {
    size_t n, elsize, rsize;
    unsigned char *radix;   /* n * rsize bytes, radix of record i at i*rsize */
};

/* Bottom-up stable merge of index runs by radix; ties keep the left run's
 * element first, which is what makes msort.c:76-167 stable. */
static void merge_sort_index(const struct keyed *k, size_t *idx, size_t *tmp)
{
    size_t n = k->n, width, i;
    for (width = 1; width < n; width *= 2) {
        for (i = 0; i < n; i += 2 * width) {
            size_t lo = i, mid = i + width, hi = i + 2 * width, a, b, o;
            if (mid > n) mid = n;
            if (hi > n) hi = n;
            a = lo; b = mid; o = lo;
            while (a < mid && b < hi) {
                if (oracle_compar(k->radix + idx[a] * k->rsize,
                                  k->radix + idx[b] * k->rsize, k->rsize) <= 0)
                    tmp[o++] = idx[a++];
                else
                    tmp[o++] = idx[b++];
            }
            while (a < mid) tmp[o++] = idx[a++];
            while (b < hi) tmp[o++] = idx[b++];
        }
        memcpy(idx, tmp, n * sizeof(size_t));
    }
}

/* Stable sort of n records of elsize bytes by radix() (radix_sort,
 * radixsort.c:35-44).  Returns 0, or -1 if memory runs out. */
int oracle_radix_sort(void *base, size_t n, size_t elsize,
                      oracle_radix_fn radix, size_t rsize, void *arg)
{
    struct keyed k;
    size_t *idx = NULL, *tmp = NULL, i;
    unsigned char *copy = NULL;
    int rc = -1;
    if (n <= 1) return 0;
    k.n = n; k.elsize = elsize; k.rsize = rsize;
    k.radix = (unsigned char *)malloc(n * rsize);
    idx = (size_t *)malloc(n * sizeof(size_t));
    tmp = (size_t *)malloc(n * sizeof(size_t));
    copy = (unsigned char *)malloc(n * elsize);
    if (!k.radix || !idx || !tmp || !copy) goto out;
    for (i = 0; i < n; i++) {
        radix((unsigned char *)base + i * elsize, k.radix + i * rsize, arg);
        idx[i] = i;
    }
    merge_sort_index(&k, idx, tmp);
    memcpy(copy, base, n * elsize);
    for (i = 0; i < n; i++)
        memcpy((unsigned char *)base + i * elsize, copy + idx[i] * elsize, elsize);
    rc = 0;
out:
    free(k.radix); free(idx); free(tmp); free(copy);
    return rc;
}

/* Stable argsort only (used to check permutations). */
int oracle_argsort(const void *base, size_t n, size_t elsize,
                   oracle_radix_fn radix, size_t rsize, void *arg, int64_t *order)
{
    struct keyed k;
    size_t *idx = NULL, *tmp = NULL, i;
    int rc = -1;
    if (n == 0) return 0;
    k.n = n; k.elsize = elsize; k.rsize = rsize;
    k.radix = (unsigned char *)malloc(n * rsize);
    idx = (size_t *)malloc(n * sizeof(size_t));
    tmp = (size_t *)malloc(n * sizeof(size_t));
    if (!k.radix || !idx || !tmp) goto out;
    for (i = 0; i < n; i++) {
        radix((const unsigned char *)base + i * elsize, k.radix + i * rsize, arg);
        idx[i] = i;
    }
    merge_sort_index(&k, idx, tmp);
    for (i = 0; i < n; i++) order[i] = (int64_t)idx[i];
    rc = 0;
out:
    free(k.radix); free(idx); free(tmp);
    return rc;
}

/* ------------------------------------------------------------------ a8 */

/* Index of the last record whose radix is < P (cmp_le == 0) or <= P
 * (cmp_le == 1) in a sorted run, -1 if none (internal-parallel.h:8-83). */
static ptrdiff_t bsearch_last(const unsigned char *P, const unsigned char *sorted_radix,
                              size_t n, size_t rsize, int cmp_le)
{
    ptrdiff_t lo = -1, hi = (ptrdiff_t)n;   /* invariant: [lo] qualifies, [hi] does not */
    while (hi - lo > 1) {
        ptrdiff_t mid = lo + (hi - lo) / 2;
        int c = oracle_compar(sorted_radix + (size_t)mid * rsize, P, rsize);
        if (cmp_le ? (c <= 0) : (c < 0)) lo = mid; else hi = mid;
    }
    return lo;
}

/* CLT[i+1] = #radix < P[i], CLE[i+1] = #radix <= P[i] over one sorted run;
 * CLT[0] = CLE[0] = 0, CLT[np+1] = CLE[np+1] = n (internal-parallel.h:85-126).
 * Exported so device splitter kernels can be pinned against it. */
void oracle_histogram(const unsigned char *P, int np, const unsigned char *sorted_radix,
                      size_t n, size_t rsize, int64_t *CLT, int64_t *CLE)
{
    int i;
    CLT[0] = 0; CLE[0] = 0;
    for (i = 0; i < np; i++) {
        CLT[i + 1] = bsearch_last(P + (size_t)i * rsize, sorted_radix, n, rsize, 0) + 1;
        CLE[i + 1] = bsearch_last(P + (size_t)i * rsize, sorted_radix, n, rsize, 1) + 1;
    }
    CLT[np + 1] = (int64_t)n;
    CLE[np + 1] = (int64_t)n;
}

/* ------------------------------------------------------------------ a7 */

struct piter {
    int np;
    size_t rsize;
    int *stable, *narrow;
    unsigned char *left, *right;
};

static int piter_init(struct piter *pi, const unsigned char *pmin, const unsigned char *pmax,
                      int np, size_t rsize)
{
    int i;
    pi->np = np; pi->rsize = rsize;
    pi->stable = (int *)calloc(np > 0 ? np : 1, sizeof(int));
    pi->narrow = (int *)calloc(np > 0 ? np : 1, sizeof(int));
    pi->left = (unsigned char *)malloc((np > 0 ? np : 1) * rsize);
    pi->right = (unsigned char *)malloc((np > 0 ? np : 1) * rsize);
    if (!pi->stable || !pi->narrow || !pi->left || !pi->right) return -1;
    for (i = 0; i < np; i++) {
        memcpy(pi->left + i * rsize, pmin, rsize);
        memcpy(pi->right + i * rsize, pmax, rsize);
    }
    return 0;
}

static void piter_free(struct piter *pi)
{
    free(pi->stable); free(pi->narrow); free(pi->left); free(pi->right);
}

/* One bisection step over the closed interval [left, right]; when the
 * midpoint no longer moves past `left`, the next step tests `right` itself
 * and the splitter becomes final (internal-parallel.h:150-198). */
static void piter_bisect(struct piter *pi, unsigned char *P)
{
    int i;
    size_t r = pi->rsize;
    for (i = 0; i < pi->np; i++) {
        if (pi->stable[i]) continue;
        if (pi->narrow[i]) {
            memcpy(P + i * r, pi->right + i * r, r);
            pi->stable[i] = 1;
        } else {
            oracle_bisect(P + i * r, pi->left + i * r, pi->right + i * r, r);
            if (oracle_compar(P + i * r, pi->left + i * r, r) <= 0) pi->narrow[i] = 1;
        }
    }
}

/* Accept P[i] when CLT < C <= CLE, else move one end (internal-parallel.h:220-248). */
static void piter_accept(struct piter *pi, const unsigned char *P, const int64_t *C,
                         const int64_t *CLT, const int64_t *CLE)
{
    int i;
    size_t r = pi->rsize;
    for (i = 0; i < pi->np; i++) {
        if (CLT[i + 1] < C[i + 1] && C[i + 1] <= CLE[i + 1]) {
            pi->stable[i] = 1;
        } else if (CLT[i + 1] >= C[i + 1]) {
            memcpy(pi->right + i * r, P + i * r, r);
        } else {
            memcpy(pi->left + i * r, P + i * r, r);
        }
    }
}

static int piter_done(const struct piter *pi)
{
    int i;
    for (i = 0; i < pi->np; i++) if (!pi->stable[i]) return 0;
    return 1;
}

/* ----------------------------------------------------------------- a10 */

/* Send matrix GL_C[sender*(T+1) + receiver] from the per-sender brackets:
 * start from CLT, then give each receiver its deficit from senders 0..T-1
 * in order (mpsort-omp.c:143-204).  Returns 0, or -1 on an inconsistent
 * bracket (where the reference calls abort()). */
int oracle_solve_layout(int T, const int64_t *C, const int64_t *GL_CLT,
                        const int64_t *GL_CLE, int64_t *GL_C)
{
    int T1 = T + 1, i, j;
    for (j = 0; j < T; j++)
        for (i = 0; i < T1; i++) GL_C[j * T1 + i] = GL_CLT[j * T1 + i];
    for (i = 0; i < T; i++) {
        int64_t sure = 0, deficit;
        for (j = 0; j < T; j++) sure += GL_C[j * T1 + i + 1] - GL_C[j * T1 + i];
        deficit = C[i + 1] - C[i] - sure;
        for (j = 0; j < T && deficit != 0; j++) {
            int64_t supply;
            if (deficit < 0) return -1;
            supply = GL_CLE[j * T1 + i + 1] - GL_C[j * T1 + i + 1];
            if (supply < 0) return -1;
            if (supply > deficit) supply = deficit;
            GL_C[j * T1 + i + 1] += supply;
            deficit -= supply;
        }
        if (deficit != 0) return -1;
    }
    return 0;
}

/* ------------------------------------------------------------ a4 - a11 */

/* The T-task histogram sort of mpsort_omp (mpsort-omp.c:47-395), with the
 * tasks executed one after another.  If `splitters_out` is not NULL it
 * receives the T-1 final splitters (rsize bytes each) and `iters_out` the
 * number of bisection rounds.  Returns 0, or -1 on error. */
int oracle_mpsort_tasks(void *base, size_t n, size_t elsize, oracle_radix_fn radix,
                        size_t rsize, void *arg, int T,
                        unsigned char *splitters_out, int *iters_out)
{
    unsigned char *rec = (unsigned char *)base;
    int T1 = T + 1, t, i, iters = 0, rc = -1;
    int64_t *C = NULL, *CLT = NULL, *CLE = NULL, *myCLT = NULL, *myCLE = NULL;
    int64_t *GL_CLT = NULL, *GL_CLE = NULL, *GL_C = NULL;
    unsigned char *P = NULL, *pmin = NULL, *pmax = NULL, *radixbuf = NULL, *outbuf = NULL;
    int have_minmax = 0;
    struct piter pi;
    memset(&pi, 0, sizeof(pi));

    if (n == 0) return 0;                          /* mpsort-omp.c:51 */
    if (T < 1) return -1;

    C = (int64_t *)calloc(T1, sizeof(int64_t));
    CLT = (int64_t *)calloc(T1, sizeof(int64_t));
    CLE = (int64_t *)calloc(T1, sizeof(int64_t));
    myCLT = (int64_t *)calloc(T1, sizeof(int64_t));
    myCLE = (int64_t *)calloc(T1, sizeof(int64_t));
    GL_CLT = (int64_t *)calloc((size_t)T1 * T1, sizeof(int64_t));
    GL_CLE = (int64_t *)calloc((size_t)T1 * T1, sizeof(int64_t));
    GL_C = (int64_t *)calloc((size_t)T1 * T1, sizeof(int64_t));
    P = (unsigned char *)calloc(T, rsize);
    pmin = (unsigned char *)malloc(rsize);
    pmax = (unsigned char *)malloc(rsize);
    radixbuf = (unsigned char *)malloc(n * rsize);
    outbuf = (unsigned char *)malloc(n * elsize);
    if (!C || !CLT || !CLE || !myCLT || !myCLE || !GL_CLT || !GL_CLE || !GL_C ||
        !P || !pmin || !pmax || !radixbuf || !outbuf) goto out;

    for (i = 0; i < T; i++) C[i + 1] = (int64_t)(n * (size_t)(i + 1) / (size_t)T);

    /* first local sort of every chunk (the tasks run on OpenMP threads when
     * built with -fopenmp, as mpsort_omp's do), then the min / max radix */
    {
        int fail = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : fail)
        for (t = 0; t < T; t++) {
            size_t lo = n * (size_t)t / (size_t)T, hi = n * (size_t)(t + 1) / (size_t)T;
            if (oracle_radix_sort(rec + lo * elsize, hi - lo, elsize, radix, rsize, arg)) fail = 1;
        }
        if (fail) goto out;
    }
    {
        long k;
#pragma omp parallel for schedule(static)
        for (k = 0; k < (long)n; k++) radix(rec + (size_t)k * elsize, radixbuf + (size_t)k * rsize, arg);
    }
    for (t = 0; t < T; t++) {
        size_t lo = n * (size_t)t / (size_t)T, hi = n * (size_t)(t + 1) / (size_t)T;
        if (hi == lo) continue;
        if (!have_minmax) {
            memcpy(pmin, radixbuf + lo * rsize, rsize);
            memcpy(pmax, radixbuf + (hi - 1) * rsize, rsize);
            have_minmax = 1;
        } else {
            if (oracle_compar(radixbuf + (hi - 1) * rsize, pmax, rsize) > 0)
                memcpy(pmax, radixbuf + (hi - 1) * rsize, rsize);
            if (oracle_compar(radixbuf + lo * rsize, pmin, rsize) < 0)
                memcpy(pmin, radixbuf + lo * rsize, rsize);
        }
    }

    /* bisection rounds (mpsort-omp.c:273-295) */
    if (piter_init(&pi, pmin, pmax, T - 1, rsize)) goto out;
    do {
        iters++;
        piter_bisect(&pi, P);
        memset(CLT, 0, T1 * sizeof(int64_t));
        memset(CLE, 0, T1 * sizeof(int64_t));
#pragma omp parallel for schedule(static)
        for (t = 0; t < T; t++) {
            size_t lo = n * (size_t)t / (size_t)T, hi = n * (size_t)(t + 1) / (size_t)T;
            oracle_histogram(P, T - 1, radixbuf + lo * rsize, hi - lo, rsize,
                             GL_CLT + (size_t)t * T1, GL_CLE + (size_t)t * T1);
        }
        for (t = 0; t < T; t++)     /* _reduce_sum, in task order */
            for (i = 0; i < T1; i++) {
                CLT[i] += GL_CLT[(size_t)t * T1 + i];
                CLE[i] += GL_CLE[(size_t)t * T1 + i];
            }
        piter_accept(&pi, P, C, CLT, CLE);
    } while (!piter_done(&pi));

    /* final per-task brackets, layout and exchange (mpsort-omp.c:315-369) */
#pragma omp parallel for schedule(static)
    for (t = 0; t < T; t++) {
        size_t lo = n * (size_t)t / (size_t)T, hi = n * (size_t)(t + 1) / (size_t)T;
        oracle_histogram(P, T - 1, radixbuf + lo * rsize, hi - lo, rsize,
                         GL_CLT + (size_t)t * T1, GL_CLE + (size_t)t * T1);
    }
    if (oracle_solve_layout(T, C, GL_CLT, GL_CLE, GL_C)) goto out;
    {
        int r, bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
        for (r = 0; r < T; r++) {   /* receiver r gathers its slices, senders in order */
            size_t o = (size_t)C[r];
            int s2;
            for (s2 = 0; s2 < T; s2++) {
                size_t slo = n * (size_t)s2 / (size_t)T;
                int64_t a = GL_C[(size_t)s2 * T1 + r], b = GL_C[(size_t)s2 * T1 + r + 1];
                memcpy(outbuf + o * elsize, rec + (slo + (size_t)a) * elsize,
                       (size_t)(b - a) * elsize);
                o += (size_t)(b - a);
            }
            if (o != (size_t)C[r + 1]) bad = 1;
        }
        if (bad) goto out;
        memcpy(rec, outbuf, n * elsize);
    }
    /* second local sort of every chunk */
    {
        int fail = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : fail)
        for (t = 0; t < T; t++) {
            size_t lo = n * (size_t)t / (size_t)T, hi = n * (size_t)(t + 1) / (size_t)T;
            if (oracle_radix_sort(rec + lo * elsize, hi - lo, elsize, radix, rsize, arg)) fail = 1;
        }
        if (fail) goto out;
    }
    if (splitters_out && T > 1) memcpy(splitters_out, P, (size_t)(T - 1) * rsize);
    if (iters_out) *iters_out = iters;
    rc = 0;
out:
    piter_free(&pi);
    free(C); free(CLT); free(CLE); free(myCLT); free(myCLE);
    free(GL_CLT); free(GL_CLE); free(GL_C);
    free(P); free(pmin); free(pmax); free(radixbuf); free(outbuf);
    return rc;
}

/* Bisection splitter search of internal-parallel.h over ONE sorted run of
 * radix values with targets C[i+1] = n*(i+1)/(np+1): the CPU statement of
 * the device "plain" splitter search.  Returns the number of rounds. */
int oracle_bisect_splitters(const unsigned char *sorted_radix, size_t n, size_t rsize,
                            int np, unsigned char *P, int64_t *CLT_out, int64_t *CLE_out)
{
    struct piter pi;
    int64_t *C, *CLT, *CLE;
    int i, iters = 0;
    if (n == 0 || np <= 0) return 0;
    C = (int64_t *)calloc(np + 2, sizeof(int64_t));
    CLT = (int64_t *)calloc(np + 2, sizeof(int64_t));
    CLE = (int64_t *)calloc(np + 2, sizeof(int64_t));
    if (!C || !CLT || !CLE) { free(C); free(CLT); free(CLE); return -1; }
    for (i = 0; i <= np; i++) C[i + 1] = (int64_t)(n * (size_t)(i + 1) / (size_t)(np + 1));
    if (piter_init(&pi, sorted_radix, sorted_radix + (n - 1) * rsize, np, rsize)) {
        piter_free(&pi); free(C); free(CLT); free(CLE); return -1;
    }
    do {
        iters++;
        piter_bisect(&pi, P);
        oracle_histogram(P, np, sorted_radix, n, rsize, CLT, CLE);
        piter_accept(&pi, P, C, CLT, CLE);
    } while (!piter_done(&pi));
    oracle_histogram(P, np, sorted_radix, n, rsize, CLT, CLE);
    if (CLT_out) memcpy(CLT_out, CLT, (np + 2) * sizeof(int64_t));
    if (CLE_out) memcpy(CLE_out, CLE, (np + 2) * sizeof(int64_t));
    piter_free(&pi);
    free(C); free(CLT); free(CLE);
    return iters;
}
