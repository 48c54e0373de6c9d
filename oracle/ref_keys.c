/*
 * ref_keys.c -- radix() callbacks for driving the UNMODIFIED reference
 * library (oracle/_ref/libref_omp.so, built from radixsort.c and
 * mpsort-omp.c) from ctypes.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference's own callbacks live in the Cython binding
 * (mpsort/binding.pyx:44-121), which cannot be built here (it needs MPI and
 * mpi4py).  These functions compute the same radix bytes: a field of
 * `nmemb` elements at `offset`, each element widened to an order-preserving
 * uint64 (u8 as is, u4 zero-extended, i8/i4 sign-extended plus 2^63).
 */
#include <stdint.h>
#include <string.h>

struct ref_radix_data {
    int64_t offset;   /* byte offset of the key field */
    int32_t kind;     /* 0 = u8, 1 = i8, 2 = u4, 3 = i4 */
    int32_t nmemb;    /* number of key elements (vector fields) */
};

void ref_radix_field(const void *ptr, void *radix, void *arg)
{
    const struct ref_radix_data *d = (const struct ref_radix_data *)arg;
    const unsigned char *p = (const unsigned char *)ptr + d->offset;
    unsigned char *r = (unsigned char *)radix;
    int i;
    for (i = 0; i < d->nmemb; i++) {
        uint64_t v;
        if (d->kind == 0) {
            memcpy(&v, p + 8 * i, 8);
        } else if (d->kind == 1) {
            int64_t s;
            memcpy(&s, p + 8 * i, 8);
            v = (uint64_t)s + 9223372036854775808ull;
        } else if (d->kind == 2) {
            uint32_t u;
            memcpy(&u, p + 4 * i, 4);
            v = u;
        } else {
            int32_t s;
            memcpy(&s, p + 4 * i, 4);
            v = (uint64_t)(int64_t)s + 9223372036854775808ull;
        }
        memcpy(r + 8 * i, &v, 8);
    }
}

/* main.c's callback: the record is an int, the radix is its 4 bytes,
 * compared as an unsigned 32-bit value by radixsort.c:47-63. */
void ref_radix_int(const void *ptr, void *radix, void *arg)
{
    (void)arg;
    memcpy(radix, ptr, 4);
}

/* test-issue7.c's callback: 16-byte radix, low word = 8 bytes at offset 16,
 * high word = 4 bytes at offset 0 (zero-extended). */
void ref_radix_issue7(const void *ptr, void *radix, void *arg)
{
    uint64_t u[2] = {0, 0};
    (void)arg;
    memcpy(&u[0], (const unsigned char *)ptr + 16, 8);
    memcpy(&u[1], (const unsigned char *)ptr + 0, 4);
    memcpy(radix, u, 16);
}
