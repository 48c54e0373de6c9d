/*
 * gbsort_key.h -- the device key descriptor.
 *
 * MP-sort asks the caller for a host function `radix(ptr, radix, arg)` that
 * writes `rsize` bytes of sort key for one record (mpsort.h:1-4).  A host
 * function pointer cannot run on the GPU, so this library describes the key
 * as data instead: up to GBSORT_MAX_KEY_WORDS integer fields of the record,
 * each mapped to an order-preserving unsigned 64-bit word exactly as the
 * Python binding's radix functions do (mpsort/binding.pyx:81-121):
 *
 *   u8 -> the value itself          i8 -> (uint64)value + 2^63
 *   u4 -> zero-extended to 64 bits  i4 -> (uint64)(int64)value + 2^63
 *
 * The resulting radix is `nwords * 8` bytes, word 0 first in memory and the
 * LAST word the most significant (the multi-word compare of radixsort.c:82-98
 * on a little-endian host, and the vector-key rule of binding.pyx:136-137).
 * Words may come from different fields, which also covers hand-written
 * composite keys such as the 16-byte radix of test-issue7.c:12-17.
 */
#ifndef GBSORT_KEY_H
#define GBSORT_KEY_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBSORT_MAX_KEY_WORDS 4

/* Symbols of the public ABI (the library is built with hidden visibility). */
#if defined(__GNUC__)
#define GBSORT_API __attribute__((visibility("default")))
#else
#define GBSORT_API
#endif

typedef struct gbsort_key_word {
    uint32_t offset;     /* byte offset of the field inside the record */
    uint32_t width;      /* 4 or 8 bytes */
    uint32_t is_signed;  /* 0: unsigned field, 1: two's complement field */
    uint32_t reserved;   /* must be 0 */
} gbsort_key_word;

typedef struct gbsort_key_desc {
    uint32_t nwords;     /* 1 .. GBSORT_MAX_KEY_WORDS; word[nwords-1] is most significant */
    uint32_t reserved;   /* must be 0 */
    gbsort_key_word word[GBSORT_MAX_KEY_WORDS];
} gbsort_key_desc;

#ifdef __cplusplus
}
#endif

#endif /* GBSORT_KEY_H */
