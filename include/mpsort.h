/*
 * mpsort.h -- drop-in for MP-sort's single-node entry points, served by the
 * GB300 sort in libgbsort.so.
 *
 *   radix_sort   replaces radix_sort   (reference mpsort.h:1-4,  radixsort.c:35-44)
 *   mpsort_omp   replaces mpsort_omp   (reference mpsort.h:8-12, mpsort-omp.c:47-74)
 *
 * Same signatures and the same result: `base` (host memory) is sorted in
 * place, ascending by the rsize radix bytes that radix() writes, compared as
 * a little-endian unsigned integer, ties in input order.  The reference's
 * mpsort_omp prints per-stage timings to stdout (mpsort-omp.c:269-392); this
 * one prints nothing.
 *
 * A host radix() cannot run on the GPU.  Pass `mpsort_radix_desc` as the
 * callback and a gbsort_key_desc as `arg` to let the GPU read the key from
 * the records itself; any other callback is evaluated on the host once per
 * record and the GPU sorts by the bytes it produced.
 *
 * The reference returns void and aborts on inconsistency; these return void
 * and never abort.  On failure (no GPU, out of memory) the data is left
 * unsorted, a message goes to stderr and mpsort_last_status() returns the
 * gbsort_status.
 */
#ifndef GBSORT_MPSORT_H
#define GBSORT_MPSORT_H

#include <stddef.h>
#include <stdint.h>

#include "gbsort_key.h"

#ifdef __cplusplus
extern "C" {
#endif

GBSORT_API void radix_sort(void *base, size_t nmemb, size_t size,
                void (*radix)(const void *ptr, void *radix, void *arg),
                size_t rsize, void *arg);

GBSORT_API void mpsort_omp(void *base, size_t nmemb, size_t size,
                void (*radix)(const void *ptr, void *radix, void *arg),
                size_t rsize, void *arg);

/* The key-descriptor radix: a real host function (arg = const
 * gbsort_key_desc *) writing nwords * 8 bytes as binding.pyx:81-121 does;
 * passing it as `radix` selects the on-device key path. */
GBSORT_API void mpsort_radix_desc(const void *ptr, void *radix, void *arg);

/* gbsort_status of the last radix_sort / mpsort_omp call on this thread. */
GBSORT_API int mpsort_last_status(void);

/* The reference's tuning flags (mpsort.h:17-24).  They steer the MPI data
 * exchange, which a single GPU does not have; they are accepted and stored so
 * callers that set them keep working. */
#define MPSORT_DISABLE_SPARSE_ALLTOALLV (1 << 1)
#define MPSORT_DISABLE_GATHER_SORT (1 << 3)
#define MPSORT_REQUIRE_GATHER_SORT (1 << 4)
#define MPSORT_REQUIRE_SPARSE_ALLTOALLV (1 << 6)

GBSORT_API void mpsort_mpi_set_options(int options);
GBSORT_API int mpsort_mpi_has_options(int options);
GBSORT_API void mpsort_mpi_unset_options(int options);

/* One-process forms of the reference's MPI entry points (reference
 * mpsort.h:26-47, mpsort-mpi.c:129-331), for callers that link against the
 * MPI interface but run one rank per GPU.  The communicator is taken as an
 * opaque integer and not read (the MPI_Comm handle of either common MPI
 * ABI passes in one register; a multi-rank sort is outside this library).
 * As in the reference with one rank, base ends sorted and out receives the
 * sorted records (outnmemb must equal nmemb, else nothing is sorted and the
 * status is GBSORT_ERR_BAD_ARG).  With mpsort_radix_desc the sort is
 * self-checked by a multiset hash of the records before and after, as the
 * reference checks its checksum.  Status: mpsort_last_status(). */
GBSORT_API void mpsort_mpi_newarray_impl(void *base, size_t nmemb, void *out, size_t outnmemb, size_t elsize,
                                         void (*radix)(const void *ptr, void *radix, void *arg),
                                         size_t rsize, void *arg, intptr_t comm, int line, const char *file);
GBSORT_API void mpsort_mpi_impl(void *base, size_t nmemb, size_t elsize,
                                void (*radix)(const void *ptr, void *radix, void *arg),
                                size_t rsize, void *arg, intptr_t comm, int line, const char *file);
/* Prints the stage times of the last sort on this thread (reference
 * mpsort.h:49). */
GBSORT_API void mpsort_mpi_report_last_run(void);

#define mpsort_mpi(base, nmemb, elsize, radix, rsize, arg, comm) \
    mpsort_mpi_impl(base, nmemb, elsize, radix, rsize, arg, (intptr_t)(comm), __LINE__, __FILE__)
#define mpsort_mpi_newarray(base, nmemb, out, outnmemb, elsize, radix, rsize, arg, comm) \
    mpsort_mpi_newarray_impl(base, nmemb, out, outnmemb, elsize, radix, rsize, arg, (intptr_t)(comm), \
                             __LINE__, __FILE__)

#ifdef __cplusplus
}
#endif

#endif /* GBSORT_MPSORT_H */
