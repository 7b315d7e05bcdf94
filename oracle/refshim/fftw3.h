/*
 * Stand-in for the subset of FFTW3 that the reference's Poisson solver uses:
 * batched 1-D real-to-real transforms of kinds REDFT10 (DCT-II) and REDFT01
 * (DCT-III) through fftw_plan_many_r2r / fftw_execute, with FFTW's documented
 * unnormalised definitions
 *   REDFT10: Y_k = 2 sum_{j=0}^{n-1} X_j cos(pi (j + 1/2) k / n)
 *   REDFT01: Y_k = X_0 + 2 sum_{j=1}^{n-1} X_j cos(pi j (k + 1/2) / n)
 * so a REDFT10 followed by a REDFT01 multiplies by 2n.  The transforms are
 * evaluated in O(n log n) through a length-n complex FFT (Makhoul's
 * reordering) when n is a power of two, else by the direct sum.
 *
 * As with FFTW, when <complex.h> is included first fftw_complex is the C99
 * double _Complex type.
 *
 * Test infrastructure only (oracle/_ref); never part of the product library.
 */
#ifndef SBFS_REFSHIM_FFTW3_H
#define SBFS_REFSHIM_FFTW3_H

#include <stddef.h>

typedef double _Complex fftw_complex;
typedef struct sbfs_fftw_plan_s *fftw_plan;
typedef enum { FFTW_REDFT00 = 3, FFTW_REDFT01 = 4, FFTW_REDFT10 = 5, FFTW_REDFT11 = 6 } fftw_r2r_kind;

#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_many_r2r(int rank, const int *n, int howmany,
                             double *in, const int *inembed, int istride, int idist,
                             double *out, const int *onembed, int ostride, int odist,
                             const fftw_r2r_kind *kind, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#endif
