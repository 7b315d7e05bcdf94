/*
 * Batched DCT-II / DCT-III along a contiguous axis, with FFTW's unnormalised
 * REDFT10 / REDFT01 definitions (a DCT-II followed by a DCT-III multiplies by
 * 2n).  Power-of-two lengths go through a length-n complex radix-2 FFT using
 * Makhoul's even/odd reordering; other lengths use the direct O(n^2) sum.
 *
 * Test infrastructure (CPU oracle and the FFTW stand-in of oracle/_ref).
 */
#ifndef SBFS_ORACLE_DCT_H
#define SBFS_ORACLE_DCT_H

typedef struct sbfs_dct_plan_s sbfs_dct_plan;

sbfs_dct_plan *sbfs_dct_plan_create(int n);
void sbfs_dct_plan_destroy(sbfs_dct_plan *plan);
int sbfs_dct_plan_size(const sbfs_dct_plan *plan);
/* y = REDFT10(x); work must hold 4 n doubles; x and y may alias */
void sbfs_dct2(const sbfs_dct_plan *plan, const double *x, double *y, double *work);
/* y = REDFT01(x); work must hold 4 n doubles; x and y may alias */
void sbfs_dct3(const sbfs_dct_plan *plan, const double *x, double *y, double *work);

#endif
