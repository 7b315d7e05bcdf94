/*
 * Data types of the SimpleBubblyFlowSolver C interface, laid out exactly as
 * the reference declares them so that a caller built against the reference
 * headers can hand its structs to this library unchanged:
 *   array_t      include/array.h:10-23
 *   domain_t     include/domain.h:20-30
 *   fluid_t      include/fluid.h:27-45
 *   interface_t  include/interface.h:13-24
 * Only NDIMS == 2 is supported.
 *
 * Storage convention (reference include/array_macros/): every field is
 * x-fastest; array_t.nadds[d][0/1] is the number of extra cells below/above
 * the interior range 1..mysizes[d] in dimension d, so element (I, J) lives at
 *   (I - 1 + nadds[0][0]) + (mysizes[0] + nadds[0][0] + nadds[0][1])
 *                         * (J - 1 + nadds[1][0])
 * in units of array_t.size bytes.  x is wall-bounded (cells 1..nx), y is
 * periodic (cells 1..ny).
 */
#ifndef SBFS_TYPES_H
#define SBFS_TYPES_H

#include <stddef.h>

#ifndef NDIMS
#define NDIMS 2
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sdecomp_info_t_ sdecomp_info_t;

typedef struct {
  size_t size;        /* bytes per element */
  int (*nadds)[2];    /* extra cells per dimension: [dim][lower, upper] */
  size_t datasize;    /* total bytes of data */
  void *data;         /* host buffer */
} array_t;

typedef struct {
  sdecomp_info_t *info;
  size_t glsizes[NDIMS];
  size_t mysizes[NDIMS];
  size_t offsets[NDIMS];
  double lengths[NDIMS];
  double *xf, *xc;       /* x face (nx+1) and centre (nx+2) positions */
  double *jdxf, *jdxc;   /* Jacobians at x faces (nx+1) and centres (nx) */
  double *hxxf, *hxxc;   /* x scale factors at faces (nx+1) and centres (nx) */
  double hy;             /* y grid spacing */
} domain_t;

typedef struct {
  array_t ux;
  array_t uy;
  array_t p;
  array_t psi[2];
  array_t den[2];
  array_t visux;
  array_t visuy;
  array_t txx;
  array_t txy;
  array_t tyy;
  array_t srcux[3];
  array_t srcuy[3];
  double Re;
  double Fr;
  double denr;
  double visr;
  double refden;
} fluid_t;

typedef double vector_t[NDIMS];
typedef double normal_t[NDIMS + 1];

typedef struct {
  array_t vof;
  array_t ifrcx;
  array_t ifrcy;
  array_t dvof;
  array_t normal;
  array_t curv;
  array_t fluxx;
  array_t fluxy;
  array_t src[2];
  double We;
} interface_t;

/* extra cells of every field, as the reference's array macros define them */
#define SBFS_NADDS_UX     {{0, 1}, {1, 1}}
#define SBFS_NADDS_UY     {{1, 1}, {1, 1}}
#define SBFS_NADDS_P      {{1, 1}, {1, 1}}
#define SBFS_NADDS_PSI    {{1, 1}, {1, 1}}
#define SBFS_NADDS_DEN    {{1, 1}, {1, 1}}
#define SBFS_NADDS_VISUX  {{0, 1}, {1, 1}}
#define SBFS_NADDS_VISUY  {{1, 1}, {1, 1}}
#define SBFS_NADDS_TXX    {{0, 0}, {1, 1}}
#define SBFS_NADDS_TXY    {{0, 1}, {1, 1}}
#define SBFS_NADDS_TYY    {{0, 0}, {1, 1}}
#define SBFS_NADDS_SRCUX  {{-1, 0}, {0, 0}}
#define SBFS_NADDS_SRCUY  {{0, 0}, {0, 0}}
#define SBFS_NADDS_VOF    {{1, 1}, {2, 2}}
#define SBFS_NADDS_IFRCX  {{-1, 0}, {0, 0}}
#define SBFS_NADDS_IFRCY  {{0, 0}, {0, 0}}
#define SBFS_NADDS_DVOF   {{0, 1}, {1, 2}}
#define SBFS_NADDS_NORMAL {{0, 0}, {1, 1}}
#define SBFS_NADDS_CURV   {{1, 1}, {1, 1}}
#define SBFS_NADDS_FLUXX  {{0, 1}, {1, 1}}
#define SBFS_NADDS_FLUXY  {{1, 1}, {1, 1}}
#define SBFS_NADDS_SRC    {{0, 0}, {0, 0}}

#ifdef __cplusplus
}
#endif

#endif
