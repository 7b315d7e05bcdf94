/*
 * Single-rank stand-in for the SimpleDecomp pencil-decomposition API, written
 * from how the reference solver calls it (the submodule's source is not part
 * of the reference snapshot).  With one rank:
 *   - every pencil holds the whole domain (size = global size, offset = 0);
 *   - y is periodic, so both y neighbours are rank 0 itself; x neighbours
 *     are MPI_PROC_NULL (walls);
 *   - an x1 -> y1 transpose turns an x-fastest (ny, nx) array into a
 *     y-fastest (nx, ny) array, and y1 -> x1 is the inverse.
 *
 * Test infrastructure only (oracle/_ref); never part of the product library.
 */
#ifndef SBFS_REFSHIM_SDECOMP_H
#define SBFS_REFSHIM_SDECOMP_H

#include <stddef.h>
#include <stdbool.h>
#include <mpi.h>

typedef enum { SDECOMP_XDIR = 0, SDECOMP_YDIR = 1, SDECOMP_ZDIR = 2 } sdecomp_dir_t;
typedef enum { SDECOMP_X1PENCIL = 0, SDECOMP_Y1PENCIL = 1 } sdecomp_pencil_t;

typedef struct sdecomp_info_t_ sdecomp_info_t;
typedef struct sdecomp_transpose_plan_t_ sdecomp_transpose_plan_t;

typedef struct {
  int (* const construct)(const sdecomp_info_t *info, const sdecomp_pencil_t from,
                          const sdecomp_pencil_t to, const size_t *glsizes,
                          const size_t size, sdecomp_transpose_plan_t **plan);
  int (* const execute)(sdecomp_transpose_plan_t *plan, const void *sendbuf, void *recvbuf);
  int (* const destruct)(sdecomp_transpose_plan_t *plan);
} sdecomp_transpose_t;

typedef struct {
  int (* const construct)(const MPI_Comm comm_default, const size_t ndims, const size_t *dims,
                          const bool *periods, sdecomp_info_t **info);
  int (* const destruct)(sdecomp_info_t *info);
  int (* const get_comm_cart)(const sdecomp_info_t *info, MPI_Comm *comm_cart);
  int (* const get_comm_rank)(const sdecomp_info_t *info, int *rank);
  int (* const get_neighbours)(const sdecomp_info_t *info, const sdecomp_pencil_t pencil,
                               const sdecomp_dir_t dir, int neighbours[2]);
  int (* const get_pencil_mysize)(const sdecomp_info_t *info, const sdecomp_pencil_t pencil,
                                  const sdecomp_dir_t dir, const size_t glsize, size_t *mysize);
  int (* const get_pencil_offset)(const sdecomp_info_t *info, const sdecomp_pencil_t pencil,
                                  const sdecomp_dir_t dir, const size_t glsize, size_t *offset);
  sdecomp_transpose_t transpose;
} sdecomp_t;

extern const sdecomp_t sdecomp;

#endif
