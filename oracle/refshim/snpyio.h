/*
 * Stand-in for the header part of SimpleNpyIO (the reference's submodule,
 * empty in the snapshot, version unknown), written from the published NPY
 * format specification (format version 1.0: magic "\x93NUMPY", two version
 * bytes, a little-endian uint16 header length, then a Python dict literal
 * with 'descr', 'fortran_order' and 'shape', padded with spaces and ended by
 * a newline so that the data start at a multiple of 64 bytes; version 2.0
 * differs only by a uint32 length).  The signatures are the ones the
 * reference's src/fileio.c calls (r_npy_header, w_npy_header).
 *
 * Test infrastructure only: lets oracle/_ref compile the reference's own
 * src/fileio.c, src/array.c and the statistics / save paths on top of it.
 */
#ifndef SBFS_REFSHIM_SNPYIO_H
#define SBFS_REFSHIM_SNPYIO_H

#include <stdbool.h>
#include <stddef.h>
#include <stdio.h>

/* writes the header at the start of fp; *header_size = bytes written */
int snpyio_w_header(const size_t ndims, const size_t *shape, const char dtype[], const bool is_fortran_order,
                    FILE *fp, size_t *header_size);

/* reads the header at the start of fp; *shape and *dtype are heap-allocated
 * (the caller frees them); dtype keeps its quotes, e.g. "'<f8'" */
int snpyio_r_header(size_t *ndims, size_t **shape, char **dtype, bool *is_fortran_order, FILE *fp,
                    size_t *header_size);

#endif
