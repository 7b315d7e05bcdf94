/*
 * Single-rank stand-in for the subset of MPI that the reference solver's
 * time-step sources call (halo exchange, reductions, abort).  Written from
 * the MPI standard's documented semantics for a communicator of size one:
 *   - every collective copies its send buffer to its receive buffer (or does
 *     nothing for MPI_IN_PLACE);
 *   - MPI_Sendrecv to/from rank 0 (self) is a memcpy, which is exactly the
 *     periodic y wrap the reference's halo exchange performs on one rank;
 *   - MPI_PROC_NULL peers send/receive nothing.
 * A datatype handle is its extent in bytes, so MPI_Type_contiguous multiplies.
 *
 * Test infrastructure only: used to build the reference's own C sources into
 * oracle/_ref for parity checks.  Never part of the product library.
 */
#ifndef SBFS_REFSHIM_MPI_H
#define SBFS_REFSHIM_MPI_H

#include <stddef.h>

typedef int MPI_Comm;
typedef long MPI_Datatype;   /* extent in bytes */
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_COMM_NULL ((MPI_Comm)-1)
#define MPI_PROC_NULL (-2)
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 64

#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_DATATYPE_NULL ((MPI_Datatype)0)

#define MPI_MIN ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_SUM ((MPI_Op)3)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *type);
int MPI_Type_free(MPI_Datatype *type);
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status);
double MPI_Wtime(void);

/* MPI-IO on one rank (src/fileio.c): a file handle is a stdio stream; a
 * subarray file type must cover its whole array (one rank owns everything),
 * so a file view is the data offset after the NPY header and the collective
 * read / write are fread / fwrite of count elements of the given extent */
typedef struct sbfs_mpi_file_s *MPI_File;
typedef long MPI_Offset;
typedef int MPI_Info;
#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_MODE_CREATE 1
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_RDWR 8
#define MPI_ORDER_C 56
#define MPI_ERR_OTHER 15
int MPI_File_open(MPI_Comm comm, const char *filename, int amode, MPI_Info info, MPI_File *fh);
int MPI_File_close(MPI_File *fh);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype, const char *datarep,
                      MPI_Info info);
int MPI_File_read_all(MPI_File fh, void *buf, int count, MPI_Datatype type, MPI_Status *status);
int MPI_File_write_all(MPI_File fh, const void *buf, int count, MPI_Datatype type, MPI_Status *status);
int MPI_Type_create_subarray(int ndims, const int sizes[], const int subsizes[], const int starts[], int order,
                             MPI_Datatype oldtype, MPI_Datatype *newtype);
int MPI_Error_string(int errorcode, char *string, int *resultlen);

#endif
