/* Single-rank stand-in for the MPI interface the MAPP sources use, so that
 * the reference compiles (unmodified, from where it lies) into a Python
 * module that serves as a second oracle.  Test infrastructure only.
 *
 * World size is 1.  Collectives copy send buffers to receive buffers; a
 * Sendrecv to the only rank copies; Send/Recv pair through a small FIFO;
 * Cartesian topologies are 1 x 1 x 1 with periodic self-neighbours.
 * A datatype handle is its element size in bytes.
 */
#ifndef MAPPG_REF_MPI_SHIM_H
#define MAPPG_REF_MPI_SHIM_H

#include <stddef.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_SUCCESS 0
#define MPI_UNDEFINED (-32766)
#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_UNSIGNED_CHAR ((MPI_Datatype)sizeof(unsigned char))
#define MPI_SHORT ((MPI_Datatype)sizeof(short))
#define MPI_UNSIGNED_SHORT ((MPI_Datatype)sizeof(unsigned short))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_UNSIGNED ((MPI_Datatype)sizeof(unsigned))
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_UNSIGNED_LONG ((MPI_Datatype)sizeof(unsigned long))
#define MPI_LONG_LONG ((MPI_Datatype)sizeof(long long))
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)sizeof(unsigned long long))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_LONG_DOUBLE ((MPI_Datatype)sizeof(long double))
#define MPI_CXX_BOOL ((MPI_Datatype)sizeof(bool))

#ifdef __cplusplus
extern "C" {
#endif
int MPI_Init(int* argc, char*** argv);
int MPI_Initialized(int* flag);
int MPI_Finalize(void);
int MPI_Finalized(int* flag);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* out);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int* result);
int MPI_Barrier(MPI_Comm comm);
int MPI_Get_processor_name(char* name, int* len);
int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Scan(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Sendrecv(const void* send, int scount, MPI_Datatype st, int dest, int stag,
                 void* recv, int rcount, MPI_Datatype rt, int source, int rtag,
                 MPI_Comm comm, MPI_Status* status);
int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Cart_create(MPI_Comm comm, int ndims, const int* dims, const int* periods, int reorder, MPI_Comm* out);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* source, int* dest);
#ifdef __cplusplus
}
#endif

#endif
