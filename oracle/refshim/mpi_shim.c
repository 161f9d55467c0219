/* Single-rank MPI stand-in: see mpi.h.  Test infrastructure only. */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>

static int g_init = 0, g_fin = 0;

int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; g_init = 1; return 0; }
int MPI_Initialized(int* flag) { *flag = g_init; return 0; }
int MPI_Finalize(void) { g_fin = 1; return 0; }
int MPI_Finalized(int* flag) { *flag = g_fin; return 0; }
int MPI_Comm_rank(MPI_Comm comm, int* rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, int* size) { (void)comm; *size = 1; return 0; }

int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* out)
{
    (void)comm; (void)key;
    *out = (color == MPI_UNDEFINED) ? MPI_COMM_NULL : MPI_COMM_WORLD;
    return 0;
}

int MPI_Comm_free(MPI_Comm* comm) { *comm = MPI_COMM_NULL; return 0; }

int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int* result)
{
    *result = (a == b) ? MPI_IDENT : MPI_CONGRUENT;
    return 0;
}

int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }

int MPI_Get_processor_name(char* name, int* len)
{
    snprintf(name, MPI_MAX_PROCESSOR_NAME, "localhost");
    *len = (int)strlen(name);
    return 0;
}

static void copy_elems(void* dst, const void* src, int count, MPI_Datatype t)
{
    if (dst != src && count > 0) memmove(dst, src, (size_t)count * (size_t)t);
}

int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    copy_elems(recv, send, count, t);
    return 0;
}

int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm)
{
    (void)op; (void)root; (void)comm;
    copy_elems(recv, send, count, t);
    return 0;
}

int MPI_Scan(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    copy_elems(recv, send, count, t);
    return 0;
}

int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm)
{
    (void)buf; (void)count; (void)t; (void)root; (void)comm;
    return 0;
}

int MPI_Sendrecv(const void* send, int scount, MPI_Datatype st, int dest, int stag,
                 void* recv, int rcount, MPI_Datatype rt, int source, int rtag,
                 MPI_Comm comm, MPI_Status* status)
{
    (void)dest; (void)stag; (void)source; (void)rtag; (void)comm;
    size_t sb = (size_t)scount * (size_t)st, rb = (size_t)rcount * (size_t)rt;
    size_t nb = sb < rb ? sb : rb;
    if (nb && recv != send) memmove(recv, send, nb);
    if (status) { status->MPI_SOURCE = 0; status->MPI_TAG = rtag; status->MPI_ERROR = 0; }
    return 0;
}

/* Send/Recv to the only rank: a FIFO of copied messages. */
typedef struct Msg { struct Msg* next; size_t n; char data[]; } Msg;
static Msg *g_head = NULL, *g_tail = NULL;

int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm)
{
    (void)dest; (void)tag; (void)comm;
    size_t n = (size_t)count * (size_t)t;
    Msg* m = (Msg*)malloc(sizeof(Msg) + n);
    if (!m) return 1;
    m->next = NULL;
    m->n = n;
    if (n) memcpy(m->data, buf, n);
    if (g_tail) g_tail->next = m; else g_head = m;
    g_tail = m;
    return 0;
}

int MPI_Recv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Status* status)
{
    (void)source; (void)tag; (void)comm;
    Msg* m = g_head;
    if (!m) {
        fprintf(stderr, "single-rank MPI shim: MPI_Recv without a matching MPI_Send\n");
        abort();
    }
    g_head = m->next;
    if (!g_head) g_tail = NULL;
    size_t n = (size_t)count * (size_t)t;
    memcpy(buf, m->data, n < m->n ? n : m->n);
    free(m);
    if (status) { status->MPI_SOURCE = 0; status->MPI_TAG = tag; status->MPI_ERROR = 0; }
    return 0;
}

int MPI_Cart_create(MPI_Comm comm, int ndims, const int* dims, const int* periods, int reorder, MPI_Comm* out)
{
    (void)comm; (void)ndims; (void)dims; (void)periods; (void)reorder;
    *out = MPI_COMM_WORLD;
    return 0;
}

int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords)
{
    (void)comm;
    for (int i = 0; i < maxdims; i++) { dims[i] = 1; periods[i] = 1; coords[i] = 0; }
    return 0;
}

int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* source, int* dest)
{
    (void)comm; (void)direction; (void)disp;
    *source = 0;
    *dest = 0;
    return 0;
}
