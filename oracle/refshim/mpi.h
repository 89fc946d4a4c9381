/* One-rank MPI declarations used to compile the EPREM reference sources into
 * the oracle harness.  Nothing here talks to other processes: the definitions
 * in oracle/ref_shims.c behave as MPI_COMM_WORLD with a single rank.  Test
 * infrastructure, not part of the product. */
#ifndef EPREM_REFSHIM_MPI_H
#define EPREM_REFSHIM_MPI_H
#include <stddef.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Win;
typedef int MPI_Request;
typedef ptrdiff_t MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 1
#define MPI_COMM_TYPE_SHARED 1
#define MPI_INFO_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_THREAD_FUNNELED 1
#define MPI_MODE_NOCHECK 1024
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_UNSIGNED 3
#define MPI_UNSIGNED_LONG 4
#define MPI_MAX 1
#define MPI_MIN 2
double MPI_Wtime(void);
int MPI_Init_thread(int *, char ***, int, int *);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm, int);
int MPI_Barrier(MPI_Comm);
int MPI_Comm_rank(MPI_Comm, int *);
int MPI_Comm_size(MPI_Comm, int *);
int MPI_Comm_split_type(MPI_Comm, int, int, MPI_Info, MPI_Comm *);
int MPI_Get_address(const void *, MPI_Aint *);
int MPI_Type_commit(MPI_Datatype *);
int MPI_Type_contiguous(int, MPI_Datatype, MPI_Datatype *);
int MPI_Type_create_struct(int, const int[], const MPI_Aint[], const MPI_Datatype[], MPI_Datatype *);
int MPI_Type_create_hvector(int, int, MPI_Aint, MPI_Datatype, MPI_Datatype *);
int MPI_Igatherv(const void *, int, MPI_Datatype, void *, const int[], const int[], MPI_Datatype, int, MPI_Comm, MPI_Request *);
int MPI_Iscatterv(const void *, const int[], const int[], MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm, MPI_Request *);
int MPI_Gatherv(const void *, int, MPI_Datatype, void *, const int[], const int[], MPI_Datatype, int, MPI_Comm);
int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *);
int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *);
int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Waitall(int, MPI_Request[], MPI_Status[]);
int MPI_Reduce(const void *, void *, int, MPI_Datatype, MPI_Op, int, MPI_Comm);
int MPI_Allgather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm);
int MPI_Win_allocate_shared(MPI_Aint, int, MPI_Info, MPI_Comm, void *, MPI_Win *);
int MPI_Win_shared_query(MPI_Win, int, MPI_Aint *, int *, void *);
int MPI_Win_lock_all(int, MPI_Win);
int MPI_Win_unlock_all(MPI_Win);
int MPI_Win_sync(MPI_Win);
int MPI_Win_free(MPI_Win *);
#endif
