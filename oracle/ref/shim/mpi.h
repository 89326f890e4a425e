/* Single-rank MPI stand-in used only to build the reference CPU code as the
 * test oracle.  Rank 0 of a world of size 1; point-to-point calls are no-ops
 * because a one-rank run never sends. */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H
#include <sys/time.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_THREAD_FUNNELED 1
#define MPI_SUCCESS 0
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline double MPI_Wtime(void) { struct timeval tv; gettimeofday(&tv, 0); return tv.tv_sec + 1e-6 * tv.tv_usec; }
static inline int MPI_Init(int* a, char*** b) { (void)a; (void)b; return 0; }
static inline int MPI_Init_thread(int* a, char*** b, int req, int* prov) { (void)a; (void)b; *prov = req; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Send(const void* p, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) { (void)p; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0; }
static inline int MPI_Recv(void* p, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status* st) { (void)p; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return 0; }
#ifdef __cplusplus
}
#endif
#endif
