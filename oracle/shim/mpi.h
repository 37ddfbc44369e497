/* Stand-in for MPI so the reference sources compile without an MPI library.
 * The point-to-point calls only appear in the global-fit exchange code, which
 * the oracle never calls; they are no-ops here. */
#ifndef GLASS_ORACLE_SHIM_MPI_H
#define GLASS_ORACLE_SHIM_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
static inline int MPI_Send(const void *b, int c, MPI_Datatype t, int d, int g, MPI_Comm m) { (void)b; (void)c; (void)t; (void)d; (void)g; (void)m; return 0; }
static inline int MPI_Recv(void *b, int c, MPI_Datatype t, int s, int g, MPI_Comm m, MPI_Status *st) { (void)b; (void)c; (void)t; (void)s; (void)g; (void)m; (void)st; return 0; }
#endif
