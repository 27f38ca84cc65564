/*
 * Single-rank implementations of the MPI / METIS / ParMETIS / PETSc calls that the
 * reference solver makes.  This file is test infrastructure: it lets the reference's
 * own C sources run as one rank so that they can serve as the oracle that the GPU
 * path is pinned against.  Nothing here is part of the product.
 */
#include <string.h>
#include <time.h>
#include "mpi.h"
#include "parmetis.h"

static size_t dt_size(MPI_Datatype dt) {
  switch (dt) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG: return sizeof(long);
    default: return 1;
  }
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
/* with one rank the reference never sends to itself; returning is enough */
int MPI_Send(const void *b, int n, MPI_Datatype d, int t, int g, MPI_Comm c) {
  (void)b; (void)n; (void)d; (void)t; (void)g; (void)c; return 0; }
int MPI_Recv(void *b, int n, MPI_Datatype d, int s, int g, MPI_Comm c, MPI_Status *st) {
  (void)b; (void)n; (void)d; (void)s; (void)g; (void)c; (void)st; return 0; }
int MPI_Isend(const void *b, int n, MPI_Datatype d, int t, int g, MPI_Comm c, MPI_Request *r) {
  (void)b; (void)n; (void)d; (void)t; (void)g; (void)c; *r = 0; return 0; }
int MPI_Irecv(void *b, int n, MPI_Datatype d, int s, int g, MPI_Comm c, MPI_Request *r) {
  (void)b; (void)n; (void)d; (void)s; (void)g; (void)c; *r = 0; return 0; }
int MPI_Wait(MPI_Request *r, MPI_Status *s) { (void)r; (void)s; return 0; }
int MPI_Request_free(MPI_Request *r) { (void)r; return 0; }
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype d, MPI_Op o, MPI_Comm c) {
  (void)o; (void)c;
  if (s != r) memmove(r, s, (size_t)n * dt_size(d));
  return 0;
}
int MPI_Bcast(void *b, int n, MPI_Datatype d, int root, MPI_Comm c) {
  (void)b; (void)n; (void)d; (void)root; (void)c; return 0; }

/* one partition: every graph vertex goes to part 0 */
int METIS_PartGraphRecursive(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy,
                             idx_t *vwgt, idx_t *vsize, idx_t *adjwgt, idx_t *nparts,
                             real_t *tpwgts, real_t *ubvec, idx_t *options, idx_t *objval,
                             idx_t *part) {
  (void)ncon; (void)xadj; (void)adjncy; (void)vwgt; (void)vsize; (void)adjwgt;
  (void)nparts; (void)tpwgts; (void)ubvec; (void)options;
  for (idx_t i = 0; i < *nvtxs; ++i) part[i] = 0;
  *objval = 0;
  return 1;
}
int ParMETIS_V3_AdaptiveRepart(idx_t *vtxdist, idx_t *xadj, idx_t *adjncy, idx_t *vwgt,
                               idx_t *vsize, idx_t *adjwgt, idx_t *wgtflag, idx_t *numflag,
                               idx_t *ncon, idx_t *nparts, real_t *tpwgts, real_t *ubvec,
                               real_t *ipc2redist, idx_t *options, idx_t *edgecut,
                               idx_t *part, MPI_Comm *comm) {
  (void)xadj; (void)adjncy; (void)vwgt; (void)vsize; (void)adjwgt; (void)wgtflag;
  (void)numflag; (void)ncon; (void)nparts; (void)tpwgts; (void)ubvec; (void)ipc2redist;
  (void)options; (void)comm;
  for (idx_t i = 0; i < vtxdist[1] - vtxdist[0]; ++i) part[i] = 0;
  *edgecut = 0;
  return 1;
}
int PetscInitialize(int *argc, char ***argv, const char *file, const char *help) {
  (void)argc; (void)argv; (void)file; (void)help; return 0; }
