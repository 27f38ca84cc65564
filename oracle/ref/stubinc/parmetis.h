/* Single-rank stand-in for the ParMETIS interface (oracle build only). */
#ifndef FFV_STUB_PARMETIS_H
#define FFV_STUB_PARMETIS_H
#include "metis.h"
#include <mpi.h>
int ParMETIS_V3_AdaptiveRepart(idx_t *vtxdist, idx_t *xadj, idx_t *adjncy, idx_t *vwgt,
                               idx_t *vsize, idx_t *adjwgt, idx_t *wgtflag, idx_t *numflag,
                               idx_t *ncon, idx_t *nparts, real_t *tpwgts, real_t *ubvec,
                               real_t *ipc2redist, idx_t *options, idx_t *edgecut,
                               idx_t *part, MPI_Comm *comm);
#endif
