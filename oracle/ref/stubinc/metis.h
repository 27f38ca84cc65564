/* Single-rank stand-in for the METIS interface (oracle build only). */
#ifndef FFV_STUB_METIS_H
#define FFV_STUB_METIS_H
#include <stdint.h>
typedef int32_t idx_t;
typedef float real_t;
int METIS_PartGraphRecursive(idx_t *nvtxs, idx_t *ncon, idx_t *xadj, idx_t *adjncy,
                             idx_t *vwgt, idx_t *vsize, idx_t *adjwgt, idx_t *nparts,
                             real_t *tpwgts, real_t *ubvec, idx_t *options, idx_t *objval,
                             idx_t *part);
#endif
