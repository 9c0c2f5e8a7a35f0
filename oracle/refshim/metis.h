// Project-written stand-in for the two METIS calls of the reference's assembly (TEST
// INFRASTRUCTURE ONLY; compiled with the reference's sources by oracle/ref.mk):
//   METIS_MeshToDual with ncommon = 1: elements are adjacent when they share a vertex. The
//     neighbour order differs from METIS's, which does not change the reference's results: the
//     breadth-first search visits the same connected set whatever the adjacency order.
//   METIS_PartMeshDual: contiguous blocks of element indices, one per thread. The partition only
//     decides which thread's map an element's contributions go to, i.e. the order of the final sums.
#pragma once
#include <cstdint>

typedef int64_t idx_t;
typedef float real_t;

#define METIS_OK 1
#define METIS_ERROR (-4)

int METIS_MeshToDual(idx_t *ne, idx_t *nn, idx_t *eptr, idx_t *eind, idx_t *ncommon, idx_t *numflag,
                     idx_t **r_xadj, idx_t **r_adjncy);
int METIS_PartMeshDual(idx_t *ne, idx_t *nn, idx_t *eptr, idx_t *eind, idx_t *vwgt, idx_t *vsize,
                       idx_t *ncommon, idx_t *nparts, real_t *tpwgts, idx_t *options, idx_t *objval,
                       idx_t *epart, idx_t *npart);
int METIS_Free(void *ptr);
