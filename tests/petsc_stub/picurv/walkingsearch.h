/* walkingsearch.h (stand-in): the prototypes of walkingsearch.h (:34-383) that the shim
 * implements, as the reference declares them. */
#ifndef WALKINGSEARCH_H
#define WALKINGSEARCH_H
#include "common.h"
PetscErrorCode GetCellCharacteristicSize(const Cell *cell, PetscReal *cellSize);
PetscErrorCode ComputeSignedDistanceToPlane(const Cmpnts v1, const Cmpnts v2, const Cmpnts v3, const Cmpnts v4,
                                            const Cmpnts cell_centroid, const Cmpnts p_target, PetscReal *d_signed,
                                            const PetscReal threshold);
PetscErrorCode CalculateDistancesToCellFaces(const Cmpnts p, const Cell *cell, PetscReal *d, const PetscReal threshold);
PetscErrorCode DeterminePointPosition(PetscReal *d, PetscInt *result);
PetscErrorCode GetCellVerticesFromGrid(Cmpnts ***coor, PetscInt idx, PetscInt idy, PetscInt idz, Cell *cell);
PetscErrorCode EvaluateParticlePosition(const Cell *cell, PetscReal *d, const Cmpnts p, PetscInt *position,
                                        const PetscReal threshold);
PetscErrorCode LocateParticleOrFindMigrationTarget_TEST(UserCtx *user, Particle *particle,
                                                        ParticleLocationStatus *status_out);
PetscErrorCode UpdateCellIndicesBasedOnDistancesTEST(PetscReal d[NUM_FACES], PetscInt *idx, PetscInt *idy,
                                                     PetscInt *idz);
#endif
