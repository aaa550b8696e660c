/* ParticleMotion.h (stand-in): the prototypes of ParticleMotion.h (:29-405) that the shim
 * implements, as the reference declares them. */
#ifndef PARTICLE_MOTION_H
#define PARTICLE_MOTION_H
#include "common.h"
PetscErrorCode UpdateParticlePosition(UserCtx *user, Cmpnts *position, const Cmpnts *velocity);
PetscErrorCode UpdateAllParticlePositions(UserCtx *user);
PetscErrorCode CheckAndRemoveOutOfBoundsParticles(UserCtx *user, PetscInt *removedCountLocal,
                                                  PetscInt *removedCountGlobal, const BoundingBox *bboxlist);
PetscErrorCode CheckAndRemoveLostParticles(UserCtx *user, PetscInt *removedCountLocal, PetscInt *removedCountGlobal);
PetscErrorCode CalculateParticleCountPerCell(UserCtx *user);
PetscErrorCode LocateAllParticlesInGrid_TEST(UserCtx *user, BoundingBox *bboxlist);
PetscErrorCode ResetAllParticleStatuses(UserCtx *user);
#endif
