/* interpolation.h (stand-in): the prototypes of interpolation.h (:175-482) that the shim
 * implements, as the reference declares them. */
#ifndef INTERPOLATION_H
#define INTERPOLATION_H
#include "common.h"
PetscErrorCode TrilinearInterpolation_Vector(const char *fieldName, Cmpnts ***fieldVec, PetscInt i, PetscInt j,
                                             PetscInt k, PetscReal a1, PetscReal a2, PetscReal a3, Cmpnts *vec);
PetscErrorCode InterpolateAllFieldsToSwarm(UserCtx *user);
PetscErrorCode ScatterAllParticleFieldsToEulerFields(UserCtx *user);
#endif
