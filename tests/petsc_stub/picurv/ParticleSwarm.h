/* ParticleSwarm.h (stand-in): UpdateParticleWeights (ParticleSwarm.h:239) as the reference declares it. */
#ifndef PARTICLE_SWARM_H
#define PARTICLE_SWARM_H
#include "common.h"
PetscErrorCode UpdateParticleWeights(PetscReal *d, Particle *particle);
#endif
