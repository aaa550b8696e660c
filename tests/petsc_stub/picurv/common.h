/*
 * common.h (stand-in) -- the data-model types of PICurv's common.h that the reference-signature
 * shim (fdf_gb300/shim/picurv_shim.c) touches, for compiling and testing the shim on a machine
 * without the reference's headers.  The types and field names are the reference's
 * (common.h:46-48, 75-167, 277-356), because the shim reads and writes them; UserCtx carries
 * only the members the shim and its test harness use.  Where the reference is present the shim
 * is compiled against the reference's own headers instead (tests/test_shim.py does both).
 */
#ifndef COMMON_H
#define COMMON_H
#include <petsc.h>
#include <petscdmda.h>
#include <petscdmswarm.h>
#include <stdbool.h>
#include <math.h>

typedef struct UserCtx_s UserCtx;

typedef struct { PetscScalar x, y, z; } Cmpnts;

typedef enum { NEEDS_LOCATION, ACTIVE_AND_LOCATED, MIGRATING_OUT, LOST, UNINITIALIZED } ParticleLocationStatus;

typedef enum { LEFT = 0, RIGHT, BOTTOM, TOP, FRONT, BACK, NUM_FACES } Face;

typedef struct { Cmpnts min_coords; Cmpnts max_coords; } BoundingBox;

typedef struct { Cmpnts vertices[8]; } Cell;

typedef struct {
  PetscInt64 PID;
  PetscInt cell[3];
  Cmpnts loc;
  Cmpnts vel;
  Cmpnts weights;
  ParticleLocationStatus location_status;
  PetscMPIInt destination_rank;
} Particle;

typedef struct { PetscMPIInt rank_xm, rank_xp, rank_ym, rank_yp, rank_zm, rank_zp; } RankNeighbors;

typedef struct { PetscInt xs_cell, ys_cell, zs_cell, xm_cell, ym_cell, zm_cell; } RankCellInfo;

struct UserCtx_s {
  DM da, fda;
  DMDALocalInfo info;
  PetscInt IM, JM, KM;
  BoundingBox bbox;
  RankNeighbors neighbors;
  Vec Ucat, lUcat;
  Vec P, lP;
  DM swarm;
  RankCellInfo *RankCellInfoMap;
  PetscInt NumberofParticles;
  Vec ParticleCount;
  PetscReal dt;
};
#endif
