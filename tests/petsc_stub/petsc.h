/* Stand-in for <petsc.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSC_H
#define MINIPETSC_PETSC_H
#include "minipetsc.h"
#endif
