/* Stand-in for <petscvec.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCVEC_H
#define MINIPETSC_PETSCVEC_H
#include "minipetsc.h"
#endif
