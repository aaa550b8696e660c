/* Stand-in for <petscerror.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCERROR_H
#define MINIPETSC_PETSCERROR_H
#include "minipetsc.h"
#endif
