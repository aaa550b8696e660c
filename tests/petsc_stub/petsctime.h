/* Stand-in for <petsctime.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCTIME_H
#define MINIPETSC_PETSCTIME_H
#include "minipetsc.h"
#endif
