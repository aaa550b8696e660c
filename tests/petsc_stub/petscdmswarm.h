/* Stand-in for <petscdmswarm.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCDMSWARM_H
#define MINIPETSC_PETSCDMSWARM_H
#include "minipetsc.h"
#endif
