/* Stand-in for <petscdmda.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCDMDA_H
#define MINIPETSC_PETSCDMDA_H
#include "minipetsc.h"
#endif
