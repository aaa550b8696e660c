/* Stand-in for <petscdm.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCDM_H
#define MINIPETSC_PETSCDM_H
#include "minipetsc.h"
#endif
