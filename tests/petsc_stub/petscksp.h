/* Stand-in for <petscksp.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCKSP_H
#define MINIPETSC_PETSCKSP_H
#include "minipetsc.h"
#endif
