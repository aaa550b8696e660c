/* Stand-in for <petscsystypes.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCSYSTYPES_H
#define MINIPETSC_PETSCSYSTYPES_H
#include "minipetsc.h"
#endif
