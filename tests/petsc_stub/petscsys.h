/* Stand-in for <petscsys.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCSYS_H
#define MINIPETSC_PETSCSYS_H
#include "minipetsc.h"
#endif
