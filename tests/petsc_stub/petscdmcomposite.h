/* Stand-in for <petscdmcomposite.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCDMCOMPOSITE_H
#define MINIPETSC_PETSCDMCOMPOSITE_H
#include "minipetsc.h"
#endif
