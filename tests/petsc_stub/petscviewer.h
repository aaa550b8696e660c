/* Stand-in for <petscviewer.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCVIEWER_H
#define MINIPETSC_PETSCVIEWER_H
#include "minipetsc.h"
#endif
