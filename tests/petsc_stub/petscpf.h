/* Stand-in for <petscpf.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_PETSCPF_H
#define MINIPETSC_PETSCPF_H
#include "minipetsc.h"
#endif
