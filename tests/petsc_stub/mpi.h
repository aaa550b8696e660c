/* Stand-in for <mpi.h>: everything is in minipetsc.h. */
#ifndef MINIPETSC_MPI_H
#define MINIPETSC_MPI_H
#include "minipetsc.h"
#endif
