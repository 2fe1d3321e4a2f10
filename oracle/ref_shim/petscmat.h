/* forwards to the single-rank PETSc stand-in used by the oracle build */
#include "petsc.h"
