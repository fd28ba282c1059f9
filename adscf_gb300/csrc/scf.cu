// scf.cu -- the single definition of the geometry-independent SCF kernels.
#define ADSCF_SCF_IMPL
#include "internal.h"
