// The persistent chemistry kernels with the right-hand side generated for
// the shipped mechanism (chem_gen.cuh): the second translation unit of
// chem.cu, compiled in parallel with the first.
#define IZEM_CHEM_UNIT 1
#include "chem.cu"
