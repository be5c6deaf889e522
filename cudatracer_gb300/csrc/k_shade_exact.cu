// Bit-reproducible build of the shading kernels: compiled with -fmad=false,
// transcendentals evaluated in double and rounded once.
#define CT_SHADE_NS exact
#define CT_EXACT 1
#include "k_shade.cuh"
