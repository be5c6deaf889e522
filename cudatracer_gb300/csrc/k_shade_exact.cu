// Bit-reproducible build of the shading kernels: compiled with -fmad=false,
// transcendentals from portable_math.h (the oracle evaluates the same ones).
#define CT_SHADE_NS exact
#define CT_EXACT 1
#include "k_shade.cuh"
