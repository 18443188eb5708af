#define FFTJ_T Fx  // ComplexF64 data, block fixed-point compute (fx64.cuh)
#define FFTJ_DIR -1
#include "recipes.inc"
