#define FFTJ_T double
#define FFTJ_DIR 1
#include "recipes.inc"
