#define FFTJ_T float
#define FFTJ_DIR -1
#include "recipes.inc"
