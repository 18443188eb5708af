#define FFTJ_T float
#define FFTJ_COLS_FIXED 1
#define FFTJ_DIR 1
#include "recipes.inc"
