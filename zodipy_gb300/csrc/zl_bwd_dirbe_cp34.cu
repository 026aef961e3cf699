// The component-paired DIRBE adjoint launches for three or four spectral sets: the same
// source as zl_bwd_dirbe_cp.cu, compiled a second time in parallel with it.
#define ZL_CP_NSPEC34
#include "zl_bwd_dirbe_cp.cu"
