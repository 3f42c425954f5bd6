// Batched WHFast in democratic heliocentric coordinates (the splitting of the
// reference's WHFast512, src/integrator_whfast512.c, and of WHFast with
// coordinates = DEMOCRATICHELIOCENTRIC), compiled with --fmad=false so that every
// system follows the plain democratic heliocentric path bit for bit.
#define ENSEMBLE_NS ens_dh
#define WH_INT_DIVSQRT 1        // IEEE division and sqrt on the integer pipes (whfast_core.cuh)
#define ENSEMBLE_STEP wh::step_safe_dh
#include "ensemble_kernels.cuh"

void* ensemble_dh_persistent_fn() { return (void*)ens_dh::persistent_kernel; }
