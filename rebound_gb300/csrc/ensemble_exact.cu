// Bit-exact flavour of the batched WHFast kernels (compiled with --fmad=false).
#define ENSEMBLE_NS ens_exact
#define WH_INT_DIVSQRT 1        // IEEE division and sqrt on the integer pipes (whfast_core.cuh)
#include "ensemble_kernels.cuh"

void* ensemble_exact_energy_fn(int nb) { return (void*)ens_exact::energy_for(nb); }
void* ensemble_exact_persistent_fn() { return (void*)ens_exact::persistent_kernel; }
