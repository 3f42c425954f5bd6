// Bit-exact flavour of the batched WHFast kernels (compiled with --fmad=false).
#define ENSEMBLE_NS ens_exact
#include "ensemble_kernels.cuh"

void* ensemble_exact_energy_fn(int nb) { return (void*)ens_exact::energy_for(nb); }
void* ensemble_exact_persistent_fn() { return (void*)ens_exact::persistent_kernel; }
