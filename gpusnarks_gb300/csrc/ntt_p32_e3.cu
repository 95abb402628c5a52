// Register-blocked 32-bit NTT kernels with radix-8 register sub-steps.
#define GSN_P32_INSTANTIATE_ET 3
#include "ntt_p32.cuh"
