// Register-blocked 32-bit NTT kernels with radix-16 register sub-steps.
#define GSN_P32_INSTANTIATE_ET 4
#include "ntt_p32.cuh"
