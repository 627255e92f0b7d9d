// Instantiation unit: convx FFT passes in float precision.
#define MF_T float
#define MF_PART_CONVX
#include "mf_launch_impl.cuh"
