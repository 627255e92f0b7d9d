// Instantiation unit: convx FFT passes in double precision.
#define MF_T double
#define MF_PART_CONVX
#include "mf_launch_impl.cuh"
