// Instantiation unit: convy FFT passes in float precision.
#define MF_T float
#define MF_PART_CONVY
#include "mf_launch_impl.cuh"
