// Instantiation unit: zconv FFT passes in float precision.
#define MF_T float
#define MF_PART_ZCONV
#include "mf_launch_impl.cuh"
