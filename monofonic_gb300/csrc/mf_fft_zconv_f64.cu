// Instantiation unit: zconv FFT passes in double precision.
#define MF_T double
#define MF_PART_ZCONV
#include "mf_launch_impl.cuh"
