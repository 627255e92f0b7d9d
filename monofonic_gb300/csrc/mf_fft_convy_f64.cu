// Instantiation unit: convy FFT passes in double precision.
#define MF_T double
#define MF_PART_CONVY
#include "mf_launch_impl.cuh"
