// Instantiation unit: plain FFT passes in double precision.
#define MF_T double
#define MF_PART_PLAIN
#include "mf_launch_impl.cuh"
