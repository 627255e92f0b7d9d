// Instantiation unit: plain FFT passes in float precision.
#define MF_T float
#define MF_PART_PLAIN
#include "mf_launch_impl.cuh"
