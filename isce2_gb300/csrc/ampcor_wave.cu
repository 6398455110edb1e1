// Translation unit of the batched chain: per-wave stage kernels and the host planning of the waves.
// The device code lives in ampcor_device.cuh; each unit compiles one part
// of it so that the parts build in parallel.
#define AMPCOR_PART_WAVE
#include "ampcor_device.cuh"
