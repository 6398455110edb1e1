// Translation unit of the fused persistent batched kernel, launch shape 256x1
// (threads x CTAs per SM).  The device code lives in ampcor_device.cuh.
#define AMPCOR_PART_PERSIST
#define AMPCOR_PERSIST_SHAPE 1
#include "ampcor_device.cuh"
