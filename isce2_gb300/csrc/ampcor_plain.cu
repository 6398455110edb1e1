// Translation unit of the plain-chain kernels (one CTA per window per stage) and the host-side sizing of every stage body.
// The device code lives in ampcor_device.cuh; each unit compiles one part
// of it so that the parts build in parallel.
#define AMPCOR_PART_PLAIN
#include "ampcor_device.cuh"
