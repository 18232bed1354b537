/* Stand-in for <cufft.h> when the reference's gputools.cu is compiled for the
 * CPU: the kernels only use the cufftComplex type. */
#pragma once
typedef struct { float x, y; } cufftComplex;
