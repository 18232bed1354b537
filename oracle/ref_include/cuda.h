/* Stand-in for <cuda.h> when the reference's gputools.cu is compiled for the
 * CPU: nothing from it is used by the kernels. */
#pragma once
