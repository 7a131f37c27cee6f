/* The reference's particles_kernel.cu includes "cutil_math.h"; the tree ships
 * the same header as cutil_math.cuh.  This one-line shim forwards to it. */
#include "cutil_math.cuh"
