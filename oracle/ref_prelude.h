/* Prelude streamed ahead of the reference's weight functions
 * (compute_matrix.cu:21-257) when oracle/build.py compiles them for the host
 * into oracle/_ref/libref_weights.so.  Test infrastructure only. */
#define _USE_MATH_DEFINES
#include <math.h>
#define __device__
#define ERR 1.0e-10
