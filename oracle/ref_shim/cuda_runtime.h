/* Empty stand-in: the host build of the reference kernels needs no runtime. */
#include <vector_types.h>
#include <vector_functions.h>
