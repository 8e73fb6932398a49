/* Stand-in for the OpenCL header, used ONLY to compile the reference's pure-C++
 * Hilbert codec in place for the oracle (test infrastructure).  The codec itself
 * never calls OpenCL; its error header only names cl_int and seven status codes
 * (include/fluidloom/common/FluidLoomError.h:44-68 in the reference).  Values
 * follow the published Khronos numbering. */
#ifndef FLUIDLOOM_ORACLE_CL_SHIM_H
#define FLUIDLOOM_ORACLE_CL_SHIM_H
#include <stdint.h>
typedef int32_t cl_int;
#define CL_SUCCESS 0
#define CL_DEVICE_NOT_FOUND -1
#define CL_DEVICE_NOT_AVAILABLE -2
#define CL_COMPILER_NOT_AVAILABLE -3
#define CL_MEM_OBJECT_ALLOCATION_FAILURE -4
#define CL_OUT_OF_RESOURCES -5
#define CL_OUT_OF_HOST_MEMORY -6
#endif
