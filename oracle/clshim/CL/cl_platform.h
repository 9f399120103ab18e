/* CPU OpenCL host shim (test infrastructure): platform header alias. */
#ifndef DPM_CLSHIM_CL_PLATFORM_H
#define DPM_CLSHIM_CL_PLATFORM_H
#include "cl.h"
#endif
