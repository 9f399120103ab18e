/*
 * CPU OpenCL host shim: scalar and vector host types.
 *
 * Test infrastructure only.  This header stands in for the Khronos CL/cl.h so
 * that the reference's host sources (src/Tissue2D.cpp, src/Tissue3D.cpp,
 * src/cell.cpp) compile unmodified on a machine without an OpenCL SDK.  It
 * declares only the names those files use.  The device kernels are run on the
 * CPU by the shim in CL/opencl.hpp.
 */
#ifndef DPM_CLSHIM_CL_H
#define DPM_CLSHIM_CL_H

#include <stddef.h>
#include <stdint.h>

typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef float cl_float;
typedef uint64_t cl_ulong;
typedef cl_ulong cl_bitfield;
typedef cl_bitfield cl_mem_flags;
typedef cl_bitfield cl_command_queue_properties;
typedef cl_uint cl_program_build_info;

/* cl_float3 / cl_uint3 are 16-byte, 4-lane vectors as in the Khronos headers
 * (a 3-vector occupies the storage of a 4-vector). */
typedef union {
  cl_float s[4];
  struct {
    cl_float x, y, z, w;
  };
} __attribute__((aligned(16))) cl_float4;
typedef cl_float4 cl_float3;

typedef union {
  cl_uint s[4];
  struct {
    cl_uint x, y, z, w;
  };
} __attribute__((aligned(16))) cl_uint4;
typedef cl_uint4 cl_uint3;

#define CL_SUCCESS 0
#define CL_INVALID_VALUE -30
#define CL_INVALID_KERNEL_NAME -46
#define CL_INVALID_ARG_INDEX -49
#define CL_BUILD_PROGRAM_FAILURE -11

#define CL_FALSE 0
#define CL_TRUE 1

#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)
#define CL_MEM_USE_HOST_PTR (1 << 3)
#define CL_MEM_ALLOC_HOST_PTR (1 << 4)
#define CL_MEM_COPY_HOST_PTR (1 << 5)

#define CL_PROGRAM_BUILD_LOG 0x1183

#endif
