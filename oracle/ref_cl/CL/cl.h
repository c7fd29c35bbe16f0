/*
 * Minimal OpenCL 1.x declarations, enough to compile the reference's host
 * Tools.cpp / Logger.cpp for their sort and event-view functions
 * (Tools.cpp:46-80,117-164).  TEST INFRASTRUCTURE ONLY: none of these entry
 * points is ever called; ref_cl_stubs.c defines them to fail.
 */
#ifndef REF_CL_STUB_H
#define REF_CL_STUB_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint64_t cl_ulong;
typedef uint64_t cl_bitfield;
typedef cl_bitfield cl_device_type;
typedef uint32_t cl_bool;
typedef int8_t cl_char;
typedef float cl_float;
typedef struct _cl_platform_id* cl_platform_id;
typedef struct _cl_device_id* cl_device_id;
typedef struct _cl_command_queue* cl_command_queue;
typedef struct _cl_mem* cl_mem;
typedef struct _cl_event* cl_event;
#define CL_SUCCESS 0
#define CL_DEVICE_TYPE_CPU (1 << 1)
#define CL_DEVICE_TYPE_GPU (1 << 2)
#define CL_DEVICE_TYPE_ACCELERATOR (1 << 3)
#define CL_DEVICE_TYPE_ALL 0xFFFFFFFF
#define CL_TRUE 1
cl_int clGetPlatformIDs(cl_uint, cl_platform_id*, cl_uint*);
cl_int clGetDeviceIDs(cl_platform_id, cl_device_type, cl_uint, cl_device_id*, cl_uint*);
cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem, cl_bool, size_t, size_t, const void*, cl_uint,
                            const cl_event*, cl_event*);
#ifdef __cplusplus
}
#endif
#endif
