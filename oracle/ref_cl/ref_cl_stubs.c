/* Failing definitions of the OpenCL entry points declared in CL/cl.h; the
 * reference's sort path never reaches them.  TEST INFRASTRUCTURE ONLY. */
#include "CL/cl.h"
cl_int clGetPlatformIDs(cl_uint a, cl_platform_id* b, cl_uint* c) { (void)a; (void)b; if (c) *c = 0; return -1; }
cl_int clGetDeviceIDs(cl_platform_id a, cl_device_type b, cl_uint c, cl_device_id* d, cl_uint* e) {
  (void)a; (void)b; (void)c; (void)d; if (e) *e = 0; return -1;
}
cl_int clEnqueueWriteBuffer(cl_command_queue a, cl_mem b, cl_bool c, size_t d, size_t e, const void* f,
                            cl_uint g, const cl_event* h, cl_event* i) {
  (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; return -1;
}
