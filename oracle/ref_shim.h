/*
 * ref_shim.h -- the OpenCL C built-ins that the reference kernel uses,
 * declared for a plain C11 compile of the reference's own KernelDefinitions.h
 * + Kernel.cl (the same concatenation KernelInvoker.cpp:41-45 hands to
 * clCreateProgramWithSource).  TEST INFRASTRUCTURE ONLY.
 *
 * Work-item built-ins are served by the cooperative work-group emulator in
 * ref_emu.c: every work-item is a fiber, barrier() yields to the scheduler,
 * and all fibers of a work-group run on one OS thread, so atomics are plain
 * read-modify-writes.
 */
#ifndef REF_SHIM_H
#define REF_SHIM_H

#include <float.h>
#include <math.h>
#include <stdbool.h>   /* before KernelDefinitions.h: its `#if X == true` tests need the macros */
#include <stddef.h>

#define __kernel
#define __global
#define __local        /* parameters and casts; the two kernel-body __local arrays are rewritten */
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

size_t get_local_id(unsigned int dim);
size_t get_local_size(unsigned int dim);
size_t get_group_id(unsigned int dim);
size_t get_num_groups(unsigned int dim);
void barrier(int flags);

int ref_atomic_add(volatile int* p, int v);
int ref_atomic_max(volatile int* p, int v);
#define atomic_add(p, v) ref_atomic_add((volatile int*)(p), (int)(v))
#define atomic_max(p, v) ref_atomic_max((volatile int*)(p), (int)(v))

static inline int ref_min_int(int a, int b) { return a < b ? a : b; }
#define min(a, b) ref_min_int((a), (b))
#define fabs(x) fabsf(x)

#endif
