/* bsacl_shim.h -- TEST INFRASTRUCTURE ONLY (part of the parity oracle).
 *
 * Lets the reference's OpenCL C kernel source (BsaCL/src/bsacl.cl, with BsaCL/src/_base.h)
 * compile as C with gcc and run on the host, so that the oracle can be pinned against the
 * reference's own Classic BFM/BRM kernel.  It is force-included (gcc -include) before that
 * source by oracle/bsacl_ref.py; nothing of the kernel is copied here.
 *
 * OpenCL C -> C: the address-space qualifiers vanish, work-group (__local) arrays become static
 * storage shared by the threads of the one work group that runs at a time, and the work-item
 * built-ins read per-thread ids set by the driver (bsacl_ref_driver.c), which runs each work
 * item on its own POSIX thread so that barrier() is a real barrier.  Work items that return
 * before a barrier leave it (the reference's kernel returns early in the last work group).
 */
#ifndef BSACL_SHIM_H_
#define BSACL_SHIM_H_
#define _GNU_SOURCE
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdbool.h>
#include <stddef.h>

typedef unsigned int uint;
typedef unsigned short ushort;
typedef int cl_int;
typedef unsigned int cl_uint;
typedef void *cl_mem;
#define CL_SUCCESS 0
#define CL_MEM_READ_ONLY 0
#define CL_MEM_WRITE_ONLY 0
#define CL_MEM_READ_WRITE 0
#define CL_MEM_HOST_NO_ACCESS 0
#define CL_MEM_HOST_READ_ONLY 0
#define CL_MEM_HOST_WRITE_ONLY 0
#define CL_MEM_USE_HOST_PTR 0
#define CL_MEM_ALLOC_HOST_PTR 0
#define CL_MEM_COPY_HOST_PTR 0

#define __kernel
#define __global
#define __private
#define __constant const
#define __local static
#define powr pow
#define CLK_LOCAL_MEM_FENCE 0

size_t get_global_id(uint d);
size_t get_local_id(uint d);
size_t get_group_id(uint d);
size_t get_num_groups(uint d);
void barrier(int flags);

#endif
