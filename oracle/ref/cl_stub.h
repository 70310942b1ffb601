/*
 * cl_stub.h -- the few OpenCL 1.2 host API declarations CLBVH.cpp uses, so the
 * reference's CLBVH class compiles on the CPU for the oracle.  The functions
 * are implemented in ref_kernels.cpp as an in-process emulation (buffers are
 * host memory, kernels run as sequential loops over the NDRange).
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef PTGPU_REF_CL_STUB_H
#define PTGPU_REF_CL_STUB_H
#include <stddef.h>
#include <stdint.h>

typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint32_t cl_bool;
typedef uint64_t cl_mem_flags;
typedef struct ref_cl_context_s *cl_context;
typedef struct ref_cl_queue_s *cl_command_queue;
typedef struct ref_cl_mem_s *cl_mem;
typedef struct ref_cl_kernel_s *cl_kernel;
typedef struct ref_cl_event_s *cl_event;

#define CL_SUCCESS 0
#define CL_TRUE 1
#define CL_FALSE 0
#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)

cl_mem clCreateBuffer(cl_context, cl_mem_flags, size_t, void *, cl_int *);
cl_int clReleaseMemObject(cl_mem);
cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem, cl_bool, size_t, size_t,
                            const void *, cl_uint, const cl_event *, cl_event *);
cl_int clEnqueueReadBuffer(cl_command_queue, cl_mem, cl_bool, size_t, size_t,
                           void *, cl_uint, const cl_event *, cl_event *);
cl_int clSetKernelArg(cl_kernel, cl_uint, size_t, const void *);
cl_int clEnqueueNDRangeKernel(cl_command_queue, cl_kernel, cl_uint, const size_t *,
                              const size_t *, const size_t *, cl_uint,
                              const cl_event *, cl_event *);
cl_int clFinish(cl_command_queue);
#endif
