/* Minimal OpenCL declarations so that the reference's host library
 * (src/sda_app/common/*.cpp) compiles without an OpenCL SDK. Only the
 * host-memory functions of that library are called from the checker; the
 * cl* entry points below are never reached and report CL_INVALID_OPERATION. */
#ifndef GBILU_STUB_CL_OPENCL_H
#define GBILU_STUB_CL_OPENCL_H
#include <stddef.h>
#include <stdint.h>
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint64_t cl_ulong;
typedef uint64_t cl_bitfield;
typedef cl_bitfield cl_mem_flags;
typedef cl_bitfield cl_map_flags;
typedef cl_bitfield cl_mem_migration_flags;
typedef cl_bitfield cl_command_queue_properties;
typedef cl_bitfield cl_device_type;
typedef cl_uint cl_platform_info;
typedef cl_uint cl_device_info;
typedef cl_uint cl_program_build_info;
typedef cl_uint cl_bool;
typedef struct _cl_platform_id *cl_platform_id;
typedef struct _cl_device_id *cl_device_id;
typedef struct _cl_context *cl_context;
typedef struct _cl_command_queue *cl_command_queue;
typedef struct _cl_mem *cl_mem;
typedef struct _cl_program *cl_program;
typedef struct _cl_kernel *cl_kernel;
typedef struct _cl_event *cl_event;
typedef intptr_t cl_context_properties;
typedef struct { unsigned flags; void *obj; void *param; } cl_mem_ext_ptr_t;
#define CL_SUCCESS 0
#define CL_INVALID_OPERATION (-59)
#define CL_TRUE 1
#define CL_FALSE 0
#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)
#define CL_MEM_USE_HOST_PTR (1 << 3)
#define CL_MEM_EXT_PTR_XILINX (1u << 31)
#define CL_MIGRATE_MEM_OBJECT_HOST (1 << 0)
#define CL_MAP_READ (1 << 0)
#define CL_MAP_WRITE (1 << 1)
#define XCL_MEM_DDR_BANK0 (1u << 0)
#define XCL_MEM_DDR_BANK1 (1u << 1)
#define XCL_MEM_DDR_BANK2 (1u << 2)
#define XCL_MEM_DDR_BANK3 (1u << 3)
#define XCL_MEM_TOPOLOGY (1u << 31)
#ifdef __cplusplus
extern "C" {
#endif
static inline cl_int clEnqueueMigrateMemObjects(cl_command_queue, cl_uint, const cl_mem *, cl_mem_migration_flags, cl_uint, const cl_event *, cl_event *) { return CL_INVALID_OPERATION; }
static inline cl_int clFinish(cl_command_queue) { return CL_INVALID_OPERATION; }
static inline cl_mem clCreateBuffer(cl_context, cl_mem_flags, size_t, void *, cl_int *e) { if (e) *e = CL_INVALID_OPERATION; return 0; }
static inline void *clEnqueueMapBuffer(cl_command_queue, cl_mem, cl_bool, cl_map_flags, size_t, size_t, cl_uint, const cl_event *, cl_event *, cl_int *e) { if (e) *e = CL_INVALID_OPERATION; return 0; }
static inline cl_int clEnqueueUnmapMemObject(cl_command_queue, cl_mem, void *, cl_uint, const cl_event *, cl_event *) { return CL_INVALID_OPERATION; }
static inline cl_int clEnqueueReadBuffer(cl_command_queue, cl_mem, cl_bool, size_t, size_t, void *, cl_uint, const cl_event *, cl_event *) { return CL_INVALID_OPERATION; }
static inline cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem, cl_bool, size_t, size_t, const void *, cl_uint, const cl_event *, cl_event *) { return CL_INVALID_OPERATION; }
static inline cl_int clSetKernelArg(cl_kernel, cl_uint, size_t, const void *) { return CL_INVALID_OPERATION; }
static inline cl_int clEnqueueTask(cl_command_queue, cl_kernel, cl_uint, const cl_event *, cl_event *) { return CL_INVALID_OPERATION; }
static inline cl_int clReleaseMemObject(cl_mem) { return CL_INVALID_OPERATION; }
#ifdef __cplusplus
}
#endif
#endif
