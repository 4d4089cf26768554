/*
 * Allocation-free single-frame render.
 *
 * Some callers cannot let a library allocate device memory: a host application
 * that hands out all device memory from its own pool and forbids libraries
 * from calling cudaMalloc, or a per-frame loop that cannot afford the implicit
 * device synchronisation a cudaMalloc/cudaFree may cause. fs_render_device
 * grows a per-context depth table with cudaMalloc when a longer draw distance
 * first appears; this entry point instead keeps that scratch -- the per-depth
 * view-line table the depth-table kernel writes and the render kernel reads --
 * in a fixed array compiled into the library, and calls no allocating routine.
 * The caller passes the inputs (context, resident map, camera, parameters) and
 * the output frame in device memory, as for fs_render_device.
 *
 * Limits and sharing:
 *  - at most FS_NOALLOC_MAX_DEPTHS depth samples per frame (65536: draw
 *    distances up to about 2.1 million map units with the default depth step);
 *    longer schedules are rejected with FS_ERR_ARG;
 *  - the array (about 1.25 MiB) stays allocated on every GPU that loads the library
 *    until the process exits;
 *  - all calls share it: each call rewrites the entries it reads before reading
 *    them (nothing needs to start at zero), so calls that overlap on the GPU --
 *    on different streams or contexts of the same device -- race and must be
 *    serialised by the caller;
 *  - the array's device address is looked up once per context, with the
 *    context's device current, when fs_ctx_new creates it (cudaGetSymbolAddress:
 *    the first lookup on a device may load this library's module there, which
 *    is when the array itself is allocated). So no render call loads a module
 *    or allocates, and no render call depends on state shared between host
 *    threads.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_internal.h"
#include "fs_priv.h"

#define FS_NOALLOC_MAX_DEPTHS 65536

/* [FS_NOALLOC_MAX_DEPTHS + FS_ZPAD] float4 {x0, y0, dx, dy}, then as many float inv_z */
#define FS_NOALLOC_ENTRIES (FS_NOALLOC_MAX_DEPTHS + FS_ZPAD)
static __device__ __align__(256) unsigned char fs_noalloc_scratch[FS_NOALLOC_ENTRIES * 20];

/* In host code the array's name only stands in for it: the kernels must be
 * given its device address, which this looks up on the current device (the
 * context's) and keeps in the context. */
extern "C" int fs_noalloc_setup(fs_ctx *ctx) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, fs_noalloc_scratch);
  if (e != cudaSuccess) return fs_cuda_fail(ctx, (int)e, "cudaGetSymbolAddress(scratch)");
  ctx->noalloc_scratch = p;
  return FS_OK;
}

extern "C" int fs_render_device_noalloc(fs_ctx *ctx, const fs_map *map, const fs_camera *cam,
                                        const fs_params *params, int32_t width, int32_t height,
                                        uint32_t *out_dev) {
  if (!ctx) return FS_ERR_ARG;
  if (ctx->broken) return fs_fail(ctx, FS_ERR_STATE, "context failed to initialise");
  if (!map || !out_dev) return fs_fail(ctx, FS_ERR_ARG, "NULL map or output");
  fs_params dp = fs_params_default();
  FsView v;
  int rc = fs_make_view(ctx, cam, params ? params : &dp, width, height, 0, &v);
  if (rc) return rc;
  if (v.n > FS_NOALLOC_MAX_DEPTHS)
    return fs_fail(ctx, FS_ERR_ARG,
                   "draw distance needs %d depth samples; the allocation-free render holds "
                   "at most %d",
                   v.n, FS_NOALLOC_MAX_DEPTHS);
  const cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fs_cuda_fail(ctx, (int)e, "cudaSetDevice");
  void *const scratch = ctx->noalloc_scratch;
  if (!scratch) return fs_fail(ctx, FS_ERR_STATE, "allocation-free scratch not set up");
  float4 *zline = reinterpret_cast<float4 *>(scratch);
  float *zinvz = reinterpret_cast<float *>(static_cast<unsigned char *>(scratch) +
                                           sizeof(float4) * FS_NOALLOC_ENTRIES);
  v.out = out_dev;
  return fs_render_view(ctx, &map->dev, &v, nullptr, zline, zinvz, nullptr, 0);
}
