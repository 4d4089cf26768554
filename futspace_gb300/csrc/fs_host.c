/*
 * Host side of the renderer: contexts, resident maps, the plain per-frame call
 * and the batched plan (persistent kernel under a captured CUDA graph).
 * C11. No CPU fallback: every render goes through the CUDA kernels, and a
 * missing device or kernel is reported as an error.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>

#include <cudaTypedefs.h>

#include "fs_internal.h"
#include "fs_priv.h"

/* ---- errors ---------------------------------------------------------------- */

int fs_fail(fs_ctx *ctx, int code, const char *fmt, ...) {
  if (ctx) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
    va_end(ap);
    ctx->has_err = 1;
  }
  return code;
}

int fs_cuda_fail(fs_ctx *ctx, int e, const char *what) {
  return fs_fail(ctx, FS_ERR_CUDA, "%s: %s", what, cudaGetErrorString((cudaError_t)e));
}

char *fs_ctx_get_error(fs_ctx *ctx) {
  if (!ctx || !ctx->has_err) return NULL;
  size_t len = strlen(ctx->err);
  char *s = (char *)malloc(len + 1);
  if (s) memcpy(s, ctx->err, len + 1);
  ctx->has_err = 0;
  ctx->err[0] = 0;
  return s;
}

/* ---- parameters -------------------------------------------------------------- */

fs_params fs_params_default(void) {
  fs_params p;
  memset(&p, 0, sizeof(p));
  p.invz_param1 = 0.001f; /* d,  fut/voxel_renderer.fut:104 */
  p.invz_param2 = 0.0f;   /* z0, fut/voxel_renderer.fut:103 */
  p.magic_number = 0.0f;  /* f32(w/2), fut/voxel_renderer.fut:217 */
  p.height_filter = FS_BILINEAR; /* fut/interactive.fut:180 */
  p.color_filter = FS_BILINEAR;  /* fut/interactive.fut:181 */
  p.gap_rule = FS_GAP_ZERO;
  p.floor_n = 1;
  return p;
}

/* get_zs depth count, fut/voxel_renderer.fut:29-32. Same f32 operations and
 * order as the reference; powf is the C library's, as in a `futhark c` build. */
int32_t fs_num_depths(float distance, const fs_params *params) {
  fs_params dp = fs_params_default();
  const fs_params *p = params ? params : &dp;
  const float d = p->invz_param1, z0 = p->invz_param2;
  const float t = d - 2.0f * z0;
  const float sq = sqrtf(powf(t, 2.0f) + 8.0f * d * distance);
  const float num = sq - 2.0f * z0 + d;
  const float div = 2.0f * d;
  const float q = num / div;
  return fs_f2i_host(p->floor_n ? floorf(q) : q);
}

int32_t fs_f2i_host(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return INT32_MAX;
  if (v <= -2147483648.0f) return INT32_MIN;
  return (int32_t)v;
}

int fs_check_params(fs_ctx *ctx, const fs_params *p) {
  if (!p) return fs_fail(ctx, FS_ERR_ARG, "params is NULL");
  if ((p->height_filter != FS_NEAREST && p->height_filter != FS_BILINEAR) ||
      (p->color_filter != FS_NEAREST && p->color_filter != FS_BILINEAR))
    return fs_fail(ctx, FS_ERR_ARG, "filter must be FS_NEAREST or FS_BILINEAR");
  if (p->gap_rule != FS_GAP_ZERO && p->gap_rule != FS_GAP_SKY)
    return fs_fail(ctx, FS_ERR_ARG, "gap_rule must be FS_GAP_ZERO or FS_GAP_SKY");
  if (p->effects & ~(FS_FX_SHADE | FS_FX_FOG))
    return fs_fail(ctx, FS_ERR_ARG, "unknown effect flags 0x%x", p->effects);
  if ((p->effects & FS_FX_FOG) && !(p->fog_end > p->fog_start))
    return fs_fail(ctx, FS_ERR_ARG, "fog needs fog_end > fog_start");
  if (p->smoothing != 0 && p->smoothing != 1)
    return fs_fail(ctx, FS_ERR_ARG, "smoothing must be 0 or 1");
  if (p->smoothing && p->gap_rule != FS_GAP_ZERO)
    return fs_fail(ctx, FS_ERR_ARG, "smoothing renders the live branch: gap_rule FS_GAP_ZERO");
  return FS_OK;
}

/* Fills the kernel view record of one camera. sin/cos come from the host C
 * library (f32.sin / f32.cos of a `futhark c` build, fut/voxel_renderer.fut:44-45). */
int fs_make_view(fs_ctx *ctx, const fs_camera *cam, const fs_params *p, int32_t W, int32_t H,
                 int32_t map, FsView *v) {
  if (!cam) return fs_fail(ctx, FS_ERR_ARG, "camera is NULL");
  if (W <= 0 || H <= 0 || H > FS_MAX_ROWS || W > 65536)
    return fs_fail(ctx, FS_ERR_ARG, "screen %dx%d out of range (H <= %d, W <= 65536)", W, H,
                   FS_MAX_ROWS);
  int rc = fs_check_params(ctx, p);
  if (rc) return rc;
  const int32_t n = fs_num_depths(cam->distance, p);
  if (n < 1)
    return fs_fail(ctx, FS_ERR_RANGE, "depth schedule for distance %g has %d samples",
                   (double)cam->distance, n);
  if (n >= FS_MAX_DEPTHS)
    return fs_fail(ctx, FS_ERR_ARG, "depth schedule too long (%d samples)", n);
  memset(v, 0, sizeof(*v));
  v->cam_x = cam->x;
  v->cam_y = cam->y;
  v->cam_h = cam->height;
  v->horizon = cam->horizon;
  v->sa = sinf(cam->angle);
  v->ca = cosf(cam->angle);
  v->fov = cam->fov;
  v->scale = p->magic_number > 0.0f ? p->magic_number : (float)(W / 2);
  v->d = p->invz_param1;
  v->z0 = p->invz_param2;
  v->W = W;
  v->H = H;
  v->n = n;
  v->map = map;
  v->sky = cam->sky_color;
  v->gap = p->gap_rule == FS_GAP_SKY ? cam->sky_color : 0u;
  v->tmap = -1;
  v->flags = (p->height_filter == FS_BILINEAR ? FSV_HEIGHT_BILINEAR : 0) |
             (p->color_filter == FS_BILINEAR ? FSV_COLOR_BILINEAR : 0) |
             ((p->effects & FS_FX_SHADE) ? FSV_SHADE : 0) | ((p->effects & FS_FX_FOG) ? FSV_FOG : 0) |
             (p->smoothing ? FSV_SMOOTH : 0);
  v->distance = cam->distance;
  v->shade = p->shade;
  v->fog_start = p->fog_start;
  v->fog_end = p->fog_end;
  v->fog_color = p->fog_color;
  v->nseg = 1;
  v->seglen = n;
  return FS_OK;
}

/* ---- context --------------------------------------------------------------- */

int fs_ctx_new(fs_ctx **out, int32_t device) {
  if (!out) return FS_ERR_ARG;
  *out = NULL;
  fs_ctx *ctx = (fs_ctx *)calloc(1, sizeof(fs_ctx));
  if (!ctx) return FS_ERR_NOMEM;
  ctx->device = device;
  int e = cudaSetDevice(device);
  if (e) {
    fs_cuda_fail(ctx, e, "cudaSetDevice");
    *out = ctx; /* keep the context so the caller can read the error */
    ctx->broken = 1;
    return FS_ERR_CUDA;
  }
  int major = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  ctx->smem_optin = (size_t)optin;
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e) {
    fs_cuda_fail(ctx, e, "cudaStreamCreate");
    ctx->broken = 1;
    *out = ctx;
    return FS_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  enum cudaDriverEntryPointQueryResult qr;
  void *fn = NULL;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &qr) == cudaSuccess &&
      qr == cudaDriverEntryPointSuccess)
    ctx->encode = fn;
  ctx->use_tma = ctx->encode != NULL;
  const char *env = getenv("FS_NO_TMA");
  if (env && env[0] == '1') ctx->use_tma = 0;
  env = getenv("FS_NO_SKIP");
  if (env && env[0] == '1') ctx->no_skip = 1;
  if (cudaMalloc((void **)&ctx->stats_dev, 2 * sizeof(unsigned long long)) != cudaSuccess) {
    ctx->broken = 1;
    *out = ctx;
    return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(stats)");
  }
  cudaMemset(ctx->stats_dev, 0, 2 * sizeof(unsigned long long));
  /* the allocation-free render's scratch address: looking it up may load the
   * library's module onto the device (which allocates its fixed arrays), so
   * it happens here, in a call that allocates anyway, and never in a render */
  e = fs_noalloc_setup(ctx);
  if (e) {
    ctx->broken = 1;
    *out = ctx;
    return e;
  }
  fs_tune_cache_load(ctx);
  *out = ctx;
  return FS_OK;
}

void fs_fill_u32(uint32_t *dst, int64_t n, uint32_t value) {
  while (n > 0 && ((uintptr_t)dst & 15u)) {
    *dst++ = value;
    n--;
  }
  const uint32_t v4[4] = {value, value, value, value};
  for (int64_t i = 0; i < n / 4; i++) memcpy(dst + 4 * i, v4, sizeof(v4)); /* 16-byte stores */
  for (int64_t i = n & ~(int64_t)3; i < n; i++) dst[i] = value;
}

void fs_ctx_free(fs_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
  cudaFree(ctx->zline);
  cudaFree(ctx->zinvz);
  cudaFree(ctx->frame_dev);
  cudaFree(ctx->segbuf);
  cudaFree(ctx->stats_dev);
  if (ctx->ev_kernel[0]) cudaEventDestroy(ctx->ev_kernel[0]);
  if (ctx->ev_kernel[1]) cudaEventDestroy(ctx->ev_kernel[1]);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  free(ctx);
}

int fs_ctx_sync(fs_ctx *ctx) {
  if (!ctx) return FS_ERR_ARG;
  cudaSetDevice(ctx->device);
  int e = cudaStreamSynchronize(ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "cudaStreamSynchronize");
  return FS_OK;
}

int fs_ctx_set_stream(fs_ctx *ctx, void *stream) {
  if (!ctx) return FS_ERR_ARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return FS_OK;
}

void *fs_ctx_get_stream(fs_ctx *ctx) { return ctx ? (void *)ctx->stream : NULL; }

int64_t fs_ctx_kernel_launches(fs_ctx *ctx) { return ctx ? ctx->launches : 0; }

int fs_ctx_set_option(fs_ctx *ctx, const char *name, int64_t value) {
  if (!ctx || !name) return FS_ERR_ARG;
  if (!strcmp(name, "skip")) {
    ctx->no_skip = value ? 0 : 1;
  } else if (!strcmp(name, "tma")) {
    ctx->use_tma = (value && ctx->encode) ? 1 : 0;
  } else if (!strcmp(name, "split")) {
    ctx->no_split = value ? 0 : 1;
  } else if (!strcmp(name, "time")) {
    if (value && !ctx->ev_kernel[0]) {
      cudaSetDevice(ctx->device);
      if (cudaEventCreate(&ctx->ev_kernel[0]) || cudaEventCreate(&ctx->ev_kernel[1]))
        return fs_fail(ctx, FS_ERR_CUDA, "cudaEventCreate(kernel timer)");
    }
    ctx->time_kernel = value ? 1 : 0;
    ctx->kernel_timed = 0;
  } else {
    return fs_fail(ctx, FS_ERR_ARG, "unknown option '%s'", name);
  }
  return FS_OK;
}

int fs_ctx_force_tune(fs_ctx *ctx, const int32_t tune5[5]) {
  if (!ctx) return FS_ERR_ARG;
  FsTune t = {0, 0, 0, 0, 0};
  if (tune5 && tune5[0]) {
    t.tw = tune5[0];
    t.lc = tune5[1];
    t.u = tune5[2];
    t.stage = tune5[3];
    if (!fsk_tune_supported(&t))
      return fs_fail(ctx, FS_ERR_ARG, "tuning (%d,%d,%d,%d) is not compiled", t.tw, t.lc, t.u,
                     t.stage);
  }
  ctx->forced = t;
  return FS_OK;
}

int fs_ctx_kernel_ms(fs_ctx *ctx, float *ms) {
  if (!ctx || !ms) return FS_ERR_ARG;
  if (!ctx->kernel_timed) return fs_fail(ctx, FS_ERR_STATE, "no timed render (option \"time\")");
  cudaSetDevice(ctx->device);
  int e = cudaEventSynchronize(ctx->ev_kernel[1]);
  if (!e) e = cudaEventElapsedTime(ms, ctx->ev_kernel[0], ctx->ev_kernel[1]);
  if (e) return fs_cuda_fail(ctx, e, "kernel timer");
  return FS_OK;
}

int fs_measure_l2_read_gbs(fs_ctx *ctx, int64_t bytes, int32_t reps, float *gbs) {
  if (!ctx || !gbs || bytes < (1 << 20) || reps < 1) return FS_ERR_ARG;
  cudaSetDevice(ctx->device);
  bytes &= ~(int64_t)15;
  void *buf = NULL;
  uint32_t *sink = NULL;
  cudaEvent_t a = NULL, b = NULL;
  int rc = FS_OK;
  if (cudaMalloc(&buf, (size_t)bytes) || cudaMalloc((void **)&sink, 4)) {
    rc = fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(L2 probe)");
    goto done;
  }
  if (cudaEventCreate(&a) || cudaEventCreate(&b)) {
    rc = fs_fail(ctx, FS_ERR_CUDA, "cudaEventCreate(L2 probe)");
    goto done;
  }
  {
    const int32_t grid = 4 * ctx->sm_count;
    int e = cudaMemsetAsync(buf, 1, (size_t)bytes, ctx->stream);
    if (!e) e = fsk_l2_read(buf, bytes, 1, grid, sink, ctx->stream); /* into L2 */
    if (!e) e = cudaEventRecord(a, ctx->stream);
    if (!e) e = fsk_l2_read(buf, bytes, reps, grid, sink, ctx->stream);
    if (!e) e = cudaEventRecord(b, ctx->stream);
    if (!e) e = cudaEventSynchronize(b);
    float ms = 0.0f;
    if (!e) e = cudaEventElapsedTime(&ms, a, b);
    if (e) {
      rc = fs_cuda_fail(ctx, e, "L2 probe");
      goto done;
    }
    *gbs = (float)((double)bytes * reps / (ms * 1e-3) / 1e9);
  }
done:
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(sink);
  cudaFree(buf);
  return rc;
}

int fs_ctx_stats(fs_ctx *ctx, int32_t enable, uint64_t out2[2]) {
  if (!ctx) return FS_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (out2) {
    unsigned long long h[2] = {0, 0};
    int e = cudaMemcpyAsync(h, ctx->stats_dev, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    if (!e) e = cudaStreamSynchronize(ctx->stream);
    if (e) return fs_cuda_fail(ctx, e, "stats readback");
    out2[0] = h[0];
    out2[1] = h[1];
  }
  cudaMemsetAsync(ctx->stats_dev, 0, 2 * sizeof(unsigned long long), ctx->stream);
  ctx->collect_stats = enable ? 1 : 0;
  return FS_OK;
}

/* Depth table for one view of n samples, plus the FS_ZPAD entries past them. */
int fs_ensure_ztable(fs_ctx *ctx, int64_t n) {
  n += FS_ZPAD;
  if (n <= ctx->zcap) return FS_OK;
  int64_t cap = n < 4096 ? 4096 : n;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->zline);
  cudaFree(ctx->zinvz);
  ctx->zline = NULL;
  ctx->zinvz = NULL;
  ctx->zcap = 0;
  if (cudaMalloc((void **)&ctx->zline, (size_t)cap * sizeof(float4)) != cudaSuccess ||
      cudaMalloc((void **)&ctx->zinvz, (size_t)cap * sizeof(float)) != cudaSuccess)
    return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(z table, %lld entries)", (long long)cap);
  ctx->zcap = cap;
  return FS_OK;
}

/* Tensor map of one frame: 2-D u32, {W, H}, row pitch W*4 bytes, boxes of
 * tw columns x 32 rows. Requires W % 4 == 0 and a 16-byte aligned base. */
int fs_encode_frame_map(fs_ctx *ctx, uint32_t *frame, int32_t W, int32_t H, int32_t tw,
                        CUtensorMap *out) {
  if (!ctx->use_tma || !ctx->encode) return 0;
  if ((W % 4) != 0 || (((uintptr_t)frame) & 15u) != 0) return 0;
  PFN_cuTensorMapEncodeTiled_v12000 enc = (PFN_cuTensorMapEncodeTiled_v12000)ctx->encode;
  cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
  cuuint64_t strides[1] = {(cuuint64_t)W * 4u};
  cuuint32_t box[2] = {(cuuint32_t)tw, 32u};
  cuuint32_t estr[2] = {1u, 1u};
  CUresult r = enc(out, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, frame, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 1 : 0;
}

void *fs_host_alloc(size_t bytes) {
  void *p = NULL;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return NULL;
  return p;
}

void fs_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

/* ---- maps -------------------------------------------------------------------- */

static int is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

/* Builds the height max pyramid after the quads (same stream). */
static int fs_map_build_pyramid(fs_ctx *ctx, fs_map *m) {
  const size_t bytes = fs_pyramid_layout(&m->dev);
  if (!bytes) return 0;
  if (cudaMalloc((void **)&m->pyr, bytes) != cudaSuccess) {
    m->pyr = NULL;
    m->dev.pyr = NULL;
    return (int)cudaErrorMemoryAllocation;
  }
  m->dev.pyr = m->pyr;
  return fsk_build_pyramid(&m->dev, m->pyr, ctx->stream);
}

static int fs_map_alloc(fs_ctx *ctx, fs_map **out, int64_t rows, int64_t cols) {
  if (!ctx || !out) return fs_fail(ctx, FS_ERR_ARG, "NULL argument");
  if (rows <= 0 || cols <= 0 || rows > 65536 || cols > 65536 || rows * cols > FS_MAX_TEXELS)
    return fs_fail(ctx, FS_ERR_ARG, "map %lldx%lld out of range", (long long)rows,
                   (long long)cols);
  fs_map *m = (fs_map *)calloc(1, sizeof(fs_map));
  if (!m) return fs_fail(ctx, FS_ERR_NOMEM, "calloc(map)");
  cudaSetDevice(ctx->device);
  const size_t cnt = (size_t)rows * (size_t)cols;
  if (cudaMalloc((void **)&m->q, cnt * 4) != cudaSuccess ||
      cudaMalloc((void **)&m->c, cnt * 4) != cudaSuccess) {
    cudaFree(m->q);
    free(m);
    return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(map %lldx%lld)", (long long)rows,
                   (long long)cols);
  }
  m->owned = 1;
  m->rows = rows;
  m->cols = cols;
  m->dev.q = m->q;
  m->dev.c = m->c;
  m->dev.MH = m->dev.CH = (int32_t)rows;
  m->dev.MW = m->dev.CW = (int32_t)cols;
  m->dev.pow2 = m->dev.cpow2 = is_pow2(rows) && is_pow2(cols);
  *out = m;
  return FS_OK;
}

int fs_map_new(fs_ctx *ctx, fs_map **out, const uint8_t *heights, const uint32_t *colors,
               int64_t rows, int64_t cols) {
  if (!heights || !colors) return fs_fail(ctx, FS_ERR_ARG, "map buffers are NULL");
  int rc = fs_map_alloc(ctx, out, rows, cols);
  if (rc) return rc;
  fs_map *m = *out;
  const size_t cnt = (size_t)rows * (size_t)cols;
  uint8_t *tmp = NULL;
  int e = cudaMalloc((void **)&tmp, cnt);
  if (!e) e = cudaMemcpyAsync(tmp, heights, cnt, cudaMemcpyHostToDevice, ctx->stream);
  if (!e) e = fsk_build_quads(tmp, m->q, (int32_t)rows, (int32_t)cols, ctx->stream);
  if (!e) e = fs_map_build_pyramid(ctx, m);
  if (!e) e = cudaMemcpyAsync(m->c, colors, cnt * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(tmp);
  if (e) {
    fs_map_free(ctx, m);
    *out = NULL;
    return fs_cuda_fail(ctx, e, "map upload");
  }
  return FS_OK;
}

int fs_map_new_i32(fs_ctx *ctx, fs_map **out, const int32_t *heights, const uint32_t *colors,
                   int64_t rows, int64_t cols) {
  if (!heights || !colors) return fs_fail(ctx, FS_ERR_ARG, "map buffers are NULL");
  int rc = fs_map_alloc(ctx, out, rows, cols);
  if (rc) return rc;
  fs_map *m = *out;
  const size_t cnt = (size_t)rows * (size_t)cols;
  int32_t *tmp = NULL;
  uint8_t *h8 = NULL;
  int e = cudaMalloc((void **)&tmp, cnt * 4);
  if (!e) e = cudaMalloc((void **)&h8, cnt);
  if (!e) e = cudaMemcpyAsync(tmp, heights, cnt * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (!e) e = fsk_mask_heights(tmp, h8, (int64_t)cnt, ctx->stream);
  if (!e) e = fsk_build_quads(h8, m->q, (int32_t)rows, (int32_t)cols, ctx->stream);
  if (!e) e = fs_map_build_pyramid(ctx, m);
  if (!e) e = cudaMemcpyAsync(m->c, colors, cnt * 4, cudaMemcpyHostToDevice, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(tmp);
  cudaFree(h8);
  if (e) {
    fs_map_free(ctx, m);
    *out = NULL;
    return fs_cuda_fail(ctx, e, "map upload (i32)");
  }
  return FS_OK;
}

int fs_map_wrap_device(fs_ctx *ctx, fs_map **out, const uint8_t *heights_dev,
                       const uint32_t *colors_dev, int64_t rows, int64_t cols) {
  if (!ctx || !out || !heights_dev || !colors_dev)
    return fs_fail(ctx, FS_ERR_ARG, "NULL argument");
  if (rows <= 0 || cols <= 0 || rows > 65536 || cols > 65536 || rows * cols > FS_MAX_TEXELS)
    return fs_fail(ctx, FS_ERR_ARG, "map %lldx%lld out of range", (long long)rows,
                   (long long)cols);
  fs_map *m = (fs_map *)calloc(1, sizeof(fs_map));
  if (!m) return fs_fail(ctx, FS_ERR_NOMEM, "calloc(map)");
  cudaSetDevice(ctx->device);
  const size_t cnt = (size_t)rows * (size_t)cols;
  if (cudaMalloc((void **)&m->q, cnt * 4) != cudaSuccess) {
    free(m);
    return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(height quads)");
  }
  m->owned = 2; /* quads owned, colours borrowed */
  m->rows = rows;
  m->cols = cols;
  m->dev.q = m->q;
  m->dev.c = colors_dev;
  m->dev.MH = m->dev.CH = (int32_t)rows;
  m->dev.MW = m->dev.CW = (int32_t)cols;
  m->dev.pow2 = m->dev.cpow2 = is_pow2(rows) && is_pow2(cols);
  int e = fsk_build_quads(heights_dev, m->q, (int32_t)rows, (int32_t)cols, ctx->stream);
  if (!e) e = fs_map_build_pyramid(ctx, m);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) {
    fs_map_free(ctx, m);
    return fs_cuda_fail(ctx, e, "height quads");
  }
  *out = m;
  return FS_OK;
}

int fs_map_free(fs_ctx *ctx, fs_map *map) {
  if (!map) return FS_OK;
  if (ctx) cudaSetDevice(ctx->device);
  if (map->owned) cudaFree(map->q);
  cudaFree(map->pyr);
  if (map->owned == 1) cudaFree(map->c);
  free(map);
  return FS_OK;
}

int fs_map_shape(const fs_map *map, int64_t *rows, int64_t *cols) {
  if (!map) return FS_ERR_ARG;
  if (rows) *rows = map->rows;
  if (cols) *cols = map->cols;
  return FS_OK;
}

const uint32_t *fs_map_quads_dev(const fs_map *map) { return map ? map->dev.q : NULL; }
const uint32_t *fs_map_colors_dev(const fs_map *map) { return map ? map->dev.c : NULL; }

/* ---- tuning ---------------------------------------------------------------- */

/* Compiled configurations {tw, lc, u, stage, ctas}, in the order a single
 * frame tries them when the tuning cache has no entry (first that fits wins).
 * Stage 0 paints directly, 1 through the shared-memory stage, 2 is the
 * cooperative tile (lc = threads per column, u = depths per thread per block). */
static const FsTune k_tune_order[] = {
    {8, 64, 8, 2, 0},  {4, 32, 2, 1, 0},  {8, 32, 2, 1, 0},  {8, 32, 1, 1, 0}, {16, 32, 2, 1, 0},
    {32, 32, 1, 1, 0}, {16, 16, 2, 1, 0}, {32, 16, 2, 1, 0}, {16, 8, 4, 1, 0},
    {32, 8, 4, 1, 0},  {8, 32, 2, 0, 0},  {16, 16, 2, 0, 0}, {32, 8, 2, 0, 0},
    {32, 8, 4, 0, 0},  {32, 4, 4, 0, 0},  {64, 4, 4, 0, 0},  {32, 4, 8, 0, 0},
    {64, 2, 4, 0, 0},  {64, 1, 4, 0, 0},  {128, 1, 4, 0, 0}, {64, 1, 8, 0, 0},
    {128, 1, 8, 0, 0}, {4, 64, 8, 2, 0},  {8, 32, 8, 2, 0},  {4, 64, 4, 2, 0},
};

int fs_tune_count(void) { return (int)(sizeof(k_tune_order) / sizeof(k_tune_order[0])); }

int fs_tune_get(int i, int32_t out5[5]) {
  if (i < 0 || i >= fs_tune_count()) return FS_ERR_ARG;
  out5[0] = k_tune_order[i].tw;
  out5[1] = k_tune_order[i].lc;
  out5[2] = k_tune_order[i].u;
  out5[3] = k_tune_order[i].stage;
  out5[4] = 0;
  return FS_OK;
}

int fs_tune_fits(fs_ctx *ctx, const FsTune *t, int32_t stride_max) {
  if (!fsk_tune_supported(t)) return 0;
  return fsk_render_smem(t, stride_max) <= ctx->smem_optin;
}

/* The kernel mode a view needs (smoothing, shading/fog epilogue) applied to a
 * tuning; a tuning with no kernel compiled for that mode becomes the mode's
 * default configuration. */
FsTune fs_tune_for_mode(FsTune t, int32_t view_flags) {
  t.smooth = (view_flags & FSV_SMOOTH) ? 1 : 0;
  t.fx = (view_flags & (FSV_SHADE | FSV_FOG)) ? 1 : 0;
  if ((t.smooth || t.fx) && !fsk_tune_supported(&t)) {
    const FsTune d = {128, 1, t.smooth ? 4 : 8, 0, t.ctas, t.smooth, t.fx};
    t = d;
  }
  return t;
}

int fs_coop_depths_ok(const FsTune *t, int32_t max_n) {
  return t->stage != 2 || max_n <= FS_COOP_MAX_DEPTHS;
}

/* The first table entry other than the cooperative tile that fits. */
FsTune fs_default_tune_without_coop(fs_ctx *ctx, int32_t stride_max) {
  for (int i = 0; i < fs_tune_count(); i++)
    if (k_tune_order[i].stage != 2 && fs_tune_fits(ctx, &k_tune_order[i], stride_max))
      return k_tune_order[i];
  FsTune none = {0, 0, 0, 0, 0};
  return none;
}

/* Default choice when the tuning cache has no entry: the first table entry
 * whose shared-memory stage fits. */
FsTune fs_default_tune(fs_ctx *ctx, int32_t stride_max) {
  for (int i = 0; i < fs_tune_count(); i++)
    if (fs_tune_fits(ctx, &k_tune_order[i], stride_max)) return k_tune_order[i];
  FsTune none = {0, 0, 0, 0, 0};
  return none;
}

/* ---- plain per-frame render ------------------------------------------------------ */

/* Depth segments per view for direct painting: enough (view, segment, strip)
 * items for two per resident warp, given `strips` strips in the launch. A
 * segment keeps at least 4 chunks (split_segments caps it per view). */
int32_t fs_split_target(fs_ctx *ctx, const FsTune *t, int32_t hf, int32_t cf, int32_t stride,
                        int64_t strips) {
  if (ctx->no_split || t->stage || t->smooth || t->fx || strips <= 0) return 1;
  int32_t occ = 0;
  if (fsk_render_max_ctas_per_sm(t, hf, cf, stride, &occ) || occ < 1) return 1;
  const int64_t warps = (int64_t)occ * ctx->sm_count * fsk_items_per_cta(t);
  int64_t nseg = (2 * warps + strips - 1) / strips;
  if (nseg < 1) nseg = 1;
  if (nseg > FS_MAX_SEGMENTS) nseg = FS_MAX_SEGMENTS;
  return (int32_t)nseg;
}

/* Splits v's n depths into at most nseg segments of a whole number of
 * `chunk`-depth chunks, at least 4 chunks each. */
void fs_set_segments(FsView *v, int32_t nseg, int32_t chunk) {
  const int32_t most = v->n / (4 * chunk);
  if (nseg > most) nseg = most;
  if (nseg <= 1) {
    v->nseg = 1;
    v->seglen = v->n;
    return;
  }
  int32_t seglen = (v->n + nseg - 1) / nseg;
  seglen = (seglen + chunk - 1) / chunk * chunk;
  v->seglen = seglen;
  v->nseg = (v->n + seglen - 1) / seglen;
}

int fs_render_view(fs_ctx *ctx, const FsMapDev *map, FsView *v, const FsTune *tune_in,
                   float4 *zline, float *zinvz, const CUtensorMap *tmap_pre,
                   int32_t allow_split) {
  const int32_t stride = v->H | 1;
  FsTune t;
  if (tune_in && tune_in->tw) t = *tune_in;
  else if (ctx->forced.tw) t = ctx->forced;
  else if (!fs_tune_lookup(ctx, v->W, v->H, map->MH, map->MW, v->flags, &t))
    t = fs_default_tune(ctx, stride);
  t = fs_tune_for_mode(t, v->flags);
  if (t.stage == 2 && v->n > FS_COOP_MAX_DEPTHS) {
    /* more depths than the cooperative tile's event entries hold */
    t = fs_tune_for_mode(fs_default_tune_without_coop(ctx, stride), v->flags);
  }
  if (!t.tw || !fs_tune_fits(ctx, &t, stride))
    return fs_fail(ctx, FS_ERR_ARG, "no kernel configuration fits screen height %d", v->H);
  const int32_t hf = (v->flags & FSV_HEIGHT_BILINEAR) != 0;
  const int32_t cf = (v->flags & FSV_COLOR_BILINEAR) != 0;
  const int32_t iw = fsk_item_width(&t), ntiles = (v->W + iw - 1) / iw;
  const int32_t per_cta = fsk_items_per_cta(&t);
  /* a frame with few strips splits each column's depths over several warps */
  fs_set_segments(v, allow_split ? fs_split_target(ctx, &t, hf, cf, stride, ntiles) : 1,
                  t.lc * t.u);
  v->segbuf = NULL;
  t.seg = v->nseg > 1;
  if (v->nseg > 1) {
    const int64_t need = (int64_t)(v->nseg + 2) * v->W;
    if (need > ctx->segcap) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->segbuf);
      ctx->segbuf = NULL;
      ctx->segcap = 0;
      if (cudaMalloc((void **)&ctx->segbuf, sizeof(int32_t) * (size_t)need) != cudaSuccess)
        return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(segment rows)");
      ctx->segcap = need;
    }
    v->segbuf = ctx->segbuf;
  }
  FsLaunch launch;
  FsLaunch *L = &launch;
  memset(L, 0, sizeof(*L));
  if (tmap_pre) {
    L->tmap0 = *tmap_pre;
    v->tmap = 0;
  } else {
    v->tmap = fs_encode_frame_map(ctx, v->out, v->W, v->H, t.tw, &L->tmap0) ? 0 : -1;
  }
  L->view0 = *v;
  L->maps[0] = *map;
  if (ctx->no_skip) L->maps[0].pyr = NULL;
  L->view0.map = 0;
  L->zline = zline;
  L->zinvz = zinvz;
  /* the work counters cost instructions per depth chunk: only when collected */
  L->stats = ctx->collect_stats ? ctx->stats_dev : NULL;
  L->nitems = ntiles * v->nseg;
  L->stride_max = stride;
  /* the timer brackets every kernel of the call; an event between two of them
   * would stop the second from starting early */
  if (ctx->time_kernel) cudaEventRecord(ctx->ev_kernel[0], ctx->stream);
  int e = fsk_ztable(NULL, &L->view0, 1, v->n, zline, zinvz, ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "z-table kernel launch");
  if (v->nseg > 1) {
    /* minimum row of every segment but the last, before the render pass */
    FsLaunch A = *L;
    A.stats = NULL;
    A.nitems = ntiles * (v->nseg - 1);
    e = fsk_segmin(&A, &t, hf, (A.nitems + per_cta - 1) / per_cta, ctx->stream);
    if (e) return fs_cuda_fail(ctx, e, "segment-minimum kernel launch");
    ctx->launches++;
  }
  /* programmatic dependent launch: the render kernel starts while the kernel
   * before it finishes and waits for its results in the kernel */
  e = fsk_render_pdl(L, &t, hf, cf, (L->nitems + per_cta - 1) / per_cta, ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "render kernel launch");
  ctx->launches += 2;
  if (v->nseg > 1) {
    e = fsk_gapfill(NULL, &L->view0, 1, v->W, ctx->stream);
    if (e) return fs_cuda_fail(ctx, e, "gap-fill kernel launch");
    ctx->launches++;
  }
  if (ctx->time_kernel) {
    cudaEventRecord(ctx->ev_kernel[1], ctx->stream);
    ctx->kernel_timed = 1;
  }
  return FS_OK;
}

int fs_render_device(fs_ctx *ctx, const fs_map *map, const fs_camera *cam,
                     const fs_params *params, int32_t width, int32_t height,
                     uint32_t *out_dev) {
  if (!ctx) return FS_ERR_ARG;
  if (ctx->broken) return fs_fail(ctx, FS_ERR_STATE, "context failed to initialise");
  if (!map || !out_dev) return fs_fail(ctx, FS_ERR_ARG, "NULL map or output");
  fs_params dp = fs_params_default();
  FsView v;
  int rc = fs_make_view(ctx, cam, params ? params : &dp, width, height, 0, &v);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  rc = fs_ensure_ztable(ctx, v.n);
  if (rc) return rc;
  v.out = out_dev;
  return fs_render_view(ctx, &map->dev, &v, NULL, ctx->zline, ctx->zinvz, NULL, 1);
}

int fs_render(fs_ctx *ctx, const fs_map *map, const fs_camera *cam, const fs_params *params,
              int32_t width, int32_t height, uint32_t *out_host) {
  if (!ctx) return FS_ERR_ARG;
  if (!out_host) return fs_fail(ctx, FS_ERR_ARG, "NULL output");
  if (width <= 0 || height <= 0) return fs_fail(ctx, FS_ERR_ARG, "bad screen size");
  cudaSetDevice(ctx->device);
  const size_t bytes = (size_t)width * (size_t)height * 4;
  if (bytes > ctx->frame_cap) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->frame_dev);
    ctx->frame_dev = NULL;
    ctx->frame_cap = 0;
    if (cudaMalloc((void **)&ctx->frame_dev, bytes) != cudaSuccess)
      return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(frame %zu bytes)", bytes);
    ctx->frame_cap = bytes;
  }
  int rc = fs_render_device(ctx, map, cam, params, width, height, ctx->frame_dev);
  if (rc) return rc;
  int e = cudaMemcpyAsync(out_host, ctx->frame_dev, bytes, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "frame download");
  return FS_OK;
}
