/*
 * The Futhark-generated C API of fut/interactive_entrypoints.fut (libfutspace.h),
 * implemented over the CUDA renderer, so c/interactive.c and lys link against
 * this library unchanged.
 *
 * The application state of fut/interactive.fut (camera, screen size, key
 * flags, sun parameters, the landscape maps) lives on the host, except for the
 * maps, which stay on the device. States are immutable; maps are shared
 * between states by reference counts. The per-frame `render` entry runs the
 * renderer with the reference's live configuration: bilinear height over the
 * altitude map and bilinear colour over the shadowed colour map
 * (fut/interactive.fut:179-183).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/libfutspace.h"
#include "fs_internal.h"
#include "fs_priv.h"

/* ---- configuration / context --------------------------------------------- */

struct futhark_context_config {
  int32_t device;
  int32_t debugging;
};

struct futhark_context {
  fs_ctx *fs;
};

struct futhark_context_config *futhark_context_config_new(void) {
  return (struct futhark_context_config *)calloc(1, sizeof(struct futhark_context_config));
}

void futhark_context_config_free(struct futhark_context_config *cfg) { free(cfg); }

void futhark_context_config_set_device(struct futhark_context_config *cfg, const char *s) {
  if (!cfg || !s) return;
  while (*s && (*s < '0' || *s > '9')) s++; /* "cuda:3", "#3", "3" */
  if (*s) cfg->device = atoi(s);
}

void futhark_context_config_set_debugging(struct futhark_context_config *cfg, int flag) {
  if (cfg) cfg->debugging = flag;
}
void futhark_context_config_set_logging(struct futhark_context_config *cfg, int flag) {
  (void)cfg;
  (void)flag;
}
void futhark_context_config_set_profiling(struct futhark_context_config *cfg, int flag) {
  (void)cfg;
  (void)flag;
}
void futhark_context_config_select_device_interactively(struct futhark_context_config *cfg) {
  (void)cfg;
}

struct futhark_context *futhark_context_new(struct futhark_context_config *cfg) {
  struct futhark_context *c = (struct futhark_context *)calloc(1, sizeof(*c));
  if (!c) return NULL;
  int rc = fs_ctx_new(&c->fs, cfg ? cfg->device : 0);
  if (rc && !c->fs) {
    free(c);
    return NULL;
  }
  /* on a CUDA failure the context is kept so futhark_context_get_error works */
  return c;
}

void futhark_context_free(struct futhark_context *ctx) {
  if (!ctx) return;
  fs_ctx_free(ctx->fs);
  free(ctx);
}

int futhark_context_sync(struct futhark_context *ctx) {
  return ctx ? fs_ctx_sync(ctx->fs) : FS_ERR_ARG;
}

char *futhark_context_get_error(struct futhark_context *ctx) {
  return ctx ? fs_ctx_get_error(ctx->fs) : NULL;
}

int futhark_context_clear_caches(struct futhark_context *ctx) { return ctx ? FS_OK : FS_ERR_ARG; }

char *futhark_context_report(struct futhark_context *ctx) {
  char *s = (char *)malloc(96);
  if (s) snprintf(s, 96, "render kernel launches: %lld\n",
                  (long long)(ctx ? fs_ctx_kernel_launches(ctx->fs) : 0));
  return s;
}

/* ---- arrays ------------------------------------------------------------------ */

struct futhark_u32_2d {
  uint32_t *dev;
  int64_t shape[2];
};
struct futhark_i32_2d {
  int32_t *dev;
  int64_t shape[2];
};

static void *compat_alloc(struct futhark_context *ctx, size_t bytes) {
  void *p = NULL;
  cudaSetDevice(ctx->fs->device);
  if (cudaMalloc(&p, bytes ? bytes : 4) != cudaSuccess) {
    fs_fail(ctx->fs, FS_ERR_NOMEM, "cudaMalloc(%zu bytes)", bytes);
    return NULL;
  }
  return p;
}

static int compat_shape_ok(struct futhark_context *ctx, int64_t d0, int64_t d1) {
  if (d0 < 0 || d1 < 0 || d0 > (1 << 20) || d1 > (1 << 20)) {
    fs_fail(ctx->fs, FS_ERR_ARG, "array shape %lldx%lld out of range", (long long)d0,
            (long long)d1);
    return 0;
  }
  return 1;
}

struct futhark_u32_2d *futhark_new_u32_2d(struct futhark_context *ctx, const uint32_t *data,
                                          int64_t dim0, int64_t dim1) {
  if (!ctx || !data || !compat_shape_ok(ctx, dim0, dim1)) return NULL;
  struct futhark_u32_2d *a = (struct futhark_u32_2d *)calloc(1, sizeof(*a));
  if (!a) return NULL;
  const size_t bytes = (size_t)dim0 * (size_t)dim1 * 4;
  a->dev = (uint32_t *)compat_alloc(ctx, bytes);
  a->shape[0] = dim0;
  a->shape[1] = dim1;
  if (!a->dev || cudaMemcpy(a->dev, data, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(a->dev);
    free(a);
    fs_fail(ctx->fs, FS_ERR_CUDA, "futhark_new_u32_2d: upload failed");
    return NULL;
  }
  return a;
}

struct futhark_i32_2d *futhark_new_i32_2d(struct futhark_context *ctx, const int32_t *data,
                                          int64_t dim0, int64_t dim1) {
  if (!ctx || !data || !compat_shape_ok(ctx, dim0, dim1)) return NULL;
  struct futhark_i32_2d *a = (struct futhark_i32_2d *)calloc(1, sizeof(*a));
  if (!a) return NULL;
  const size_t bytes = (size_t)dim0 * (size_t)dim1 * 4;
  a->dev = (int32_t *)compat_alloc(ctx, bytes);
  a->shape[0] = dim0;
  a->shape[1] = dim1;
  if (!a->dev || cudaMemcpy(a->dev, data, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(a->dev);
    free(a);
    fs_fail(ctx->fs, FS_ERR_CUDA, "futhark_new_i32_2d: upload failed");
    return NULL;
  }
  return a;
}

int futhark_free_u32_2d(struct futhark_context *ctx, struct futhark_u32_2d *arr) {
  if (!arr) return FS_OK;
  if (ctx) cudaSetDevice(ctx->fs->device);
  cudaFree(arr->dev);
  free(arr);
  return FS_OK;
}

int futhark_free_i32_2d(struct futhark_context *ctx, struct futhark_i32_2d *arr) {
  if (!arr) return FS_OK;
  if (ctx) cudaSetDevice(ctx->fs->device);
  cudaFree(arr->dev);
  free(arr);
  return FS_OK;
}

int futhark_values_u32_2d(struct futhark_context *ctx, struct futhark_u32_2d *arr,
                          uint32_t *data) {
  if (!ctx || !arr || !data) return FS_ERR_ARG;
  cudaSetDevice(ctx->fs->device);
  int e = cudaMemcpyAsync(data, arr->dev, (size_t)arr->shape[0] * arr->shape[1] * 4,
                          cudaMemcpyDeviceToHost, ctx->fs->stream);
  if (!e) e = cudaStreamSynchronize(ctx->fs->stream);
  return e ? fs_cuda_fail(ctx->fs, e, "futhark_values_u32_2d") : FS_OK;
}

int futhark_values_i32_2d(struct futhark_context *ctx, struct futhark_i32_2d *arr,
                          int32_t *data) {
  if (!ctx || !arr || !data) return FS_ERR_ARG;
  cudaSetDevice(ctx->fs->device);
  int e = cudaMemcpyAsync(data, arr->dev, (size_t)arr->shape[0] * arr->shape[1] * 4,
                          cudaMemcpyDeviceToHost, ctx->fs->stream);
  if (!e) e = cudaStreamSynchronize(ctx->fs->stream);
  return e ? fs_cuda_fail(ctx->fs, e, "futhark_values_i32_2d") : FS_OK;
}

const int64_t *futhark_shape_u32_2d(struct futhark_context *ctx, struct futhark_u32_2d *arr) {
  (void)ctx;
  return arr ? arr->shape : NULL;
}

const int64_t *futhark_shape_i32_2d(struct futhark_context *ctx, struct futhark_i32_2d *arr) {
  (void)ctx;
  return arr ? arr->shape : NULL;
}

unsigned char *futhark_values_raw_u32_2d(struct futhark_context *ctx,
                                         struct futhark_u32_2d *arr) {
  (void)ctx;
  return arr ? (unsigned char *)arr->dev : NULL;
}

/* ---- landscape: device maps shared between states ----------------------------- */

typedef struct {
  int32_t refs;
  int32_t rows, cols;
  void *dev;     /* device data */
  uint8_t *host; /* masked altitude on the host (terrain_collision) or NULL */
} fs_buf;

static fs_buf *buf_new(int32_t rows, int32_t cols, void *dev, uint8_t *host) {
  fs_buf *b = (fs_buf *)calloc(1, sizeof(fs_buf));
  if (!b) return NULL;
  b->refs = 1;
  b->rows = rows;
  b->cols = cols;
  b->dev = dev;
  b->host = host;
  return b;
}

static fs_buf *buf_ref(fs_buf *b) {
  if (b) b->refs++;
  return b;
}

static void buf_unref(fs_buf *b) {
  if (!b || --b->refs > 0) return;
  cudaFree(b->dev);
  free(b->host);
  free(b);
}

/* landscape record, fut/voxel_renderer.fut:14-18 */
typedef struct {
  fs_buf *altitude; /* dev: height quads */
  fs_buf *color;    /* dev: u32 colours */
  fs_buf *shadowed; /* dev: u32 colours (1024x1024 once a map is loaded) */
} fs_landscape;

/* ---- state, fut/interactive.fut:9-24 --------------------------------------------
 * Key flags in input order of fut/interactive_input.fut:6-48: a..z, arrow up,
 * left, down, right, 1..9, 0. */
enum { K_ARROW_UP = 26, K_ARROW_LEFT = 27, K_ARROW_DOWN = 28, K_ARROW_RIGHT = 29, K_DIGIT1 = 30,
       K_DIGIT0 = 39, K_COUNT = 40 };
enum { MODE_PNG = 0, MODE_MATH = 1 };

struct futhark_opaque_state {
  int32_t mode;
  int32_t smoothing; /* 0: #off, 1: #on */
  fs_camera cam;
  fs_landscape lsc;
  int32_t height, width;
  int8_t inputs[K_COUNT];
  float random, sun_height, sun_ang;
  float sun[3];
};

static struct futhark_opaque_state *state_copy(const struct futhark_opaque_state *s) {
  struct futhark_opaque_state *n =
      (struct futhark_opaque_state *)malloc(sizeof(struct futhark_opaque_state));
  if (!n) return NULL;
  *n = *s;
  buf_ref(n->lsc.altitude);
  buf_ref(n->lsc.color);
  buf_ref(n->lsc.shadowed);
  return n;
}

int futhark_free_opaque_state(struct futhark_context *ctx, struct futhark_opaque_state *obj) {
  (void)ctx;
  if (!obj) return FS_OK;
  if (ctx) cudaSetDevice(ctx->fs->device);
  buf_unref(obj->lsc.altitude);
  buf_unref(obj->lsc.color);
  buf_unref(obj->lsc.shadowed);
  free(obj);
  return FS_OK;
}

/* SDL keycode -> input slot (fut/interactive_input.fut:50-134) */
static int key_slot(int32_t key) {
  if (key >= 'a' && key <= 'z') return key - 'a';
  if (key >= '1' && key <= '9') return K_DIGIT1 + (key - '1');
  if (key == '0') return K_DIGIT0;
  switch (key) {
    case 0x40000052: return K_ARROW_UP;    /* SDLK_UP */
    case 0x40000050: return K_ARROW_LEFT;  /* SDLK_LEFT */
    case 0x40000051: return K_ARROW_DOWN;  /* SDLK_DOWN */
    case 0x4000004F: return K_ARROW_RIGHT; /* SDLK_RIGHT */
    default: return -1;
  }
}

/* matte 0.1.2 colourspace.scale, restated: RGB times s, alpha kept, then
 * from_rgba (clamp to [0,1], times 255, truncate). */
static uint32_t to_byte_host(float x) {
  x = (x < 0.0f) ? 0.0f : ((x > 1.0f) ? 1.0f : x);
  const float v = x * 255.0f;
  return (v != v) ? 0u : (uint32_t)v;
}

static uint32_t argb_scale(uint32_t c, float s) {
  const float r = (float)((c >> 16) & 0xFFu) / 255.0f, g = (float)((c >> 8) & 0xFFu) / 255.0f;
  const float b = (float)(c & 0xFFu) / 255.0f, a = (float)((c >> 24) & 0xFFu) / 255.0f;
  return (to_byte_host(a) << 24) | (to_byte_host(r * s) << 16) | (to_byte_host(g * s) << 8) |
         to_byte_host(b * s);
}

/* vec3_rotate #y sun_ang (vec3_rotate #z sun_height sun) (fut/effects.fut:6-25,
 * fut/interactive.fut:126-145): rotation matrices times the vector, each
 * component a dot product summed left to right from 0 (linalg matvecmul_row). */
static void sun_vector(const float sun[3], float sun_height, float sun_ang, float out[3]) {
  const float ch = cosf(sun_height), sh = sinf(sun_height);
  const float rz[3][3] = {{ch, -sh, 0.0f}, {sh, ch, 0.0f}, {0.0f, 0.0f, 1.0f}};
  float v1[3];
  for (int i = 0; i < 3; i++) v1[i] = ((0.0f + rz[i][0] * sun[0]) + rz[i][1] * sun[1]) + rz[i][2] * sun[2];
  const float ca = cosf(sun_ang), sa = sinf(sun_ang);
  const float ry[3][3] = {{ca, 0.0f, sa}, {0.0f, 1.0f, 0.0f}, {-sa, 0.0f, ca}};
  for (int i = 0; i < 3; i++) out[i] = ((0.0f + ry[i][0] * v1[0]) + ry[i][1] * v1[1]) + ry[i][2] * v1[2];
}

/* generate_shadowmap_accumulated over the state's maps (1024x1024 result). */
static fs_buf *make_shadowed(struct futhark_context *ctx, const fs_landscape *l, float sun_height,
                             float sun_ang, const float sun[3]) {
  float sv[3];
  sun_vector(sun, sun_height, sun_ang, sv);
  uint32_t *out = (uint32_t *)compat_alloc(ctx, 1024 * 1024 * 4);
  if (!out) return NULL;
  FsMapDev M;
  memset(&M, 0, sizeof(M));
  M.q = (const uint32_t *)l->altitude->dev;
  M.c = (const uint32_t *)l->color->dev;
  M.MH = M.CH = l->altitude->rows;
  M.MW = M.CW = l->altitude->cols;
  M.pow2 = M.cpow2 = ((M.MH & (M.MH - 1)) == 0) && ((M.MW & (M.MW - 1)) == 0);
  int e = fsk_shadowmap(&M, sv, out, ctx->fs->stream);
  if (e) {
    cudaFree(out);
    fs_cuda_fail(ctx->fs, e, "shadow-map kernel");
    return NULL;
  }
  ctx->fs->launches++;
  fs_buf *b = buf_new(1024, 1024, out, NULL);
  if (!b) cudaFree(out);
  return b;
}

/* init, fut/interactive.fut:28-57 */
int futhark_entry_init(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                       const uint32_t seed) {
  (void)seed;
  if (!ctx || !out0) return FS_ERR_ARG;
  struct futhark_opaque_state *s =
      (struct futhark_opaque_state *)calloc(1, sizeof(struct futhark_opaque_state));
  if (!s) return fs_fail(ctx->fs, FS_ERR_NOMEM, "init: out of memory");
  s->mode = MODE_PNG;
  s->smoothing = 0;
  s->cam.x = 0.98f;
  s->cam.y = 0.6f;
  s->cam.height = 58.0f;
  s->cam.angle = 2.2f;
  s->cam.horizon = 200.0f;
  s->cam.distance = 800.0f;
  s->cam.fov = 1.2f;
  s->cam.sky_color = 0;
  s->height = 1024;
  s->width = 1024;
  s->random = 1.0f;
  s->sun_height = 0.1f;
  s->sun_ang = 0.1f;
  s->sun[0] = 0.0f;
  s->sun[1] = 1.0f / sqrtf(1.0f);
  s->sun[2] = 0.0f;
  /* dummy 2x1 landscape of zeros until update_map loads a map */
  uint32_t *q = (uint32_t *)compat_alloc(ctx, 2 * 4), *c = (uint32_t *)compat_alloc(ctx, 2 * 4),
           *sc = (uint32_t *)compat_alloc(ctx, 2 * 4);
  uint8_t *hh = (uint8_t *)calloc(2, 1);
  if (!q || !c || !sc || !hh) {
    cudaFree(q);
    cudaFree(c);
    cudaFree(sc);
    free(hh);
    free(s);
    return fs_fail(ctx->fs, FS_ERR_NOMEM, "init: out of memory");
  }
  cudaMemset(q, 0, 8);
  cudaMemset(c, 0, 8);
  cudaMemset(sc, 0, 8);
  s->lsc.altitude = buf_new(2, 1, q, hh);
  s->lsc.color = buf_new(2, 1, c, NULL);
  s->lsc.shadowed = buf_new(2, 1, sc, NULL);
  *out0 = s;
  return FS_OK;
}

/* resize, fut/interactive.fut:59-61 */
int futhark_entry_resize(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                         const int32_t h, const int32_t w,
                         const struct futhark_opaque_state *in) {
  if (!ctx || !out0 || !in) return FS_ERR_ARG;
  struct futhark_opaque_state *s = state_copy(in);
  if (!s) return fs_fail(ctx->fs, FS_ERR_NOMEM, "resize: out of memory");
  s->height = h;
  s->width = w;
  *out0 = s;
  return FS_OK;
}

/* key (fut/interactive_entrypoints.fut:9-11): e == 0 is keydown */
int futhark_entry_key(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                      const int32_t e, const int32_t key, const struct futhark_opaque_state *in) {
  if (!ctx || !out0 || !in) return FS_ERR_ARG;
  struct futhark_opaque_state *s = state_copy(in);
  if (!s) return fs_fail(ctx->fs, FS_ERR_NOMEM, "key: out of memory");
  const int slot = key_slot(key);
  if (slot >= 0) s->inputs[slot] = (e == 0) ? 1 : 0;
  *out0 = s;
  return FS_OK;
}

/* mouse and wheel events leave the state unchanged (fut/interactive.fut:166-171) */
int futhark_entry_mouse(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                        const int32_t buttons, const int32_t x, const int32_t y,
                        const struct futhark_opaque_state *in) {
  (void)buttons;
  (void)x;
  (void)y;
  if (!ctx || !out0 || !in) return FS_ERR_ARG;
  *out0 = state_copy(in);
  return *out0 ? FS_OK : fs_fail(ctx->fs, FS_ERR_NOMEM, "mouse: out of memory");
}

int futhark_entry_wheel(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                        const int32_t dx, const int32_t dy,
                        const struct futhark_opaque_state *in) {
  (void)dx;
  (void)dy;
  if (!ctx || !out0 || !in) return FS_ERR_ARG;
  *out0 = state_copy(in);
  return *out0 ? FS_OK : fs_fail(ctx->fs, FS_ERR_NOMEM, "wheel: out of memory");
}

/* `squares` of fut/render_functions.fut:4-11 (math-mode terrain), with the
 * floored float modulo. */
static float squares(float x, float y) {
  x = x - 1024.0f * floorf(x / 1024.0f);
  y = y - 1024.0f * floorf(y / 1024.0f);
  return (x > 256.0f && fabsf(x) < 768.0f && fabsf(y) > 256.0f && fabsf(y) < 768.0f) ? 200.0f
                                                                                      : 0.0f;
}

/* terrain_collision, fut/interactive.fut:67-87 */
static void terrain_collision(struct futhark_opaque_state *s) {
  float th;
  if (s->mode == MODE_MATH) {
    th = squares(s->cam.x, s->cam.y);
  } else {
    const fs_buf *a = s->lsc.altitude;
    const int32_t x = fs_f2i_host(s->cam.x), y = fs_f2i_host(s->cam.y);
    int32_t iy = y % a->rows, ix = x % a->cols;
    if (iy < 0) iy += a->rows;
    if (ix < 0) ix += a->cols;
    th = (float)a->host[(size_t)iy * a->cols + ix];
  }
  if (s->cam.height <= th) s->cam.height = th;
}

/* step, fut/interactive.fut:161-164, with process_inputs (:89-159). Every new
 * field is computed from the state before the step (Futhark record updates
 * read the original record). */
int futhark_entry_step(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                       const float td, const struct futhark_opaque_state *in) {
  (void)td;
  if (!ctx || !out0 || !in) return FS_ERR_ARG;
  struct futhark_opaque_state *s = state_copy(in);
  if (!s) return fs_fail(ctx->fs, FS_ERR_NOMEM, "step: out of memory");
  s->random = in->random + 0.005f;
  s->cam.sky_color = argb_scale(0xFF9090E0u, in->sun_height);
  const struct futhark_opaque_state o = *s; /* the record process_inputs reads */
  const int8_t *k = o.inputs;
  const float sa = sinf(o.cam.angle), ca = cosf(o.cam.angle);
  s->cam.x = k['w' - 'a'] == 1 ? o.cam.x - 3.0f * sa : (k['s' - 'a'] == 1 ? o.cam.x + 3.0f * sa : o.cam.x);
  s->cam.y = k['w' - 'a'] == 1 ? o.cam.y - 3.0f * ca : (k['s' - 'a'] == 1 ? o.cam.y + 3.0f * ca : o.cam.y);
  s->cam.angle = k['d' - 'a'] == 1 ? o.cam.angle - 0.10f
                                   : (k['a' - 'a'] == 1 ? o.cam.angle + 0.10f : o.cam.angle);
  s->cam.horizon = k['e' - 'a'] == 1 ? o.cam.horizon - 20.0f
                                     : (k['q' - 'a'] == 1 ? o.cam.horizon + 20.0f : o.cam.horizon);
  s->cam.height = k['r' - 'a'] == 1 ? o.cam.height + 10.0f
                                    : (k['f' - 'a'] == 1 ? o.cam.height - 10.0f : o.cam.height);
  s->cam.distance = k[K_ARROW_UP] == 1 ? o.cam.distance + 30.0f
                                       : (k[K_ARROW_DOWN] == 1 ? o.cam.distance - 30.0f
                                                               : o.cam.distance);
  s->cam.fov = k['o' - 'a'] == 1 ? o.cam.fov + 0.1f
                                 : (k['l' - 'a'] == 1 ? o.cam.fov - 0.1f : o.cam.fov);
  s->sun_height = k['u' - 'a'] == 1 ? o.sun_height + 0.005f
                                    : (k['j' - 'a'] == 1 ? o.sun_height - 0.005f : o.sun_height);
  s->sun_ang = k['n' - 'a'] == 1 ? o.sun_ang + 0.005f
                                 : (k['m' - 'a'] == 1 ? o.sun_ang - 0.005f : o.sun_ang);
  if (k['u' - 'a'] == 1 || k['j' - 'a'] == 1 || k['n' - 'a'] == 1 || k['m' - 'a'] == 1) {
    fs_buf *sh = make_shadowed(ctx, &o.lsc, o.sun_height, o.sun_ang, o.sun);
    if (!sh) {
      futhark_free_opaque_state(ctx, s);
      return FS_ERR_CUDA;
    }
    buf_unref(s->lsc.shadowed);
    s->lsc.shadowed = sh;
  }
  if (k[K_DIGIT1] == 1) s->mode = o.mode == MODE_PNG ? MODE_MATH : MODE_PNG;
  if (k[K_DIGIT1 + 1] == 1) s->smoothing = o.smoothing ? 0 : 1;
  terrain_collision(s);
  *out0 = s;
  return FS_OK;
}

/* render, fut/interactive.fut:173-183 (`#png` mode): bilinear height over the
 * altitude map, bilinear colour over the shadowed colour map, reference depth
 * schedule, [height][width] frame. */
int futhark_entry_render(struct futhark_context *ctx, struct futhark_u32_2d **out0,
                         const struct futhark_opaque_state *in) {
  if (!ctx || !out0 || !in) return FS_ERR_ARG;
  if (in->mode == MODE_MATH)
    return fs_fail(ctx->fs, FS_ERR_STATE,
                   "render: math mode (fut/interactive.fut:175-178) is not provided");
  const int32_t H = in->height, W = in->width;
  fs_params p = fs_params_default();
  p.smoothing = in->smoothing; /* key 2 toggles `#on` (fut/interactive.fut:120-125) */
  FsView v;
  int rc = fs_make_view(ctx->fs, &in->cam, &p, W, H, 0, &v);
  if (rc) return rc;
  rc = fs_ensure_ztable(ctx->fs, v.n);
  if (rc) return rc;
  struct futhark_u32_2d *a = (struct futhark_u32_2d *)calloc(1, sizeof(*a));
  if (!a) return fs_fail(ctx->fs, FS_ERR_NOMEM, "render: out of memory");
  a->shape[0] = H;
  a->shape[1] = W;
  a->dev = (uint32_t *)compat_alloc(ctx, (size_t)W * H * 4);
  if (!a->dev) {
    free(a);
    return FS_ERR_NOMEM;
  }
  FsMapDev M;
  memset(&M, 0, sizeof(M));
  M.q = (const uint32_t *)in->lsc.altitude->dev;
  M.c = (const uint32_t *)in->lsc.shadowed->dev;
  M.MH = in->lsc.altitude->rows;
  M.MW = in->lsc.altitude->cols;
  M.CH = in->lsc.shadowed->rows;
  M.CW = in->lsc.shadowed->cols;
  M.pow2 = ((M.MH & (M.MH - 1)) == 0) && ((M.MW & (M.MW - 1)) == 0);
  M.cpow2 = ((M.CH & (M.CH - 1)) == 0) && ((M.CW & (M.CW - 1)) == 0);
  v.out = a->dev;
  rc = fs_render_view(ctx->fs, &M, &v, NULL, ctx->fs->zline, ctx->fs->zinvz, NULL, 1);
  if (rc) {
    futhark_free_u32_2d(ctx, a);
    return rc;
  }
  *out0 = a;
  return FS_OK;
}

/* text_content, fut/interactive.fut:185-186 */
int futhark_entry_text_content(struct futhark_context *ctx, float *x, float *y, float *angle,
                               float *height, float *horizon, float *distance,
                               float *sun_height, float *sun_ang, float *fov,
                               const struct futhark_opaque_state *in) {
  if (!ctx || !in || !x || !y || !angle || !height || !horizon || !distance || !sun_height ||
      !sun_ang || !fov)
    return FS_ERR_ARG;
  *x = in->cam.x;
  *y = in->cam.y;
  *angle = in->cam.angle;
  *height = in->cam.height;
  *horizon = in->cam.horizon;
  *distance = in->cam.distance;
  *sun_height = in->sun_height;
  *sun_ang = in->sun_ang;
  *fov = in->cam.fov;
  return FS_OK;
}

/* update_map, fut/interactive.fut:188-198: heights masked to their low byte,
 * colours copied, shadowed colours recomputed with the current sun. */
int futhark_entry_update_map(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                             const struct futhark_u32_2d *color_map,
                             const struct futhark_i32_2d *height_map,
                             const struct futhark_opaque_state *in) {
  if (!ctx || !out0 || !in || !color_map || !height_map) return FS_ERR_ARG;
  const int64_t rows = height_map->shape[0], cols = height_map->shape[1];
  if (color_map->shape[0] != rows || color_map->shape[1] != cols || rows < 1 || cols < 1 ||
      rows > 65536 || cols > 65536 || rows * cols > FS_MAX_TEXELS)
    return fs_fail(ctx->fs, FS_ERR_ARG, "update_map: colour %lldx%lld vs height %lldx%lld",
                   (long long)color_map->shape[0], (long long)color_map->shape[1],
                   (long long)rows, (long long)cols);
  cudaSetDevice(ctx->fs->device);
  const size_t cnt = (size_t)rows * (size_t)cols;
  uint8_t *h8 = (uint8_t *)compat_alloc(ctx, cnt);
  uint32_t *q = (uint32_t *)compat_alloc(ctx, cnt * 4);
  uint32_t *c = (uint32_t *)compat_alloc(ctx, cnt * 4);
  uint8_t *host = (uint8_t *)malloc(cnt);
  int e = (!h8 || !q || !c || !host) ? (int)cudaErrorMemoryAllocation : 0;
  cudaStream_t st = ctx->fs->stream;
  if (!e) e = fsk_mask_heights(height_map->dev, h8, (int64_t)cnt, st);
  if (!e) e = fsk_build_quads(h8, q, (int32_t)rows, (int32_t)cols, st);
  if (!e) e = cudaMemcpyAsync(c, color_map->dev, cnt * 4, cudaMemcpyDeviceToDevice, st);
  if (!e) e = cudaMemcpyAsync(host, h8, cnt, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  cudaFree(h8);
  if (e) {
    cudaFree(q);
    cudaFree(c);
    free(host);
    return fs_cuda_fail(ctx->fs, e, "update_map");
  }
  struct futhark_opaque_state *s = state_copy(in);
  if (!s) {
    cudaFree(q);
    cudaFree(c);
    free(host);
    return fs_fail(ctx->fs, FS_ERR_NOMEM, "update_map: out of memory");
  }
  buf_unref(s->lsc.altitude);
  buf_unref(s->lsc.color);
  s->lsc.altitude = buf_new((int32_t)rows, (int32_t)cols, q, host);
  s->lsc.color = buf_new((int32_t)rows, (int32_t)cols, c, NULL);
  fs_buf *sh = (s->lsc.altitude && s->lsc.color)
                   ? make_shadowed(ctx, &s->lsc, in->sun_height, in->sun_ang, in->sun)
                   : NULL;
  if (!sh) {
    futhark_free_opaque_state(ctx, s);
    return FS_ERR_CUDA;
  }
  buf_unref(s->lsc.shadowed);
  s->lsc.shadowed = sh;
  *out0 = s;
  return FS_OK;
}
