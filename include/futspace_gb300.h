/*
 * futspace_gb300: Voxel Space terrain renderer for one NVIDIA GB300 (sm_103a).
 *
 * Direct C ABI. Plain pointers and sizes; every function returns an int status
 * (FS_OK == 0) and never exits the process. The Futhark-compatible names that
 * the reference's host program links against are in libfutspace.h.
 *
 * The renderer is the reference's per-frame `render`
 * (fut/voxel_renderer.fut:101-251, `#off` branch) with the samplers of
 * fut/render_functions.fut:63-105, reached from fut/interactive.fut:173-183.
 */
#ifndef FUTSPACE_GB300_H
#define FUTSPACE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define FS_OK 0
#define FS_ERR_ARG 1      /* bad argument (null pointer, size out of range, ...) */
#define FS_ERR_CUDA 2     /* a CUDA runtime call failed (text in fs_ctx_get_error) */
#define FS_ERR_RANGE 3    /* depth schedule has no samples: the reference raises an
                             invalid-range error on `1...n` (fut/voxel_renderer.fut:33) */
#define FS_ERR_NOMEM 4    /* host or device allocation failed */
#define FS_ERR_BUDGET 5   /* serving: request exceeds the framebuffer budget */
#define FS_ERR_STATE 6    /* object used in the wrong state */
#define FS_ERR_IO 7       /* file missing, unreadable or not in the expected format */

/* ---- value types ---------------------------------------------------------- */

/* Camera record of fut/voxel_renderer.fut:5-12. `horizon` is the screen row of
 * the horizon (the reference's pitch control, fut/interactive.fut:102-104);
 * `angle` is the yaw in radians; `distance` the draw distance. */
typedef struct {
  float x, y, height, angle, horizon, distance, fov;
  uint32_t sky_color; /* ARGB */
} fs_camera;

enum { FS_NEAREST = 0, FS_BILINEAR = 1 };
enum { FS_GAP_ZERO = 0, FS_GAP_SKY = 1 };
/* Optional colour epilogue (not in the reference; 0 renders the reference's
 * frames). Applied to every depth sample's colour before occlusion, in matte's
 * colour arithmetic, with z the sample's depth and D the draw distance:
 *   FS_FX_SHADE: c = scale(c, 1 - shade * (z / D))                 depth shading
 *   FS_FX_FOG:   f = clamp((z - fog_start) / (fog_end - fog_start), 0, 1);
 *                c = mix(1 - f, c, f, fog_color)                     distance fog */
enum { FS_FX_SHADE = 1, FS_FX_FOG = 2 };

/* Render parameters.
 *  invz_param1 : depth step d of the arithmetic depth series
 *                (reference default 0.001, fut/voxel_renderer.fut:104)
 *  invz_param2 : first depth z0 (default 0.0, :103)
 *  magic_number: projection scale in inv_z = (1/z) * scale; <= 0 selects the
 *                reference's f32(w/2) with integer division (:217)
 *  height_filter, color_filter: FS_BILINEAR is png_height_filtered /
 *                png_color_filtered (fut/render_functions.fut:67-77, 95-105),
 *                FS_NEAREST is png_height / png_color (:63-64, 91-92).
 *  gap_rule    : FS_GAP_ZERO fills colour-0 gaps and then paints 0 as sky
 *                (fut/voxel_renderer.fut:78-81, 246-248); FS_GAP_SKY treats the
 *                sky colour as the gap (tests/futspace.fut:110-121).
 *  floor_n     : 1 floors the depth count before the i32 conversion
 *                (fut/voxel_renderer.fut:32); 0 converts directly
 *                (tests/futspace.fut:51). Identical for positive counts.
 *  effects, shade, fog_start, fog_end, fog_color: the optional epilogue
 *                above (FS_FX_* flags; fog needs fog_end > fog_start).
 *  smoothing   : 1 renders the reference's `#on` smoothing branch
 *                (fut/voxel_renderer.fut:175-213, key 2 of the interactive app):
 *                rows between two consecutive new minima blend their colours;
 *                colour 0 becomes sky. Requires FS_GAP_ZERO.
 * fs_params_default() gives the live reference path: 0.001, 0.0, w/2,
 * bilinear height and colour, FS_GAP_ZERO, floor_n 1, no effects. */
typedef struct {
  float invz_param1;
  float invz_param2;
  float magic_number;
  int32_t height_filter;
  int32_t color_filter;
  int32_t gap_rule;
  int32_t floor_n;
  int32_t effects;
  float shade;
  float fog_start, fog_end;
  uint32_t fog_color;
  int32_t smoothing;
} fs_params;

/* One view of a batch: a camera, a screen size and the map it samples. */
typedef struct {
  fs_camera cam;
  int32_t width, height; /* W columns x H rows */
  int32_t map;           /* index into the maps given to fs_plan_new */
  int32_t reserved;
} fs_view;

typedef struct fs_ctx fs_ctx;
typedef struct fs_map fs_map;
typedef struct fs_plan fs_plan;

/* ---- context ------------------------------------------------------------- */
fs_params fs_params_default(void);
int fs_ctx_new(fs_ctx **out, int32_t device);
void fs_ctx_free(fs_ctx *ctx);
/* Last error text as a malloc'd string the caller frees; NULL when none. */
char *fs_ctx_get_error(fs_ctx *ctx);
int fs_ctx_sync(fs_ctx *ctx);
/* Stream used by every asynchronous call of this context (a cudaStream_t);
 * NULL restores the context's own stream. */
int fs_ctx_set_stream(fs_ctx *ctx, void *stream);
void *fs_ctx_get_stream(fs_ctx *ctx);
/* Number of render kernels this context launched so far. */
int64_t fs_ctx_kernel_launches(fs_ctx *ctx);
/* Kernel configurations are int32_t[5]: {tile width (columns per CTA), lanes
 * per column, depth samples per lane per chunk, stage (1: shared-memory column
 * stage + TMA row stores, 0: direct painting), persistent CTAs (0: fill GPU)}.
 * fs_ctx_force_tune fixes the configuration of every following single-frame
 * render; NULL or tile width 0 restores the tuning-cache / default choice. */
int fs_ctx_force_tune(fs_ctx *ctx, const int32_t tune5[5]);
/* Context options: "skip" (1, default: skip depth chunks that a max-pyramid
 * bound proves cannot change the frame; 0: march every depth sample), "tma"
 * (1, default when the driver provides tensor maps: TMA row stores from the
 * staged kernels; 0: plain stores) and "split" (1, default: when a launch has
 * too few column strips to occupy the GPU, split each column's depth range
 * into segments marched by separate warps, after a pass that finds each
 * segment's minimum row; 0: never). Plans capture the options at creation or
 * retuning. Pixels are identical either way. Option "time" (0, default; 1:
 * record CUDA events around the kernels of every plain per-frame call, read
 * with fs_ctx_kernel_ms) changes no pixel either. */
int fs_ctx_set_option(fs_ctx *ctx, const char *name, int64_t value);
/* Device time in ms of the kernels (depth table and render) of the last plain
 * per-frame call made with option "time" on; waits for that call.
 * FS_ERR_STATE when no such call was made. */
int fs_ctx_kernel_ms(fs_ctx *ctx, float *ms);

/* Page-locked host memory (cudaMallocHost) for frame downloads that should not
 * block the calling thread, e.g. fs_request.host_out. */
void *fs_host_alloc(size_t bytes);
void fs_host_free(void *p);

/* ---- maps ---------------------------------------------------------------- */
/* Copies a [rows][cols] u8 height map and ARGB colour map from host memory to
 * the device. The maps stay resident until fs_map_free. */
int fs_map_new(fs_ctx *ctx, fs_map **out, const uint8_t *heights, const uint32_t *colors,
               int64_t rows, int64_t cols);
/* Same from i32 heights, keeping the low 8 bits as fut/interactive.fut:189
 * does (`elem & 0xFF`). */
int fs_map_new_i32(fs_ctx *ctx, fs_map **out, const int32_t *heights, const uint32_t *colors,
                   int64_t rows, int64_t cols);
/* Device-resident inputs: the colours are used in place (the caller keeps them
 * alive); the heights are read once to build the height quads. */
int fs_map_wrap_device(fs_ctx *ctx, fs_map **out, const uint8_t *heights_dev,
                       const uint32_t *colors_dev, int64_t rows, int64_t cols);
int fs_map_free(fs_ctx *ctx, fs_map *map);
int fs_map_shape(const fs_map *map, int64_t *rows, int64_t *cols);
/* Device height quads: [rows][cols] u32, bytes 0..3 = heights at (y,x),
 * (y,x+1), (y+1,x), (y+1,x+1) with wrapped indices. */
const uint32_t *fs_map_quads_dev(const fs_map *map);
const uint32_t *fs_map_colors_dev(const fs_map *map);

/* ---- depth schedule ------------------------------------------------------- */
/* Number of depth samples get_zs yields for draw distance D
 * (fut/voxel_renderer.fut:28-34). */
int32_t fs_num_depths(float distance, const fs_params *params);

/* ---- plain per-frame render ---------------------------------------------- */
/* Renders one [height][width] ARGB frame into device memory `out_dev`
 * (row-major, pitch = width), asynchronously on the context stream. */
int fs_render_device(fs_ctx *ctx, const fs_map *map, const fs_camera *cam,
                     const fs_params *params, int32_t width, int32_t height,
                     uint32_t *out_dev);
/* Same into HOST memory `out_host`: renders, copies the frame back and waits. */
int fs_render(fs_ctx *ctx, const fs_map *map, const fs_camera *cam, const fs_params *params,
              int32_t width, int32_t height, uint32_t *out_host);
/* Allocation-free variant of fs_render_device (no counterpart in the
 * reference). For callers that cannot let a library call cudaMalloc -- hosts
 * that own all device memory through their own pool, or per-frame loops that
 * cannot take the device synchronisation an allocation may cause: it calls no
 * allocating routine. Its one scratch buffer, the per-depth view-line table, is
 * a fixed 1.25 MiB array compiled into the library (held on every GPU that
 * loads the library until exit), so a frame may use at most 65536 depth
 * samples; longer schedules fail with FS_ERR_ARG. All calls share that array:
 * calls that overlap on the GPU race. The array's device address is looked up
 * once, by fs_ctx_new (which may load the library's module onto the device and
 * so allocate the array there), so the render calls themselves do no set-up. */
int fs_render_device_noalloc(fs_ctx *ctx, const fs_map *map, const fs_camera *cam,
                             const fs_params *params, int32_t width, int32_t height,
                             uint32_t *out_dev);

/* ---- batched multi-view render -------------------------------------------
 * A plan fixes the views' screen sizes and draw distances, owns a device
 * framebuffer arena with one frame per view, and renders every view with one
 * persistent kernel that pulls (view, column-tile) items from a device queue.
 * The launch sequence is captured once into a CUDA graph and replayed. */
int fs_plan_new(fs_ctx *ctx, fs_plan **out, const fs_map *const *maps, int32_t nmaps,
                const fs_params *params, const fs_view *views, int32_t nviews);
void fs_plan_free(fs_plan *plan);
/* Replaces the cameras (same count; draw distances must not raise any view's
 * depth count above the one the plan was built with). */
int fs_plan_set_cameras(fs_plan *plan, const fs_camera *cams, int32_t ncams);
/* Enqueues one render of every view on the context stream. */
int fs_plan_run(fs_plan *plan);
/* Device time in ms of the persistent render kernel alone in the most recent
 * fs_plan_run (events recorded inside the graph around that kernel); waits
 * for that run to finish. */
int fs_plan_kernel_ms(fs_plan *plan, float *ms);
/* Renders with one plain launch pair per view instead (the comparison loop). */
int fs_plan_run_per_view(fs_plan *plan);
uint32_t *fs_plan_frame_dev(fs_plan *plan, int32_t view);
int64_t fs_plan_frame_offset(const fs_plan *plan, int32_t view); /* in pixels */
int64_t fs_plan_total_pixels(const fs_plan *plan);
/* Copies every frame to `host` (fs_plan_total_pixels u32 values, frames laid
 * out at fs_plan_frame_offset) and waits. */
int fs_plan_download(fs_plan *plan, uint32_t *host);
/* Renders every view and writes every frame to `host` (the fs_plan_download
 * layout), with the views split into `groups` contiguous groups of about equal
 * pixel count (1..16): group g+1 renders while group g's frames are copied, so
 * with pinned host memory the copy time mostly hides the render time. A small
 * kernel after each group's render finds, per view, the leading rows that hold
 * nothing but the sky value; only the rows below them are copied, and the
 * calling thread's OpenMP team writes the sky rows into `host` meanwhile (the
 * same pixels as a full copy). A team of fewer than 4 threads (e.g.
 * OMP_NUM_THREADS=1) gets whole frames copied instead. Waits for the copies. */
int fs_plan_run_download(fs_plan *plan, uint32_t *host, int32_t groups);
/* Bytes of the last fs_plan_run_download: copied device to host (frame rows
 * and the per-view sky row counts) and written on the host (sky rows). */
int fs_plan_download_bytes(const fs_plan *plan, int64_t *copied, int64_t *filled);
/* Kernel configuration the plan uses (see fs_ctx_force_tune); out5[4] is the
 * persistent grid size actually launched. */
int fs_plan_get_tune(const fs_plan *plan, int32_t out5[5]);
int fs_plan_set_tune(fs_plan *plan, const int32_t tune5[5]);
/* Order-independent hash of the plan's resolution multiset (tuning-cache key). */
int fs_plan_signature(const fs_plan *plan, int64_t *sig);

/* ---- autotuner -------------------------------------------------------------
 * Times every compiled (tile width, lanes per column, depth samples per lane)
 * configuration that fits in shared memory and caches the fastest per
 * (resolution, map size, filters) -- or per batch resolution multiset -- in the
 * text file $FS_TUNE_CACHE (default ./.futspace_tune.txt). */
int fs_autotune_frame(fs_ctx *ctx, const fs_map *map, const fs_camera *cam,
                      const fs_params *params, int32_t width, int32_t height, int32_t reps,
                      int32_t out5[5], float *best_ms);
int fs_plan_autotune(fs_plan *plan, int32_t reps, int32_t out5[5], float *best_ms);
/* Number of compiled configurations and the i-th one as {tw, lc, u, stage, 0}. */
int fs_tune_count(void);
int fs_tune_get(int i, int32_t out5[5]);

/* Work counters of the render kernel: when enabled, every following launch adds
 * the depth samples it evaluated and the occlusion events it coloured (when
 * disabled, the kernels skip the counting). Reading (out2 != NULL) waits for
 * the stream and resets the counters. A plan recaptures its graph at its next
 * run after the setting changes. */
int fs_ctx_stats(fs_ctx *ctx, int32_t enable, uint64_t out2[2]);

/* Roofline denominator: L2 read bandwidth in GB/s, from one kernel reading a
 * `bytes`-long device buffer (at least 1 MiB, small enough to stay in L2)
 * `reps` times with L2-only loads after a pass that brings it into L2; CUDA
 * events on the context stream around the timed launch. Allocates and frees
 * the buffer. */
int fs_measure_l2_read_gbs(fs_ctx *ctx, int64_t bytes, int32_t reps, float *gbs);

/* ---- serving: continuous batching of render requests -----------------------
 * A server keeps the maps and one view record per session resident on the
 * device. Requests arrive over time; each is admitted when its session has no
 * request in flight and its frame fits in the free part of a device
 * framebuffer arena of `budget_bytes`. Admitted requests are launched in
 * batches -- every admitted request that is ready when a launch slot frees up
 * -- through the same persistent kernel, with up to `slots` batches in flight
 * on separate streams, so new work overlaps work already on the GPU. A frame's
 * memory returns to the arena when its request completes. Pixels do not depend
 * on batching: a frame rendered alone equals the same frame rendered in a mix. */
typedef struct {
  int64_t budget_bytes; /* device framebuffer arena */
  int32_t nsessions;
  int32_t max_batch;    /* requests per launch */
  int32_t slots;        /* launches in flight */
  int32_t max_depths;   /* depth capacity per session (fs_num_depths of the largest distance) */
  int32_t tune[5];      /* kernel configuration {tw, lc, u, stage, ctas}; tile width 0 =
                         * default: each launch uses the cooperative tile when its
                         * tallest frame fits the tile's stage, else direct painting;
                         * stage 0 = direct painting only; stage 2 = that cooperative
                         * tile, direct painting for frames too tall for it */
} fs_server_config;

typedef struct {
  int32_t session, map;  /* session id in [0, nsessions); map index */
  int32_t width, height;
  fs_camera cam;
  uint32_t *host_out;    /* if not NULL the frame is copied here before completion */
  int64_t arrival_ns;    /* release time, relative to the start of fs_server_run */
  int64_t start_ns;      /* filled: launch time */
  int64_t done_ns;       /* filled: completion time (frame in device memory or host_out) */
  int32_t status;        /* filled: FS_OK or an error code */
  int32_t batch;         /* filled: index of the launch that rendered it */
} fs_request;

typedef struct {
  double wall_s, gpix_s;
  double p50_ms, p99_ms, mean_ms, max_ms; /* latency: arrival -> done */
  int64_t requests, pixels, batches;
  double mean_batch;
  int64_t peak_arena_bytes;
  int32_t max_inflight;
  int32_t errors;
  /* where the slowest moments of the run went (diagnostics): the longest
   * single CUDA runtime call of the loop and its FS_SERVE_SITE_*, the longest
   * idle sleep (2 us requested), the longest loop iteration without its calls
   * and sleeps (host time), and the longest launch on the GPU (from the event
   * before its first copy to its completion event) with its launch time */
  double max_call_ms;
  int32_t max_call_site;
  int32_t reserved;
  double max_sleep_ms;
  double max_host_ms;
  double max_batch_gpu_ms;
  int64_t max_batch_gpu_at_ns;
  int64_t max_host_at_ns;      /* when the longest host-only iteration started */
  int64_t involuntary_switches; /* of the loop's thread during the run (getrusage) */
  int64_t voluntary_switches;
} fs_serve_stats;
enum {
  FS_SERVE_SITE_EVENT_QUERY = 1,
  FS_SERVE_SITE_COPY_IN = 2,
  FS_SERVE_SITE_COUNTER_RESET = 3,
  FS_SERVE_SITE_PROLOGUE = 4,
  FS_SERVE_SITE_RENDER = 5,
  FS_SERVE_SITE_COPY_OUT = 6,
  FS_SERVE_SITE_EVENT_RECORD = 7
};

typedef struct fs_server fs_server;
int fs_server_new(fs_ctx *ctx, fs_server **out, const fs_map *const *maps, int32_t nmaps,
                  const fs_params *params, const fs_server_config *cfg);
void fs_server_free(fs_server *srv);
/* Runs the request loop until every request completes. realtime = 1 releases
 * each request at its arrival_ns (the loop paces itself on the host clock);
 * realtime = 0 releases all at once. Requests need not be sorted. */
int fs_server_run(fs_server *srv, fs_request *reqs, int32_t n, int32_t realtime,
                  fs_serve_stats *stats);

/* ---- synthetic inputs (seeded, identical on every host) -------------------- */
/* Toroidal diamond-square height map, rescaled to 0..255. size must be a power
 * of two. */
int fsgen_heights(uint64_t seed, int32_t size, float roughness, uint8_t *out);
/* 5-stop terrain palette indexed by height, plus uniform +-noise per channel,
 * alpha 0xFF. */
int fsgen_colors(uint64_t seed, const uint8_t *heights, int64_t count, int32_t noise,
                 uint32_t *out);
/* Maximum height in the 16x16 window centred on (x, y), wrapping. */
int32_t fsgen_local_max(const uint8_t *heights, int32_t rows, int32_t cols, float x, float y);
/* `count` cameras uniform on the map: yaw uniform in [0, 2pi), height in
 * [lo, hi] above the local maximum, horizon = screen_h / 2, fov 1.2. */
int fsgen_cameras(uint64_t seed, const uint8_t *heights, int32_t rows, int32_t cols,
                  int32_t count, float above_lo, float above_hi, float distance_lo,
                  float distance_hi, int32_t screen_h, fs_camera *out);
/* A random walk of `count` frames: each frame turns by U(-yaw, yaw), moves
 * `step` map units forward and keeps the height within [lo, hi] above the
 * local maximum. */
int fsgen_walk(uint64_t seed, const uint8_t *heights, int32_t rows, int32_t cols,
               int32_t count, float step, float yaw, float above_lo, float above_hi,
               float distance, int32_t screen_h, fs_camera *out);

/* ---- map ingest and frame output (host) ------------------------------------
 * PNG images as the reference's front end loads them through FreeImage
 * (c/freeimage_futspace.h:19-58): 8-bit greyscale, RGB, palette, grey+alpha
 * or RGBA, not interlaced, to 0xFF000000 | R << 16 | G << 8 | B words, rows top
 * to bottom. Writing produces an 8-bit RGB PNG (alpha dropped). The Futhark
 * binary data format is the one tools/png2data.py writes and
 * tools/data2png.py reads: 'b', version 2, rank, a 4-character element type
 * such as " i32", " u32" or "  u8", little-endian u64 dimensions, little-endian
 * elements. Buffers these calls return are released with fs_free. Status:
 * FS_OK, FS_ERR_ARG, FS_ERR_NOMEM or FS_ERR_IO. */
int fs_png_read(const char *path, uint32_t **argb, int64_t *rows, int64_t *cols);
int fs_png_decode(const uint8_t *png, size_t nbytes, uint32_t **argb, int64_t *rows,
                  int64_t *cols);
int fs_png_write(const char *path, const uint32_t *argb, int64_t rows, int64_t cols);
int fs_data_read(const char *path, void **data, char type[5], int32_t *rank, int64_t dims[8]);
int fs_data_write(const char *path, const void *data, const char *type, int32_t rank,
                  const int64_t *dims);
void fs_free(void *p);
/* A map from a colour PNG and a height PNG of the same size, as
 * c/interactive.c:43-56 loads data/converted-maps/C<n>W.png and D<n>.png:
 * heights are the low byte (blue channel) of each height-image word. */
int fs_map_load_png(fs_ctx *ctx, fs_map **out, const char *color_png, const char *height_png);

#ifdef __cplusplus
}
#endif
#endif
