/*
 * Autotuner for the render kernel's knobs -- column-tile width (TW), lanes per
 * column (LC: 32 = one warp per column, 16/8/4 = two/four/eight columns per
 * warp), depth samples per lane per chunk (U: chunk = LC*U depths) and the
 * form (direct painting, shared-memory stage + TMA store, or the cooperative
 * tile with LC threads per column and U depths per thread per block) -- plus
 * its cache. Each candidate that fits in shared memory is timed with CUDA
 * events on the context stream; the fastest is stored under a key made of the
 * screen resolution (or a batch's resolution multiset), the map size and the
 * filters. The cache is a text file, one "key tw lc u stage" line per entry, read at
 * context creation from $FS_TUNE_CACHE (default ./.futspace_tune.txt) and
 * rewritten after every tuning run.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fs_internal.h"
#include "fs_priv.h"

static const FsTune k_batch_order[] = {
    {64, 1, 4, 0, 0}, {64, 4, 4, 0, 0}, {32, 4, 4, 0, 0}, {8, 32, 1, 1, 0},
    {8, 32, 2, 1, 0}, {16, 32, 2, 1, 0}, {32, 32, 1, 1, 0}, {8, 32, 2, 0, 0},
};

FsTune fs_default_batch_tune(fs_ctx *ctx, int32_t stride_max) {
  for (size_t i = 0; i < sizeof(k_batch_order) / sizeof(k_batch_order[0]); i++)
    if (fs_tune_fits(ctx, &k_batch_order[i], stride_max)) return k_batch_order[i];
  FsTune none = {0, 0, 0, 0, 0};
  return none;
}

void fs_tune_cache_load(fs_ctx *ctx) {
  const char *path = getenv("FS_TUNE_CACHE");
  snprintf(ctx->tune_path, sizeof(ctx->tune_path), "%s",
           (path && path[0]) ? path : ".futspace_tune.txt");
  ctx->ntune = 0;
  FILE *f = fopen(ctx->tune_path, "r");
  if (!f) return;
  char key[96];
  int tw, lc, u, stg;
  while (ctx->ntune < FS_TUNE_CACHE_MAX &&
         fscanf(f, "%95s %d %d %d %d", key, &tw, &lc, &u, &stg) == 5) {
    FsTune t = {tw, lc, u, stg, 0};
    if (!fsk_tune_supported(&t)) continue;
    fs_tune_entry *e = &ctx->tunes[ctx->ntune++];
    snprintf(e->key, sizeof(e->key), "%s", key);
    e->tune = t;
  }
  fclose(f);
}

static void fs_tune_cache_save(fs_ctx *ctx) {
  FILE *f = fopen(ctx->tune_path, "w");
  if (!f) return;
  for (int i = 0; i < ctx->ntune; i++)
    fprintf(f, "%s %d %d %d %d\n", ctx->tunes[i].key, ctx->tunes[i].tune.tw,
            ctx->tunes[i].tune.lc, ctx->tunes[i].tune.u, ctx->tunes[i].tune.stage);
  fclose(f);
}

static void fs_tune_store(fs_ctx *ctx, const char *key, const FsTune *t) {
  for (int i = 0; i < ctx->ntune; i++)
    if (!strcmp(ctx->tunes[i].key, key)) {
      ctx->tunes[i].tune = *t;
      fs_tune_cache_save(ctx);
      return;
    }
  if (ctx->ntune < FS_TUNE_CACHE_MAX) {
    fs_tune_entry *e = &ctx->tunes[ctx->ntune++];
    snprintf(e->key, sizeof(e->key), "%s", key);
    e->tune = *t;
  }
  fs_tune_cache_save(ctx);
}

int fs_tune_lookup_key(fs_ctx *ctx, const char *key, FsTune *out) {
  for (int i = 0; i < ctx->ntune; i++)
    if (!strcmp(ctx->tunes[i].key, key)) {
      *out = ctx->tunes[i].tune;
      return 1;
    }
  return 0;
}

static void frame_key(char *key, size_t cap, int32_t W, int32_t H, int32_t MH, int32_t MW,
                      int32_t flags) {
  snprintf(key, cap, "frame:%dx%d:map%dx%d:f%d", W, H, MH, MW, flags);
}

int fs_tune_lookup(fs_ctx *ctx, int32_t W, int32_t H, int32_t MH, int32_t MW, int32_t flags,
                   FsTune *out) {
  char key[96];
  frame_key(key, sizeof(key), W, H, MH, MW, flags);
  return fs_tune_lookup_key(ctx, key, out);
}

static int time_ms(fs_ctx *ctx, float *ms, int (*fn)(void *), void *arg, int reps) {
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) || cudaEventCreate(&b)) return fs_fail(ctx, FS_ERR_CUDA, "events");
  int rc = fn(arg); /* warm-up */
  if (!rc) rc = fn(arg);
  if (!rc) {
    cudaEventRecord(a, ctx->stream);
    for (int i = 0; i < reps && !rc; i++) rc = fn(arg);
    cudaEventRecord(b, ctx->stream);
    int e = cudaEventSynchronize(b);
    if (e) rc = fs_cuda_fail(ctx, e, "tuning run");
    else cudaEventElapsedTime(ms, a, b);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!rc) *ms /= (float)reps;
  return rc;
}

typedef struct {
  fs_ctx *ctx;
  const fs_map *map;
  FsView view;
  FsTune tune;
} frame_job;

static int frame_once(void *arg) {
  frame_job *j = (frame_job *)arg;
  FsView v = j->view;
  return fs_render_view(j->ctx, &j->map->dev, &v, &j->tune, j->ctx->zline, j->ctx->zinvz, NULL,
                        1);
}

/* Times every fitting configuration on one frame and caches the fastest for
 * (W, H, map size, filters). out5 = {tw, lc, u, stage, 0}; *best_ms its time. */
int fs_autotune_frame(fs_ctx *ctx, const fs_map *map, const fs_camera *cam,
                      const fs_params *params, int32_t width, int32_t height, int32_t reps,
                      int32_t out5[5], float *best_ms) {
  if (!ctx || !map || !cam || !out5) return FS_ERR_ARG;
  fs_params dp = fs_params_default();
  if (!params) params = &dp;
  cudaSetDevice(ctx->device);
  frame_job j;
  j.ctx = ctx;
  j.map = map;
  int rc = fs_make_view(ctx, cam, params, width, height, 0, &j.view);
  if (rc) return rc;
  rc = fs_ensure_ztable(ctx, j.view.n);
  if (rc) return rc;
  uint32_t *frame = NULL;
  if (cudaMalloc((void **)&frame, (size_t)width * height * 4) != cudaSuccess)
    return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(tuning frame)");
  j.view.out = frame;
  if (reps < 1) reps = 5;
  float best = 1e30f;
  FsTune bt = {0, 0, 0, 0, 0};
  for (int i = 0; i < fs_tune_count(); i++) {
    int32_t t5[5];
    fs_tune_get(i, t5);
    FsTune t = {t5[0], t5[1], t5[2], t5[3], 0, (j.view.flags & FSV_SMOOTH) ? 1 : 0,
                (j.view.flags & (FSV_SHADE | FSV_FOG)) ? 1 : 0};
    if (!fs_tune_fits(ctx, &t, height | 1)) continue;
    j.tune = t;
    float ms = 0.0f;
    rc = time_ms(ctx, &ms, frame_once, &j, reps);
    if (rc) break;
    if (ms < best) {
      best = ms;
      bt = t;
    }
  }
  cudaStreamSynchronize(ctx->stream);
  cudaFree(frame);
  if (rc) return rc;
  if (!bt.tw) return fs_fail(ctx, FS_ERR_ARG, "no configuration fits");
  char key[96];
  frame_key(key, sizeof(key), width, height, map->dev.MH, map->dev.MW, j.view.flags);
  fs_tune_store(ctx, key, &bt);
  out5[0] = bt.tw;
  out5[1] = bt.lc;
  out5[2] = bt.u;
  out5[3] = bt.stage;
  out5[4] = 0;
  if (best_ms) *best_ms = best;
  return FS_OK;
}

static int plan_once(void *arg) { return fs_plan_run((fs_plan *)arg); }

/* Times every fitting configuration on a whole batch and caches the fastest
 * under the batch's resolution signature and map size. */
int fs_plan_autotune(fs_plan *p, int32_t reps, int32_t out5[5], float *best_ms) {
  if (!p || !out5) return FS_ERR_ARG;
  fs_ctx *ctx = p->ctx;
  if (reps < 1) reps = 3;
  float best = 1e30f;
  int32_t bt[5] = {0, 0, 0, 0, 0};
  int rc = FS_OK;
  for (int i = 0; i < fs_tune_count(); i++) {
    int32_t t5[5];
    fs_tune_get(i, t5);
    FsTune t = {t5[0], t5[1], t5[2], t5[3], 0, (p->fv_h[0].flags & FSV_SMOOTH) ? 1 : 0,
                (p->fv_h[0].flags & (FSV_SHADE | FSV_FOG)) ? 1 : 0};
    if (!fs_tune_fits(ctx, &t, p->stride_max) || !fs_coop_depths_ok(&t, fs_plan_max_depths(p)))
      continue;
    rc = fs_plan_set_tune(p, t5);
    if (rc) break;
    float ms = 0.0f;
    rc = time_ms(ctx, &ms, plan_once, p, reps);
    if (rc) break;
    if (ms < best) {
      best = ms;
      memcpy(bt, t5, sizeof(bt));
    }
  }
  if (rc) return rc;
  if (!bt[0]) return fs_fail(ctx, FS_ERR_ARG, "no configuration fits");
  rc = fs_plan_set_tune(p, bt);
  if (rc) return rc;
  int64_t sig = 0;
  fs_plan_signature(p, &sig);
  char key[96];
  snprintf(key, sizeof(key), "batch:%016llx:map%dx%d:f%d", (unsigned long long)sig,
           p->maps[0].MH, p->maps[0].MW, p->hf | (p->cf << 1));
  FsTune t = {bt[0], bt[1], bt[2], bt[3], 0, 0};
  fs_tune_store(ctx, key, &t);
  memcpy(out5, bt, sizeof(bt));
  out5[4] = p->grid;
  if (best_ms) *best_ms = best;
  return FS_OK;
}
