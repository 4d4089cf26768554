/*
 * Serving: a request loop with continuous batching over the persistent render
 * kernel.
 *
 *  - Maps and a view record per session live on the device. The render kernel
 *    reads views through the session table: a work item names (session, tile).
 *  - Admission: a released request is admitted when its session has no request
 *    in flight and its frame fits in the free part of the framebuffer arena
 *    (first fit, 256-byte blocks, coalescing free list). A request larger than
 *    the whole arena fails with FS_ERR_BUDGET.
 *  - Launch: whenever a slot (stream) is free, every admitted request that is
 *    ready (up to max_batch) goes into one launch: one host->device copy of the
 *    packed view records, session ids and work items; a prepare kernel that
 *    writes the records into the session table and builds their depth tables;
 *    the persistent render kernel; optional frame downloads. Up to `slots`
 *    launches are in flight, so arrivals during a launch start on the GPU
 *    before it finishes.
 *  - Completion: the loop polls the slots' events; a finished request frees its
 *    frame memory and its session.
 */
#ifndef _GNU_SOURCE
#define _GNU_SOURCE
#endif
#include <stdlib.h>
#include <string.h>
#include <sys/resource.h>
#include <time.h>

#include "fs_internal.h"
#include "fs_priv.h"

typedef struct {
  int64_t off, len;
} fs_blk;

typedef struct {
  int64_t size, used, peak;
  fs_blk *free;
  int32_t nfree, cap;
} fs_arena;

static int arena_init(fs_arena *a, int64_t size) {
  memset(a, 0, sizeof(*a));
  a->cap = 64;
  a->free = (fs_blk *)malloc(sizeof(fs_blk) * (size_t)a->cap);
  if (!a->free) return 0;
  a->size = size;
  a->free[0].off = 0;
  a->free[0].len = size;
  a->nfree = 1;
  return 1;
}

static int64_t round256(int64_t v) { return (v + 255) & ~(int64_t)255; }

/* first fit; returns the offset or -1 */
static int64_t arena_alloc(fs_arena *a, int64_t len) {
  len = round256(len);
  for (int32_t i = 0; i < a->nfree; i++) {
    if (a->free[i].len >= len) {
      const int64_t off = a->free[i].off;
      a->free[i].off += len;
      a->free[i].len -= len;
      if (a->free[i].len == 0) {
        memmove(&a->free[i], &a->free[i + 1], sizeof(fs_blk) * (size_t)(a->nfree - i - 1));
        a->nfree--;
      }
      a->used += len;
      if (a->used > a->peak) a->peak = a->used;
      return off;
    }
  }
  return -1;
}

static int arena_free(fs_arena *a, int64_t off, int64_t len) {
  len = round256(len);
  int32_t i = 0;
  while (i < a->nfree && a->free[i].off < off) i++;
  if (a->nfree == a->cap) {
    fs_blk *nb = (fs_blk *)realloc(a->free, sizeof(fs_blk) * (size_t)a->cap * 2);
    if (!nb) return 0;
    a->free = nb;
    a->cap *= 2;
  }
  memmove(&a->free[i + 1], &a->free[i], sizeof(fs_blk) * (size_t)(a->nfree - i));
  a->free[i].off = off;
  a->free[i].len = len;
  a->nfree++;
  a->used -= len;
  /* coalesce with the right and the left neighbour */
  if (i + 1 < a->nfree && a->free[i].off + a->free[i].len == a->free[i + 1].off) {
    a->free[i].len += a->free[i + 1].len;
    memmove(&a->free[i + 1], &a->free[i + 2], sizeof(fs_blk) * (size_t)(a->nfree - i - 2));
    a->nfree--;
  }
  if (i > 0 && a->free[i - 1].off + a->free[i - 1].len == a->free[i].off) {
    a->free[i - 1].len += a->free[i].len;
    memmove(&a->free[i], &a->free[i + 1], sizeof(fs_blk) * (size_t)(a->nfree - i - 1));
    a->nfree--;
  }
  return 1;
}

typedef struct {
  cudaStream_t st;
  cudaEvent_t ev0; /* recorded before the launch's first copy */
  cudaEvent_t ev;  /* after its last operation */
  int32_t busy;
  int32_t nreq;
  int32_t *req;    /* request indices of the launch */
  uint8_t *pinned; /* [FsView x max_batch][int32 ids x max_batch, padded to 8 bytes]
                      [int64 items x max_items] */
  uint8_t *dev;    /* same layout on the device */
  int32_t *head_d;
  int64_t launch_ns; /* when the current launch was enqueued (run clock) */
} fs_slot;

struct fs_server {
  fs_ctx *ctx;
  int32_t nmaps;
  FsMapDev maps[FS_MAX_MAPS];
  fs_params params;
  fs_server_config cfg;
  FsTune tune;      /* direct painting */
  FsTune tune_coop; /* the cooperative tile, when use_coop */
  int32_t use_coop;
  int32_t hf, cf, grid, max_items;
  int32_t iw;      /* screen columns per work item, direct painting */
  int32_t iw_coop; /* and the cooperative tile */
  /* cooperative-tile CTAs per SM by frame height in 32-row steps (0: not
   * queried yet, -1: the stage does not fit) */
  int16_t coop_occ[FS_MAX_ROWS / 32 + 2];
  uint8_t *arena_base;
  fs_arena arena;
  FsView *sess_d;
  float4 *zline;
  float *zinvz;
  int8_t *sess_busy;
  fs_slot *slots;
  int64_t iter_call_ns; /* CUDA call time within the current loop iteration */
};

static int64_t now_ns(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (int64_t)t.tv_sec * 1000000000LL + t.tv_nsec;
}

/* Diagnostics: a CUDA call of the loop took dt_ns at `site`. */
static void note_call(fs_server *s, fs_serve_stats *st, int32_t site, int64_t dt_ns) {
  s->iter_call_ns += dt_ns;
  const double ms = (double)dt_ns * 1e-6;
  if (ms > st->max_call_ms) {
    st->max_call_ms = ms;
    st->max_call_site = site;
  }
}

void fs_server_free(fs_server *s) {
  if (!s) return;
  cudaSetDevice(s->ctx->device);
  if (s->slots) {
    for (int i = 0; i < s->cfg.slots; i++) {
      fs_slot *sl = &s->slots[i];
      if (sl->st) cudaStreamSynchronize(sl->st);
      if (sl->ev) cudaEventDestroy(sl->ev);
      if (sl->ev0) cudaEventDestroy(sl->ev0);
      if (sl->st) cudaStreamDestroy(sl->st);
      cudaFreeHost(sl->pinned);
      cudaFree(sl->dev);
      cudaFree(sl->head_d);
      free(sl->req);
    }
    free(s->slots);
  }
  cudaFree(s->arena_base);
  cudaFree(s->sess_d);
  cudaFree(s->zline);
  cudaFree(s->zinvz);
  free(s->arena.free);
  free(s->sess_busy);
  free(s);
}

/* Byte offset of the work items in a slot buffer (8-byte aligned). */
static size_t items_offset(const fs_server *s) {
  return (sizeof(FsView) * (size_t)s->cfg.max_batch + 4 * (size_t)s->cfg.max_batch + 7) & ~(size_t)7;
}

static size_t slot_bytes(const fs_server *s) {
  return items_offset(s) + 8 * (size_t)s->max_items;
}

int fs_server_new(fs_ctx *ctx, fs_server **out, const fs_map *const *maps, int32_t nmaps,
                  const fs_params *params, const fs_server_config *cfg) {
  if (!ctx || !out || !cfg) return FS_ERR_ARG;
  *out = NULL;
  if (ctx->broken) return fs_fail(ctx, FS_ERR_STATE, "context failed to initialise");
  if (!maps || nmaps < 1 || nmaps > FS_MAX_MAPS)
    return fs_fail(ctx, FS_ERR_ARG, "need 1..%d maps", FS_MAX_MAPS);
  if (cfg->nsessions < 1 || cfg->nsessions >= FS_ITEM_VIEWS || cfg->max_batch < 1 ||
      cfg->slots < 1 || cfg->slots > 16 || cfg->max_depths < 1 ||
      cfg->max_depths >= FS_MAX_DEPTHS || cfg->budget_bytes < 256)
    return fs_fail(ctx, FS_ERR_ARG, "bad server configuration");
  fs_params dp = fs_params_default();
  if (!params) params = &dp;
  int rc = fs_check_params(ctx, params);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  fs_server *s = (fs_server *)calloc(1, sizeof(fs_server));
  if (!s) return fs_fail(ctx, FS_ERR_NOMEM, "calloc(server)");
  s->ctx = ctx;
  s->cfg = *cfg;
  s->params = *params;
  s->nmaps = nmaps;
  for (int i = 0; i < nmaps; i++) {
    if (!maps[i]) {
      fs_server_free(s);
      return fs_fail(ctx, FS_ERR_ARG, "map %d is NULL", i);
    }
    s->maps[i] = maps[i]->dev;
    if (ctx->no_skip) s->maps[i].pyr = NULL;
  }
  s->hf = params->height_filter == FS_BILINEAR;
  s->cf = params->color_filter == FS_BILINEAR;
  /* Two forms, chosen per launch: the cooperative tile (CTA tiles, frames
   * stored from shared memory with plain stores, no tensor maps) for every
   * launch whose tallest frame fits its stage, else direct painting. Serving
   * batches are small, and few strips leave direct painting latency-bound. An
   * explicit tuning names one form: stage 0 direct only; stage 2 the
   * cooperative tile, with direct painting for frames too tall for it. */
  FsTune t = {cfg->tune[0], cfg->tune[1], cfg->tune[2], cfg->tune[3], cfg->tune[4]};
  FsTune c = {0, 0, 0, 0, 0};
  const FsTune def = {128, 1, 4, 0, 0};
  const FsTune def_coop = {8, 64, 8, 2, 0};
  if (!t.tw) {
    t = def;
    c = def_coop;
  } else if (t.stage == 2) {
    c = t;
    t = def;
  }
  {
    /* the mode (smoothing, epilogue) follows the parameters; an explicit
     * tuning must have a kernel compiled for it */
    const int32_t flags = (params->smoothing ? FSV_SMOOTH : 0) |
                          ((params->effects & FS_FX_SHADE) ? FSV_SHADE : 0) |
                          ((params->effects & FS_FX_FOG) ? FSV_FOG : 0);
    if (cfg->tune[0] && cfg->tune[3] == 0) {
      t.smooth = (flags & FSV_SMOOTH) ? 1 : 0;
      t.fx = (flags & (FSV_SHADE | FSV_FOG)) ? 1 : 0;
    } else {
      t = fs_tune_for_mode(t, flags);
    }
    c.smooth = (flags & FSV_SMOOTH) ? 1 : 0;
    c.fx = (flags & (FSV_SHADE | FSV_FOG)) ? 1 : 0;
  }
  if (t.stage != 0 || !fsk_tune_supported(&t)) {
    fs_server_free(s);
    return fs_fail(ctx, FS_ERR_ARG, "serving needs a compiled direct-paint configuration");
  }
  s->use_coop = c.tw && fsk_tune_supported(&c) && fs_coop_depths_ok(&c, cfg->max_depths);
  if (cfg->tune[0] && cfg->tune[3] == 2 && !s->use_coop) {
    fs_server_free(s);
    return fs_fail(ctx, FS_ERR_ARG, "no cooperative tile compiled for this mode");
  }
  s->tune = t;
  s->iw = fsk_item_width(&t);
  s->tune_coop = c;
  s->iw_coop = s->use_coop ? fsk_item_width(&c) : s->iw;
  {
    const int32_t iw_min = s->iw < s->iw_coop ? s->iw : s->iw_coop;
    s->max_items = cfg->max_batch * ((65536 + iw_min - 1) / iw_min);
  }
  if (s->use_coop) {
    /* raise the kernel's shared-memory limit once, for the tallest frame
     * whose stage fits, so no launch changes a function attribute */
    int32_t rows = (FS_MAX_ROWS + 31) / 32 * 32;
    while (rows > 32 && fsk_render_smem(&c, rows - 1) > ctx->smem_optin) rows -= 32;
    int32_t occ = 0;
    if (fsk_render_smem(&c, rows - 1) <= ctx->smem_optin)
      fsk_render_max_ctas_per_sm(&c, s->hf, s->cf, rows - 1, &occ);
  }
  int32_t occ = 0;
  int e = fsk_render_max_ctas_per_sm(&t, s->hf, s->cf, 1, &occ);
  if (e || occ < 1) {
    fs_server_free(s);
    return e ? fs_cuda_fail(ctx, e, "occupancy query") : fs_fail(ctx, FS_ERR_ARG, "no fit");
  }
  s->grid = occ * ctx->sm_count;
  if (t.ctas > 0 && t.ctas < s->grid) s->grid = t.ctas;
  const size_t zcnt = (size_t)cfg->nsessions * ((size_t)cfg->max_depths + FS_ZPAD);
  s->sess_busy = (int8_t *)calloc((size_t)cfg->nsessions, 1);
  s->slots = (fs_slot *)calloc((size_t)cfg->slots, sizeof(fs_slot));
  if (!s->sess_busy || !s->slots || !arena_init(&s->arena, cfg->budget_bytes) ||
      cudaMalloc((void **)&s->arena_base, (size_t)cfg->budget_bytes) != cudaSuccess ||
      cudaMalloc((void **)&s->sess_d, sizeof(FsView) * (size_t)cfg->nsessions) != cudaSuccess ||
      cudaMalloc((void **)&s->zline, sizeof(float4) * zcnt) != cudaSuccess ||
      cudaMalloc((void **)&s->zinvz, sizeof(float) * zcnt) != cudaSuccess) {
    fs_server_free(s);
    return fs_fail(ctx, FS_ERR_NOMEM, "server allocation (budget %lld bytes)",
                   (long long)cfg->budget_bytes);
  }
  for (int i = 0; i < cfg->slots; i++) {
    fs_slot *sl = &s->slots[i];
    sl->req = (int32_t *)malloc(sizeof(int32_t) * (size_t)cfg->max_batch);
    if (!sl->req || cudaStreamCreateWithFlags(&sl->st, cudaStreamNonBlocking) ||
        cudaEventCreate(&sl->ev) || cudaEventCreate(&sl->ev0) ||
        cudaMallocHost((void **)&sl->pinned, slot_bytes(s)) ||
        cudaMalloc((void **)&sl->dev, slot_bytes(s)) ||
        cudaMalloc((void **)&sl->head_d, sizeof(int32_t))) {
      fs_server_free(s);
      return fs_fail(ctx, FS_ERR_NOMEM, "server slot allocation");
    }
  }
  *out = s;
  return FS_OK;
}

typedef struct {
  int64_t cost;
  int64_t item;
} srv_item;

static int cmp_item(const void *a, const void *b) {
  const srv_item *x = (const srv_item *)a, *y = (const srv_item *)b;
  if (x->cost != y->cost) return x->cost > y->cost ? -1 : 1;
  return (x->item > y->item) - (x->item < y->item);
}

typedef struct {
  int32_t *q;
  int32_t head, tail, cap; /* ring of request indices */
} fs_fifo;

static void fifo_push(fs_fifo *f, int32_t v) {
  f->q[f->tail % f->cap] = v;
  f->tail++;
}

static int64_t req_frame_bytes(const fs_request *r) {
  return (int64_t)r->width * (int64_t)r->height * 4;
}

/* Builds and enqueues one launch on a free slot from the ready requests. */
static int launch_batch(fs_server *s, fs_slot *sl, fs_request *reqs, fs_fifo *ready,
                        int64_t *frame_off, srv_item *scratch, int64_t t0, int32_t batch_id,
                        int32_t *completed, fs_serve_stats *st) {
  fs_ctx *ctx = s->ctx;
  const int32_t mb = s->cfg.max_batch;
  FsView *packed = (FsView *)sl->pinned;
  int32_t *ids = (int32_t *)(sl->pinned + sizeof(FsView) * (size_t)mb);
  int64_t *items = (int64_t *)(sl->pinned + items_offset(s));
  int32_t nb = 0, ni = 0, hmax = 0;
  const int32_t iw_min = s->iw < s->iw_coop ? s->iw : s->iw_coop;
  sl->nreq = 0;
  while (ready->head < ready->tail && nb < mb) {
    const int32_t ri = ready->q[ready->head % ready->cap];
    fs_request *r = &reqs[ri];
    const int32_t tiles = (r->width + iw_min - 1) / iw_min;
    if (ni + tiles > s->max_items) break;
    ready->head++;
    FsView v;
    int rc = fs_make_view(ctx, &r->cam, &s->params, r->width, r->height, r->map, &v);
    if (!rc && v.n > s->cfg.max_depths)
      rc = fs_fail(ctx, FS_ERR_ARG, "request depth count %d exceeds max_depths %d", v.n,
                   s->cfg.max_depths);
    if (rc) {
      r->status = rc;
      r->done_ns = now_ns() - t0;
      arena_free(&s->arena, frame_off[ri], req_frame_bytes(r));
      s->sess_busy[r->session] = 0;
      (*completed)++;
      st->errors++;
      continue;
    }
    v.zoff = (int64_t)r->session * ((int64_t)s->cfg.max_depths + FS_ZPAD);
    v.out = (uint32_t *)(s->arena_base + frame_off[ri]);
    v.tmap = -1;
    packed[nb] = v;
    ids[nb] = r->session;
    ni += tiles; /* capacity at the narrower item width */
    if (v.H > hmax) hmax = v.H;
    sl->req[nb] = ri;
    r->batch = batch_id;
    r->start_ns = now_ns() - t0;
    nb++;
  }
  if (nb == 0) return FS_OK;
  /* the form of this launch: the cooperative tile if the tallest frame's
   * stage fits in shared memory */
  const FsTune *tune = &s->tune;
  int32_t iw = s->iw, grid_max = s->grid, stride = 1;
  if (s->use_coop) {
    const int32_t cls = (hmax | 1) / 32; /* stages of one class round to the same rows */
    if (!s->coop_occ[cls]) {
      const int32_t st_rows = cls * 32 + 31; /* the class's tallest stride */
      int32_t occ = 0;
      if (fsk_render_smem(&s->tune_coop, st_rows) > ctx->smem_optin ||
          fsk_render_max_ctas_per_sm(&s->tune_coop, s->hf, s->cf, st_rows, &occ) || occ < 1)
        occ = -1;
      s->coop_occ[cls] = (int16_t)occ;
    }
    if (s->coop_occ[cls] > 0) {
      tune = &s->tune_coop;
      iw = s->iw_coop;
      grid_max = s->coop_occ[cls] * ctx->sm_count;
      stride = cls * 32 + 31;
    }
  }
  ni = 0;
  for (int32_t b = 0; b < nb; b++) {
    const int32_t tiles = (packed[b].W + iw - 1) / iw;
    for (int32_t t = 0; t < tiles; t++) {
      scratch[ni].cost = (int64_t)packed[b].n * 8 + packed[b].H;
      scratch[ni].item = FS_ITEM(ids[b], 0, t);
      ni++;
    }
  }
  qsort(scratch, (size_t)ni, sizeof(srv_item), cmp_item);
  for (int32_t i = 0; i < ni; i++) items[i] = scratch[i].item;
  sl->nreq = nb;
  const size_t used = items_offset(s) + 8 * (size_t)ni;
  int64_t tc = now_ns();
  int e = cudaEventRecord(sl->ev0, sl->st);
  if (!e) e = cudaMemcpyAsync(sl->dev, sl->pinned, used, cudaMemcpyHostToDevice, sl->st);
  note_call(s, st, FS_SERVE_SITE_COPY_IN, now_ns() - tc);
  const FsView *packed_d = (const FsView *)sl->dev;
  const int32_t *ids_d = (const int32_t *)(sl->dev + sizeof(FsView) * (size_t)mb);
  const int64_t *items_d = (const int64_t *)(sl->dev + items_offset(s));
  int32_t max_n = 0;
  for (int32_t i = 0; i < nb; i++)
    if (packed[i].n > max_n) max_n = packed[i].n;
  /* the work counter is reset before the prologue kernel, so the render
   * kernel (a programmatic dependent launch) follows that kernel directly */
  tc = now_ns();
  if (!e) e = cudaMemsetAsync(sl->head_d, 0, sizeof(int32_t), sl->st);
  note_call(s, st, FS_SERVE_SITE_COUNTER_RESET, now_ns() - tc);
  tc = now_ns();
  if (!e) e = fsk_serve_prepare(packed_d, ids_d, nb, max_n, s->sess_d, s->zline, s->zinvz, sl->st);
  note_call(s, st, FS_SERVE_SITE_PROLOGUE, now_ns() - tc);
  if (!e) {
    FsLaunch L;
    memset(&L, 0, sizeof(L));
    for (int i = 0; i < s->nmaps; i++) L.maps[i] = s->maps[i];
    L.views = s->sess_d;
    L.items = items_d;
    L.zline = s->zline;
    L.zinvz = s->zinvz;
    L.head = sl->head_d;
    L.stats = ctx->collect_stats ? ctx->stats_dev : NULL;
    L.nitems = ni;
    L.stride_max = stride;
    const int32_t per_cta = fsk_items_per_cta(tune);
    const int32_t need = (ni + per_cta - 1) / per_cta;
    const int32_t grid = need < grid_max ? need : grid_max;
    tc = now_ns();
    e = fsk_render_pdl(&L, tune, s->hf, s->cf, grid, sl->st);
    note_call(s, st, FS_SERVE_SITE_RENDER, now_ns() - tc);
    ctx->launches += 2;
  }
  for (int32_t i = 0; i < nb && !e; i++) {
    const fs_request *r = &reqs[sl->req[i]];
    if (r->host_out) {
      tc = now_ns();
      e = cudaMemcpyAsync(r->host_out, s->arena_base + frame_off[sl->req[i]],
                          (size_t)req_frame_bytes(r), cudaMemcpyDeviceToHost, sl->st);
      note_call(s, st, FS_SERVE_SITE_COPY_OUT, now_ns() - tc);
    }
  }
  tc = now_ns();
  if (!e) e = cudaEventRecord(sl->ev, sl->st);
  note_call(s, st, FS_SERVE_SITE_EVENT_RECORD, now_ns() - tc);
  if (e) return fs_cuda_fail(ctx, e, "serving launch");
  sl->busy = 1;
  sl->launch_ns = now_ns() - t0;
  st->batches++;
  st->mean_batch += nb;
  return FS_OK;
}

static int cmp_arrival(const void *a, const void *b, void *arg) {
  const fs_request *r = (const fs_request *)arg;
  const int32_t i = *(const int32_t *)a, j = *(const int32_t *)b;
  if (r[i].arrival_ns != r[j].arrival_ns) return r[i].arrival_ns < r[j].arrival_ns ? -1 : 1;
  return i - j;
}

static int cmp_double(const void *a, const void *b) {
  const double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : (x > y);
}

int fs_server_run(fs_server *s, fs_request *reqs, int32_t n, int32_t realtime,
                  fs_serve_stats *stats) {
  if (!s || (!reqs && n > 0)) return FS_ERR_ARG;
  fs_ctx *ctx = s->ctx;
  cudaSetDevice(ctx->device);
  fs_serve_stats st;
  memset(&st, 0, sizeof(st));
  for (int32_t i = 0; i < n; i++) {
    fs_request *r = &reqs[i];
    r->status = -1;
    r->start_ns = r->done_ns = 0;
    r->batch = -1;
    if (r->session < 0 || r->session >= s->cfg.nsessions || r->map < 0 || r->map >= s->nmaps ||
        r->width <= 0 || r->height <= 0 || r->height > FS_MAX_ROWS || r->width > 16384)
      return fs_fail(ctx, FS_ERR_ARG, "request %d: bad session, map or size", i);
  }
  int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
  int32_t *pq = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
  int32_t *rq = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
  int64_t *frame_off = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
  srv_item *scratch = (srv_item *)malloc(sizeof(srv_item) * (size_t)s->max_items);
  if (!order || !pq || !rq || !frame_off || !scratch) {
    free(order);
    free(pq);
    free(rq);
    free(frame_off);
    free(scratch);
    return fs_fail(ctx, FS_ERR_NOMEM, "server run buffers");
  }
  for (int32_t i = 0; i < n; i++) order[i] = i;
  qsort_r(order, (size_t)n, sizeof(int32_t), cmp_arrival, reqs);
  fs_fifo pending = {pq, 0, 0, n ? n : 1}, ready = {rq, 0, 0, n ? n : 1};
  int32_t next = 0, completed = 0, batch_id = 0, inflight = 0;
  int rc = FS_OK;
  struct rusage ru0;
  memset(&ru0, 0, sizeof(ru0));
  getrusage(RUSAGE_THREAD, &ru0);
  const int64_t t0 = now_ns();
  while (completed < n && !rc) {
    int progress = 0;
    const int64_t t_iter = now_ns();
    int64_t slept = 0;
    s->iter_call_ns = 0;
    const int64_t now = t_iter - t0;
    /* release arrivals */
    while (next < n && (!realtime || reqs[order[next]].arrival_ns <= now)) {
      fifo_push(&pending, order[next++]);
      progress = 1;
    }
    /* admission: FIFO, skipping requests whose session is busy or whose frame
     * does not fit yet (they keep their place) */
    int32_t keep = pending.head;
    for (int32_t p = pending.head; p < pending.tail; p++) {
      const int32_t ri = pending.q[p % pending.cap];
      fs_request *r = &reqs[ri];
      const int64_t bytes = req_frame_bytes(r);
      if (round256(bytes) > s->arena.size) {
        r->status = fs_fail(ctx, FS_ERR_BUDGET, "frame of %lld bytes exceeds the budget",
                            (long long)bytes);
        r->done_ns = now;
        completed++;
        st.errors++;
        continue;
      }
      int64_t off = -1;
      if (!s->sess_busy[r->session]) off = arena_alloc(&s->arena, bytes);
      if (off >= 0) {
        s->sess_busy[r->session] = 1;
        frame_off[ri] = off;
        fifo_push(&ready, ri);
        inflight++;
        if (inflight > st.max_inflight) st.max_inflight = inflight;
        progress = 1;
      } else {
        pending.q[keep % pending.cap] = ri;
        keep++;
      }
    }
    pending.tail = keep;
    /* completions */
    for (int i = 0; i < s->cfg.slots; i++) {
      fs_slot *sl = &s->slots[i];
      if (!sl->busy) continue;
      const int64_t tq = now_ns();
      const cudaError_t q = cudaEventQuery(sl->ev);
      note_call(s, &st, FS_SERVE_SITE_EVENT_QUERY, now_ns() - tq);
      if (q == cudaErrorNotReady) continue;
      if (q != cudaSuccess) {
        rc = fs_cuda_fail(ctx, q, "serving batch");
        break;
      }
      const int64_t done = now_ns() - t0;
      float gpu_ms = 0.0f;
      if (cudaEventElapsedTime(&gpu_ms, sl->ev0, sl->ev) == cudaSuccess &&
          (double)gpu_ms > st.max_batch_gpu_ms) {
        st.max_batch_gpu_ms = (double)gpu_ms;
        st.max_batch_gpu_at_ns = sl->launch_ns;
      }
      for (int32_t k = 0; k < sl->nreq; k++) {
        const int32_t ri = sl->req[k];
        fs_request *r = &reqs[ri];
        r->status = FS_OK;
        r->done_ns = done;
        arena_free(&s->arena, frame_off[ri], req_frame_bytes(r));
        s->sess_busy[r->session] = 0;
        st.pixels += (int64_t)r->width * r->height;
        completed++;
        inflight--;
      }
      sl->busy = 0;
      progress = 1;
    }
    /* launches: every free slot takes the ready requests */
    for (int i = 0; i < s->cfg.slots && !rc && ready.head < ready.tail; i++) {
      fs_slot *sl = &s->slots[i];
      if (sl->busy) continue;
      const int32_t before = completed;
      rc = launch_batch(s, sl, reqs, &ready, frame_off, scratch, t0, batch_id++, &completed, &st);
      inflight -= completed - before;
      progress = 1;
    }
    if (!progress && realtime && next < n) {
      /* idle until the next arrival or a completion: short sleeps keep the
       * host clock pacing accurate to a few microseconds */
      struct timespec ts = {0, 2000};
      const int64_t ts0 = now_ns();
      nanosleep(&ts, NULL);
      slept = now_ns() - ts0;
      if ((double)slept * 1e-6 > st.max_sleep_ms) st.max_sleep_ms = (double)slept * 1e-6;
    }
    const double host_ms = (double)(now_ns() - t_iter - slept - s->iter_call_ns) * 1e-6;
    if (host_ms > st.max_host_ms) {
      st.max_host_ms = host_ms;
      st.max_host_at_ns = now;
    }
  }
  {
    struct rusage ru1;
    memset(&ru1, 0, sizeof(ru1));
    getrusage(RUSAGE_THREAD, &ru1);
    st.involuntary_switches = (int64_t)(ru1.ru_nivcsw - ru0.ru_nivcsw);
    st.voluntary_switches = (int64_t)(ru1.ru_nvcsw - ru0.ru_nvcsw);
  }
  const int64_t t_end = now_ns() - t0;
  /* drain anything still in flight after an error */
  for (int i = 0; i < s->cfg.slots; i++)
    if (s->slots[i].busy) cudaStreamSynchronize(s->slots[i].st);
  if (!rc) {
    double *lat = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
    int32_t m = 0;
    double sum = 0.0;
    for (int32_t i = 0; i < n; i++)
      if (reqs[i].status == FS_OK) {
        lat[m] = (double)(reqs[i].done_ns - reqs[i].arrival_ns * (realtime ? 1 : 0)) * 1e-6;
        sum += lat[m];
        m++;
      }
    if (lat && m > 0) {
      qsort(lat, (size_t)m, sizeof(double), cmp_double);
      st.p50_ms = lat[(int64_t)(0.50 * (m - 1) + 0.5)];
      st.p99_ms = lat[(int64_t)(0.99 * (m - 1) + 0.5)];
      st.max_ms = lat[m - 1];
      st.mean_ms = sum / m;
    }
    free(lat);
    st.requests = n;
    st.wall_s = (double)t_end * 1e-9;
    st.gpix_s = st.wall_s > 0 ? (double)st.pixels / st.wall_s * 1e-9 : 0.0;
    st.mean_batch = st.batches ? st.mean_batch / (double)st.batches : 0.0;
    st.peak_arena_bytes = s->arena.peak;
    if (stats) *stats = st;
  }
  free(order);
  free(pq);
  free(rq);
  free(frame_off);
  free(scratch);
  return rc;
}
