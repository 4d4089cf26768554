/*
 * Batched multi-view rendering. A plan owns one framebuffer arena with a frame
 * per view, a depth table per view, the tensor maps of the frames and a list of
 * (view, column-tile) work items sorted by estimated cost. One run is three
 * stream operations -- reset the work counter, build every view's depth table,
 * launch the persistent render kernel sized to fill the GPU -- captured once
 * into a CUDA graph and replayed. The items are pulled from the counter in
 * cost order, so large and small views balance across the SMs.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#include "fs_internal.h"
#include "fs_priv.h"

typedef struct {
  int64_t cost;
  int64_t item;
} fs_item_cost;

static int cmp_cost_desc(const void *a, const void *b) {
  const fs_item_cost *x = (const fs_item_cost *)a, *y = (const fs_item_cost *)b;
  if (x->cost != y->cost) return x->cost > y->cost ? -1 : 1;
  return x->item < y->item ? -1 : (x->item > y->item);
}

static void plan_release_graph(fs_plan *p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = NULL;
  p->graph = NULL;
  p->graph_ok = 0;
}

void fs_plan_free(fs_plan *p) {
  if (!p) return;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  plan_release_graph(p);
  for (int i = 0; i < 2; i++)
    if (p->ev_render[i]) cudaEventDestroy(p->ev_render[i]);
  for (int i = 0; i < FS_PLAN_MAX_GROUPS; i++) {
    if (p->grp_done[i]) cudaEventDestroy(p->grp_done[i]);
    if (p->grp_meta[i]) cudaEventDestroy(p->grp_meta[i]);
  }
  if (p->copy_stream) cudaStreamDestroy(p->copy_stream);
  if (p->meta_stream) cudaStreamDestroy(p->meta_stream);
  cudaFree(p->sky_d);
  cudaFreeHost(p->sky_h);
  cudaFree(p->grp_items_d);
  cudaFree(p->grp_heads_d);
  free(p->items_h);
  cudaFree(p->fv_d);
  cudaFree(p->tm_d);
  cudaFree(p->items_d);
  cudaFree(p->head_d);
  cudaFree(p->segitems_d);
  cudaFree(p->segbuf_d);
  cudaFree(p->zline);
  cudaFree(p->zinvz);
  cudaFree(p->frames);
  free(p->views_h);
  free(p->fv_h);
  free(p->ncap);
  free(p->tm_h);
  free(p->offsets);
  free(p);
}

static void plan_fill_launch(fs_plan *p, FsLaunch *L) {
  memset(L, 0, sizeof(*L));
  for (int i = 0; i < p->nmaps; i++) {
    L->maps[i] = p->maps[i];
    if (p->ctx->no_skip) L->maps[i].pyr = NULL;
  }
  L->views = p->fv_d;
  L->items = p->items_d;
  L->tmaps = p->tm_d;
  L->zline = p->zline;
  L->zinvz = p->zinvz;
  L->head = p->head_d;
  L->nitems = p->nitems;
  L->stride_max = p->stride_max;
  /* the work counters cost instructions per depth chunk: only when collected */
  L->stats = p->ctx->collect_stats ? p->ctx->stats_dev : NULL;
}

/* The segment-minimum pass over every split view (none when nothing is split). */
static int plan_segmin(fs_plan *p) {
  if (!p->nsegitems) return 0;
  FsLaunch L;
  plan_fill_launch(p, &L);
  L.items = p->segitems_d;
  L.nitems = p->nsegitems;
  L.head = p->head_d + 1;
  L.stats = NULL;
  const int32_t per_cta = fsk_items_per_cta(&p->tune);
  int32_t grid = (p->nsegitems + per_cta - 1) / per_cta;
  if (grid > p->grid) grid = p->grid;
  return fsk_segmin(&L, &p->tune, p->hf, grid, p->ctx->stream);
}

/* The render kernel's configuration with the segment-reading variant when some
 * view is split. */
static FsTune plan_kernel_tune(const fs_plan *p) {
  FsTune t = p->tune;
  t.seg = p->segbuf_d != NULL;
  return t;
}

static int plan_enqueue(fs_plan *p) {
  fs_ctx *ctx = p->ctx;
  const FsTune kt = plan_kernel_tune(p);
  FsLaunch launch;
  plan_fill_launch(p, &launch);
  int32_t max_n = 0;
  for (int v = 0; v < p->nviews; v++)
    if (p->ncap[v] > max_n) max_n = p->ncap[v];
  int e = cudaMemsetAsync(p->head_d, 0, 2 * sizeof(int32_t), ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "work counter reset");
  e = fsk_ztable(p->fv_d, NULL, p->nviews, max_n, p->zline, p->zinvz, ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "z-table kernel launch");
  e = plan_segmin(p);
  if (e) return fs_cuda_fail(ctx, e, "segment-minimum kernel launch");
  /* external event nodes bracket the render kernel, so its device time is
   * readable after every replay of the graph */
  e = cudaEventRecordWithFlags(p->ev_render[0], ctx->stream, cudaEventRecordExternal);
  if (e) return fs_cuda_fail(ctx, e, "render start event");
  e = fsk_render(&launch, &kt, p->hf, p->cf, p->grid, ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "persistent render kernel launch");
  e = cudaEventRecordWithFlags(p->ev_render[1], ctx->stream, cudaEventRecordExternal);
  if (e) return fs_cuda_fail(ctx, e, "render end event");
  if (p->segbuf_d) {
    e = fsk_gapfill(p->fv_d, NULL, p->nviews, p->wmax, ctx->stream);
    if (e) return fs_cuda_fail(ctx, e, "gap-fill kernel launch");
  }
  return FS_OK;
}

/* (Re)builds everything that depends on the tuning: tensor maps (box width),
 * work items (tile width), grid size and the captured graph. */
/* The largest depth count of the plan's views (their capacity). */
int32_t fs_plan_max_depths(const fs_plan *p) {
  int32_t m = 0;
  for (int v = 0; v < p->nviews; v++)
    if (p->ncap[v] > m) m = p->ncap[v];
  return m;
}

static int plan_build(fs_plan *p) {
  fs_ctx *ctx = p->ctx;
  const int32_t tw = p->tune.tw;
  const int32_t iw = fsk_item_width(&p->tune);
  const int32_t chunk = p->tune.lc * p->tune.u;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  plan_release_graph(p);
  p->built_stats = ctx->collect_stats;
  int32_t occ = 0;
  int e = fsk_render_max_ctas_per_sm(&p->tune, p->hf, p->cf, p->stride_max, &occ);
  if (e) return fs_cuda_fail(ctx, e, "occupancy query");
  if (occ < 1) return fs_fail(ctx, FS_ERR_ARG, "render kernel does not fit on an SM");
  /* few strips in the whole batch: split every column's depths into segments */
  int64_t strips = 0;
  for (int v = 0; v < p->nviews; v++) strips += (p->fv_h[v].W + iw - 1) / iw;
  const int32_t target = fs_split_target(ctx, &p->tune, p->hf, p->cf, p->stride_max, strips);
  int64_t nitems = 0, nseg_items = 0, seg_rows = 0;
  for (int v = 0; v < p->nviews; v++) {
    FsView *fv = &p->fv_h[v];
    fv->out = p->frames + p->offsets[v];
    fv->tmap = fs_encode_frame_map(ctx, fv->out, fv->W, fv->H, tw, &p->tm_h[v]) ? v : -1;
    const int32_t tiles = (fv->W + iw - 1) / iw;
    if (tiles > FS_ITEM_TILES) return fs_fail(ctx, FS_ERR_ARG, "view %d: too many column tiles", v);
    /* segments from the depth count the plan was built with; a later shorter
     * draw distance leaves trailing segments empty */
    const int32_t n_now = fv->n;
    fv->n = p->ncap[v];
    fs_set_segments(fv, target, chunk);
    fv->n = n_now;
    nitems += (int64_t)tiles * fv->nseg;
    if (fv->nseg > 1) {
      nseg_items += (int64_t)tiles * (fv->nseg - 1);
      seg_rows += (int64_t)(fv->nseg + 2) * fv->W;
    }
  }
  cudaFree(p->segbuf_d);
  p->segbuf_d = NULL;
  if (seg_rows) {
    e = cudaMalloc((void **)&p->segbuf_d, sizeof(int32_t) * (size_t)seg_rows);
    if (e) return fs_cuda_fail(ctx, e, "cudaMalloc(segment rows)");
  }
  fs_item_cost *ic = (fs_item_cost *)malloc(sizeof(fs_item_cost) * (size_t)nitems);
  int64_t *items = (int64_t *)malloc(sizeof(int64_t) * (size_t)nitems);
  int64_t *segitems = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nseg_items ? nseg_items : 1));
  if (!ic || !items || !segitems) {
    free(ic);
    free(items);
    free(segitems);
    return fs_fail(ctx, FS_ERR_NOMEM, "malloc(items)");
  }
  int64_t k = 0, ks = 0, row_off = 0;
  for (int v = 0; v < p->nviews; v++) {
    FsView *fv = &p->fv_h[v];
    fv->segbuf = NULL;
    if (fv->nseg > 1) {
      fv->segbuf = p->segbuf_d + row_off;
      row_off += (int64_t)(fv->nseg + 2) * fv->W;
    }
    const int32_t tiles = (fv->W + iw - 1) / iw;
    for (int s = 0; s < fv->nseg; s++) {
      for (int t = 0; t < tiles; t++) {
        /* depth march dominates, then the store */
        ic[k].cost = (int64_t)(fv->nseg > 1 ? fv->seglen : fv->n) * 8 + fv->H;
        ic[k].item = FS_ITEM(v, s, t);
        k++;
        if (s < fv->nseg - 1) segitems[ks++] = FS_ITEM(v, s, t);
      }
    }
  }
  qsort(ic, (size_t)nitems, sizeof(fs_item_cost), cmp_cost_desc);
  for (int64_t i = 0; i < nitems; i++) items[i] = ic[i].item;
  free(ic);
  cudaFree(p->items_d);
  p->items_d = NULL;
  cudaFree(p->segitems_d);
  p->segitems_d = NULL;
  e = cudaMalloc((void **)&p->items_d, sizeof(int64_t) * (size_t)nitems);
  if (!e) e = cudaMemcpy(p->items_d, items, sizeof(int64_t) * (size_t)nitems,
                         cudaMemcpyHostToDevice);
  if (!e && ks) e = cudaMalloc((void **)&p->segitems_d, sizeof(int64_t) * (size_t)ks);
  if (!e && ks)
    e = cudaMemcpy(p->segitems_d, segitems, sizeof(int64_t) * (size_t)ks, cudaMemcpyHostToDevice);
  free(segitems);
  free(p->items_h);
  p->items_h = items;
  p->ngroups = 0; /* group lists follow the items */
  if (e) return fs_cuda_fail(ctx, e, "items upload");
  p->nitems = (int32_t)nitems;
  p->nsegitems = (int32_t)ks;
  e = cudaMemcpy(p->fv_d, p->fv_h, sizeof(FsView) * (size_t)p->nviews, cudaMemcpyHostToDevice);
  if (!e && p->tm_d)
    e = cudaMemcpy(p->tm_d, p->tm_h, sizeof(CUtensorMap) * (size_t)p->nviews,
                   cudaMemcpyHostToDevice);
  if (e) return fs_cuda_fail(ctx, e, "view upload");
  int64_t grid = (int64_t)occ * ctx->sm_count;
  if (p->tune.ctas > 0 && p->tune.ctas < grid) grid = p->tune.ctas;
  const int64_t per_cta = fsk_items_per_cta(&p->tune);
  if (grid > (nitems + per_cta - 1) / per_cta) grid = (nitems + per_cta - 1) / per_cta;
  p->grid = (int32_t)grid;

  for (int i = 0; i < 2; i++) {
    if (!p->ev_render[i]) {
      e = cudaEventCreate(&p->ev_render[i]);
      if (e) return fs_cuda_fail(ctx, e, "cudaEventCreate");
    }
  }
  /* capture reset + depth tables + persistent render into one graph */
  e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e) return fs_cuda_fail(ctx, e, "cudaStreamBeginCapture");
  int rc = plan_enqueue(p);
  cudaGraph_t g = NULL;
  e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e) return fs_cuda_fail(ctx, e, "cudaStreamEndCapture");
  p->graph = g;
  e = cudaGraphInstantiate(&p->exec, g, 0);
  if (e) return fs_cuda_fail(ctx, e, "cudaGraphInstantiate");
  p->graph_ok = 1;
  return FS_OK;
}

static int64_t batch_signature(const fs_plan *p) {
  /* order-independent hash of the (W, H) multiset */
  uint64_t h = 0;
  for (int v = 0; v < p->nviews; v++) {
    uint64_t x = ((uint64_t)(uint32_t)p->fv_h[v].W << 32) | (uint32_t)p->fv_h[v].H;
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    h += x;
  }
  return (int64_t)(h ^ (uint64_t)p->nviews);
}

int fs_plan_signature(const fs_plan *p, int64_t *sig) {
  if (!p || !sig) return FS_ERR_ARG;
  *sig = batch_signature(p);
  return FS_OK;
}

int fs_plan_new(fs_ctx *ctx, fs_plan **out, const fs_map *const *maps, int32_t nmaps,
                const fs_params *params, const fs_view *views, int32_t nviews) {
  if (!ctx || !out) return FS_ERR_ARG;
  *out = NULL;
  if (ctx->broken) return fs_fail(ctx, FS_ERR_STATE, "context failed to initialise");
  if (!maps || nmaps < 1 || nmaps > FS_MAX_MAPS)
    return fs_fail(ctx, FS_ERR_ARG, "need 1..%d maps", FS_MAX_MAPS);
  if (!views || nviews < 1 || nviews >= FS_ITEM_VIEWS)
    return fs_fail(ctx, FS_ERR_ARG, "need 1..%d views", FS_ITEM_VIEWS - 1);
  for (int i = 0; i < nmaps; i++)
    if (!maps[i]) return fs_fail(ctx, FS_ERR_ARG, "map %d is NULL", i);
  fs_params dp = fs_params_default();
  if (!params) params = &dp;
  int rc = fs_check_params(ctx, params);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  fs_plan *p = (fs_plan *)calloc(1, sizeof(fs_plan));
  if (!p) return fs_fail(ctx, FS_ERR_NOMEM, "calloc(plan)");
  p->ctx = ctx;
  p->nviews = nviews;
  p->nmaps = nmaps;
  p->params = *params;
  p->hf = params->height_filter == FS_BILINEAR;
  p->cf = params->color_filter == FS_BILINEAR;
  for (int i = 0; i < nmaps; i++) p->maps[i] = maps[i]->dev;
  p->views_h = (fs_view *)malloc(sizeof(fs_view) * (size_t)nviews);
  p->fv_h = (FsView *)malloc(sizeof(FsView) * (size_t)nviews);
  p->ncap = (int32_t *)malloc(sizeof(int32_t) * (size_t)nviews);
  p->offsets = (int64_t *)malloc(sizeof(int64_t) * (size_t)nviews);
  p->tm_h = (CUtensorMap *)aligned_alloc(128, sizeof(CUtensorMap) * (size_t)nviews);
  if (!p->views_h || !p->fv_h || !p->ncap || !p->offsets || !p->tm_h) {
    fs_plan_free(p);
    return fs_fail(ctx, FS_ERR_NOMEM, "malloc(plan arrays)");
  }
  memcpy(p->views_h, views, sizeof(fs_view) * (size_t)nviews);
  int64_t zoff = 0, px = 0;
  int32_t hmax = 1;
  for (int v = 0; v < nviews; v++) {
    const fs_view *vw = &views[v];
    if (vw->map < 0 || vw->map >= nmaps) {
      fs_plan_free(p);
      return fs_fail(ctx, FS_ERR_ARG, "view %d: map index %d out of range", v, vw->map);
    }
    rc = fs_make_view(ctx, &vw->cam, params, vw->width, vw->height, vw->map, &p->fv_h[v]);
    if (rc) {
      fs_plan_free(p);
      return rc;
    }
    p->fv_h[v].zoff = zoff;
    p->ncap[v] = p->fv_h[v].n;
    zoff += p->fv_h[v].n + FS_ZPAD;
    p->offsets[v] = px;
    px += ((int64_t)vw->width * vw->height + 63) & ~(int64_t)63; /* 256-byte aligned frames */
    if (vw->height > hmax) hmax = vw->height;
    if (vw->width > p->wmax) p->wmax = vw->width;
  }
  p->ztotal = zoff;
  p->total_px = px;
  p->stride_max = hmax | 1;
  int e = cudaMalloc((void **)&p->fv_d, sizeof(FsView) * (size_t)nviews);
  if (!e) e = cudaMalloc((void **)&p->head_d, 2 * sizeof(int32_t));
  if (!e) e = cudaMalloc((void **)&p->zline, sizeof(float4) * (size_t)zoff);
  if (!e) e = cudaMalloc((void **)&p->zinvz, sizeof(float) * (size_t)zoff);
  if (!e) e = cudaMalloc((void **)&p->frames, sizeof(uint32_t) * (size_t)px);
  if (!e && ctx->use_tma) e = cudaMalloc((void **)&p->tm_d, sizeof(CUtensorMap) * (size_t)nviews);
  if (e) {
    fs_plan_free(p);
    return fs_fail(ctx, FS_ERR_NOMEM, "cudaMalloc(plan: %lld frame pixels)", (long long)px);
  }
  /* tuning: cache entry for this batch signature, else the default */
  char key[96];
  snprintf(key, sizeof(key), "batch:%016llx:map%dx%d:f%d", (unsigned long long)batch_signature(p),
           p->maps[0].MH, p->maps[0].MW, p->hf | (p->cf << 1));
  FsTune t;
  if (!fs_tune_lookup_key(ctx, key, &t) || !fs_tune_fits(ctx, &t, p->stride_max) ||
      !fs_coop_depths_ok(&t, fs_plan_max_depths(p)))
    t = fs_default_batch_tune(ctx, p->stride_max);
  if (!t.tw) {
    fs_plan_free(p);
    return fs_fail(ctx, FS_ERR_ARG, "no kernel configuration fits screen height %d", hmax);
  }
  p->tune = fs_tune_for_mode(t, p->fv_h[0].flags);
  rc = plan_build(p);
  if (rc) {
    fs_plan_free(p);
    return rc;
  }
  *out = p;
  return FS_OK;
}

int fs_plan_set_cameras(fs_plan *p, const fs_camera *cams, int32_t ncams) {
  if (!p || !cams) return FS_ERR_ARG;
  fs_ctx *ctx = p->ctx;
  if (ncams != p->nviews) return fs_fail(ctx, FS_ERR_ARG, "expected %d cameras", p->nviews);
  for (int v = 0; v < p->nviews; v++) {
    FsView nv;
    const fs_view *vw = &p->views_h[v];
    int rc = fs_make_view(ctx, &cams[v], &p->params, vw->width, vw->height, vw->map, &nv);
    if (rc) return rc;
    if (nv.n > p->ncap[v])
      return fs_fail(ctx, FS_ERR_ARG, "view %d: %d depth samples exceed the plan's %d", v, nv.n,
                     p->ncap[v]);
    nv.zoff = p->fv_h[v].zoff;
    nv.out = p->fv_h[v].out;
    nv.tmap = p->fv_h[v].tmap;
    /* segments stay as built (from the depth capacity) */
    nv.nseg = p->fv_h[v].nseg;
    nv.seglen = p->fv_h[v].seglen;
    nv.segbuf = p->fv_h[v].segbuf;
    p->fv_h[v] = nv;
    p->views_h[v].cam = cams[v];
  }
  cudaSetDevice(ctx->device);
  int e = cudaMemcpyAsync(p->fv_d, p->fv_h, sizeof(FsView) * (size_t)p->nviews,
                          cudaMemcpyHostToDevice, ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "camera upload");
  return FS_OK;
}

int fs_plan_run(fs_plan *p) {
  if (!p) return FS_ERR_ARG;
  fs_ctx *ctx = p->ctx;
  if (!p->graph_ok) return fs_fail(ctx, FS_ERR_STATE, "plan has no graph");
  cudaSetDevice(ctx->device);
  /* the graph holds the launch parameters: rebuild it when the context
   * started or stopped collecting work counters since it was captured */
  if (p->built_stats != ctx->collect_stats) {
    const int rc = plan_build(p);
    if (rc) return rc;
  }
  int e = cudaGraphLaunch(p->exec, ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "cudaGraphLaunch");
  /* depth tables + render, plus the segment-minimum and gap-fill passes */
  ctx->launches += 2 + (p->nsegitems ? 1 : 0) + (p->segbuf_d ? 1 : 0);
  return FS_OK;
}

int fs_plan_kernel_ms(fs_plan *p, float *ms) {
  if (!p || !ms) return FS_ERR_ARG;
  fs_ctx *ctx = p->ctx;
  if (!p->graph_ok) return fs_fail(ctx, FS_ERR_STATE, "plan has no graph");
  cudaSetDevice(ctx->device);
  int e = cudaEventSynchronize(p->ev_render[1]);
  if (!e) e = cudaEventElapsedTime(ms, p->ev_render[0], p->ev_render[1]);
  if (e) return fs_cuda_fail(ctx, e, "render kernel timing");
  return FS_OK;
}

int fs_plan_run_per_view(fs_plan *p) {
  if (!p) return FS_ERR_ARG;
  fs_ctx *ctx = p->ctx;
  cudaSetDevice(ctx->device);
  for (int v = 0; v < p->nviews; v++) {
    FsView fv = p->fv_h[v];
    FsTune t;
    if (!fs_tune_lookup(ctx, fv.W, fv.H, p->maps[fv.map].MH, p->maps[fv.map].MW, fv.flags, &t) ||
        !fs_tune_fits(ctx, &t, fv.H | 1))
      t = fs_default_tune(ctx, fv.H | 1);
    CUtensorMap tm __attribute__((aligned(128)));
    const int have_tm = fs_encode_frame_map(ctx, fv.out, fv.W, fv.H, t.tw, &tm);
    int rc = fs_render_view(ctx, &p->maps[fv.map], &fv, &t, p->zline, p->zinvz,
                            have_tm ? &tm : NULL, 1);
    if (rc) return rc;
  }
  return FS_OK;
}

uint32_t *fs_plan_frame_dev(fs_plan *p, int32_t view) {
  if (!p || view < 0 || view >= p->nviews) return NULL;
  return p->frames + p->offsets[view];
}

int64_t fs_plan_frame_offset(const fs_plan *p, int32_t view) {
  if (!p || view < 0 || view >= p->nviews) return -1;
  return p->offsets[view];
}

int64_t fs_plan_total_pixels(const fs_plan *p) { return p ? p->total_px : 0; }

int fs_plan_download(fs_plan *p, uint32_t *host) {
  if (!p || !host) return FS_ERR_ARG;
  fs_ctx *ctx = p->ctx;
  cudaSetDevice(ctx->device);
  int e = cudaMemcpyAsync(host, p->frames, sizeof(uint32_t) * (size_t)p->total_px,
                          cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return fs_cuda_fail(ctx, e, "frame download");
  return FS_OK;
}

/* Splits the views into `groups` contiguous ranges of about equal pixel count
 * and uploads each range's items (in launch order) with its own work counter. */
static int plan_build_groups(fs_plan *p, int32_t groups) {
  fs_ctx *ctx = p->ctx;
  int64_t done_px = 0, v = 0;
  p->grp_first[0] = 0;
  for (int g = 0; g < groups; g++) {
    const int64_t target = p->total_px * (g + 1) / groups;
    const int64_t left = groups - g - 1; /* keep a view for every later group */
    while (v < p->nviews - left && (done_px < target || v == p->grp_first[g])) {
      done_px += (int64_t)p->fv_h[v].W * p->fv_h[v].H;
      v++;
    }
    p->grp_first[g + 1] = (int32_t)v;
  }
  p->grp_first[groups] = p->nviews;
  int64_t *sorted = (int64_t *)malloc(sizeof(int64_t) * (size_t)(p->nitems ? p->nitems : 1));
  if (!sorted) return fs_fail(ctx, FS_ERR_NOMEM, "malloc(group items)");
  int32_t k = 0;
  for (int g = 0; g < groups; g++) {
    p->grp_item_off[g] = k;
    for (int32_t i = 0; i < p->nitems; i++) {
      const int32_t view = FS_ITEM_VIEW(p->items_h[i]);
      if (view >= p->grp_first[g] && view < p->grp_first[g + 1]) sorted[k++] = p->items_h[i];
    }
  }
  p->grp_item_off[groups] = k;
  cudaFree(p->grp_items_d);
  p->grp_items_d = NULL;
  int e = cudaMalloc((void **)&p->grp_items_d, sizeof(int64_t) * (size_t)(k ? k : 1));
  if (!e) e = cudaMemcpy(p->grp_items_d, sorted, sizeof(int64_t) * (size_t)k, cudaMemcpyHostToDevice);
  free(sorted);
  if (!e && !p->grp_heads_d)
    e = cudaMalloc((void **)&p->grp_heads_d, sizeof(int32_t) * FS_PLAN_MAX_GROUPS);
  if (!e && !p->copy_stream) e = cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking);
  if (!e && !p->meta_stream) e = cudaStreamCreateWithFlags(&p->meta_stream, cudaStreamNonBlocking);
  if (!e && !p->sky_d) e = cudaMalloc((void **)&p->sky_d, sizeof(int32_t) * (size_t)p->nviews);
  if (!e && !p->sky_h) e = cudaMallocHost((void **)&p->sky_h, sizeof(int32_t) * (size_t)p->nviews);
  for (int g = 0; !e && g < FS_PLAN_MAX_GROUPS; g++) {
    if (!p->grp_done[g]) e = cudaEventCreateWithFlags(&p->grp_done[g], cudaEventDisableTiming);
    if (!e && !p->grp_meta[g])
      e = cudaEventCreateWithFlags(&p->grp_meta[g], cudaEventDisableTiming);
  }
  if (e) return fs_cuda_fail(ctx, e, "group set-up");
  p->ngroups = groups;
  return FS_OK;
}

/* The sky rows [0, s_v) of views [v0, v1) of `host` (frames at the plan's
 * offsets): split into pieces of at most 256 K pixels, written by the host's
 * threads. Returns the bytes written. */
static int64_t fill_sky_rows(const fs_plan *p, uint32_t *host, int32_t v0, int32_t v1) {
  enum { PIECE = 256 * 1024 };
  int64_t pieces = 0, bytes = 0;
  for (int32_t v = v0; v < v1; v++) {
    const int64_t px = (int64_t)p->sky_h[v] * p->fv_h[v].W;
    pieces += (px + PIECE - 1) / PIECE;
    bytes += 4 * px;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < pieces; k++) {
    /* the piece's view: walk the group's views (a few dozen) */
    int64_t base = 0;
    int32_t v = v0;
    for (;; v++) {
      const int64_t np = ((int64_t)p->sky_h[v] * p->fv_h[v].W + PIECE - 1) / PIECE;
      if (k < base + np) break;
      base += np;
    }
    const int64_t px = (int64_t)p->sky_h[v] * p->fv_h[v].W;
    const int64_t a = (k - base) * PIECE, b = a + PIECE < px ? a + PIECE : px;
    fs_fill_u32(host + p->offsets[v] + a, b - a, p->fv_h[v].sky);
  }
  return bytes;
}

int fs_plan_run_download(fs_plan *p, uint32_t *host, int32_t groups) {
  if (!p || !host) return FS_ERR_ARG;
  fs_ctx *ctx = p->ctx;
  if (!p->graph_ok) return fs_fail(ctx, FS_ERR_STATE, "plan has no kernel configuration");
  if (groups < 1) groups = 1;
  if (groups > FS_PLAN_MAX_GROUPS) groups = FS_PLAN_MAX_GROUPS;
  if (groups > p->nviews) groups = p->nviews;
  cudaSetDevice(ctx->device);
  int rc = FS_OK;
  if (p->ngroups != groups) {
    cudaStreamSynchronize(ctx->stream);
    rc = plan_build_groups(p, groups);
    if (rc) return rc;
  }
  /* the host writes the sky rows when its OpenMP team can outrun the link (one
   * thread writes about 44 GB/s, the link moves 193); a smaller team (e.g.
   * OMP_NUM_THREADS=1) gets whole frames over the link, a copy per group */
  const int host_sky = omp_get_max_threads() >= 4;
  int32_t max_n = 0;
  for (int v = 0; v < p->nviews; v++)
    if (p->ncap[v] > max_n) max_n = p->ncap[v];
  int e = cudaMemsetAsync(p->grp_heads_d, 0, sizeof(int32_t) * (size_t)groups, ctx->stream);
  if (!e) e = cudaMemsetAsync(p->head_d, 0, 2 * sizeof(int32_t), ctx->stream);
  /* every view's all-sky row count starts above any frame height */
  if (!e && host_sky)
    e = cudaMemsetAsync(p->sky_d, 0x7F, sizeof(int32_t) * (size_t)p->nviews, ctx->stream);
  if (!e) e = fsk_ztable(p->fv_d, NULL, p->nviews, max_n, p->zline, p->zinvz, ctx->stream);
  if (!e) e = plan_segmin(p);
  const int32_t per_cta = fsk_items_per_cta(&p->tune);
  const FsTune kt = plan_kernel_tune(p);
  /* every group's render, then its views' sky rows to the host */
  for (int g = 0; !e && g < groups; g++) {
    FsLaunch L;
    plan_fill_launch(p, &L);
    L.items = p->grp_items_d + p->grp_item_off[g];
    L.nitems = p->grp_item_off[g + 1] - p->grp_item_off[g];
    L.head = p->grp_heads_d + g;
    int32_t grid = (L.nitems + per_cta - 1) / per_cta;
    if (grid > p->grid) grid = p->grid;
    if (L.nitems > 0) e = fsk_render(&L, &kt, p->hf, p->cf, grid, ctx->stream);
    if (!e && p->segbuf_d)
      e = fsk_gapfill(p->fv_d + p->grp_first[g], NULL, p->grp_first[g + 1] - p->grp_first[g],
                      p->wmax, ctx->stream);
    const int32_t v0 = p->grp_first[g], v1 = p->grp_first[g + 1];
    /* each finished frame's leading rows that hold nothing but sky */
    if (!e && host_sky)
      e = fsk_sky_rows(p->fv_d + v0, NULL, v1 - v0, p->stride_max, p->sky_d + v0, ctx->stream);
    if (!e) e = cudaEventRecord(p->grp_done[g], ctx->stream);
    if (!e && host_sky) {
      e = cudaStreamWaitEvent(p->meta_stream, p->grp_done[g], 0);
      if (!e)
        e = cudaMemcpyAsync(p->sky_h + v0, p->sky_d + v0, sizeof(int32_t) * (size_t)(v1 - v0),
                            cudaMemcpyDeviceToHost, p->meta_stream);
      if (!e) e = cudaEventRecord(p->grp_meta[g], p->meta_stream);
    }
  }
  ctx->launches += 1 + (host_sky ? 2 : 1) * groups + (p->nsegitems ? 1 : 0) +
                   (p->segbuf_d ? groups : 0);
  /* per group, once its sky rows are known: the rows below them cross the
   * link (one copy per view, after the group's render), and the host's
   * threads write the sky rows meanwhile */
  int64_t copied = host_sky ? 4 * (int64_t)p->nviews : 0, filled = 0;
  for (int g = 0; !e && g < groups; g++) {
    const int32_t v0 = p->grp_first[g], v1 = p->grp_first[g + 1];
    if (!host_sky) {
      const int64_t a = p->offsets[v0], b = v1 < p->nviews ? p->offsets[v1] : p->total_px;
      e = cudaStreamWaitEvent(p->copy_stream, p->grp_done[g], 0);
      if (!e && b > a)
        e = cudaMemcpyAsync(host + a, p->frames + a, sizeof(uint32_t) * (size_t)(b - a),
                            cudaMemcpyDeviceToHost, p->copy_stream);
      copied += 4 * (b - a);
      continue;
    }
    e = cudaEventSynchronize(p->grp_meta[g]);
    if (!e) e = cudaStreamWaitEvent(p->copy_stream, p->grp_done[g], 0);
    for (int32_t v = v0; !e && v < v1; v++) {
      const int32_t H = p->fv_h[v].H, W = p->fv_h[v].W;
      int32_t s = p->sky_h[v];
      s = s < 0 ? 0 : (s > H ? H : s);
      p->sky_h[v] = s;
      const int64_t a = p->offsets[v] + (int64_t)s * W, px = (int64_t)(H - s) * W;
      if (px > 0) {
        e = cudaMemcpyAsync(host + a, p->frames + a, sizeof(uint32_t) * (size_t)px,
                            cudaMemcpyDeviceToHost, p->copy_stream);
        copied += 4 * px;
      }
    }
    if (!e) filled += fill_sky_rows(p, host, v0, v1);
  }
  if (!e) e = cudaStreamSynchronize(p->copy_stream);
  if (e) {
    /* no copy into the caller's buffer outlives the call */
    cudaStreamSynchronize(p->copy_stream);
    return fs_cuda_fail(ctx, e, "pipelined render and download");
  }
  p->dl_copied = copied;
  p->dl_filled = filled;
  return FS_OK;
}

int fs_plan_download_bytes(const fs_plan *p, int64_t *copied, int64_t *filled) {
  if (!p) return FS_ERR_ARG;
  if (copied) *copied = p->dl_copied;
  if (filled) *filled = p->dl_filled;
  return FS_OK;
}

int fs_plan_get_tune(const fs_plan *p, int32_t out5[5]) {
  if (!p || !out5) return FS_ERR_ARG;
  out5[0] = p->tune.tw;
  out5[1] = p->tune.lc;
  out5[2] = p->tune.u;
  out5[3] = p->tune.stage;
  out5[4] = p->grid;
  return FS_OK;
}

int fs_plan_set_tune(fs_plan *p, const int32_t tune5[5]) {
  if (!p || !tune5) return FS_ERR_ARG;
  FsTune t = {tune5[0], tune5[1], tune5[2], tune5[3], tune5[4], 0, 0};
  t.smooth = (p->fv_h[0].flags & FSV_SMOOTH) ? 1 : 0;
  t.fx = (p->fv_h[0].flags & (FSV_SHADE | FSV_FOG)) ? 1 : 0;
  if (!fs_tune_fits(p->ctx, &t, p->stride_max))
    return fs_fail(p->ctx, FS_ERR_ARG, "tuning (%d,%d,%d,%d) unsupported or too large", t.tw,
                   t.lc, t.u, t.stage);
  if (!fs_coop_depths_ok(&t, fs_plan_max_depths(p)))
    return fs_fail(p->ctx, FS_ERR_ARG, "the cooperative tile holds at most %d depths per view",
                   FS_COOP_MAX_DEPTHS);
  p->tune = t;
  return plan_build(p);
}
