/* Private host-side definitions of the C library (not part of the ABI). */
#ifndef FS_PRIV_H
#define FS_PRIV_H

#include <stdint.h>

#include "fs_internal.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FS_TUNE_CACHE_MAX 256

typedef struct {
  char key[96];
  FsTune tune;
} fs_tune_entry;

struct fs_ctx {
  int32_t device;
  int32_t broken;
  cudaStream_t own_stream;
  cudaStream_t stream;
  char err[1024];
  int32_t has_err;
  void *encode; /* cuTensorMapEncodeTiled, NULL when the driver lacks it */
  int32_t use_tma;
  int32_t no_skip; /* 1: ignore the height max pyramid (no chunk skipping) */
  int32_t no_split; /* 1: never split a column's depth range into segments */
  int32_t sm_count;
  size_t smem_optin;
  float4 *zline; /* single-frame depth table */
  float *zinvz;
  int64_t zcap;
  int32_t *segbuf; /* single-frame segment minima, final rows, gap flags */
  int64_t segcap;
  uint32_t *frame_dev; /* device frame for fs_render with host output */
  size_t frame_cap;
  unsigned long long *stats_dev;
  int32_t collect_stats;
  int64_t launches;
  int32_t time_kernel;   /* 1: events around the render kernels of each plain call */
  int32_t kernel_timed;  /* the events hold a completed call's timing */
  cudaEvent_t ev_kernel[2];
  /* device address of the allocation-free render's fixed scratch array on
   * this context's device, looked up once at context creation */
  void *noalloc_scratch;
  FsTune forced; /* tw == 0: choose per frame */
  int32_t ntune;
  fs_tune_entry tunes[FS_TUNE_CACHE_MAX];
  char tune_path[512];
};

struct fs_map {
  FsMapDev dev;
  int32_t owned; /* 1: quads and colours owned; 2: quads owned, colours borrowed */
  uint8_t *pyr;  /* height max pyramid (owned), NULL when not built */
  uint32_t *q;
  uint32_t *c;
  int64_t rows, cols;
};

#define FS_PLAN_MAX_GROUPS 16

struct fs_plan {
  fs_ctx *ctx;
  int32_t nviews, nmaps;
  fs_params params;
  fs_view *views_h;
  FsView *fv_h;        /* host copy of the kernel view records */
  int32_t *ncap;       /* depth capacity per view (n at plan creation) */
  FsView *fv_d;
  CUtensorMap *tm_h;   /* 128-byte aligned host array */
  CUtensorMap *tm_d;
  int64_t *items_d;  /* render items (FS_ITEM), launch order */
  int32_t nitems;
  int64_t *segitems_d; /* segment-minimum items of split views */
  int32_t nsegitems;
  int32_t *segbuf_d;   /* segment rows of split views (NULL: none split) */
  int32_t *head_d;     /* [0] render work counter, [1] segment-minimum counter */
  float4 *zline;
  float *zinvz;
  int64_t ztotal;
  uint32_t *frames;
  int64_t *offsets;
  int64_t total_px;
  FsMapDev maps[FS_MAX_MAPS];
  FsTune tune;
  int32_t grid;
  int32_t stride_max;
  int32_t wmax; /* widest view */
  int32_t hf, cf;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
  int32_t graph_ok;
  int32_t built_stats; /* ctx->collect_stats when the graph was captured */
  cudaEvent_t ev_render[2]; /* recorded around the render kernel inside the graph */
  int64_t *items_h;          /* the items in launch order (host copy) */
  /* pipelined render + download (fs_plan_run_download): views split into
   * contiguous groups, each rendered by its own launch while earlier groups'
   * frames are copied to the host on copy_stream */
  int32_t ngroups; /* 0: not built for the current items */
  int32_t grp_first[FS_PLAN_MAX_GROUPS + 1];
  int32_t grp_item_off[FS_PLAN_MAX_GROUPS + 1];
  int64_t *grp_items_d;
  int32_t *grp_heads_d;
  cudaStream_t copy_stream;
  cudaEvent_t grp_done[FS_PLAN_MAX_GROUPS];
  /* per view, the rows at the top that are sky in every column (the render
   * kernels' atomicMin of the columns' final minimum rows): only the rows
   * below them cross the device-to-host link, the host writes the sky rows */
  int32_t *sky_d;
  int32_t *sky_h;                           /* pinned */
  cudaStream_t meta_stream;                 /* the group's sky rows to the host */
  cudaEvent_t grp_meta[FS_PLAN_MAX_GROUPS];
  int64_t dl_copied, dl_filled;             /* bytes of the last run_download */
};

int fs_fail(fs_ctx *ctx, int code, const char *fmt, ...);
/* Writes `value` to n consecutive u32 (16-byte stores after a short head). */
void fs_fill_u32(uint32_t *dst, int64_t n, uint32_t value);
/* Looks up the allocation-free render's scratch address on ctx's (current)
 * device into ctx->noalloc_scratch (fs_noalloc.cu). */
int fs_noalloc_setup(fs_ctx *ctx);
int fs_cuda_fail(fs_ctx *ctx, int e, const char *what);
int32_t fs_f2i_host(float v);
int fs_check_params(fs_ctx *ctx, const fs_params *p);
int fs_make_view(fs_ctx *ctx, const fs_camera *cam, const fs_params *p, int32_t W, int32_t H,
                 int32_t map, FsView *v);
int fs_ensure_ztable(fs_ctx *ctx, int64_t n);
int fs_encode_frame_map(fs_ctx *ctx, uint32_t *frame, int32_t W, int32_t H, int32_t tw,
                        CUtensorMap *out);
int fs_render_view(fs_ctx *ctx, const FsMapDev *map, FsView *v, const FsTune *tune,
                   float4 *zline, float *zinvz, const CUtensorMap *tmap_pre, int32_t allow_split);
int32_t fs_split_target(fs_ctx *ctx, const FsTune *t, int32_t hf, int32_t cf, int32_t stride,
                        int64_t strips);
void fs_set_segments(FsView *v, int32_t nseg, int32_t chunk);
int fs_tune_fits(fs_ctx *ctx, const FsTune *t, int32_t stride_max);
FsTune fs_tune_for_mode(FsTune t, int32_t view_flags);
FsTune fs_default_tune(fs_ctx *ctx, int32_t stride_max);
FsTune fs_default_tune_without_coop(fs_ctx *ctx, int32_t stride_max);
/* 1 unless t is the cooperative tile and a view has more depths than its
 * event entries hold */
int fs_coop_depths_ok(const FsTune *t, int32_t max_n);
int32_t fs_plan_max_depths(const fs_plan *p);
int fs_tune_count(void);
int fs_tune_get(int i, int32_t out5[5]);

/* tuning cache (fs_tune.c) */
void fs_tune_cache_load(fs_ctx *ctx);
int fs_tune_lookup(fs_ctx *ctx, int32_t W, int32_t H, int32_t MH, int32_t MW, int32_t flags,
                   FsTune *out);
int fs_tune_lookup_key(fs_ctx *ctx, const char *key, FsTune *out);
FsTune fs_default_batch_tune(fs_ctx *ctx, int32_t stride_max);

#ifdef __cplusplus
}
#endif
#endif
