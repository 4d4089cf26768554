/*
 * Internal types shared by the C host code (fs_host.c, fs_serve.c) and the CUDA
 * kernels (fs_kernels.cu). Plain C11 layout: no C++ in here.
 */
#ifndef FS_INTERNAL_H
#define FS_INTERNAL_H

#include <cuda.h>
#include <cuda_runtime_api.h>
#include <stdint.h>

#include "../../include/futspace_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Largest screen height the column stage supports (rows are packed in 16 bits
 * in the per-warp event queues). */
#define FS_MAX_ROWS 16383
/* Largest depth-sample count per view (depth index packed in 20 bits). */
#define FS_MAX_DEPTHS (1 << 20)
/* Largest texel count of a map (the kernels index texels with 32-bit ints). */
#define FS_MAX_TEXELS (1ll << 30)
/* Readable depth-table entries past the n samples of every view's slice: the
 * render kernel loads whole chunks of depths (at most FS_ZPAD) without a bound
 * check and discards the rows of depths past n. The entries are zeros. */
#define FS_ZPAD 64
/* Limits of the cooperative tile's 32-bit event entries (pack_coop_event in
 * fs_render.cuh): depths per view, screen rows. Views beyond them render with
 * the other kernel forms. */
#define FS_COOP_MAX_DEPTHS (1 << 17)
#define FS_COOP_MAX_ROWS 4095
/* Maps bound to one launch. */
#define FS_MAX_MAPS 4
/* Levels of the height max pyramid (2^16 texels per side). */
#define FS_PYR_MAX 16

/* Flags of a view. */
#define FSV_HEIGHT_BILINEAR 1
#define FSV_COLOR_BILINEAR 2
#define FSV_SHADE 4 /* FS_FX_SHADE epilogue */
#define FSV_FOG 8   /* FS_FX_FOG epilogue */
#define FSV_SMOOTH 16 /* `#on` smoothing */

/* One view (camera + screen) as the kernels read it. 128 bytes. */
typedef struct {
  float cam_x, cam_y, cam_h, horizon;
  float sa, ca, fov, scale; /* sin/cos of the yaw from the host C library */
  float d, z0;
  int32_t W, H;
  int32_t n, map;
  uint32_t sky, gap;
  uint32_t *out;    /* frame base in device memory, row-major H x W */
  int64_t zoff;     /* first z-table entry of this view */
  int32_t tmap;     /* index into the tensor-map array, -1: plain stores */
  int32_t flags;    /* FSV_* */
  float distance;   /* draw distance D (depth shading) */
  float shade, fog_start, fog_end;
  uint32_t fog_color;
  /* depth segments (direct painting only): the column's depth schedule split
   * into nseg ranges of seglen samples, each marched by its own work item;
   * segbuf holds [nseg + 2][W] ints: the minimum row of each segment but the
   * last, the column's final minimum row, and gap-colour flags */
  int32_t nseg;
  int32_t *segbuf;
  int32_t seglen;
  int32_t pad1;
} FsView;

/* One height/colour map pair resident in device memory. Heights are stored as
 * 2x2 quads: q[y][x] packs the u8 heights of (y,x), (y,x+1), (y+1,x) and
 * (y+1,x+1) (indices wrapped) in bytes 0..3, so one 4-byte gather yields the
 * whole bilinear footprint; byte 0 alone is the nearest sample. */
typedef struct {
  const uint32_t *q;  /* [MH][MW] height quads */
  const uint32_t *c;  /* [CH][CW] ARGB colours */
  int32_t MH, MW;     /* height map rows, columns */
  int32_t CH, CW;     /* colour map rows, columns (the interactive app samples a
                         1024x1024 shadowed colour map over any height map) */
  int32_t pow2;       /* MH and MW are powers of two: wrap with a mask */
  int32_t cpow2;      /* CH and CW are powers of two */
  /* Max pyramid of the heights (power-of-two maps only; NULL: none). Level l
   * (1..pyr_levels) has (MH>>l) x (MW>>l) u8 cells, each the maximum height of
   * its 2^l x 2^l texels, stored at pyr + pyr_off[l-1]. */
  const uint8_t *pyr;
  int32_t pyr_levels;
  int32_t pyr_off[FS_PYR_MAX];
} FsMapDev;

/* Everything one render launch needs, passed by value (__grid_constant__), so
 * a single-view launch touches no host-written device memory. */
typedef struct {
  CUtensorMap tmap0;           /* frame tensor map of view0 (when tmap == 0 and views == NULL) */
  FsView view0;                /* the view when views == NULL */
  FsMapDev maps[FS_MAX_MAPS];
  const FsView *views;         /* NULL: single view0 */
  const int64_t *items;        /* work items (FS_ITEM); NULL: item i of view0 is segment
                                * i / ntiles, tile i % ntiles */
  const CUtensorMap *tmaps;    /* tensor maps of `views` */
  const float4 *zline;         /* per depth: x0, y0, dx, dy */
  const float *zinvz;          /* per depth: inv_z */
  int32_t *head;               /* persistent work counter; NULL: one item per CTA */
  unsigned long long *stats;   /* optional counters: samples, events; NULL: off */
  int32_t nitems;
  int32_t stride_max;          /* stage column stride (>= max H, odd) */
  int32_t pad[2];
} FsLaunch;

/* Launch configuration of the render kernel (the autotuned knobs). */
typedef struct {
  int32_t tw;    /* column-tile width: columns per CTA */
  int32_t lc;    /* lanes per column (32: one warp per column) */
  int32_t u;     /* depth samples per lane per chunk: chunk = lc * u depths */
  int32_t stage; /* 0: direct painting; 1: shared-memory column stage + TMA store;
                  * 2: cooperative tile (lc = threads per column) */
  int32_t ctas;  /* persistent CTAs (0: as many as fit) */
  int32_t smooth; /* 1: the `#on` smoothing kernels (FS_TUNE_LIST_SM) */
  int32_t fx;     /* 1: kernels with the shading / fog epilogue compiled in */
  int32_t seg;    /* 1: kernels that read depth segments (some view is split) */
} FsTune;

/* Kernel-side entry points (fs_kernels.cu). Each returns a cudaError_t. */
int fsk_ztable(const FsView *views_dev, const FsView *view0, int32_t nviews, int32_t max_n,
               float4 *zline, float *zinvz, cudaStream_t st);
int fsk_render(const FsLaunch *L, const FsTune *t, int32_t hf, int32_t cf, int32_t grid,
               cudaStream_t st);
int fsk_render_pdl(const FsLaunch *L, const FsTune *t, int32_t hf, int32_t cf, int32_t grid,
                   cudaStream_t st);
int fsk_serve_prepare(const FsView *packed_dev, const int32_t *ids_dev, int32_t nb, int32_t max_n,
                      FsView *sess_dev, float4 *zline, float *zinvz, cudaStream_t st);
size_t fsk_render_smem(const FsTune *t, int32_t stride_max);
int fsk_render_max_ctas_per_sm(const FsTune *t, int32_t hf, int32_t cf, int32_t stride_max,
                               int32_t *out);
int fsk_tune_supported(const FsTune *t);
int32_t fsk_item_width(const FsTune *t);
int fsk_segmin(const FsLaunch *L, const FsTune *t, int32_t hf, int32_t grid, cudaStream_t st);
int fsk_gapfill(const FsView *views_dev, const FsView *view0, int32_t nviews, int32_t max_w,
                cudaStream_t st);
int32_t fsk_items_per_cta(const FsTune *t);
int fsk_l2_read(const void *buf, int64_t bytes, int32_t reps, int32_t grid, uint32_t *sink,
                cudaStream_t st);
/* Per view, into out[v] (set to INT32_MAX beforehand): the smallest row index
 * holding a pixel other than the view's sky value, so rows [0, min(out, H))
 * of its frame are all sky. Views from views_dev (nviews of them), or view0. */
int fsk_sky_rows(const FsView *views_dev, const FsView *view0, int32_t nviews, int32_t max_h,
                 int32_t *out, cudaStream_t st);
/* A work item names a view (or serving session), a depth segment and a column
 * tile (shared-memory stage) or strip (direct painting). */
#define FS_ITEM_VIEWS 32768
#define FS_ITEM_TILES 65536
#define FS_MAX_SEGMENTS 32
#define FS_ITEM(view, seg, tile) (((int64_t)(view) << 40) | ((int64_t)(seg) << 32) | (int64_t)(tile))
#define FS_ITEM_VIEW(it) ((int32_t)((it) >> 40))
#define FS_ITEM_SEG(it) ((int32_t)(((it) >> 32) & 0xFF))
#define FS_ITEM_TILE(it) ((int32_t)((it)&0xFFFFFFFF))
int fsk_shadowmap(const FsMapDev *map, const float sun[3], uint32_t *out, cudaStream_t st);
int fsk_mask_heights(const int32_t *in, uint8_t *out, int64_t count, cudaStream_t st);
int fsk_build_quads(const uint8_t *h, uint32_t *q, int32_t MH, int32_t MW, cudaStream_t st);
/* Builds the max pyramid of M (M->q, MH, MW set; pyr, levels, offsets filled). */
int fsk_build_pyramid(const FsMapDev *M, uint8_t *pyr, cudaStream_t st);
/* Bytes of the max pyramid of a map; fills levels and offsets into *M. 0 when
 * the map is not power-of-two sized. */
size_t fs_pyramid_layout(FsMapDev *M);

#ifdef __cplusplus
}
#endif
#endif
