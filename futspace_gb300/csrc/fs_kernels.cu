/*
 * Small kernels around the renderer and the host-facing launch wrappers:
 *  - the per-view depth table (get_zs + get_h_line + inv_z, once per depth),
 *  - the shadowed-colour precompute of update_map,
 *  - the i32 -> u8 height mask of update_map,
 *  - dispatch of the render kernel over the four filter pairs.
 */
#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "fs_device.cuh"
#include "fs_render.cuh"

using namespace fsd;

extern "C" int fsk_render_h0c0(int, const FsLaunch *, const FsTune *, int, size_t, cudaStream_t,
                               int *);
extern "C" int fsk_render_h0c1(int, const FsLaunch *, const FsTune *, int, size_t, cudaStream_t,
                               int *);
extern "C" int fsk_render_h1c0(int, const FsLaunch *, const FsTune *, int, size_t, cudaStream_t,
                               int *);
extern "C" int fsk_render_h1c1(int, const FsLaunch *, const FsTune *, int, size_t, cudaStream_t,
                               int *);
extern "C" int fsk_segmin_h0(const FsLaunch *, const FsTune *, int, cudaStream_t);
extern "C" int fsk_segmin_h1(const FsLaunch *, const FsTune *, int, cudaStream_t);

namespace {

/* The depth table of one view (DepthLine per depth), then FS_ZPAD zero entries. */
__device__ __forceinline__ void ztable_fill(const FsView *Vp, float4 *zline, float *zinvz) {
  const int n = Vp->n;
  const DepthLine dl(*Vp);
  float4 *zl = zline + Vp->zoff;
  float *zi = zinvz + Vp->zoff;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n + FS_ZPAD;
       k += gridDim.x * blockDim.x) {
    float4 L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float iz = 0.0f;
    if (k < n) dl.entry(k, L, iz);
    zl[k] = L;
    zi[k] = iz;
  }
}

__global__ void ztable_kernel(const FsView *views, FsView view0, float4 *zline, float *zinvz) {
  allow_dependent_launch();
  ztable_fill(views ? views + blockIdx.y : &view0, zline, zinvz);
}

/* Serving launch prologue: record i of the packed launch goes to the session
 * table at ids[i], and its depth table is built. */
__global__ void serve_prepare_kernel(const FsView *packed, const int32_t *ids, FsView *sess,
                                     float4 *zline, float *zinvz) {
  allow_dependent_launch();
  const FsView *Vp = packed + blockIdx.y;
  if (blockIdx.x == 0 && threadIdx.x == 0) sess[ids[blockIdx.y]] = *Vp;
  ztable_fill(Vp, zline, zinvz);
}

/* generate_shadowmap_accumulated, fut/effects.fut:108-125, with the nearest
 * samplers of update_map (fut/interactive.fut:344-346). 1024x1024 output. */
__global__ void shadow_kernel(FsMapDev M, float s0, float s1, float s2, uint32_t *out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= 1024 || y >= 1024) return;
  const float fx = (float)x, fy = (float)y;
  const float step_size = 4.0f; /* f32(1024 / 256) */
  const float height = height_nearest(M, fx, fy);
  int count = 0;
  for (int dist = 1; dist < 256; dist++) {
    const float t = fm((float)dist, step_size);
    const float hx = fa(fx, fm(t, s0));
    const float hy = fa(fy, fm(t, s2));
    const float lhs = fs(fa(height, fm(t, s1)), height_nearest(M, hx, hy));
    if (lhs < -0.5f) count += 1;
  }
  const uint32_t black = 0xFF000000u; /* argb.black = from_rgba 0 0 0 1 */
  const DivChannels ch;
  out[(size_t)y * 1024 + x] = mix(ch, fm(step_size, (float)count), black, 1.0f,
                                  color_nearest(M, fx, fy));
}

__global__ void mask_kernel(const int32_t *in, uint8_t *out, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint8_t)(in[i] & 0xFF);
}

int queue_cap(int u) {
  const int raw = 31 + 32 * u;
  return raw <= 64 ? 64 : (raw <= 128 ? 128 : (raw <= 256 ? 256 : 512));
}

/* Height quads: q[y][x] = h[y][x] | h[y][x+1] << 8 | h[y+1][x] << 16 |
 * h[y+1][x+1] << 24, indices wrapped with Futhark's floored `%`. */
__global__ void quad_kernel(const uint8_t *h, uint32_t *q, int MH, int MW) {
  const int y = blockIdx.y;
  const int y1 = (y + 1) % MH;
  const uint8_t *r0 = h + (size_t)y * MW;
  const uint8_t *r1 = h + (size_t)y1 * MW;
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < MW; x += gridDim.x * blockDim.x) {
    const int x1 = (x + 1) % MW;
    q[(size_t)y * MW + x] = (uint32_t)r0[x] | ((uint32_t)r0[x1] << 8) | ((uint32_t)r1[x] << 16) |
                            ((uint32_t)r1[x1] << 24);
  }
}

typedef int (*render_entry)(int, const FsLaunch *, const FsTune *, int, size_t, cudaStream_t,
                            int *);

render_entry pick(int hf, int cf) {
  if (hf) return cf ? fsk_render_h1c1 : fsk_render_h1c0;
  return cf ? fsk_render_h0c1 : fsk_render_h0c0;
}

/* Gap-fill pass of split views: the reference's forward fill over the rows of
 * every column a segment flagged for painting the gap colour. A warp per
 * column; blockIdx.y is the view. */
__global__ void gapfill_kernel(const FsView *views, FsView view0) {
  const FsView *Vp = views ? views + blockIdx.y : &view0;
  if (Vp->nseg <= 1) return;
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int W = Vp->W, nseg = Vp->nseg;
  if (col >= W || !Vp->segbuf[(size_t)(nseg + 1) * W + col]) return;
  const int mf = Vp->segbuf[(size_t)nseg * W + col];
  uint32_t *oc = Vp->out + col;
  fill_column([oc, W](int y) { return oc + (size_t)y * W; }, mf, Vp->H, mf, Vp->gap, Vp->sky,
              lane);
}

/* Roofline denominator: reads a buffer that fits in L2 `reps` times with
 * L2-only loads (ld.global.cg), so after the first pass every sector comes
 * from L2. The XOR of everything read is stored only if it equals a constant,
 * which keeps the loads alive. */
__global__ void l2_read_kernel(const uint4 *buf, int64_t n16, int reps, uint32_t *sink) {
  uint32_t acc = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; r++)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
      const uint4 v = __ldcg(buf + i);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  if (acc == 0x9E3779B9u) sink[0] = acc;
}

}  // namespace

extern "C" int fsk_l2_read(const void *buf, int64_t bytes, int32_t reps, int32_t grid,
                           uint32_t *sink, cudaStream_t st) {
  if (bytes < 16 || reps < 1 || grid < 1) return (int)cudaErrorInvalidValue;
  l2_read_kernel<<<grid, 512, 0, st>>>(static_cast<const uint4 *>(buf), bytes / 16, reps, sink);
  return (int)cudaGetLastError();
}

/* The first row of a frame holding a non-sky pixel, top down: block (x, v)
 * scans rows [x*R, x*R + R) of view v (a thread per pixel, striding), skips
 * them when a row above is already known to hold one, and folds the first such
 * row into out[v]. */
constexpr int kSkyRowsPerBlock = 4;
__global__ void sky_rows_kernel(const FsView *views, FsView view0, int32_t *out) {
  const FsView &V = views ? views[blockIdx.y] : view0;
  int32_t *slot = out + (views ? blockIdx.y : 0);
  const int W = V.W, H = V.H;
  const int r0 = blockIdx.x * kSkyRowsPerBlock;
  if (r0 >= H) return;
  /* the row already known to hold a non-sky pixel, read once per warp so the
   * warp's reduction below has every lane */
  const int known = __shfl_sync(0xffffffffu, *(volatile int32_t *)slot, 0);
  if (r0 >= known) return;
  const int r1 = min(H, r0 + kSkyRowsPerBlock);
  const uint32_t sky = V.sky;
  const uint32_t *f = V.out + (size_t)r0 * W;
  const int n = (r1 - r0) * W;
  int first = INT_MAX;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (__ldcs(f + i) != sky) {
      first = r0 + i / W;
      break;
    }
  first = (int)__reduce_min_sync(0xffffffffu, (unsigned)first);
  if ((threadIdx.x & 31) == 0 && first != INT_MAX) atomicMin(slot, first);
}

extern "C" int fsk_sky_rows(const FsView *views_dev, const FsView *view0, int32_t nviews,
                            int32_t max_h, int32_t *out, cudaStream_t st) {
  if (nviews <= 0 || max_h <= 0) return (int)cudaSuccess;
  FsView v0;
  if (view0) v0 = *view0;
  else memset(&v0, 0, sizeof(v0));
  dim3 grid((max_h + kSkyRowsPerBlock - 1) / kSkyRowsPerBlock, views_dev ? nviews : 1);
  sky_rows_kernel<<<grid, 256, 0, st>>>(views_dev, v0, out);
  return (int)cudaGetLastError();
}

extern "C" int fsk_ztable(const FsView *views_dev, const FsView *view0, int32_t nviews,
                          int32_t max_n, float4 *zline, float *zinvz, cudaStream_t st) {
  if (nviews <= 0 || max_n <= 0) return (int)cudaSuccess;
  const int threads = 256;
  int bx = (max_n + threads - 1) / threads;
  if (bx > 64) bx = 64;
  FsView v0;
  if (view0) v0 = *view0;
  else memset(&v0, 0, sizeof(v0));
  dim3 grid(bx, views_dev ? nviews : 1);
  ztable_kernel<<<grid, threads, 0, st>>>(views_dev, v0, zline, zinvz);
  return (int)cudaGetLastError();
}

extern "C" int fsk_serve_prepare(const FsView *packed_dev, const int32_t *ids_dev, int32_t nb,
                                 int32_t max_n, FsView *sess_dev, float4 *zline, float *zinvz,
                                 cudaStream_t st) {
  if (nb <= 0 || max_n <= 0) return (int)cudaSuccess;
  int bx = (max_n + 255) / 256;
  if (bx > 64) bx = 64;
  serve_prepare_kernel<<<dim3(bx, nb), 256, 0, st>>>(packed_dev, ids_dev, sess_dev, zline, zinvz);
  return (int)cudaGetLastError();
}

extern "C" int fsk_tune_supported(const FsTune *t) {
#define FS_CASE(TW_, LC_, U_, STG_) \
  if (t->tw == TW_ && t->lc == LC_ && t->u == U_ && t->stage == STG_ && !t->smooth && !t->fx) return 1;
#define FS_CASE_M(TW_, LC_, U_, STG_, SM_, FX_)                                                \
  if (t->tw == TW_ && t->lc == LC_ && t->u == U_ && t->stage == STG_ && t->smooth == SM_ && \
      t->fx == FX_)                                                                         \
    return 1;
#define FS_CASE_C(TW_, TPC_, U_)                                                      \
  if (t->stage == 2 && t->tw == TW_ && t->lc == TPC_ && t->u == U_ && !t->smooth && !t->fx) \
    return 1;
#define FS_CASE_CF(TW_, TPC_, U_)                                                    \
  if (t->stage == 2 && t->tw == TW_ && t->lc == TPC_ && t->u == U_ && !t->smooth && t->fx) \
    return 1;
  FS_TUNE_LIST(FS_CASE)
  FS_TUNE_LIST_MODES(FS_CASE_M)
  FS_COOP_LIST(FS_CASE_C)
  FS_COOP_LIST_FX(FS_CASE_CF)
#undef FS_CASE
#undef FS_CASE_M
#undef FS_CASE_C
#undef FS_CASE_CF
  return 0;
}

extern "C" size_t fsk_render_smem(const FsTune *t, int32_t stride_max) {
  /* the cooperative tile: fixed part, stage and event list; taller frames
   * than its event entries hold never fit */
  if (t->stage == 2 && stride_max > FS_COOP_MAX_ROWS) return (size_t)1 << 40;
#define FS_COOP_SMEM(TW_, TPC_, U_)                                  \
  if (t->stage == 2 && t->tw == TW_ && t->lc == TPC_ && t->u == U_) \
    return CoopShape<TW_, TPC_, U_>::fixed_bytes + CoopShape<TW_, TPC_, U_>::tile_bytes(stride_max);
  FS_COOP_LIST(FS_COOP_SMEM)
#undef FS_COOP_SMEM
  /* must match RenderShape<...>::fixed_bytes + stage */
  const size_t nw = (size_t)t->tw * t->lc / 32;
  const size_t box = t->stage ? 2ull * kBoxRows * t->tw * 4 : 0;
  const size_t stage = t->stage ? (size_t)t->tw * stride_max * 4 : 0;
  return box + nw * queue_cap(t->u) * 8 * (t->smooth ? 2 : 1) + 256 * 4 + (t->stage ? 16 : 0) +
         stage;
}

/* Screen columns per work item: a CTA tile with the shared-memory stage (and
 * the cooperative tile), a warp strip with direct painting. */
extern "C" int32_t fsk_item_width(const FsTune *t) { return t->stage ? t->tw : 32 / t->lc; }

/* Work items one CTA takes at a time (warps per CTA with direct painting). */
extern "C" int32_t fsk_items_per_cta(const FsTune *t) {
  return t->stage ? 1 : t->tw * t->lc / 32;
}

/* Level 1 of the max pyramid: each cell is the maximum of the 2x2 texels that
 * quad (2y, 2x) packs. */
__global__ void pyr1_kernel(const uint32_t *q, int MW, uint8_t *out, int ch, int cw) {
  const int y = blockIdx.y;
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < cw; x += gridDim.x * blockDim.x) {
    const uint32_t v = q[(size_t)(2 * y) * MW + 2 * x];
    const uint32_t a = max(v & 0xFFu, (v >> 8) & 0xFFu), b = max((v >> 16) & 0xFFu, v >> 24);
    out[(size_t)y * cw + x] = (uint8_t)max(a, b);
  }
}

/* Level l+1 from level l: maximum of 2x2 cells. */
__global__ void pyr_kernel(const uint8_t *in, int iw, uint8_t *out, int ch, int cw) {
  const int y = blockIdx.y;
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < cw; x += gridDim.x * blockDim.x) {
    const uint8_t *r0 = in + (size_t)(2 * y) * iw + 2 * x;
    const uint8_t *r1 = r0 + iw;
    out[(size_t)y * cw + x] = (uint8_t)max(max(r0[0], r0[1]), max(r1[0], r1[1]));
  }
}

extern "C" size_t fs_pyramid_layout(FsMapDev *M) {
  M->pyr = nullptr;
  M->pyr_levels = 0;
  if (!M->pow2 || M->MH < 4 || M->MW < 4) return 0;
  size_t off = 0;
  int l = 1;
  for (; l <= FS_PYR_MAX && (M->MH >> l) >= 1 && (M->MW >> l) >= 1; l++) {
    M->pyr_off[l - 1] = (int32_t)off;
    off += (size_t)(M->MH >> l) * (size_t)(M->MW >> l);
  }
  M->pyr_levels = l - 1;
  return off;
}

extern "C" int fsk_build_pyramid(const FsMapDev *M, uint8_t *pyr, cudaStream_t st) {
  for (int l = 1; l <= M->pyr_levels; l++) {
    const int ch = M->MH >> l, cw = M->MW >> l;
    const int bx = cw < 256 ? 1 : (cw / 256 > 16 ? 16 : cw / 256);
    if (l == 1)
      pyr1_kernel<<<dim3(bx, ch), 256, 0, st>>>(M->q, M->MW, pyr + M->pyr_off[0], ch, cw);
    else
      pyr_kernel<<<dim3(bx, ch), 256, 0, st>>>(pyr + M->pyr_off[l - 2], M->MW >> (l - 1),
                                               pyr + M->pyr_off[l - 1], ch, cw);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
  }
  return (int)cudaSuccess;
}

extern "C" int fsk_build_quads(const uint8_t *h, uint32_t *q, int32_t MH, int32_t MW,
                               cudaStream_t st) {
  if (MH <= 0 || MW <= 0) return (int)cudaErrorInvalidValue;
  int bx = (MW + 255) / 256;
  if (bx > 16) bx = 16;
  quad_kernel<<<dim3(bx, MH), 256, 0, st>>>(h, q, MH, MW);
  return (int)cudaGetLastError();
}

extern "C" int fsk_render(const FsLaunch *L, const FsTune *t, int32_t hf, int32_t cf,
                          int32_t grid, cudaStream_t st) {
  if (grid <= 0) return (int)cudaSuccess;
  return pick(hf, cf)(0, L, t, grid, fsk_render_smem(t, L->stride_max), st, nullptr);
}

/* The same launch with programmatic stream serialization: it may start while
 * the kernel before it on the stream runs, and waits for it in the kernel. */
extern "C" int fsk_render_pdl(const FsLaunch *L, const FsTune *t, int32_t hf, int32_t cf,
                              int32_t grid, cudaStream_t st) {
  if (grid <= 0) return (int)cudaSuccess;
  return pick(hf, cf)(2, L, t, grid, fsk_render_smem(t, L->stride_max), st, nullptr);
}

extern "C" int fsk_gapfill(const FsView *views_dev, const FsView *view0, int32_t nviews,
                           int32_t max_w, cudaStream_t st) {
  if (nviews <= 0 || max_w <= 0) return (int)cudaSuccess;
  FsView v0;
  if (view0) v0 = *view0;
  else memset(&v0, 0, sizeof(v0));
  dim3 grid((max_w + 7) / 8, views_dev ? nviews : 1);
  gapfill_kernel<<<grid, 256, 0, st>>>(views_dev, v0);
  return (int)cudaGetLastError();
}

extern "C" int fsk_segmin(const FsLaunch *L, const FsTune *t, int32_t hf, int32_t grid,
                          cudaStream_t st) {
  if (grid <= 0) return (int)cudaSuccess;
  return (hf ? fsk_segmin_h1 : fsk_segmin_h0)(L, t, grid, st);
}

extern "C" int fsk_render_max_ctas_per_sm(const FsTune *t, int32_t hf, int32_t cf,
                                          int32_t stride_max, int32_t *out) {
  int occ = 0;
  const int e = pick(hf, cf)(1, nullptr, t, 0, fsk_render_smem(t, stride_max), 0, &occ);
  *out = occ;
  return e;
}

extern "C" int fsk_shadowmap(const FsMapDev *map, const float sun[3], uint32_t *out,
                             cudaStream_t st) {
  dim3 grid(1024 / 128, 1024);
  shadow_kernel<<<grid, 128, 0, st>>>(*map, sun[0], sun[1], sun[2], out);
  return (int)cudaGetLastError();
}

extern "C" int fsk_mask_heights(const int32_t *in, uint8_t *out, int64_t count,
                                cudaStream_t st) {
  if (count <= 0) return (int)cudaSuccess;
  int64_t blocks = (count + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  mask_kernel<<<(int)blocks, 256, 0, st>>>(in, out, count);
  return (int)cudaGetLastError();
}
