/*
 * The voxel-space column renderer (fut/voxel_renderer.fut:214-251, `#off`).
 *
 * Work items: with the shared-memory stage (STG = 1) an item is (view, tile of
 * TW screen columns) and one CTA renders it; with direct painting (STG = 0)
 * an item is (view, strip of 32/LC columns) and one warp renders it, with no
 * CTA barrier between items. With a work counter the CTAs (warps) are
 * persistent and pull items until the queue is empty, so views of uneven size
 * and depth share one launch.
 *
 * Lanes: each screen column is marched by LC lanes of a warp (32/LC columns
 * per warp). A chunk covers LC*U consecutive depths; at step u the LC lanes of
 * a column take depths k0 + u*LC + 0..LC-1, so every gather instruction covers
 * a compact patch of the map (LC consecutive depths x 32/LC neighbouring
 * columns). For each sample the lanes gather the height quad, project the
 * height to a screen row in f32 and clamp it to [0, H].
 *
 * Occlusion: the reference's inclusive `occlude` scan keeps the nearer sample
 * on ties (:69-72), the scatter writes a colour at every new minimum row (:244)
 * and the forward fill (:246) paints each row with the nearest sample whose row
 * lies at or above it. So a sample is an EVENT iff its row is strictly below the
 * running minimum row of its column, and it paints rows [row, previous minimum).
 * A segmented warp scan (__shfl_up_sync) over the LC lanes gives each sample the
 * running minimum before it. Rows >= H are never events, and once the minimum
 * reaches row 0 no later sample can be one, so the column stops early without
 * changing a pixel.
 *
 * Colours are needed only for events: they go to a warp-private ring in shared
 * memory and are coloured 32 at a time (all lanes busy). Painting then takes one
 * of two forms (template STG):
 *  STG = 1: into a column stage in shared memory (column-major, odd stride: no
 *           bank conflicts when painting a column or reading a row across
 *           columns); after the march each column gets the reference's gap fill
 *           and sky, and the tile is transposed through a row-major box buffer
 *           and written with TMA bulk tensor stores (cp.async.bulk.tensor.2d),
 *           32 rows per box, double buffered.
 *  STG = 0: straight into the frame in global memory (tiny shared-memory
 *           footprint, full occupancy); the warp then writes its columns' sky
 *           rows, a row per store instruction, and re-runs the gap fill over a
 *           column that painted the gap colour.
 * A third kernel, the cooperative tile (coop_kernel, tuning stage 2, at the
 * end of this file), marches all depths of a column tile at once for frames
 * with too few columns to keep the GPU busy.
 */
#pragma once
#include "fs_device.cuh"

namespace fsd {

template <int U>
struct QueueCap {
  static constexpr int raw = 31 + 32 * U;
  static constexpr int value = raw <= 64 ? 64 : (raw <= 128 ? 128 : (raw <= 256 ? 256 : 512));
  static_assert(raw <= value, "ring too small for 31 waiting events plus one chunk");
};

constexpr int kBoxRows = 32;

/* Queue entry: depth index (20 bits) | item column (7) | row (16) | prev (16). */
__device__ __forceinline__ unsigned long long pack_event(int k, int col, int row, int prev) {
  return ((unsigned long long)(uint32_t)k << 39) | ((unsigned long long)(uint32_t)col << 32) |
         ((unsigned long long)(uint32_t)row << 16) | (unsigned long long)(uint32_t)prev;
}

/* Depth-table entry of depth k (z = z_{k+1}) of one view: get_zs
 * (fut/voxel_renderer.fut:34), get_h_line (:43-60) and inv_z = (1/z) * scale
 * (:217), which the reference evaluates once per depth slice in its outer map
 * (:215-217). L = {left_x + cam_x, left_y + cam_y, dx, dy}. */
struct DepthLine {
  float a1, a2, a3, a4, fw, d, z0, cam_x, cam_y, scale;
  __device__ __forceinline__ explicit DepthLine(const FsView &V)
      : a1(fs(-V.ca, fm(V.sa, V.fov))), /* left_x / z  */
        a2(fs(V.sa, fm(V.ca, V.fov))),  /* left_y / z  */
        a3(fs(V.ca, fm(V.sa, V.fov))),  /* right_x / z */
        a4(fs(-V.sa, fm(V.ca, V.fov))), /* right_y / z */
        fw((float)V.W),
        d(V.d),
        z0(V.z0),
        cam_x(V.cam_x),
        cam_y(V.cam_y),
        scale(V.scale) {}
  __device__ __forceinline__ void entry(int k, float4 &L, float &iz) const {
    const float fi = (float)(k + 1);
    const float z = fm(fd(fi, 2.0f), fa(fm(2.0f, z0), fm(fs(fi, 1.0f), d)));
    const float lx = fm(a1, z), ly = fm(a2, z), rx = fm(a3, z), ry = fm(a4, z);
    L = make_float4(fa(lx, cam_x), fa(ly, cam_y), fd(fs(rx, lx), fw), fd(fs(ry, ly), fw));
    iz = fm(fd(1.0f, z), scale);
  }
};

__device__ __forceinline__ void fence_proxy_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *tm, const void *src, int x, int y) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(src);
  asm volatile(
      "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
          (unsigned long long)tm),
      "r"(s), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

/* Programmatic dependent launch: a render kernel launched with programmatic
 * stream serialization may start while the kernel before it (the depth table,
 * the serving prologue, the segment pass) still runs; it waits here, before
 * its first read of anything that kernel writes. Without that launch
 * attribute the wait returns at once. */
__device__ __forceinline__ void wait_prior_grid() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
/* Lets the dependent grid launch before this one finishes. */
__device__ __forceinline__ void allow_dependent_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

/* fill_vline scan + sky (fut/voxel_renderer.fut:78-81, 246-248) over rows
 * [y_begin, H) of one column, one warp, 32 rows per step. `at(y)` addresses row
 * y. Rows above the column's final minimum row `mf` were never painted and
 * hold the gap value. */
template <class At>
__device__ __forceinline__ void fill_column(At at, int y_begin, int H, int mf, uint32_t gap,
                                            uint32_t sky, int lane) {
  unsigned lemask;
  asm("mov.u32 %0, %%lanemask_le;" : "=r"(lemask));
  uint32_t carry = gap;
  for (int y0 = y_begin; y0 < H; y0 += 32) {
    const int y = y0 + lane;
    uint32_t v = gap;
    if (y < H && y >= mf) v = *at(y);
    const unsigned nz = __ballot_sync(FS_FULL_MASK, v != gap);
    const unsigned le = nz & lemask;
    const int src = le ? 31 - __clz(le) : 0;
    const uint32_t t = __shfl_sync(FS_FULL_MASK, v, src);
    const uint32_t val = le ? t : carry;
    if (y < H) *at(y) = (val == gap) ? sky : val;
    if (nz) carry = __shfl_sync(FS_FULL_MASK, v, 31 - __clz(nz));
  }
}

template <int TW, int LC, int U, int STG, int SM = 0>
struct RenderShape {
  static constexpr int NT = TW * LC;
  static constexpr int NW = NT / 32;
  static constexpr int CPW = 32 / LC;
  static constexpr int QCAP = QueueCap<U>::value;
  static constexpr int QW = SM ? 2 : 1; /* 8-byte words per queue entry */
  static constexpr size_t box_bytes = STG ? 2ull * kBoxRows * TW * 4 : 0;
  static constexpr size_t queue_bytes = (size_t)NW * QCAP * 8 * QW;
  static constexpr size_t lut_bytes = 256 * 4;
  static constexpr size_t item_bytes = STG ? 16 : 0; /* the CTA's next item */
  static constexpr size_t fixed_bytes = box_bytes + queue_bytes + lut_bytes + item_bytes;
  /* direct painting keeps 64 registers per thread so 32 warps fit per SM:
   * the march is bound by gather latency, and occupancy hides it */
  static constexpr int min_blocks = STG ? 1 : (NT >= 1024 ? 1 : 1024 / NT);
};

/* SM = 1: the `#on` smoothing branch (fut/voxel_renderer.fut:175-213). Its
 * scatter writes, at every prefix-minimum row, the tuple of the LAST sample
 * holding that minimum (a sequential scatter: later writes win), so an event's
 * rows blend with the previous event's colour only when the event held the
 * minimum for a single sample (the next sample is an event too, or it is the
 * last sample) and the previous event is the sample just before it (or there
 * is none and the event is sample 1). The blend of row y in [row, prev) is
 * mix(|row - y| / range, previous colour, |y - prev| / range, colour) with
 * range = max(1, prev - row); colour 0 becomes sky, with no gap fill.
 * Compiled for one lane per column and direct painting only.
 * FX = 1: the optional shading / fog epilogue (views with FSV_SHADE/FSV_FOG).
 * SEG = 1: direct painting of views split into depth segments (reads the
 * segment-minimum rows; a separate instantiation so the common kernel keeps
 * its registers). */
template <bool B>
struct BoolTag {
  static constexpr bool value = B;
};

/* What one warp needs to march the columns of an item, held in registers: the
 * view's fields (the frame stores below may alias the view records as far as
 * the compiler can tell, so nothing is re-read), the map and the depth table. */
template <int LC, int U, int HF>
struct Marcher {
  static constexpr int CH = LC * U;
  const FsMapDev &M; /* read in place: no local copy to index */
  HeightMap hmap;
  const float4 *zl;
  const float *zi;
  float cam_h, horizon, fcol;
  int H;

  __device__ __forceinline__ Marcher(const FsLaunch &P, const FsView *Vp, int col)
      : M(P.maps[Vp->map]),
        hmap{P.maps[Vp->map].q, P.maps[Vp->map].MW, P.maps[Vp->map].MH},
        zl(P.zline + Vp->zoff),
        zi(P.zinvz + Vp->zoff),
        cam_h(Vp->cam_h),
        horizon(Vp->horizon),
        fcol((float)col),
        H(Vp->H) {}

  /* screen row of depth sample k of this lane's column, clamped to [0, H] */
  template <bool P2>
  __device__ __forceinline__ int row(int k) const {
    const float4 L = __ldg(zl + k);
    const float2 xy = axpy2(fcol, make_float2(L.z, L.w), make_float2(L.x, L.y));
    const float hh =
        HF ? height_bilinear<P2>(hmap, xy.x, xy.y) : height_nearest<P2>(hmap, xy.x, xy.y);
    return min(max(f2i(fa(fm(fs(cam_h, hh), __ldg(zi + k)), horizon)), 0), H);
  }
};

/* Depth range [k_begin, k_end) of segment `seg` of a view with n samples. */
__device__ __forceinline__ void segment_range(const FsView *Vp, int seg, int &k_begin,
                                              int &k_end) {
  if (Vp->nseg > 1) {
    k_begin = seg * Vp->seglen;
    k_end = min(k_begin + Vp->seglen, Vp->n);
  } else {
    k_begin = 0;
    k_end = Vp->n;
  }
}

/* Exact skip bound: rows are monotone in the height and in inv_z, so a row
 * computed from an upper bound of every height the samples of columns
 * [cf, cl] at depths [ka, kb] can read, at the nearest or farthest of those
 * depths, bounds every such sample's row from below. Sample coordinates are
 * bilinear in (column, depth along the view line), so the four corner samples
 * bound the box. A chunk whose bound is not above any of the strip's running
 * minima holds no event. (Power-of-two maps with a max pyramid only.) */
__device__ __forceinline__ int box_row_bound(const FsMapDev &M, float4 La, float iza, float4 Lb,
                                             float izb, float cam_h, float horizon, int H,
                                             float cf, float cl) {
  const float2 a0 = axpy2(cf, make_float2(La.z, La.w), make_float2(La.x, La.y));
  const float2 a1 = axpy2(cl, make_float2(La.z, La.w), make_float2(La.x, La.y));
  const float2 b0 = axpy2(cf, make_float2(Lb.z, Lb.w), make_float2(Lb.x, Lb.y));
  const float2 b1 = axpy2(cl, make_float2(Lb.z, Lb.w), make_float2(Lb.x, Lb.y));
  const float x0 = fminf(fminf(a0.x, a1.x), fminf(b0.x, b1.x));
  const float x1 = fmaxf(fmaxf(a0.x, a1.x), fmaxf(b0.x, b1.x));
  const float y0 = fminf(fminf(a0.y, a1.y), fminf(b0.y, b1.y));
  const float y1 = fmaxf(fmaxf(a0.y, a1.y), fmaxf(b0.y, b1.y));
  const float dh = fs(cam_h, fa((float)box_max_height(M, x0, x1, y0, y1), 1.0f));
  const int ra = min(max(f2i(fa(fm(dh, iza), horizon)), 0), H);
  const int rb = min(max(f2i(fa(fm(dh, izb), horizon)), 0), H);
  return min(ra, rb);
}

/* The same bound for depths [ka, kb] of a view's depth table. */
__device__ __forceinline__ int chunk_row_bound(const FsMapDev &M, const float4 *zl,
                                               const float *zi, float cam_h, float horizon,
                                               int H, float cf, float cl, int ka, int kb) {
  return box_row_bound(M, __ldg(zl + ka), __ldg(zi + ka), __ldg(zl + kb), __ldg(zi + kb), cam_h,
                       horizon, H, cf, cl);
}

/* Skip bounds of 32 chunks at a time: lane j holds the bound of the chunk
 * that starts at depth base + j * CH, so one pass of the bound arithmetic
 * serves 32 chunks; each chunk then costs a shuffle and a max-reduction.
 * [wfirst, wlast] are the warp's screen columns. */
template <int CH>
struct ChunkBounds {
  int bound = 0;
  int base = -(1 << 30); /* first depth of lane 0's chunk */
  /* true when the chunk [kc, kc + CH) of a march ending at k_end can be skipped */
  __device__ __forceinline__ bool skip(const FsMapDev &M, const float4 *zl, const float *zi,
                                       float cam_h, float horizon, int H, int wfirst, int wlast,
                                       int kc, int k_end, int m, int lane) {
    if (kc >= base + 32 * CH) {
      base = kc;
      const int ka = kc + lane * CH;
      bound = H + 1; /* past the end: never consulted */
      if (ka < k_end)
        bound = chunk_row_bound(M, zl, zi, cam_h, horizon, H, (float)wfirst, (float)wlast, ka,
                                min(ka + CH, k_end) - 1);
    }
    const int b = __shfl_sync(FS_FULL_MASK, bound, (kc - base) / CH);
    return b >= (int)__reduce_max_sync(FS_FULL_MASK, (unsigned)m);
  }
};

/* Per-warp work of one item: the march over the depth chunks of [k_begin,
 * k_end), the event ring, colouring and painting. Both kernel layouts call it;
 * `cl` is the lane's column within the item, `c0` the item's first screen
 * column, `m_init` the column's minimum row before k_begin. On return `m`
 * holds the column's minimum row after k_end and `gapcols` (direct painting)
 * has bit c set when column c painted the gap colour. */
template <int TW, int LC, int U, int HF, int CF, int STG, int SM, int FX>
__device__ __forceinline__ void render_strip(const FsLaunch &P, const FsView *Vp, int c0, int cl,
                                             int lane, unsigned lanemask_lt,
                                             unsigned long long *q, uint32_t *stage,
                                             const LutChannels &chan, int k_begin, int k_end,
                                             int m_init, int &m_out, uint32_t &gapcols,
                                             uint32_t &n_samples, uint32_t &n_events) {
  using S = RenderShape<TW, LC, U, STG, SM>;
  constexpr int CH = LC * U;
  constexpr int QCAP = S::QCAP;
  const int dl = lane % LC;
  const int W = Vp->W, H = Vp->H, n = Vp->n;
  const uint32_t sky = Vp->sky, gap = Vp->gap;
  const int vflags = Vp->flags;
  uint32_t *const out = Vp->out;
  const int stride = H | 1;
  const int col = c0 + cl;
  const bool valid = col < W;
  const float cam_h = Vp->cam_h, horizon = Vp->horizon;
  const FsMapDev &M = P.maps[Vp->map]; /* read in place: no local copy to index */
  const HeightMap hmap{M.q, M.MW, M.MH};
  const bool p2 = M.pow2 != 0;
  const float4 *zl = P.zline + Vp->zoff;
  const float *zi = P.zinvz + Vp->zoff;
  const float fcol = (float)col;

  /* running minimum row of this column; 0 also marks a column past the
   * frame's right edge, which never has an event */
  int m = valid ? m_init : 0;
  int qh = 0, qt = 0; /* ring head / tail, warp-uniform */
  uint32_t gapbits = 0;
  /* smoothing: the last event of this lane's column, queued once the sample
   * after it shows whether it held the minimum for a single sample */
  int pend_k = -1, pend_r = 0, pend_p = 0, pend_kprev = -1;

  /* colour of depth sample k of item column ecl (with the optional epilogue) */
  auto sample_colour = [&](int k, int ecl) -> uint32_t {
    const float ec = (float)(c0 + ecl);
    const float4 L = __ldg(zl + k);
    const float2 xy = axpy2(ec, make_float2(L.z, L.w), make_float2(L.x, L.y));
    uint32_t colour = color_sample<CF>(M, chan, M.cpow2 != 0, xy.x, xy.y);
    if constexpr (FX) {
      if (vflags & (FSV_SHADE | FSV_FOG)) {
        /* depth of sample k, as the depth table computes it */
        const float fi = (float)(k + 1);
        const float z = fm(fd(fi, 2.0f), fa(fm(2.0f, Vp->z0), fm(fs(fi, 1.0f), Vp->d)));
        colour = apply_effects(chan, *Vp, colour, z);
      }
    }
    return colour;
  };

  /* screen row of depth sample k of this lane's column, clamped to [0, H] */
  auto sample_row = [&](auto p2tag, int k) -> int {
    constexpr bool P2 = decltype(p2tag)::value;
    const float4 L = __ldg(zl + k);
    const float2 xy = axpy2(fcol, make_float2(L.z, L.w), make_float2(L.x, L.y));
    const float hh =
        HF ? height_bilinear<P2>(hmap, xy.x, xy.y) : height_nearest<P2>(hmap, xy.x, xy.y);
    return min(max(f2i(fa(fm(fs(cam_h, hh), __ldg(zi + k)), horizon)), 0), H);
  };

  /* colour the queued events [qh, qh+cnt) and paint their intervals */
  auto drain = [&](int cnt) {
    uint32_t gb = 0;
    if (lane < cnt) {
      const int slot = (qh + lane) & (QCAP - 1);
      const unsigned long long e = q[slot * S::QW];
      const int k = (int)(e >> 39);
      const int ecl = (int)((e >> 32) & 127u);
      const int er = (int)((e >> 16) & 0xFFFFu);
      const int ep = (int)(e & 0xFFFFu);
      const uint32_t colour = sample_colour(k, ecl);
      if (SM) {
        const unsigned long long e1 = q[slot * S::QW + S::QW - 1];
        const int kprev = (int)(e1 & 0x1FFFFFu) - 1; /* previous event, -1: none */
        const bool blend = ((e1 >> 32) & 1u) != 0;
        uint32_t cprev = 0u;                         /* the scan's neutral colour */
        if (blend && kprev >= 0) cprev = sample_colour(kprev, ecl);
        const float range = fmaxf(1.0f, (float)(ep - er));
        uint32_t *o = out + (size_t)er * W + c0 + ecl;
        for (int yy = er; yy < ep; yy++, o += W) {
          uint32_t c = colour;
          if (blend) {
            const float d1 = fd(fabsf(fs((float)yy, (float)ep)), range);
            const float d2 = fd(fabsf(fs((float)er, (float)yy)), range);
            c = mix(chan, d2, cprev, d1, colour);
          }
          __stcs(o, c == 0u ? sky : c);
        }
      } else if (STG) {
        uint32_t *sc = stage + ecl * stride;
        for (int yy = er; yy < ep; yy++) sc[yy] = colour;
      } else {
        /* most intervals are a few rows: the first four stores are predicated
         * straight-line code, the rest a loop */
        uint32_t *o = out + (size_t)er * W + c0 + ecl;
        const int len = ep - er;
#pragma unroll
        for (int j = 0; j < 4; j++)
          if (j < len) __stcs(o + (size_t)j * W, colour);
        for (int j = 4; j < len; j++) __stcs(o + (size_t)j * W, colour);
        if (colour == gap) gb = 1u << ecl;
      }
    }
    if (!STG && !SM) gapbits |= __reduce_or_sync(FS_FULL_MASK, gb);
    __syncwarp();
  };

  /* A chunk none of whose rows is smaller than its column's running minimum
   * m holds no event and leaves m as it is (an event needs a row smaller than
   * the minimum before it, which is at most m): its per-depth scans are
   * skipped. Warp-uniform. */
  auto no_event = [&](const int(&r)[U]) -> bool {
    int rmin = r[0];
#pragma unroll
    for (int u = 1; u < U; u++) rmin = min(rmin, r[u]);
    return !__any_sync(FS_FULL_MASK, rmin < m);
  };

  /* rows of one chunk of depth samples, then its events into the ring */
  auto march_chunk = [&](auto p2tag, int k0) {
    int r[U];
    if constexpr (LC == 1) {
      /* one lane per column: every lane is at the same depth, so the depth
       * table loads are uniform and the occlusion test is a plain compare */
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int k = k0 + u;
        const int rr = sample_row(p2tag, k);
        r[u] = k < k_end ? rr : H;
      }
      if (no_event(r)) return;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const bool ev = r[u] < m;
        if constexpr (SM) {
          const int k = k0 + u;
          const bool fin = ev && pend_k >= 0;
          const unsigned msk = __ballot_sync(FS_FULL_MASK, fin);
          if (fin) {
            const int pos = (qt + __popc(msk & lanemask_lt)) & (QCAP - 1);
            const bool blend = (k == pend_k + 1) &&
                               (pend_kprev == pend_k - 1 || (pend_kprev < 0 && pend_k == 1));
            q[pos * S::QW] = pack_event(pend_k, cl, pend_r, pend_p);
            q[pos * S::QW + S::QW - 1] =
                (unsigned long long)(uint32_t)(pend_kprev + 1) | ((unsigned long long)blend << 32);
          }
          qt += __popc(msk);
          if (ev) {
            pend_kprev = pend_k;
            pend_k = k;
            pend_r = r[u];
            pend_p = m;
          }
        } else {
          const unsigned msk = __ballot_sync(FS_FULL_MASK, ev);
          if (ev) q[(qt + __popc(msk & lanemask_lt)) & (QCAP - 1)] = pack_event(k0 + u, cl, r[u], m);
          qt += __popc(msk);
        }
        m = min(m, r[u]);
      }
    } else {
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int k = k0 + u * LC + dl;
        const int rr = sample_row(p2tag, k);
        r[u] = k < k_end ? rr : H;
      }
      if (no_event(r)) return;
#pragma unroll
      for (int u = 0; u < U; u++) {
        int incl = r[u];
#pragma unroll
        for (int off = 1; off < LC; off <<= 1) {
          const int t = __shfl_up_sync(FS_FULL_MASK, incl, off, LC);
          if (dl >= off) incl = min(incl, t);
        }
        const int excl = __shfl_up_sync(FS_FULL_MASK, incl, 1, LC);
        const int prev = (dl == 0) ? m : min(m, excl);
        const bool ev = r[u] < prev;
        const unsigned msk = __ballot_sync(FS_FULL_MASK, ev);
        if (ev) {
          const int pos = (qt + __popc(msk & lanemask_lt)) & (QCAP - 1);
          q[pos] = pack_event(k0 + u * LC + dl, cl, r[u], prev);
        }
        qt += __popc(msk);
        m = min(m, __shfl_sync(FS_FULL_MASK, incl, LC - 1, LC));
      }
    }
    __syncwarp();
  };

  /* One loop, one drain site: march a chunk while fewer than 32 events wait,
   * colour and paint 32 at a time, and flush the rest once the march ends. */
  int k0 = k_begin;
  bool marching = true;
  ChunkBounds<CH> cb;
  for (;;) {
    if (marching && qt - qh < 32) {
      if (k0 >= k_end || __all_sync(FS_FULL_MASK, m == 0)) {
        marching = false;
        if constexpr (SM) {
          /* the column's last event: no later sample is an event, so it held
           * the minimum for a single sample only if it is the last sample */
          const bool fin = pend_k >= 0;
          const unsigned msk = __ballot_sync(FS_FULL_MASK, fin);
          if (fin) {
            const int pos = (qt + __popc(msk & lanemask_lt)) & (QCAP - 1);
            const bool blend = (pend_k == n - 1) &&
                               (pend_kprev == pend_k - 1 || (pend_kprev < 0 && pend_k == 1));
            q[pos * S::QW] = pack_event(pend_k, cl, pend_r, pend_p);
            q[pos * S::QW + S::QW - 1] =
                (unsigned long long)(uint32_t)(pend_kprev + 1) | ((unsigned long long)blend << 32);
          }
          qt += __popc(msk);
          __syncwarp();
        }
      } else {
        const int kc = k0;
        k0 += CH;
        /* the warp's columns: [c0 + cl - lane / LC, + CPW) within the frame */
        const bool skip =
            M.pyr && cb.skip(M, zl, zi, cam_h, horizon, H, c0 + cl - lane / LC,
                             max(c0 + cl - lane / LC, min(c0 + cl - lane / LC + S::CPW, W) - 1), kc,
                             k_end, m, lane);
        if (!skip) {
          if (P.stats && m > 0) {
            int c = 0;
#pragma unroll
            for (int u = 0; u < U; u++) c += (kc + u * LC + dl < k_end) ? 1 : 0;
            n_samples += (uint32_t)c;
          }
          if (p2)
            march_chunk(BoolTag<true>{}, kc);
          else
            march_chunk(BoolTag<false>{}, kc);
        }
      }
    }
    const int avail = qt - qh;
    if (avail >= 32 || (!marching && avail > 0)) {
      const int cnt = min(avail, 32);
      drain(cnt);
      qh += cnt;
    } else if (!marching) {
      break;
    }
  }
  n_events += (uint32_t)qt;
  m_out = m;
  gapcols = gapbits;
}

/* Writes the stage's TW columns (rows [0, H)) to the frame: transposed
 * through the two row-major box buffers and stored with TMA, or with plain
 * stores when the frame has no tensor map. Ends with a barrier after every
 * bulk store has read its box, so the stage and the boxes are free again. */
template <int TW, int NT>
__device__ __forceinline__ void store_tile(const FsLaunch &P, const FsView *Vp, int c0,
                                           const uint32_t *stage, uint32_t *box, int tid) {
  const int W = Vp->W, H = Vp->H, stride = H | 1;
  if (Vp->tmap >= 0) {
    const CUtensorMap *tm = P.views ? P.tmaps + Vp->tmap : &P.tmap0;
    const int nb = (H + kBoxRows - 1) / kBoxRows;
    for (int b = 0; b < nb; b++) {
      uint32_t *buf = box + (b & 1) * kBoxRows * TW;
      if (b >= 2) {
        if (tid == 0) bulk_wait_read<1>();
        __syncthreads();
      }
      for (int e = tid; e < kBoxRows * TW; e += NT) {
        const int rr = e / TW, cc = e - rr * TW;
        const int y = b * kBoxRows + rr;
        buf[e] = (y < H) ? stage[cc * stride + y] : 0u;
      }
      fence_proxy_async_shared();
      __syncthreads();
      if (tid == 0) {
        tma_store_2d(tm, buf, c0, b * kBoxRows);
        bulk_commit();
      }
    }
    if (tid == 0) bulk_wait_read<0>();
  } else {
    uint32_t *const out = Vp->out;
    for (int e = tid; e < H * TW; e += NT) {
      const int y = e / TW, cc = e - y * TW;
      if (c0 + cc < W) __stcs(out + (size_t)y * W + c0 + cc, stage[cc * stride + y]);
    }
  }
  __syncthreads();
}

/* The view, depth segment and first column of work item `item`. */
template <int IW>
__device__ __forceinline__ const FsView *decode_item(const FsLaunch &P, int item, int &seg,
                                                     int &c0) {
  if (P.items) {
    const int64_t it = P.items[item];
    seg = FS_ITEM_SEG(it);
    c0 = FS_ITEM_TILE(it) * IW;
    return P.views + FS_ITEM_VIEW(it);
  }
  const int ntiles = (P.view0.W + IW - 1) / IW;
  seg = item / ntiles;
  c0 = (item - seg * ntiles) * IW;
  return &P.view0;
}

template <int TW, int LC, int U, int HF, int CF, int STG, int SM, int FX, int SEG>
__global__ void __launch_bounds__(TW *LC, (RenderShape<TW, LC, U, STG, SM>::min_blocks))
    render_kernel(const __grid_constant__ FsLaunch P) {
  using S = RenderShape<TW, LC, U, STG, SM>;
  constexpr int NT = S::NT;
  constexpr int NW = S::NW;
  constexpr int CPW = S::CPW;
  constexpr int CH = LC * U;
  constexpr int QCAP = S::QCAP;
  static_assert(NT % 32 == 0 && 32 % LC == 0 && TW % 4 == 0 && TW <= 128, "shape");
  static_assert(!SM || (LC == 1 && STG == 0), "smoothing: one lane per column, direct paint");
  static_assert(CH <= FS_ZPAD, "a chunk reads at most FS_ZPAD depth-table entries past n");

  extern __shared__ __align__(1024) unsigned char smem[];
  uint32_t *box = reinterpret_cast<uint32_t *>(smem);
  unsigned long long *queues = reinterpret_cast<unsigned long long *>(smem + S::box_bytes);
  float *lut = reinterpret_cast<float *>(smem + S::box_bytes + S::queue_bytes);
  int *s_next = reinterpret_cast<int *>(smem + S::box_bytes + S::queue_bytes + S::lut_bytes);
  uint32_t *stage = reinterpret_cast<uint32_t *>(smem + S::fixed_bytes);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int dl = lane % LC;
  unsigned long long *q = queues + warp * QCAP * S::QW;
  unsigned lanemask_lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lanemask_lt));
  for (int i = tid; i < 256; i += NT) lut[i] = __fdiv_rn((float)i, 255.0f);
  wait_prior_grid();
  __syncthreads();
  const LutChannels chan{lut};
  uint32_t n_samples = 0, n_events = 0; /* work counters (ctx stats) */

  if constexpr (STG) {
    /* a CTA per (view, tile of TW columns): march into the column stage,
     * fill, then transpose and store with TMA (whole columns: one segment) */
    const int cl = warp * CPW + lane / LC;
    for (int iter = 0;; iter++) {
      int item;
      if (P.head) {
        if (tid == 0) *s_next = atomicAdd(P.head, 1);
        __syncthreads();
        item = *s_next;
      } else {
        item = iter == 0 ? (int)blockIdx.x : P.nitems;
      }
      if (item >= P.nitems) break;
      int seg, c0;
      const FsView *Vp = decode_item<TW>(P, item, seg, c0);
      const int W = Vp->W, H = Vp->H, stride = H | 1;
      const uint32_t sky = Vp->sky, gap = Vp->gap;
      int m;
      uint32_t gapcols;
      render_strip<TW, LC, U, HF, CF, STG, SM, FX>(P, Vp, c0, cl, lane, lanemask_lt, q, stage,
                                                   chan, 0, Vp->n, H, m, gapcols, n_samples,
                                                   n_events);
      /* gap fill + sky for this warp's columns, then the transposed store */
#pragma unroll 1
      for (int c = 0; c < CPW; c++) {
        const int mf = __shfl_sync(FS_FULL_MASK, m, c * LC);
        const int lcl = warp * CPW + c;
        uint32_t *sc = stage + lcl * stride;
        if (c0 + lcl < W) fill_column([sc](int y) { return sc + y; }, 0, H, mf, gap, sky, lane);
      }
      __syncthreads();
      store_tile<TW, NT>(P, Vp, c0, stage, box, tid);
    }
    if (tid == 0) bulk_wait_all();
  } else {
    /* a warp per (view, depth segment, strip of CPW columns): no barrier
     * between items */
    const int cl = lane / LC;
    for (int iter = 0;; iter++) {
      int item;
      if (P.head) {
        int got = 0;
        if (lane == 0) got = atomicAdd(P.head, 1);
        item = __shfl_sync(FS_FULL_MASK, got, 0);
      } else {
        item = iter == 0 ? (int)blockIdx.x * NW + warp : P.nitems;
      }
      if (item >= P.nitems) break;
      int seg, c0;
      const FsView *Vp = decode_item<CPW>(P, item, seg, c0);
      const int W = Vp->W, H = Vp->H, nseg = Vp->nseg;
      const int col = c0 + cl;
      int kb = 0, ke = Vp->n;
      if constexpr (SEG) segment_range(Vp, seg, kb, ke);
      /* the column's minimum row before this segment: the minima of the
       * earlier segments (the segment-minimum pass) */
      int m0 = H;
      if constexpr (SEG) {
        if (seg > 0 && col < W)
          for (int s = 0; s < seg; s++) m0 = min(m0, __ldg(Vp->segbuf + (size_t)s * W + col));
      }
      int m;
      uint32_t gapcols;
      render_strip<TW, LC, U, HF, CF, STG, SM, FX>(P, Vp, c0, cl, lane, lanemask_lt, q, stage,
                                                   chan, kb, ke, m0, m, gapcols, n_samples,
                                                   n_events);
      const uint32_t sky = Vp->sky, gap = Vp->gap;
      uint32_t *const out = Vp->out;
      if (SEG && nseg > 1) {
        /* gap fill needs the whole column: flag it for the gap-fill pass */
        while (gapcols) {
          const int c = __ffs(gapcols) - 1;
          gapcols &= gapcols - 1;
          if (lane == 0) Vp->segbuf[(size_t)(nseg + 1) * W + c0 + c] = 1;
        }
      } else {
        /* gap fill over the rows of columns that painted the gap colour */
        while (gapcols) {
          const int c = __ffs(gapcols) - 1;
          gapcols &= gapcols - 1;
          const int mf = __shfl_sync(FS_FULL_MASK, m, c * LC);
          uint32_t *oc = out + c0 + c;
          fill_column([oc, W](int y) { return oc + (size_t)y * W; }, mf, H, mf, gap, sky, lane);
        }
      }
      if (!SEG || seg == nseg - 1 || nseg <= 1) {
        /* the last segment knows the column's final minimum row */
        if (SEG && nseg > 1 && dl == 0 && col < W) Vp->segbuf[(size_t)nseg * W + col] = m;
        /* sky rows [0, m) of each column: lane (r, c) with c = lane % CPW
         * writes column c of rows r, r + LC, ... (a row per store for LC = 1) */
        const int sc = lane % CPW, sr = lane / CPW;
        const int msc = __shfl_sync(FS_FULL_MASK, m, sc * LC);
        const int mtop = __reduce_max_sync(FS_FULL_MASK, (unsigned)m);
        uint32_t *os = out + (size_t)sr * W + c0 + sc;
        for (int y = sr; y < mtop; y += LC, os += (size_t)LC * W)
          if (y < msc) __stcs(os, sky);
      }
    }
  }
  if (P.stats) {
    unsigned long long ns = n_samples;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) ns += __shfl_down_sync(FS_FULL_MASK, ns, off);
    if (lane == 0) {
      atomicAdd(reinterpret_cast<unsigned long long *>(P.stats), ns);
      atomicAdd(reinterpret_cast<unsigned long long *>(P.stats) + 1, (unsigned long long)n_events);
    }
  }
}

/* Segment-minimum pass of split views: a warp per (view, segment, strip)
 * marches the segment's depths from row H and keeps only the minimum row of
 * each column (no events, no colours); the render pass starts each segment
 * from the minimum of the segments before it. Segment 0 also clears the
 * column's gap flag. Items are those of segments 0 .. nseg-2. */
template <int TW, int LC, int U, int HF>
__global__ void __launch_bounds__(TW *LC, 1024 / (TW * LC)) segmin_kernel(
    const __grid_constant__ FsLaunch P) {
  constexpr int NW = TW * LC / 32;
  constexpr int CPW = 32 / LC;
  constexpr int CH = LC * U;
  static_assert(CH <= FS_ZPAD, "a chunk reads at most FS_ZPAD depth-table entries past n");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int dl = lane % LC, cl = lane / LC;
  wait_prior_grid();
  for (int iter = 0;; iter++) {
    int item;
    if (P.head) {
      int got = 0;
      if (lane == 0) got = atomicAdd(P.head, 1);
      item = __shfl_sync(FS_FULL_MASK, got, 0);
    } else {
      item = iter == 0 ? (int)blockIdx.x * NW + warp : P.nitems;
    }
    if (item >= P.nitems) break;
    int seg, c0;
    const FsView *Vp = decode_item<CPW>(P, item, seg, c0);
    const int W = Vp->W, nseg = Vp->nseg;
    const int col = c0 + cl;
    const bool valid = col < W;
    int kb, ke;
    segment_range(Vp, seg, kb, ke);
    const Marcher<LC, U, HF> mc(P, Vp, col);
    const bool p2 = mc.M.pow2 != 0;
    int m = valid ? mc.H : 0;
    auto chunk_min = [&](auto p2tag, int k0) {
      constexpr bool P2 = decltype(p2tag)::value;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int k = k0 + u * LC + dl;
        const int rr = mc.template row<P2>(k);
        int v = k < ke ? rr : mc.H;
#pragma unroll
        for (int off = 1; off < LC; off <<= 1) v = min(v, __shfl_xor_sync(FS_FULL_MASK, v, off, LC));
        m = min(m, v);
      }
    };
    ChunkBounds<CH> cb;
    const int wlast = max(c0, min(c0 + CPW, W) - 1);
    for (int k0 = kb; k0 < ke; k0 += CH) {
      if (__all_sync(FS_FULL_MASK, m == 0)) break;
      if (mc.M.pyr &&
          cb.skip(mc.M, mc.zl, mc.zi, mc.cam_h, mc.horizon, mc.H, c0, wlast, k0, ke, m, lane))
        continue;
      if (p2)
        chunk_min(BoolTag<true>{}, k0);
      else
        chunk_min(BoolTag<false>{}, k0);
    }
    if (dl == 0 && valid) {
      Vp->segbuf[(size_t)seg * W + col] = m;
      if (seg == 0) Vp->segbuf[(size_t)(nseg + 1) * W + col] = 0;
    }
  }
}

/* ---- the cooperative tile form (stage 2) -------------------------------------
 * A CTA renders a tile of TW columns with TPC threads per column, marching the
 * depths in blocks of NB = TPC * U: thread (c, j) of the tile takes the U
 * consecutive depths j*U .. j*U + U-1 of each block for column c. Per block b:
 *  A. every thread computes the rows of its U samples at once (all gathers in
 *     flight), unless a max-pyramid bound over its warp's columns and depths
 *     shows that none can be below the column minima at the block's start
 *     (the bounds of 32 blocks come from one pass, a lane per block);
 *  B. the running minimum before each sample comes from a min-scan over the
 *     column's threads: the thread's own U rows, a warp scan (__shfl_up_sync
 *     in steps of TW lanes) and the warp totals in shared memory; events (row
 *     below that minimum) go to the tile's event list in shared memory.
 * Block b+1's depth-table entries load into registers at the end of A and go
 * to shared memory during B (two buffers), so a block costs two barriers. A
 * plain call (the view is a kernel parameter) computes block 0's entries in
 * the CTA and marches it while the depth-table kernel finishes. (Copying the
 * next block's entries with cp.async while block b marches, into a third
 * buffer, made the 1920x1080 frame 20 % slower.) The column chain is one
 * block per step instead of one chunk, so a single frame with few columns
 * keeps every SM busy.
 * Colouring does not feed the march (the running minima come from rows
 * alone), so it stays off the chain of blocks: after the last block (or once
 * every column's minimum is row 0, or no later block can hold an event) every
 * thread colours the listed events and writes each colour at its event's row
 * of the stage, which starts the tile filled with the gap value: this is the
 * reference's scatter (fut/voxel_renderer.fut:244). (Colouring block b-1's
 * events beside block b's rows put the near blocks' many events on the
 * chain: 36.9 against 35.5 us for both kernels of a 1920x1080 call.) Then
 * the forward fill (:246)
 * and sky, spread over all threads of the tile. The stage is row-major, so
 * every 32-row box of the tile goes to the frame straight from it with TMA,
 * all boxes back to back. */
template <int TW, int TPC, int U>
struct CoopShape {
  static constexpr int NT = TW * TPC;
  static constexpr int NW = NT / 32;
  static constexpr int NB = TPC * U;   /* depths per block */
  static constexpr size_t lut_bytes = 256 * 4;
  static constexpr size_t zl_bytes = 2ull * NB * 16; /* two blocks' entries */
  static constexpr size_t zi_bytes = 2ull * NB * 4;
  /* warp totals [NW][TW], block-start minima [2][TW], event count, item */
  static constexpr size_t misc_bytes = ((size_t)NW * TW + 2 * TW + 4) * 4;
  /* the stage starts on a 128-byte boundary, as do its boxes (TMA sources) */
  static constexpr size_t fixed_bytes =
      (lut_bytes + zl_bytes + zi_bytes + misc_bytes + 127) / 128 * 128;
  static constexpr int min_blocks = NT >= 1024 ? 1 : 1024 / NT;
  /* the stage: row-major [H rounded up to whole boxes][TW] */
  static __host__ __device__ constexpr size_t stage_bytes(int H) {
    return (size_t)TW * (size_t)((H + kBoxRows - 1) / kBoxRows * kBoxRows) * 4;
  }
  /* the stage, then the tile's event list: every event lowers its column's
   * minimum row, so a tile holds at most TW * H of them (4 bytes each) */
  static __host__ __device__ constexpr size_t tile_bytes(int H) { return 2 * stage_bytes(H); }
};

/* Writes a row-major [rows][TW] stage to the frame: every 32-row box straight
 * from the stage with TMA (no copy, no wait between boxes), or with plain
 * stores when the frame has no tensor map. Ends with a barrier after the bulk
 * stores have read the stage. */
template <int TW, int NT>
__device__ __forceinline__ void store_rows(const FsLaunch &P, const FsView *Vp, int c0,
                                           const uint32_t *stage, int tid) {
  const int W = Vp->W, H = Vp->H;
  if (Vp->tmap >= 0) {
    fence_proxy_async_shared();
    __syncthreads();
    if (tid == 0) {
      const CUtensorMap *tm = P.views ? P.tmaps + Vp->tmap : &P.tmap0;
      for (int b = 0; b * kBoxRows < H; b++)
        tma_store_2d(tm, stage + b * kBoxRows * TW, c0, b * kBoxRows);
      bulk_commit();
      bulk_wait_read<0>();
    }
  } else {
    __syncthreads();
    uint32_t *const out = Vp->out;
    for (int e = tid; e < H * TW; e += NT) {
      const int y = e / TW, cc = e - y * TW;
      if (c0 + cc < W) __stcs(out + (size_t)y * W + c0 + cc, stage[e]);
    }
  }
  __syncthreads();
}

/* Event list entry of the cooperative tile: depth (17 bits), tile column
 * (3), row (12). The host keeps views with more depths, taller frames or
 * wider tiles off this kernel (FS_COOP_MAX_DEPTHS, FS_COOP_MAX_ROWS). */
__device__ __forceinline__ uint32_t pack_coop_event(int k, int c, int row) {
  return ((uint32_t)k << 15) | ((uint32_t)c << 12) | (uint32_t)row;
}

template <int TW, int TPC, int U, int HF, int CF, int FX>
__global__ void __launch_bounds__(TW *TPC, (CoopShape<TW, TPC, U>::min_blocks))
    coop_kernel(const __grid_constant__ FsLaunch P) {
  using S = CoopShape<TW, TPC, U>;
  constexpr int NT = S::NT, NW = S::NW, NB = S::NB;
  static_assert(TW >= 4 && 32 % TW == 0 && NT % 32 == 0, "a warp holds whole runs of TW columns");
  static_assert(TW <= 8, "event fields: tile column in 3 bits");
  static_assert(NB % NT == 0, "a block's depth-table entries split evenly over the threads");

  extern __shared__ __align__(1024) unsigned char smem[];
  float *lut = reinterpret_cast<float *>(smem);
  float4 *zt = reinterpret_cast<float4 *>(smem + S::lut_bytes);
  float *zv = reinterpret_cast<float *>(smem + S::lut_bytes + S::zl_bytes);
  int *wtot = reinterpret_cast<int *>(smem + S::lut_bytes + S::zl_bytes + S::zi_bytes);
  int *mcol = wtot + NW * TW;
  /* [0] events of the tile, [2] next item, [3] every column at row 0 after
   * the block */
  int *scal = mcol + 2 * TW;
  uint32_t *stage = reinterpret_cast<uint32_t *>(smem + S::fixed_bytes);
  /* the tile's event list, after the stage sized for the launch's tallest view */
  uint32_t *evq = stage + S::stage_bytes(P.stride_max) / 4;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c = tid % TW; /* the thread's column within the tile (lane % TW) */
  const int j = tid / TW; /* its run within each depth block */
  /* a plain call's view is a kernel parameter, so its stage can be filled
   * with the gap value before the depth-table kernel has finished */
  const bool param_view = !P.head && !P.items;
  if (param_view) {
    for (int e = tid; e < P.view0.H * TW; e += NT) stage[e] = P.view0.gap;
    /* block 0's depth-table entries straight from the camera, as the
     * depth-table kernel computes them, so the march starts before that
     * kernel has finished; its results are read from block 1 on */
    const DepthLine dl(P.view0);
    for (int p = tid; p < NB; p += NT) {
      const int e = (p % TPC) * U + p / TPC;
      float4 L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      float iz = 0.0f;
      if (e < P.view0.n) dl.entry(e, L, iz);
      zt[p] = L;
      zv[p] = iz;
    }
  }
  for (int i = tid; i < 256; i += NT) lut[i] = __fdiv_rn((float)i, 255.0f);
  if (!param_view) wait_prior_grid();
  const LutChannels chan{lut};
  uint32_t n_samples = 0, n_events = 0;

  for (int iter = 0;; iter++) {
    int item;
    if (P.head) {
      if (tid == 0) scal[2] = atomicAdd(P.head, 1);
      __syncthreads();
      item = scal[2];
    } else {
      item = iter == 0 ? (int)blockIdx.x : P.nitems;
    }
    if (item >= P.nitems) break;
    int seg, c0;
    const FsView *Vp = decode_item<TW>(P, item, seg, c0);
    const int W = Vp->W, H = Vp->H, n = Vp->n;
    const uint32_t sky = Vp->sky, gap = Vp->gap;
    const FsMapDev &M = P.maps[Vp->map];
    const HeightMap hmap{M.q, M.MW, M.MH};
    const bool p2 = M.pow2 != 0;
    const float cam_h = Vp->cam_h, horizon = Vp->horizon;
    const float fcol = (float)(c0 + c);
    const float4 *zl = P.zline + Vp->zoff;
    const float *zi = P.zinvz + Vp->zoff;

    /* depth-table entries of block kb into buffer half: position p holds
     * depth kb + (p % TPC) * U + p / TPC, so step i of run j reads i*TPC + j */
    auto load_table = [&](int kb, int half) {
      for (int p = tid; p < NB; p += NT) {
        const int e = (p % TPC) * U + p / TPC;
        float4 L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float iz = 0.0f;
        if (kb + e < n) {
          L = __ldg(zl + kb + e);
          iz = __ldg(zi + kb + e);
        }
        zt[half * NB + p] = L;
        zv[half * NB + p] = iz;
      }
    };
    /* colour the tile's listed events, each at its row (the depth-table
     * entries from global memory: the list spans every block) */
    auto colour_list = [&](auto c2tag) {
      constexpr bool C2 = decltype(c2tag)::value;
      const int ne = scal[0];
      if (P.stats && tid == 0) n_events += (uint32_t)ne;
      for (int e = tid; e < ne; e += NT) {
        const uint32_t ev = evq[e];
        const int k = (int)(ev >> 15), ec = (int)((ev >> 12) & 7u), er = (int)(ev & 0xFFFu);
        const float4 L = __ldg(zl + k);
        const float2 xy =
            axpy2((float)(c0 + ec), make_float2(L.z, L.w), make_float2(L.x, L.y));
        uint32_t colour = CF ? color_bilinear<C2>(M, chan, xy.x, xy.y)
                             : color_nearest<C2>(M, xy.x, xy.y);
        if constexpr (FX) {
          if (Vp->flags & (FSV_SHADE | FSV_FOG)) {
            /* depth of sample k, as the depth table computes it */
            const float fi = (float)(k + 1);
            const float z = fm(fd(fi, 2.0f), fa(fm(2.0f, Vp->z0), fm(fs(fi, 1.0f), Vp->d)));
            colour = apply_effects(chan, *Vp, colour, z);
          }
        }
        stage[er * TW + ec] = colour;
      }
    };
    const bool cp2 = M.cpow2 != 0;

    /* a column past the frame's right edge starts (and stays) at row 0 */
    if (tid < TW) mcol[tid] = (c0 + tid < W) ? H : 0;
    if (tid == 0) scal[0] = 0;
    if (!(param_view && iter == 0)) {
      for (int e = tid; e < H * TW; e += NT) stage[e] = gap;
      load_table(0, 0);
    }
    __syncthreads();

    /* skip bounds of the warp's runs, 32 blocks at a time: lane l holds the
     * bound of block bbase + l (its depth-table entries read from global
     * memory), so one pass of the bound arithmetic and one round of
     * max-pyramid loads serve 32 blocks */
    int bbound = 0, bbase = -(1 << 30);
    for (int kb = 0, par = 0, bi = 0;; kb += NB, par ^= 1, bi++) {
      /* X: rows of block kb (A) with the colours of the previous block (C) */
      const int mstart = mcol[par * TW + c];
      int r[U];
#pragma unroll
      for (int i = 0; i < U; i++) r[i] = H;
      const float4 *ztb = zt + par * NB;
      const float *zvb = zv + par * NB;
      /* the warp's depths [ka, kz] over its TW columns */
      const int jw = warp * (32 / TW);
      const int ka = kb + jw * U, kz = min(kb + (jw + 32 / TW) * U, n) - 1;
      /* rest: every later block of the warp's depths is skipped too. The
       * column minima only decrease, so a bound not above today's largest
       * minimum stays so; when every warp agrees, the tile ends after this
       * block (its trailing blocks would find no event). */
      bool rest = ka > kz || __all_sync(FS_FULL_MASK, mstart == 0);
      bool skip = rest;
      if (!skip && M.pyr) {
        const float cf = (float)c0, cl = (float)max(c0, min(c0 + TW, W) - 1);
        const int mmax = (int)__reduce_max_sync(FS_FULL_MASK, (unsigned)mstart);
        int b;
        if (param_view && bi == 0) {
          /* a plain call's block 0 marches before the depth-table kernel has
           * finished: its bound comes from the entries in shared memory */
          const int ea = ka - kb, ez = kz - kb;
          const int pa = (ea % U) * TPC + ea / U, pz = (ez % U) * TPC + ez / U;
          b = box_row_bound(M, ztb[pa], zvb[pa], ztb[pz], zvb[pz], cam_h, horizon, H, cf, cl);
        } else {
          if (bi >= bbase + 32) {
            bbase = bi;
            const int kbl = (bi + lane) * NB;
            const int kal = kbl + jw * U, kzl = min(kbl + (jw + 32 / TW) * U, n) - 1;
            bbound = H + 1; /* past the last block: never consulted */
            if (kal <= kzl)
              bbound = chunk_row_bound(M, zl, zi, cam_h, horizon, H, cf, cl, kal, kzl);
          }
          b = __shfl_sync(FS_FULL_MASK, bbound, bi - bbase);
          /* lane l bounds block bbase + l; the window must reach the last block */
          rest = (n - 1) / NB <= bbase + 31 &&
                 __all_sync(FS_FULL_MASK, bbase + lane <= bi || bbound >= mmax);
        }
        skip = b >= mmax;
      }
      if (!skip && mstart > 0) {
        auto rows = [&](auto p2tag) {
          constexpr bool P2 = decltype(p2tag)::value;
#pragma unroll
          for (int i = 0; i < U; i++) {
            const float4 L = ztb[i * TPC + j];
            const float2 xy = axpy2(fcol, make_float2(L.z, L.w), make_float2(L.x, L.y));
            const float hh = HF ? height_bilinear<P2>(hmap, xy.x, xy.y)
                                : height_nearest<P2>(hmap, xy.x, xy.y);
            const int rr = min(max(f2i(fa(fm(fs(cam_h, hh), zvb[i * TPC + j]), horizon)), 0), H);
            r[i] = (kb + j * U + i < n) ? rr : H;
          }
        };
        if (p2)
          rows(BoolTag<true>{});
        else
          rows(BoolTag<false>{});
        if (P.stats) n_samples += (uint32_t)max(0, min(U, n - kb - j * U));
      }
      int run = H;
#pragma unroll
      for (int i = 0; i < U; i++) run = min(run, r[i]);
      int incl = run;
#pragma unroll
      for (int off = TW; off < 32; off <<= 1) {
        const int t = __shfl_up_sync(FS_FULL_MASK, incl, off);
        if (lane >= off) incl = min(incl, t);
      }
      const int ex = __shfl_up_sync(FS_FULL_MASK, incl, TW);
      if (lane >= 32 - TW) wtot[warp * TW + c] = incl;
      /* the next block's depth-table entries: loaded here, stored to shared
       * memory at the end of B, so the loads' latency overlaps the barrier */
      if (param_view && kb == 0) wait_prior_grid();
      const bool more = kb + NB < n;
      float4 Lnext[NB / NT];
      float iznext[NB / NT];
#pragma unroll
      for (int q = 0; q < NB / NT; q++) {
        const int p = tid + q * NT, e = (p % TPC) * U + p / TPC;
        Lnext[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        iznext[q] = 0.0f;
        if (kb + NB + e < n) {
          Lnext[q] = __ldg(zl + kb + NB + e);
          iznext[q] = __ldg(zi + kb + NB + e);
        }
      }
      const bool tile_rest = __syncthreads_and(rest ? 1 : 0) != 0;

      /* Y: the minimum before each sample, the block's events (B), and the
       * next block's depth-table entries */
      /* a run whose rows are all at or below the column's minimum at the
       * block start holds no event; a warp of such runs skips the prefix,
       * except the last warp, which records the columns' new minima */
      if (warp == NW - 1 || __any_sync(FS_FULL_MASK, run < mstart)) {
        /* the minimum over the earlier warps' totals of column c: the 32/TW
         * lanes of the column read every (32/TW)-th warp each, then combine */
        constexpr int Q = 32 / TW;
        int prev = mstart;
#pragma unroll
        for (int w0 = 0; w0 < NW; w0 += Q)
          if (w0 + lane / TW < warp) prev = min(prev, wtot[(w0 + lane / TW) * TW + c]);
#pragma unroll
        for (int off = TW; off < 32; off <<= 1)
          prev = min(prev, __shfl_xor_sync(FS_FULL_MASK, prev, off));
        if (lane >= TW) prev = min(prev, ex);
        if (j == TPC - 1) mcol[(par ^ 1) * TW + c] = min(prev, run);
        if (warp == NW - 1) {
          const bool z = __all_sync(FS_FULL_MASK, lane < 32 - TW || min(prev, run) == 0);
          if (lane == 31) scal[3] = z;
        }
        int cnt = 0;
        if (run < prev) {
          int pv = prev;
#pragma unroll
          for (int i = 0; i < U; i++)
            if (r[i] < pv) {
              cnt++;
              pv = r[i];
            }
        }
        int csum = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const int t = __shfl_up_sync(FS_FULL_MASK, csum, off);
          if (lane >= off) csum += t;
        }
        const int total = __shfl_sync(FS_FULL_MASK, csum, 31);
        if (total) {
          int base = 0;
          if (lane == 31) base = atomicAdd(&scal[0], total);
          base = __shfl_sync(FS_FULL_MASK, base, 31) + csum - cnt;
          if (cnt) {
#pragma unroll
            for (int i = 0; i < U; i++)
              if (r[i] < prev) {
                evq[base++] = pack_coop_event(kb + j * U + i, c, r[i]);
                prev = r[i];
              }
          }
        }
      }
      if (more) {
#pragma unroll
        for (int q = 0; q < NB / NT; q++) {
          zt[(par ^ 1) * NB + tid + q * NT] = Lnext[q];
          zv[(par ^ 1) * NB + tid + q * NT] = iznext[q];
        }
      }
      __syncthreads();

      /* the last block, every column at row 0, or no event possible in any
       * later block */
      bool done = !more;
      if (more) done = scal[3] != 0 || tile_rest;
      if (done) break;
    }
    /* every block's events are listed: colour them into the stage */
    if (cp2)
      colour_list(BoolTag<true>{});
    else
      colour_list(BoolTag<false>{});
    __syncthreads();

    /* fill_vline + sky (fut/voxel_renderer.fut:246-248) over the tile: thread
     * (c, j) takes rows [j*R, j*R + R) of column c (R odd, so the column
     * threads of a warp read distinct banks). Rows no event wrote still
     * hold the gap value, so each row becomes the last non-gap value at or
     * above it, or sky: the thread's last non-gap value, a scan of
     * "the later non-gap value wins" over the column's threads (warp
     * shuffles in steps of TW, then the warp totals), and a second pass. */
    {
      const int R = ((H + TPC - 1) / TPC) | 1;
      const int ya = min(j * R, H), yz = min(ya + R, H);
      uint32_t last = gap;
      for (int y = ya; y < yz; y++) {
        const uint32_t v = stage[y * TW + c];
        if (v != gap) last = v;
      }
      uint32_t incl = last;
#pragma unroll
      for (int off = TW; off < 32; off <<= 1) {
        const uint32_t t = __shfl_up_sync(FS_FULL_MASK, incl, off);
        if (lane >= off && incl == gap) incl = t;
      }
      const uint32_t exw = __shfl_up_sync(FS_FULL_MASK, incl, TW);
      uint32_t *const wlast = reinterpret_cast<uint32_t *>(wtot);
      if (lane >= 32 - TW) wlast[warp * TW + c] = incl;
      __syncthreads();
      uint32_t carry = gap;
      for (int w = 0; w < warp; w++) {
        const uint32_t t = wlast[w * TW + c];
        if (t != gap) carry = t;
      }
      if (lane >= TW && exw != gap) carry = exw;
      for (int y = ya; y < yz; y++) {
        const uint32_t v = stage[y * TW + c];
        if (v != gap) carry = v;
        stage[y * TW + c] = carry == gap ? sky : carry;
      }
    }
    store_rows<TW, NT>(P, Vp, c0, stage, tid);
  }
  if (tid == 0) bulk_wait_all();
  if (P.stats) {
    unsigned long long ns = n_samples, ne = n_events;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) ns += __shfl_down_sync(FS_FULL_MASK, ns, off);
    if (lane == 0) {
      atomicAdd(reinterpret_cast<unsigned long long *>(P.stats), ns);
      if (tid == 0) atomicAdd(reinterpret_cast<unsigned long long *>(P.stats) + 1, ne);
    }
  }
}

}  // namespace fsd

/* Cooperative tile configurations (TW, threads per column, depths per thread
 * per block), stage 2 of the tuning tuple. */
#define FS_COOP_LIST(X) \
  X(8, 64, 8)           \
  X(4, 64, 8)           \
  X(8, 32, 8)           \
  X(4, 64, 4)

/* Cooperative tile configurations with the shading / fog epilogue. */
#define FS_COOP_LIST_FX(X) \
  X(8, 64, 8)              \
  X(4, 64, 8)

/* Kernel modes beyond the plain render, each compiled for a few configurations
 * and every filter pair: (TW, LC, U, STG, smoothing, epilogue). The epilogue
 * is its own instantiation because its code, present but unused, makes the
 * plain kernel measurably slower. */
#define FS_TUNE_LIST_MODES(X) \
  X(8, 32, 2, 1, 0, 1)        \
  X(16, 16, 2, 1, 0, 1)       \
  X(32, 8, 4, 0, 0, 1)        \
  X(64, 2, 4, 0, 0, 1)        \
  X(64, 1, 4, 0, 0, 1)        \
  X(128, 1, 4, 0, 0, 1)       \
  X(128, 1, 8, 0, 0, 1)       \
  X(64, 1, 4, 0, 1, 0)        \
  X(128, 1, 4, 0, 1, 0)       \
  X(64, 1, 4, 0, 1, 1)        \
  X(128, 1, 4, 0, 1, 1)

/* The tuning table: (TW, LC, U, STG) compiled for every filter pair. */
#define FS_TUNE_LIST(X) \
  X(4, 32, 2, 1)        \
  X(8, 32, 1, 1)        \
  X(8, 32, 2, 1)        \
  X(16, 32, 2, 1)       \
  X(32, 32, 1, 1)       \
  X(16, 16, 2, 1)       \
  X(32, 16, 2, 1)       \
  X(16, 8, 4, 1)        \
  X(32, 8, 4, 1)        \
  X(8, 32, 2, 0)        \
  X(16, 16, 2, 0)       \
  X(32, 8, 2, 0)        \
  X(32, 8, 4, 0)        \
  X(32, 4, 4, 0)        \
  X(64, 4, 4, 0)        \
  X(32, 4, 8, 0)        \
  X(64, 2, 4, 0)        \
  X(64, 1, 4, 0)        \
  X(128, 1, 4, 0)       \
  X(64, 1, 8, 0)        \
  X(128, 1, 8, 0)
