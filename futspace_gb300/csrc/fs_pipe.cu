/*
 * The row pipeline (tuning stage 3): one plain call's frame as four
 * data-parallel kernels instead of a chain of depth blocks per column tile.
 *
 * The reference computes every (depth, column) sample (fut/voxel_renderer.fut:
 * 215-228), then per column an inclusive `occlude` scan (:231), the scatter of
 * each new minimum row (:244), the forward fill (:246) and the sky (:248).
 * Here:
 *  1. rows_kernel: the screen row of every sample, all at once (a thread per
 *     column and 8 consecutive depths, a warp per 4 columns x 64 depths), into
 *     a u16 table [W][depth], plus the minimum row of every 64-depth segment
 *     of every column;
 *  2. events_kernel: a warp per (32 columns, segment); a lane starts from the
 *     minimum of its column's earlier segments (the running minimum before the
 *     segment) and finds the segment's events -- samples whose row is strictly
 *     below the running minimum, each painting [row, previous minimum) -- and
 *     appends them to the frame's event list; a segment whose own minimum is
 *     not below the running minimum holds none. The warps of segment 0 also
 *     write each column's sky rows [0, final minimum);
 *  3. paint_kernel: a thread per event colours its sample (the colour
 *     samplers of fut/render_functions.fut:91-105, the optional epilogue) and
 *     paints its rows. Intervals of different events are disjoint, so the
 *     order does not matter; a column that painted the gap colour is flagged;
 *  4. fix_kernel: the reference's forward fill over the rows of flagged
 *     columns (none unless a colour equals the gap value).
 * Every kernel is launched with programmatic stream serialization and waits
 * for its predecessor (griddepcontrol.wait) before reading its results.
 * Pixels are those of the other kernel forms bit for bit: the same row and
 * colour arithmetic, the same event rule.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "fs_device.cuh"
#include "fs_render.cuh"

namespace fsd {
namespace {

constexpr int kSeg = FS_PIPE_SEG;  /* depths per segment */
constexpr int kDepthsPerThread = 8; /* rows_kernel: one 16-byte store of rows */

/* Event: depth (20 bits) | column (16) | row (14) | rows painted (14). */
__device__ __forceinline__ unsigned long long pack_pipe_event(int k, int c, int row, int len) {
  return ((unsigned long long)(uint32_t)k << 44) | ((unsigned long long)(uint32_t)c << 28) |
         ((unsigned long long)(uint32_t)row << 14) | (unsigned long long)(uint32_t)len;
}

template <int HF>
__global__ void __launch_bounds__(256) rows_kernel(const __grid_constant__ FsLaunch P,
                                                   const __grid_constant__ FsPipe Q) {
  allow_dependent_launch();
  const FsView &V = P.view0;
  const int lane = threadIdx.x & 31;
  const int wi = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int ngroups = (V.W + 3) >> 2;
  const int seg = wi / ngroups, cg = wi - seg * ngroups;
  const int c = cg * 4 + (lane >> 3);
  const int k0 = seg * kSeg + (lane & 7) * kDepthsPerThread;
  wait_prior_grid();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *Q.count = 0;
    if (P.stats)
      atomicAdd(reinterpret_cast<unsigned long long *>(P.stats),
                (unsigned long long)V.n * (unsigned long long)V.W);
  }
  if (seg >= Q.nseg) return; /* warp-uniform */
  const int W = V.W, H = V.H, n = V.n;
  const bool valid = c < W;
  const FsMapDev &M = P.maps[0];
  const HeightMap hmap{M.q, M.MW, M.MH};
  const float4 *zl = P.zline + V.zoff;
  const float *zi = P.zinvz + V.zoff;
  const float cam_h = V.cam_h, horizon = V.horizon, fcol = (float)c;
  int r[kDepthsPerThread];
  auto rows = [&](auto p2tag) {
    constexpr bool P2 = decltype(p2tag)::value;
#pragma unroll
    for (int i = 0; i < kDepthsPerThread; i++) {
      /* entries past n are the table's zero padding: read, then discarded */
      const float4 L = __ldg(zl + k0 + i);
      const float2 xy = axpy2(fcol, make_float2(L.z, L.w), make_float2(L.x, L.y));
      const float hh =
          HF ? height_bilinear<P2>(hmap, xy.x, xy.y) : height_nearest<P2>(hmap, xy.x, xy.y);
      const int rr = min(max(f2i(fa(fm(fs(cam_h, hh), __ldg(zi + k0 + i)), horizon)), 0), H);
      r[i] = (k0 + i < n) ? rr : H;
    }
  };
  if (valid) {
    if (M.pow2)
      rows(BoolTag<true>{});
    else
      rows(BoolTag<false>{});
    uint4 v;
    v.x = (uint32_t)r[0] | ((uint32_t)r[1] << 16);
    v.y = (uint32_t)r[2] | ((uint32_t)r[3] << 16);
    v.z = (uint32_t)r[4] | ((uint32_t)r[5] << 16);
    v.w = (uint32_t)r[6] | ((uint32_t)r[7] << 16);
    *reinterpret_cast<uint4 *>(Q.rows + (size_t)c * Q.rpitch + k0) = v;
  } else {
#pragma unroll
    for (int i = 0; i < kDepthsPerThread; i++) r[i] = H;
  }
  int m = r[0];
#pragma unroll
  for (int i = 1; i < kDepthsPerThread; i++) m = min(m, r[i]);
  /* the segment's minimum over the 8 lanes of the column */
  m = min(m, __shfl_xor_sync(FS_FULL_MASK, m, 1));
  m = min(m, __shfl_xor_sync(FS_FULL_MASK, m, 2));
  m = min(m, __shfl_xor_sync(FS_FULL_MASK, m, 4));
  if (valid && (lane & 7) == 0) Q.segmin[(size_t)c * Q.spitch + seg] = (uint16_t)m;
}

__global__ void __launch_bounds__(128) events_kernel(const __grid_constant__ FsLaunch P,
                                                     const __grid_constant__ FsPipe Q) {
  allow_dependent_launch();
  const FsView &V = P.view0;
  const int lane = threadIdx.x & 31;
  const int wi = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nseg = Q.nseg;
  const int strip = wi / nseg, s = wi - strip * nseg;
  const int W = V.W, H = V.H;
  if (strip * 32 >= W) return; /* warp-uniform */
  const int c = strip * 32 + lane;
  const bool valid = c < W;
  wait_prior_grid();
  /* the running minimum before the segment (earlier segments' minima) and,
   * for segment 0, the column's final minimum (all segments) */
  const uint16_t *sm = Q.segmin + (size_t)(valid ? c : 0) * Q.spitch;
  const int upto = s == 0 ? nseg : s;
  int m0 = H, mall = H;
  if (valid) {
    for (int j0 = 0; j0 < upto; j0 += 8) {
      const uint4 v = __ldg(reinterpret_cast<const uint4 *>(sm + j0));
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const int j = j0 + i;
        const int val = (int)((w[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu);
        if (j < s) m0 = min(m0, val);
        if (j < nseg) mall = min(mall, val);
      }
    }
  }
  if (s == 0) {
    if (valid) {
      Q.colmin[c] = mall;
      Q.flags[c] = 0;
    }
    /* sky rows [0, final minimum): a row of 32 columns per store */
    const int mine = valid ? mall : 0;
    const int mtop = (int)__reduce_max_sync(FS_FULL_MASK, (unsigned)mine);
    uint32_t *o = V.out + c;
    const uint32_t sky = V.sky;
    for (int y = 0; y < mtop; y++)
      if (y < mine) __stcs(o + (size_t)y * W, sky);
  }
  /* the segment's events: none when its minimum is not below m0 */
  int cnt = 0;
  uint4 rv[kSeg / 8];
  const bool any = valid && (int)sm[s] < m0;
  if (any) {
    const uint4 *src = reinterpret_cast<const uint4 *>(Q.rows + (size_t)c * Q.rpitch + s * kSeg);
#pragma unroll
    for (int i = 0; i < kSeg / 8; i++) rv[i] = __ldg(src + i);
    int m = m0;
#pragma unroll
    for (int i = 0; i < kSeg / 8; i++) {
      const uint32_t w[4] = {rv[i].x, rv[i].y, rv[i].z, rv[i].w};
#pragma unroll
      for (int h = 0; h < 8; h++) {
        const int r = (int)((w[h >> 1] >> ((h & 1) * 16)) & 0xFFFFu);
        if (r < m) {
          cnt++;
          m = r;
        }
      }
    }
  }
  /* one atomic per warp for the list positions */
  int incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int t = __shfl_up_sync(FS_FULL_MASK, incl, off);
    if (lane >= off) incl += t;
  }
  const int total = __shfl_sync(FS_FULL_MASK, incl, 31);
  if (total == 0) return;
  int base = 0;
  if (lane == 31) base = atomicAdd(Q.count, total);
  base = __shfl_sync(FS_FULL_MASK, base, 31) + incl - cnt;
  if (cnt) {
    int m = m0;
#pragma unroll
    for (int i = 0; i < kSeg / 8; i++) {
      const uint32_t w[4] = {rv[i].x, rv[i].y, rv[i].z, rv[i].w};
#pragma unroll
      for (int h = 0; h < 8; h++) {
        const int r = (int)((w[h >> 1] >> ((h & 1) * 16)) & 0xFFFFu);
        if (r < m) {
          if (base < Q.ecap) Q.events[base] = pack_pipe_event(s * kSeg + i * 8 + h, c, r, m - r);
          base++;
          m = r;
        }
      }
    }
  }
}

template <int CF, int FX>
__global__ void __launch_bounds__(256) paint_kernel(const __grid_constant__ FsLaunch P,
                                                    const __grid_constant__ FsPipe Q) {
  __shared__ float lut[256];
  allow_dependent_launch();
  lut[threadIdx.x] = __fdiv_rn((float)threadIdx.x, 255.0f);
  wait_prior_grid();
  __syncthreads();
  const LutChannels chan{lut};
  const FsView &V = P.view0;
  const FsMapDev &M = P.maps[0];
  const int W = V.W;
  const uint32_t gap = V.gap;
  const float4 *zl = P.zline + V.zoff;
  uint32_t *const out = V.out;
  const int64_t count = min((int64_t)*Q.count, Q.ecap);
  if (P.stats && blockIdx.x == 0 && threadIdx.x == 0)
    atomicAdd(reinterpret_cast<unsigned long long *>(P.stats) + 1, (unsigned long long)count);
  auto paint_all = [&](auto c2tag) {
    constexpr bool C2 = decltype(c2tag)::value;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
      const unsigned long long e = __ldg(Q.events + i);
      const int k = (int)(e >> 44), c = (int)((e >> 28) & 0xFFFFu);
      const int row = (int)((e >> 14) & 0x3FFFu), len = (int)(e & 0x3FFFu);
      const float4 L = __ldg(zl + k);
      const float2 xy = axpy2((float)c, make_float2(L.z, L.w), make_float2(L.x, L.y));
      uint32_t colour =
          CF ? color_bilinear<C2>(M, chan, xy.x, xy.y) : color_nearest<C2>(M, xy.x, xy.y);
      if constexpr (FX) {
        if (V.flags & (FSV_SHADE | FSV_FOG)) {
          /* depth of sample k, as the depth table computes it */
          const float fi = (float)(k + 1);
          const float z = fm(fd(fi, 2.0f), fa(fm(2.0f, V.z0), fm(fs(fi, 1.0f), V.d)));
          colour = apply_effects(chan, V, colour, z);
        }
      }
      uint32_t *o = out + (size_t)row * W + c;
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (j < len) __stcs(o + (size_t)j * W, colour);
      for (int j = 4; j < len; j++) __stcs(o + (size_t)j * W, colour);
      if (colour == gap) Q.flags[c] = 1;
    }
  };
  if (M.cpow2)
    paint_all(BoolTag<true>{});
  else
    paint_all(BoolTag<false>{});
}

/* The forward fill (fut/voxel_renderer.fut:246-248) over the painted rows of
 * every column that painted the gap colour: a warp per column. */
__global__ void __launch_bounds__(256) fix_kernel(const __grid_constant__ FsLaunch P,
                                                  const __grid_constant__ FsPipe Q) {
  wait_prior_grid();
  const FsView &V = P.view0;
  const int lane = threadIdx.x & 31;
  const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int W = V.W;
  if (c >= W || !Q.flags[c]) return;
  const int mf = Q.colmin[c];
  uint32_t *oc = V.out + c;
  fill_column([oc, W](int y) { return oc + (size_t)y * W; }, mf, V.H, mf, V.gap, V.sky, lane);
}

template <class K>
int launch_pdl(K kern, int grid, int block, cudaStream_t st, const FsLaunch *L,
               const FsPipe *Q) {
  if (grid <= 0) return (int)cudaSuccess;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return (int)cudaLaunchKernelEx(&cfg, kern, *L, *Q);
}

}  // namespace
}  // namespace fsd

extern "C" int fsk_pipe(const FsLaunch *L, const FsPipe *Q, int32_t hf, int32_t cf, int32_t fx,
                        int32_t sm_count, cudaStream_t st) {
  using namespace fsd;
  const FsView &V = L->view0;
  if (V.W <= 0 || V.H <= 0 || Q->nseg <= 0) return (int)cudaErrorInvalidValue;
  const int64_t rows_warps = (int64_t)((V.W + 3) / 4) * Q->nseg;
  const int64_t event_warps = (int64_t)((V.W + 31) / 32) * Q->nseg;
  int e = launch_pdl(hf ? rows_kernel<1> : rows_kernel<0>, (int)((rows_warps + 7) / 8), 256, st,
                     L, Q);
  if (!e) e = launch_pdl(events_kernel, (int)((event_warps + 3) / 4), 128, st, L, Q);
  if (!e) {
    auto pk = cf ? (fx ? paint_kernel<1, 1> : paint_kernel<1, 0>)
                 : (fx ? paint_kernel<0, 1> : paint_kernel<0, 0>);
    e = launch_pdl(pk, 4 * (sm_count > 0 ? sm_count : 1), 256, st, L, Q);
  }
  if (!e) e = launch_pdl(fix_kernel, (V.W + 7) / 8, 256, st, L, Q);
  return e;
}
