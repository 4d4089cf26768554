/*
 * Device arithmetic shared by the render, z-table and shadow kernels.
 *
 * Every f32 operation is an explicit round-to-nearest intrinsic, so no
 * multiply-add is ever contracted into an FMA (the build also passes
 * --fmad=false). Operation order follows the reference source line by line,
 * which is what makes the frames bit-identical to the CPU restatement.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_internal.h"

#define FS_FULL_MASK 0xffffffffu

namespace fsd {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

/* `i32.f32` / `u32.f32`: cvt.rzi saturates out-of-range values and maps NaN to
 * 0, which is the conversion the reference's GPU targets perform. */
__device__ __forceinline__ int32_t f2i(float v) { return __float2int_rz(v); }
__device__ __forceinline__ uint32_t f2u(float v) { return __float2uint_rz(v); }

/* Futhark `%` on i32 (floored; the map sizes are positive). For power-of-two
 * sizes the two's-complement mask gives the same result. */
__device__ __forceinline__ int32_t wrap(int32_t a, int32_t m, int32_t pow2) {
  if (pow2) return a & (m - 1);
  int32_t r = a % m;
  return r < 0 ? r + m : r;
}

/* Exact u8 -> f32: the byte placed in the mantissa of 2^23, minus 2^23.
 * `sel` is a byte_perm selector picking byte 0..3 of q (0x7540 + i). */
__device__ __forceinline__ float byte_f(uint32_t q, uint32_t sel) {
  return fs(__uint_as_float(__byte_perm(q, 0x4B000000u, sel)), 8388608.0f);
}

/* png_height_filtered, fut/render_functions.fut:67-77, on the quad map. The
 * quad at (floor y, floor x) holds the corners (fy,fx), (fy,fx+1), (fy+1,fx),
 * (fy+1,fx+1). For non-integral x the reference's ceil(x) is floor(x)+1, so the
 * corners are the same texels; for integral x both x weights (cx-x, x-fx) are
 * exactly zero and the corner values do not affect the result (likewise y). */
__device__ __forceinline__ float height_bilinear(const FsMapDev &M, float x, float y) {
  const float fx = floorf(x), cx = ceilf(x), fy = floorf(y), cy = ceilf(y);
  const int32_t ix = wrap(f2i(fx), M.MW, M.pow2), iy = wrap(f2i(fy), M.MH, M.pow2);
  const uint32_t q = __ldg(M.q + (size_t)iy * (size_t)M.MW + ix);
  const float h00 = byte_f(q, 0x7540), h01 = byte_f(q, 0x7541);
  const float h10 = byte_f(q, 0x7542), h11 = byte_f(q, 0x7543);
  const float wx0 = fs(cx, x), wx1 = fs(x, fx);
  const float x1 = fa(fm(wx0, h00), fm(wx1, h01));
  const float x2 = fa(fm(wx0, h10), fm(wx1, h11));
  return fa(fm(fs(cy, y), x1), fm(fs(y, fy), x2));
}

/* png_height, fut/render_functions.fut:63-64 */
__device__ __forceinline__ float height_nearest(const FsMapDev &M, float x, float y) {
  const int32_t ix = wrap(f2i(x), M.MW, M.pow2), iy = wrap(f2i(y), M.MH, M.pow2);
  return byte_f(__ldg(M.q + (size_t)iy * (size_t)M.MW + ix), 0x7540);
}

/* Upper bound of every height the samplers can read for samples on the segment
 * between (xa, ya) and (xb, yb): the max pyramid over the texel box
 * [floor(min x) - 1, floor(max x) + 2] x (same in y), which holds every
 * bilinear corner of every sample on the segment with a margin for rounding,
 * at the level where the box spans at most 2 x 2 cells (4 lookups). */
__device__ __forceinline__ int segment_max_height(const FsMapDev &M, float xa, float ya, float xb,
                                                  float yb) {
  const float lim = 1.0e9f; /* also rejects NaN */
  if (!(fabsf(xa) < lim && fabsf(xb) < lim && fabsf(ya) < lim && fabsf(yb) < lim)) return 255;
  const int ix0 = __float2int_rd(fminf(xa, xb)) - 1, ix1 = __float2int_rd(fmaxf(xa, xb)) + 2;
  const int iy0 = __float2int_rd(fminf(ya, yb)) - 1, iy1 = __float2int_rd(fmaxf(ya, yb)) + 2;
  const int span = max(ix1 - ix0, iy1 - iy0) + 1;
  const int L = 32 - __clz(span - 1); /* ceil(log2(span)): cells of 2^L texels */
  if (L > M.pyr_levels) return 255;
  const uint8_t *P = M.pyr + M.pyr_off[L - 1];
  const int cw = M.MW >> L, chh = M.MH >> L;
  const int cx0 = (ix0 >> L) & (cw - 1), cx1 = (ix1 >> L) & (cw - 1);
  const int cy0 = (iy0 >> L) & (chh - 1), cy1 = (iy1 >> L) & (chh - 1);
  const int a = max(__ldg(P + cy0 * cw + cx0), __ldg(P + cy0 * cw + cx1));
  const int b = max(__ldg(P + cy1 * cw + cx0), __ldg(P + cy1 * cw + cx1));
  return max(a, b);
}

/* ---- matte 0.1.2 argb colour arithmetic (to_rgba / from_rgba / mix) ----------
 * Channel values byte/255 come from `lut` (256 entries, each an IEEE division
 * computed once per CTA) or, with lut == nullptr, from the division itself. */
struct Channels {
  const float *lut;
  __device__ __forceinline__ float operator()(uint32_t c, int sh) const {
    const uint32_t b = (c >> sh) & 0xFFu;
    return lut ? lut[b] : fd((float)b, 255.0f);
  }
};

/* clamp_channel: NaN passes through (both comparisons are false). */
__device__ __forceinline__ float clamp_channel(float x) {
  return (x < 0.0f) ? 0.0f : ((x > 1.0f) ? 1.0f : x);
}
__device__ __forceinline__ uint32_t to_byte(float x) { return f2u(fm(clamp_channel(x), 255.0f)); }

__device__ __forceinline__ uint32_t mix(const Channels &ch, float w1, uint32_t c1, float w2,
                                        uint32_t c2) {
  /* w1 / (w1 + w2): when the sum is exactly 1 the quotient is w1 itself */
  const float w = fa(w1, w2);
  float w1n, w2n;
  if (w == 1.0f) {
    w1n = w1;
    w2n = w2;
  } else {
    w1n = fd(w1, w);
    w2n = fd(w2, w);
  }
  const float r = fa(fm(ch(c1, 16), w1n), fm(ch(c2, 16), w2n));
  const float g = fa(fm(ch(c1, 8), w1n), fm(ch(c2, 8), w2n));
  const float b = fa(fm(ch(c1, 0), w1n), fm(ch(c2, 0), w2n));
  const float a = fa(fm(ch(c1, 24), w1n), fm(ch(c2, 24), w2n));
  return (to_byte(a) << 24) | (to_byte(r) << 16) | (to_byte(g) << 8) | to_byte(b);
}

/* matte colourspace.scale: RGB times s, alpha kept, then from_rgba. */
__device__ __forceinline__ uint32_t scale(const Channels &ch, uint32_t c, float s) {
  return (to_byte(ch(c, 24)) << 24) | (to_byte(fm(ch(c, 16), s)) << 16) |
         (to_byte(fm(ch(c, 8), s)) << 8) | to_byte(fm(ch(c, 0), s));
}

/* The optional shading / fog epilogue of one sample at depth z (FSV_SHADE,
 * FSV_FOG); not part of the reference's path. */
__device__ __forceinline__ uint32_t apply_effects(const Channels &ch, const FsView &V,
                                                  uint32_t c, float z) {
  if (V.flags & FSV_SHADE) c = scale(ch, c, fs(1.0f, fm(V.shade, fd(z, V.distance))));
  if (V.flags & FSV_FOG) {
    float f = fd(fs(z, V.fog_start), fs(V.fog_end, V.fog_start));
    f = (f < 0.0f) ? 0.0f : ((f > 1.0f) ? 1.0f : f);
    c = mix(ch, fs(1.0f, f), c, f, V.fog_color);
  }
  return c;
}

/* png_color_filtered, fut/render_functions.fut:95-105 */
__device__ __forceinline__ uint32_t color_bilinear(const FsMapDev &M, const Channels &ch,
                                                   float x, float y) {
  const float fx = floorf(x), cx = ceilf(x), fy = floorf(y), cy = ceilf(y);
  const int32_t ix0 = wrap(f2i(fx), M.CW, M.cpow2), ix1 = wrap(f2i(cx), M.CW, M.cpow2);
  const int32_t iy0 = wrap(f2i(fy), M.CH, M.cpow2), iy1 = wrap(f2i(cy), M.CH, M.cpow2);
  const uint32_t *r0 = M.c + (size_t)iy0 * (size_t)M.CW;
  const uint32_t *r1 = M.c + (size_t)iy1 * (size_t)M.CW;
  const uint32_t c00 = __ldg(r0 + ix0), c01 = __ldg(r0 + ix1);
  const uint32_t c10 = __ldg(r1 + ix0), c11 = __ldg(r1 + ix1);
  const uint32_t x1 = mix(ch, fs(cx, x), c00, fs(x, fx), c01);
  const uint32_t x2 = mix(ch, fs(cx, x), c10, fs(x, fx), c11);
  return mix(ch, fs(cy, y), x1, fs(y, fy), x2);
}

/* png_color, fut/render_functions.fut:91-92 */
__device__ __forceinline__ uint32_t color_nearest(const FsMapDev &M, float x, float y) {
  const int32_t ix = wrap(f2i(x), M.CW, M.cpow2), iy = wrap(f2i(y), M.CH, M.cpow2);
  return __ldg(M.c + (size_t)iy * (size_t)M.CW + ix);
}

}  // namespace fsd
