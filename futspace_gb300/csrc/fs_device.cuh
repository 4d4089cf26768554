/*
 * Device arithmetic shared by the render, z-table and shadow kernels.
 *
 * Every f32 operation is an explicit round-to-nearest intrinsic, so no
 * multiply-add is ever contracted into an FMA (the build also passes
 * --fmad=false). Operation order follows the reference source line by line,
 * which is what makes the frames bit-identical to the CPU restatement.
 *
 * Where two independent operations of the same kind sit side by side (the x
 * and y coordinates of a sample, two bilinear products, two colour channels)
 * they go through one packed f32x2 instruction (mul.rn.f32x2): each half is
 * an IEEE binary32 operation with round-to-nearest, the same result as the two
 * scalar operations, in half the issue slots.
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

/* Packed pairs through inline PTX with explicit rounding modifiers. ptxas
 * contracts a packed multiply that feeds a packed add into a fused
 * multiply-add even then (and under --fmad=false), which changes the last bit
 * of about half the results; a packed multiply followed by scalar adds is left
 * alone. So a mul2 result here only ever feeds scalar operations, and add2
 * only ever adds operands that no multiply produced. */
__device__ __forceinline__ unsigned long long pk2(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 up2(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
  return up2(d);
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
  return up2(d);
}

/* (base.x + s * step.x, base.y + s * step.y): one packed multiply, two scalar
 * adds (a sample's map coordinates from its depth-table line). */
__device__ __forceinline__ float2 axpy2(float s, float2 step, float2 base) {
  const float2 p = mul2(make_float2(s, s), step);
  return make_float2(fa(base.x, p.x), fa(base.y, p.y));
}

/* a + b rounded to nearest, then clamped to [0, 1]; a NaN sum becomes +0. */
__device__ __forceinline__ float sat_add(float a, float b) {
  float d;
  asm("add.rn.sat.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
  return d;
}

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
template <bool P2>
__device__ __forceinline__ int32_t wrap_t(int32_t a, int32_t m) {
  if (P2) return a & (m - 1);
  const int32_t r = a % m;
  return r < 0 ? r + m : r;
}

/* Exact u8 -> f32: the byte placed in the mantissa of 2^23, minus 2^23.
 * `sel` is a byte_perm selector picking byte 0..3 of q (0x7540 + i). */
__device__ __forceinline__ float byte_f(uint32_t q, uint32_t sel) {
  return fs(__uint_as_float(__byte_perm(q, 0x4B000000u, sel)), 8388608.0f);
}
/* Two bytes of q as an exact float pair. */
__device__ __forceinline__ float2 byte_pair(uint32_t q, uint32_t sel_lo, uint32_t sel_hi) {
  return add2(make_float2(__uint_as_float(__byte_perm(q, 0x4B000000u, sel_lo)),
                          __uint_as_float(__byte_perm(q, 0x4B000000u, sel_hi))),
              make_float2(-8388608.0f, -8388608.0f));
}

/* The height quads of one map as a render item reads them, in registers. */
struct HeightMap {
  const uint32_t *q;
  int32_t MW, MH;
};

template <bool P2>
__device__ __forceinline__ uint32_t height_quad(const HeightMap &M, int32_t ix, int32_t iy) {
  const int32_t x = wrap_t<P2>(ix, M.MW), y = wrap_t<P2>(iy, M.MH);
  return __ldg(M.q + (uint32_t)(y * M.MW + x));
}

/* png_height_filtered, fut/render_functions.fut:67-77, on the quad map. The
 * quad at (floor y, floor x) holds the corners (fy,fx), (fy,fx+1), (fy+1,fx),
 * (fy+1,fx+1). For non-integral x the reference's ceil(x) is floor(x)+1, so the
 * corners are the same texels; for integral x both x weights (cx-x, x-fx) are
 * exactly zero and the corner values do not affect the result (likewise y).
 * x1 = (cx-x)*h00 + (x-fx)*h01 and x2 = (cx-x)*h10 + (x-fx)*h11 take one
 * packed multiply each; the final (cy-y)*x1 + (y-fy)*x2 one more. */
template <bool P2>
__device__ __forceinline__ float height_bilinear(const HeightMap &M, float x, float y) {
  const float fx = floorf(x), cx = ceilf(x), fy = floorf(y), cy = ceilf(y);
  const uint32_t q = height_quad<P2>(M, f2i(fx), f2i(fy));
  const float2 top = byte_pair(q, 0x7540, 0x7541); /* (fy,fx), (fy,cx) */
  const float2 bot = byte_pair(q, 0x7542, 0x7543); /* (cy,fx), (cy,cx) */
  const float2 wx = make_float2(fs(cx, x), fs(x, fx));
  const float2 pt = mul2(wx, top), pb = mul2(wx, bot);
  const float2 py = mul2(make_float2(fs(cy, y), fs(y, fy)),
                         make_float2(fa(pt.x, pt.y), fa(pb.x, pb.y)));
  return fa(py.x, py.y);
}

/* png_height, fut/render_functions.fut:63-64 (i32 truncates toward zero) */
template <bool P2>
__device__ __forceinline__ float height_nearest(const HeightMap &M, float x, float y) {
  return byte_f(height_quad<P2>(M, f2i(x), f2i(y)), 0x7540);
}

/* png_height on a map record (shadow-map kernel) */
__device__ __forceinline__ float height_nearest(const FsMapDev &M, float x, float y) {
  const int32_t ix = wrap(f2i(x), M.MW, M.pow2), iy = wrap(f2i(y), M.MH, M.pow2);
  return byte_f(__ldg(M.q + (size_t)iy * (size_t)M.MW + ix), 0x7540);
}

/* Upper bound of every height the samplers can read for samples whose
 * coordinates lie in [x0, x1] x [y0, y1]: the max pyramid over the texel box
 * [floor(x0) - 1, floor(x1) + 2] x (same in y), which holds every bilinear
 * corner of every such sample with a margin for rounding, at the level where
 * the box spans at most 2 x 2 cells (4 lookups). */
__device__ __forceinline__ int box_max_height(const FsMapDev &M, float x0, float x1, float y0,
                                              float y1) {
  const float lim = 1.0e9f; /* also rejects NaN */
  if (!(fabsf(x0) < lim && fabsf(x1) < lim && fabsf(y0) < lim && fabsf(y1) < lim)) return 255;
  const int ix0 = __float2int_rd(x0) - 1, ix1 = __float2int_rd(x1) + 2;
  const int iy0 = __float2int_rd(y0) - 1, iy1 = __float2int_rd(y1) + 2;
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

/* The same over the segment between (xa, ya) and (xb, yb). */
__device__ __forceinline__ int segment_max_height(const FsMapDev &M, float xa, float ya, float xb,
                                                  float yb) {
  return box_max_height(M, fminf(xa, xb), fmaxf(xa, xb), fminf(ya, yb), fmaxf(ya, yb));
}

/* ---- matte 0.1.2 argb colour arithmetic (to_rgba / from_rgba / mix) ----------
 * A channel fetcher returns byte i of an ARGB word (0 blue, 1 green, 2 red,
 * 3 alpha) as the IEEE quotient byte / 255: from a 256-entry table of those
 * quotients in shared memory, or from the division itself. `bits(v)` takes
 * the byte from a channel held as the bit pattern of the float 2^23 + byte. */
struct LutChannels {
  const float *lut;
  __device__ __forceinline__ float operator()(uint32_t c, int i) const {
    return lut[__byte_perm(c, 0u, 0x4440u + (uint32_t)i)];
  }
  __device__ __forceinline__ float bits(uint32_t v) const { return lut[v - 0x4B000000u]; }
};
struct DivChannels {
  __device__ __forceinline__ float operator()(uint32_t c, int i) const {
    return fd((float)__byte_perm(c, 0u, 0x4440u + (uint32_t)i), 255.0f);
  }
  __device__ __forceinline__ float bits(uint32_t v) const {
    return fd(fs(__uint_as_float(v), 8388608.0f), 255.0f);
  }
};

/* A colour between two mixes: each channel byte as the bit pattern of the float
 * 2^23 + byte. */
struct Argb {
  uint32_t r, g, b, a;
};

/* from_rgba of channel pairs (r, g) and (b, a), each already clamped to
 * [0, 1]: byte = trunc(v * 255). v * 255 lies in [0, 255], so adding 2^23 with
 * round-toward-zero leaves trunc(v * 255) in the low mantissa bits. */
__device__ __forceinline__ Argb to_bytes(float2 rg, float2 ba) {
  const float2 k255 = make_float2(255.0f, 255.0f);
  const float2 srg = mul2(rg, k255), sba = mul2(ba, k255);
  return Argb{__float_as_uint(__fadd_rz(srg.x, 8388608.0f)),
              __float_as_uint(__fadd_rz(srg.y, 8388608.0f)),
              __float_as_uint(__fadd_rz(sba.x, 8388608.0f)),
              __float_as_uint(__fadd_rz(sba.y, 8388608.0f))};
}
__device__ __forceinline__ uint32_t pack(const Argb &c) {
  return __byte_perm(__byte_perm(c.b, c.g, 0x0040u), __byte_perm(c.r, c.a, 0x0040u), 0x5410u);
}
__device__ __forceinline__ uint32_t pack_argb(float2 rg, float2 ba) { return pack(to_bytes(rg, ba)); }

/* mix's weight normalisation w1 / (w1 + w2), w2 / (w1 + w2): when the sum is
 * exactly 1 the quotients are the weights themselves. */
__device__ __forceinline__ void mix_weights(float w1, float w2, float &w1n, float &w2n) {
  const float w = fa(w1, w2);
  w1n = w1;
  w2n = w2;
  if (w != 1.0f) {
    w1n = fd(w1, w);
    w2n = fd(w2, w);
  }
}

/* argb.mix with normalised weights on channel values: per channel
 * c1*w1n + c2*w2n, clamped to [0, 1] (a NaN channel gives byte 0), times 255,
 * truncated. */
__device__ __forceinline__ Argb mix_ch(float w1n, float2 rg1, float2 ba1, float w2n, float2 rg2,
                                       float2 ba2) {
  const float2 W1 = make_float2(w1n, w1n), W2 = make_float2(w2n, w2n);
  const float2 p_rg = mul2(rg1, W1), q_rg = mul2(rg2, W2);
  const float2 p_ba = mul2(ba1, W1), q_ba = mul2(ba2, W2);
  return to_bytes(make_float2(sat_add(p_rg.x, q_rg.x), sat_add(p_rg.y, q_rg.y)),
                  make_float2(sat_add(p_ba.x, q_ba.x), sat_add(p_ba.y, q_ba.y)));
}

template <class Ch>
__device__ __forceinline__ Argb mix_n(const Ch &ch, float w1n, uint32_t c1, float w2n,
                                      uint32_t c2) {
  return mix_ch(w1n, make_float2(ch(c1, 2), ch(c1, 1)), make_float2(ch(c1, 0), ch(c1, 3)), w2n,
                make_float2(ch(c2, 2), ch(c2, 1)), make_float2(ch(c2, 0), ch(c2, 3)));
}

template <class Ch>
__device__ __forceinline__ uint32_t mix(const Ch &ch, float w1, uint32_t c1, float w2,
                                        uint32_t c2) {
  float w1n, w2n;
  mix_weights(w1, w2, w1n, w2n);
  return pack(mix_n(ch, w1n, c1, w2n, c2));
}

/* matte colourspace.scale: RGB times s, alpha kept, then from_rgba. */
template <class Ch>
__device__ __forceinline__ uint32_t scale(const Ch &ch, uint32_t c, float s) {
  const float2 rg = mul2(make_float2(ch(c, 2), ch(c, 1)), make_float2(s, s));
  const float b = fm(ch(c, 0), s);
  return pack_argb(make_float2(sat_add(rg.x, 0.0f), sat_add(rg.y, 0.0f)),
                   make_float2(sat_add(b, 0.0f), sat_add(ch(c, 3), 0.0f)));
}

/* The optional shading / fog epilogue of one sample at depth z (FSV_SHADE,
 * FSV_FOG); not part of the reference's path. */
template <class Ch>
__device__ __forceinline__ uint32_t apply_effects(const Ch &ch, const FsView &V, uint32_t c,
                                                  float z) {
  if (V.flags & FSV_SHADE) c = scale(ch, c, fs(1.0f, fm(V.shade, fd(z, V.distance))));
  if (V.flags & FSV_FOG) {
    float f = fd(fs(z, V.fog_start), fs(V.fog_end, V.fog_start));
    f = (f < 0.0f) ? 0.0f : ((f > 1.0f) ? 1.0f : f);
    c = mix(ch, fs(1.0f, f), c, f, V.fog_color);
  }
  return c;
}

/* png_color_filtered, fut/render_functions.fut:95-105. Both x mixes share one
 * weight normalisation. P2: the colour map's sides are powers of two (the
 * wrap is a mask), known at compile time so the four index computations and
 * gathers form one straight-line block. */
template <bool P2, class Ch>
__device__ __forceinline__ uint32_t color_bilinear(const FsMapDev &M, const Ch &ch, float x,
                                                   float y) {
  const float fx = floorf(x), cx = ceilf(x), fy = floorf(y), cy = ceilf(y);
  const int32_t ix0 = wrap_t<P2>(f2i(fx), M.CW), ix1 = wrap_t<P2>(f2i(cx), M.CW);
  const int32_t iy0 = wrap_t<P2>(f2i(fy), M.CH), iy1 = wrap_t<P2>(f2i(cy), M.CH);
  const uint32_t *r0 = M.c + (uint32_t)(iy0 * M.CW);
  const uint32_t *r1 = M.c + (uint32_t)(iy1 * M.CW);
  const uint32_t c00 = __ldg(r0 + ix0), c01 = __ldg(r0 + ix1);
  const uint32_t c10 = __ldg(r1 + ix0), c11 = __ldg(r1 + ix1);
  float w0, w1;
  mix_weights(fs(cx, x), fs(x, fx), w0, w1);
  const Argb x1 = mix_n(ch, w0, c00, w1, c01);
  const Argb x2 = mix_n(ch, w0, c10, w1, c11);
  /* the y mix reads the channels of x1 and x2 straight from their bytes */
  float v0, v1;
  mix_weights(fs(cy, y), fs(y, fy), v0, v1);
  return pack(mix_ch(v0, make_float2(ch.bits(x1.r), ch.bits(x1.g)),
                     make_float2(ch.bits(x1.b), ch.bits(x1.a)), v1,
                     make_float2(ch.bits(x2.r), ch.bits(x2.g)),
                     make_float2(ch.bits(x2.b), ch.bits(x2.a))));
}

/* png_color, fut/render_functions.fut:91-92 */
template <bool P2>
__device__ __forceinline__ uint32_t color_nearest(const FsMapDev &M, float x, float y) {
  const int32_t ix = wrap_t<P2>(f2i(x), M.CW), iy = wrap_t<P2>(f2i(y), M.CH);
  return __ldg(M.c + (uint32_t)(iy * M.CW) + ix);
}
__device__ __forceinline__ uint32_t color_nearest(const FsMapDev &M, float x, float y) {
  return M.cpow2 ? color_nearest<true>(M, x, y) : color_nearest<false>(M, x, y);
}

/* The sample colour with the chosen filter (CF: bilinear), the wrap picked
 * once per call from the colour map's shape. */
template <int CF, class Ch>
__device__ __forceinline__ uint32_t color_sample(const FsMapDev &M, const Ch &ch, bool p2,
                                                 float x, float y) {
  if (p2) return CF ? color_bilinear<true>(M, ch, x, y) : color_nearest<true>(M, x, y);
  return CF ? color_bilinear<false>(M, ch, x, y) : color_nearest<false>(M, x, y);
}

}  // namespace fsd
