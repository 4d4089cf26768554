/*
 * CPU oracle for the voxel-space render path: TEST INFRASTRUCTURE ONLY.
 * PARITY UNPINNED (no reference outputs exist; see fs_oracle.h).
 *
 * A plain-C restatement of the reference arithmetic, compiled with
 * -ffp-contract=off so every f32 operation rounds exactly once, in the order the
 * Futhark source writes it. The render follows the reference's data-parallel
 * structure literally: a [n][w] map of (colour,row) pairs, then per column an
 * inclusive `occlude` scan, a scatter into an [h] column, a `fill_vline` scan,
 * the sky substitution and a transpose (fut/voxel_renderer.fut:214-251). The
 * GPU kernels use a different (event/interval) formulation; the tests check
 * that the two agree bit for bit.
 */
#include "fs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* f32 -> i32 conversion `i32.f32`. The reference's GPU targets convert with a
 * saturating instruction: NaN -> 0, values beyond the i32 range clamp, finite
 * values truncate toward zero. The explicit form matters at z = 0, where
 * inv_z = +inf (fut/voxel_renderer.fut:217, z_1 = 0 from :34). */
int32_t fso_f2i(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return INT32_MAX;
  if (v <= -2147483648.0f) return INT32_MIN;
  return (int32_t)v;
}

/* f32 -> u32 conversion `u32.f32`, same saturating rule (NaN -> 0). */
uint32_t fso_f2u(float v) {
  if (v != v) return 0u;
  if (v <= 0.0f) return 0u;
  if (v >= 4294967296.0f) return UINT32_MAX;
  return (uint32_t)v;
}

/* Futhark `%` on i32 rounds toward negative infinity: the result takes the
 * sign of the divisor (fut/render_functions.fut:64,73-76 index with it). */
int32_t fso_mod(int32_t a, int32_t m) {
  int32_t r = a % m;
  return (r < 0) ? r + m : r;
}

/* ---- matte 0.1.2 (#2ce1a39) colour arithmetic, restated ------------------
 * argb_colour.to_rgba: each byte / 255 as f32 (channel order R,G,B,A).
 * argb_colour.from_rgba: each channel clamped to [0,1], times 255, truncated
 * with u32.f32, packed A<<24 | R<<16 | G<<8 | B.
 * colourspace.mix w1 c1 w2 c2: weights normalised by (w1+w2), each channel
 * r1*w1' + r2*w2', then from_rgba.  colourspace.scale c s: RGB times s, alpha
 * kept, then from_rgba.
 * Call sites on the path: fut/render_functions.fut:101-103 (bilinear colour),
 * fut/interactive.fut:163 (sky = argb.scale 0xFF9090e0 sun_height),
 * fut/effects.fut:123 (shadow darkening). */
static float fso_channel(uint32_t x, int shift) {
  return (float)((x >> shift) & 0xFFu) / 255.0f;
}

static float fso_clamp_channel(float x) {
  return (x < 0.0f) ? 0.0f : ((x > 1.0f) ? 1.0f : x);
}

static uint32_t fso_from_rgba(float r, float g, float b, float a) {
  return (fso_f2u(fso_clamp_channel(a) * 255.0f) << 24) |
         (fso_f2u(fso_clamp_channel(r) * 255.0f) << 16) |
         (fso_f2u(fso_clamp_channel(g) * 255.0f) << 8) |
         fso_f2u(fso_clamp_channel(b) * 255.0f);
}

uint32_t fso_mix(float w1, uint32_t c1, float w2, uint32_t c2) {
  float r1 = fso_channel(c1, 16), g1 = fso_channel(c1, 8), b1 = fso_channel(c1, 0),
        a1 = fso_channel(c1, 24);
  float r2 = fso_channel(c2, 16), g2 = fso_channel(c2, 8), b2 = fso_channel(c2, 0),
        a2 = fso_channel(c2, 24);
  float w1n = w1 / (w1 + w2);
  float w2n = w2 / (w1 + w2);
  float r = r1 * w1n + r2 * w2n;
  float g = g1 * w1n + g2 * w2n;
  float b = b1 * w1n + b2 * w2n;
  float a = a1 * w1n + a2 * w2n;
  return fso_from_rgba(r, g, b, a);
}

uint32_t fso_scale(uint32_t c, float s) {
  float r = fso_channel(c, 16), g = fso_channel(c, 8), b = fso_channel(c, 0),
        a = fso_channel(c, 24);
  return fso_from_rgba(r * s, g * s, b * s, a);
}

/* ---- depth schedule, get_zs (fut/voxel_renderer.fut:28-34) ---------------
 * n = i32(floor((sqrt((d-2*z0)**2 + 8*d*D) - 2*z0 + d) / (2*d)));
 * z_i = (f32 i / 2) * (2*z0 + (f32 i - 1) * d),  i = 1..n.
 * `**` is f32.pow (powf). tests/futspace.fut:47-53 is the same without floor. */
int32_t fso_num_depths(float D, float d, float z0, int32_t floor_n) {
  float t = d - 2.0f * z0;
  float sq = sqrtf(powf(t, 2.0f) + 8.0f * d * D);
  float num = sq - 2.0f * z0 + d;
  float div = 2.0f * d;
  float q = num / div;
  return fso_f2i(floor_n ? floorf(q) : q);
}

int32_t fso_get_zs(float D, float d, float z0, int32_t floor_n, float *zs, int32_t cap) {
  int32_t n = fso_num_depths(D, d, z0, floor_n);
  if (n < 1) return n;
  for (int32_t i = 1; i <= n && i <= cap; i++) {
    float fi = (float)i;
    zs[i - 1] = (fi / 2.0f) * (2.0f * z0 + (fi - 1.0f) * d);
  }
  return n;
}

/* ---- samplers (fut/render_functions.fut) --------------------------------- */

/* png_height_filtered, fut/render_functions.fut:67-77 */
float fso_height_bilinear(const uint8_t *hm, int32_t MH, int32_t MW, float x, float y) {
  float fx = floorf(x), cx = ceilf(x), fy = floorf(y), cy = ceilf(y);
  int32_t iy0 = fso_mod(fso_f2i(fy), MH), iy1 = fso_mod(fso_f2i(cy), MH);
  int32_t ix0 = fso_mod(fso_f2i(fx), MW), ix1 = fso_mod(fso_f2i(cx), MW);
  float h00 = (float)hm[(int64_t)iy0 * MW + ix0];
  float h01 = (float)hm[(int64_t)iy0 * MW + ix1];
  float h10 = (float)hm[(int64_t)iy1 * MW + ix0];
  float h11 = (float)hm[(int64_t)iy1 * MW + ix1];
  float x1 = (cx - x) * h00 + (x - fx) * h01;
  float x2 = (cx - x) * h10 + (x - fx) * h11;
  return (cy - y) * x1 + (y - fy) * x2;
}

/* png_height, fut/render_functions.fut:63-64 (i32.f32 truncates toward zero) */
float fso_height_nearest(const uint8_t *hm, int32_t MH, int32_t MW, float x, float y) {
  int32_t iy = fso_mod(fso_f2i(y), MH), ix = fso_mod(fso_f2i(x), MW);
  return (float)hm[(int64_t)iy * MW + ix];
}

/* png_color_filtered, fut/render_functions.fut:95-105 */
uint32_t fso_color_bilinear(const uint32_t *cm, int32_t MH, int32_t MW, float x, float y) {
  float fx = floorf(x), cx = ceilf(x), fy = floorf(y), cy = ceilf(y);
  int32_t iy0 = fso_mod(fso_f2i(fy), MH), iy1 = fso_mod(fso_f2i(cy), MH);
  int32_t ix0 = fso_mod(fso_f2i(fx), MW), ix1 = fso_mod(fso_f2i(cx), MW);
  uint32_t x1 = fso_mix(cx - x, cm[(int64_t)iy0 * MW + ix0], x - fx, cm[(int64_t)iy0 * MW + ix1]);
  uint32_t x2 = fso_mix(cx - x, cm[(int64_t)iy1 * MW + ix0], x - fx, cm[(int64_t)iy1 * MW + ix1]);
  return fso_mix(cy - y, x1, y - fy, x2);
}

/* png_color, fut/render_functions.fut:91-92 */
uint32_t fso_color_nearest(const uint32_t *cm, int32_t MH, int32_t MW, float x, float y) {
  int32_t iy = fso_mod(fso_f2i(y), MH), ix = fso_mod(fso_f2i(x), MW);
  return cm[(int64_t)iy * MW + ix];
}

/* ---- optional epilogue (not in the reference) ------------------------------
 * Applied to a sample's colour at depth z with draw distance D, in matte's
 * arithmetic: shade c = scale(c, 1 - shade * (z / D)); fog f = clamp((z -
 * fog_start) / (fog_end - fog_start), 0, 1), c = mix(1 - f, c, f, fog). */
static uint32_t fso_effects(const fso_params *p, uint32_t c, float z, float D) {
  if (p->effects & 1) c = fso_scale(c, 1.0f - p->shade * (z / D));
  if (p->effects & 2) {
    float f = (z - p->fog_start) / (p->fog_end - p->fog_start);
    f = (f < 0.0f) ? 0.0f : ((f > 1.0f) ? 1.0f : f);
    c = fso_mix(1.0f - f, c, f, p->fog_color);
  }
  return c;
}

/* ---- render (fut/voxel_renderer.fut:101-251, `#off` branch) -------------- */

typedef struct {
  float start_x, start_y, end_x, end_y;
} fso_line;

/* get_h_line, fut/voxel_renderer.fut:43-60 */
static fso_line fso_get_h_line(float z, const fso_camera *c, int32_t w) {
  float sin_ang = sinf(c->angle);
  float cos_ang = cosf(c->angle);
  float view = c->fov;
  float left_x = (-cos_ang - sin_ang * view) * z;
  float left_y = (sin_ang - cos_ang * view) * z;
  float right_x = (cos_ang - sin_ang * view) * z;
  float right_y = (-sin_ang - cos_ang * view) * z;
  float dx = (right_x - left_x) / (float)w;
  float dy = (right_y - left_y) / (float)w;
  fso_line l;
  l.start_x = left_x + c->x;
  l.start_y = left_y + c->y;
  l.end_x = dx;
  l.end_y = dy;
  return l;
}

static int fso_check(const fso_params *p, const uint8_t *hm, const uint32_t *cm, int32_t MH,
                     int32_t MW, int32_t W, int32_t H, const uint32_t *out) {
  if (!p || !hm || !cm || !out) return -1;
  if (MH <= 0 || MW <= 0 || W <= 0 || H <= 0) return -1;
  return 0;
}

/* Samples one (z, column) pair: lines 218-226 (get_segment :63-66, the
 * samplers, the projection `i32.max 0 (i32.f32 relative_height)`). */
static void fso_sample(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                       int32_t MH, int32_t MW, const uint32_t *cm, int32_t CH, int32_t CW,
                       const fso_line *l, float z, float inv_z, int32_t i, uint32_t *colour,
                       int32_t *row) {
  float x = l->start_x + (float)i * l->end_x;
  float y = l->start_y + (float)i * l->end_y;
  uint32_t c = p->color_filter == FSO_BILINEAR ? fso_color_bilinear(cm, CH, CW, x, y)
                                               : fso_color_nearest(cm, CH, CW, x, y);
  float mh = p->height_filter == FSO_BILINEAR ? fso_height_bilinear(hm, MH, MW, x, y)
                                              : fso_height_nearest(hm, MH, MW, x, y);
  float height_diff = cam->height - mh;
  float relative_height = height_diff * inv_z + cam->horizon;
  int32_t r = fso_f2i(relative_height);
  if (p->effects) c = fso_effects(p, c, z, cam->distance);
  *colour = c;
  *row = r > 0 ? r : 0;
}

/* One screen column: scan occlude (:69-72, :231) with neutral (0, h), scatter
 * into `replicate h gap` dropping rows >= h (:244), scan fill_vline (:78-81,
 * :246) and the sky substitution (:248). The gap value is 0 in the live
 * renderer and the sky colour in tests/futspace.fut:110-121. */
static void fso_column(const uint32_t *cs, const int32_t *rs, int32_t n, int32_t H,
                       uint32_t gap, uint32_t sky, uint32_t *col_acc_c, int32_t *col_acc_r,
                       uint32_t *vline) {
  /* inclusive scan with the reference's operator and neutral element */
  uint32_t acc_c = 0;
  int32_t acc_r = H;
  for (int32_t k = 0; k < n; k++) {
    if (!(acc_r <= rs[k])) {
      acc_c = cs[k];
      acc_r = rs[k];
    }
    col_acc_c[k] = acc_c;
    col_acc_r[k] = acc_r;
  }
  for (int32_t y = 0; y < H; y++) vline[y] = gap;
  for (int32_t k = 0; k < n; k++) {
    int32_t r = col_acc_r[k];
    if (r >= 0 && r < H) vline[r] = col_acc_c[k];
  }
  uint32_t fill = gap;
  for (int32_t y = 0; y < H; y++) {
    if (vline[y] != gap) fill = vline[y];
    vline[y] = (fill == gap) ? sky : fill;
  }
}

/* One screen column of the `#on` branch (fut/voxel_renderer.fut:175-213):
 * scan occlude2 (:88-91) with neutral (0, h, 0) carrying the depth index; the
 * tuples (colour, previous colour, row, previous row, index, previous index)
 * with `rotate (-1)` (the previous element, wrapping to the last); scatter into
 * rows, duplicates written in index order so the last write wins (a sequential
 * `futhark c` scatter); forward fill of whole tuples against the empty tuple
 * (0,0,0,0,1000,1000) (fill_vline3, :93-96); the per-row blend when the two
 * indices are adjacent; 0 -> sky. */
typedef struct {
  uint32_t c, cp;
  int32_t r, rp, i, ip;
} fso_tuple;

static int fso_tuple_empty(const fso_tuple *t) {
  return t->c == 0 && t->cp == 0 && t->r == 0 && t->rp == 0 && t->i == 1000 && t->ip == 1000;
}

static void fso_column_smooth(const uint32_t *cs, const int32_t *rs, int32_t n, int32_t H,
                              uint32_t sky, uint32_t *sc, int32_t *sr, int32_t *si,
                              fso_tuple *line, uint32_t *vline) {
  uint32_t acc_c = 0;
  int32_t acc_r = H, acc_i = 0;
  for (int32_t k = 0; k < n; k++) {
    if (!(acc_r <= rs[k])) {
      acc_c = cs[k];
      acc_r = rs[k];
      acc_i = k;
    }
    sc[k] = acc_c;
    sr[k] = acc_r;
    si[k] = acc_i;
  }
  const fso_tuple empty = {0, 0, 0, 0, 1000, 1000};
  for (int32_t y = 0; y < H; y++) line[y] = empty;
  for (int32_t k = 0; k < n; k++) {
    const int32_t kp = (k == 0) ? n - 1 : k - 1;
    const int32_t r = sr[k];
    if (r >= 0 && r < H) {
      fso_tuple t = {sc[k], sc[kp], sr[k], sr[kp], si[k], si[kp]};
      line[r] = t;
    }
  }
  fso_tuple fill = empty;
  for (int32_t y = 0; y < H; y++) {
    if (!fso_tuple_empty(&line[y])) fill = line[y];
    const fso_tuple *t = &fill;
    const float range = fmaxf(1.0f, (float)(t->rp - t->r));
    const float delta1 = fabsf((float)y - (float)t->rp) / range;
    const float delta2 = fabsf((float)t->r - (float)y) / range;
    const uint32_t col = (t->i - t->ip == 1) ? fso_mix(delta2, t->cp, delta1, t->c) : t->c;
    vline[y] = (col == 0) ? sky : col;
  }
}

static int32_t fso_render_impl(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                               int32_t MH, int32_t MW, const uint32_t *cm, int32_t CH,
                               int32_t CW, int32_t W, int32_t H, uint32_t *out,
                               int32_t threads) {
  if (!cam || fso_check(p, hm, cm, MH, MW, W, H, out) || CH <= 0 || CW <= 0) return -1;
  int32_t n = fso_num_depths(cam->distance, p->d, p->z0, p->floor_n);
  if (n < 1) return -2;
  float *zs = (float *)malloc(sizeof(float) * (size_t)n);
  uint32_t *pc = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n * (size_t)W);
  int32_t *pr = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * (size_t)W);
  if (!zs || !pc || !pr) {
    free(zs);
    free(pc);
    free(pr);
    return -3;
  }
  fso_get_zs(cam->distance, p->d, p->z0, p->floor_n, zs, n);
  float scale = p->scale > 0.0f ? p->scale : (float)(W / 2);
  uint32_t gap = p->gap_rule == FSO_GAP_SKY ? cam->sky_color : 0u;
  int32_t failed = 0;
  (void)threads;

  /* height_color_map: [n][w] pairs (:215-228) */
#pragma omp parallel for schedule(static) num_threads(threads) if (threads != 1)
  for (int32_t k = 0; k < n; k++) {
    fso_line l = fso_get_h_line(zs[k], cam, W);
    float inv_z = (1.0f / zs[k]) * scale;
    for (int32_t i = 0; i < W; i++)
      fso_sample(cam, p, hm, MH, MW, cm, CH, CW, &l, zs[k], inv_z, i, &pc[(size_t)k * W + i],
                 &pr[(size_t)k * W + i]);
  }

  /* per column of (transpose height_color_map) (:229-250), then transpose (:251) */
#pragma omp parallel num_threads(threads) if (threads != 1)
  {
    uint32_t *cs = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
    int32_t *rs = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint32_t *ac = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
    int32_t *ar = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    uint32_t *vline = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)H);
    int32_t *ai = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    fso_tuple *line = (fso_tuple *)malloc(sizeof(fso_tuple) * (size_t)H);
    if (!cs || !rs || !ac || !ar || !vline || !ai || !line) {
#pragma omp atomic write
      failed = 1;
    } else {
#pragma omp for schedule(static)
      for (int32_t i = 0; i < W; i++) {
        for (int32_t k = 0; k < n; k++) {
          cs[k] = pc[(size_t)k * W + i];
          rs[k] = pr[(size_t)k * W + i];
        }
        if (p->smoothing)
          fso_column_smooth(cs, rs, n, H, cam->sky_color, ac, ar, ai, line, vline);
        else
          fso_column(cs, rs, n, H, gap, cam->sky_color, ac, ar, vline);
        for (int32_t y = 0; y < H; y++) out[(size_t)y * W + i] = vline[y];
      }
    }
    free(cs);
    free(rs);
    free(ac);
    free(ar);
    free(vline);
    free(ai);
    free(line);
  }
  free(zs);
  free(pc);
  free(pr);
  return failed ? -3 : 0;
}

int32_t fso_render(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                   const uint32_t *cm, int32_t MH, int32_t MW, int32_t W, int32_t H,
                   uint32_t *out) {
  return fso_render_impl(cam, p, hm, MH, MW, cm, MH, MW, W, H, out, 1);
}

int32_t fso_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int32_t fso_render_mt(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                      const uint32_t *cm, int32_t MH, int32_t MW, int32_t W, int32_t H,
                      uint32_t *out, int32_t threads) {
  if (threads <= 0) threads = fso_max_threads();
  return fso_render_impl(cam, p, hm, MH, MW, cm, MH, MW, W, H, out, threads);
}

int32_t fso_render_split(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                         int32_t MH, int32_t MW, const uint32_t *cm, int32_t CH, int32_t CW,
                         int32_t W, int32_t H, uint32_t *out, int32_t threads) {
  if (threads <= 0) threads = fso_max_threads();
  return fso_render_impl(cam, p, hm, MH, MW, cm, CH, CW, W, H, out, threads);
}

/* ---- shadowed colour map, generate_shadowmap_accumulated ------------------
 * fut/effects.fut:108-125 with height_fun = png_height and color_fun =
 * png_color (fut/interactive.fut:344-346). Output is fixed at 1024x1024
 * (:124-125) whatever the map size; samples wrap with the map's own size. */
int32_t fso_shadowmap(const uint8_t *hm, const uint32_t *cm, int32_t MH, int32_t MW,
                      const float sun[3], uint32_t *out, int32_t threads) {
  if (!hm || !cm || !sun || !out || MH <= 0 || MW <= 0) return -1;
  if (threads <= 0) threads = fso_max_threads();
  const int32_t max_dist = 1024, steps_per_ray = 256;
  const float step_size = (float)(max_dist / steps_per_ray);
  const uint32_t black = fso_from_rgba(0.0f, 0.0f, 0.0f, 1.0f);
  (void)threads;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads != 1)
  for (int32_t y = 0; y < 1024; y++) {
    for (int32_t x = 0; x < 1024; x++) {
      float fx = (float)x, fy = (float)y;
      float height = fso_height_nearest(hm, MH, MW, fx, fy);
      int32_t count = 0;
      for (int32_t dist = 1; dist < steps_per_ray; dist++) {
        float fdist = (float)dist;
        float hx = fx + fdist * step_size * sun[0];
        float hy = fy + fdist * step_size * sun[2];
        float lhs = height + fdist * step_size * sun[1] - fso_height_nearest(hm, MH, MW, hx, hy);
        if (lhs < -0.5f) count += 1;
      }
      float amount = (float)count;
      out[(size_t)y * 1024 + x] =
          fso_mix(step_size * amount, black, 1.0f, fso_color_nearest(cm, MH, MW, fx, fy));
    }
  }
  return 0;
}
