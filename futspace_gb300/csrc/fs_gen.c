/*
 * Seeded synthetic inputs: diamond-square height maps, palette colour maps and
 * cameras. Built with -ffp-contract=off and using only + - * / on doubles and
 * floats (no libm), so x86 and Arm hosts produce identical bytes for a seed.
 * The PRNG is splitmix64.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/futspace_gb300.h"

static uint64_t sm64(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* uniform in [0, 1) with 53 random bits */
static double u01(uint64_t *s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }

/* sin and cos by argument reduction to [-pi, pi] and Taylor series; only the
 * camera-walk generator uses them, never the renderer. */
static void gen_sincos(double a, double *sn, double *cs) {
  const double two_pi = 6.283185307179586476925;
  const double pi = 3.141592653589793238463;
  double k = (double)(int64_t)(a / two_pi);
  double r = a - k * two_pi;
  while (r > pi) r -= two_pi;
  while (r < -pi) r += two_pi;
  double r2 = r * r;
  double term = r, s = r;
  for (int i = 1; i < 14; i++) {
    term = -term * r2 / (double)((2 * i) * (2 * i + 1));
    s = s + term;
  }
  term = 1.0;
  double c = 1.0;
  for (int i = 1; i < 14; i++) {
    term = -term * r2 / (double)((2 * i - 1) * (2 * i));
    c = c + term;
  }
  *sn = s;
  *cs = c;
}

int fsgen_heights(uint64_t seed, int32_t size, float roughness, uint8_t *out) {
  if (!out || size < 2 || (size & (size - 1)) != 0) return FS_ERR_ARG;
  const int64_t N = size;
  float *f = (float *)malloc(sizeof(float) * (size_t)(N * N));
  if (!f) return FS_ERR_NOMEM;
  uint64_t s = seed ^ 0x5eed0f7e11a1ull;
#define F(yy, xx) f[(((yy) & (N - 1)) * N) + ((xx) & (N - 1))]
  F(0, 0) = 0.0f;
  float amp = 1.0f;
  for (int64_t step = N; step > 1; step /= 2) {
    const int64_t half = step / 2;
    /* diamond: centre of each square */
    for (int64_t y = 0; y < N; y += step)
      for (int64_t x = 0; x < N; x += step) {
        float avg = (F(y, x) + F(y, x + step) + F(y + step, x) + F(y + step, x + step)) * 0.25f;
        F(y + half, x + half) = avg + (float)(u01(&s) * 2.0 - 1.0) * amp;
      }
    /* square: midpoint of each edge */
    for (int64_t y = 0; y < N; y += half)
      for (int64_t x = ((y / half) & 1) ? 0 : half; x < N; x += step) {
        float avg = (F(y - half, x) + F(y + half, x) + F(y, x - half) + F(y, x + half)) * 0.25f;
        F(y, x) = avg + (float)(u01(&s) * 2.0 - 1.0) * amp;
      }
    amp = amp * roughness;
  }
#undef F
  float mn = f[0], mx = f[0];
  for (int64_t i = 1; i < N * N; i++) {
    if (f[i] < mn) mn = f[i];
    if (f[i] > mx) mx = f[i];
  }
  const double span = (double)mx - (double)mn;
  for (int64_t i = 0; i < N * N; i++) {
    double v = span > 0.0 ? ((double)f[i] - (double)mn) / span * 255.0 : 0.0;
    int32_t b = (int32_t)(v + 0.5);
    out[i] = (uint8_t)(b < 0 ? 0 : (b > 255 ? 255 : b));
  }
  free(f);
  return FS_OK;
}

/* 5-stop terrain palette: deep water, sand, grass, rock, snow. */
static const int32_t k_stops[5][4] = {
    {0, 24, 52, 120}, {72, 196, 178, 128}, {120, 62, 138, 52}, {190, 116, 104, 92},
    {255, 246, 246, 250}};

int fsgen_colors(uint64_t seed, const uint8_t *heights, int64_t count, int32_t noise,
                 uint32_t *out) {
  if (!heights || !out || count < 0 || noise < 0 || noise > 127) return FS_ERR_ARG;
  uint64_t s = seed ^ 0xc01065eedull;
  for (int64_t i = 0; i < count; i++) {
    const int32_t h = heights[i];
    int seg = 0;
    while (seg < 3 && h > k_stops[seg + 1][0]) seg++;
    const int32_t h0 = k_stops[seg][0], h1 = k_stops[seg + 1][0];
    const int32_t span = h1 - h0, t = h - h0;
    int32_t ch[3];
    for (int c = 0; c < 3; c++) {
      int32_t v = (k_stops[seg][c + 1] * (span - t) + k_stops[seg + 1][c + 1] * t + span / 2) / span;
      v += (int32_t)(sm64(&s) % (uint64_t)(2 * noise + 1)) - noise;
      ch[c] = v < 0 ? 0 : (v > 255 ? 255 : v);
    }
    out[i] = 0xFF000000u | ((uint32_t)ch[0] << 16) | ((uint32_t)ch[1] << 8) | (uint32_t)ch[2];
  }
  return FS_OK;
}

int32_t fsgen_local_max(const uint8_t *heights, int32_t rows, int32_t cols, float x, float y) {
  if (!heights || rows <= 0 || cols <= 0) return 0;
  int64_t ix = (int64_t)x, iy = (int64_t)y;
  if ((float)ix > x) ix -= 1; /* floor */
  if ((float)iy > y) iy -= 1;
  int32_t mx = 0;
  for (int64_t dy = -8; dy < 8; dy++)
    for (int64_t dx = -8; dx < 8; dx++) {
      int64_t yy = ((iy + dy) % rows + rows) % rows;
      int64_t xx = ((ix + dx) % cols + cols) % cols;
      int32_t h = heights[yy * cols + xx];
      if (h > mx) mx = h;
    }
  return mx;
}

int fsgen_cameras(uint64_t seed, const uint8_t *heights, int32_t rows, int32_t cols,
                  int32_t count, float above_lo, float above_hi, float distance_lo,
                  float distance_hi, int32_t screen_h, fs_camera *out) {
  if (!heights || !out || rows <= 0 || cols <= 0 || count < 0) return FS_ERR_ARG;
  uint64_t s = seed ^ 0xca3e7a5ull;
  for (int32_t i = 0; i < count; i++) {
    fs_camera c;
    memset(&c, 0, sizeof(c));
    c.x = (float)(u01(&s) * (double)cols);
    c.y = (float)(u01(&s) * (double)rows);
    c.angle = (float)(u01(&s) * 6.283185307179586);
    const double above = (double)above_lo + u01(&s) * ((double)above_hi - (double)above_lo);
    c.height = (float)((double)fsgen_local_max(heights, rows, cols, c.x, c.y) + above);
    c.distance =
        (float)((double)distance_lo + u01(&s) * ((double)distance_hi - (double)distance_lo));
    c.horizon = (float)(screen_h / 2);
    c.fov = 1.2f; /* fut/interactive.fut:35 */
    c.sky_color = 0xFF9090E0u; /* tests/futspace.fut:143 */
    out[i] = c;
  }
  return FS_OK;
}

int fsgen_walk(uint64_t seed, const uint8_t *heights, int32_t rows, int32_t cols, int32_t count,
               float step, float yaw, float above_lo, float above_hi, float distance,
               int32_t screen_h, fs_camera *out) {
  if (!heights || !out || rows <= 0 || cols <= 0 || count < 0) return FS_ERR_ARG;
  uint64_t s = seed ^ 0x3a1c3a1cull;
  double x = u01(&s) * (double)cols, y = u01(&s) * (double)rows;
  double ang = u01(&s) * 6.283185307179586;
  double above = ((double)above_lo + (double)above_hi) * 0.5;
  for (int32_t i = 0; i < count; i++) {
    if (i > 0) {
      ang = ang + (u01(&s) * 2.0 - 1.0) * (double)yaw;
      double sn, cs;
      gen_sincos(ang, &sn, &cs);
      /* forward is (-sin, -cos), as the W key moves (fut/interactive.fut:91-97) */
      x = x - (double)step * sn;
      y = y - (double)step * cs;
      above = above + (u01(&s) * 2.0 - 1.0) * 5.0;
      if (above < (double)above_lo) above = (double)above_lo;
      if (above > (double)above_hi) above = (double)above_hi;
    }
    fs_camera c;
    memset(&c, 0, sizeof(c));
    c.x = (float)x;
    c.y = (float)y;
    c.angle = (float)ang;
    c.height = (float)((double)fsgen_local_max(heights, rows, cols, c.x, c.y) + above);
    c.distance = distance;
    c.horizon = (float)(screen_h / 2);
    c.fov = 1.2f;
    c.sky_color = 0xFF9090E0u;
    out[i] = c;
  }
  return FS_OK;
}
