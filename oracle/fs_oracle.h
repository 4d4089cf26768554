/*
 * CPU oracle for the voxel-space render path: TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this library, and only as the checker (or the timed CPU stand-in). The product
 * path (futspace_gb300/) never links or calls it.
 *
 * PARITY UNPINNED: the reference (MrHootJones/futspace) ships no golden outputs
 * and its Futhark sources cannot be compiled in this environment (no `futhark`
 * compiler; lys/matte/linalg are not vendored). This file is a line-by-line C
 * restatement of the reference arithmetic; every function cites the reference
 * line it follows. The colour arithmetic of `argb.mix` / `argb.scale` lives in
 * the third-party package github.com/athas/matte 0.1.2 (#2ce1a39, pinned in
 * futhark.pkg:3), which is absent; it is restated from that package's published
 * definition (see fso_mix below).
 */
#ifndef FS_ORACLE_H
#define FS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* camera record, fut/voxel_renderer.fut:5-12 */
typedef struct {
  float x, y, height, angle, horizon, distance, fov;
  uint32_t sky_color;
} fso_camera;

enum { FSO_NEAREST = 0, FSO_BILINEAR = 1 };
enum { FSO_GAP_ZERO = 0, FSO_GAP_SKY = 1 };

/* render parameters (see futspace_gb300.h fs_params for the meaning of each) */
typedef struct {
  float d;          /* depth step (invz_param1), fut/voxel_renderer.fut:104 */
  float z0;         /* first depth (invz_param2), fut/voxel_renderer.fut:103 */
  float scale;      /* projection scale (magic_number); <= 0 means f32(w/2), :217 */
  int32_t height_filter;
  int32_t color_filter;
  int32_t gap_rule;
  int32_t floor_n;  /* 1: n = i32(floor(num/div)) (:32); 0: i32(num/div) (tests/futspace.fut:51) */
  int32_t effects;  /* optional epilogue, not in the reference: 1 shade, 2 fog */
  float shade;
  float fog_start, fog_end;
  uint32_t fog_color;
  int32_t smoothing; /* 1: the `#on` branch, fut/voxel_renderer.fut:175-213 */
} fso_params;

int32_t  fso_f2i(float v);
uint32_t fso_f2u(float v);
int32_t  fso_mod(int32_t a, int32_t m);
uint32_t fso_mix(float w1, uint32_t c1, float w2, uint32_t c2);
uint32_t fso_scale(uint32_t c, float s);
int32_t  fso_num_depths(float D, float d, float z0, int32_t floor_n);
int32_t  fso_get_zs(float D, float d, float z0, int32_t floor_n, float *zs, int32_t cap);
float    fso_height_bilinear(const uint8_t *hm, int32_t MH, int32_t MW, float x, float y);
float    fso_height_nearest(const uint8_t *hm, int32_t MH, int32_t MW, float x, float y);
uint32_t fso_color_bilinear(const uint32_t *cm, int32_t MH, int32_t MW, float x, float y);
uint32_t fso_color_nearest(const uint32_t *cm, int32_t MH, int32_t MW, float x, float y);

/* Renders one [H][W] ARGB frame exactly as the reference's scan/scatter/scan
 * pipeline does (fut/voxel_renderer.fut:214-251). Returns 0, or -1 on bad
 * arguments, -2 when the depth schedule is empty, -3 on allocation failure. */
int32_t fso_render(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                   const uint32_t *cm, int32_t MH, int32_t MW, int32_t W, int32_t H,
                   uint32_t *out);
/* Same result; columns are split across `threads` OpenMP threads (0 = all). */
int32_t fso_render_mt(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                      const uint32_t *cm, int32_t MH, int32_t MW, int32_t W, int32_t H,
                      uint32_t *out, int32_t threads);
int32_t fso_max_threads(void);
/* Height map [MH][MW] and colour map [CH][CW] of different sizes (the
 * interactive app samples the 1024x1024 shadowed colours over any height map). */
int32_t fso_render_split(const fso_camera *cam, const fso_params *p, const uint8_t *hm,
                         int32_t MH, int32_t MW, const uint32_t *cm, int32_t CH, int32_t CW,
                         int32_t W, int32_t H, uint32_t *out, int32_t threads);

/* Shadowed colour map, fut/effects.fut:108-125 (1024x1024 output, fixed). */
int32_t fso_shadowmap(const uint8_t *hm, const uint32_t *cm, int32_t MH, int32_t MW,
                      const float sun[3], uint32_t *out /* [1024][1024] */, int32_t threads);

#ifdef __cplusplus
}
#endif
#endif
