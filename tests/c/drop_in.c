/*
 * A C consumer of include/libfutspace.h, the drop-in for the header that
 * `futhark opencl --library` generates. It makes the calls the reference's host
 * program makes, with that program's own types and call shapes:
 *   - futhark_entry_init(ctx, &state, seed)                  (c/interactive.c:99)
 *   - map load: futhark_new_u32_2d / futhark_new_i32_2d from uint32_t* and
 *     int32_t* host buffers that are freed right after, then
 *     futhark_entry_update_map(ctx, &state, colour, height, state) and
 *     futhark_free_u32_2d / futhark_free_i32_2d          (c/interactive.c:43-56)
 *   - futhark_entry_text_content with nine float pointers  (c/interactive.c:60-71)
 * and then what the lys front end drives each frame: resize, key, step, render,
 * futhark_shape_u32_2d and futhark_values_u32_2d.
 *
 * Usage: drop_in COLOUR.raw HEIGHT.raw ROWS COLS OUT.raw
 * COLOUR.raw holds ROWS*COLS u32 ARGB words, HEIGHT.raw ROWS*COLS i32 heights
 * (little-endian). OUT.raw receives the nine text_content floats, then the
 * frame's two i64 dimensions and its u32 pixels, after this session: a
 * 160x120 screen, W held for three 16 ms steps, then one more step.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "libfutspace.h"

#define CHECK(ctx, call)                                            \
  do {                                                              \
    if ((call) != 0) {                                              \
      char *msg_ = futhark_context_get_error(ctx);                  \
      fprintf(stderr, "%s failed: %s\n", #call, msg_ ? msg_ : "?"); \
      free(msg_);                                                   \
      return 1;                                                     \
    }                                                               \
  } while (0)

static void *load_raw(const char *path, size_t bytes) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  void *p = malloc(bytes);
  if (p && fread(p, 1, bytes, f) != bytes) {
    free(p);
    p = NULL;
  }
  fclose(f);
  return p;
}

/* Replaces *state with the result of an entry point, freeing the old state. */
static void swap_state(struct futhark_context *ctx, struct futhark_opaque_state **state,
                       struct futhark_opaque_state *next) {
  futhark_free_opaque_state(ctx, *state);
  *state = next;
}

int main(int argc, char **argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s COLOUR.raw HEIGHT.raw ROWS COLS OUT.raw\n", argv[0]);
    return 2;
  }
  const int width = atoi(argv[4]), height = atoi(argv[3]);
  struct futhark_context_config *cfg = futhark_context_config_new();
  futhark_context_config_set_device(cfg, "0");
  struct futhark_context *ctx = futhark_context_new(cfg);
  if (!ctx) {
    fprintf(stderr, "futhark_context_new failed\n");
    return 1;
  }
  struct futhark_opaque_state *state = NULL;
  int seed = 7;
  CHECK(ctx, futhark_entry_init(ctx, &state, seed));

  /* the map load, with the reference's buffer types and call shapes */
  uint32_t *colormap_data = (uint32_t *)load_raw(argv[1], (size_t)width * height * 4);
  int32_t *heightmap_data = (int32_t *)load_raw(argv[2], (size_t)width * height * 4);
  if (!colormap_data || !heightmap_data) {
    fprintf(stderr, "cannot read the map files\n");
    return 1;
  }
  struct futhark_u32_2d *colormap_fut = futhark_new_u32_2d(ctx, colormap_data, height, width);
  struct futhark_i32_2d *heightmap_fut = futhark_new_i32_2d(ctx, heightmap_data, height, width);
  free(colormap_data);
  free(heightmap_data);
  if (!colormap_fut || !heightmap_fut) {
    fprintf(stderr, "futhark_new_*_2d failed\n");
    return 1;
  }
  struct futhark_opaque_state *before = state;
  CHECK(ctx, futhark_entry_update_map(ctx, &state, colormap_fut, heightmap_fut, state));
  futhark_free_opaque_state(ctx, before);
  futhark_free_u32_2d(ctx, colormap_fut);
  futhark_free_i32_2d(ctx, heightmap_fut);

  /* a session: 160x120 screen, W held for three steps, then released */
  struct futhark_opaque_state *next = NULL;
  CHECK(ctx, futhark_entry_resize(ctx, &next, 120, 160, state));
  swap_state(ctx, &state, next);
  CHECK(ctx, futhark_entry_key(ctx, &next, 0, 'w', state));
  swap_state(ctx, &state, next);
  for (int i = 0; i < 3; i++) {
    CHECK(ctx, futhark_entry_step(ctx, &next, 0.016f, state));
    swap_state(ctx, &state, next);
  }
  CHECK(ctx, futhark_entry_key(ctx, &next, 1, 'w', state));
  swap_state(ctx, &state, next);
  CHECK(ctx, futhark_entry_step(ctx, &next, 0.016f, state));
  swap_state(ctx, &state, next);

  float x, y, angle, cam_height, horizon, distance, sun_height, sun_ang, fov;
  CHECK(ctx, futhark_entry_text_content(ctx, &x, &y, &angle, &cam_height, &horizon, &distance,
                                        &sun_height, &sun_ang, &fov, state));
  struct futhark_u32_2d *frame = NULL;
  CHECK(ctx, futhark_entry_render(ctx, &frame, state));
  const int64_t *shape = futhark_shape_u32_2d(ctx, frame);
  const int64_t dims[2] = {shape[0], shape[1]};
  uint32_t *pixels = (uint32_t *)malloc((size_t)(dims[0] * dims[1]) * sizeof(uint32_t));
  if (!pixels) return 1;
  CHECK(ctx, futhark_values_u32_2d(ctx, frame, pixels));
  CHECK(ctx, futhark_context_sync(ctx));

  FILE *out = fopen(argv[5], "wb");
  if (!out) return 1;
  const float text[9] = {x, y, angle, cam_height, horizon, distance, sun_height, sun_ang, fov};
  int ok = fwrite(text, sizeof(float), 9, out) == 9 && fwrite(dims, sizeof(int64_t), 2, out) == 2 &&
           fwrite(pixels, sizeof(uint32_t), (size_t)(dims[0] * dims[1]), out) ==
               (size_t)(dims[0] * dims[1]);
  fclose(out);
  free(pixels);
  futhark_free_u32_2d(ctx, frame);
  futhark_free_opaque_state(ctx, state);
  futhark_context_free(ctx);
  futhark_context_config_free(cfg);
  return ok ? 0 : 1;
}
