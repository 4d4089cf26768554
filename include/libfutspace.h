/*
 * Drop-in replacement for the header that `futhark opencl --library
 * fut/interactive_entrypoints.fut` generates (Makefile:24-25, consumed through
 * -DPROGHEADER='"libfutspace.h"' at Makefile:19). The reference's host program
 * c/interactive.c and the lys front end link against these names unchanged;
 * behind them is the futspace_gb300 CUDA renderer.
 *
 * Conventions of the generated API, kept here:
 *  - functions return int, 0 on success; futhark_context_get_error returns the
 *    last error as a malloc'd string the caller frees;
 *  - every array or opaque value returned is owned by the caller and released
 *    with the matching futhark_free_*; entry points never consume inputs;
 *  - opaque states are immutable: every entry returns a new state;
 *  - one context must not be used by two threads at once;
 *  - results may be asynchronous until futhark_context_sync or futhark_values_*.
 */
#ifndef LIBFUTSPACE_H
#define LIBFUTSPACE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct futhark_context_config;
struct futhark_context;
struct futhark_u32_2d;
struct futhark_i32_2d;
struct futhark_opaque_state;

/* ---- configuration and context ------------------------------------------ */
struct futhark_context_config *futhark_context_config_new(void);
void futhark_context_config_free(struct futhark_context_config *cfg);
/* Selects the CUDA device: "3", "cuda:3" or "#3". Unparsable names keep 0. */
void futhark_context_config_set_device(struct futhark_context_config *cfg, const char *s);
void futhark_context_config_set_debugging(struct futhark_context_config *cfg, int flag);
void futhark_context_config_set_logging(struct futhark_context_config *cfg, int flag);
void futhark_context_config_set_profiling(struct futhark_context_config *cfg, int flag);
void futhark_context_config_select_device_interactively(struct futhark_context_config *cfg);
struct futhark_context *futhark_context_new(struct futhark_context_config *cfg);
void futhark_context_free(struct futhark_context *ctx);
int futhark_context_sync(struct futhark_context *ctx);
char *futhark_context_get_error(struct futhark_context *ctx);
int futhark_context_clear_caches(struct futhark_context *ctx);
char *futhark_context_report(struct futhark_context *ctx);

/* ---- arrays ---------------------------------------------------------------
 * futhark_new_*: copies host data [dim0][dim1] to the device (the caller keeps
 * its buffer, c/interactive.c:50-53). futhark_values_*: copies back to host and
 * waits. */
struct futhark_u32_2d *futhark_new_u32_2d(struct futhark_context *ctx, const uint32_t *data,
                                          int64_t dim0, int64_t dim1);
struct futhark_i32_2d *futhark_new_i32_2d(struct futhark_context *ctx, const int32_t *data,
                                          int64_t dim0, int64_t dim1);
int futhark_free_u32_2d(struct futhark_context *ctx, struct futhark_u32_2d *arr);
int futhark_free_i32_2d(struct futhark_context *ctx, struct futhark_i32_2d *arr);
int futhark_values_u32_2d(struct futhark_context *ctx, struct futhark_u32_2d *arr,
                          uint32_t *data);
int futhark_values_i32_2d(struct futhark_context *ctx, struct futhark_i32_2d *arr,
                          int32_t *data);
const int64_t *futhark_shape_u32_2d(struct futhark_context *ctx, struct futhark_u32_2d *arr);
const int64_t *futhark_shape_i32_2d(struct futhark_context *ctx, struct futhark_i32_2d *arr);
/* Device address of the array's data (a CUdeviceptr). */
unsigned char *futhark_values_raw_u32_2d(struct futhark_context *ctx,
                                         struct futhark_u32_2d *arr);
int futhark_free_opaque_state(struct futhark_context *ctx, struct futhark_opaque_state *obj);

/* ---- entry points (fut/interactive_entrypoints.fut:6-32) ------------------ */
int futhark_entry_init(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                       const uint32_t seed);
int futhark_entry_resize(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                         const int32_t h, const int32_t w,
                         const struct futhark_opaque_state *in);
int futhark_entry_key(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                      const int32_t e, const int32_t key, const struct futhark_opaque_state *in);
int futhark_entry_mouse(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                        const int32_t buttons, const int32_t x, const int32_t y,
                        const struct futhark_opaque_state *in);
int futhark_entry_wheel(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                        const int32_t dx, const int32_t dy,
                        const struct futhark_opaque_state *in);
int futhark_entry_step(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                       const float td, const struct futhark_opaque_state *in);
int futhark_entry_render(struct futhark_context *ctx, struct futhark_u32_2d **out0,
                         const struct futhark_opaque_state *in);
int futhark_entry_text_content(struct futhark_context *ctx, float *x, float *y, float *angle,
                               float *height, float *horizon, float *distance,
                               float *sun_height, float *sun_ang, float *fov,
                               const struct futhark_opaque_state *in);
int futhark_entry_update_map(struct futhark_context *ctx, struct futhark_opaque_state **out0,
                             const struct futhark_u32_2d *color_map,
                             const struct futhark_i32_2d *height_map,
                             const struct futhark_opaque_state *in);

#ifdef __cplusplus
}
#endif
#endif
