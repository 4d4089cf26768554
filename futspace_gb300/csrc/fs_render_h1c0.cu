/* Render kernels with height filter 1 and colour filter 0 (1 = bilinear). */
#define FS_HF 1
#define FS_CF 0
#define FS_RENDER_ENTRY fsk_render_h1c0
#define FS_SEGMIN_ENTRY fsk_segmin_h1
#include "fs_render_inst.cuh"
