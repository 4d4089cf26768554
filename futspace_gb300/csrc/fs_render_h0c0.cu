/* Render kernels with height filter 0 and colour filter 0 (1 = bilinear). */
#define FS_HF 0
#define FS_CF 0
#define FS_RENDER_ENTRY fsk_render_h0c0
#define FS_SEGMIN_ENTRY fsk_segmin_h0
#include "fs_render_inst.cuh"
