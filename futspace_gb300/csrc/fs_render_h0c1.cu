/* Render kernels with height filter 0 and colour filter 1 (1 = bilinear). */
#define FS_HF 0
#define FS_CF 1
#define FS_RENDER_ENTRY fsk_render_h0c1
#include "fs_render_inst.cuh"
