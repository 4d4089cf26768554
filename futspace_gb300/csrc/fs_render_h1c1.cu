/* Render kernels with height filter 1 and colour filter 1 (1 = bilinear). */
#define FS_HF 1
#define FS_CF 1
#define FS_RENDER_ENTRY fsk_render_h1c1
#include "fs_render_inst.cuh"
