/*
 * Instantiates the render kernels for one (height filter, colour filter) pair:
 * every configuration of FS_TUNE_LIST, FS_TUNE_LIST_MODES, FS_COOP_LIST and
 * FS_COOP_LIST_FX. Included by fs_render_h?c?.cu with
 * FS_HF, FS_CF and FS_RENDER_ENTRY defined, so the four pairs compile as
 * separate translation units in parallel.
 *
 * op 0: launch `grid` CTAs; op 1: occupancy query (CTAs per SM) into *occ;
 * op 2: launch with programmatic stream serialization.
 */
#include <string.h>

#include "fs_render.cuh"

#ifndef FS_LAUNCH_HELPER
#define FS_LAUNCH_HELPER
/* op 0: a plain launch; op 2: with programmatic stream serialization */
template <class K>
static int fs_launch(int op, K kern, int grid, int block, size_t smem, cudaStream_t st,
                     const FsLaunch *L) {
  if (op == 2) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return (int)cudaLaunchKernelEx(&cfg, kern, *L);
  }
  kern<<<grid, block, smem, st>>>(*L);
  return (int)cudaGetLastError();
}
#endif

extern "C" int FS_RENDER_ENTRY(int op, const FsLaunch *L, const FsTune *t, int grid,
                               size_t smem, cudaStream_t st, int *occ) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= 64) return (int)cudaErrorInvalidDevice;
#define FS_CASE(TW_, LC_, U_, STG_) \
  FS_CASE_S(TW_, LC_, U_, STG_, 0, 0, 0) FS_CASE_S(TW_, LC_, U_, STG_, 0, 0, 1)
#define FS_CASE_M(TW_, LC_, U_, STG_, SM_, FX_) FS_CASE_S(TW_, LC_, U_, STG_, SM_, FX_, 0)
/* SEG: kernels that read depth segments, for direct painting only (a staged
 * configuration maps to its one kernel) */
#define FS_CASE_S(TW_, LC_, U_, STG_, SM_, FX_, SEG_)                                        \
  if (t->tw == TW_ && t->lc == LC_ && t->u == U_ && t->stage == STG_ && t->smooth == SM_ &&  \
      t->fx == FX_ && (t->seg != 0) == (SEG_ != 0)) {                                       \
    static int smem_set[64];                                                               \
    auto kern = fsd::render_kernel<TW_, LC_, U_, FS_HF, FS_CF, STG_, SM_, FX_, (SEG_ && !STG_)>; \
    if (smem_set[dev] < (int)smem) {                                                       \
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
      if (e != cudaSuccess) return (int)e;                                                 \
      smem_set[dev] = (int)smem;                                                           \
    }                                                                                      \
    if (op == 1) return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern,      \
                                                                           TW_ * LC_, smem); \
    return fs_launch(op, kern, grid, TW_ * LC_, smem, st, L);                             \
  }
  FS_TUNE_LIST(FS_CASE)
  FS_TUNE_LIST_MODES(FS_CASE_M)
#undef FS_CASE
#undef FS_CASE_M
#undef FS_CASE_S
/* the cooperative tile form (plain mode; a few configurations with the
 * epilogue) */
#define FS_COOP_CASE(TW_, TPC_, U_) FS_COOP_CASE_F(TW_, TPC_, U_, 0)
#define FS_COOP_CASE_FX(TW_, TPC_, U_) FS_COOP_CASE_F(TW_, TPC_, U_, 1)
#define FS_COOP_CASE_F(TW_, TPC_, U_, FX_)                                                   \
  if (t->stage == 2 && t->tw == TW_ && t->lc == TPC_ && t->u == U_ && !t->smooth &&         \
      t->fx == FX_) {                                                                      \
    static int smem_set[64];                                                               \
    auto kern = fsd::coop_kernel<TW_, TPC_, U_, FS_HF, FS_CF, FX_>;                        \
    if (smem_set[dev] < (int)smem) {                                                       \
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
      if (e != cudaSuccess) return (int)e;                                                 \
      smem_set[dev] = (int)smem;                                                           \
    }                                                                                      \
    if (op == 1) return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern,      \
                                                                           TW_ * TPC_, smem); \
    return fs_launch(op, kern, grid, TW_ * TPC_, smem, st, L);                            \
  }
  FS_COOP_LIST(FS_COOP_CASE)
  FS_COOP_LIST_FX(FS_COOP_CASE_FX)
#undef FS_COOP_CASE
#undef FS_COOP_CASE_FX
#undef FS_COOP_CASE_F
  return (int)cudaErrorInvalidValue;
}

#if FS_CF == 0
/* The segment-minimum pass (no colours: compiled once per height filter) for
 * every direct-paint configuration. */
extern "C" int FS_SEGMIN_ENTRY(const FsLaunch *L, const FsTune *t, int grid, cudaStream_t st) {
#define FS_SEG_CASE(TW_, LC_, U_, STG_)                                   \
  if (STG_ == 0 && t->tw == TW_ && t->lc == LC_ && t->u == U_ && !t->stage) { \
    fsd::segmin_kernel<TW_, LC_, U_, FS_HF><<<grid, TW_ * LC_, 0, st>>>(*L); \
    return (int)cudaGetLastError();                                       \
  }
  FS_TUNE_LIST(FS_SEG_CASE)
#undef FS_SEG_CASE
  return (int)cudaErrorInvalidValue;
}
#endif
