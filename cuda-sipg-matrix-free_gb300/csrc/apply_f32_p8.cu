// Instantiates the fused apply (single-operator and batched launches) for
// float, degree 8: one translation unit per precision and degree, so the
// build compiles them in parallel.
#include "sipg_apply.cuh"
namespace sipg {
cudaError_t launch_apply_f32_p8(const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const HostTables& h,
                                  cudaStream_t s) {
  return launch_apply_p<float, 8>(cfg, mode, a, h, s);
}
cudaError_t launch_apply_batched_f32_p8(const TileCfg& cfg, int mode, const ApplyArgs<float>* insts,
                                          const int* tile_start, int ninst, int total_tiles, const HostTables& h,
                                          cudaStream_t s) {
  return launch_apply_batched_p<float, 8>(cfg, mode, insts, tile_start, ninst, total_tiles, h, s);
}
}  // namespace sipg
