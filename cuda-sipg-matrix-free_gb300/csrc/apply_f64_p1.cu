// Instantiates the fused apply for double, degree 1: single-operator
// launches (element-per-thread and per-node tiles) and batched ones.  One
// translation unit per precision and degree, so the build compiles them in
// parallel.
#include "sipg_apply_pernode.cuh"
namespace sipg {
cudaError_t launch_apply_f64_p1(const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h,
                                  cudaStream_t s) {
  if (is_pernode(cfg, 1)) return launch_apply_pernode<double, 1>(cfg, apply_base_mode(mode), a, h, s);
  return launch_apply_p<double, 1>(cfg, mode, a, h, s);
}
cudaError_t launch_apply_batched_f64_p1(const TileCfg& cfg, int mode, const ApplyArgs<double>* insts,
                                          const int* tile_start, int ninst, int total_tiles, const HostTables& h,
                                          cudaStream_t s) {
  return launch_apply_batched_p<double, 1>(cfg, mode, insts, tile_start, ninst, total_tiles, h, s);
}
}  // namespace sipg
