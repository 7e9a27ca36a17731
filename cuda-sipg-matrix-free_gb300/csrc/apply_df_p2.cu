// Instantiates the compensated apply on pair vectors (single and batched) for degree 2.
#include "sipg_apply_df.cuh"
namespace sipg {
cudaError_t launch_apply_df_p2(const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const ApplyArgs<float>* insts,
                                 const int* tile_start, int ninst, int total_tiles, const HostTables& h, cudaStream_t s) {
  return launch_apply_df_p<2>(cfg, mode, a, insts, tile_start, ninst, total_tiles, h, s);
}
}  // namespace sipg
