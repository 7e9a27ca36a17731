// Instantiates the fused apply for float, degrees 1 2 3 4 (one translation unit per
// precision and degree group, so the build compiles them in parallel).
#include "sipg_apply.cuh"
namespace sipg {
cudaError_t launch_apply_f32_lo(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const HostTables& h, cudaStream_t s) {
  switch (p) {
    case 1: return launch_apply_p<float, 1>(cfg, mode, a, h, s);
    case 2: return launch_apply_p<float, 2>(cfg, mode, a, h, s);
    case 3: return launch_apply_p<float, 3>(cfg, mode, a, h, s);
    case 4: return launch_apply_p<float, 4>(cfg, mode, a, h, s);
  }
  return cudaErrorInvalidValue;
}
}  // namespace sipg
