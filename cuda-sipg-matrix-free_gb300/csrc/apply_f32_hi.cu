// Instantiates the fused apply for float, degrees 5 6 7 8 (one translation unit per
// precision and degree group, so the build compiles them in parallel).
#include "sipg_apply.cuh"
namespace sipg {
cudaError_t launch_apply_f32_hi(int p, const TileCfg& cfg, int mode, const ApplyArgs<float>& a, const HostTables& h, cudaStream_t s) {
  switch (p) {
    case 5: return launch_apply_p<float, 5>(cfg, mode, a, h, s);
    case 6: return launch_apply_p<float, 6>(cfg, mode, a, h, s);
    case 7: return launch_apply_p<float, 7>(cfg, mode, a, h, s);
    case 8: return launch_apply_p<float, 8>(cfg, mode, a, h, s);
  }
  return cudaErrorInvalidValue;
}
}  // namespace sipg
