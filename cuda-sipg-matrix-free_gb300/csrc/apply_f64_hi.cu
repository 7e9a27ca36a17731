// Instantiates the fused apply for double, degrees 5 6 7 8 (one translation unit per
// precision and degree group, so the build compiles them in parallel).
#include "sipg_apply.cuh"
namespace sipg {
cudaError_t launch_apply_f64_hi(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h, cudaStream_t s) {
  switch (p) {
    case 5: return launch_apply_p<double, 5>(cfg, mode, a, h, s);
    case 6: return launch_apply_p<double, 6>(cfg, mode, a, h, s);
    case 7: return launch_apply_p<double, 7>(cfg, mode, a, h, s);
    case 8: return launch_apply_p<double, 8>(cfg, mode, a, h, s);
  }
  return cudaErrorInvalidValue;
}
}  // namespace sipg
