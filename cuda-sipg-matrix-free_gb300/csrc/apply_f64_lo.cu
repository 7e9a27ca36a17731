// Instantiates the fused apply for double, degrees 1 2 3 4 (one translation unit per
// precision and degree group, so the build compiles them in parallel).
#include "sipg_apply.cuh"
namespace sipg {
cudaError_t launch_apply_f64_lo(int p, const TileCfg& cfg, int mode, const ApplyArgs<double>& a, const HostTables& h, cudaStream_t s) {
  switch (p) {
    case 1: return launch_apply_p<double, 1>(cfg, mode, a, h, s);
    case 2: return launch_apply_p<double, 2>(cfg, mode, a, h, s);
    case 3: return launch_apply_p<double, 3>(cfg, mode, a, h, s);
    case 4: return launch_apply_p<double, 4>(cfg, mode, a, h, s);
  }
  return cudaErrorInvalidValue;
}
}  // namespace sipg
