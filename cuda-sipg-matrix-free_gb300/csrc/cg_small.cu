// cg_small.cu -- CG on small FP64 meshes (up to kSmallCgDim elements per
// edge) as one persistent kernel.
//
// On a mesh of a few hundred elements an iteration of the graph-driven CG
// (capi.cu) is two short kernels whose cost is launch and reduction latency:
// 15 us at 16 x 16, p = 4, of which the arithmetic is a fraction.  Here one
// cooperative launch (every CTA resident) runs all iterations: 12.7 us per
// iteration there, the rest being the two grid barriers' L2 round trips
// (fence, arrival, polls, partial reads) that the two reductions of an
// iteration need.  Per iteration:
//   A  the per-node apply of the CTA's tiles with the direction p = r + beta
//      p_old formed on the fly (the same per-tile code as
//      k_sipg_apply_pernode), its p.Ap partial stored; grid barrier;
//   B  every CTA sums the partials in index order -- the same operations in
//      every CTA, so every CTA holds the same alpha -- and updates x and r on
//      the nodes it computed in A (its own values, no cross-CTA read), its
//      r.r partial stored; grid barrier; every CTA sums those the same way
//      and does the iteration bookkeeping (it, beta, the stop test) itself.
// All CTAs reach the same decisions, so they leave the loop at the same
// iteration.  Data other CTAs write during the kernel (r, the direction) is
// read through L2 (__ldcg).  Every barrier wait is bounded: a wait that gives
// up raises an abort flag that ends every CTA's loop, and the solve returns
// an error.
#include <algorithm>

#include "sipg_apply_pernode.cuh"
#include "sipg_cg.cuh"

namespace sipg {

// polls of the arrival count (an L2 round trip, ~0.7 us, and a 32 ns sleep
// each): a wait gives up after about a second; a barrier that completes
// takes tens of polls
constexpr unsigned kBarrierSpins = 1u << 20;

// Grid barrier: every CTA arrives once; the barrier is complete when the
// arrival count reaches `target` (the count only grows: target = barrier
// number x gridDim.x).  Returns false if the wait gave up or another CTA's
// did.
__device__ bool grid_barrier(unsigned long long* bar, int* abort, unsigned long long target) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1ull);
    int res = 1;
    for (unsigned spins = 0;; ++spins) {
      if (*(volatile unsigned long long*)bar >= target) break;
      if (*(volatile int*)abort || spins >= kBarrierSpins) {
        atomicExch(abort, 1);
        res = 0;
        break;
      }
      __nanosleep(32);  // spaces the polls of up to a thousand CTAs on one L2 line
    }
    __threadfence();
    ok = res;
  }
  __syncthreads();
  return ok != 0;
}

// The sum of partials written by the grid's CTAs, in index order, the same
// in every CTA; valid in every thread.
template <int NT>
__device__ double sum_partials(const double* part, int n, double* red_sh, double* out_sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += NT) s += __ldcg(part + i);
  s = block_sum<double, NT>(s, red_sh);
  if (threadIdx.x == 0) *out_sh = s;
  __syncthreads();
  const double v = *out_sh;
  __syncthreads();  // red_sh / out_sh are reused
  return v;
}

template <int P, int SHAPE>
__global__ void __launch_bounds__(PernodeShape<P, SHAPE>::NT)
    k_cg_small(const __grid_constant__ SmallCgArgs g, const __grid_constant__ Tab<double, P> tb) {
  using S = PernodeShape<P, SHAPE>;
  constexpr int N1 = S::N1, NN = S::NN, EX = S::EX, EY = S::EY, NE = S::NE, NT = S::NT;
  __shared__ PernodeSmem<double, P, SHAPE> sm;
  __shared__ double red_sh[32];
  __shared__ double sc;
  const int t = threadIdx.x;
  const int nb = (int)gridDim.x;
  const int dim = g.dim;
  const size_t noe = (size_t)dim * dim;
  const int tiles_x = (dim + EX - 1) / EX, ntiles = tiles_x * ((dim + EY - 1) / EY);
  pernode_tables<double, P, SHAPE>(sm, tb);

  CgState<double> st = *g.st;  // the same copy in every CTA from here on
  ApplyArgs<double> a{};
  a.in = g.r;
  a.out = g.Ap;
  a.dim = dim;
  a.nu = g.nu;
  unsigned long long target = 0;
  bool aborted = false;
  while (!st.done) {
    const int par = st.parity;
    const double* pold = par ? g.p1 : g.p0;
    double* pnew = par ? g.p0 : g.p1;
    // A: direction, Ap and the p.Ap partial
    double acc = 0.0;
    for (int tile = blockIdx.x; tile < ntiles; tile += nb) {
      const int x0 = (tile % tiles_x) * EX, y0 = (tile / tiles_x) * EY;
      acc += pernode_tile<double, P, SHAPE, APPLY_CG, true>(a, sm, x0, y0, st.first != 0, st.beta, pold, pnew);
    }
    const double bt = block_sum<double, NT>(acc, red_sh);
    if (t == 0) g.part_a[blockIdx.x] = bt;
    target += nb;
    if (!grid_barrier(g.bar, g.abort, target)) {
      aborted = true;
      break;
    }
    const double pAp = sum_partials<NT>(g.part_a, nb, red_sh, &sc);
    const double alpha = st.rr / pAp;
    st.pAp = pAp;
    st.alpha = alpha;
    if (!(pAp > 0.0) || !isfinite(alpha)) {
      st.status = (int)SIPG_ERR_BREAKDOWN;
      st.done = 1;
      break;
    }
    // B: x and r on the nodes this thread computed in A, the r.r partial
    double acc2 = 0.0;
    for (int tile = blockIdx.x; tile < ntiles; tile += nb) {
      const int x0 = (tile % tiles_x) * EX, y0 = (tile / tiles_x) * EY;
      if (t < NE * NN) {
        const int le = t % NE, k = t / NE;
        const int gx = x0 + le % EX, gy = y0 + le / EX;
        if (gx < dim && gy < dim) {
          const size_t gk = (size_t)k * noe + (size_t)gy * dim + gx;
          // (values this thread wrote; read through L2 all the same, as r's
          // cache lines also hold other CTAs' nodes)
          g.x[gk] = fma(alpha, __ldcg(pnew + gk), __ldcg(g.x + gk));
          const double ri = fma(-alpha, __ldcg(g.Ap + gk), __ldcg(g.r + gk));
          g.r[gk] = ri;
          acc2 = fma(ri, ri, acc2);
        }
      }
    }
    const double bt2 = block_sum<double, NT>(acc2, red_sh);
    if (t == 0) g.part_b[blockIdx.x] = bt2;
    target += nb;
    if (!grid_barrier(g.bar, g.abort, target)) {
      aborted = true;
      break;
    }
    const double rr = sum_partials<NT>(g.part_b, nb, red_sh, &sc);
    // the bookkeeping of cg_bookkeep (no reliable updates on this path)
    const double rn = sqrt(rr);
    st.it += 1;
    st.first = 0;
    st.rr_prev = st.rr;
    st.beta = rr / st.rr;
    st.rr = rr;
    st.rmax = fmax(st.rmax, rn);
    st.parity = 1 - par;
    st.done = !(rn > st.stop && st.it < st.max_it);
    if (!isfinite(rr)) {
      st.status = (int)SIPG_ERR_BREAKDOWN;
      st.done = 1;
    }
  }
  if (aborted) {
    st.status = (int)SIPG_ERR_CUDA;
    st.done = 1;
  }
  if (blockIdx.x == 0 && t == 0) *g.st = st;
  (void)N1;
}

template <int P, int SHAPE>
cudaError_t launch_cg_small_shape(const SmallCgArgs& g, const HostTables& h, cudaStream_t s) {
  using S = PernodeShape<P, SHAPE>;
  auto k = k_cg_small<P, SHAPE>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, S::NT, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const long long ntiles = (long long)((g.dim + S::EX - 1) / S::EX) * ((g.dim + S::EY - 1) / S::EY);
  // every CTA resident (a cooperative launch checks it), at most one per
  // tile and one partial slot each
  const int grid = (int)std::max<long long>(1, std::min<long long>({ntiles, (long long)sms * per_sm,
                                                                    (long long)kSmallCgMaxBlocks}));
  const Tab<double, P> tb = make_tab<double, P>(h);
  void* args[] = {(void*)&g, (void*)&tb};
  e = cudaLaunchCooperativeKernel((const void*)k, dim3(grid), dim3(S::NT), args, 0, s);
  count_launch();
  return e;
}

template <int P>
cudaError_t launch_cg_small_p(const TileCfg& cfg, const SmallCgArgs& g, const HostTables& h, cudaStream_t s) {
  if (cfg.tpe != (P + 1) * (P + 1) || cfg.ty != pernode_ey(P)) return cudaErrorInvalidConfiguration;
  if (cfg.tx == pernode_ex(P, 0)) return launch_cg_small_shape<P, 0>(g, h, s);
  if (cfg.tx == pernode_ex(P, 1)) return launch_cg_small_shape<P, 1>(g, h, s);
  return cudaErrorInvalidConfiguration;
}

// The barrier's give-up path, for the self-test: every CTA waits for one
// arrival more than the grid has, so each wait runs out (bounded), raises
// the abort flag and returns; out[blockIdx.x] = 1 where the barrier reported
// failure.
__global__ void k_barrier_selftest(unsigned long long* bar, int* abort, int* out) {
  const bool ok = grid_barrier(bar, abort, (unsigned long long)gridDim.x + 1ull);
  if (threadIdx.x == 0) out[blockIdx.x] = ok ? 0 : 1;
}

cudaError_t launch_cg_small(int p, const TileCfg& cfg, const SmallCgArgs& g, const HostTables& h, cudaStream_t s) {
  switch (p) {
    case 1: return launch_cg_small_p<1>(cfg, g, h, s);
    case 2: return launch_cg_small_p<2>(cfg, g, h, s);
    case 3: return launch_cg_small_p<3>(cfg, g, h, s);
    case 4: return launch_cg_small_p<4>(cfg, g, h, s);
    case 5: return launch_cg_small_p<5>(cfg, g, h, s);
    case 6: return launch_cg_small_p<6>(cfg, g, h, s);
    case 7: return launch_cg_small_p<7>(cfg, g, h, s);
    case 8: return launch_cg_small_p<8>(cfg, g, h, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace sipg

using namespace sipg;

extern "C" sipg_status sipg_selftest_barrier_timeout(int* gave_up) {
  if (!gave_up) return SIPG_ERR_INVALID;
  *gave_up = 0;
  constexpr int kBlocks = 4;
  void* mem = nullptr;
  SIPG_CUDA_TRY(cudaMalloc(&mem, 512));
  unsigned long long* bar = (unsigned long long*)mem;
  int* abort = (int*)((char*)mem + 128);
  int* out = (int*)((char*)mem + 256);
  cudaError_t e = cudaMemset(mem, 0, 512);
  if (e == cudaSuccess) {
    void* args[] = {(void*)&bar, (void*)&abort, (void*)&out};
    e = cudaLaunchCooperativeKernel((const void*)k_barrier_selftest, dim3(kBlocks), dim3(32), args, 0, nullptr);
    count_launch();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int h_out[kBlocks] = {0, 0, 0, 0}, h_abort = 0;
  if (e == cudaSuccess) e = cudaMemcpy(h_out, out, sizeof(h_out), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&h_abort, abort, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(mem);
  if (e != cudaSuccess) {
    set_error(std::string("sipg_selftest_barrier_timeout: ") + cudaGetErrorString(e));
    return SIPG_ERR_CUDA;
  }
  int n = 0;
  for (int v : h_out) n += v;
  *gave_up = (n == kBlocks && h_abort == 1) ? 1 : 0;
  return SIPG_OK;
}
