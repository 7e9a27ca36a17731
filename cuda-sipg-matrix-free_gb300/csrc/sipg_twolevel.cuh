// sipg_twolevel.cuh -- the data of the two-level preconditioner
// (twolevel.cu) that its users build: the vertex-grid level descriptor, and
// the per-instance operands of its batched form (many problems, each with its
// own scratch, in one launch per kernel).
#pragma once

#include <vector>

#include "sipg_internal.cuh"

namespace sipg {

constexpr int kTlMaxLevels = 12;  // vertex-grid levels: meshes up to 8 * 2^11 elements per side

// One level of the vertex grid (device pointers).
template <typename T>
struct TlLev {
  int m;        // cells per side; (m + 1)^2 vertices, v = vy * (m + 1) + vx, vy bottom-up
  const T* S;   // stencil planes [9][nv], entry k = (dy + 1) * 3 + (dx + 1)
  const T* wd;  // omega / diagonal
  T* b;         // right-hand side
  T* x;         // pre-smoothed iterate
  T* y;         // V-cycle result
};

// One problem's preconditioner operands: z = M r with its own scratch (the
// corner sums and every level's b, x, y), the op's shared tables.
struct TlInst {
  const float* r;
  float* z;
  float* cp;           // [4][noe] corner sums
  const float* fdm;    // [16][3][nn] element block factors (fast diagonalisation)
  const float* ainv;   // the coarsest level's dense inverse
  CgState<float>* st;  // the inner PCG state (r.z and beta are set here)
  ReduceScratch red;
  int dim, p, nl;      // mesh, degree, levels
  int tail0;           // first level of the one-block tail (levels of at most 32 cells per side)
  int nblk;            // blocks of the element kernels (and of its r.z reduction)
  TlLev<float> lev[kTlMaxLevels];
};

// How a batched application runs: instances in the device array are grouped
// by degree (group g: [first, first + count)).
struct TlPlan {
  int n = 0;
  int maxl = 0;
  int nblk_max = 0;
  int max_tail0 = 0;
  std::vector<int> side_max;  // per level: the largest vertices per side
  struct Group {
    int p, first, count, nblk_max;
    const HostTables* tab;
  };
  std::vector<Group> groups;
};

// Scratch floats one instance of the op's preconditioner needs (the same
// from the mesh size alone, before the op's preconditioner exists).
size_t twolevel_scratch_floats(const void* handle);
size_t twolevel_scratch_floats_for(int dim);
// An instance over `scratch` (twolevel_scratch_floats floats, 16-byte
// aligned) for z = M r with the inner state st.
TlInst twolevel_inst(const void* handle, float* scratch, const float* r, float* z, CgState<float>* st,
                     const ReduceScratch& red);
// The launch plan of h_insts[0..n) (degree-sorted; tabs[i]: instance i's op tables).
TlPlan twolevel_plan(const TlInst* h_insts, const HostTables* const* tabs, int n);
// Enqueues z = M r for every instance of d_insts (the device copy of the
// planned array); each instance is skipped once its state says done.
sipg_status twolevel_enqueue_batched(const TlInst* d_insts, const TlPlan& plan, cudaStream_t s);

}  // namespace sipg
