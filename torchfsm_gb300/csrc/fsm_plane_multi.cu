// The 2D column and row passes of several plans (square grids of 64, 128 or 256 points per
// axis, one nonlinear kind) advanced by one launch each: CTAs [cta0[j], cta0[j + 1]) run the
// register-FFT pass of plan j (fsm_plane_reg.cuh) on their (tile or row block, sample), with
// the plan's own arguments. Serving groups use them so that requests of different grid sizes
// share one column and one row launch per stage (fsm_serve.cu).
#include "fsm_plane_reg.cuh"

namespace fsm {

namespace {

__device__ __forceinline__ int multi_entry(const PlaneMulti& m, int* local) {
  int j = 0;
  while (j + 1 < m.count && (int)blockIdx.x >= m.cta0[j + 1]) ++j;
  *local = (int)blockIdx.x - m.cta0[j];
  return j;
}

template <int N>
constexpr int kept_prefix() {
  return N / 3 + 1;  // the 2/3 rule's stored columns (FsmPlan::hk)
}

}  // namespace

template <int KIND, bool FAST>
__device__ __forceinline__ void axis0_multi_body(const PlaneMulti& m) {
  int local = 0;
  const int j = multi_entry(m, &local);
  const int tile = local % m.gx[j], b = local / m.gx[j];
  switch (m.n[j]) {
    case 64: axis0_body<64, KIND, 2, FAST>(m.a[j], tile, b); break;
    case 128: axis0_body<128, KIND, 2, FAST>(m.a[j], tile, b); break;
    case 256: axis0_body<256, KIND, 2, FAST>(m.a[j], tile, b); break;
  }
}

// The SETDRK4 stage launches (the hoisted update, two CTAs per SM) and the priming launch.
template <int KIND>
__global__ void __launch_bounds__(256, 2) k_axis0_multi2(const __grid_constant__ PlaneMulti m) {
  axis0_multi_body<KIND, true>(m);
}

template <int KIND>
__global__ void __launch_bounds__(256) k_axis0_multi(const __grid_constant__ PlaneMulti m) {
  axis0_multi_body<KIND, false>(m);
}

template <int KIND>
__global__ void __launch_bounds__(256, 2) k_plane_row_multi(const __grid_constant__ PlaneMulti m) {
  int local = 0;
  const int j = multi_entry(m, &local);
  const int blk = local % m.gx[j], b = local / m.gx[j];
  const bool cut = m.a[j].hk != m.n[j] / 2 + 1;
  switch (m.n[j]) {
    case 64:
      if (cut) plane_row_body<64, KIND, kept_prefix<64>()>(m.a[j], blk, b);
      else plane_row_body<64, KIND, 33>(m.a[j], blk, b);
      break;
    case 128:
      if (cut) plane_row_body<128, KIND, kept_prefix<128>()>(m.a[j], blk, b);
      else plane_row_body<128, KIND, 65>(m.a[j], blk, b);
      break;
    case 256:
      if (cut) plane_row_body<256, KIND, kept_prefix<256>()>(m.a[j], blk, b);
      else plane_row_body<256, KIND, 129>(m.a[j], blk, b);
      break;
  }
}

namespace {

// Shared memory and CTAs per sample of plan entry a (N points per axis).
template <int N, int KIND>
void col_shape(const StepArgs& a, size_t* smem, int* per_sample) {
  using Cfg = ColCfg<N>;
  *smem = (size_t)(N + (RegKind<KIND, 2>::CG + 1) * Cfg::W * Cfg::P) * sizeof(float2);
  *per_sample = (int)((a.S / N + Cfg::W - 1) / Cfg::W);
}

template <int N>
void row_shape(size_t* smem, int* per_sample) {
  using Cfg = RowCfgR<N>;
  constexpr int groups = 256 / Cfg::T;  // 256 threads: every size here has at least 256 row-pair lanes
  *smem = (size_t)(N + groups * Cfg::SCR) * sizeof(float2);
  *per_sample = (N / 2) / groups;
}

// Fill in cta0 / gx for the launch and return the total CTAs and the largest shared memory.
template <int KIND>
int multi_layout(PlaneMulti& m, bool column, size_t* smem, int* total) {
  if (m.count < 1 || m.count > kPlaneMultiMax) return set_error(FSM_ERR_INVALID, "plane multi: plan count");
  *smem = 0;
  *total = 0;
  for (int j = 0; j < m.count; ++j) {
    if (m.a[j].B < 1) return set_error(FSM_ERR_INVALID, "plane multi: empty plan entry");
    size_t sm = 0;
    int per = 0;
    switch (m.n[j]) {
      case 64: column ? col_shape<64, KIND>(m.a[j], &sm, &per) : row_shape<64>(&sm, &per); break;
      case 128: column ? col_shape<128, KIND>(m.a[j], &sm, &per) : row_shape<128>(&sm, &per); break;
      case 256: column ? col_shape<256, KIND>(m.a[j], &sm, &per) : row_shape<256>(&sm, &per); break;
      default: return set_error(FSM_ERR_UNSUPPORTED, "plane multi: grids of 64, 128 or 256 points per axis only");
    }
    m.gx[j] = per;
    m.cta0[j] = *total;
    *total += per * m.a[j].B;
    *smem = sm > *smem ? sm : *smem;
  }
  m.cta0[m.count] = *total;
  return FSM_OK;
}

template <int KIND>
int launch_col_multi_kind(PlaneMulti& m, bool fast, cudaStream_t st) {
  size_t smem = 0;
  int total = 0;
  int rc = multi_layout<KIND>(m, true, &smem, &total);
  if (rc) return rc;
  if (fast) {
    if ((rc = prep_smem(k_axis0_multi2<KIND>, smem))) return rc;
    k_axis0_multi2<KIND><<<total, 256, smem, st>>>(m);
    return cuda_check(cudaGetLastError(), "k_axis0_multi2");
  }
  if ((rc = prep_smem(k_axis0_multi<KIND>, smem))) return rc;
  k_axis0_multi<KIND><<<total, 256, smem, st>>>(m);
  return cuda_check(cudaGetLastError(), "k_axis0_multi");
}

template <int KIND>
int launch_row_multi_kind(PlaneMulti& m, cudaStream_t st) {
  size_t smem = 0;
  int total = 0;
  int rc = multi_layout<KIND>(m, false, &smem, &total);
  if (rc) return rc;
  if ((rc = prep_smem(k_plane_row_multi<KIND>, smem))) return rc;
  k_plane_row_multi<KIND><<<total, 256, smem, st>>>(m);
  return cuda_check(cudaGetLastError(), "k_plane_row_multi");
}

}  // namespace

int launch_plane_col_multi(PlaneMulti& m, int kind, bool fast, cudaStream_t st) {
  switch (kind) {
    case FSM_NL_CONVECTION: return launch_col_multi_kind<FSM_NL_CONVECTION>(m, fast, st);
    case FSM_NL_VORTICITY: return launch_col_multi_kind<FSM_NL_VORTICITY>(m, fast, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "plane multi: Convection or VorticityConvection only");
}

int launch_plane_row_multi(PlaneMulti& m, int kind, cudaStream_t st) {
  switch (kind) {
    case FSM_NL_CONVECTION: return launch_row_multi_kind<FSM_NL_CONVECTION>(m, st);
    case FSM_NL_VORTICITY: return launch_row_multi_kind<FSM_NL_VORTICITY>(m, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "plane multi: Convection or VorticityConvection only");
}

}  // namespace fsm
