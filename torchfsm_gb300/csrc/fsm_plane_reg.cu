// Register-FFT versions of the 2D column and row passes (64..256 points per axis): the kernels of
// one plan and their launchers. The device bodies are in fsm_plane_reg.cuh.
#include "fsm_plane_reg.cuh"

namespace fsm {

template <int NX, int KIND, int DIM>
__global__ void __launch_bounds__(256) k_axis0_r(StepArgs a) {
  axis0_body<NX, KIND, DIM, false>(a, blockIdx.x, blockIdx.y);
}

template <int NX, int KIND, int DIM>
__global__ void __launch_bounds__(256, 2) k_axis0_r2(StepArgs a) {
  axis0_body<NX, KIND, DIM, true>(a, blockIdx.x, blockIdx.y);
}

template <int NY, int KIND, int HK>
__global__ void __launch_bounds__(256, 2) k_plane_row_r(StepArgs a) {
  plane_row_body<NY, KIND, HK>(a, blockIdx.x, blockIdx.y);
}

template <int NX, int KIND, int DIM, bool FAST>
static int launch_axis0_r_mode(const StepArgs& a, cudaStream_t st) {
  using Cfg = ColCfg<NX>;
  using K = RegKind<KIND, DIM>;
  const size_t smem = (size_t)(NX + (K::CG + 1) * Cfg::W * Cfg::P) * sizeof(float2);
  const int64_t inner = a.S / NX;
  dim3 grid((unsigned)((inner + Cfg::W - 1) / Cfg::W), a.B);
  if constexpr (FAST) {
    int rc = prep_smem(k_axis0_r2<NX, KIND, DIM>, smem);
    if (rc) return rc;
    k_axis0_r2<NX, KIND, DIM><<<grid, 256, smem, st>>>(a);
    return cuda_check(cudaGetLastError(), "k_axis0_r2");
  } else {
    int rc = prep_smem(k_axis0_r<NX, KIND, DIM>, smem);
    if (rc) return rc;
    k_axis0_r<NX, KIND, DIM><<<grid, 256, smem, st>>>(a);
    return cuda_check(cudaGetLastError(), "k_axis0_r");
  }
}

template <int NX, int KIND, int DIM>
static int launch_axis0_r(const StepArgs& a, cudaStream_t st) {
  // the hoisted update for vorticity and convection (KS keeps the generic kernel: its hoisted
  // instance does not fit two CTAs' registers per SM)
  constexpr bool fast = RegKind<KIND, DIM>::CG == 1 && KIND != FSM_NL_KS;
  if (fast && a.integ == FSM_SETDRK4 && a.stage >= 0) return launch_axis0_r_mode<NX, KIND, DIM, fast>(a, st);
  return launch_axis0_r_mode<NX, KIND, DIM, false>(a, st);
}

template <int NY, int KIND, int HK>
static int launch_row_r_hk(int nx, const StepArgs& a, cudaStream_t st) {
  using Cfg = RowCfgR<NY>;
  const int groups_needed = nx / 2;
  int threads = groups_needed * Cfg::T;
  if (threads > 256) threads = 256;
  const int groups = threads / Cfg::T;
  const size_t smem = (size_t)(NY + groups * Cfg::SCR) * sizeof(float2);
  int rc = prep_smem(k_plane_row_r<NY, KIND, HK>, smem);
  if (rc) return rc;
  dim3 grid(groups_needed / groups, a.B);
  k_plane_row_r<NY, KIND, HK><<<grid, threads, smem, st>>>(a);
  return cuda_check(cudaGetLastError(), "k_plane_row_r");
}

// The 2/3 rule's stored prefix (NY/3 + 1 columns) or every column.
template <int NY, int KIND>
static int launch_row_r(int nx, const StepArgs& a, cudaStream_t st) {
  if (a.hk == NY / 3 + 1) return launch_row_r_hk<NY, KIND, NY / 3 + 1>(nx, a, st);
  if (a.hk != NY / 2 + 1) return set_error(FSM_ERR_INVALID, "row pass: unexpected stored column count");
  return launch_row_r_hk<NY, KIND, NY / 2 + 1>(nx, a, st);
}

template <int KIND, int DIM>
static int col_r_dispatch(int nx, const StepArgs& a, cudaStream_t st) {
  switch (nx) {
    case 16: return launch_axis0_r<16, KIND, DIM>(a, st);
    case 32: return launch_axis0_r<32, KIND, DIM>(a, st);
    case 64: return launch_axis0_r<64, KIND, DIM>(a, st);
    case 128: return launch_axis0_r<128, KIND, DIM>(a, st);
    case 256: return launch_axis0_r<256, KIND, DIM>(a, st);
  }
  return -1;
}

template <int KIND>
static int row_r_dispatch(int nx, int ny, const StepArgs& a, cudaStream_t st) {
  if (nx < 2) return -1;
  switch (ny) {
    case 16: return launch_row_r<16, KIND>(nx, a, st);
    case 32: return launch_row_r<32, KIND>(nx, a, st);
    case 64: return launch_row_r<64, KIND>(nx, a, st);
    case 128: return launch_row_r<128, KIND>(nx, a, st);
    case 256: return launch_row_r<256, KIND>(nx, a, st);
  }
  return -1;
}

// Returns -1 when no register-FFT kernel exists for the sizes (caller falls back).
int launch_plane_col_reg(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  if (p->ndim == 3) {
    switch (p->nl) {
      case FSM_NL_CONVECTION: return col_r_dispatch<FSM_NL_CONVECTION, 3>(p->n[0], a, st);
      case FSM_NL_LERAY: return col_r_dispatch<FSM_NL_LERAY, 3>(p->n[0], a, st);
      case FSM_NL_KS: return col_r_dispatch<FSM_NL_KS, 3>(p->n[0], a, st);
    }
    return -1;
  }
  switch (p->nl) {
    case FSM_NL_VORTICITY: return col_r_dispatch<FSM_NL_VORTICITY, 2>(p->n[0], a, st);
    case FSM_NL_CONVECTION: return col_r_dispatch<FSM_NL_CONVECTION, 2>(p->n[0], a, st);
    case FSM_NL_LERAY: return col_r_dispatch<FSM_NL_LERAY, 2>(p->n[0], a, st);
    case FSM_NL_KS: return col_r_dispatch<FSM_NL_KS, 2>(p->n[0], a, st);
  }
  return -1;
}

int launch_plane_row_reg(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  switch (p->nl) {
    case FSM_NL_VORTICITY: return row_r_dispatch<FSM_NL_VORTICITY>(p->n[0], p->n[1], a, st);
    case FSM_NL_CONVECTION:
    case FSM_NL_LERAY: return row_r_dispatch<FSM_NL_CONVECTION>(p->n[0], p->n[1], a, st);
    case FSM_NL_KS: return row_r_dispatch<FSM_NL_KS>(p->n[0], p->n[1], a, st);
  }
  return -1;
}

}  // namespace fsm
