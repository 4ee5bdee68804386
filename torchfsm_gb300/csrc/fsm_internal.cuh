// Internal launchers shared between the torchfsm_gb300 CUDA sources.
#pragma once

#include "fsm_common.cuh"

namespace fsm {

// Arguments of the fused kernels that advance a batch of half spectra.
struct StepArgs {
  float2* state;              // [B][C][S]
  float2* aux;                // [B][n_aux*C][S] scheme running sums (acc, q)
  float2* mid;                // [B][n_mid][S]  stage fields after the outer-axis inverse transform
  float2* prod;               // [B][n_prod][S] products after the last-axis forward transform
  float2* traj;               // [B][n_frames][C][S]
  int n_frames;
  int slot;                   // frame written at the end of this launch, or -1
  const int32_t* slots;       // device copy of the record slots (single-launch kernels)
  const float2* tab;          // coefficient tables
  int64_t ts;                 // distance between tables
  int lin_batch, lin_ch;
  const float2* src;          // explicit source or null
  int src_batch;
  const float* kx;            // 2 pi f of the first axis
  const float* ky;            // 2 pi f of the last axis
  const float* km;            // 2 pi f of the middle axis (3D)
  const uint8_t* keepx;
  const uint8_t* keepy;
  const uint8_t* keepm;       // middle axis (3D)
  float2* mid2;               // [B][n_mid2][S] fields after the middle-axis inverse transform (3D)
  int n_mid2;
  int nm;                     // points of the middle axis (3D)
  const float2* tw;           // master twiddles
  float2* dc;                 // batch-mean scratch of the KS mean removal
  float coef;                 // nonlinear coefficient
  float scale;                // 1 / (points per field)
  int C, n_aux, n_mid, n_prod;
  int integ, nstages;
  int stage;                  // stage whose nonlinear value the launch consumes; -1 primes
  int emit;                   // write the next stage's fields
  int steps;
  int B;
  int flags;
  int64_t S;
  int H;
  const uint8_t* tile_zero;  // register axis-0 pass: column tiles whose next-stage fields are zero
  int hk;                     // 2D: last-axis columns of the stage fields stored and read (FsmPlan::hk)
  int64_t wp, ms;             // row pitch and field stride of mid / prod (FsmPlan::wp, ms)
  const int32_t* tab_entry;   // per sample: its coefficient-table entry (serving), or null
};

// The coefficient-table entry of sample b: its own entry from tab_entry when given (a serving
// engine's slots share their request's entry), else entry b of per-sample tables or the one entry.
__device__ __forceinline__ int64_t tab_batch(const StepArgs& a, int b) {
  return a.tab_entry ? (int64_t)a.tab_entry[b] : (int64_t)(a.lin_batch > 1 ? b : 0);
}

// The kernels' arguments for `batch` samples of `state` advanced by `steps` steps of plan p,
// without recording (fsm_api.cu).
StepArgs base_args(const FsmPlan* p, void* state, int32_t batch, int32_t steps);

int transform_r2c_last(int n, const float* in, float2* out, int64_t rows, const float2* tw, cudaStream_t st);
int transform_c2r_last(int n, const float2* in, float* out, int64_t rows, float scale, const float2* tw,
                       cudaStream_t st);
int transform_c2c_strided(int n, bool inverse, float2* data, int64_t outer, int64_t inner, const float2* tw,
                          cudaStream_t st);
int launch_nonfinite(const float2* f, int64_t count, int64_t S, int32_t* flags, cudaStream_t st);

// fsm_integrate without recording on a caller-provided workspace (fsm_api.cu).
int integrate_with_workspace(const FsmPlan* p, int32_t batch, void* state, int32_t steps, void* workspace,
                             size_t workspace_bytes, cudaStream_t st);
size_t integrate_workspace_bytes(const FsmPlan* p, int32_t batch, int32_t steps);
// fsm_integrate without recording on a caller-provided workspace; large batches may run in
// parts on the library's streams (outside stream capture), as fsm_integrate does. tab_entry
// (device, one per sample, or null): each sample's coefficient-table entry.
int integrate_on_workspace(const FsmPlan* p, int32_t batch, void* state, int32_t steps, void* workspace,
                           size_t workspace_bytes, cudaStream_t st, const int32_t* tab_entry = nullptr);
// Recompute the coefficient tables of batch entries [b0, b0 + n) for time step dt (one launch).
int set_batch_dt_range(FsmPlan* p, int32_t b0, int32_t n, double dt, cudaStream_t st);

int transform_c2c_strided_reg(int n, bool inverse, float2* data, int64_t outer, int64_t inner, const float2* tw,
                              cudaStream_t st);  // -1: no register kernel for n
int launch_volume_axis1_inv(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
int launch_volume_axis2(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
int launch_volume_axis1_fwd(const FsmPlan* p, const StepArgs& a, cudaStream_t st);

int launch_line(const FsmPlan* p, const StepArgs& a, cudaStream_t st);

// One launch of the 1D line kernel over the samples of several plans of different lengths
// (256..4096 points, one nonlinear kind): entry j advances a[j].B samples of a[j] by a[j].steps
// steps (the same for every entry), without recording. cta0 is filled in by the launcher.
constexpr int kLineMultiMax = 8;
constexpr int kLineMultiThreads = 256;
struct LineMulti {
  StepArgs a[kLineMultiMax];
  int32_t n[kLineMultiMax];
  int32_t cta0[kLineMultiMax + 1];
  int32_t count;
};
int launch_line_multi(LineMulti& m, int kind, cudaStream_t st);

// One launch of the 2D register column (or row) pass over the samples of several plans of square
// grids (64, 128 or 256 points per axis, Convection or VorticityConvection): entry j runs the pass
// on a[j].B samples of a[j] (arguments of plane_args, stage and emit set by the caller). gx and
// cta0 are filled in by the launchers. fast: the SETDRK4 stage launch (stage >= 0).
constexpr int kPlaneMultiMax = 8;
struct PlaneMulti {
  StepArgs a[kPlaneMultiMax];
  int32_t n[kPlaneMultiMax];
  int32_t gx[kPlaneMultiMax];
  int32_t cta0[kPlaneMultiMax + 1];
  int32_t count;
};
int launch_plane_col_multi(PlaneMulti& m, int kind, bool fast, cudaStream_t st);
int launch_plane_row_multi(PlaneMulti& m, int kind, cudaStream_t st);
// The plane passes' arguments for `batch` samples of `state` advanced by `steps` steps without
// recording, with the pass arrays in `workspace` laid out as fsm_integrate lays them out (fsm_api.cu).
int plane_args(const FsmPlan* p, void* state, int32_t batch, int32_t steps, void* workspace, size_t workspace_bytes,
               StepArgs* out);
// Register-FFT plane passes (64..256 points per axis); return -1 when no kernel covers the sizes.
int launch_plane_col_reg(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
int launch_plane_row_reg(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
int launch_plane_col(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
int launch_plane_row(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
int launch_ks_mean(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
int launch_pointwise(const FsmPlan* p, const StepArgs& a, cudaStream_t st);
// Parts (streams) an uncaptured integrate of `batch` samples is split into; 1: one sequence.
int split_parts(const FsmPlan* p, int batch);

// Raise a kernel's dynamic shared-memory limit when it needs more than 48 KB. The
// attribute is per function and per device; the size set is remembered per
// (kernel, device) so that repeated launches skip the attribute call.
bool smem_attr_known(const void* kernel, int device, size_t smem);
void smem_attr_record(const void* kernel, int device, size_t smem);

template <class K>
inline int prep_smem(K kernel, size_t smem) {
  if (smem <= 48 * 1024) return FSM_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  const void* key = (const void*)kernel;
  if (smem_attr_known(key, dev, smem)) return FSM_OK;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_check(e, "cudaFuncSetAttribute");
  smem_attr_record(key, dev, smem);
  return FSM_OK;
}

}  // namespace fsm
