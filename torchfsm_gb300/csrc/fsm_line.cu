// Fused 1D integration: one CTA per sample runs every step and stage of the
// exponential Runge-Kutta scheme with the state, the scheme's running sums
// and the transform buffer resident in shared memory, and writes recorded
// frames straight into the trajectory. One launch per integrate call.
//
// Nonlinear terms (input dealiased, output not, operator/_base.py:375-403):
//  FSM_NL_CONVECTION  u u_x: one inverse complex FFT of Z = D + i G with
//                     D = mask*u_hat/N and G = i k D gives z = u + i u_x
//                     (operator/generic/_convection.py:43-46);
//  FSM_NL_KS          0.5 u_x^2 (operator/dedicated/_ks_convection.py:27-38).
// followed by one forward FFT of the real product.
#include "fsm_internal.cuh"

namespace fsm {

template <int N>
struct LineCfg {
  static constexpr int G = (N / 16 < 32) ? 32 : N / 16;
  static constexpr bool BLOCK = G > 32;
  static constexpr int H = N / 2 + 1;
  // twiddles, transform buffer, state and the scheme's running sums (at least acc and q)
  static size_t smem(int n_aux) { return (size_t)(2 * N + (1 + (n_aux > 2 ? n_aux : 2)) * H) * sizeof(float2); }
};

// Build the inverse-transform input of the stage field `a` at index k.
template <int N, int KIND>
__device__ __forceinline__ void line_build(float2* __restrict__ Z, int k, float2 a, float keep, float kxv,
                                           float scale) {
  const float2 d = cscale(a, keep * scale);
  float2 G = make_float2(-kxv * d.y, kxv * d.x);  // i k d
  const bool selfc = (k == 0) || (k == N / 2);
  if (KIND == FSM_NL_CONVECTION) {
    float2 D = d;
    if (selfc) {
      D.y = 0.f;
      G.y = 0.f;
    }
    Z[k] = make_float2(D.x - G.y, D.y + G.x);
    if (!selfc) Z[N - k] = make_float2(D.x + G.y, G.x - D.y);
  } else {  // FSM_NL_KS
    if (selfc) G.y = 0.f;
    Z[k] = G;
    if (!selfc) Z[N - k] = cconj(G);
  }
}

// One sample's integration by G = LineCfg<N>::G threads (t < G): the twiddles `tw` are in shared
// memory already (visible after the body's first barrier); Z (N), u, acc, q (running sums, n_aux
// arrays H apart) are the sample's shared-memory region. Every thread of the CTA runs the body the
// same number of times (its barriers are CTA-wide); `active` false runs it on the data of a valid
// sample without writing global memory (spare sub-groups of a k_line_multi CTA).
template <int N, int KIND>
__device__ __forceinline__ void line_body(const StepArgs& a, int b, int t, const float2* __restrict__ tw,
                                          float2* __restrict__ Z, float2* __restrict__ u, bool active) {
  using Cfg = LineCfg<N>;
  constexpr int H = Cfg::H;
  constexpr int G = Cfg::G;
  float2* acc = u + H;  // running sums: acc, q (Runge-Kutta: n_aux arrays H apart)
  float2* q = acc + H;
  float2* gstate = a.state + (int64_t)b * H;
  for (int k = t; k < H; k += G) u[k] = gstate[k];
  const int64_t toff = tab_batch(a, b) * H;
  const float2* tab = a.tab + toff;
  const float2* src = a.src ? a.src + (int64_t)(a.src_batch > 1 ? b : 0) * H : nullptr;
  const int slot0 = a.slots ? a.slots[0] : -1;
  const bool dc = KIND == FSM_NL_KS && (a.flags & FSM_FLAG_REMOVE_MEAN) && active;
  if (dc && t == 0) a.dc[(int64_t)a.steps * a.nstages * a.B + b] = u[0];  // initial k = 0 value
  for (int k = t; k < H; k += G) {
    if (slot0 >= 0 && active) a.traj[((int64_t)b * a.n_frames + slot0) * H + k] = u[k];
    if (a.steps > 0) line_build<N, KIND>(Z, k, u[k], (float)a.keepx[k], a.kx[k], a.scale);
  }
  __syncthreads();
  const int ns = a.nstages;
  for (int step = 0; step < a.steps; ++step) {
    for (int s = 0; s < ns; ++s) {
      fft<N, G, Cfg::BLOCK, true>(Z, tw, t);
      for (int n = t; n < N; n += G) {
        const float2 z = Z[n];
        const float p = (KIND == FSM_NL_CONVECTION) ? z.x * z.y : 0.5f * z.x * z.x;
        Z[n] = make_float2(p, 0.f);
      }
      __syncthreads();
      fft<N, G, Cfg::BLOCK, false>(Z, tw, t);
      const bool last = (s == ns - 1);
      const bool final_stage = last && (step == a.steps - 1);
      const int slot = (last && a.slots) ? a.slots[step + 1] : -1;
      for (int k = t; k < H; k += G) {
        float2 nv = cscale(Z[k], a.coef);
        // k = 0 of the product, for the batch-mean fix-up (k_line_dc_fixup)
        if (dc && k == 0) a.dc[((int64_t)step * ns + s) * a.B + b] = Z[0];
        if (src) nv = cadd(nv, src[k]);
        const float2 nxt = etd_stage(a.integ, s, nv, u + k, acc + k, q + k, tab + k, a.ts, H);
        if (!final_stage) line_build<N, KIND>(Z, k, nxt, (float)a.keepx[k], a.kx[k], a.scale);
        if (slot >= 0 && active) a.traj[((int64_t)b * a.n_frames + slot) * H + k] = u[k];
      }
      __syncthreads();
    }
  }
  if (active)
    for (int k = t; k < H; k += G) gstate[k] = u[k];
}

template <int N, int KIND>
__global__ void __launch_bounds__(LineCfg<N>::G) k_line(StepArgs a) {
  extern __shared__ float2 smem[];
  float2* tw = smem;
  load_twiddles(tw, a.tw, kTwiddleMax, N, threadIdx.x, LineCfg<N>::G);
  line_body<N, KIND>(a, blockIdx.x, threadIdx.x, tw, tw + N, tw + 2 * N, true);
}

// Serving: the lines of several plans (one per grid size) advanced by one launch. CTAs
// [cta0[j], cta0[j + 1]) belong to plan j; each holds kLineMultiThreads / G samples of its plan,
// one per sub-group of G threads, with the twiddles shared and a region per sample.
template <int N>
struct LineMultiCfg {
  static constexpr int G = LineCfg<N>::G;
  static constexpr int P = kLineMultiThreads / G;  // samples per CTA
  static constexpr int H = N / 2 + 1;
  __host__ __device__ static size_t region(int n_aux) { return (size_t)N + (size_t)(1 + (n_aux > 2 ? n_aux : 2)) * H; }
  static size_t smem(int n_aux) { return ((size_t)N + P * region(n_aux)) * sizeof(float2); }
};

template <int N, int KIND>
__device__ __forceinline__ void line_multi_cta(const StepArgs& a, int cta) {
  using Cfg = LineMultiCfg<N>;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  load_twiddles(tw, a.tw, kTwiddleMax, N, threadIdx.x, kLineMultiThreads);
  const int sub = threadIdx.x / Cfg::G, t = threadIdx.x % Cfg::G;
  const int b = cta * Cfg::P + sub;
  const bool active = b < a.B;
  float2* Z = smem + N + (size_t)sub * Cfg::region(a.n_aux);
  line_body<N, KIND>(a, active ? b : a.B - 1, t, tw, Z, Z + N, active);
}

template <int KIND>
__global__ void __launch_bounds__(kLineMultiThreads) k_line_multi(const __grid_constant__ LineMulti m) {
  int j = 0;
  while (j + 1 < m.count && (int)blockIdx.x >= m.cta0[j + 1]) ++j;
  const int cta = (int)blockIdx.x - m.cta0[j];
  switch (m.n[j]) {
    case 256: line_multi_cta<256, KIND>(m.a[j], cta); break;
    case 512: line_multi_cta<512, KIND>(m.a[j], cta); break;
    case 1024: line_multi_cta<1024, KIND>(m.a[j], cta); break;
    case 2048: line_multi_cta<2048, KIND>(m.a[j], cta); break;
    case 4096: line_multi_cta<4096, KIND>(m.a[j], cta); break;
  }
}

template <int N>
static void line_multi_shape(int n_aux, int batch, size_t* smem, int* ctas) {
  using Cfg = LineMultiCfg<N>;
  *smem = Cfg::smem(n_aux);
  *ctas = (batch + Cfg::P - 1) / Cfg::P;
}

template <int N, int KIND>
static int launch_line_n(const StepArgs& a, cudaStream_t st) {
  using Cfg = LineCfg<N>;
  const size_t smem = Cfg::smem(a.n_aux);
  int rc = prep_smem(k_line<N, KIND>, smem);
  if (rc) return rc;
  k_line<N, KIND><<<a.B, Cfg::G, smem, st>>>(a);
  return cuda_check(cudaGetLastError(), "k_line");
}

template <int KIND>
static int launch_line_kind(int n, const StepArgs& a, cudaStream_t st) {
  switch (n) {
    case 16: return launch_line_n<16, KIND>(a, st);
    case 32: return launch_line_n<32, KIND>(a, st);
    case 64: return launch_line_n<64, KIND>(a, st);
    case 128: return launch_line_n<128, KIND>(a, st);
    case 256: return launch_line_n<256, KIND>(a, st);
    case 512: return launch_line_n<512, KIND>(a, st);
    case 1024: return launch_line_n<1024, KIND>(a, st);
    case 2048: return launch_line_n<2048, KIND>(a, st);
    case 4096: return launch_line_n<4096, KIND>(a, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "1D: unsupported length " + std::to_string(n));
}

// KSConvection with the mean removed over a batch (operator/dedicated/_ks_convection.py:35-36:
// re.mean() spans the whole batch). The mean only changes the k = 0 value of the nonlinear
// term, and the k = 0 mode never feeds back into the product (it is a gradient), so the line
// kernel runs with the per-sample values and records every stage's k = 0 product P_b in
// dc[step][stage][b]. k_line_dc_mean reduces each (step, stage) row over the batch, in a fixed
// order, into dc[steps * stages * B + B + row]; k_line_dc_fixup then replays the k = 0
// recurrence of each sample with coef * (P_b - mean) + source, the same arithmetic as the line
// kernel, and overwrites k = 0 of the state and of the recorded frames.
__global__ void __launch_bounds__(256) k_line_dc_mean(StepArgs a) {
  __shared__ float2 red[256];
  const int row = blockIdx.x;
  const float2* P = a.dc + (int64_t)row * a.B;
  float2 sum = make_float2(0.f, 0.f);
  for (int i = threadIdx.x; i < a.B; i += 256) sum = cadd(sum, P[i]);
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const float inv = 1.f / (float)a.B;
    a.dc[(int64_t)a.steps * a.nstages * a.B + a.B + row] = cscale(red[0], inv);
  }
}

__global__ void k_line_dc_fixup(StepArgs a) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.B) return;
  const int ns = a.nstages;
  const int H = a.H;
  const float2* mean = a.dc + (int64_t)a.steps * ns * a.B + a.B;
  float2 u = a.dc[(int64_t)a.steps * ns * a.B + b];
  float2 aux[6] = {};  // the scheme's running sums at k = 0
  const float2* tab = a.tab + tab_batch(a, b) * H;
  const float2 src0 = a.src ? a.src[(int64_t)(a.src_batch > 1 ? b : 0) * H] : make_float2(0.f, 0.f);
  for (int step = 0; step < a.steps; ++step) {
    for (int s = 0; s < ns; ++s) {
      const int64_t row = (int64_t)step * ns + s;
      const float2 nv = cadd(cscale(csub(a.dc[row * a.B + b], mean[row]), a.coef), src0);
      (void)etd_stage(a.integ, s, nv, &u, aux, aux + 1, tab, a.ts, 1);
    }
    const int slot = a.slots ? a.slots[step + 1] : -1;
    if (slot >= 0) a.traj[((int64_t)b * a.n_frames + slot) * H] = u;
  }
  a.state[(int64_t)b * H] = u;
}

int launch_line_multi(LineMulti& m, int kind, cudaStream_t st) {
  if (m.count < 1 || m.count > kLineMultiMax) return set_error(FSM_ERR_INVALID, "line multi: plan count");
  size_t smem = 0;
  int total = 0;
  for (int j = 0; j < m.count; ++j) {
    size_t sm = 0;
    int ctas = 0;
    const int B = m.a[j].B, na = m.a[j].n_aux;
    if (B < 1) return set_error(FSM_ERR_INVALID, "line multi: empty plan entry");
    switch (m.n[j]) {
      case 256: line_multi_shape<256>(na, B, &sm, &ctas); break;
      case 512: line_multi_shape<512>(na, B, &sm, &ctas); break;
      case 1024: line_multi_shape<1024>(na, B, &sm, &ctas); break;
      case 2048: line_multi_shape<2048>(na, B, &sm, &ctas); break;
      case 4096: line_multi_shape<4096>(na, B, &sm, &ctas); break;
      default: return set_error(FSM_ERR_UNSUPPORTED, "line multi: lengths 256..4096 only");
    }
    m.cta0[j] = total;
    total += ctas;
    smem = sm > smem ? sm : smem;
  }
  m.cta0[m.count] = total;
  int rc;
  if (kind == FSM_NL_KS) {
    if ((rc = prep_smem(k_line_multi<FSM_NL_KS>, smem))) return rc;
    k_line_multi<FSM_NL_KS><<<total, kLineMultiThreads, smem, st>>>(m);
  } else if (kind == FSM_NL_CONVECTION) {
    if ((rc = prep_smem(k_line_multi<FSM_NL_CONVECTION>, smem))) return rc;
    k_line_multi<FSM_NL_CONVECTION><<<total, kLineMultiThreads, smem, st>>>(m);
  } else {
    return set_error(FSM_ERR_UNSUPPORTED, "line multi: unsupported nonlinear term");
  }
  return cuda_check(cudaGetLastError(), "k_line_multi");
}

int launch_line(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  switch (p->nl) {
    case FSM_NL_CONVECTION: return launch_line_kind<FSM_NL_CONVECTION>(p->n[0], a, st);
    case FSM_NL_KS: {
      int rc = launch_line_kind<FSM_NL_KS>(p->n[0], a, st);
      if (rc || !(p->flags & FSM_FLAG_REMOVE_MEAN) || a.steps == 0) return rc;
      k_line_dc_mean<<<a.steps * a.nstages, 256, 0, st>>>(a);
      rc = cuda_check(cudaGetLastError(), "k_line_dc_mean");
      if (rc) return rc;
      k_line_dc_fixup<<<(a.B + 127) / 128, 128, 0, st>>>(a);
      return cuda_check(cudaGetLastError(), "k_line_dc_fixup");
    }
  }
  return set_error(FSM_ERR_UNSUPPORTED, "1D: unsupported nonlinear term");
}

}  // namespace fsm
