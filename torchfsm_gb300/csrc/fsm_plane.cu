// Fused 2D exponential Runge-Kutta stages on half spectra [B][C][NX][H],
// H = NY/2 + 1. Each stage of the scheme is two passes over the batch:
//
//  column pass (k_plane_col): per tile of 8 adjacent ky columns of one sample
//    1. forward FFT along x of the products left by the row pass -> N_s(kx, ky)
//       (plus the Leray projection for velocity Navier-Stokes, plus the source);
//    2. the scheme's stage update at every point (etd_stage), recording the
//       state when a step completes;
//    3. the next stage's field: 2/3 mask, 1/(NX NY), the x-derivative and
//       streamfunction factors, then the inverse FFT along x -> mid arrays.
//  row pass (k_plane_row): per pair of rows of one sample
//    c2r along y of the mid arrays (with the y-derivative factor), the
//    physical-space product of the nonlinear term, r2c along y -> products.
//
// Programs (nonlinear term, operator/_base.py:375-403; input masked only):
//  FSM_NL_VORTICITY  psi = -w/lap (1 at k = 0), u = (d_y psi, -d_x psi),
//                    product u.grad(w) (operator/dedicated/_navier_stokes.py:40-46)
//                    mid: psi, i kx psi, w, i kx w
//  FSM_NL_CONVECTION (u.grad)u with C = 2 (operator/generic/_convection.py:43-46)
//                    mid: u0, i kx u0, u1, i kx u1; products conv0 + i conv1
//  FSM_NL_LERAY      convection, then N = i k p - conv, p = (i k . conv)/lap
//                    (operator/dedicated/_navier_stokes.py:246-254)
//  FSM_NL_KS         0.5|grad phi|^2, mean over the batch removed on request
//                    (operator/dedicated/_ks_convection.py:27-38); mid: phi, i kx phi
#include "fsm_internal.cuh"

namespace fsm {

constexpr int kTileW = 8;  // ky columns per column-pass CTA (one warp each)

template <int KIND>
struct PlaneKind {
  static constexpr int NP = (KIND == FSM_NL_CONVECTION || KIND == FSM_NL_LERAY) ? 2 : 1;
  static constexpr int NM = (KIND == FSM_NL_KS) ? 2 : 4;
  static constexpr int NF = NP > NM ? NP : NM;
  static constexpr int C = (KIND == FSM_NL_CONVECTION || KIND == FSM_NL_LERAY) ? 2 : 1;
};

template <int NX, int KIND>
__global__ void __launch_bounds__(256) k_plane_col(StepArgs a) {
  using K = PlaneKind<KIND>;
  constexpr int P = NX + 2;
  constexpr int C = K::C;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* fld = smem + NX;  // [NF][kTileW][P]
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.y;
  const int c0 = blockIdx.x * kTileW;
  const int H = a.H;
  const int64_t S = a.S;
  const bool colw_ok = (c0 + w) < H;
  load_twiddles(tw, a.tw, kTwiddleMax, NX, threadIdx.x, 256);
  if (a.stage >= 0) {
    for (int f = 0; f < K::NP; ++f) {
      const float2* src = a.prod + ((int64_t)b * a.n_prod + f) * S;
      for (int idx = threadIdx.x; idx < NX * kTileW; idx += 256) {
        const int row = idx / kTileW, col = idx % kTileW;
        if (c0 + col < H) fld[(f * kTileW + col) * P + row] = src[(int64_t)row * H + c0 + col];
      }
    }
    __syncthreads();
    if (colw_ok) {
      for (int f = 0; f < K::NP; ++f) fft<NX, 32, false, false>(fld + (f * kTileW + w) * P, tw, lane);
    }
    __syncthreads();
  } else {
    __syncthreads();
  }
  const bool last = a.stage == a.nstages - 1;
  for (int idx = threadIdx.x; idx < NX * kTileW; idx += 256) {
    const int row = idx / kTileW, col = idx % kTileW;
    const int ky_i = c0 + col;
    if (ky_i >= H) continue;
    const int64_t sidx = (int64_t)row * H + ky_i;
    const float kxv = a.kx[row], kyv = a.ky[ky_i];
    float2 nv[C];
    if (a.stage >= 0) {
#pragma unroll
      for (int c = 0; c < C; ++c) nv[c] = fld[(c * kTileW + col) * P + row];
      if (KIND == FSM_NL_LERAY) {
        // conv -> i k p - conv with p = (i kx conv0 + i ky conv1) / lap (1 where lap == 0); at the
        // x Nyquist row with ky strictly inside, the Hermitian part keeps the two axes apart
        // (see nv_leray in fsm_plane_reg.cu)
        const float lap = -(kxv * kxv + kyv * kyv);
        const float il = (lap == 0.f) ? 1.f : 1.f / lap;
        const float2 dx = cscale(cmuli(nv[0]), kxv), dy = cscale(cmuli(nv[1]), kyv);
        const bool split = (row == NX / 2) && ky_i > 0 && ky_i < H - 1;
        const float2 p0 = cscale(split ? dx : cadd(dx, dy), il);
        const float2 p1 = cscale(split ? dy : cadd(dx, dy), il);
        const float2 n0 = csub(cscale(cmuli(p0), kxv), nv[0]);
        const float2 n1 = csub(cscale(cmuli(p1), kyv), nv[1]);
        nv[0] = n0;
        nv[1] = n1;
      }
      if (KIND == FSM_NL_KS && (a.flags & FSM_FLAG_REMOVE_MEAN) && row == 0 && ky_i == 0) {
        nv[0] = csub(nv[0], a.dc[0]);
      }
#pragma unroll
      for (int c = 0; c < C; ++c) {
        nv[c] = cscale(nv[c], a.coef);
        if (a.src) nv[c] = cadd(nv[c], a.src[((int64_t)(a.src_batch > 1 ? b : 0) * C + c) * S + sidx]);
      }
    }
    float2 st[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      float2* up = a.state + ((int64_t)b * C + c) * S + sidx;
      if (a.stage < 0) {
        st[c] = *up;
      } else {
        float2* accp = a.aux + ((int64_t)b * a.n_aux * C + c) * S + sidx;
        float2* qp = a.aux + ((int64_t)b * a.n_aux * C + (a.n_aux > 1 ? C : 0) + c) * S + sidx;
        const int64_t toff = (tab_batch(a, b) * a.lin_ch + (a.lin_ch > 1 ? c : 0)) * S + sidx;
        st[c] = etd_stage(a.integ, a.stage, nv[c], up, accp, qp, a.tab + toff, a.ts, (int64_t)C * S);
      }
      if (a.slot >= 0 && (a.stage < 0 || last))
        a.traj[(((int64_t)b * a.n_frames + a.slot) * C + c) * S + sidx] = st[c];
    }
    if (a.emit) {
      const float m = (float)(a.keepx[row] & a.keepy[ky_i]) * a.scale;
      float2* f = fld + col * P + row;
      if (KIND == FSM_NL_VORTICITY) {
        const float2 d = cscale(st[0], m);
        const float lap = -(kxv * kxv + kyv * kyv);
        const float il = (lap == 0.f) ? 1.f : 1.f / lap;
        const float2 psi = cscale(d, -il);
        f[0 * kTileW * P] = psi;
        f[1 * kTileW * P] = cscale(cmuli(psi), kxv);
        f[2 * kTileW * P] = d;
        f[3 * kTileW * P] = cscale(cmuli(d), kxv);
      } else if (KIND == FSM_NL_KS) {
        const float2 d = cscale(st[0], m);
        f[0] = d;
        f[1 * kTileW * P] = cscale(cmuli(d), kxv);
      } else {
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float2 d = cscale(st[c], m);
          f[(2 * c) * kTileW * P] = d;
          f[(2 * c + 1) * kTileW * P] = cscale(cmuli(d), kxv);
        }
      }
    }
  }
  if (!a.emit) return;
  __syncthreads();
  if (colw_ok) {
    for (int m = 0; m < K::NM; ++m) fft<NX, 32, false, true>(fld + (m * kTileW + w) * P, tw, lane);
  }
  __syncthreads();
  for (int m = 0; m < K::NM; ++m) {
    float2* dst = a.mid + ((int64_t)b * a.n_mid + m) * S;
    for (int idx = threadIdx.x; idx < NX * kTileW; idx += 256) {
      const int row = idx / kTileW, col = idx % kTileW;
      if (c0 + col < H) dst[(int64_t)row * H + c0 + col] = fld[(m * kTileW + col) * P + row];
    }
  }
}

// Hermitian pair: Z = A + i B over k = 0..NY/2, mirrored for NY/2 < k < NY.
template <int NY>
__device__ __forceinline__ void herm_pair(float2* __restrict__ Z, int k, float2 A, float2 B) {
  const bool selfc = (k == 0) || (k == NY / 2);
  if (selfc) {
    A.y = 0.f;
    B.y = 0.f;
  }
  Z[k] = make_float2(A.x - B.y, A.y + B.x);
  if (!selfc) Z[NY - k] = make_float2(A.x + B.y, B.x - A.y);
}

// Split the FFT of p0 + i p1 into the half spectra of p0 and p1 and store them.
template <int NY>
__device__ __forceinline__ void split_store(const float2* __restrict__ Z, int lane, float2* __restrict__ out0,
                                            float2* __restrict__ out1) {
  constexpr int H = NY / 2 + 1;
  for (int k = lane; k < H; k += 32) {
    const float2 zk = Z[k];
    const float2 zm = cconj(Z[(NY - k) & (NY - 1)]);
    out0[k] = cscale(cadd(zk, zm), 0.5f);
    out1[k] = cscale(cmulmi(csub(zk, zm)), 0.5f);
  }
}

constexpr int kRowsPerCta = 16;  // 8 warps x 2 rows

template <int NY, int KIND>
__global__ void __launch_bounds__(256) k_plane_row(StepArgs a) {
  constexpr int H = NY / 2 + 1;
  constexpr int NBUF = (KIND == FSM_NL_VORTICITY) ? 4 : (KIND == FSM_NL_KS ? 2 : 3);
  extern __shared__ float2 smem[];
  float2* tw = smem;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* buf = smem + NY + w * NBUF * NY;
  const int b = blockIdx.y;
  const int r0 = blockIdx.x * kRowsPerCta + 2 * w;
  const int64_t S = a.S;
  const float* ky = a.ky;
  load_twiddles(tw, a.tw, kTwiddleMax, NY, threadIdx.x, 256);
  __syncthreads();
  const float2* mid = a.mid + (int64_t)b * a.n_mid * S;
  float2* prod = a.prod + (int64_t)b * a.n_prod * S;
  if (KIND == FSM_NL_VORTICITY || KIND == FSM_NL_KS) {
    for (int rr = 0; rr < 2; ++rr) {
      const int64_t roff = (int64_t)(r0 + rr) * H;
      for (int k = lane; k < H; k += 32) {
        const float kyv = ky[k];
        if (KIND == FSM_NL_VORTICITY) {
          const float2 m0 = mid[0 * S + roff + k], m1 = mid[1 * S + roff + k];
          const float2 m2 = mid[2 * S + roff + k], m3 = mid[3 * S + roff + k];
          // u_x + i u_y  with u_x <- i ky psi, u_y <- -i kx psi
          herm_pair<NY>(buf + (2 * rr) * NY, k, cscale(cmuli(m0), kyv), make_float2(-m1.x, -m1.y));
          // w_x + i w_y  with w_x <- i kx w, w_y <- i ky w
          herm_pair<NY>(buf + (2 * rr + 1) * NY, k, m3, cscale(cmuli(m2), kyv));
        } else {
          const float2 m0 = mid[0 * S + roff + k], m1 = mid[1 * S + roff + k];
          // phi_x + i phi_y
          herm_pair<NY>(buf + rr * NY, k, m1, cscale(cmuli(m0), kyv));
        }
      }
    }
    __syncwarp();
    constexpr int NIFFT = (KIND == FSM_NL_VORTICITY) ? 4 : 2;
#pragma unroll
    for (int i = 0; i < NIFFT; ++i) fft<NY, 32, false, true>(buf + i * NY, tw, lane);
    for (int n = lane; n < NY; n += 32) {
      float p0, p1;
      if (KIND == FSM_NL_VORTICITY) {
        const float2 u0 = buf[n], w0 = buf[NY + n], u1 = buf[2 * NY + n], w1 = buf[3 * NY + n];
        p0 = u0.x * w0.x + u0.y * w0.y;
        p1 = u1.x * w1.x + u1.y * w1.y;
      } else {
        const float2 g0 = buf[n], g1 = buf[NY + n];
        p0 = 0.5f * (g0.x * g0.x + g0.y * g0.y);
        p1 = 0.5f * (g1.x * g1.x + g1.y * g1.y);
      }
      buf[n] = make_float2(p0, p1);
    }
    __syncwarp();
    fft<NY, 32, false, false>(buf, tw, lane);
    split_store<NY>(buf, lane, prod + (int64_t)r0 * H, prod + (int64_t)(r0 + 1) * H);
  } else {
    // convection, C = 2: conv_c = u0 d_x u_c + u1 d_y u_c
    for (int rr = 0; rr < 2; ++rr) {
      const int64_t roff = (int64_t)(r0 + rr) * H;
      for (int k = lane; k < H; k += 32) {
        const float kyv = ky[k];
        const float2 d0 = mid[0 * S + roff + k], g0 = mid[1 * S + roff + k];
        const float2 d1 = mid[2 * S + roff + k], g1 = mid[3 * S + roff + k];
        herm_pair<NY>(buf, k, d0, d1);                                                  // u0 + i u1
        herm_pair<NY>(buf + NY, k, g0, g1);                                             // dx u0 + i dx u1
        herm_pair<NY>(buf + 2 * NY, k, cscale(cmuli(d0), kyv), cscale(cmuli(d1), kyv));  // dy u0 + i dy u1
      }
      __syncwarp();
      fft<NY, 32, false, true>(buf, tw, lane);
      fft<NY, 32, false, true>(buf + NY, tw, lane);
      fft<NY, 32, false, true>(buf + 2 * NY, tw, lane);
      for (int n = lane; n < NY; n += 32) {
        const float2 u = buf[n], gx = buf[NY + n], gy = buf[2 * NY + n];
        buf[n] = make_float2(u.x * gx.x + u.y * gy.x, u.x * gx.y + u.y * gy.y);
      }
      __syncwarp();
      fft<NY, 32, false, false>(buf, tw, lane);
      split_store<NY>(buf, lane, prod + roff, prod + S + roff);
      __syncwarp();
    }
  }
}

// Batch mean of the k = 0 product (KS mean removal): dc = (1/B) sum_b sum_x prod[b][0][x][0..0],
// the products being transformed along every axis but the first.
__global__ void k_ks_mean(StepArgs a, int nx) {
  float acc = 0.f;
  const int total = a.B * nx;
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int b = i / nx, x = i % nx;
    acc += a.prod[((int64_t)b * a.n_prod) * a.ms + (int64_t)x * a.wp].x;
  }
  __shared__ float red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.dc[0] = make_float2(red[0] / (float)a.B, 0.f);
}

template <int NX, int KIND>
static int launch_col_n(const StepArgs& a, cudaStream_t st) {
  using K = PlaneKind<KIND>;
  const size_t smem = (size_t)(NX + K::NF * kTileW * (NX + 2)) * sizeof(float2);
  int rc = prep_smem(k_plane_col<NX, KIND>, smem);
  if (rc) return rc;
  dim3 grid((a.H + kTileW - 1) / kTileW, a.B);
  k_plane_col<NX, KIND><<<grid, 256, smem, st>>>(a);
  return cuda_check(cudaGetLastError(), "k_plane_col");
}

template <int NY, int KIND>
static int launch_row_n(int nx, const StepArgs& a, cudaStream_t st) {
  constexpr int NBUF = (KIND == FSM_NL_VORTICITY) ? 4 : (KIND == FSM_NL_KS ? 2 : 3);
  const size_t smem = (size_t)(NY + 8 * NBUF * NY) * sizeof(float2);
  int rc = prep_smem(k_plane_row<NY, KIND>, smem);
  if (rc) return rc;
  dim3 grid(nx / kRowsPerCta, a.B);
  k_plane_row<NY, KIND><<<grid, 256, smem, st>>>(a);
  return cuda_check(cudaGetLastError(), "k_plane_row");
}

template <int KIND>
static int col_dispatch(int nx, const StepArgs& a, cudaStream_t st) {
  switch (nx) {
    case 16: return launch_col_n<16, KIND>(a, st);
    case 32: return launch_col_n<32, KIND>(a, st);
    case 64: return launch_col_n<64, KIND>(a, st);
    case 128: return launch_col_n<128, KIND>(a, st);
    case 256: return launch_col_n<256, KIND>(a, st);
    case 512: return launch_col_n<512, KIND>(a, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "2D: unsupported first-axis length " + std::to_string(nx));
}

template <int KIND>
static int row_dispatch(int nx, int ny, const StepArgs& a, cudaStream_t st) {
  switch (ny) {
    case 16: return launch_row_n<16, KIND>(nx, a, st);
    case 32: return launch_row_n<32, KIND>(nx, a, st);
    case 64: return launch_row_n<64, KIND>(nx, a, st);
    case 128: return launch_row_n<128, KIND>(nx, a, st);
    case 256: return launch_row_n<256, KIND>(nx, a, st);
    case 512: return launch_row_n<512, KIND>(nx, a, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "2D: unsupported last-axis length " + std::to_string(ny));
}

int launch_plane_col(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  const int r = launch_plane_col_reg(p, a, st);
  if (r != -1) return r;
  switch (p->nl) {
    case FSM_NL_VORTICITY: return col_dispatch<FSM_NL_VORTICITY>(p->n[0], a, st);
    case FSM_NL_CONVECTION: return col_dispatch<FSM_NL_CONVECTION>(p->n[0], a, st);
    case FSM_NL_LERAY: return col_dispatch<FSM_NL_LERAY>(p->n[0], a, st);
    case FSM_NL_KS: return col_dispatch<FSM_NL_KS>(p->n[0], a, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "2D: unsupported nonlinear term");
}

int launch_plane_row(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  const int r = launch_plane_row_reg(p, a, st);
  if (r != -1) return r;
  switch (p->nl) {
    case FSM_NL_VORTICITY: return row_dispatch<FSM_NL_VORTICITY>(p->n[0], p->n[1], a, st);
    case FSM_NL_CONVECTION:
    case FSM_NL_LERAY: return row_dispatch<FSM_NL_CONVECTION>(p->n[0], p->n[1], a, st);
    case FSM_NL_KS: return row_dispatch<FSM_NL_KS>(p->n[0], p->n[1], a, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "2D: unsupported nonlinear term");
}

int launch_ks_mean(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  k_ks_mean<<<1, 256, 0, st>>>(a, p->n[0]);
  return cuda_check(cudaGetLastError(), "k_ks_mean");
}

}  // namespace fsm
