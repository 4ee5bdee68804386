// 3D stages on half spectra [B][C][n0][n1][H], H = n2/2 + 1. One stage of the
// scheme is four passes:
//   axis 1 inverse (k_axis1_inv_r): per (sample, channel, x) plane and tile of
//     kz columns, the y inverse transforms of the x-pass output:
//       Y(X u_c), Y(X (i kx u_c)), Y(i ky X u_c)      (mid -> mid2, 2 -> 3 fields)
//   axis 2 (k_axis2_r): per (sample, x, y) row, z c2r of the twelve velocity
//     gradients (i kz applied here), the product sum_i u_i d_i u_c, z r2c
//     (Convection, operator/generic/_convection.py:43-46), or 0.5 |grad phi|^2
//     (KSConvection, operator/dedicated/_ks_convection.py:27-38);
//   axis 1 forward: in-place y transform of the products (k_c2c_strided_r);
//   axis 0 (k_axis0_r in fsm_plane_reg.cu): x transform, stage update, next fields.
#include "fsm_internal.cuh"
#include "fsm_regfft.cuh"

namespace fsm {

template <int N>
struct TileCfg {
  using RS = RegShape<N>;
  static constexpr int T = RS::T;
  static constexpr int E = RS::E;
  static constexpr int W = 256 / T;
  static constexpr int NEED = (N > E * (T + 1)) ? N : E * (T + 1);
  static constexpr int P = NEED | 1;
};

// In-place transform along the middle axis of data [outer][N][inner]
// (complex), tiles of W adjacent inner columns staged through shared memory.
template <int N, bool INV>
__global__ void __launch_bounds__(256) k_c2c_strided_r(float2* __restrict__ data, int64_t inner,
                                                       const float2* __restrict__ master) {
  using Cfg = TileCfg<N>;
  constexpr int T = Cfg::T, E = Cfg::E, W = Cfg::W, P = Cfg::P;
  extern __shared__ float2 smem[];
  float2* twt = smem;
  float2* tile = smem + N;
  float2* scr = tile + W * P;
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int64_t c0 = (int64_t)blockIdx.x * W;
  float2* base = data + (int64_t)blockIdx.y * N * inner;
  load_reg_twiddles<N>(twt, master, threadIdx.x, 256);
  {
    float2 buf[N * W / 256];
#pragma unroll
    for (int it = 0; it < N * W / 256; ++it) {
      const int idx = threadIdx.x + it * 256;
      const int row = idx / W, col = idx % W;
      if (c0 + col < inner) buf[it] = base[(int64_t)row * inner + c0 + col];
    }
#pragma unroll
    for (int it = 0; it < N * W / 256; ++it) {
      const int idx = threadIdx.x + it * 256;
      const int row = idx / W, col = idx % W;
      if (c0 + col < inner) tile[col * P + row] = buf[it];
    }
  }
  __syncthreads();
  float2 v[E];
#pragma unroll
  for (int j = 0; j < E; ++j) v[j] = tile[g * P + t + T * j];
  reg_fft<N, INV>(v, scr + g * P, twt, t);
#pragma unroll
  for (int j = 0; j < E; ++j) tile[g * P + t + T * j] = v[j];
  __syncthreads();
  for (int idx = threadIdx.x; idx < N * W; idx += 256) {
    const int row = idx / W, col = idx % W;
    if (c0 + col < inner) base[(int64_t)row * inner + c0 + col] = tile[col * P + row];
  }
}

template <int N, bool INV>
static int launch_c2c_r(float2* data, int64_t outer, int64_t inner, const float2* tw, cudaStream_t st) {
  using Cfg = TileCfg<N>;
  const size_t smem = (size_t)(N + 2 * Cfg::W * Cfg::P) * sizeof(float2);
  int rc = prep_smem(k_c2c_strided_r<N, INV>, smem);
  if (rc) return rc;
  if (outer > 65535) return set_error(FSM_ERR_UNSUPPORTED, "c2c: too many transforms in one launch");
  dim3 grid((unsigned)((inner + Cfg::W - 1) / Cfg::W), (unsigned)outer);
  k_c2c_strided_r<N, INV><<<grid, 256, smem, st>>>(data, inner, tw);
  return cuda_check(cudaGetLastError(), "k_c2c_strided_r");
}

int transform_c2c_strided_reg(int n, bool inverse, float2* data, int64_t outer, int64_t inner, const float2* tw,
                              cudaStream_t st) {
#define FSM_C2CR_CASE(NN)                                                                    \
  case NN:                                                                                   \
    return inverse ? launch_c2c_r<NN, true>(data, outer, inner, tw, st)                      \
                   : launch_c2c_r<NN, false>(data, outer, inner, tw, st);
  switch (n) {
    FSM_C2CR_CASE(16)
    FSM_C2CR_CASE(32)
    FSM_C2CR_CASE(64)
    FSM_C2CR_CASE(128)
    FSM_C2CR_CASE(256)
  }
#undef FSM_C2CR_CASE
  return -1;
}

// ---------------------------------------------------------------------------
// axis 1 inverse (3D)
// ---------------------------------------------------------------------------
template <int NY>
__global__ void __launch_bounds__(256) k_axis1_inv_r(StepArgs a) {
  using Cfg = TileCfg<NY>;
  constexpr int T = Cfg::T, E = Cfg::E, W = Cfg::W, P = Cfg::P;
  extern __shared__ float2 smem[];
  float2* twt = smem;
  float2* tA = smem + NY;   // X u_c            -> Y(i ky X u_c)
  float2* tB = tA + W * P;  // X (i kx u_c)     -> Y(X (i kx u_c))
  float2* tC = tB + W * P;  //                  -> Y(X u_c)
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int H = a.H;
  const int x = blockIdx.y;
  const int groups_c = a.n_mid / 2;
  const int b = blockIdx.z / groups_c, c = blockIdx.z % groups_c;
  const int64_t c0 = (int64_t)blockIdx.x * W;
  const int64_t plane = (int64_t)NY * H;
  const int64_t S = a.S;
  load_reg_twiddles<NY>(twt, a.tw, threadIdx.x, 256);
  const float2* in0 = a.mid + ((int64_t)b * a.n_mid + 2 * c) * S + (int64_t)x * plane;
  const float2* in1 = in0 + S;
  {
    float2 b0[NY * W / 256], b1[NY * W / 256];
#pragma unroll
    for (int it = 0; it < NY * W / 256; ++it) {
      const int idx = threadIdx.x + it * 256;
      const int row = idx / W, col = idx % W;
      if (c0 + col < H) {
        b0[it] = in0[(int64_t)row * H + c0 + col];
        b1[it] = in1[(int64_t)row * H + c0 + col];
      }
    }
#pragma unroll
    for (int it = 0; it < NY * W / 256; ++it) {
      const int idx = threadIdx.x + it * 256;
      const int row = idx / W, col = idx % W;
      if (c0 + col < H) {
        tA[col * P + row] = b0[it];
        tB[col * P + row] = b1[it];
      }
    }
  }
  __syncthreads();
  {
    float2 v[E], w[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
      v[j] = tA[g * P + t + T * j];
      w[j] = cscale(cmuli(v[j]), a.km[t + T * j]);
    }
    reg_fft<NY, true>(v, tC + g * P, twt, t);
#pragma unroll
    for (int j = 0; j < E; ++j) tC[g * P + t + T * j] = v[j];
    reg_fft<NY, true>(w, tA + g * P, twt, t);
#pragma unroll
    for (int j = 0; j < E; ++j) tA[g * P + t + T * j] = w[j];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = tB[g * P + t + T * j];
    reg_fft<NY, true>(v, tB + g * P, twt, t);
#pragma unroll
    for (int j = 0; j < E; ++j) tB[g * P + t + T * j] = v[j];
  }
  __syncthreads();
  float2* out = a.mid2 + ((int64_t)b * a.n_mid2 + 3 * c) * S + (int64_t)x * plane;
  for (int idx = threadIdx.x; idx < NY * W; idx += 256) {
    const int row = idx / W, col = idx % W;
    if (c0 + col < H) {
      const int64_t o = (int64_t)row * H + c0 + col;
      out[o] = tC[col * P + row];          // Y(X u_c)
      out[S + o] = tB[col * P + row];      // Y(X (i kx u_c))
      out[2 * S + o] = tA[col * P + row];  // Y(i ky X u_c)
    }
  }
}

// ---------------------------------------------------------------------------
// axis 2 (3D): contiguous z rows, products
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 herm_z3(float2 A, float2 B, bool selfc, bool hi) {
  if (selfc) {
    A.y = 0.f;
    B.y = 0.f;
  }
  if (hi) {
    A.y = -A.y;
    B.y = -B.y;
  }
  return make_float2(A.x - B.y, A.y + B.x);
}

// Build Z = A + i B (Hermitian extension over the row) from two mid2 fields;
// `da`/`db` apply the i kz factor to A / B.
template <int NZ>
__device__ __forceinline__ void build_row(float2 (&Z)[RegShape<NZ>::E], const float2* __restrict__ fa,
                                          const float2* __restrict__ fb, bool da, bool db, const float* __restrict__ kz,
                                          int t) {
  constexpr int T = RegShape<NZ>::T, E = RegShape<NZ>::E;
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const int k = t + T * j;
    const bool hi = k > NZ / 2;
    const int kk = hi ? NZ - k : k;
    const bool selfc = (kk == 0) || (kk == NZ / 2);
    const float kzv = kz[kk];
    float2 A = fa ? fa[kk] : make_float2(0.f, 0.f);
    float2 B = fb ? fb[kk] : make_float2(0.f, 0.f);
    if (da) A = cscale(cmuli(A), kzv);
    if (db) B = cscale(cmuli(B), kzv);
    Z[j] = herm_z3(A, B, selfc, hi);
  }
}

template <int NZ>
__device__ __forceinline__ void split_one(const float2 (&zp)[RegShape<NZ>::E], int t, int lane,
                                          float2* __restrict__ out0, float2* __restrict__ out1) {
  constexpr int T = RegShape<NZ>::T, E = RegShape<NZ>::E;
  constexpr int J = NZ / (2 * T);
  const int partner_lane = (lane & ~(T - 1)) | ((T - t) & (T - 1));
#pragma unroll
  for (int j = 0; j <= J; ++j) {
    const float2 send = zp[E - 1 - j];
    float2 recv;
    recv.x = __shfl_sync(0xffffffffu, send.x, partner_lane);
    recv.y = __shfl_sync(0xffffffffu, send.y, partner_lane);
    const float2 partner = (t == 0) ? zp[(E - j) & (E - 1)] : recv;
    const int k = t + T * j;
    if (k <= NZ / 2) {
      const float2 zm = cconj(partner);
      out0[k] = cscale(cadd(zp[j], zm), 0.5f);
      if (out1) out1[k] = cscale(cmulmi(csub(zp[j], zm)), 0.5f);
    }
  }
}

template <int NZ, int KIND>
__global__ void __launch_bounds__(256, 2) k_axis2_r(StepArgs a) {
  using RS = RegShape<NZ>;
  constexpr int T = RS::T, E = RS::E, SCR = reg_scratch<NZ>();
  constexpr int H = NZ / 2 + 1;
  extern __shared__ float2 smem[];
  float2* twt = smem;
  const int lane = threadIdx.x & 31;
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int groups = blockDim.x / T;
  float2* scr = smem + NZ + g * SCR;
  float* ust = (float*)(smem + NZ + groups * SCR) + (size_t)g * 3 * NZ;  // u0, u1, u2 of the group's row
  load_reg_twiddles<NZ>(twt, a.tw, threadIdx.x, blockDim.x);
  __syncthreads();
  const int b = blockIdx.y;
  const int64_t S = a.S;
  const float* kz = a.ky;
  const int64_t rows = S / H;
  const float2* m2 = a.mid2 + (int64_t)b * a.n_mid2 * S;
  float2* prod = a.prod + (int64_t)b * a.n_prod * S;
#pragma unroll 1
  for (int rr = 0; rr < 2; ++rr) {
    const int64_t r = ((int64_t)blockIdx.x * groups + g) * 2 + rr;
    if (r >= rows) break;  // uniform per group; rows is a multiple of 2 * groups
    const int64_t roff = r * H;
    float2 Z[E];
    if (KIND == FSM_NL_CONVECTION) {
      // mid2 layout per channel c: 3c: Y(X u_c), 3c+1: -> d_x u_c, 3c+2: -> d_y u_c
      const float2* F[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) F[i] = m2 + i * S + roff;
      float c0v[E], c1v[E], c2v[E];
      build_row<NZ>(Z, F[0], F[3], false, false, kz, t);  // u0 + i u1
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        ust[t + T * j] = Z[j].x;
        ust[NZ + t + T * j] = Z[j].y;
      }
      build_row<NZ>(Z, F[6], F[1], false, false, kz, t);  // u2 + i dx u0
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        ust[2 * NZ + t + T * j] = Z[j].x;
        c0v[j] = ust[t + T * j] * Z[j].y;
      }
      build_row<NZ>(Z, F[2], F[0], false, true, kz, t);  // dy u0 + i dz u0
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) c0v[j] += ust[NZ + t + T * j] * Z[j].x + ust[2 * NZ + t + T * j] * Z[j].y;
      build_row<NZ>(Z, F[4], F[5], false, false, kz, t);  // dx u1 + i dy u1
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) c1v[j] = ust[t + T * j] * Z[j].x + ust[NZ + t + T * j] * Z[j].y;
      build_row<NZ>(Z, F[3], F[7], true, false, kz, t);  // dz u1 + i dx u2
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        c1v[j] += ust[2 * NZ + t + T * j] * Z[j].x;
        c2v[j] = ust[t + T * j] * Z[j].y;
      }
      build_row<NZ>(Z, F[8], F[6], false, true, kz, t);  // dy u2 + i dz u2
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) c2v[j] += ust[NZ + t + T * j] * Z[j].x + ust[2 * NZ + t + T * j] * Z[j].y;
#pragma unroll
      for (int j = 0; j < E; ++j) Z[j] = make_float2(c0v[j], c1v[j]);
      reg_fft<NZ, false>(Z, scr, twt, t);
      split_one<NZ>(Z, t, lane, prod + roff, prod + S + roff);
#pragma unroll
      for (int j = 0; j < E; ++j) Z[j] = make_float2(c2v[j], 0.f);
      reg_fft<NZ, false>(Z, scr, twt, t);
      split_one<NZ>(Z, t, lane, prod + 2 * S + roff, nullptr);
    } else {
      // KS: mid2 0: Y(X phi) -> dz via i kz, 1: -> dx phi, 2: -> dy phi
      float p[E];
      build_row<NZ>(Z, m2 + S + roff, m2 + 2 * S + roff, false, false, kz, t);  // dx + i dy
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) p[j] = 0.5f * (Z[j].x * Z[j].x + Z[j].y * Z[j].y);
      build_row<NZ>(Z, m2 + roff, nullptr, true, false, kz, t);  // dz
      reg_fft<NZ, true>(Z, scr, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) Z[j] = make_float2(p[j] + 0.5f * Z[j].x * Z[j].x, 0.f);
      reg_fft<NZ, false>(Z, scr, twt, t);
      split_one<NZ>(Z, t, lane, prod + roff, nullptr);
    }
  }
}

template <int NY>
static int launch_axis1_inv(int n0, const StepArgs& a, cudaStream_t st) {
  using Cfg = TileCfg<NY>;
  const size_t smem = (size_t)(NY + 3 * Cfg::W * Cfg::P) * sizeof(float2);
  int rc = prep_smem(k_axis1_inv_r<NY>, smem);
  if (rc) return rc;
  dim3 grid((unsigned)((a.H + Cfg::W - 1) / Cfg::W), (unsigned)n0, (unsigned)(a.B * (a.n_mid / 2)));
  k_axis1_inv_r<NY><<<grid, 256, smem, st>>>(a);
  return cuda_check(cudaGetLastError(), "k_axis1_inv_r");
}

template <int NZ, int KIND>
static int launch_axis2(const StepArgs& a, cudaStream_t st) {
  using RS = RegShape<NZ>;
  constexpr int H = NZ / 2 + 1;
  const int64_t rows = a.S / H;
  int64_t groups_needed = rows / 2;
  int threads = (int)((groups_needed * RS::T < 256) ? groups_needed * RS::T : 256);
  const int groups = threads / RS::T;
  const size_t smem = (size_t)(NZ + groups * reg_scratch<NZ>()) * sizeof(float2) + (size_t)groups * 3 * NZ * sizeof(float);
  int rc = prep_smem(k_axis2_r<NZ, KIND>, smem);
  if (rc) return rc;
  dim3 grid((unsigned)((groups_needed + groups - 1) / groups), a.B);
  k_axis2_r<NZ, KIND><<<grid, threads, smem, st>>>(a);
  return cuda_check(cudaGetLastError(), "k_axis2_r");
}

int launch_volume_axis1_inv(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  switch (p->n[1]) {
    case 16: return launch_axis1_inv<16>(p->n[0], a, st);
    case 32: return launch_axis1_inv<32>(p->n[0], a, st);
    case 64: return launch_axis1_inv<64>(p->n[0], a, st);
    case 128: return launch_axis1_inv<128>(p->n[0], a, st);
    case 256: return launch_axis1_inv<256>(p->n[0], a, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "3D: unsupported second-axis length");
}

template <int KIND>
static int axis2_dispatch(int nz, const StepArgs& a, cudaStream_t st) {
  switch (nz) {
    case 16: return launch_axis2<16, KIND>(a, st);
    case 32: return launch_axis2<32, KIND>(a, st);
    case 64: return launch_axis2<64, KIND>(a, st);
    case 128: return launch_axis2<128, KIND>(a, st);
    case 256: return launch_axis2<256, KIND>(a, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "3D: unsupported last-axis length");
}

int launch_volume_axis2(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  if (p->nl == FSM_NL_KS) return axis2_dispatch<FSM_NL_KS>(p->n[2], a, st);
  return axis2_dispatch<FSM_NL_CONVECTION>(p->n[2], a, st);
}

int launch_volume_axis1_fwd(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  const int rc = transform_c2c_strided_reg(p->n[1], false, a.prod, (int64_t)a.B * a.n_prod * p->n[0], a.H, p->tw, st);
  if (rc == -1) return set_error(FSM_ERR_UNSUPPORTED, "3D: unsupported second-axis length");
  return rc;
}

}  // namespace fsm
