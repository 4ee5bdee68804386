// Elementwise kernels of the hand-written SETDRK4 adjoint (torchfsm_gb300/adjoint.py): the
// Convection vector-Jacobian product's physical-space products and spectral combination, and
// the accumulation of the coefficient-table cotangents. Each replaces a chain of small tensor
// operations of one adjoint step (the step is a CUDA graph of a few hundred launches, so the
// launches, not the bytes, set its time).
#include "fsm_internal.cuh"

namespace {

// tbar[i] += Re(conj(x[i]) y[i])
__global__ void k_adj_accumulate(int64_t n, const float2* __restrict__ x, const float2* __restrict__ y,
                                 double* __restrict__ tbar) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = x[i], b = y[i];
    tbar[i] += (double)(a.x * b.x + a.y * b.y);
  }
}

// Per grid point r of sample b: w_c = scale nbar_c; ubar_c = sum_c' w_c' g_c[c'] (g_c = d_c u,
// channel c'); uw_i[c] = u_i w_c. Arrays [B][C][R]; uw is [nd][B][C][R].
template <int ND>
__global__ void k_adj_vjp_products(int B, int64_t R, float scale, const float* __restrict__ nbar,
                                   const float* __restrict__ u, const float* __restrict__ g0,
                                   const float* __restrict__ g1, const float* __restrict__ g2,
                                   float* __restrict__ ubar, float* __restrict__ uw) {
  constexpr int C = ND;
  const float* g[3] = {g0, g1, g2};
  const int64_t total = (int64_t)B * R;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / R, r = q - b * R;
    const int64_t base = b * C * R + r;
    float w[C], uu[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      w[c] = scale * nbar[base + c * R];
      uu[c] = u[base + c * R];
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
      float s = 0.f;
#pragma unroll
      for (int cp = 0; cp < C; ++cp) s += w[cp] * g[c][base + cp * R];
      ubar[base + c * R] = s;
    }
#pragma unroll
    for (int i = 0; i < ND; ++i)
#pragma unroll
      for (int c = 0; c < C; ++c) uw[(int64_t)i * B * C * R + base + c * R] = uu[i] * w[c];
  }
}

// out[b][c][s] = m[s] (sub[b][c][s] - i sum_i k_i[s] suw[i][b][c][s])
template <int ND>
__global__ void k_adj_vjp_combine(int BC, int64_t S, const float2* __restrict__ sub, const float2* __restrict__ suw,
                                  const float* __restrict__ k0, const float* __restrict__ k1,
                                  const float* __restrict__ k2, const float* __restrict__ m,
                                  float2* __restrict__ out) {
  const float* k[3] = {k0, k1, k2};
  const int64_t total = (int64_t)BC * S;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = q % S;
    float2 acc = make_float2(0.f, 0.f);  // sum_i k_i suw_i
#pragma unroll
    for (int i = 0; i < ND; ++i) {
      const float2 v = suw[(int64_t)i * total + q];
      acc.x += k[i][s] * v.x;
      acc.y += k[i][s] * v.y;
    }
    const float2 a = sub[q];
    // a - i acc = (a.x + acc.y, a.y - acc.x)
    out[q] = make_float2(m[s] * (a.x + acc.y), m[s] * (a.y - acc.x));
  }
}

inline unsigned grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (unsigned)(g > 152 * 16 ? 152 * 16 : (g < 1 ? 1 : g));
}

}  // namespace

using namespace fsm;

extern "C" {

int fsm_adj_accumulate(int64_t n, const void* x, const void* y, double* tbar, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y || !tbar))) return set_error(FSM_ERR_INVALID, "adj_accumulate arguments");
  if (n == 0) return FSM_OK;
  k_adj_accumulate<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, (const float2*)x, (const float2*)y, tbar);
  return cuda_check(cudaGetLastError(), "k_adj_accumulate");
}

int fsm_adj_vjp_products(int32_t batch, int32_t nd, int64_t points, float scale, const float* nbar, const float* u,
                         const float* g0, const float* g1, const float* g2, float* ubar, float* uw, void* stream) {
  if (batch < 1 || points < 1 || nd < 1 || nd > 3 || !nbar || !u || !g0 || (nd > 1 && !g1) || (nd > 2 && !g2) ||
      !ubar || !uw)
    return set_error(FSM_ERR_INVALID, "adj_vjp_products arguments");
  const unsigned grid = grid_for((int64_t)batch * points);
  cudaStream_t st = (cudaStream_t)stream;
  switch (nd) {
    case 1: k_adj_vjp_products<1><<<grid, 256, 0, st>>>(batch, points, scale, nbar, u, g0, g1, g2, ubar, uw); break;
    case 2: k_adj_vjp_products<2><<<grid, 256, 0, st>>>(batch, points, scale, nbar, u, g0, g1, g2, ubar, uw); break;
    default: k_adj_vjp_products<3><<<grid, 256, 0, st>>>(batch, points, scale, nbar, u, g0, g1, g2, ubar, uw); break;
  }
  return cuda_check(cudaGetLastError(), "k_adj_vjp_products");
}

int fsm_adj_vjp_combine(int32_t batch_channels, int32_t nd, int64_t points, const void* sub, const void* suw,
                        const float* k0, const float* k1, const float* k2, const float* m, void* out, void* stream) {
  if (batch_channels < 1 || points < 1 || nd < 1 || nd > 3 || !sub || !suw || !k0 || (nd > 1 && !k1) ||
      (nd > 2 && !k2) || !m || !out)
    return set_error(FSM_ERR_INVALID, "adj_vjp_combine arguments");
  const unsigned grid = grid_for((int64_t)batch_channels * points);
  cudaStream_t st = (cudaStream_t)stream;
  const float2* a = (const float2*)sub;
  const float2* w = (const float2*)suw;
  float2* o = (float2*)out;
  switch (nd) {
    case 1: k_adj_vjp_combine<1><<<grid, 256, 0, st>>>(batch_channels, points, a, w, k0, k1, k2, m, o); break;
    case 2: k_adj_vjp_combine<2><<<grid, 256, 0, st>>>(batch_channels, points, a, w, k0, k1, k2, m, o); break;
    default: k_adj_vjp_combine<3><<<grid, 256, 0, st>>>(batch_channels, points, a, w, k0, k1, k2, m, o); break;
  }
  return cuda_check(cudaGetLastError(), "k_adj_vjp_combine");
}

}  // extern "C"
