// The hand-written SETDRK4 adjoint (gradients of integrate, torchfsm_gb300/adjoint.py):
// fsm_step_adjoint runs one whole adjoint step of a Convection program (the four stages
// recomputed with the library's transforms, their vector-Jacobian products, the backward
// recurrence and the coefficient-table cotangents) in about 50 launches; the elementwise kernels
// of its vector-Jacobian product are also exported on their own.
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

// ---- one SETDRK4 adjoint step of a Convection program (fsm_step_adjoint) -------------------
//
// Forward step (integrator/_stable_etdrk/_setdrk_step.py:55-82, tables E, E2, c1, c4, c5, c6 of
// the plan): a1 = E2 u + c1 n0, a2 = E2 u + c1 n1, a3 = E2 a1 + c1 (2 n2 - n0),
// u' = E u + c4 n0 + 2 c5 (n1 + n2) + c6 n3 with n_s = N(a_s), N(a) = coef rfft(sum_i u_i d_i u_c)
// over the dealiased fields u = irfft(m a), d_i u = irfft(i k_i m a)
// (operator/generic/_convection.py:43-46). Real symbols: the tables are real, so their adjoint is
// the same multiplication; only their real parts are read.

// Geometry of the half spectrum: per-axis wavenumbers 2 pi f and keep flags (fftfreq order).
struct AdjGeom {
  int nd;
  int n[3];
  int h;
  const float* k[3];
  const uint8_t* keep[3];
};

__device__ __forceinline__ float adj_point(const AdjGeom& g, int64_t s, float (&k)[3]) {
  int idx[3] = {0, 0, 0};
  int64_t rest = s;
  idx[g.nd - 1] = (int)(rest % g.h);
  rest /= g.h;
  for (int ax = g.nd - 2; ax >= 0; --ax) {
    idx[ax] = (int)(rest % g.n[ax]);
    rest /= g.n[ax];
  }
  float m = 1.f;
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    k[ax] = 0.f;
    if (ax < g.nd) {
      k[ax] = g.k[ax][idx[ax]];
      m *= (float)g.keep[ax][idx[ax]];
    }
  }
  return m;
}

// Real parts of the plan's coefficient tables (SETDRK4 order E - 1, E2 - 1, c1, c4, c5, c6).
struct AdjTabs {
  const float2* tab;
  int64_t ts;
  int lin_batch, lin_ch;
  int64_t S;
  __device__ __forceinline__ float operator()(int t, int64_t b, int c, int64_t s) const {
    return tab[t * ts + ((lin_batch > 1 ? b : 0) * lin_ch + (lin_ch > 1 ? c : 0)) * S + s].x;
  }
};

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 sc(float2 a, float k) { return make_float2(k * a.x, k * a.y); }
__device__ __forceinline__ float2 ad(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float redot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }  // Re(conj(a) b)
// E a from the table value em1 = E - 1 (real): a + em1 a
__device__ __forceinline__ float2 xe(float2 a, float em1) { return make_float2(fmaf(em1, a.x, a.x), fmaf(em1, a.y, a.y)); }

// Stage input a = x (combine 0) or E2 x + c1 (alpha y + beta z) (z may be null), optionally stored,
// and the fields of the nonlinear term: F[0] = m a, F[1 + i] = i k_i m a ([1 + nd][B][C][S]).
__global__ void k_adjs_fields(AdjGeom g, AdjTabs T, int64_t total, int C, int combine, const float2* __restrict__ x,
                              const float2* __restrict__ y, float alpha, const float2* __restrict__ z, float beta,
                              float2* __restrict__ store, float2* __restrict__ F) {
  const int64_t S = T.S;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = q % S;
    const int c = (int)((q / S) % C);
    const int64_t b = q / ((int64_t)C * S);
    float2 a = x[q];
    if (combine) {
      float2 r = sc(y[q], alpha);
      if (z) r = ad(r, sc(z[q], beta));
      a = ad(xe(a, T(1, b, c, s)), sc(r, T(2, b, c, s)));
      if (store) store[q] = a;
    }
    float k[3];
    const float m = adj_point(g, s, k);
    const float2 d = sc(a, m);
    F[q] = d;
    for (int i = 0; i < g.nd; ++i) F[(int64_t)(1 + i) * total + q] = f2(-k[i] * d.y, k[i] * d.x);
  }
}

// p[b][c][r] = coef sum_i u_i g_i[c] with u_i = P[0][b][i][r], g_i[c] = P[1 + i][b][c][r].
__global__ void k_adjs_product(int64_t total, int C, int64_t R, float coef, const float* __restrict__ P,
                               float* __restrict__ p) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = q % R;
    const int64_t b = q / ((int64_t)C * R);
    float acc = 0.f;
    for (int i = 0; i < C; ++i) acc += P[(b * C + i) * R + r] * P[(int64_t)(1 + i) * total + q];
    p[q] = coef * acc;
  }
}

// Start of the backward pass from ub = dLoss/du': u_bar = E ub, n0b = c4 ub, n1b = n2b = 2 c5 ub,
// nbs = c6 ub (= n3b, the first vector-Jacobian product's input); table cotangents
// tb[0] += Re(ub* u), tb[3] += Re(ub* n0), tb[4] += Re(ub* 2 (n1 + n2)), tb[5] += Re(ub* n3).
__global__ void k_adjs_begin(AdjTabs T, int64_t total, int C, const float2* __restrict__ ub,
                             const float2* __restrict__ u, const float2* __restrict__ n0, const float2* __restrict__ n1,
                             const float2* __restrict__ n2, const float2* __restrict__ n3, float2* __restrict__ ubar,
                             float2* __restrict__ n0b, float2* __restrict__ n1b, float2* __restrict__ n2b,
                             float2* __restrict__ nbs, double* __restrict__ tb) {
  const int64_t S = T.S;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = q % S;
    const int c = (int)((q / S) % C);
    const int64_t b = q / ((int64_t)C * S);
    const float2 v = ub[q];
    ubar[q] = xe(v, T(0, b, c, s));
    n0b[q] = sc(v, T(3, b, c, s));
    const float2 w = sc(v, 2.f * T(4, b, c, s));
    n1b[q] = w;
    n2b[q] = w;
    nbs[q] = sc(v, T(5, b, c, s));
    if (tb) {
      tb[q] += (double)redot(v, u[q]);
      tb[3 * total + q] += (double)redot(v, n0[q]);
      tb[4 * total + q] += (double)redot(v, sc(ad(n1[q], n2[q]), 2.f));
      tb[5 * total + q] += (double)redot(v, n3[q]);
    }
  }
}

// End of a vector-Jacobian product: abar = (m / N) (SQ[0] - i sum_i k_i SQ[1 + i]), then the
// backward recurrence of the stage it belongs to (mode = stage):
//  3: a1b = E2 abar; nbs = n2b + 2 c1 abar; n0b -= c1 abar; tb1 += Re(abar* a1); tb2 += Re(abar* (2 n2 - n0))
//  2: ubar += E2 abar; nbs = n1b + c1 abar; tb1 += Re(abar* u); tb2 += Re(abar* n1)
//  1: t = a1b + abar; ubar += E2 t; nbs = n0b + c1 t; tb1 += Re(t* u); tb2 += Re(t* n0)
//  0: out = ubar + abar
struct AdjEnd {
  const float2* SQ;
  const float2 *u, *a1, *n0, *n1, *n2;
  float2 *ubar, *a1b, *n0b, *n1b, *n2b, *nbs, *out;
  double* tb;
};

__global__ void k_adjs_end(AdjGeom g, AdjTabs T, int64_t total, int C, float inv_n, int mode, AdjEnd e) {
  const int64_t S = T.S;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = q % S;
    const int c = (int)((q / S) % C);
    const int64_t b = q / ((int64_t)C * S);
    float k[3];
    const float m = adj_point(g, s, k) * inv_n;
    float2 acc = f2(0.f, 0.f);  // sum_i k_i SQ[1 + i]
    for (int i = 0; i < g.nd; ++i) acc = ad(acc, sc(e.SQ[(int64_t)(1 + i) * total + q], k[i]));
    const float2 sub = e.SQ[q];
    const float2 abar = f2(m * (sub.x + acc.y), m * (sub.y - acc.x));  // m (sub - i acc)
    if (mode == 0) {
      e.out[q] = ad(e.ubar[q], abar);
      continue;
    }
    const float E2m1 = T(1, b, c, s), c1 = T(2, b, c, s);
    if (mode == 3) {
      e.a1b[q] = xe(abar, E2m1);
      e.nbs[q] = ad(e.n2b[q], sc(abar, 2.f * c1));
      const float2 n0 = e.n0[q];
      e.n0b[q] = ad(e.n0b[q], sc(abar, -c1));
      if (e.tb) {
        e.tb[total + q] += (double)redot(abar, e.a1[q]);
        e.tb[2 * total + q] += (double)redot(abar, ad(sc(e.n2[q], 2.f), sc(n0, -1.f)));
      }
    } else if (mode == 2) {
      e.ubar[q] = ad(e.ubar[q], xe(abar, E2m1));
      e.nbs[q] = ad(e.n1b[q], sc(abar, c1));
      if (e.tb) {
        e.tb[total + q] += (double)redot(abar, e.u[q]);
        e.tb[2 * total + q] += (double)redot(abar, e.n1[q]);
      }
    } else {
      const float2 t = ad(e.a1b[q], abar);
      e.ubar[q] = ad(e.ubar[q], xe(t, E2m1));
      e.nbs[q] = ad(e.n0b[q], sc(t, c1));
      if (e.tb) {
        e.tb[total + q] += (double)redot(t, e.u[q]);
        e.tb[2 * total + q] += (double)redot(t, e.n0[q]);
      }
    }
  }
}

// Workspace of fsm_step_adjoint: per-stage physical fields, physical and half-spectrum scratch,
// the stage values and the backward accumulators.
struct AdjLayout {
  size_t P[4], Q, nbp, F, half[11], bytes;
};

inline size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

AdjLayout adj_layout(const FsmPlan* p, int32_t batch) {
  AdjLayout L;
  const size_t nb = 1 + (size_t)p->ndim;
  const size_t tr = (size_t)batch * p->C * p->R, th = (size_t)batch * p->C * p->S;
  size_t o = 0;
  for (int s = 0; s < 4; ++s) {
    L.P[s] = o;
    o += a256(nb * tr * sizeof(float));
  }
  L.Q = o;
  o += a256(nb * tr * sizeof(float));
  L.nbp = o;
  o += a256(tr * sizeof(float));
  L.F = o;
  o += a256(nb * th * sizeof(float2));
  for (int i = 0; i < 11; ++i) {
    L.half[i] = o;
    o += a256(th * sizeof(float2));
  }
  L.bytes = o;
  return L;
}

int check_adjoint_plan(const FsmPlan* p) {
  if (p->integ != FSM_SETDRK4 || p->nl != FSM_NL_CONVECTION || p->source || p->C != p->ndim)
    return fsm::set_error(FSM_ERR_UNSUPPORTED, "step_adjoint: SETDRK4 Convection programs (C == ndim) without sources");
  return FSM_OK;
}

}  // namespace

using namespace fsm;

extern "C" {

int fsm_step_adjoint_workspace_bytes(const FsmPlan* p, int32_t batch, size_t* bytes) {
  if (!p || batch < 1 || !bytes) return set_error(FSM_ERR_INVALID, "step_adjoint_workspace_bytes arguments");
  int rc = check_adjoint_plan(p);
  if (rc) return rc;
  *bytes = adj_layout(p, batch).bytes;
  return FSM_OK;
}

int fsm_step_adjoint(const FsmPlan* p, int32_t batch, const void* u, const void* ubar_next, void* ubar, double* tbar,
                     void* workspace, size_t workspace_bytes, void* stream) {
  if (!p || batch < 1 || !u || !ubar_next || !ubar || !workspace)
    return set_error(FSM_ERR_INVALID, "step_adjoint arguments");
  int rc = check_adjoint_plan(p);
  if (rc) return rc;
  if (p->lin_batch > 1 && batch > p->lin_batch) return set_error(FSM_ERR_INVALID, "step_adjoint: batch above the plan's table entries");
  const AdjLayout L = adj_layout(p, batch);
  if (workspace_bytes < L.bytes)
    return set_error(FSM_ERR_INVALID, "step_adjoint: workspace too small: need " + std::to_string(L.bytes) + " bytes");
  cudaStream_t st = (cudaStream_t)stream;
  const int nd = p->ndim, C = p->C, nb = 1 + nd;
  const int64_t th = (int64_t)batch * C * p->S, tr = (int64_t)batch * C * p->R;
  char* ws = (char*)workspace;
  float* P[4];
  for (int s = 0; s < 4; ++s) P[s] = (float*)(ws + L.P[s]);
  float* Q = (float*)(ws + L.Q);
  float* nbp = (float*)(ws + L.nbp);
  float2* F = (float2*)(ws + L.F);
  float2* h[11];
  for (int i = 0; i < 11; ++i) h[i] = (float2*)(ws + L.half[i]);
  float2 *n0 = h[0], *n1 = h[1], *n2 = h[2], *n3 = h[3], *a1 = h[4], *ubar_acc = h[5], *a1b = h[6], *n0b = h[7],
         *n1b = h[8], *n2b = h[9], *nbs = h[10];
  const float2* uu = (const float2*)u;
  AdjGeom g;
  g.nd = nd;
  g.h = p->h;
  for (int i = 0; i < 3; ++i) {
    g.n[i] = i < nd ? p->n[i] : 1;
    g.k[i] = i < nd ? p->kvec + p->koff[i] : nullptr;
    g.keep[i] = i < nd ? p->keep + p->koff[i] : nullptr;
  }
  AdjTabs T{p->tab, p->tstride, p->lin_batch, p->lin_ch, p->S};
  const unsigned gh = grid_for(th), gr = grid_for(tr);

  // forward stages, keeping each stage's physical fields for its vector-Jacobian product
  const float2* xs[4] = {uu, uu, uu, a1};
  const float2* ys[4] = {nullptr, n0, n1, n2};
  const float2* zs[4] = {nullptr, nullptr, nullptr, n0};
  const float al[4] = {0.f, 1.f, 1.f, 2.f}, be[4] = {0.f, 0.f, 0.f, -1.f};
  float2* outs[4] = {n0, n1, n2, n3};
  for (int s = 0; s < 4; ++s) {
    k_adjs_fields<<<gh, 256, 0, st>>>(g, T, th, C, s > 0, xs[s], ys[s], al[s], zs[s], be[s], s == 1 ? a1 : nullptr, F);
    if ((rc = cuda_check(cudaGetLastError(), "k_adjs_fields"))) return rc;
    if ((rc = fsm_irfftn(p, nb * batch * C, F, P[s], stream))) return rc;
    k_adjs_product<<<gr, 256, 0, st>>>(tr, C, p->R, p->nl_coef, P[s], Q);
    if ((rc = cuda_check(cudaGetLastError(), "k_adjs_product"))) return rc;
    if ((rc = fsm_rfftn(p, batch * C, Q, outs[s], stream))) return rc;
  }

  // backward
  k_adjs_begin<<<gh, 256, 0, st>>>(T, th, C, (const float2*)ubar_next, uu, n0, n1, n2, n3, ubar_acc, n0b, n1b, n2b,
                                   nbs, tbar);
  if ((rc = cuda_check(cudaGetLastError(), "k_adjs_begin"))) return rc;
  AdjEnd e{F, uu, a1, n0, n1, n2, ubar_acc, a1b, n0b, n1b, n2b, nbs, (float2*)ubar, tbar};
  const float scale = p->nl_coef * (float)p->R;
  for (int s = 3; s >= 0; --s) {
    // w = coef N irfft(nbar); ubar_c = sum_c' w_c' d_c u_c', u_i w_c -> rfft -> combination
    if ((rc = fsm_irfftn(p, batch * C, nbs, nbp, stream))) return rc;
    const float* Ps = P[s];
    const float* g1 = nd > 1 ? Ps + 2 * tr : nullptr;
    const float* g2 = nd > 2 ? Ps + 3 * tr : nullptr;
    switch (nd) {
      case 1: k_adj_vjp_products<1><<<gr / C + 1, 256, 0, st>>>(batch, p->R, scale, nbp, Ps, Ps + tr, g1, g2, Q, Q + tr); break;
      case 2: k_adj_vjp_products<2><<<gr / C + 1, 256, 0, st>>>(batch, p->R, scale, nbp, Ps, Ps + tr, g1, g2, Q, Q + tr); break;
      default: k_adj_vjp_products<3><<<gr / C + 1, 256, 0, st>>>(batch, p->R, scale, nbp, Ps, Ps + tr, g1, g2, Q, Q + tr); break;
    }
    if ((rc = cuda_check(cudaGetLastError(), "k_adj_vjp_products"))) return rc;
    if ((rc = fsm_rfftn(p, nb * batch * C, Q, F, stream))) return rc;
    k_adjs_end<<<gh, 256, 0, st>>>(g, T, th, C, (float)(1.0 / (double)p->R), s, e);
    if ((rc = cuda_check(cudaGetLastError(), "k_adjs_end"))) return rc;
  }
  return FSM_OK;
}

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
