// Internal definitions shared by the torchfsm_gb300 CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/torchfsm_gb300.h"
#include "fsm_fft.cuh"

namespace fsm {

constexpr int kTwiddleMax = 4096;  // master twiddle table W_4096^k
constexpr int kMaxTables = 7;

// Number of nonlinear evaluations per step of each scheme.
// Explicit Runge-Kutta tableaus (integrator/_rk.py:82-255), stages that feed the step only:
// a[i][j] weighs stage j's slope in the input of stage i (j < i), b[i] in the new state. The
// reference evaluates one more slope for Euler (a zero-weight repeat) and for BogackiShampine23
// and Dorpi45 (the first-same-as-last stage, used only by the adaptive error estimate); those
// evaluations do not enter the fixed-step result and are not run here.
struct RKTableau {
  int s;
  float a[6][6];
  float b[6];
};

__host__ __device__ constexpr bool is_rk(int integ) { return integ >= FSM_RK_EULER && integ <= FSM_RK_CASHKARP45; }

__host__ __device__ constexpr RKTableau rk_tableau(int integ) {
  switch (integ) {
    case FSM_RK_EULER: return {1, {{0}}, {1.f}};
    case FSM_RK_MIDPOINT: return {2, {{0}, {0.5f}}, {0.f, 1.f}};
    case FSM_RK_HEUN12: return {2, {{0}, {1.f}}, {0.5f, 0.5f}};
    case FSM_RK_RALSTON12: return {2, {{0}, {2.f / 3.f}}, {0.25f, 0.75f}};
    case FSM_RK_BOGACKI_SHAMPINE23: return {3, {{0}, {0.5f}, {0.f, 0.75f}}, {2.f / 9.f, 1.f / 3.f, 4.f / 9.f}};
    case FSM_RK4: return {4, {{0}, {0.5f}, {0.f, 0.5f}, {0.f, 0.f, 1.f}}, {1.f / 6.f, 1.f / 3.f, 1.f / 3.f, 1.f / 6.f}};
    case FSM_RK4_38RULE:
      // the reference's last row [1, -1, 1, 1] read as [c, a30, a31, a32] gives a3 = (-1, 1, 1)
      // (the textbook 3/8 rule has (1, -1, 1)); kept as the reference runs it
      return {4, {{0}, {1.f / 3.f}, {-1.f / 3.f, 1.f}, {-1.f, 1.f, 1.f}}, {0.125f, 0.375f, 0.375f, 0.125f}};
    case FSM_RK_DORPI45:
      return {6,
              {{0},
               {1.f / 5.f},
               {3.f / 40.f, 9.f / 40.f},
               {44.f / 45.f, -56.f / 15.f, 32.f / 9.f},
               {19372.f / 6561.f, -25360.f / 2187.f, 64448.f / 6561.f, -212.f / 729.f},
               {9017.f / 3168.f, -355.f / 33.f, 46732.f / 5247.f, 49.f / 176.f, -5103.f / 18656.f}},
              {35.f / 384.f, 0.f, 500.f / 1113.f, 125.f / 192.f, -2187.f / 6784.f, 11.f / 84.f}};
    case FSM_RK_FEHLBERG45:
      return {6,
              {{0},
               {1.f / 4.f},
               {3.f / 32.f, 9.f / 32.f},
               {1932.f / 2197.f, -7200.f / 2197.f, 7296.f / 2197.f},
               {439.f / 216.f, -8.f, 3680.f / 513.f, -845.f / 4104.f},
               {-8.f / 27.f, 2.f, -3544.f / 2565.f, 1859.f / 4104.f, -11.f / 40.f}},
              {16.f / 135.f, 0.f, 6656.f / 12825.f, 28561.f / 56430.f, -9.f / 50.f, 2.f / 55.f}};
    case FSM_RK_CASHKARP45:
      return {6,
              {{0},
               {1.f / 5.f},
               {3.f / 40.f, 9.f / 40.f},
               {3.f / 10.f, -9.f / 10.f, 6.f / 5.f},
               {-11.f / 54.f, 5.f / 2.f, -70.f / 27.f, 35.f / 27.f},
               {1631.f / 55296.f, 175.f / 512.f, 575.f / 13824.f, 44275.f / 110592.f, 253.f / 4096.f}},
              {37.f / 378.f, 0.f, 250.f / 621.f, 125.f / 594.f, 0.f, 512.f / 1771.f}};
  }
  return {0, {{0}}, {0}};
}

// The tableaus in constant memory for the kernels (indexed by integ - FSM_RK_EULER).
static __constant__ RKTableau kRKTab[10] = {
    rk_tableau(FSM_RK_EULER),   rk_tableau(FSM_RK_MIDPOINT),       rk_tableau(FSM_RK_HEUN12),
    rk_tableau(FSM_RK_RALSTON12), rk_tableau(FSM_RK_BOGACKI_SHAMPINE23), rk_tableau(FSM_RK4),
    rk_tableau(FSM_RK4_38RULE), rk_tableau(FSM_RK_DORPI45),         rk_tableau(FSM_RK_FEHLBERG45),
    rk_tableau(FSM_RK_CASHKARP45)};

__host__ __device__ inline int scheme_stages(int integ) {
  if (is_rk(integ)) return rk_tableau(integ).s;
  if (integ == FSM_APPLY) return 1;
  switch (integ) {
    case FSM_SETDRK4: return 4;
    case FSM_SETDRK3: return 3;
    case FSM_SETDRK2:
    case FSM_ETDRK2: return 2;
    case FSM_SETDRK1:
    case FSM_ETDRK1: return 1;
    default: return 0;
  }
}

// Number of coefficient tables of each scheme (order of the tables below).
//  SETDRK4: E, E2, c1, c4, c5, c6        (c2 = c3 = c1)
//  SETDRK3: E, E2, c1, c2, c3, c4, c5
//  SETDRK2 / ETDRK2: E, c1, c2
//  SETDRK1 / ETDRK1: E, c1
//  ETDRK0: E
// The exponential tables E = exp(dt L) and E2 = exp(dt L / 2) are stored as E - 1 and E2 - 1
// (evaluated in FP64, then rounded) and applied as u + (E - 1) u with fused multiply-adds
// (cexpmul). E itself rounded to FP32 carries a fixed relative error of up to 2^-25 per mode,
// which the step repeats: after n steps the state is off by n times that error (2D vorticity
// NS 256^2, 1000 steps: rel-L2 1.8e-5 against FP64, all of it from this rounding). E - 1 is
// small where E is close to 1, so its rounding error is smaller by the same factor.
__host__ __device__ inline int scheme_tables(int integ) {
  if (is_rk(integ)) return 2;  // dt L, dt
  if (integ == FSM_APPLY) return 1;  // L
  switch (integ) {
    case FSM_SETDRK4: return 6;
    case FSM_SETDRK3: return 7;
    case FSM_SETDRK2:
    case FSM_ETDRK2: return 3;
    case FSM_SETDRK1:
    case FSM_ETDRK1: return 2;
    case FSM_ETDRK0: return 1;
    default: return 0;
  }
}

// Auxiliary per-point state arrays a scheme keeps between stages (acc, q).
__host__ __device__ inline int scheme_aux(int integ) {
  if (is_rk(integ)) {
    const int st = rk_tableau(integ).s;
    return st > 1 ? st : 0;  // partial inputs of stages 1..s-1 and the weighted slope sum
  }
  switch (integ) {
    case FSM_SETDRK4:
    case FSM_SETDRK3: return 2;
    case FSM_SETDRK2:
    case FSM_ETDRK2: return 1;
    default: return 0;
  }
}

// exp(dt L) u from the table value e = exp(dt L) - 1: u + e u, each component one fused
// multiply-add chain (exact product, one rounding for a real e).
__device__ __forceinline__ float2 cexpmul(float2 e, float2 u) { return cfma(e, u, u); }

// One stage of an exponential Runge-Kutta step at one spectral point.
//
// `nv` is the nonlinear value N_s of stage s (s = 0 .. stages-1), `u` the
// state, `acc`/`q` the scheme's running sums, `tab` the point's entry of the
// first coefficient table and `ts` the distance between tables. Returns the
// input of stage s+1, or the new state after the last stage (which is also
// stored to *u). The recurrences are the reference's stage formulas
// (integrator/_stable_etdrk/_setdrk_step.py:5-82, integrator/_etdrk.py:62-82)
// regrouped into running sums so that each stage reads the fewest arrays:
//  SETDRK4: acc = E u + c4 n0 (+ 2 c5 n1 + 2 c5 n2), q = E2 (E2 u + c1 n0) - c1 n0,
//           a1 = E2 u + c1 n0, a2 = E2 u + c1 n1, a3 = q + 2 c1 n2, u' = acc + c6 n3.
//  SETDRK3: acc = E u + c3 n0 (+ c4 n1), q = E u - c2 n0, a1 = E2 u + c1 n0,
//           a2 = q + 2 c2 n1, u' = acc + c5 n2.
//  (S)ETDRK2: a1 = E u + c1 n0, acc = a1 - c2 n0, u' = acc + c2 n1.
//  (S)ETDRK1: u' = E u + c1 n0.
template <int INTEG, int S>
__device__ __forceinline__ float2 etd_stage_c(float2 nv, float2* __restrict__ u, float2* __restrict__ acc,
                                              float2* __restrict__ q, const float2* __restrict__ tab, int64_t ts) {
  if (INTEG == FSM_SETDRK4) {
    if (S == 0) {
      const float2 uu = *u;
      const float2 Em1 = tab[0], E2m1 = tab[ts], c1 = tab[2 * ts], c4 = tab[3 * ts];
      const float2 a1 = cfma(c1, nv, cexpmul(E2m1, uu));
      *acc = cfma(c4, nv, cexpmul(Em1, uu));
      *q = cfma(make_float2(-c1.x, -c1.y), nv, cexpmul(E2m1, a1));
      return a1;
    } else if (S == 1) {
      const float2 uu = *u;
      const float2 E2m1 = tab[ts], c1 = tab[2 * ts], c5 = tab[4 * ts];
      *acc = cfma(cscale(c5, 2.f), nv, *acc);
      return cfma(c1, nv, cexpmul(E2m1, uu));
    } else if (S == 2) {
      const float2 c1 = tab[2 * ts], c5 = tab[4 * ts];
      *acc = cfma(cscale(c5, 2.f), nv, *acc);
      return cfma(cscale(c1, 2.f), nv, *q);
    } else {
      const float2 c6 = tab[5 * ts];
      const float2 un = cfma(c6, nv, *acc);
      *u = un;
      return un;
    }
  } else if (INTEG == FSM_SETDRK3) {
    if (S == 0) {
      const float2 uu = *u;
      const float2 Em1 = tab[0], E2m1 = tab[ts], c1 = tab[2 * ts], c2 = tab[3 * ts], c3 = tab[4 * ts];
      const float2 Eu = cexpmul(Em1, uu);
      *acc = cfma(c3, nv, Eu);
      *q = cfma(make_float2(-c2.x, -c2.y), nv, Eu);
      return cfma(c1, nv, cexpmul(E2m1, uu));
    } else if (S == 1) {
      const float2 c2 = tab[3 * ts], c4 = tab[5 * ts];
      *acc = cfma(c4, nv, *acc);
      return cfma(cscale(c2, 2.f), nv, *q);
    } else {
      const float2 c5 = tab[6 * ts];
      const float2 un = cfma(c5, nv, *acc);
      *u = un;
      return un;
    }
  } else if (INTEG == FSM_SETDRK2 || INTEG == FSM_ETDRK2) {
    if (S == 0) {
      const float2 uu = *u;
      const float2 Em1 = tab[0], c1 = tab[ts], c2 = tab[2 * ts];
      const float2 a1 = cfma(c1, nv, cexpmul(Em1, uu));
      *acc = cfma(make_float2(-c2.x, -c2.y), nv, a1);
      return a1;
    } else {
      const float2 c2 = tab[2 * ts];
      const float2 un = cfma(c2, nv, *acc);
      *u = un;
      return un;
    }
  } else {  // (S)ETDRK1, ETDRK0
    const float2 Em1 = tab[0], c1 = tab[ts];
    const float2 un = cfma(c1, nv, cexpmul(Em1, *u));
    *u = un;
    return un;
  }
}

// One explicit Runge-Kutta stage at one point (integrator/_rk.py:43-58 with f = L u + N(u),
// operator/_base.py:408-431). Slopes are kept scaled by dt: K = (dt L) a + dt N(a), from the
// tables dt L (tab[0]) and dt (tab[ts].x). aux[j * astride] holds, for j < s-1, the partial
// input P_{j+1} = sum_i a[j+1][i] K_i of stage j+1 and, at j = s-1, the sum B = sum_i b[i] K_i.
// Stage i reads the state u and P_i (a_i = u + P_i), adds its slope to every later partial
// input and to B, and returns a_{i+1}; the last stage writes u + B + b[s-1] K to u.
__device__ __forceinline__ float2 rk_stage(int integ, int i, float2 nv, float2* __restrict__ u,
                                           float2* __restrict__ aux, int64_t astride,
                                           const float2* __restrict__ tab, int64_t ts) {
  const RKTableau& T = kRKTab[integ - FSM_RK_EULER];
  const float2 uu = *u;
  const float2 a = (i == 0) ? uu : cadd(uu, aux[(int64_t)(i - 1) * astride]);
  const float dt = tab[ts].x;
  const float2 K = cfma(tab[0], a, cscale(nv, dt));
  if (i == T.s - 1) {
    float2 un = cadd(uu, cscale(K, T.b[i]));
    if (i > 0) un = cadd(un, aux[(int64_t)(T.s - 1) * astride]);
    *u = un;
    return un;
  }
  float2 next = uu;
  for (int m = i + 1; m < T.s; ++m) {
    float2* pm = aux + (int64_t)(m - 1) * astride;
    const float w = T.a[m][i];
    float2 p;
    if (i == 0) {
      p = cscale(K, w);
      *pm = p;
    } else if (w != 0.f) {
      p = cfma(make_float2(w, 0.f), K, *pm);
      *pm = p;
    } else if (m == i + 1) {
      p = *pm;
    } else {
      continue;
    }
    if (m == i + 1) next = cadd(uu, p);
  }
  float2* pb = aux + (int64_t)(T.s - 1) * astride;
  *pb = (i == 0) ? cscale(K, T.b[i]) : cfma(make_float2(T.b[i], 0.f), K, *pb);
  return next;
}

// Run-time dispatch onto etd_stage_c / rk_stage. `astride` is the distance between the
// Runge-Kutta aux arrays (acc is the first of them); the exponential schemes use acc and q.
__device__ __forceinline__ float2 etd_stage(int integ, int s, float2 nv, float2* __restrict__ u,
                                            float2* __restrict__ acc, float2* __restrict__ q,
                                            const float2* __restrict__ tab, int64_t ts, int64_t astride = 0) {
  if (is_rk(integ)) return rk_stage(integ, s, nv, u, acc, astride, tab, ts);
  if (integ == FSM_APPLY) {  // the right-hand side L u + N(u) replaces the state
    const float2 r = cfma(tab[0], *u, nv);
    *u = r;
    return r;
  }
  switch (integ) {
    case FSM_SETDRK4:
      switch (s) {
        case 0: return etd_stage_c<FSM_SETDRK4, 0>(nv, u, acc, q, tab, ts);
        case 1: return etd_stage_c<FSM_SETDRK4, 1>(nv, u, acc, q, tab, ts);
        case 2: return etd_stage_c<FSM_SETDRK4, 2>(nv, u, acc, q, tab, ts);
        default: return etd_stage_c<FSM_SETDRK4, 3>(nv, u, acc, q, tab, ts);
      }
    case FSM_SETDRK3:
      switch (s) {
        case 0: return etd_stage_c<FSM_SETDRK3, 0>(nv, u, acc, q, tab, ts);
        case 1: return etd_stage_c<FSM_SETDRK3, 1>(nv, u, acc, q, tab, ts);
        default: return etd_stage_c<FSM_SETDRK3, 2>(nv, u, acc, q, tab, ts);
      }
    case FSM_SETDRK2:
    case FSM_ETDRK2:
      return s == 0 ? etd_stage_c<FSM_SETDRK2, 0>(nv, u, acc, q, tab, ts)
                    : etd_stage_c<FSM_SETDRK2, 1>(nv, u, acc, q, tab, ts);
    default:
      return etd_stage_c<FSM_SETDRK1, 0>(nv, u, acc, q, tab, ts);
  }
}

}  // namespace fsm

// The plan: constant device tables of one (program, mesh, dt).
struct FsmPlan {
  int device = 0;
  int ndim = 0;
  int n[3] = {1, 1, 1};
  int h = 0;         // n[ndim-1]/2 + 1
  int64_t S = 0;     // spectral points per field
  int64_t R = 0;     // real points per field
  int C = 1;
  int nl = FSM_NL_NONE;
  int flags = 0;
  int integ = FSM_SETDRK4;
  int nstages = 4;
  int ntab = 0;
  float nl_coef = 0.f;
  int lin_batch = 1, lin_ch = 1;
  int src_batch = 0;
  int koff[3] = {0, 0, 0};
  float* kvec = nullptr;     // 2 pi f per axis, concatenated (axis i at koff[i])
  uint8_t* keep = nullptr;   // dealias keep flags per axis, concatenated
  float2* tw = nullptr;      // W_4096^k, k < 4096
  float2* tab = nullptr;     // [ntab][lin_batch][lin_ch][S]
  int64_t tstride = 0;       // lin_batch * lin_ch * S
  float2* source = nullptr;  // [src_batch][C][S] or null
  double2* lin = nullptr;    // FP64 linear symbol [lin_src_batch][lin_ch][S] kept for per-entry dt changes
  int lin_src_batch = 1;
  int lin_present = 0;
  double dt = 0.0;
  int n_points = 16;
  double radius = 1.0;
  // fused-path array counts per sample (2D / 3D)
  int n_mid = 0, n_prod = 0, n_aux = 0, n_mid2 = 0;
  int path = 0;  // 1: line kernel (1D), 2: plane passes (2D), 3: pointwise, 4: volume passes (3D)
  // per column tile of the register axis-0 pass (W adjacent inner columns): 1 where every column
  // is dealiased, so that the next-stage fields built there are zero (null: no such pass)
  uint8_t* tile_zero = nullptr;
  // 2D plane passes: the leading last-axis columns of the stage fields that the row pass reads.
  // Below h when the dealias mask keeps the prefix of n1/3 + 1 columns (the 2/3 rule) and the
  // register passes run both axes: the fields beyond it are zero, so the column pass does not
  // store them and the row pass does not load them.
  int hk = 0;
  // Row pitch (complex entries) and field stride of the stage fields and products (workspace
  // arrays exchanged between the passes). 2D register passes: n1/2 + 1 rounded up to even, so that
  // rows start on 16-byte boundaries (tensor-map strides); otherwise the unpadded S / n0 and S.
  int64_t wp = 0, ms = 0;
};

namespace fsm {
int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);
}  // namespace fsm
