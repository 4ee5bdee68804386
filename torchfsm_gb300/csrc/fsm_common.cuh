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
__host__ __device__ inline int scheme_stages(int integ) {
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
__host__ __device__ inline int scheme_tables(int integ) {
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
  switch (integ) {
    case FSM_SETDRK4:
    case FSM_SETDRK3: return 2;
    case FSM_SETDRK2:
    case FSM_ETDRK2: return 1;
    default: return 0;
  }
}

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
      const float2 E = tab[0], E2 = tab[ts], c1 = tab[2 * ts], c4 = tab[3 * ts];
      const float2 a1 = cfma(c1, nv, cmul(E2, uu));
      *acc = cfma(c4, nv, cmul(E, uu));
      *q = cfma(make_float2(-c1.x, -c1.y), nv, cmul(E2, a1));
      return a1;
    } else if (S == 1) {
      const float2 uu = *u;
      const float2 E2 = tab[ts], c1 = tab[2 * ts], c5 = tab[4 * ts];
      *acc = cfma(cscale(c5, 2.f), nv, *acc);
      return cfma(c1, nv, cmul(E2, uu));
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
      const float2 E = tab[0], E2 = tab[ts], c1 = tab[2 * ts], c2 = tab[3 * ts], c3 = tab[4 * ts];
      const float2 Eu = cmul(E, uu);
      *acc = cfma(c3, nv, Eu);
      *q = cfma(make_float2(-c2.x, -c2.y), nv, Eu);
      return cfma(c1, nv, cmul(E2, uu));
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
      const float2 E = tab[0], c1 = tab[ts], c2 = tab[2 * ts];
      const float2 a1 = cfma(c1, nv, cmul(E, uu));
      *acc = cfma(make_float2(-c2.x, -c2.y), nv, a1);
      return a1;
    } else {
      const float2 c2 = tab[2 * ts];
      const float2 un = cfma(c2, nv, *acc);
      *u = un;
      return un;
    }
  } else {  // (S)ETDRK1, ETDRK0
    const float2 E = tab[0], c1 = tab[ts];
    const float2 un = cfma(c1, nv, cmul(E, *u));
    *u = un;
    return un;
  }
}

// Run-time dispatch onto etd_stage_c.
__device__ __forceinline__ float2 etd_stage(int integ, int s, float2 nv, float2* __restrict__ u,
                                            float2* __restrict__ acc, float2* __restrict__ q,
                                            const float2* __restrict__ tab, int64_t ts) {
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
};

namespace fsm {
int set_error(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);
}  // namespace fsm
