// Device bodies of the register-FFT 2D column and row passes (64..256 points per axis; the
// column pass is also the 3D x pass), shared by the kernels of one plan (fsm_plane_reg.cu) and
// the kernels that advance several plans in one launch (fsm_plane_multi.cu). Same arithmetic
// and layout as fsm_plane.cu; the transforms run in registers (fsm_regfft.cuh), so each 1D
// transform touches shared memory once (the pass-1/pass-2 transpose).
//
// Row pass: a group of T lanes owns a pair of rows. It loads the mid fields
// straight from global memory into the transform layout (the Hermitian
// extension k > NY/2 comes from the mirrored entry), runs the inverse
// transforms, forms the physical product in registers, runs the forward
// transform of the two rows' products packed as one complex row and splits
// the half spectra with one shuffle per output register.
//
// Column pass: a CTA owns W = 256/T adjacent ky columns of one sample. The
// products are staged into a padded column-major tile (coalesced loads), each
// group transforms one column, the stage update runs with a coalesced point
// mapping, and each next-stage field is transformed per column and staged
// through a second tile for coalesced stores.
#pragma once

#include "fsm_internal.cuh"
#include "fsm_regfft.cuh"

namespace fsm {

template <int KIND, int DIM>
struct RegKind {
  // channels of the state
  static constexpr int C = (KIND == FSM_NL_CONVECTION || KIND == FSM_NL_LERAY) ? DIM : 1;
  // channels whose stage update runs together (the Leray projection mixes all of them)
  static constexpr int CG = (KIND == FSM_NL_LERAY) ? C : 1;
  // mid fields written per channel group
  static constexpr int NMG = (KIND == FSM_NL_VORTICITY) ? 4 : 2 * CG;
};

template <int NX>
struct ColCfg {
  using RS = RegShape<NX>;
  static constexpr int T = RS::T;
  static constexpr int E = RS::E;
  static constexpr int W = 256 / T;
  static constexpr int NEED = (NX > E * (T + 1)) ? NX : E * (T + 1);
  static constexpr int P = NEED | 1;  // odd pitch: a row across W columns hits W distinct banks
};

// Wavenumbers and dealias factor of the point (row, inner index j). 2D: j is
// the last-axis index; 3D: j = jm * H + jl (middle, last axis).
template <int DIM>
struct PointK {
  float kx, ky, kz;  // ky: second axis, kz: third axis (3D)
  float mask;
};

template <int DIM>
__device__ __forceinline__ PointK<DIM> point_k(const StepArgs& a, int row, int64_t j) {
  PointK<DIM> p;
  p.kx = a.kx[row];
  if (DIM == 2) {
    p.ky = a.ky[j];
    p.kz = 0.f;
    p.mask = (float)(a.keepx[row] & a.keepy[j]);
  } else {
    const int jm = (int)(j / a.H), jl = (int)(j % a.H);
    p.ky = a.km[jm];
    p.kz = a.ky[jl];
    p.mask = (float)(a.keepx[row] & a.keepm[jm] & a.keepy[jl]);
  }
  p.mask *= a.scale;
  return p;
}

// Leray projection of the convection term at one point: N_c = i k_c p - conv_c,
// p = (sum_i i k_i conv_i) / lap (1 where lap == 0), operator/dedicated/_navier_stokes.py:246-254.
// The state stores only the last axis' first half, so at points whose mirror -k
// is not stored (last-axis index strictly inside) the kernel must advance the
// Hermitian part (N(k) + conj N(-k)) / 2, which is what ifftn(...).real of the
// reference's state follows. Where a non-last axis sits at its Nyquist index its
// wavenumber does not change sign under k -> -k, and that Hermitian part is the
// projection restricted to axes with the same Nyquist status as c.
template <int DIM, int CG>
__device__ __forceinline__ void nv_leray(float2 (&nv)[CG], const PointK<DIM>& pk, int row, int64_t j,
                                         const StepArgs& a, int nx) {
  const float kk[3] = {pk.kx, pk.ky, pk.kz};
  float sgn[3] = {1.f, 1.f, 1.f};
  int jl, jm = 0;
  if (DIM == 2) {
    jl = (int)j;
  } else {
    jm = (int)(j / a.H);
    jl = (int)(j % a.H);
  }
  const bool inside = jl > 0 && jl < a.H - 1;
  if (inside) {
    if (row == nx / 2) sgn[0] = -1.f;
    if (DIM == 3 && jm == a.nm / 2) sgn[1] = -1.f;
  }
  float lap = 0.f;
#pragma unroll
  for (int f = 0; f < CG; ++f) lap -= kk[f] * kk[f];
  const float il = (lap == 0.f) ? 1.f : 1.f / lap;
  float2 out[CG];
#pragma unroll
  for (int c = 0; c < CG; ++c) {
    float2 div = make_float2(0.f, 0.f);
#pragma unroll
    for (int f = 0; f < CG; ++f)
      if (sgn[f] == sgn[c]) div = cadd(div, cscale(cmuli(nv[f]), kk[f]));
    out[c] = csub(cscale(cmuli(cscale(div, il)), kk[c]), nv[c]);
  }
#pragma unroll
  for (int c = 0; c < CG; ++c) nv[c] = out[c];
}

// One SETDRK4 stage at one point from its operands already in registers (the recurrences of
// etd_stage_c): ua is u at stages 0 and 1, acc at stages 2 and 3; ub is acc at stage 1, q at stage
// 2. The running sums the stage writes are returned in acc / q, the new state (stage 3) in the
// return value, which is otherwise the next stage's input.
template <int S>
__device__ __forceinline__ float2 setdrk4_pre(float2 nv, float2 ua, float2 ub, const float2* __restrict__ tab,
                                              int64_t ts, float2& acc, float2& q) {
  if (S == 0) {
    const float2 Em1 = tab[0], E2m1 = tab[ts], c1 = tab[2 * ts], c4 = tab[3 * ts];
    const float2 a1 = cfma(c1, nv, cexpmul(E2m1, ua));
    acc = cfma(c4, nv, cexpmul(Em1, ua));
    q = cfma(make_float2(-c1.x, -c1.y), nv, cexpmul(E2m1, a1));
    return a1;
  } else if (S == 1) {
    const float2 E2m1 = tab[ts], c1 = tab[2 * ts], c5 = tab[4 * ts];
    acc = cfma(cscale(c5, 2.f), nv, ub);
    return cfma(c1, nv, cexpmul(E2m1, ua));
  } else if (S == 2) {
    const float2 c1 = tab[2 * ts], c5 = tab[4 * ts];
    acc = cfma(cscale(c5, 2.f), nv, ua);
    return cfma(cscale(c1, 2.f), nv, ub);
  } else {
    return cfma(tab[5 * ts], nv, ua);
  }
}

// Phase 2 of k_axis0_r for SETDRK4 stages of one-channel groups: the state operands the thread's
// points need from HBM (u at stages 0 and 1, acc at 1, 2 and 3, q at 2) are loaded first for a
// group of points, in one round, then those points are updated with their table loads (which hit
// L2). Loading them four points at a time left four rounds of HBM latency in each CTA's critical
// path (on 2D vorticity 256^2 x 64 the column pass went from 55 to 43 us per launch).
template <int NX, int KIND, int DIM, int STG>
__device__ __forceinline__ void axis0_update_hoisted(const StepArgs& a, float2* __restrict__ tileA, int b, int64_t c0,
                                                     int cg, bool last) {
  using Cfg = ColCfg<NX>;
  using K = RegKind<KIND, DIM>;
  constexpr int W = Cfg::W, P = Cfg::P, C = K::C;
  constexpr int PPT = NX * W / 256, RSTEP = 256 / W;
  const int64_t S = a.S;
  const int64_t inner = S / NX;
  const int col = threadIdx.x % W, row0 = threadIdx.x / W;
  const int64_t j = c0 + col;
  if (j >= inner) return;
  const int c = cg;
  float2* __restrict__ up = a.state + ((int64_t)b * C + c) * S + j;
  float2* __restrict__ accp = a.aux + ((int64_t)b * a.n_aux * C + c) * S + j;
  float2* __restrict__ qp = a.aux + ((int64_t)b * a.n_aux * C + C + c) * S + j;
  const float2* __restrict__ tab = a.tab + (tab_batch(a, b) * a.lin_ch + (a.lin_ch > 1 ? c : 0)) * S + j;
  const float2* __restrict__ srcp =
      a.src ? a.src + ((int64_t)(a.src_batch > 1 ? b : 0) * C + c) * S + j : nullptr;
  const float2* __restrict__ o1p = (STG <= 1) ? up : accp;
  const float2* __restrict__ o2p = (STG == 1) ? accp : qp;
  // operands of HALF points at a time, one HBM round per group: eight points (vorticity) and four
  // (convection, whose kernel holds more) keep the kernels inside two CTAs' registers per SM
  constexpr int HMAX = (KIND == FSM_NL_CONVECTION) ? 4 : 8;
  constexpr int HALF = PPT > HMAX ? HMAX : PPT;
#pragma unroll 1
  for (int h0 = 0; h0 < PPT; h0 += HALF) {
  float2 o1[HALF], o2[HALF];
#pragma unroll
  for (int ih = 0; ih < HALF; ++ih) {
    const int64_t r = (int64_t)(row0 + RSTEP * (h0 + ih)) * inner;
    o1[ih] = o1p[r];
    if (STG == 1 || STG == 2) o2[ih] = o2p[r];
  }
#pragma unroll
  for (int ih = 0; ih < HALF; ++ih) {
    const int it = h0 + ih;
    // the table loads of four points at a time: without this fence the compiler issues those of
    // every point at once, beside the operands, and runs out of registers
    
    const int row = row0 + RSTEP * it;
    const int64_t r = (int64_t)row * inner;
    const PointK<DIM> pk = point_k<DIM>(a, row, j);
    float2 nv = tileA[col * P + row];
    if (KIND == FSM_NL_KS && (a.flags & FSM_FLAG_REMOVE_MEAN) && row == 0 && j == 0) nv = csub(nv, a.dc[0]);
    nv = cscale(nv, a.coef);
    if (srcp) nv = cadd(nv, srcp[r]);
    float2 acc, q;
    const float2 st = setdrk4_pre<STG>(nv, o1[ih], (STG == 1 || STG == 2) ? o2[ih] : o1[ih], tab + r, a.ts, acc, q);
    if (STG <= 2) accp[r] = acc;
    if (STG == 0) qp[r] = q;
    if (STG == 3) {
      up[r] = st;
      if (a.slot >= 0 && last) a.traj[(((int64_t)b * a.n_frames + a.slot) * C + c) * S + r + j] = st;
    }
    tileA[col * P + row] = cscale(st, pk.mask);
  }
  }
}

// Phase 2 of k_axis0_r: the stage update at every point of the tile, in a coalesced point
// mapping, leaving the masked next-stage field in tileA. INTEG/STG name the scheme and stage
// at compile time (so that the loads of several points are issued together); -1 dispatches
// at run time.
template <int NX, int KIND, int DIM, int INTEG, int STG>
__device__ __forceinline__ void axis0_update(const StepArgs& a, float2* __restrict__ tileA, int b, int64_t c0, int cg,
                                             bool last) {
  using Cfg = ColCfg<NX>;
  using K = RegKind<KIND, DIM>;
  constexpr int W = Cfg::W, P = Cfg::P, C = K::C, CG = K::CG;
  const int64_t S = a.S;
  const int64_t inner = S / NX;
  const bool update = STG >= 0 || a.stage >= 0;  // false: the priming launch (mask and emit only)
  // restrict-qualified views so that loads of later points may be issued ahead of the stores of earlier ones
  float2* __restrict__ state = a.state;
  float2* __restrict__ aux = a.aux;
  float2* __restrict__ traj = a.traj;
  const float2* __restrict__ tab = a.tab;
  const float2* __restrict__ srcp = a.src;
  constexpr int PPT = NX * W / 256;  // points per thread
#pragma unroll 4
  for (int it = 0; it < PPT; ++it) {
    const int idx = threadIdx.x + it * 256;
    const int row = idx / W, col = idx % W;
    const int64_t j = c0 + col;
    if (j >= inner) continue;
    const int64_t sidx = (int64_t)row * inner + j;
    const PointK<DIM> pk = point_k<DIM>(a, row, j);
    float2 nv[CG];
    if (update) {
#pragma unroll
      for (int f = 0; f < CG; ++f) nv[f] = tileA[(f * W + col) * P + row];
      if (KIND == FSM_NL_LERAY) nv_leray<DIM, CG>(nv, pk, row, j, a, NX);
      if (KIND == FSM_NL_KS && (a.flags & FSM_FLAG_REMOVE_MEAN) && row == 0 && j == 0) nv[0] = csub(nv[0], a.dc[0]);
#pragma unroll
      for (int f = 0; f < CG; ++f) {
        const int c = cg * CG + f;
        nv[f] = cscale(nv[f], a.coef);
        if (srcp) nv[f] = cadd(nv[f], srcp[((int64_t)(a.src_batch > 1 ? b : 0) * C + c) * S + sidx]);
      }
    }
#pragma unroll
    for (int f = 0; f < CG; ++f) {
      const int c = cg * CG + f;
      float2* up = state + ((int64_t)b * C + c) * S + sidx;
      float2 st;
      if (!update) {
        st = *up;
      } else {
        float2* accp = aux + ((int64_t)b * a.n_aux * C + c) * S + sidx;
        float2* qp = aux + ((int64_t)b * a.n_aux * C + (a.n_aux > 1 ? C : 0) + c) * S + sidx;
        const int64_t toff = (tab_batch(a, b) * a.lin_ch + (a.lin_ch > 1 ? c : 0)) * S + sidx;
        if (STG >= 0)
          st = etd_stage_c<INTEG, STG>(nv[f], up, accp, qp, tab + toff, a.ts);
        else
          st = etd_stage(a.integ, a.stage, nv[f], up, accp, qp, tab + toff, a.ts, (int64_t)C * S);
      }
      if (a.slot >= 0 && (!update || last)) traj[(((int64_t)b * a.n_frames + a.slot) * C + c) * S + sidx] = st;
      tileA[(f * W + col) * P + row] = cscale(st, pk.mask);
    }
  }
}

// Axis-0 pass (2D: the column pass; 3D: the x pass). A CTA owns W adjacent
// inner columns (contiguous in memory) of one sample, all NX rows:
//   1. forward transform along axis 0 of the products -> N (+ Leray projection, + source)
//   2. stage update at every point, recording when a step completes
//   3. next stage field (mask, 1/N, i kx, streamfunction) -> inverse transform -> mid fields
// Channels are processed in groups so that Convection needs one staging tile.
// FAST: a SETDRK4 stage launch of a vorticity or convection program (channel groups of one
// channel; the hoisted update, two CTAs per SM, k_axis0_r2); otherwise any scheme, the priming
// launch included (k_axis0_r).
template <int NX, int KIND, int DIM, bool FAST>
__device__ __forceinline__ void axis0_body(const StepArgs& a, int tile, int b) {
  using Cfg = ColCfg<NX>;
  using K = RegKind<KIND, DIM>;
  constexpr int T = Cfg::T, E = Cfg::E, W = Cfg::W, P = Cfg::P, C = K::C, CG = K::CG;
  extern __shared__ float2 smem[];
  float2* twt = smem;                 // NX
  float2* tileA = smem + NX;          // CG * W * P: products -> N -> next stage field
  float2* tileB = tileA + CG * W * P; // W * P: transpose scratch and output staging
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int64_t c0 = (int64_t)tile * W;
  const int64_t S = a.S;
  const int64_t inner = S / NX;
  load_reg_twiddles<NX>(twt, a.tw, threadIdx.x, 256);
  const bool last = a.stage == a.nstages - 1;
  float kxr[E];
#pragma unroll
  for (int j = 0; j < E; ++j) kxr[j] = a.kx[t + T * j];
  const int64_t gcol = c0 + g;
  const PointK<DIM> gk = point_k<DIM>(a, 0, gcol < inner ? gcol : inner - 1);

  for (int cg = 0; cg < C / CG; ++cg) {
    if (a.stage >= 0) {
      for (int f = 0; f < CG; ++f) {
        const float2* src = a.prod + ((int64_t)b * a.n_prod + cg * CG + f) * a.ms;
        // all loads of the tile are issued before the shared-memory stores
        float2 buf[NX * W / 256];
#pragma unroll
        for (int it = 0; it < NX * W / 256; ++it) {
          const int idx = threadIdx.x + it * 256;
          const int row = idx / W, col = idx % W;
          if (c0 + col < inner) buf[it] = src[(int64_t)row * a.wp + c0 + col];
        }
#pragma unroll
        for (int it = 0; it < NX * W / 256; ++it) {
          const int idx = threadIdx.x + it * 256;
          const int row = idx / W, col = idx % W;
          if (c0 + col < inner) tileA[(f * W + col) * P + row] = buf[it];
        }
      }
      __syncthreads();
      for (int f = 0; f < CG; ++f) {
        float2* colp = tileA + (f * W + g) * P;
        float2 v[E];
#pragma unroll
        for (int j = 0; j < E; ++j) v[j] = colp[t + T * j];
        reg_fft<NX, false>(v, tileB + g * P, twt, t);
#pragma unroll
        for (int j = 0; j < E; ++j) colp[t + T * j] = v[j];
      }
    }
    __syncthreads();

    if constexpr (FAST) {
      switch (a.stage) {
        case 0: axis0_update_hoisted<NX, KIND, DIM, 0>(a, tileA, b, c0, cg, last); break;
        case 1: axis0_update_hoisted<NX, KIND, DIM, 1>(a, tileA, b, c0, cg, last); break;
        case 2: axis0_update_hoisted<NX, KIND, DIM, 2>(a, tileA, b, c0, cg, last); break;
        default: axis0_update_hoisted<NX, KIND, DIM, 3>(a, tileA, b, c0, cg, last); break;
      }
    } else if (a.stage >= 0 && a.integ == FSM_SETDRK4) {
      switch (a.stage) {
        case 0: axis0_update<NX, KIND, DIM, FSM_SETDRK4, 0>(a, tileA, b, c0, cg, last); break;
        case 1: axis0_update<NX, KIND, DIM, FSM_SETDRK4, 1>(a, tileA, b, c0, cg, last); break;
        case 2: axis0_update<NX, KIND, DIM, FSM_SETDRK4, 2>(a, tileA, b, c0, cg, last); break;
        default: axis0_update<NX, KIND, DIM, FSM_SETDRK4, 3>(a, tileA, b, c0, cg, last); break;
      }
    } else {
      axis0_update<NX, KIND, DIM, -1, -1>(a, tileA, b, c0, cg, last);
    }
    if (!a.emit) continue;  // uniform: no further barriers in this group
    // 2D: columns from hk on are dealiased and the row pass does not read them: nothing to store
    if (c0 >= ((DIM == 2) ? (int64_t)a.hk : inner)) continue;  // uniform
    if (a.tile_zero && a.tile_zero[tile]) {
      // every column of this tile is dealiased: the next-stage fields are zero here, written
      // directly (coalesced rows of W columns) without the transforms
      constexpr int NMO = (KIND == FSM_NL_CONVECTION) ? 2 : K::NMG;  // fields of this channel group
      const int m0 = (KIND == FSM_NL_CONVECTION) ? cg * 2 : 0;
#pragma unroll 1
      for (int mf = 0; mf < NMO; ++mf) {
        float2* dst = a.mid + ((int64_t)b * a.n_mid + m0 + mf) * a.ms;
#pragma unroll
        for (int it = 0; it < NX * W / 256; ++it) {
          const int idx = threadIdx.x + it * 256;
          const int row = idx / W, cc = idx % W;
          if (c0 + cc < inner) dst[(int64_t)row * a.wp + c0 + cc] = make_float2(0.f, 0.f);
        }
      }
      continue;  // uniform across the CTA
    }
    __syncthreads();

    // Next-stage fields: each group transforms its own column into tileB, then the CTA
    // stores the tile with a coalesced mapping (rows of W adjacent columns).
    for (int mf = 0; mf < K::NMG; ++mf) {
      const int f = (KIND == FSM_NL_VORTICITY || KIND == FSM_NL_KS) ? 0 : (mf >> 1);
      const float2* colp = tileA + (f * W + g) * P;
      float2 v[E];
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const float2 d = colp[t + T * j];
        const float kxv = kxr[j];
        float2 x;
        if (KIND == FSM_NL_VORTICITY) {
          // 0: psi = -w/lap, 1: i kx psi, 2: w, 3: i kx w
          if (mf < 2) {
            const float lap = -(kxv * kxv + gk.ky * gk.ky);
            // fast division: within 2 ulp for |lap| below 2^126, far above any mesh's 2 (pi NX / L)^2
            const float il = (lap == 0.f) ? 1.f : __fdividef(1.f, lap);
            const float2 psi = cscale(d, -il);
            x = (mf == 0) ? psi : cscale(cmuli(psi), kxv);
          } else {
            x = (mf == 2) ? d : cscale(cmuli(d), kxv);
          }
        } else {
          // KS: 0: phi, 1: i kx phi; convection (per channel): u_c, i kx u_c
          x = (mf & 1) ? cscale(cmuli(d), kxv) : d;
        }
        v[j] = x;
      }
      float2* ob = tileB + g * P;
      reg_fft<NX, true>(v, ob, twt, t);
#pragma unroll
      for (int j = 0; j < E; ++j) ob[t + T * j] = v[j];
      __syncthreads();
      const int mout = (KIND == FSM_NL_CONVECTION) ? cg * 2 + mf : mf;
      float2* dst = a.mid + ((int64_t)b * a.n_mid + mout) * a.ms;
#pragma unroll
      for (int it = 0; it < NX * W / 256; ++it) {
        const int idx = threadIdx.x + it * 256;
        const int row = idx / W, cc = idx % W;
        if (c0 + cc < ((DIM == 2) ? (int64_t)a.hk : inner)) dst[(int64_t)row * a.wp + c0 + cc] = tileB[cc * P + row];
      }
      __syncthreads();
    }
  }
}

template <int NY>
struct RowCfgR {
  using RS = RegShape<NY>;
  static constexpr int T = RS::T;
  static constexpr int E = RS::E;
  static constexpr int SCR = reg_scratch<NY>();
};

__device__ __forceinline__ float2 herm_z(float2 A, float2 B, bool selfc, bool hi) {
  if (selfc) {
    A.y = 0.f;
    B.y = 0.f;
  }
  if (hi) {
    A.y = -A.y;
    B.y = -B.y;
  }
  return make_float2(A.x - B.y, A.y + B.x);  // A + i B
}

// Split the transform of p0 + i p1 (lane t holds K = t + T j in register j)
// into the half spectra of p0 and p1 and store k = 0..NY/2.
template <int NY>
__device__ __forceinline__ void split_store_r(const float2 (&zp)[RegShape<NY>::E], int t, int lane,
                                              float2* __restrict__ out0, float2* __restrict__ out1) {
  constexpr int T = RegShape<NY>::T, E = RegShape<NY>::E;
  constexpr int J = NY / (2 * T);
  const int partner_lane = (lane & ~(T - 1)) | ((T - t) & (T - 1));
#pragma unroll
  for (int j = 0; j <= J; ++j) {
    const float2 send = zp[E - 1 - j];
    float2 recv;
    recv.x = __shfl_sync(0xffffffffu, send.x, partner_lane);
    recv.y = __shfl_sync(0xffffffffu, send.y, partner_lane);
    const float2 partner = (t == 0) ? zp[(E - j) & (E - 1)] : recv;
    const int k = t + T * j;
    if (k <= NY / 2) {
      const float2 zm = cconj(partner);
      out0[k] = cscale(cadd(zp[j], zm), 0.5f);
      out1[k] = cscale(cmulmi(csub(zp[j], zm)), 0.5f);
    }
  }
}

// Whether every lane of register j (indices k = t + T j, folded to kk = min(k, NY - k)) lies at
// or beyond the kept prefix HK of the last axis: such registers hold zeros and load nothing.
template <int NY, int T, int HK>
__device__ __forceinline__ constexpr bool reg_dead(int j) {
  int mn = NY;
  for (int t = 0; t < T; ++t) {
    const int k = t + T * j;
    const int kk = k <= NY / 2 ? k : NY - k;
    mn = kk < mn ? kk : mn;
  }
  return mn >= HK;
}

// HK: the stage fields' stored columns (FsmPlan::hk), NY/2 + 1 when every column is stored.
template <int NY, int KIND, int HK>
__device__ __forceinline__ void plane_row_body(const StepArgs& a, int blk, int b) {
  using Cfg = RowCfgR<NY>;
  constexpr int T = Cfg::T, E = Cfg::E, SCR = Cfg::SCR;
  extern __shared__ float2 smem[];
  float2* twt = smem;
  const int lane = threadIdx.x & 31;
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int groups = blockDim.x / T;
  float2* scr = smem + NY + g * SCR;
  load_reg_twiddles<NY>(twt, a.tw, threadIdx.x, blockDim.x);
  __syncthreads();
  const int r0 = (blk * groups + g) * 2;
  const int64_t S = a.ms;  // field stride of the stage fields and products
  const int64_t WP = a.wp;  // their row pitch
  const float* ky = a.ky;
  const float2* mid = a.mid + (int64_t)b * a.n_mid * S;
  float2* prod = a.prod + (int64_t)b * a.n_prod * S;

  const float2 zero = make_float2(0.f, 0.f);
  if (KIND == FSM_NL_VORTICITY || KIND == FSM_NL_KS) {
    float p[2][E];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
      const int64_t roff = (int64_t)(r0 + rr) * WP;
      float2 Z1[E], Z2[E];
#pragma unroll
      for (int j = 0; j < E; ++j) {
        if (reg_dead<NY, T, HK>(j)) {
          Z1[j] = zero;
          Z2[j] = zero;
          continue;
        }
        const int k = t + T * j;
        const bool hi = k > NY / 2;
        const int kk = hi ? NY - k : k;
        const bool selfc = (kk == 0) || (kk == NY / 2);
        const bool live = HK > NY / 2 || kk < HK;
        const float kyv = ky[kk];
        if (KIND == FSM_NL_VORTICITY) {
          const float2 m0 = live ? mid[roff + kk] : zero, m1 = live ? mid[S + roff + kk] : zero;
          const float2 m2 = live ? mid[2 * S + roff + kk] : zero, m3 = live ? mid[3 * S + roff + kk] : zero;
          // u_x + i u_y with u_x <- i ky psi, u_y <- -(i kx psi); w_x + i w_y with w_x <- i kx w, w_y <- i ky w
          Z1[j] = herm_z(cscale(cmuli(m0), kyv), make_float2(-m1.x, -m1.y), selfc, hi);
          Z2[j] = herm_z(m3, cscale(cmuli(m2), kyv), selfc, hi);
        } else {
          const float2 m0 = live ? mid[roff + kk] : zero, m1 = live ? mid[S + roff + kk] : zero;
          Z1[j] = herm_z(m1, cscale(cmuli(m0), kyv), selfc, hi);  // phi_x + i phi_y
        }
      }
      reg_fft<NY, true>(Z1, scr, twt, t);
      if (KIND == FSM_NL_VORTICITY) {
        reg_fft<NY, true>(Z2, scr, twt, t);
#pragma unroll
        for (int j = 0; j < E; ++j) p[rr][j] = Z1[j].x * Z2[j].x + Z1[j].y * Z2[j].y;
      } else {
#pragma unroll
        for (int j = 0; j < E; ++j) p[rr][j] = 0.5f * (Z1[j].x * Z1[j].x + Z1[j].y * Z1[j].y);
      }
    }
    float2 zp[E];
#pragma unroll
    for (int j = 0; j < E; ++j) zp[j] = make_float2(p[0][j], p[1][j]);
    reg_fft<NY, false>(zp, scr, twt, t);
    split_store_r<NY>(zp, t, lane, prod + (int64_t)r0 * WP, prod + (int64_t)(r0 + 1) * WP);
  } else {
    // convection, C = 2: conv_c = u0 dx u_c + u1 dy u_c
#pragma unroll 1
    for (int rr = 0; rr < 2; ++rr) {
      const int64_t roff = (int64_t)(r0 + rr) * WP;
      float2 Z1[E], Z2[E];
#pragma unroll
      for (int j = 0; j < E; ++j) {
        if (reg_dead<NY, T, HK>(j)) {
          Z1[j] = zero;
          Z2[j] = zero;
          continue;
        }
        const int k = t + T * j;
        const bool hi = k > NY / 2;
        const int kk = hi ? NY - k : k;
        const bool selfc = (kk == 0) || (kk == NY / 2);
        const bool live = HK > NY / 2 || kk < HK;
        Z1[j] = live ? herm_z(mid[roff + kk], mid[2 * S + roff + kk], selfc, hi) : zero;       // u0 + i u1
        Z2[j] = live ? herm_z(mid[S + roff + kk], mid[3 * S + roff + kk], selfc, hi) : zero;   // dx u0 + i dx u1
      }
      reg_fft<NY, true>(Z1, scr, twt, t);
      reg_fft<NY, true>(Z2, scr, twt, t);
      float2 acc[E];
      float u1[E];
#pragma unroll
      for (int j = 0; j < E; ++j) {
        acc[j] = make_float2(Z1[j].x * Z2[j].x, Z1[j].x * Z2[j].y);
        u1[j] = Z1[j].y;
      }
#pragma unroll
      for (int j = 0; j < E; ++j) {
        if (reg_dead<NY, T, HK>(j)) {
          Z2[j] = zero;
          continue;
        }
        const int k = t + T * j;
        const bool hi = k > NY / 2;
        const int kk = hi ? NY - k : k;
        const bool selfc = (kk == 0) || (kk == NY / 2);
        const bool live = HK > NY / 2 || kk < HK;
        const float kyv = ky[kk];
        Z2[j] = live ? herm_z(cscale(cmuli(mid[roff + kk]), kyv), cscale(cmuli(mid[2 * S + roff + kk]), kyv), selfc, hi)
                     : zero;
      }
      reg_fft<NY, true>(Z2, scr, twt, t);  // dy u0 + i dy u1
#pragma unroll
      for (int j = 0; j < E; ++j) {
        acc[j].x += u1[j] * Z2[j].x;
        acc[j].y += u1[j] * Z2[j].y;
      }
      reg_fft<NY, false>(acc, scr, twt, t);
      split_store_r<NY>(acc, t, lane, prod + roff, prod + S + roff);
    }
  }
}

}  // namespace fsm
