// Shared-memory Stockham FFTs for the spectral ETD kernels (sm_103a).
//
// One transform of N = 2^m complex points is done by a group of G threads
// (one warp, or a whole block) on a buffer in shared memory. Each pass takes
// R inputs at stride N/R, applies the twiddles W_{R p}^{j k}, does an R-point
// DFT in registers and stores the outputs at the auto-sorted (Stockham)
// positions, so the result comes out in natural order with no bit reversal.
// Passes are chosen at compile time (radix 8 first, then 4/2), every pass is
// in place: all loads of the pass, a barrier, all stores, a barrier.
//
// Sign convention: forward = exp(-2 pi i k n / N), inverse = exp(+...), both
// unnormalised (the caller folds the 1/N of torch's "backward" norm into the
// spectral arithmetic). Twiddles come from a table W_N^k = exp(-2 pi i k/N),
// k < N, computed in FP64 on the host and rounded to FP32.
#pragma once

#include <cuda_runtime.h>

namespace fsm {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// i * a
__device__ __forceinline__ float2 cmuli(float2 a) { return make_float2(-a.y, a.x); }
// -i * a
__device__ __forceinline__ float2 cmulmi(float2 a) { return make_float2(a.y, -a.x); }
// a + s * b (complex a, b; real s)
__device__ __forceinline__ float2 caxpy(float2 a, float s, float2 b) {
  return make_float2(fmaf(s, b.x, a.x), fmaf(s, b.y, a.y));
}
// a + c * b (complex)
__device__ __forceinline__ float2 cfma(float2 c, float2 b, float2 a) {
  return make_float2(fmaf(c.x, b.x, fmaf(-c.y, b.y, a.x)), fmaf(c.x, b.y, fmaf(c.y, b.x, a.y)));
}

template <bool INV>
__device__ __forceinline__ void dft2(float2* v) {
  float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2* v) {
  float2 t0 = cadd(v[0], v[2]);
  float2 t1 = csub(v[0], v[2]);
  float2 t2 = cadd(v[1], v[3]);
  float2 d = csub(v[1], v[3]);
  float2 t3 = INV ? cmuli(d) : cmulmi(d);  // W4^1 = -i (forward), +i (inverse)
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2* v) {
  const float h = 0.70710678118654752440f;
  float2 a[4], b[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    a[j] = cadd(v[j], v[j + 4]);
    b[j] = csub(v[j], v[j + 4]);
  }
  // b_j *= W8^j
  if (!INV) {
    b[1] = make_float2(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));   // (1 - i)/sqrt2
    b[2] = cmulmi(b[2]);                                                   // -i
    b[3] = make_float2(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));   // (-1 - i)/sqrt2
  } else {
    b[1] = make_float2(h * (b[1].x - b[1].y), h * (b[1].y + b[1].x));   // (1 + i)/sqrt2
    b[2] = cmuli(b[2]);                                                    // +i
    b[3] = make_float2(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y));   // (-1 + i)/sqrt2
  }
  dft4<INV>(a);
  dft4<INV>(b);
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    v[2 * m] = a[m];
    v[2 * m + 1] = b[m];
  }
}

template <int R, bool INV>
__device__ __forceinline__ void dftR(float2* v) {
  if constexpr (R == 8) dft8<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v);
  else dft2<INV>(v);
}

template <bool BLOCK>
__device__ __forceinline__ void group_sync() {
  if constexpr (BLOCK) __syncthreads();
  else __syncwarp();
}

// Radix of the next pass when REM points remain to be combined.
template <int REM>
struct NextRadix {
  static constexpr int value = (REM == 16) ? 4 : (REM >= 8 ? 8 : (REM >= 4 ? 4 : 2));
};

// One Stockham pass with span P (product of the radices already applied).
template <int N, int R, int P, int G, bool BLOCK, bool INV>
__device__ __forceinline__ void stockham_pass(float2* x, const float2* __restrict__ tw, int tid) {
  constexpr int NB = N / R;
  constexpr int PER = (NB + G - 1) / G;
  constexpr int TSTRIDE = N / (R * P);
  float2 v[PER][R];
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int i = tid + b * G;
    if ((NB % G == 0) || i < NB) {
      const int k = i & (P - 1);
#pragma unroll
      for (int j = 0; j < R; ++j) v[b][j] = x[i + j * NB];
      if constexpr (P > 1) {
#pragma unroll
        for (int j = 1; j < R; ++j) {
          float2 w = tw[j * k * TSTRIDE];
          if (INV) w.y = -w.y;
          v[b][j] = cmul(v[b][j], w);
        }
      }
      dftR<R, INV>(v[b]);
    }
  }
  group_sync<BLOCK>();
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int i = tid + b * G;
    if ((NB % G == 0) || i < NB) {
      const int k = i & (P - 1);
      const int base = (i - k) * R + k;
#pragma unroll
      for (int j = 0; j < R; ++j) x[base + j * P] = v[b][j];
    }
  }
  group_sync<BLOCK>();
}

template <int N, int P, int G, bool BLOCK, bool INV>
__device__ __forceinline__ void fft_passes(float2* x, const float2* __restrict__ tw, int tid) {
  if constexpr (P < N) {
    constexpr int R = NextRadix<N / P>::value;
    stockham_pass<N, R, P, G, BLOCK, INV>(x, tw, tid);
    fft_passes<N, P * R, G, BLOCK, INV>(x, tw, tid);
  }
}

// In-place N-point FFT of x (shared memory) by G threads (tid in [0, G)).
// The caller must have synchronised the group before the call (x complete);
// on return x is complete and visible to the whole group.
template <int N, int G, bool BLOCK, bool INV>
__device__ __forceinline__ void fft(float2* x, const float2* __restrict__ tw, int tid) {
  fft_passes<N, 1, G, BLOCK, INV>(x, tw, tid);
}

// Copy the N-entry twiddle table W_N^k from the master table of size NMAX.
__device__ __forceinline__ void load_twiddles(float2* dst, const float2* __restrict__ master, int nmax, int n,
                                              int tid, int nthreads) {
  const int stride = nmax / n;
  for (int k = tid; k < n; k += nthreads) dst[k] = master[k * stride];
}

}  // namespace fsm
