// Register-resident FFTs: an N-point transform (N = T * E, E = T or 2T) by a
// group of T consecutive lanes of one warp. Lane t holds element t + T*j in
// register j (j < E) on entry and on exit, so transforms can be chained
// (inverse -> pointwise product -> forward) without leaving registers.
//
//   X[m + E k] = sum_t W_T^{t k} * ( W_N^{t m} * sum_j x[t + T j] W_E^{j m} )
//
// Pass 1: radix-E DFT over j in registers, then the twiddles W_N^{t m} from a
// table laid out [m][t] (consecutive lanes read consecutive words). One
// transpose through shared memory (pitch T+1, conflict-free for 8-byte
// words), then pass 2: E/T radix-T DFTs over t per lane, which leave output
// K = t + T j' in register j'.
#pragma once

#include "fsm_fft.cuh"

namespace fsm {

template <int N>
struct RegShape;
template <>
struct RegShape<256> {
  static constexpr int T = 16, E = 16;
};
template <>
struct RegShape<128> {
  static constexpr int T = 8, E = 16;
};
template <>
struct RegShape<64> {
  static constexpr int T = 8, E = 8;
};
template <>
struct RegShape<32> {
  static constexpr int T = 4, E = 8;
};
template <>
struct RegShape<16> {
  static constexpr int T = 4, E = 4;
};

template <int N>
struct HasRegShape {
  static constexpr bool value = (N == 16 || N == 32 || N == 64 || N == 128 || N == 256);
};

// 16-point DFT as 4 x 4 (inputs v[r + 4 l], outputs X[q + 4 s]).
template <bool INV>
__device__ __forceinline__ void dft16(float2* v) {
  const float c1 = 0.92387953251128675613f;  // cos(pi/8)
  const float s1 = 0.38268343236508977173f;  // sin(pi/8)
  const float h = 0.70710678118654752440f;
  float2 a[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    float2 w[4] = {v[r], v[r + 4], v[r + 8], v[r + 12]};
    dft4<INV>(w);
#pragma unroll
    for (int q = 0; q < 4; ++q) a[r][q] = w[q];
  }
  // a[r][q] *= W16^{r q}   (forward W16 = exp(-2 pi i/16); inverse: conjugate)
  const float sg = INV ? -1.f : 1.f;
  auto tw = [&](float2 x, float cr, float ci) {  // x * (cr - i*sg*ci)
    return make_float2(x.x * cr + sg * x.y * ci, x.y * cr - sg * x.x * ci);
  };
  a[1][1] = tw(a[1][1], c1, s1);    // W^1
  a[1][2] = tw(a[1][2], h, h);      // W^2
  a[1][3] = tw(a[1][3], s1, c1);    // W^3
  a[2][1] = tw(a[2][1], h, h);      // W^2
  a[2][2] = INV ? cmuli(a[2][2]) : cmulmi(a[2][2]);  // W^4
  a[2][3] = tw(a[2][3], -h, h);     // W^6
  a[3][1] = tw(a[3][1], s1, c1);    // W^3
  a[3][2] = tw(a[3][2], -h, h);     // W^6
  a[3][3] = tw(a[3][3], -c1, -s1);  // W^9
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float2 w[4] = {a[0][q], a[1][q], a[2][q], a[3][q]};
    dft4<INV>(w);
#pragma unroll
    for (int s = 0; s < 4; ++s) v[q + 4 * s] = w[s];
  }
}

template <int R, bool INV>
__device__ __forceinline__ void dft_reg(float2* v) {
  if constexpr (R == 16) dft16<INV>(v);
  else if constexpr (R == 8) dft8<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v);
  else dft2<INV>(v);
}

// Twiddle table twt[m * T + t] = W_N^{t m} (m < E, t < T), from the master table W_4096^k.
template <int N>
__device__ __forceinline__ void load_reg_twiddles(float2* twt, const float2* __restrict__ master, int tid,
                                                  int nthreads) {
  constexpr int T = RegShape<N>::T, E = RegShape<N>::E;
  for (int i = tid; i < T * E; i += nthreads) {
    const int m = i / T, t = i % T;
    twt[i] = master[(t * m) * (kTwiddleMax / N)];
  }
}

// Scratch a group needs: E rows of T+1 words.
template <int N>
constexpr int reg_scratch() {
  return RegShape<N>::E * (RegShape<N>::T + 1);
}

// In-register FFT of the group's N points (see file comment). `scratch` holds
// reg_scratch<N>() float2 private to the group; t is the lane's index in the group.
// Every lane of the warp must call this together (warp-synchronous).
template <int N, bool INV>
__device__ __forceinline__ void reg_fft(float2 (&v)[RegShape<N>::E], float2* __restrict__ scratch,
                                        const float2* __restrict__ twt, int t) {
  constexpr int T = RegShape<N>::T, E = RegShape<N>::E;
  constexpr int PER = E / T;
  dft_reg<E, INV>(v);
#pragma unroll
  for (int m = 1; m < E; ++m) {
    float2 w = twt[m * T + t];
    if (INV) w.y = -w.y;
    v[m] = cmul(v[m], w);
  }
#pragma unroll
  for (int m = 0; m < E; ++m) scratch[m * (T + 1) + t] = v[m];
  __syncwarp();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int m = t + p * T;
    float2 w[T];
#pragma unroll
    for (int tt = 0; tt < T; ++tt) w[tt] = scratch[m * (T + 1) + tt];
    dft_reg<T, INV>(w);
#pragma unroll
    for (int k = 0; k < T; ++k) v[p + PER * k] = w[k];
  }
  __syncwarp();
}

}  // namespace fsm
