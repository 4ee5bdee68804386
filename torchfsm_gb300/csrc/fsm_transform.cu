// Multi-dimensional real transforms built from two axis kernels:
//  * r2c / c2r along the contiguous last axis: two real rows travel as one
//    complex row z = a + i b (forward: split with Hermitian symmetry;
//    inverse: Z = A + i B over the Hermitian extension of each half spectrum);
//  * complex-to-complex along a strided outer axis on tiles of 8 adjacent
//    columns, staged through shared memory so that global accesses stay
//    coalesced and each warp transforms one column.
// These serve fsm_rfftn / fsm_irfftn (FourierMesh.fft / ifft(...).real,
// mesh.py:481-491) for the initial spectrum, the returned fields and the
// recorded trajectories.
#include "fsm_internal.cuh"

namespace fsm {

template <int N>
struct RowCfg {
  static constexpr int G = (N / 16 < 32) ? 32 : N / 16;
  static constexpr bool BLOCK = G > 32;
  static constexpr int GROUPS = BLOCK ? 1 : 8;
  static constexpr int THREADS = G * GROUPS;
  static constexpr size_t SMEM = (size_t)(GROUPS + 1) * N * sizeof(float2);
};

// rows: [rows][N] real -> [rows][N/2+1] complex (unnormalised forward)
template <int N>
__global__ void __launch_bounds__(RowCfg<N>::THREADS) k_r2c_last(const float* __restrict__ in, float2* __restrict__ out,
                                                                  int64_t rows, const float2* __restrict__ master) {
  using Cfg = RowCfg<N>;
  constexpr int H = N / 2 + 1;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  const int g = threadIdx.x / Cfg::G;
  const int t = threadIdx.x % Cfg::G;
  float2* z = smem + N + g * N;
  load_twiddles(tw, master, kTwiddleMax, N, threadIdx.x, Cfg::THREADS);
  const int64_t r0 = ((int64_t)blockIdx.x * Cfg::GROUPS + g) * 2;
  const bool has0 = r0 < rows, has1 = r0 + 1 < rows;
  for (int n = t; n < N; n += Cfg::G) {
    const float a = has0 ? in[r0 * N + n] : 0.f;
    const float b = has1 ? in[(r0 + 1) * N + n] : 0.f;
    z[n] = make_float2(a, b);
  }
  __syncthreads();
  fft<N, Cfg::G, Cfg::BLOCK, false>(z, tw, t);
  for (int k = t; k < H; k += Cfg::G) {
    const float2 zk = z[k];
    const float2 zm = cconj(z[(N - k) & (N - 1)]);
    if (has0) out[r0 * H + k] = cscale(cadd(zk, zm), 0.5f);
    if (has1) out[(r0 + 1) * H + k] = cscale(cmulmi(csub(zk, zm)), 0.5f);
  }
}

// rows: [rows][N/2+1] complex -> [rows][N] real, times `scale`
template <int N>
__global__ void __launch_bounds__(RowCfg<N>::THREADS) k_c2r_last(const float2* __restrict__ in, float* __restrict__ out,
                                                                  int64_t rows, float scale,
                                                                  const float2* __restrict__ master) {
  using Cfg = RowCfg<N>;
  constexpr int H = N / 2 + 1;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  const int g = threadIdx.x / Cfg::G;
  const int t = threadIdx.x % Cfg::G;
  float2* z = smem + N + g * N;
  load_twiddles(tw, master, kTwiddleMax, N, threadIdx.x, Cfg::THREADS);
  const int64_t r0 = ((int64_t)blockIdx.x * Cfg::GROUPS + g) * 2;
  const bool has0 = r0 < rows, has1 = r0 + 1 < rows;
  for (int k = t; k < H; k += Cfg::G) {
    float2 A = has0 ? in[r0 * H + k] : make_float2(0.f, 0.f);
    float2 B = has1 ? in[(r0 + 1) * H + k] : make_float2(0.f, 0.f);
    if (k == 0 || k == N / 2) {
      A.y = 0.f;
      B.y = 0.f;
    }
    z[k] = make_float2(A.x - B.y, A.y + B.x);  // A + i B
    if (k > 0 && k < N / 2) z[N - k] = make_float2(A.x + B.y, B.x - A.y);  // conj(A) + i conj(B)
  }
  __syncthreads();
  fft<N, Cfg::G, Cfg::BLOCK, true>(z, tw, t);
  for (int n = t; n < N; n += Cfg::G) {
    const float2 v = z[n];
    if (has0) out[r0 * N + n] = v.x * scale;
    if (has1) out[(r0 + 1) * N + n] = v.y * scale;
  }
}

// data: [outer][N][inner] complex; transform along the middle axis, in place.
constexpr int kColW = 8;
template <int N, bool INV>
__global__ void __launch_bounds__(256) k_c2c_strided(float2* __restrict__ data, int64_t inner,
                                                     const float2* __restrict__ master) {
  constexpr int P = N + 2;  // column pitch (bank-conflict-free transposed writes)
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* tile = smem + N;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t c0 = (int64_t)blockIdx.x * kColW;
  float2* base = data + (int64_t)blockIdx.y * N * inner;
  load_twiddles(tw, master, kTwiddleMax, N, threadIdx.x, 256);
  for (int idx = threadIdx.x; idx < N * kColW; idx += 256) {
    const int row = idx / kColW, col = idx % kColW;
    if (c0 + col < inner) tile[col * P + row] = base[(int64_t)row * inner + c0 + col];
  }
  __syncthreads();
  if (c0 + w < inner) fft<N, 32, false, INV>(tile + w * P, tw, lane);
  __syncthreads();
  for (int idx = threadIdx.x; idx < N * kColW; idx += 256) {
    const int row = idx / kColW, col = idx % kColW;
    if (c0 + col < inner) base[(int64_t)row * inner + c0 + col] = tile[col * P + row];
  }
}

template <int N>
static int launch_r2c(const float* in, float2* out, int64_t rows, const float2* tw, cudaStream_t st) {
  using Cfg = RowCfg<N>;
  int rc = prep_smem(k_r2c_last<N>, Cfg::SMEM);
  if (rc) return rc;
  const int64_t pairs = (rows + 1) / 2;
  const int64_t blocks = (pairs + Cfg::GROUPS - 1) / Cfg::GROUPS;
  k_r2c_last<N><<<(unsigned)blocks, Cfg::THREADS, Cfg::SMEM, st>>>(in, out, rows, tw);
  return cuda_check(cudaGetLastError(), "k_r2c_last");
}

template <int N>
static int launch_c2r(const float2* in, float* out, int64_t rows, float scale, const float2* tw, cudaStream_t st) {
  using Cfg = RowCfg<N>;
  int rc = prep_smem(k_c2r_last<N>, Cfg::SMEM);
  if (rc) return rc;
  const int64_t pairs = (rows + 1) / 2;
  const int64_t blocks = (pairs + Cfg::GROUPS - 1) / Cfg::GROUPS;
  k_c2r_last<N><<<(unsigned)blocks, Cfg::THREADS, Cfg::SMEM, st>>>(in, out, rows, scale, tw);
  return cuda_check(cudaGetLastError(), "k_c2r_last");
}

template <int N, bool INV>
static int launch_c2c(float2* data, int64_t outer, int64_t inner, const float2* tw, cudaStream_t st) {
  const size_t smem = (size_t)(N + kColW * (N + 2)) * sizeof(float2);
  int rc = prep_smem(k_c2c_strided<N, INV>, smem);
  if (rc) return rc;
  dim3 grid((unsigned)((inner + kColW - 1) / kColW), (unsigned)outer);
  k_c2c_strided<N, INV><<<grid, 256, smem, st>>>(data, inner, tw);
  return cuda_check(cudaGetLastError(), "k_c2c_strided");
}

int transform_r2c_last(int n, const float* in, float2* out, int64_t rows, const float2* tw, cudaStream_t st) {
  switch (n) {
    case 16: return launch_r2c<16>(in, out, rows, tw, st);
    case 32: return launch_r2c<32>(in, out, rows, tw, st);
    case 64: return launch_r2c<64>(in, out, rows, tw, st);
    case 128: return launch_r2c<128>(in, out, rows, tw, st);
    case 256: return launch_r2c<256>(in, out, rows, tw, st);
    case 512: return launch_r2c<512>(in, out, rows, tw, st);
    case 1024: return launch_r2c<1024>(in, out, rows, tw, st);
    case 2048: return launch_r2c<2048>(in, out, rows, tw, st);
    case 4096: return launch_r2c<4096>(in, out, rows, tw, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "r2c: unsupported length " + std::to_string(n));
}

int transform_c2r_last(int n, const float2* in, float* out, int64_t rows, float scale, const float2* tw,
                       cudaStream_t st) {
  switch (n) {
    case 16: return launch_c2r<16>(in, out, rows, scale, tw, st);
    case 32: return launch_c2r<32>(in, out, rows, scale, tw, st);
    case 64: return launch_c2r<64>(in, out, rows, scale, tw, st);
    case 128: return launch_c2r<128>(in, out, rows, scale, tw, st);
    case 256: return launch_c2r<256>(in, out, rows, scale, tw, st);
    case 512: return launch_c2r<512>(in, out, rows, scale, tw, st);
    case 1024: return launch_c2r<1024>(in, out, rows, scale, tw, st);
    case 2048: return launch_c2r<2048>(in, out, rows, scale, tw, st);
    case 4096: return launch_c2r<4096>(in, out, rows, scale, tw, st);
  }
  return set_error(FSM_ERR_UNSUPPORTED, "c2r: unsupported length " + std::to_string(n));
}

int transform_c2c_strided(int n, bool inverse, float2* data, int64_t outer, int64_t inner, const float2* tw,
                          cudaStream_t st) {
#define FSM_C2C_CASE(NN)                                                                        \
  case NN:                                                                                      \
    return inverse ? launch_c2c<NN, true>(data, outer, inner, tw, st)                           \
                   : launch_c2c<NN, false>(data, outer, inner, tw, st);
  switch (n) {
    FSM_C2C_CASE(16)
    FSM_C2C_CASE(32)
    FSM_C2C_CASE(64)
    FSM_C2C_CASE(128)
    FSM_C2C_CASE(256)
    FSM_C2C_CASE(512)
  }
#undef FSM_C2C_CASE
  return set_error(FSM_ERR_UNSUPPORTED, "c2c: unsupported length " + std::to_string(n));
}

// Per-field NaN/Inf flags: one block per field.
__global__ void k_nonfinite(const float2* __restrict__ f, int64_t S, int32_t* __restrict__ flags) {
  const float2* p = f + (int64_t)blockIdx.x * S;
  int bad = 0;
  for (int64_t i = threadIdx.x; i < S; i += blockDim.x) {
    const float2 v = p[i];
    bad |= !(isfinite(v.x) && isfinite(v.y));
  }
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) flags[blockIdx.x] = bad ? 1 : 0;
}

int launch_nonfinite(const float2* f, int64_t count, int64_t S, int32_t* flags, cudaStream_t st) {
  if (count <= 0) return FSM_OK;
  k_nonfinite<<<(unsigned)count, 256, 0, st>>>(f, S, flags);
  return cuda_check(cudaGetLastError(), "k_nonfinite");
}

}  // namespace fsm
