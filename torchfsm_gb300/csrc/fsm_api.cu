// C ABI of torchfsm_gb300: plans, the FP64 coefficient kernel, the
// integrate loop and the transforms. Declarations and the reference
// interfaces each entry point replaces are in include/torchfsm_gb300.h.
#include <math.h>
#include <string.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "fsm_internal.cuh"

namespace fsm {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FSM_OK;
  const int code = (e == cudaErrorMemoryAllocation) ? FSM_ERR_OOM : FSM_ERR_CUDA;
  return set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

static std::mutex g_attr_mutex;
static std::map<std::pair<const void*, int>, size_t> g_attr;

bool smem_attr_known(const void* kernel, int device, size_t smem) {
  std::lock_guard<std::mutex> lock(g_attr_mutex);
  auto it = g_attr.find({kernel, device});
  return it != g_attr.end() && it->second >= smem;
}

void smem_attr_record(const void* kernel, int device, size_t smem) {
  std::lock_guard<std::mutex> lock(g_attr_mutex);
  size_t& v = g_attr[{kernel, device}];
  if (smem > v) v = smem;
}

// ---------------------------------------------------------------------------
// FP64 coefficient tables
// ---------------------------------------------------------------------------
struct cd {
  double x, y;
};
__device__ __forceinline__ cd mk(double x, double y) { return cd{x, y}; }
__device__ __forceinline__ cd operator+(cd a, cd b) { return mk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cd operator-(cd a, cd b) { return mk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ cd operator*(cd a, cd b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cd operator*(double s, cd a) { return mk(s * a.x, s * a.y); }
__device__ __forceinline__ cd operator+(double s, cd a) { return mk(s + a.x, a.y); }
__device__ __forceinline__ cd cdiv(cd a, cd b) {
  // Smith's algorithm (scaled by the larger component of b)
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, den = b.x + b.y * r;
    return mk((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  } else {
    const double r = b.x / b.y, den = b.x * r + b.y;
    return mk((a.x * r + a.y) / den, (a.y * r - a.x) / den);
  }
}
__device__ __forceinline__ cd cexpd(cd z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double e = exp(z.x);
  return mk(e * c, e * s);
}
__device__ __forceinline__ float2 tof(cd z) { return make_float2((float)z.x, (float)z.y); }
// exp(z) - 1 without the cancellation of exp(z) - 1 near z = 0:
// Re = e^x cos y - 1 = expm1(x) cos y - 2 sin^2(y/2), Im = e^x sin y.
__device__ __forceinline__ cd cexpm1d(cd z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double em = expm1(z.x);
  const double sh = sin(0.5 * z.y);
  return mk(em * c - 2.0 * sh * sh, (em + 1.0) * s);
}

// One thread per (batch, channel, point) entry of L. Tables (float2) are
// written at tab[t * ts + idx] in the scheme's order (fsm_common.cuh); the exponential tables
// hold exp(dt L) - 1 and exp(dt L / 2) - 1.
// SETDRK: phi-functions as the mean over M contour points z_j = r e^{i pi (2j-1)/M} + dt L
// of the Kassam-Trefethen integrands, real part kept (integrator/_stable_etdrk/_uncached.py:8-43, 46-211);
// ETDRK1/2: closed forms with the L == 0 limits (integrator/_etdrk.py:30-82).
// `count` entries starting at table entry offset `first`; L is indexed modulo `lcount`
// (L shared by every table entry when the symbol has no batch dimension).
__global__ void k_phi_tables(const double2* __restrict__ L, int64_t lcount, int64_t first, int64_t count, double dt,
                             int integ, int M, double r, int exact, float2* __restrict__ tab, int64_t ts) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int64_t idx = first + k;
  const cd l = L ? mk(L[idx % lcount].x, L[idx % lcount].y) : mk(0.0, 0.0);
  const cd hl = dt * l;
  if (integ == FSM_APPLY) {
    tab[idx] = tof(l);
    return;
  }
  if (is_rk(integ)) {
    // explicit Runge-Kutta slopes dt (L a + N): the tables are dt L and dt
    tab[idx] = tof(hl);
    tab[ts + idx] = make_float2((float)dt, 0.f);
    return;
  }
  const cd Em1 = cexpm1d(hl);
  tab[idx] = tof(Em1);
  if (integ == FSM_ETDRK0) return;
  if (integ == FSM_ETDRK1 || integ == FSM_ETDRK2) {
    const bool zero = (l.x == 0.0 && l.y == 0.0);
    const cd c1 = zero ? mk(dt, 0.0) : cdiv(Em1, l);
    tab[ts + idx] = tof(c1);
    if (integ == FSM_ETDRK2) {
      const cd c2 = zero ? mk(0.5 * dt, 0.0) : cdiv(Em1 - hl, dt * (l * l));
      tab[2 * ts + idx] = tof(c2);
    }
    return;
  }
  // phi-function values: s_e1 = (e^z-1)/z, s_e2 = (e^z-1-z)/z^2, s_h = (e^{z/2}-1)/z,
  // s_a = (-4-z+e^z(4-3z+z^2))/z^3, s_b = (2+z+e^z(z-2))/z^3, s_c = (-4-3z-z^2+e^z(4-z))/z^3
  cd s_e1 = mk(0, 0), s_e2 = mk(0, 0), s_h = mk(0, 0), s_a = mk(0, 0), s_b = mk(0, 0), s_c = mk(0, 0);
  const cd one = mk(1.0, 0.0);
  if (exact) {
    // The mean over M contour points equals the function up to r^M / M! (the host checked that
    // this is below 1e-10), so the functions are evaluated directly at z = dt L: Taylor series
    // near 0 (coefficients from expanding e^z), closed forms elsewhere.
    const cd z = hl;
    const double az = sqrt(z.x * z.x + z.y * z.y);
    if (az < 0.5) {
      cd zk = one;
      double fact = 1.0;  // k!
      for (int k = 0; k < 24; ++k) {
        const double f1 = fact * (k + 1), f2 = f1 * (k + 2), f3 = f2 * (k + 3);  // (k+1)!, (k+2)!, (k+3)!
        s_e1 = s_e1 + (1.0 / f1) * zk;
        s_e2 = s_e2 + (1.0 / f2) * zk;
        s_h = s_h + (ldexp(1.0, -(k + 1)) / f1) * zk;
        s_a = s_a + ((double)(k + 1) * (k + 1) / f3) * zk;
        s_b = s_b + ((double)(k + 1) / f3) * zk;
        s_c = s_c + ((double)(1 - k) / f3) * zk;
        zk = zk * z;
        fact = f1;
      }
    } else {
      const cd ez = cexpd(z);
      const cd z2 = z * z, z3 = z2 * z;
      s_e1 = cdiv(ez - one, z);
      s_e2 = cdiv(ez - one - z, z2);
      s_h = cdiv(cexpd(0.5 * z) - one, z);
      s_a = cdiv(mk(-4.0, 0.0) - z + ez * (mk(4.0, 0.0) - 3.0 * z + z2), z3);
      s_b = cdiv(mk(2.0, 0.0) + z + ez * (mk(-2.0, 0.0) + z), z3);
      s_c = cdiv(mk(-4.0, 0.0) - 3.0 * z - z2 + ez * (mk(4.0, 0.0) - z), z3);
    }
    const double m = (double)M;  // the writes below divide by M
    s_e1 = m * s_e1; s_e2 = m * s_e2; s_h = m * s_h; s_a = m * s_a; s_b = m * s_b; s_c = m * s_c;
  } else {
    for (int j = 1; j <= M; ++j) {
      double sn, cs;
      sincospi((double)(2 * j - 1) / (double)M, &sn, &cs);
      const cd z = mk(r * cs, r * sn) + hl;
      const cd ez = cexpd(z);
      const cd z2 = z * z, z3 = z2 * z;
      s_e1 = s_e1 + cdiv(ez - one, z);
      s_e2 = s_e2 + cdiv(ez - one - z, z2);
      s_h = s_h + cdiv(cexpd(0.5 * z) - one, z);
      s_a = s_a + cdiv(mk(-4.0, 0.0) - z + ez * (mk(4.0, 0.0) - 3.0 * z + z2), z3);
      s_b = s_b + cdiv(mk(2.0, 0.0) + z + ez * (mk(-2.0, 0.0) + z), z3);
      s_c = s_c + cdiv(mk(-4.0, 0.0) - 3.0 * z - z2 + ez * (mk(4.0, 0.0) - z), z3);
    }
  }
  const double inv = dt / (double)M;
  auto re = [&](cd s) { return make_float2((float)(inv * s.x), 0.f); };
  switch (integ) {
    case FSM_SETDRK1:
      tab[ts + idx] = re(s_e1);
      break;
    case FSM_SETDRK2:
      tab[ts + idx] = re(s_e1);
      tab[2 * ts + idx] = re(s_e2);
      break;
    case FSM_SETDRK3:
      tab[ts + idx] = tof(cexpm1d(0.5 * hl));
      tab[2 * ts + idx] = re(s_h);
      tab[3 * ts + idx] = re(s_e1);
      tab[4 * ts + idx] = re(s_a);
      tab[5 * ts + idx] = make_float2((float)(4.0 * inv * s_b.x), 0.f);
      tab[6 * ts + idx] = re(s_c);
      break;
    case FSM_SETDRK4:
    default:
      tab[ts + idx] = tof(cexpm1d(0.5 * hl));
      tab[2 * ts + idx] = re(s_h);
      tab[3 * ts + idx] = re(s_a);
      tab[4 * ts + idx] = re(s_b);
      tab[5 * ts + idx] = re(s_c);
      break;
  }
}

// Linear programs (and explicit-source-only ones): the nonlinear value is the
// constant source, so every point advances independently through all steps.
__global__ void k_pointwise(StepArgs a, int64_t total) {
  const int C = a.C;
  const int64_t S = a.S;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = idx % S;
    const int c = (int)((idx / S) % C);
    const int b = (int)(idx / (S * C));
    float2 u = a.state[idx];
    float2 aux[6] = {};  // scheme running sums (acc, q; Runge-Kutta partial inputs)
    const int64_t toff = (tab_batch(a, b) * a.lin_ch + (a.lin_ch > 1 ? c : 0)) * S + s;
    const float2* tab = a.tab + toff;
    const float2 nv = a.src ? a.src[((int64_t)(a.src_batch > 1 ? b : 0) * C + c) * S + s] : make_float2(0.f, 0.f);
    const int slot0 = a.slots ? a.slots[0] : -1;
    if (slot0 >= 0) a.traj[(((int64_t)b * a.n_frames + slot0) * C + c) * S + s] = u;
    for (int step = 0; step < a.steps; ++step) {
      if (a.integ == FSM_ETDRK0) {
        u = cexpmul(tab[0], u);
      } else {
        for (int st = 0; st < a.nstages; ++st) (void)etd_stage(a.integ, st, nv, &u, aux, aux + 1, tab, a.ts, 1);
      }
      const int slot = a.slots ? a.slots[step + 1] : -1;
      if (slot >= 0) a.traj[(((int64_t)b * a.n_frames + slot) * C + c) * S + s] = u;
    }
    a.state[idx] = u;
  }
}

int launch_pointwise(const FsmPlan* p, const StepArgs& a, cudaStream_t st) {
  const int64_t total = (int64_t)a.B * a.C * a.S;
  if (total == 0) return FSM_OK;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_pointwise<<<blocks, 256, 0, st>>>(a, total);
  return cuda_check(cudaGetLastError(), "k_pointwise");
}

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// The M-point contour mean of an entire function around z differs from its value at z by
// about r^M / M! (the M-th Taylor term); below 1e-10 the tables use the direct evaluation.
static int phi_exact(const FsmPlan* p) {
  const double bound = exp((double)p->n_points * log(p->radius) - lgamma((double)p->n_points + 1.0));
  return bound < 1e-10 ? 1 : 0;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static void free_plan(FsmPlan* p) {
  if (!p) return;
  cudaFree(p->kvec);
  cudaFree(p->keep);
  cudaFree(p->tile_zero);
  cudaFree(p->tw);
  cudaFree(p->tab);
  cudaFree(p->source);
  cudaFree(p->lin);
  delete p;
}

}  // namespace fsm

using namespace fsm;

namespace fsm {
int set_batch_dt_range(FsmPlan* p, int32_t b0, int32_t n, double dt, cudaStream_t st) {
  if (!p || b0 < 0 || n < 1 || (int64_t)b0 + n > p->lin_batch || p->lin_batch < 2 || !(dt > 0.0))
    return set_error(FSM_ERR_INVALID, "set_batch_dt arguments");
  const int64_t per = (int64_t)p->lin_ch * p->S;
  const int64_t lcount = (int64_t)p->lin_src_batch * per;
  const int64_t count = per * n;
  const int threads = 128;
  k_phi_tables<<<(unsigned)((count + threads - 1) / threads), threads, 0, st>>>(
      p->lin, lcount, (int64_t)b0 * per, count, dt, p->integ, p->n_points, p->radius, phi_exact(p), p->tab,
      p->tstride);
  return cuda_check(cudaGetLastError(), "k_phi_tables (batch entries)");
}
}  // namespace fsm

extern "C" {

int fsm_abi_version(void) { return 1; }

int fsm_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return FSM_ERR_INVALID;
  strncpy(buf, g_last_error.c_str(), len - 1);
  buf[len - 1] = '\0';
  return FSM_OK;
}

int fsm_plan_create(const FsmMeshDesc* mesh, const FsmProgramDesc* prog, double dt, void* stream, FsmPlan** out) {
  if (!mesh || !prog || !out) return set_error(FSM_ERR_INVALID, "null argument");
  *out = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  const int nd = mesh->ndim;
  if (nd < 1 || nd > 3) return set_error(FSM_ERR_INVALID, "ndim must be 1..3");
  for (int i = 0; i < nd; ++i) {
    const int n = mesh->n[i];
    const int hi = (i == nd - 1) ? 4096 : 512;
    if (!is_pow2(n) || n < 16 || n > hi)
      return set_error(FSM_ERR_UNSUPPORTED, "axis " + std::to_string(i) + ": " + std::to_string(n) +
                                                " points (need a power of two in 16.." + std::to_string(hi) + ")");
    if (!(mesh->length[i] > 0.0)) return set_error(FSM_ERR_INVALID, "mesh length must be positive");
  }
  if (nd > 1 && mesh->n[nd - 1] > 512) return set_error(FSM_ERR_UNSUPPORTED, "multi-D last axis above 512 points");
  const int C = prog->n_channel;
  if (C < 1 || C > 8) return set_error(FSM_ERR_INVALID, "n_channel must be 1..8");
  const int integ = prog->integrator;
  if (scheme_tables(integ) == 0) return set_error(FSM_ERR_INVALID, "unknown integrator");
  const int nl = prog->nonlinear;
  int path = 0;
  switch (nl) {
    case FSM_NL_NONE:
      path = 3;
      break;
    case FSM_NL_CONVECTION:
      if (C != nd) return set_error(FSM_ERR_INVALID, "convection needs n_channel == ndim");
      path = nd == 1 ? 1 : (nd == 2 ? 2 : 4);
      break;
    case FSM_NL_VORTICITY:
      if (nd != 2 || C != 1) return set_error(FSM_ERR_INVALID, "vorticity convection needs a 2D scalar field");
      path = 2;
      break;
    case FSM_NL_KS:
      if (C != 1) return set_error(FSM_ERR_INVALID, "KS convection needs a scalar field");
      path = nd == 1 ? 1 : (nd == 2 ? 2 : 4);
      break;
    case FSM_NL_LERAY:
      if (C != nd) return set_error(FSM_ERR_INVALID, "Leray-projected convection needs n_channel == ndim");
      path = nd == 2 ? 2 : (nd == 3 ? 4 : 0);
      break;
    default:
      return set_error(FSM_ERR_INVALID, "unknown nonlinear term");
  }
  if (path == 0) return set_error(FSM_ERR_UNSUPPORTED, "no fused kernel for this program on a " + std::to_string(nd) + "D mesh");
  if (path == 4) {
    for (int i = 0; i < 3; ++i)
      if (mesh->n[i] > 256)
        return set_error(FSM_ERR_UNSUPPORTED, "3D fused kernels take 16..256 points per axis");
  }
  if (integ == FSM_ETDRK0 && (nl != FSM_NL_NONE || prog->source))
    return set_error(FSM_ERR_INVALID, "ETDRK0 only supports linear programs");
  if (nl == FSM_NL_NONE && integ != FSM_ETDRK0 && !prog->source && scheme_stages(integ) == 0)
    return set_error(FSM_ERR_INVALID, "bad integrator");
  if (prog->lin_batch < 1 || prog->lin_channel < 1 || (prog->lin_channel != 1 && prog->lin_channel != C))
    return set_error(FSM_ERR_INVALID, "lin_batch/lin_channel");
  if (prog->source && prog->src_batch < 1) return set_error(FSM_ERR_INVALID, "src_batch");
  if (integ >= FSM_SETDRK1 && (prog->n_integration_points < 1 || !(prog->integration_radius > 0.0)))
    return set_error(FSM_ERR_INVALID, "n_integration_points / integration_radius");

  FsmPlan* p = new FsmPlan();
  cudaGetDevice(&p->device);
  p->ndim = nd;
  for (int i = 0; i < 3; ++i) p->n[i] = i < nd ? mesh->n[i] : 1;
  p->h = mesh->n[nd - 1] / 2 + 1;
  p->S = p->h;
  p->R = mesh->n[nd - 1];
  for (int i = 0; i < nd - 1; ++i) {
    p->S *= mesh->n[i];
    p->R *= mesh->n[i];
  }
  p->C = C;
  p->nl = nl;
  p->flags = prog->flags;
  p->integ = integ;
  p->nstages = scheme_stages(integ);
  p->ntab = scheme_tables(integ);
  p->nl_coef = (float)prog->nonlinear_coef;
  p->lin_src_batch = prog->linear_coef ? prog->lin_batch : 1;
  p->lin_ch = prog->linear_coef ? prog->lin_channel : 1;
  p->lin_batch = prog->table_batch > 0 ? prog->table_batch : p->lin_src_batch;
  if (p->lin_src_batch > 1 && p->lin_batch != p->lin_src_batch) {
    delete p;
    return set_error(FSM_ERR_INVALID, "table_batch must equal lin_batch for a batched linear coefficient");
  }
  p->lin_present = prog->linear_coef != nullptr;
  p->dt = dt;
  p->n_points = prog->n_integration_points > 0 ? prog->n_integration_points : 16;
  p->radius = prog->integration_radius > 0 ? prog->integration_radius : 1.0;
  p->path = path;
  p->n_aux = scheme_aux(integ);
  if (path == 2) {
    p->n_mid = (nl == FSM_NL_KS) ? 2 : 4;
    p->n_prod = (nl == FSM_NL_CONVECTION || nl == FSM_NL_LERAY) ? 2 : 1;
  } else if (path == 4) {
    p->n_mid = (nl == FSM_NL_KS) ? 2 : 2 * C;
    p->n_mid2 = 3 * (p->n_mid / 2);
    p->n_prod = (nl == FSM_NL_KS) ? 1 : C;
  }

  int rc = FSM_OK;
  // wavenumbers 2 pi f and keep flags per axis
  int total_k = 0;
  for (int i = 0; i < nd; ++i) {
    p->koff[i] = total_k;
    total_k += mesh->n[i];
  }
  std::vector<float> kv(total_k);
  std::vector<uint8_t> keep(total_k, 1);
  for (int i = 0; i < nd; ++i) {
    const int n = mesh->n[i];
    for (int j = 0; j < n; ++j) {
      const int idx = (j < (n + 1) / 2) ? j : j - n;  // fftfreq ordering (n/2 -> -n/2)
      kv[p->koff[i] + j] = (float)(2.0 * M_PI * (double)idx / mesh->length[i]);
      if (prog->keep[i]) keep[p->koff[i] + j] = prog->keep[i][j] ? 1 : 0;
    }
  }
  // Column tiles of the register axis-0 pass (2D column pass, 3D x pass) whose inner columns
  // are all dealiased: the fields built from the masked state are zero there.
  std::vector<uint8_t> tile_zero;
  {
    const int n0 = mesh->n[0];
    const int w = n0 == 256 ? 16 : (n0 == 128 || n0 == 64) ? 32 : (n0 == 32 || n0 == 16) ? 64 : 0;
    if (w && (path == 2 || path == 4)) {
      const int h = mesh->n[nd - 1] / 2 + 1;
      const int64_t inner = p->S / n0;
      auto kept = [&](int64_t j) {
        if (nd == 2) return keep[p->koff[1] + j] != 0;
        return keep[p->koff[1] + j / h] != 0 && keep[p->koff[2] + j % h] != 0;
      };
      tile_zero.resize((size_t)((inner + w - 1) / w));
      for (size_t t = 0; t < tile_zero.size(); ++t) {
        bool any = false;
        for (int64_t j = (int64_t)t * w; j < (int64_t)(t + 1) * w && j < inner; ++j) any = any || kept(j);
        tile_zero[t] = any ? 0 : 1;
      }
    }
  }
  p->hk = p->h;
  if (path == 2) {
    const int n0 = mesh->n[0], n1 = mesh->n[1];
    const bool reg = is_pow2(n0) && n0 >= 16 && n0 <= 256 && is_pow2(n1) && n1 >= 16 && n1 <= 256;
    int pre = 0;
    while (pre < p->h && keep[p->koff[1] + pre]) ++pre;
    bool prefix = true;
    for (int j = pre; j < p->h; ++j) prefix = prefix && !keep[p->koff[1] + j];
    if (reg && prefix && pre == n1 / 3 + 1) p->hk = pre;
  }
  p->wp = p->S / mesh->n[0];
  if (path == 2) {
    const int n0 = mesh->n[0], n1 = mesh->n[1];
    if (is_pow2(n0) && n0 >= 16 && n0 <= 256 && is_pow2(n1) && n1 >= 16 && n1 <= 256) p->wp = (p->h + 1) & ~1;
  }
  p->ms = (int64_t)mesh->n[0] * p->wp;
  std::vector<float2> tw(kTwiddleMax);
  for (int k = 0; k < kTwiddleMax; ++k) {
    const double ang = 2.0 * M_PI * (double)k / (double)kTwiddleMax;
    tw[k] = make_float2((float)cos(ang), (float)(-sin(ang)));
  }
  p->tstride = (int64_t)p->lin_batch * p->lin_ch * p->S;
  const size_t tab_bytes = (size_t)p->ntab * p->tstride * sizeof(float2);
  if ((rc = cuda_check(cudaMalloc(&p->kvec, total_k * sizeof(float)), "cudaMalloc kvec")) ||
      (rc = cuda_check(cudaMalloc(&p->keep, total_k), "cudaMalloc keep")) ||
      (rc = cuda_check(cudaMalloc(&p->tw, kTwiddleMax * sizeof(float2)), "cudaMalloc twiddles")) ||
      (rc = cuda_check(cudaMalloc(&p->tab, tab_bytes), "cudaMalloc tables"))) {
    free_plan(p);
    return rc;
  }
  if (!tile_zero.empty() &&
      ((rc = cuda_check(cudaMalloc(&p->tile_zero, tile_zero.size()), "cudaMalloc tile flags")) ||
       (rc = cuda_check(cudaMemcpyAsync(p->tile_zero, tile_zero.data(), tile_zero.size(), cudaMemcpyHostToDevice, st),
                        "copy tile flags")))) {
    free_plan(p);
    return rc;
  }
  if ((rc = cuda_check(cudaMemcpyAsync(p->kvec, kv.data(), total_k * sizeof(float), cudaMemcpyHostToDevice, st), "copy kvec")) ||
      (rc = cuda_check(cudaMemcpyAsync(p->keep, keep.data(), total_k, cudaMemcpyHostToDevice, st), "copy keep")) ||
      (rc = cuda_check(cudaMemcpyAsync(p->tw, tw.data(), kTwiddleMax * sizeof(float2), cudaMemcpyHostToDevice, st), "copy twiddles"))) {
    free_plan(p);
    return rc;
  }
  if (prog->source) {
    p->src_batch = prog->src_batch;
    const size_t sb = (size_t)p->src_batch * C * p->S * sizeof(float2);
    if ((rc = cuda_check(cudaMalloc(&p->source, sb), "cudaMalloc source")) ||
        (rc = cuda_check(cudaMemcpyAsync(p->source, prog->source, sb, cudaMemcpyDeviceToDevice, st), "copy source"))) {
      free_plan(p);
      return rc;
    }
  }
  const int64_t lcount = (int64_t)p->lin_src_batch * p->lin_ch * p->S;
  if (p->lin_present) {
    // keep the FP64 symbol for later per-entry time-step changes
    if ((rc = cuda_check(cudaMalloc(&p->lin, lcount * sizeof(double2)), "cudaMalloc linear symbol")) ||
        (rc = cuda_check(cudaMemcpyAsync(p->lin, prog->linear_coef, lcount * sizeof(double2), cudaMemcpyDeviceToDevice,
                                         st), "copy linear symbol"))) {
      free_plan(p);
      return rc;
    }
  }
  const int64_t count = p->tstride;
  const int threads = 128;
  k_phi_tables<<<(unsigned)((count + threads - 1) / threads), threads, 0, st>>>(
      p->lin, lcount, 0, count, dt, integ, p->n_points, p->radius, phi_exact(p), p->tab, p->tstride);
  if ((rc = cuda_check(cudaGetLastError(), "k_phi_tables"))) {
    free_plan(p);
    return rc;
  }
  // The host vectors above are pageable: make sure the copies have consumed them.
  if ((rc = cuda_check(cudaStreamSynchronize(st), "plan synchronise"))) {
    free_plan(p);
    return rc;
  }
  *out = p;
  return FSM_OK;
}

int fsm_plan_set_batch_dt(FsmPlan* p, int32_t b, double dt, void* stream) {
  return fsm::set_batch_dt_range(p, b, 1, dt, (cudaStream_t)stream);
}

int fsm_plan_move_batch(FsmPlan* p, int32_t dst, int32_t src, void* stream) {
  if (!p || dst < 0 || src < 0 || dst >= p->lin_batch || src >= p->lin_batch)
    return set_error(FSM_ERR_INVALID, "move_batch arguments");
  if (dst == src) return FSM_OK;
  const int64_t per = (int64_t)p->lin_ch * p->S;
  for (int t = 0; t < p->ntab; ++t) {
    int rc = cuda_check(cudaMemcpyAsync(p->tab + t * p->tstride + dst * per, p->tab + t * p->tstride + src * per,
                                        per * sizeof(float2), cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
                        "move tables");
    if (rc) return rc;
  }
  return FSM_OK;
}

int fsm_plan_tables(const FsmPlan* p, void* dst, size_t capacity_bytes, int32_t* ntab, int64_t* entries,
                    void* stream) {
  if (!p) return set_error(FSM_ERR_INVALID, "plan_tables arguments");
  if (ntab) *ntab = p->ntab;
  if (entries) *entries = p->tstride;
  if (!dst) return FSM_OK;
  const size_t need = (size_t)p->ntab * p->tstride * sizeof(float2);
  if (capacity_bytes < need) return set_error(FSM_ERR_INVALID, "plan_tables: buffer too small");
  return cuda_check(cudaMemcpyAsync(dst, p->tab, need, cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
                    "copy tables");
}

int fsm_plan_destroy(FsmPlan* plan) {
  if (!plan) return FSM_OK;
  cudaDeviceSynchronize();
  free_plan(plan);
  return FSM_OK;
}

static size_t workspace_layout(const FsmPlan* p, int32_t batch, int32_t steps, size_t* off_arrays) {
  size_t bytes = align256((size_t)(steps + 1) * sizeof(int32_t));  // record slots
  size_t dc = 256;                                                 // KS batch-mean scratch
  if (p->path == 1 && p->nl == FSM_NL_KS && (p->flags & FSM_FLAG_REMOVE_MEAN))
    // 1D: per-stage k = 0 products, initial k = 0 values, per-stage batch means
    dc = align256(((size_t)steps * p->nstages * (batch + 1) + batch) * sizeof(float2));
  bytes += dc;
  if (off_arrays) *off_arrays = bytes;
  if (p->path == 2 || p->path == 4) {
    const size_t per = ((size_t)(p->n_aux * p->C + p->n_mid2) * p->S + (size_t)(p->n_mid + p->n_prod) * p->ms) *
                       sizeof(float2);
    bytes += align256(per * (size_t)batch);
  }
  return bytes;
}

int fsm_plan_workspace_bytes(const FsmPlan* plan, int32_t batch, int32_t steps, size_t* bytes) {
  if (!plan || !bytes || batch < 0 || steps < 0) return set_error(FSM_ERR_INVALID, "workspace_bytes arguments");
  *bytes = workspace_layout(plan, batch, steps, nullptr);
  return FSM_OK;
}

int fsm_plan_launch_count(const FsmPlan* plan, int32_t batch, int32_t steps, int64_t* launches) {
  if (!plan || !launches || steps < 0 || batch < 0) return set_error(FSM_ERR_INVALID, "launch_count arguments");
  if (plan->path == 2 || plan->path == 4) {
    const int64_t per_stage = (plan->path == 4 ? 4 : 2) +
                              ((plan->nl == FSM_NL_KS && (plan->flags & FSM_FLAG_REMOVE_MEAN)) ? 1 : 0);
    *launches = (int64_t)fsm::split_parts(plan, batch) * (1 + (int64_t)steps * plan->nstages * per_stage);
  } else if (plan->path == 1 && plan->nl == FSM_NL_KS && (plan->flags & FSM_FLAG_REMOVE_MEAN)) {
    *launches = steps > 0 ? 3 : 1;  // line kernel, batch means of k = 0, k = 0 fix-up
  } else {
    *launches = 1;
  }
  return FSM_OK;
}

}  // extern "C"

namespace {

// Optional per-launch CUDA-event timing (fsm_integrate_profiled).
struct LaunchProfile {
  std::vector<cudaEvent_t> start, stop;
  std::vector<int> kind;
  cudaStream_t st;
  int begin(int k) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return FSM_ERR_CUDA;
    cudaEventRecord(e, st);
    start.push_back(e);
    kind.push_back(k);
    return FSM_OK;
  }
  int end() {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return FSM_ERR_CUDA;
    cudaEventRecord(e, st);
    stop.push_back(e);
    return FSM_OK;
  }
  int collect(double* ms, int64_t* count) {
    if (!stop.empty()) {
      cudaError_t err = cudaEventSynchronize(stop.back());
      if (err != cudaSuccess) return cuda_check(err, "profile synchronise");
    }
    for (size_t i = 0; i < stop.size(); ++i) {
      float t = 0.f;
      cudaEventElapsedTime(&t, start[i], stop[i]);
      ms[kind[i]] += t;
      count[kind[i]] += 1;
    }
    for (auto e : start) cudaEventDestroy(e);
    for (auto e : stop) cudaEventDestroy(e);
    return FSM_OK;
  }
};

enum { kProfColumn = 0, kProfRow = 1, kProfPrime = 2, kProfOther = 3 };

template <class F>
int timed(LaunchProfile* prof, int kind, F&& launch) {
  if (prof) prof->begin(kind);
  int rc = launch();
  if (prof) prof->end();
  return rc;
}

}  // namespace

namespace fsm {
size_t integrate_workspace_bytes(const FsmPlan* p, int32_t batch, int32_t steps) {
  return workspace_layout(p, batch, steps, nullptr);
}
}  // namespace fsm

namespace fsm {
// Batches at or above kSplitPoints spectral points run in parts of about kPartPoints points
// (2 to kMaxParts parts, at most one per sample) on as many streams. Measured on 256^2 x 64
// (2.1 M points): one sequence 322 us per step, 2 parts 284, 4 parts 270, 8 parts 261.
constexpr int64_t kSplitPoints = (int64_t)3 << 19;
constexpr int64_t kPartPoints = (int64_t)1 << 18;
constexpr int kMaxParts = 8;

// Number of parts an uncaptured, unprofiled integrate of `batch` samples runs in (1: one sequence).
int split_parts(const FsmPlan* p, int batch) {
  if (p->path != 2 && p->path != 4) return 1;
  if (p->nl == FSM_NL_KS && (p->flags & FSM_FLAG_REMOVE_MEAN)) return 1;  // the batch mean couples the samples
  if (batch < 2 || (int64_t)batch * p->S < kSplitPoints) return 1;
  int64_t parts = (int64_t)batch * p->S / kPartPoints;
  parts = parts < 2 ? 2 : (parts > kMaxParts ? kMaxParts : parts);
  return (int)(parts < batch ? parts : batch);
}
}  // namespace fsm

namespace {
using fsm::kMaxParts;

// kMaxParts non-blocking streams per (device, caller stream), with the caller's priority, for
// the parts of a split batch. The sets of the kSplitCallers most recently used caller streams
// are kept; an older set is released when the last call using it returns (cudaStreamDestroy
// lets work already queued on a stream finish), so callers that create and drop streams do not
// accumulate library streams.
constexpr size_t kSplitCallers = 32;

struct SplitStreams {
  cudaStream_t s[kMaxParts] = {};
  int n = 0;
  ~SplitStreams() {
    for (int h = 0; h < n; ++h) cudaStreamDestroy(s[h]);
  }
};

static std::mutex g_split_mutex;
static std::map<std::pair<int, cudaStream_t>, std::pair<std::shared_ptr<SplitStreams>, uint64_t>> g_split;
static uint64_t g_split_clock = 0;

int split_streams(cudaStream_t st, std::shared_ptr<SplitStreams>* out) {
  int dev = 0;
  int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_split_mutex);
  auto it = g_split.find({dev, st});
  if (it == g_split.end()) {
    int prio = 0;
    if ((rc = cuda_check(cudaStreamGetPriority(st, &prio), "cudaStreamGetPriority"))) return rc;
    auto set = std::make_shared<SplitStreams>();
    for (; set->n < kMaxParts; ++set->n)
      if ((rc = cuda_check(cudaStreamCreateWithPriority(&set->s[set->n], cudaStreamNonBlocking, prio), "stream")))
        return rc;  // the streams created so far are destroyed with the set
    if (g_split.size() >= kSplitCallers) {  // drop the least recently used caller's set
      auto old = g_split.begin();
      for (auto j = g_split.begin(); j != g_split.end(); ++j)
        if (j->second.second < old->second.second) old = j;
      g_split.erase(old);
    }
    it = g_split.emplace(std::make_pair(dev, st), std::make_pair(set, (uint64_t)0)).first;
  }
  it->second.second = ++g_split_clock;
  *out = it->second.first;
  return FSM_OK;
}

// Events of one split integrate, destroyed on every return path (a destroyed event that is still
// recorded on a stream is released once the stream has passed it).
struct SplitEvents {
  cudaEvent_t fork = nullptr;
  cudaEvent_t done[kMaxParts] = {};
  ~SplitEvents() {
    if (fork) cudaEventDestroy(fork);
    for (int h = 0; h < kMaxParts; ++h)
      if (done[h]) cudaEventDestroy(done[h]);
  }
  int create(int np) {
    int rc = cuda_check(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "event");
    for (int h = 0; h < np && !rc; ++h) rc = cuda_check(cudaEventCreateWithFlags(&done[h], cudaEventDisableTiming), "event");
    return rc;
  }
};

// The arguments of samples [b0, b0 + n) of a batch: state, trajectory, per-sample tables and
// sources offset to the first sample, the pass arrays laid out for n samples in their own
// slice of the workspace (the workspace holds the arrays of all samples, sample-major slices).
StepArgs batch_arrays(const FsmPlan* p, StepArgs a, float2* arr, int b0, int n) {
  const int64_t S = p->S;
  const int64_t per_sample = (int64_t)(p->n_aux * p->C + p->n_mid2) * S + (int64_t)(p->n_mid + p->n_prod) * p->ms;
  a.state += (int64_t)b0 * p->C * S;
  if (a.traj) a.traj += (int64_t)b0 * a.n_frames * p->C * S;
  if (a.tab_entry) a.tab_entry += b0;  // the samples' own entries
  else if (p->lin_batch > 1) a.tab += (int64_t)b0 * p->lin_ch * S;
  if (a.src && p->src_batch > 1) a.src += (int64_t)b0 * p->C * S;
  a.aux = arr + (int64_t)b0 * per_sample;
  a.mid = a.aux + (int64_t)n * p->n_aux * p->C * S;
  a.mid2 = a.mid + (int64_t)n * p->n_mid * p->ms;
  a.prod = a.mid2 + (int64_t)n * p->n_mid2 * S;
  a.B = n;
  return a;
}

}  // namespace

namespace fsm {
int plane_args(const FsmPlan* p, void* state, int32_t batch, int32_t steps, void* workspace, size_t workspace_bytes,
               StepArgs* out) {
  if (!p || !state || !workspace || !out || batch < 1 || steps < 0) return set_error(FSM_ERR_INVALID, "plane_args");
  if (p->path != 2) return set_error(FSM_ERR_INVALID, "plane_args: not a 2D plane-pass plan");
  size_t off_arrays = 0;
  if (workspace_bytes < workspace_layout(p, batch, steps, &off_arrays))
    return set_error(FSM_ERR_INVALID, "plane_args: workspace too small");
  char* ws = (char*)workspace;
  StepArgs a = base_args(p, state, batch, steps);
  a.dc = (float2*)(ws + align256((size_t)(steps + 1) * sizeof(int32_t)));
  *out = batch_arrays(p, a, (float2*)(ws + off_arrays), 0, batch);
  return FSM_OK;
}
}  // namespace fsm

namespace {

// The launch sequence of the plane (2D) / volume (3D) passes, step by step: prime() before
// the first step, then step(k) for k = 0 .. steps-1, on one stream.
struct PlaneSequence {
  const FsmPlan* p;
  StepArgs a;
  const int32_t* record_slot;
  int32_t steps;
  cudaStream_t st;
  LaunchProfile* prof;

  int prime() {
    a.stage = -1;
    a.emit = steps > 0;
    a.slot = record_slot ? record_slot[0] : -1;
    return timed(prof, kProfPrime, [&] { return launch_plane_col(p, a, st); });
  }
  int step(int k) {
    int rc;
    const bool ks_mean = p->nl == FSM_NL_KS && (p->flags & FSM_FLAG_REMOVE_MEAN);
    const bool vol = p->path == 4;
    for (int s = 0; s < p->nstages; ++s) {
      if (vol) {
        if ((rc = timed(prof, kProfOther, [&] { return launch_volume_axis1_inv(p, a, st); }))) return rc;
        if ((rc = timed(prof, kProfRow, [&] { return launch_volume_axis2(p, a, st); }))) return rc;
        if ((rc = timed(prof, kProfOther, [&] { return launch_volume_axis1_fwd(p, a, st); }))) return rc;
      } else {
        if ((rc = timed(prof, kProfRow, [&] { return launch_plane_row(p, a, st); }))) return rc;
      }
      if (ks_mean && (rc = timed(prof, kProfOther, [&] { return launch_ks_mean(p, a, st); }))) return rc;
      const bool last = s == p->nstages - 1;
      a.stage = s;
      a.emit = !(last && k == steps - 1);
      a.slot = (last && record_slot) ? record_slot[k + 1] : -1;
      if ((rc = timed(prof, kProfColumn, [&] { return launch_plane_col(p, a, st); }))) return rc;
    }
    return FSM_OK;
  }
};

}  // namespace

namespace fsm {
// The kernels' arguments for `batch` samples of `state` advanced by `steps` steps, without
// recording (no trajectory, no record slots, no batch-mean scratch).
StepArgs base_args(const FsmPlan* p, void* state, int32_t batch, int32_t steps) {
  StepArgs a;
  memset(&a, 0, sizeof(a));
  a.state = (float2*)state;
  a.slot = -1;
  a.tab = p->tab;
  a.ts = p->tstride;
  a.lin_batch = p->lin_batch;
  a.lin_ch = p->lin_ch;
  a.src = p->source;
  a.src_batch = p->src_batch;
  a.kx = p->kvec + p->koff[0];
  a.ky = p->kvec + p->koff[p->ndim - 1];
  a.km = p->kvec + p->koff[p->ndim == 3 ? 1 : 0];
  a.keepx = p->keep + p->koff[0];
  a.keepy = p->keep + p->koff[p->ndim - 1];
  a.keepm = p->keep + p->koff[p->ndim == 3 ? 1 : 0];
  a.tile_zero = p->tile_zero;
  a.hk = p->hk;
  a.wp = p->wp;
  a.ms = p->ms;
  a.nm = p->ndim == 3 ? p->n[1] : 1;
  a.tw = p->tw;
  a.coef = p->nl_coef;
  a.scale = (float)(1.0 / (double)p->R);
  a.C = p->C;
  a.n_aux = p->n_aux;
  a.n_mid = p->n_mid;
  a.n_prod = p->n_prod;
  a.n_mid2 = p->n_mid2;
  a.integ = p->integ;
  a.nstages = p->nstages;
  a.steps = steps;
  a.B = batch;
  a.flags = p->flags;
  a.S = p->S;
  a.H = p->h;
  return a;
}
}  // namespace fsm

namespace {

int integrate_impl(const FsmPlan* p, int32_t batch, void* state, int32_t steps, const int32_t* record_slot, void* traj,
                   int32_t n_frames, void* workspace, size_t workspace_bytes, cudaStream_t st, LaunchProfile* prof,
                   bool allow_split = true, const int32_t* tab_entry = nullptr) {
  if (!p || !state || batch < 1 || steps < 0) return set_error(FSM_ERR_INVALID, "integrate arguments");
  size_t off_arrays = 0;
  const size_t need = workspace_layout(p, batch, steps, &off_arrays);
  if (!workspace || workspace_bytes < need)
    return set_error(FSM_ERR_INVALID, "workspace too small: need " + std::to_string(need) + " bytes");
  if (p->lin_batch > 1 && batch > p->lin_batch) return set_error(FSM_ERR_INVALID, "batch above the plan's table entries");
  if (p->source && p->src_batch > 1 && p->src_batch != batch) return set_error(FSM_ERR_INVALID, "batch != src_batch");
  if ((int64_t)batch * p->C > 65535 && p->path == 2) return set_error(FSM_ERR_UNSUPPORTED, "batch too large for one launch");
  if (p->path == 4 && (int64_t)batch * p->n_prod * p->n[0] > 65535)
    return set_error(FSM_ERR_UNSUPPORTED, "batch too large for one launch");
  bool any_record = false;
  if (record_slot) {
    for (int i = 0; i <= steps; ++i) {
      if (record_slot[i] >= n_frames) return set_error(FSM_ERR_INVALID, "record slot out of range");
      any_record |= record_slot[i] >= 0;
    }
  }
  if (any_record && !traj) return set_error(FSM_ERR_INVALID, "trajectory buffer missing");

  char* ws = (char*)workspace;
  int32_t* d_slots = (int32_t*)ws;
  int rc;
  // The line (1D) and pointwise kernels read the record slots from the device; the plane and
  // volume passes take them per launch from the host array. The copy reads the caller's host
  // array when it runs, so a captured graph would read it again at every replay: recording is
  // refused while the stream is being captured.
  if (record_slot && (p->path == 1 || p->path == 3)) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if ((rc = cuda_check(cudaStreamIsCapturing(st, &cs), "stream capture query"))) return rc;
    if (cs != cudaStreamCaptureStatusNone)
      return set_error(FSM_ERR_INVALID, "integrate: recording is not supported while the stream is being captured");
    if ((rc = cuda_check(cudaMemcpyAsync(d_slots, record_slot, (size_t)(steps + 1) * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, st), "copy record slots")))
      return rc;
  }
  StepArgs a = base_args(p, state, batch, steps);
  a.tab_entry = tab_entry;
  a.traj = (float2*)traj;
  a.n_frames = n_frames;
  a.slots = record_slot ? d_slots : nullptr;
  a.dc = (float2*)(ws + align256((size_t)(steps + 1) * sizeof(int32_t)));

  if (p->path == 3) return timed(prof, kProfOther, [&] { return launch_pointwise(p, a, st); });
  if (p->path == 1) return timed(prof, kProfOther, [&] { return launch_line(p, a, st); });

  // plane (2D) / volume (3D) passes
  float2* arr = (float2*)(ws + off_arrays);
  a.slots = nullptr;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if ((rc = cuda_check(cudaStreamIsCapturing(st, &cap), "stream capture query"))) return rc;
  // Large batches run in parts on streams forked from the caller's: the parts' launches
  // interleave on the device (the column passes of one overlap the row passes of another),
  // which fills the SMs better than one launch sequence of the whole batch.
  // Samples are independent except under the KS batch-wide mean; capture and the profiled
  // (per-launch timed) call keep one sequence.
  const int NP = (!allow_split || prof || cap != cudaStreamCaptureStatusNone) ? 1 : fsm::split_parts(p, batch);
  const bool split = NP > 1;
  if (!split) {
    PlaneSequence q{p, batch_arrays(p, a, arr, 0, batch), record_slot, steps, st, prof};
    if ((rc = q.prime())) return rc;
    for (int k = 0; k < steps; ++k)
      if ((rc = q.step(k))) return rc;
    return FSM_OK;
  }
  // The parts are enqueued step by step, each part's step waiting for the previous step of
  // the part before it (a ring), so that none runs ahead and leaves the others alone at the end.
  std::shared_ptr<SplitStreams> streams;
  if ((rc = split_streams(st, &streams))) return rc;
  const cudaStream_t* sub = streams->s;
  SplitEvents ev;
  if ((rc = ev.create(NP))) return rc;
  const cudaEvent_t fork = ev.fork;
  const cudaEvent_t* done = ev.done;
  PlaneSequence q[kMaxParts];
  for (int h = 0; h < NP; ++h) {
    const int b0 = (int)((int64_t)batch * h / NP), b1 = (int)((int64_t)batch * (h + 1) / NP);
    q[h] = PlaneSequence{p, batch_arrays(p, a, arr, b0, b1 - b0), record_slot, steps, sub[h], nullptr};
  }
  rc = cuda_check(cudaEventRecord(fork, st), "fork");
  for (int h = 0; h < NP && !rc; ++h) {
    rc = cuda_check(cudaStreamWaitEvent(sub[h], fork, 0), "fork wait");
    if (!rc) rc = q[h].prime();
    if (!rc) rc = cuda_check(cudaEventRecord(done[h], sub[h]), "step event");
  }
  for (int k = 0; k < steps && !rc; ++k) {
    for (int h = 0; h < NP && !rc; ++h) {
      rc = cuda_check(cudaStreamWaitEvent(sub[h], done[(h + NP - 1) % NP], 0), "step wait");
      if (!rc) rc = q[h].step(k);
    }
    for (int h = 0; h < NP && !rc; ++h) rc = cuda_check(cudaEventRecord(done[h], sub[h]), "step event");
  }
  for (int h = 0; h < NP && !rc; ++h) rc = cuda_check(cudaStreamWaitEvent(st, done[h], 0), "join wait");
  return rc;
}


}  // namespace

namespace fsm {
int integrate_on_workspace(const FsmPlan* p, int32_t batch, void* state, int32_t steps, void* workspace,
                           size_t workspace_bytes, cudaStream_t st, const int32_t* tab_entry) {
  return integrate_impl(p, batch, state, steps, nullptr, nullptr, 0, workspace, workspace_bytes, st, nullptr, true,
                        tab_entry);
}

int integrate_with_workspace(const FsmPlan* p, int32_t batch, void* state, int32_t steps, void* workspace,
                             size_t workspace_bytes, cudaStream_t st) {
  // one launch sequence on the caller's stream: no library streams for allocation-free callers
  return integrate_impl(p, batch, state, steps, nullptr, nullptr, 0, workspace, workspace_bytes, st, nullptr, false);
}
}  // namespace fsm

extern "C" {

int fsm_integrate(const FsmPlan* p, int32_t batch, void* state, int32_t steps, const int32_t* record_slot, void* traj,
                  int32_t n_frames, void* workspace, size_t workspace_bytes, void* stream) {
  return integrate_impl(p, batch, state, steps, record_slot, traj, n_frames, workspace, workspace_bytes,
                        (cudaStream_t)stream, nullptr);
}

int fsm_integrate_profiled(const FsmPlan* p, int32_t batch, void* state, int32_t steps, void* workspace,
                           size_t workspace_bytes, void* stream, double* kernel_ms, int64_t* kernel_launches) {
  if (!kernel_ms || !kernel_launches) return set_error(FSM_ERR_INVALID, "profile outputs");
  for (int i = 0; i < 4; ++i) {
    kernel_ms[i] = 0.0;
    kernel_launches[i] = 0;
  }
  LaunchProfile prof;
  prof.st = (cudaStream_t)stream;
  int rc = integrate_impl(p, batch, state, steps, nullptr, nullptr, 0, workspace, workspace_bytes, prof.st, &prof);
  int rc2 = prof.collect(kernel_ms, kernel_launches);
  return rc ? rc : rc2;
}

int fsm_rfftn(const FsmPlan* p, int32_t count, const float* in, void* out, void* stream) {
  if (!p || !in || !out || count < 0) return set_error(FSM_ERR_INVALID, "rfftn arguments");
  if (count == 0) return FSM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int nd = p->ndim;
  const int nl = p->n[nd - 1];
  int64_t rows = (int64_t)count * (p->R / nl);
  int rc = transform_r2c_last(nl, in, (float2*)out, rows, p->tw, st);
  if (rc) return rc;
  // outer axes, innermost first
  int64_t inner = p->h;
  for (int ax = nd - 2; ax >= 0; --ax) {
    int64_t outer = count;
    for (int j = 0; j < ax; ++j) outer *= p->n[j];
    if (outer > 65535) return set_error(FSM_ERR_UNSUPPORTED, "rfftn: too many fields in one call");
    rc = transform_c2c_strided_reg(p->n[ax], false, (float2*)out, outer, inner, p->tw, st);
    if (rc == -1) rc = transform_c2c_strided(p->n[ax], false, (float2*)out, outer, inner, p->tw, st);
    if (rc) return rc;
    inner *= p->n[ax];
  }
  return FSM_OK;
}

int fsm_irfftn(const FsmPlan* p, int32_t count, void* in, float* out, void* stream) {
  if (!p || !in || !out || count < 0) return set_error(FSM_ERR_INVALID, "irfftn arguments");
  if (count == 0) return FSM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int nd = p->ndim;
  int rc;
  int64_t inner = p->h;
  for (int ax = nd - 2; ax >= 0; --ax) {
    int64_t outer = count;
    for (int j = 0; j < ax; ++j) outer *= p->n[j];
    if (outer > 65535) return set_error(FSM_ERR_UNSUPPORTED, "irfftn: too many fields in one call");
    rc = transform_c2c_strided_reg(p->n[ax], true, (float2*)in, outer, inner, p->tw, st);
    if (rc == -1) rc = transform_c2c_strided(p->n[ax], true, (float2*)in, outer, inner, p->tw, st);
    if (rc) return rc;
    inner *= p->n[ax];
  }
  const int nl = p->n[nd - 1];
  const int64_t rows = (int64_t)count * (p->R / nl);
  return transform_c2r_last(nl, (const float2*)in, out, rows, (float)(1.0 / (double)p->R), p->tw, st);
}

int fsm_nonfinite_flags(const FsmPlan* p, int32_t count, const void* fields, int32_t* flags, void* stream) {
  if (!p || !fields || !flags || count < 0) return set_error(FSM_ERR_INVALID, "nonfinite arguments");
  return launch_nonfinite((const float2*)fields, count, p->S, flags, (cudaStream_t)stream);
}

}  // extern "C"
