// Serving engine: a slot pool of one plan advancing many independent solve requests together.
//
// The engine owns no device memory: the caller passes the slot-batched state [capacity][C][S]
// and a workspace for (capacity, chunk). Requests are queued by fsm_serve_submit; each
// fsm_serve_tick admits the waiting requests that fit (their initial spectra are copied into
// their slots and their slots' coefficient tables recomputed for their dt), then launches k steps
// of every occupied slot as one integration. Ticks of at most kGraphMaxSteps steps run as CUDA
// graphs captured per (occupied slots, steps) on the shape's second occurrence, with the step
// count rounded down to a power of two so that few shapes recur. fsm_serve_poll completes the
// tick in flight: requests whose steps are done copy their slots to their output, leave, and the
// remaining slots are compacted (fsm_serve_pool.h).
//
// Samples do not interact in these kernels, so a request's result does not depend on the other
// requests in its ticks. The reference has no serving layer; each request is the solve of
// Operator.integrate (operator/_base.py:676-751) with its own dt.
#include <iterator>
#include <list>
#include <mutex>
#include <unordered_map>
#include <unordered_set>

#include "fsm_internal.cuh"
#include "fsm_serve_pool.h"

namespace {

constexpr int kGraphMaxSteps = 64;
constexpr size_t kGraphCache = 48;

}  // namespace

struct FsmServe {
  FsmPlan* plan = nullptr;
  int32_t capacity = 0;
  int32_t chunk = 0;
  float2* state = nullptr;
  void* ws = nullptr;
  size_t ws_bytes = 0;     // the integration's part of the workspace
  int32_t* d_tabs = nullptr;  // the occupied slots' table entries (end of the workspace)
  std::vector<int32_t> h_tabs;
  int32_t flags = 0;
  double tick_ms = 0.0;
  cudaStream_t st = nullptr;
  int device = 0;
  int64_t sample = 0;  // complex values per sample (C * S)
  fsm::SlotPool pool;
  // tick in flight
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool in_flight = false;
  int32_t tick_k = 0, tick_n = 0;
  double step_ms = 0.0;  // device time per step and slot, running mean over ticks
  // captured ticks, least recently used first
  std::list<std::pair<uint64_t, cudaGraphExec_t>> lru;
  std::unordered_map<uint64_t, std::list<std::pair<uint64_t, cudaGraphExec_t>>::iterator> graphs;
  std::unordered_set<uint64_t> seen;
  std::vector<int64_t> done_ids;  // completed, not yet reported
  FsmServeGroup* group = nullptr;  // ticked by this group (fsm_serve_group_*), not on its own
  int64_t launches = 0, replays = 0, ticks = 0, slot_steps = 0, completed = 0, cancelled = 0;
  std::mutex mu;

  explicit FsmServe(int32_t cap) : pool(cap) {}
};

namespace {

using fsm::cuda_check;
using fsm::set_error;

// Copy `count` samples starting at slot `slot` to (or from) a caller buffer.
int copy_slots(FsmServe* s, int32_t slot, int32_t count, void* other, bool to_slots) {
  const size_t bytes = (size_t)s->sample * count * sizeof(float2);
  float2* slots = s->state + (int64_t)slot * s->sample;
  return cuda_check(to_slots ? cudaMemcpyAsync(slots, other, bytes, cudaMemcpyDeviceToDevice, s->st)
                             : cudaMemcpyAsync(other, slots, bytes, cudaMemcpyDeviceToDevice, s->st),
                    "serve copy");
}

// Copy the samples of a request from its slots to its output, merging runs of adjacent slots.
int copy_out(FsmServe* s, const fsm::ServeRequest* r) {
  const int32_t n = (int32_t)r->slots.size();
  int32_t i = 0;
  while (i < n) {
    int32_t j = i + 1;
    while (j < n && r->slots[(size_t)j] == r->slots[(size_t)(j - 1)] + 1) ++j;
    int rc = copy_slots(s, r->slots[(size_t)i], j - i, (float2*)r->out + (int64_t)i * s->sample, false);
    if (rc) return rc;
    i = j;
  }
  return FSM_OK;
}

// Requests leave: outputs written, slots freed and compacted (state and coefficient tables).
int retire(FsmServe* s, const std::vector<fsm::ServeRequest*>& leaving) {
  if (leaving.empty()) return FSM_OK;
  int rc;
  for (const fsm::ServeRequest* r : leaving)
    if ((rc = copy_out(s, r))) return rc;
  // the slots' table entries follow their requests (slot_tables), so a move copies the state only
  for (const fsm::SlotMove& m : s->pool.release(leaving))
    if ((rc = copy_slots(s, m.dst, 1, s->state + (int64_t)m.src * s->sample, true))) return rc;
  return FSM_OK;
}

void drop_graphs(FsmServe* s) {
  for (auto& e : s->lru) cudaGraphExecDestroy(e.second);
  s->lru.clear();
  s->graphs.clear();
}

// k steps of slots [0, n): a graph replay when the shape has been captured, a capture on its
// second occurrence (the first direct run has set the kernels' attributes), a direct run
// otherwise. Returns the launches the device sees.
int advance(FsmServe* s, int32_t n, int32_t k, int64_t* launches) {
  const bool graphs = (s->flags & FSM_SERVE_GRAPHS) && k <= kGraphMaxSteps;
  int rc;
  if (graphs) {
    const uint64_t key = ((uint64_t)(uint32_t)n << 32) | (uint32_t)k;
    auto it = s->graphs.find(key);
    if (it == s->graphs.end() && s->seen.count(key)) {
      cudaGraph_t g = nullptr;
      if ((rc = cuda_check(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal), "serve capture")))
        return rc;
      const int irc = fsm::integrate_on_workspace(s->plan, n, s->state, k, s->ws, s->ws_bytes, s->st, s->d_tabs);
      const cudaError_t ec = cudaStreamEndCapture(s->st, &g);
      if (irc) {
        if (g) cudaGraphDestroy(g);
        return irc;
      }
      if ((rc = cuda_check(ec, "serve end capture"))) return rc;
      cudaGraphExec_t ex = nullptr;
      rc = cuda_check(cudaGraphInstantiate(&ex, g, 0), "serve graph instantiate");
      cudaGraphDestroy(g);
      if (rc) return rc;
      s->lru.emplace_back(key, ex);
      it = s->graphs.emplace(key, std::prev(s->lru.end())).first;
      while (s->lru.size() > kGraphCache) {
        s->graphs.erase(s->lru.front().first);
        cudaGraphExecDestroy(s->lru.front().second);  // freed once a replay in flight completes
        s->lru.pop_front();
      }
    }
    if (it != s->graphs.end()) {
      s->lru.splice(s->lru.end(), s->lru, it->second);
      if ((rc = cuda_check(cudaGraphLaunch(it->second->second, s->st), "serve graph launch"))) return rc;
      ++s->replays;
      return fsm_plan_launch_count(s->plan, 0, k, launches);
    }
    s->seen.insert(key);
  }
  if ((rc = fsm::integrate_on_workspace(s->plan, n, s->state, k, s->ws, s->ws_bytes, s->st, s->d_tabs))) return rc;
  return fsm_plan_launch_count(s->plan, n, k, launches);
}

// Account a completed tick of k steps: finished requests write their outputs and leave, cancelled
// ones leave, the remaining slots are compacted.
int complete_tick(FsmServe* s) {
  s->in_flight = false;
  std::vector<fsm::ServeRequest*> fin = s->pool.advance(s->tick_k);
  std::vector<fsm::ServeRequest*> cancels = s->pool.pending_cancels();
  std::vector<fsm::ServeRequest*> leaving = fin;
  leaving.insert(leaving.end(), cancels.begin(), cancels.end());
  int rc;
  if ((rc = retire(s, leaving))) return rc;
  for (fsm::ServeRequest* r : fin) {
    r->status = fsm::kServeDone;
    s->done_ids.push_back(r->id);
    ++s->completed;
  }
  for (fsm::ServeRequest* r : cancels) {
    ++s->cancelled;
    s->pool.erase(r->id);
  }
  return FSM_OK;
}

// Complete the tick in flight if the device has finished it (or, with wait, once it has).
// An engine of a group completes its ticks through fsm_serve_group_poll.
int finish_tick(FsmServe* s, bool wait) {
  if (!s->in_flight || s->group) return FSM_OK;
  cudaError_t q = wait ? cudaEventSynchronize(s->e1) : cudaEventQuery(s->e1);
  if (q == cudaErrorNotReady) return FSM_OK;
  int rc;
  if ((rc = cuda_check(q, "serve tick query"))) return rc;
  float ms = 0.f;
  if ((rc = cuda_check(cudaEventElapsedTime(&ms, s->e0, s->e1), "serve tick time"))) return rc;
  const double per = (double)ms / ((double)s->tick_k * s->tick_n);
  s->step_ms = s->step_ms > 0.0 ? 0.5 * (s->step_ms + per) : per;
  return complete_tick(s);
}

// Admit the waiting requests that fit: their spectra copied into their slots, their slots'
// coefficient tables recomputed for their dt.
int admit(FsmServe* s) {
  int rc;
  for (const fsm::ServeRequest* r : s->pool.admit()) {
    if ((rc = copy_slots(s, r->slots.front(), r->batch, const_cast<void*>(r->u0), true))) return rc;
    if ((rc = fsm::set_batch_dt_range(s->plan, r->tab, 1, r->dt, s->st))) return rc;  // its samples share it
  }
  return FSM_OK;
}

// The occupied slots' table entries to the device, before a tick's launches (outside any capture:
// the captured ticks read them from d_tabs when they replay).
int upload_tables(FsmServe* s) {
  const int32_t n = s->pool.occupied();
  if (n == 0) return FSM_OK;
  s->pool.slot_tables(s->h_tabs.data());
  return cuda_check(cudaMemcpyAsync(s->d_tabs, s->h_tabs.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice,
                                    s->st),
                    "serve table entries");
}

// Round a graph-replayed tick's step count down to a power of two.
int32_t graph_steps(int32_t flags, int32_t k) {
  if ((flags & FSM_SERVE_GRAPHS) && k <= kGraphMaxSteps) {
    int32_t p2 = 1;
    while (p2 * 2 <= k) p2 *= 2;
    return p2;
  }
  return k;
}

// The engine's workspace: the integration's workspace for (capacity, chunk), then the slots'
// table entries (capacity int32, 256-byte aligned).
int serve_layout(const FsmPlan* plan, int32_t capacity, int32_t chunk, size_t* tabs_off, size_t* total) {
  size_t integ = 0;
  int rc = fsm_plan_workspace_bytes(plan, capacity, chunk, &integ);
  if (rc) return rc;
  *tabs_off = (integ + 255) & ~(size_t)255;
  *total = *tabs_off + (size_t)capacity * sizeof(int32_t);
  return FSM_OK;
}

}  // namespace

extern "C" {

int fsm_serve_workspace_bytes(const FsmPlan* plan, int32_t capacity, int32_t chunk, size_t* bytes) {
  if (!plan || !bytes || capacity < 1 || chunk < 1) return set_error(FSM_ERR_INVALID, "serve_workspace_bytes arguments");
  size_t off = 0;
  return serve_layout(plan, capacity, chunk, &off, bytes);
}

int fsm_serve_create(FsmPlan* plan, int32_t capacity, int32_t chunk, void* state, void* workspace,
                     size_t workspace_bytes, int32_t flags, double tick_ms, void* stream, FsmServe** out) {
  if (!plan || !out || capacity < 1 || chunk < 1 || !state || !workspace || tick_ms < 0.0)
    return set_error(FSM_ERR_INVALID, "serve_create arguments");
  if (plan->lin_batch < capacity || plan->lin_batch < 2)
    return set_error(FSM_ERR_INVALID, "serve_create: the plan needs table_batch >= capacity (and >= 2)");
  if (plan->source && plan->src_batch > 1)
    return set_error(FSM_ERR_UNSUPPORTED, "serve_create: per-sample sources are not served");
  if (plan->nl == FSM_NL_KS && (plan->flags & FSM_FLAG_REMOVE_MEAN))
    return set_error(FSM_ERR_UNSUPPORTED, "serve_create: the batch-wide mean couples the samples");
  size_t need = 0, tabs_off = 0;
  int rc = serve_layout(plan, capacity, chunk, &tabs_off, &need);
  if (rc) return rc;
  if (workspace_bytes < need)
    return set_error(FSM_ERR_INVALID, "serve_create: workspace too small: need " + std::to_string(need) +
                                          " bytes (fsm_serve_workspace_bytes)");
  FsmServe* s = new FsmServe(capacity);
  s->plan = plan;
  s->capacity = capacity;
  s->chunk = chunk;
  s->state = (float2*)state;
  s->ws = workspace;
  s->ws_bytes = tabs_off;
  s->d_tabs = (int32_t*)((char*)workspace + tabs_off);
  s->h_tabs.assign((size_t)capacity, 0);
  s->flags = flags;
  s->tick_ms = tick_ms;
  s->st = (cudaStream_t)stream;
  s->sample = (int64_t)plan->C * plan->S;
  if ((rc = cuda_check(cudaGetDevice(&s->device), "serve device")) ||
      (rc = cuda_check(cudaEventCreate(&s->e0), "serve event")) ||
      (rc = cuda_check(cudaEventCreate(&s->e1), "serve event"))) {
    if (s->e0) cudaEventDestroy(s->e0);
    delete s;
    return rc;
  }
  *out = s;
  return FSM_OK;
}

int fsm_serve_submit(FsmServe* s, int64_t request_id, int32_t batch, int32_t steps, double dt, const void* u0,
                     void* out) {
  if (!s || !u0 || !out) return set_error(FSM_ERR_INVALID, "serve_submit arguments");
  std::lock_guard<std::mutex> g(s->mu);
  if (s->pool.submit(request_id, batch, steps, dt, u0, out))
    return set_error(FSM_ERR_INVALID, "serve_submit: duplicate id, batch outside [1, capacity], steps < 1 or dt <= 0");
  return FSM_OK;
}

int fsm_serve_tick(FsmServe* s, int32_t* steps_launched) {
  if (!s) return set_error(FSM_ERR_INVALID, "serve_tick arguments");
  std::lock_guard<std::mutex> g(s->mu);
  if (steps_launched) *steps_launched = 0;
  if (s->group) return set_error(FSM_ERR_INVALID, "serve_tick: the engine belongs to a group (fsm_serve_group_tick)");
  if (s->in_flight) return FSM_OK;
  int rc;
  if ((rc = admit(s))) return rc;
  const int32_t n = s->pool.occupied();
  if (n == 0) return FSM_OK;
  int32_t limit = 0;
  if (s->step_ms > 0.0 && s->tick_ms > 0.0)
    limit = (int32_t)std::max(1.0, std::min(1e9, s->tick_ms / (s->step_ms * n)));
  const int32_t k = graph_steps(s->flags, s->pool.tick_steps(s->chunk, limit));
  if ((rc = upload_tables(s))) return rc;
  if ((rc = cuda_check(cudaEventRecord(s->e0, s->st), "serve tick event"))) return rc;
  int64_t launched = 0;
  if ((rc = advance(s, n, k, &launched))) return rc;
  if ((rc = cuda_check(cudaEventRecord(s->e1, s->st), "serve tick event"))) return rc;
  s->in_flight = true;
  s->tick_k = k;
  s->tick_n = n;
  s->launches += launched;
  s->slot_steps += (int64_t)k * n;
  ++s->ticks;
  if (steps_launched) *steps_launched = k;
  return FSM_OK;
}

int fsm_serve_poll(FsmServe* s, int32_t wait, int64_t* done_ids, int32_t max_ids, int32_t* n_done,
                   int32_t* in_flight) {
  if (!s || max_ids < 0 || (max_ids > 0 && !done_ids)) return set_error(FSM_ERR_INVALID, "serve_poll arguments");
  std::lock_guard<std::mutex> g(s->mu);
  int rc = finish_tick(s, wait != 0);
  if (rc) return rc;
  const int32_t n = (int32_t)std::min<size_t>((size_t)max_ids, s->done_ids.size());
  for (int32_t i = 0; i < n; ++i) {
    done_ids[i] = s->done_ids[(size_t)i];
    s->pool.erase(done_ids[i]);
  }
  s->done_ids.erase(s->done_ids.begin(), s->done_ids.begin() + n);
  if (n_done) *n_done = n;
  if (in_flight) *in_flight = s->in_flight ? 1 : 0;
  return FSM_OK;
}

int fsm_serve_cancel(FsmServe* s, int64_t request_id) {
  if (!s) return set_error(FSM_ERR_INVALID, "serve_cancel arguments");
  std::lock_guard<std::mutex> g(s->mu);
  fsm::ServeRequest* r = s->pool.find(request_id);
  if (!r || r->status == fsm::kServeDone) return set_error(FSM_ERR_INVALID, "serve_cancel: no such pending request");
  if (s->pool.drop_waiting(request_id)) {
    ++s->cancelled;
    return FSM_OK;
  }
  if (s->in_flight) {  // leaves when the tick completes
    r->cancel_pending = true;
    return FSM_OK;
  }
  int rc = retire(s, {r});
  if (rc) return rc;
  ++s->cancelled;
  s->pool.erase(request_id);
  return FSM_OK;
}

int fsm_serve_request_status(FsmServe* s, int64_t request_id, int32_t* status, int32_t* remaining) {
  if (!s || !status) return set_error(FSM_ERR_INVALID, "serve_request_status arguments");
  std::lock_guard<std::mutex> g(s->mu);
  const fsm::ServeRequest* r = s->pool.find(request_id);
  *status = r ? r->status : fsm::kServeUnknown;
  if (remaining) *remaining = r ? r->remaining : 0;
  return FSM_OK;
}

int fsm_serve_stats(FsmServe* s, int64_t* stats, int32_t n) {
  if (!s || !stats || n < 0) return set_error(FSM_ERR_INVALID, "serve_stats arguments");
  std::lock_guard<std::mutex> g(s->mu);
  const int64_t v[FSM_SERVE_NSTATS] = {s->pool.occupied(), s->pool.waiting(), s->pool.active_requests(),
                                       s->in_flight ? 1 : 0, s->ticks, s->launches, s->replays, s->slot_steps,
                                       s->completed, s->cancelled};
  for (int32_t i = 0; i < n && i < FSM_SERVE_NSTATS; ++i) stats[i] = v[i];
  return FSM_OK;
}

int fsm_serve_destroy(FsmServe* s) {
  if (!s) return FSM_OK;
  if (s->group) return set_error(FSM_ERR_INVALID, "serve_destroy: destroy the engine's group first");
  int rc;
  {
    std::lock_guard<std::mutex> g(s->mu);
    rc = cuda_check(cudaStreamSynchronize(s->st), "serve destroy");
    drop_graphs(s);
    cudaEventDestroy(s->e0);
    cudaEventDestroy(s->e1);
  }
  delete s;
  return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Groups: engines of different grid sizes (and PDEs) ticked together on one stream. A group tick
// admits into every member, advances every occupied slot of every member by the same k steps and
// completes them together. Members whose plans are 1D lines of one nonlinear kind advance in ONE
// launch (k_line_multi: a per-CTA table of (plan, first sample)); other members are launched one
// after the other in the same tick (lockstep). Requests are still submitted to, polled from and
// cancelled at the member engines.
// ---------------------------------------------------------------------------
struct FsmServeGroup {
  std::vector<FsmServe*> m;
  std::vector<int32_t> tick_n;  // occupied slots of each member in the tick in flight
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool in_flight = false;
  bool line = false;   // every member a 1D line plan of one kind: one launch per tick
  bool plane = false;  // every member a square 2D register-pass plan of one kind: one launch per pass
  int kind = 0;
  int32_t chunk = 0, tick_k = 0;
  double tick_ms = 0.0;
  double slot_step_ms = 0.0;  // device time per step and occupied slot, running mean over ticks
  int64_t ticks = 0, launches = 0;
  std::mutex mu;
};

namespace {

bool line_member(const FsmServe* s) {
  const FsmPlan* p = s->plan;
  return p->path == 1 && p->n[0] >= 256 && p->n[0] <= 4096 &&
         (p->nl == FSM_NL_KS || p->nl == FSM_NL_CONVECTION);
}

bool plane_member(const FsmServe* s) {
  const FsmPlan* p = s->plan;
  const int n = p->n[0];
  return p->path == 2 && p->ndim == 2 && p->n[1] == n && (n == 64 || n == 128 || n == 256) &&
         (p->nl == FSM_NL_CONVECTION || p->nl == FSM_NL_VORTICITY) && p->integ == FSM_SETDRK4 &&
         (p->hk == n / 3 + 1 || p->hk == n / 2 + 1);
}

// k SETDRK4 steps of the occupied slots of every member: a priming column pass, then per stage
// one row pass and one column pass, each a single launch over all members (fsm_plane_multi.cu).
int plane_tick(FsmServeGroup* g, int32_t k, int64_t* launched) {
  fsm::PlaneMulti pm;
  memset(&pm, 0, sizeof(pm));
  int rc;
  for (FsmServe* s : g->m) {
    const int32_t n = s->pool.occupied();
    if (n == 0) continue;
    if ((rc = fsm::plane_args(s->plan, s->state, n, k, s->ws, s->ws_bytes, &pm.a[pm.count]))) return rc;
    pm.a[pm.count].tab_entry = s->d_tabs;
    pm.n[pm.count] = s->plan->n[0];
    ++pm.count;
  }
  for (int j = 0; j < pm.count; ++j) {
    pm.a[j].stage = -1;
    pm.a[j].emit = 1;
  }
  if ((rc = fsm::launch_plane_col_multi(pm, g->kind, false, g->st))) return rc;
  *launched = 1;
  const int ns = g->m[0]->plan->nstages;
  for (int32_t step = 0; step < k; ++step) {
    for (int st = 0; st < ns; ++st) {
      if ((rc = fsm::launch_plane_row_multi(pm, g->kind, g->st))) return rc;
      for (int j = 0; j < pm.count; ++j) {
        pm.a[j].stage = st;
        pm.a[j].emit = !(st == ns - 1 && step == k - 1);
      }
      if ((rc = fsm::launch_plane_col_multi(pm, g->kind, true, g->st))) return rc;
      *launched += 2;
    }
  }
  return FSM_OK;
}

// Lock every member of the group, in member order (the only place that holds several).
struct MemberLocks {
  std::vector<std::unique_lock<std::mutex>> held;
  explicit MemberLocks(FsmServeGroup* g) {
    for (FsmServe* s : g->m) held.emplace_back(s->mu);
  }
};

}  // namespace

extern "C" {

int fsm_serve_group_create(FsmServe* const* engines, int32_t count, double tick_ms, FsmServeGroup** out) {
  if (!engines || !out || count < 1 || count > fsm::kLineMultiMax || tick_ms < 0.0)
    return set_error(FSM_ERR_INVALID, "serve_group_create arguments (1 to 8 engines)");
  for (int32_t i = 0; i < count; ++i) {
    if (!engines[i] || engines[i]->group) return set_error(FSM_ERR_INVALID, "serve_group_create: engine missing or grouped");
    for (int32_t j = 0; j < i; ++j)
      if (engines[j] == engines[i]) return set_error(FSM_ERR_INVALID, "serve_group_create: engine listed twice");
    if (engines[i]->st != engines[0]->st || engines[i]->device != engines[0]->device)
      return set_error(FSM_ERR_INVALID, "serve_group_create: the engines must share one stream");
    if (engines[i]->in_flight) return set_error(FSM_ERR_INVALID, "serve_group_create: an engine has a tick in flight");
  }
  FsmServeGroup* g = new FsmServeGroup();
  g->m.assign(engines, engines + count);
  g->tick_n.assign((size_t)count, 0);
  g->st = engines[0]->st;
  g->tick_ms = tick_ms;
  g->chunk = engines[0]->chunk;
  g->line = true;
  g->plane = true;
  g->kind = engines[0]->plan->nl;
  for (FsmServe* s : g->m) {
    g->chunk = std::min(g->chunk, s->chunk);
    g->line = g->line && line_member(s) && s->plan->nl == g->kind;
    g->plane = g->plane && plane_member(s) && s->plan->nl == g->kind;
  }
  int rc;
  if ((rc = cuda_check(cudaEventCreate(&g->e0), "serve group event")) ||
      (rc = cuda_check(cudaEventCreate(&g->e1), "serve group event"))) {
    if (g->e0) cudaEventDestroy(g->e0);
    delete g;
    return rc;
  }
  for (FsmServe* s : g->m) {
    std::lock_guard<std::mutex> l(s->mu);
    s->group = g;
  }
  *out = g;
  return FSM_OK;
}

int fsm_serve_group_tick(FsmServeGroup* g, int32_t* steps_launched) {
  if (!g) return set_error(FSM_ERR_INVALID, "serve_group_tick arguments");
  std::lock_guard<std::mutex> gl(g->mu);
  MemberLocks locks(g);
  if (steps_launched) *steps_launched = 0;
  if (g->in_flight) return FSM_OK;
  int rc;
  int64_t total = 0;
  for (FsmServe* s : g->m) {
    if ((rc = admit(s))) return rc;
    if ((rc = upload_tables(s))) return rc;
    total += s->pool.occupied();
  }
  if (total == 0) return FSM_OK;
  int32_t limit = 0;
  if (g->slot_step_ms > 0.0 && g->tick_ms > 0.0)
    limit = (int32_t)std::max(1.0, std::min(1e9, g->tick_ms / (g->slot_step_ms * (double)total)));
  int32_t k = g->chunk;
  for (FsmServe* s : g->m)
    if (s->pool.occupied() > 0) k = std::min(k, s->pool.tick_steps(g->chunk, limit));
  if ((rc = cuda_check(cudaEventRecord(g->e0, g->st), "serve group event"))) return rc;
  int64_t launched = 0;
  if (g->line) {
    fsm::LineMulti lm;
    memset(&lm, 0, sizeof(lm));
    for (FsmServe* s : g->m) {
      const int32_t n = s->pool.occupied();
      if (n == 0) continue;
      lm.a[lm.count] = fsm::base_args(s->plan, s->state, n, k);
      lm.a[lm.count].tab_entry = s->d_tabs;
      lm.n[lm.count] = s->plan->n[0];
      ++lm.count;
    }
    if ((rc = fsm::launch_line_multi(lm, g->kind, g->st))) return rc;
    launched = 1;
  } else if (g->plane) {
    if ((rc = plane_tick(g, k, &launched))) return rc;
  } else {
    k = graph_steps(g->m[0]->flags, k);
    for (FsmServe* s : g->m) {
      const int32_t n = s->pool.occupied();
      if (n == 0) continue;
      int64_t l = 0;
      if ((rc = advance(s, n, k, &l))) return rc;
      launched += l;
    }
  }
  if ((rc = cuda_check(cudaEventRecord(g->e1, g->st), "serve group event"))) return rc;
  for (size_t i = 0; i < g->m.size(); ++i) {
    FsmServe* s = g->m[i];
    const int32_t n = s->pool.occupied();
    g->tick_n[i] = n;
    if (n == 0) continue;
    s->in_flight = true;
    s->tick_k = k;
    s->tick_n = n;
    s->slot_steps += (int64_t)k * n;
    ++s->ticks;
  }
  g->in_flight = true;
  g->tick_k = k;
  g->launches += launched;
  ++g->ticks;
  if (steps_launched) *steps_launched = k;
  return FSM_OK;
}

int fsm_serve_group_poll(FsmServeGroup* g, int32_t wait, int32_t* in_flight) {
  if (!g) return set_error(FSM_ERR_INVALID, "serve_group_poll arguments");
  std::lock_guard<std::mutex> gl(g->mu);
  if (in_flight) *in_flight = g->in_flight ? 1 : 0;
  if (!g->in_flight) return FSM_OK;
  cudaError_t q = wait ? cudaEventSynchronize(g->e1) : cudaEventQuery(g->e1);
  if (q == cudaErrorNotReady) return FSM_OK;
  int rc;
  if ((rc = cuda_check(q, "serve group query"))) return rc;
  float ms = 0.f;
  if ((rc = cuda_check(cudaEventElapsedTime(&ms, g->e0, g->e1), "serve group time"))) return rc;
  int64_t total = 0;
  for (int32_t n : g->tick_n) total += n;
  const double per = (double)ms / ((double)g->tick_k * (double)std::max<int64_t>(1, total));
  g->slot_step_ms = g->slot_step_ms > 0.0 ? 0.5 * (g->slot_step_ms + per) : per;
  MemberLocks locks(g);
  g->in_flight = false;
  for (size_t i = 0; i < g->m.size(); ++i) {
    if (g->tick_n[i] == 0) continue;
    if ((rc = complete_tick(g->m[i]))) return rc;
  }
  if (in_flight) *in_flight = 0;
  return FSM_OK;
}

int fsm_serve_group_stats(FsmServeGroup* g, int64_t* stats, int32_t n) {
  if (!g || !stats || n < 0) return set_error(FSM_ERR_INVALID, "serve_group_stats arguments");
  std::lock_guard<std::mutex> gl(g->mu);
  const int64_t v[FSM_SERVE_GROUP_NSTATS] = {g->ticks, g->launches, g->in_flight ? 1 : 0, g->line ? 1 : 0,
                                            g->plane ? 1 : 0};
  for (int32_t i = 0; i < n && i < FSM_SERVE_GROUP_NSTATS; ++i) stats[i] = v[i];
  return FSM_OK;
}

int fsm_serve_group_destroy(FsmServeGroup* g) {
  if (!g) return FSM_OK;
  int rc;
  {
    std::lock_guard<std::mutex> gl(g->mu);
    rc = cuda_check(cudaStreamSynchronize(g->st), "serve group destroy");
    MemberLocks locks(g);
    if (g->in_flight && !rc) {
      // the device has finished the tick: account it, so that the members stay consistent
      for (size_t i = 0; i < g->m.size() && !rc; ++i)
        if (g->tick_n[i] > 0) rc = complete_tick(g->m[i]);
      g->in_flight = false;
    }
    for (FsmServe* s : g->m) s->group = nullptr;
    cudaEventDestroy(g->e0);
    cudaEventDestroy(g->e1);
  }
  delete g;
  return rc;
}

}  // extern "C"
