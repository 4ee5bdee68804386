// Slot bookkeeping of the serving engine (fsm_serve.cu). Plain C++ without CUDA, so that the
// admission, accounting and compaction rules compile and run on a host without a GPU.
//
// A pool has `capacity` slots, one per sample of the slot-batched spectral state. Requests wait
// in submission order and are admitted at tick boundaries while the request at the head of the
// queue fits (first come, first served: a large request is not overtaken). An admitted request
// of `batch` samples takes the slots [occupied, occupied + batch). Every tick advances all
// occupied slots by the same number of steps. A request whose steps are done (or that was
// cancelled) leaves, and the highest occupied slots move into the holes it left, so that the
// occupied slots are always [0, occupied) and one launch covers them.
#pragma once

#include <algorithm>
#include <cstdint>
#include <deque>
#include <memory>
#include <unordered_map>
#include <vector>

namespace fsm {

enum ServeStatus : int32_t {
  kServeUnknown = -1,
  kServeWaiting = 0,
  kServeActive = 1,
  kServeDone = 2,       // steps completed, result copied; until reported by a poll
  kServeCancelled = 3,  // transient: cancelled requests are erased when they leave
};

struct ServeRequest {
  int64_t id = 0;
  int32_t batch = 0;
  int32_t steps = 0;
  int32_t remaining = 0;
  double dt = 0.0;
  const void* u0 = nullptr;  // caller's input, read at admission
  void* out = nullptr;       // caller's output, written when the request leaves
  int32_t status = kServeWaiting;
  bool cancel_pending = false;  // active request cancelled while a tick was in flight
  std::vector<int32_t> slots;   // slot of each sample while active
  int32_t tab = -1;             // coefficient-table entry of the request's dt while active
};

struct SlotMove {
  int32_t dst, src;
};

class SlotPool {
 public:
  explicit SlotPool(int32_t capacity) : cap_(capacity), owner_((size_t)(capacity > 0 ? capacity : 0)) {
    // one coefficient-table entry per active request (its samples share its dt): at most one per slot
    for (int32_t e = cap_ - 1; e >= 0; --e) free_tabs_.push_back(e);
  }

  int32_t capacity() const { return cap_; }
  int32_t occupied() const { return occ_; }
  int32_t waiting() const { return (int32_t)queue_.size(); }
  int32_t active_requests() const { return (int32_t)active_.size(); }

  // 0: queued; 1: invalid (duplicate id, batch outside [1, capacity], steps < 1, dt <= 0).
  int submit(int64_t id, int32_t batch, int32_t steps, double dt, const void* u0, void* out) {
    if (batch < 1 || batch > cap_ || steps < 1 || !(dt > 0.0) || reqs_.count(id)) return 1;
    auto r = std::make_unique<ServeRequest>();
    r->id = id;
    r->batch = batch;
    r->steps = steps;
    r->remaining = steps;
    r->dt = dt;
    r->u0 = u0;
    r->out = out;
    queue_.push_back(r.get());
    reqs_.emplace(id, std::move(r));
    return 0;
  }

  // Admit waiting requests in submission order while the head fits into the free slots.
  std::vector<ServeRequest*> admit() {
    std::vector<ServeRequest*> in;
    while (!queue_.empty() && cap_ - occ_ >= queue_.front()->batch) {
      ServeRequest* r = queue_.front();
      queue_.pop_front();
      r->status = kServeActive;
      r->tab = free_tabs_.back();  // never empty here: each active request holds a slot and at most one entry
      free_tabs_.pop_back();
      r->slots.resize((size_t)r->batch);
      for (int32_t i = 0; i < r->batch; ++i) {
        r->slots[(size_t)i] = occ_ + i;
        owner_[(size_t)(occ_ + i)] = Owner{r, i};
      }
      occ_ += r->batch;
      active_.push_back(r);
      in.push_back(r);
    }
    return in;
  }

  // Steps of the next tick: the fewest remaining steps of the active requests, at most `chunk`,
  // and at most `limit` when limit > 0. 0 when no slot is occupied.
  int32_t tick_steps(int32_t chunk, int32_t limit) const {
    if (active_.empty()) return 0;
    int32_t k = chunk;
    for (const ServeRequest* r : active_) k = std::min(k, r->remaining);
    if (limit > 0) k = std::min(k, limit);
    return std::max(k, 1);
  }

  // Account k steps of every active request; returns those whose steps are done (they keep
  // their slots until released).
  std::vector<ServeRequest*> advance(int32_t k) {
    std::vector<ServeRequest*> fin;
    for (ServeRequest* r : active_) {
      r->remaining -= std::min(k, r->remaining);
      if (r->remaining == 0) fin.push_back(r);
    }
    return fin;
  }

  // Active requests cancelled while a tick was in flight.
  std::vector<ServeRequest*> pending_cancels() const {
    std::vector<ServeRequest*> out;
    for (ServeRequest* r : active_)
      if (r->cancel_pending && r->remaining > 0) out.push_back(r);
    return out;
  }

  // Free the slots of the given active requests and return the moves (in order) that refill the
  // holes below the new occupied count from the highest occupied slots. Every dst is a hole and
  // every src lies at or above the new count, so no move reads a slot an earlier move wrote.
  std::vector<SlotMove> release(const std::vector<ServeRequest*>& leaving) {
    for (ServeRequest* r : leaving) {
      for (int32_t s : r->slots) owner_[(size_t)s] = Owner{};
      occ_ -= r->batch;
      r->slots.clear();
      free_tabs_.push_back(r->tab);
      r->tab = -1;
      active_.erase(std::remove(active_.begin(), active_.end(), r), active_.end());
    }
    std::vector<SlotMove> moves;
    int32_t src = cap_ - 1;
    for (int32_t dst = 0; dst < occ_; ++dst) {
      if (owner_[(size_t)dst].req) continue;
      while (src > dst && !owner_[(size_t)src].req) --src;
      // src >= occ_ here: the occupied slots above occ_ match the holes below it one to one
      Owner o = owner_[(size_t)src];
      owner_[(size_t)dst] = o;
      owner_[(size_t)src] = Owner{};
      o.req->slots[(size_t)o.index] = dst;
      moves.push_back(SlotMove{dst, src});
      --src;
    }
    return moves;
  }

  // The table entry of each occupied slot [0, occupied) into out.
  void slot_tables(int32_t* out) const {
    for (int32_t s = 0; s < occ_; ++s) out[s] = owner_[(size_t)s].req ? owner_[(size_t)s].req->tab : 0;
  }

  int32_t free_tables() const { return (int32_t)free_tabs_.size(); }

  ServeRequest* find(int64_t id) const {
    auto it = reqs_.find(id);
    return it == reqs_.end() ? nullptr : it->second.get();
  }

  void erase(int64_t id) {
    ServeRequest* r = find(id);
    if (!r) return;
    queue_.erase(std::remove(queue_.begin(), queue_.end(), r), queue_.end());
    active_.erase(std::remove(active_.begin(), active_.end(), r), active_.end());
    reqs_.erase(id);
  }

  // Remove a waiting request from the queue (true), or false when it is not waiting.
  bool drop_waiting(int64_t id) {
    ServeRequest* r = find(id);
    if (!r || r->status != kServeWaiting) return false;
    erase(id);
    return true;
  }

  // Slot owner (request id, sample index), or id -1 for a free slot.
  void owner(int32_t slot, int64_t* id, int32_t* index) const {
    const Owner& o = owner_[(size_t)slot];
    *id = o.req ? o.req->id : -1;
    *index = o.req ? o.index : -1;
  }

 private:
  struct Owner {
    ServeRequest* req = nullptr;
    int32_t index = 0;
  };
  int32_t cap_;
  int32_t occ_ = 0;
  std::vector<Owner> owner_;
  std::vector<int32_t> free_tabs_;  // coefficient-table entries not held by an active request
  std::deque<ServeRequest*> queue_;
  std::vector<ServeRequest*> active_;  // in admission order
  std::unordered_map<int64_t, std::unique_ptr<ServeRequest>> reqs_;
};

}  // namespace fsm
