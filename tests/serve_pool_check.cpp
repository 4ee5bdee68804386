// Randomised check of the serving engine's slot bookkeeping (torchfsm_gb300/csrc/fsm_serve_pool.h),
// run by tests/test_serve_pool.py. A stand-in for the device state holds, per slot, the tag
// (request id, sample index, steps advanced) of the sample it carries; ticks advance every
// occupied slot, leaving requests copy their slots to their own output, and the pool's moves
// are applied as the engine applies them. Checks: occupied slots are always [0, occupied),
// admission follows submission order without overtaking, every output receives its own
// samples in order with exactly the requested steps, cancelled requests leave at the next
// boundary with the steps they reached, every active request holds one coefficient-table entry
// of its own that all its slots map to. Prints "ok" and exits 0, or names the failure.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <vector>

#include "fsm_serve_pool.h"

struct Tag {
  int64_t id = -1;
  int32_t index = -1;
  int32_t steps = 0;
};

#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      std::printf("FAIL line %d: ", __LINE__); \
      std::printf(__VA_ARGS__);          \
      std::printf("\n");                 \
      std::exit(1);                      \
    }                                    \
  } while (0)

int main(int argc, char** argv) {
  const unsigned seed = argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u;
  std::mt19937 rng(seed);
  for (int trial = 0; trial < 200; ++trial) {
    const int32_t cap = 1 + (int32_t)(rng() % 40);
    const int32_t chunk = 1 + (int32_t)(rng() % 20);
    fsm::SlotPool pool(cap);
    std::vector<Tag> slots((size_t)cap);
    std::map<int64_t, std::vector<Tag>> outputs;  // written when a request leaves
    std::map<int64_t, int32_t> wanted;            // steps requested
    std::map<int64_t, bool> cancelled;
    std::vector<int64_t> order;                   // submission order
    std::vector<int64_t> admitted_order;
    int64_t next_id = 0;
    int leaving_total = 0;
    // rejections
    CHECK(pool.submit(999999, cap + 1, 5, 0.1, &slots, &slots) == 1, "batch above capacity accepted");
    CHECK(pool.submit(999998, 1, 0, 0.1, &slots, &slots) == 1, "zero steps accepted");
    CHECK(pool.submit(999997, 1, 3, 0.0, &slots, &slots) == 1, "dt 0 accepted");
    for (int tick = 0; tick < 300; ++tick) {
      // arrivals
      const int arrivals = (int)(rng() % 3);
      for (int a = 0; a < arrivals; ++a) {
        const int32_t batch = 1 + (int32_t)(rng() % cap);
        const int32_t steps = 1 + (int32_t)(rng() % 60);
        const int64_t id = next_id++;
        CHECK(pool.submit(id, batch, steps, 0.01, &slots, &slots) == 0, "submit refused");
        CHECK(pool.submit(id, 1, 1, 0.01, &slots, &slots) == 1, "duplicate id accepted");
        wanted[id] = steps;
        order.push_back(id);
      }
      // occasionally cancel a random pending request
      if (!order.empty() && rng() % 7 == 0) {
        const int64_t id = order[rng() % order.size()];
        fsm::ServeRequest* r = pool.find(id);
        if (r && r->status == fsm::kServeWaiting) {
          CHECK(pool.drop_waiting(id), "drop_waiting failed");
          cancelled[id] = true;
        } else if (r && r->status == fsm::kServeActive) {
          r->cancel_pending = true;  // leaves at the next tick boundary
        }
      }
      // admission at the tick boundary
      for (fsm::ServeRequest* r : pool.admit()) {
        admitted_order.push_back(r->id);
        for (int32_t i = 0; i < r->batch; ++i) {
          const int32_t s = r->slots[(size_t)i];
          CHECK(slots[(size_t)s].id == -1, "admitted into an occupied slot %d", s);
          slots[(size_t)s] = Tag{r->id, i, 0};
        }
      }
      const int32_t occ = pool.occupied();
      for (int32_t s = 0; s < cap; ++s)
        CHECK((slots[(size_t)s].id != -1) == (s < occ), "slot %d occupancy does not match [0, %d)", s, occ);
      if (occ == 0) continue;
      const int32_t limit = (rng() % 3 == 0) ? 1 + (int32_t)(rng() % 8) : 0;
      const int32_t k = pool.tick_steps(chunk, limit);
      CHECK(k >= 1 && k <= chunk && (limit == 0 || k <= limit), "tick of %d steps", k);
      for (int32_t s = 0; s < occ; ++s) slots[(size_t)s].steps += k;  // the device advances [0, occ)
      std::vector<fsm::ServeRequest*> fin = pool.advance(k);
      std::vector<fsm::ServeRequest*> cancels = pool.pending_cancels();
      std::vector<fsm::ServeRequest*> leaving = fin;
      leaving.insert(leaving.end(), cancels.begin(), cancels.end());
      for (fsm::ServeRequest* r : leaving) {
        std::vector<Tag> out;
        for (int32_t s : r->slots) out.push_back(slots[(size_t)s]);
        outputs[r->id] = out;
        for (int32_t s : r->slots) slots[(size_t)s] = Tag{};
      }
      std::vector<fsm::SlotMove> moves = pool.release(leaving);
      const int32_t occ2 = pool.occupied();
      for (const fsm::SlotMove& m : moves) {
        CHECK(m.dst < occ2 && m.src >= occ2, "move %d <- %d with %d occupied", m.dst, m.src, occ2);
        CHECK(slots[(size_t)m.dst].id == -1 && slots[(size_t)m.src].id != -1, "move between wrong slots");
        slots[(size_t)m.dst] = slots[(size_t)m.src];
        slots[(size_t)m.src] = Tag{};
      }
      for (fsm::ServeRequest* r : fin) pool.erase(r->id);
      for (fsm::ServeRequest* r : cancels) {
        cancelled[r->id] = true;
        pool.erase(r->id);
      }
      leaving_total += (int)leaving.size();
      for (int32_t s = 0; s < cap; ++s)
        CHECK((slots[(size_t)s].id != -1) == (s < occ2), "after compaction slot %d vs %d occupied", s, occ2);
      // every remaining active request's slots carry its own samples, and map to its table entry
      std::vector<int32_t> tabs((size_t)cap, -1);
      pool.slot_tables(tabs.data());
      std::map<int32_t, int64_t> entry_owner;
      for (int32_t s = 0; s < occ2; ++s) {
        int64_t id;
        int32_t index;
        pool.owner(s, &id, &index);
        CHECK(id == slots[(size_t)s].id && index == slots[(size_t)s].index, "slot %d owner mismatch", s);
        fsm::ServeRequest* r = pool.find(id);
        CHECK(r && r->slots[(size_t)index] == s, "request %lld does not list slot %d", (long long)id, s);
        CHECK(r->tab >= 0 && r->tab < cap && tabs[(size_t)s] == r->tab, "slot %d table entry %d, request's %d", s,
              tabs[(size_t)s], r->tab);
        auto e = entry_owner.emplace(r->tab, id);
        CHECK(e.first->second == id, "table entry %d held by requests %lld and %lld", r->tab,
              (long long)e.first->second, (long long)id);
      }
      CHECK((int32_t)entry_owner.size() + pool.free_tables() == cap, "table entries: %zu held + %d free != %d",
            entry_owner.size(), pool.free_tables(), cap);
    }
    // outputs: own samples, in order, with the requested steps (or fewer when cancelled)
    for (const auto& kv : outputs) {
      const int64_t id = kv.first;
      const std::vector<Tag>& out = kv.second;
      for (size_t i = 0; i < out.size(); ++i) {
        CHECK(out[i].id == id && out[i].index == (int32_t)i, "request %lld got sample (%lld, %d) at %zu",
              (long long)id, (long long)out[i].id, out[i].index, i);
        if (cancelled.count(id))
          CHECK(out[i].steps <= wanted[id], "cancelled request %lld ran %d of %d steps", (long long)id,
                out[i].steps, wanted[id]);
        else
          CHECK(out[i].steps == wanted[id], "request %lld ran %d of %d steps", (long long)id, out[i].steps,
                wanted[id]);
      }
    }
    // admission follows submission order (cancelled waiting requests are skipped)
    std::vector<int64_t> expect;
    for (int64_t id : order)
      if (!(cancelled.count(id) && !outputs.count(id))) expect.push_back(id);
    for (size_t i = 0; i < admitted_order.size(); ++i)
      CHECK(i < expect.size() && admitted_order[i] == expect[i], "admission %zu out of order", i);
    CHECK(leaving_total == (int)outputs.size(), "leaving count");
  }
  std::printf("ok\n");
  return 0;
}
