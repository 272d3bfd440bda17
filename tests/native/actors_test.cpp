// actors_test -- self-checks of the actor runtime (no GPU involved).
// Exits 0 and prints "actors: all checks passed" when every check holds.
#include <atomic>
#include <cstdio>
#include <string>
#include <vector>

#include "actors.hpp"

using namespace wahact;

namespace {

int failures = 0;
#define CHECK(cond)                                                   \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #cond); \
      ++failures;                                                     \
    }                                                                 \
  } while (0)

struct ping {};
struct pong {};
struct add {};
struct get {};
struct stop {};

struct counter_state {
  uint64_t sum = 0;
  uint64_t messages = 0;
};

// A counter: add(x) accumulates (one message at a time, so no lock), get
// replies with the sum, stop ends it.
behavior counter(actor_ctx<counter_state>& self) {
  auto& s = self.state;
  return {
      handler<add, uint64_t>([&](add, uint64_t x) {
        s.sum += x;
        ++s.messages;
      }),
      handler_from<get>([&](const actor& from, get) { self.send(from, s.sum, s.messages); }),
      handler<stop>([&](stop) { self.quit(); }),
  };
}

struct pinger_state {
  actor peer, done;
  int left = 0;
};

}  // namespace

int main() {
  // 1. request/reply with a scoped actor, typed dispatch
  {
    actor_system sys{4};
    actor c = sys.spawn<counter_state>([](actor_ctx<counter_state>& self) { return counter(self); });
    scoped_actor self{sys};
    for (uint64_t i = 1; i <= 1000; ++i) self.send(c, add{}, i);
    self.send(c, get{});
    uint64_t sum = 0, msgs = 0;
    self.receive(handler<uint64_t, uint64_t>([&](uint64_t s, uint64_t m) {
      sum = s;
      msgs = m;
    }));
    CHECK(sum == 500500);
    CHECK(msgs == 1000);
    self.send(c, stop{});
  }  // the system waits for the counter to quit

  // 2. many senders, one actor: every message processed exactly once
  {
    actor_system sys{8};
    actor c = sys.spawn<counter_state>([](actor_ctx<counter_state>& self) { return counter(self); });
    std::vector<std::thread> ts;
    for (int t = 0; t < 8; ++t)
      ts.emplace_back([&sys, c] {
        for (uint64_t i = 0; i < 10000; ++i) sys.send(c, add{}, uint64_t{1});
      });
    for (auto& t : ts) t.join();
    scoped_actor self{sys};
    self.send(c, get{});
    uint64_t sum = 0;
    self.receive(handler<uint64_t, uint64_t>([&](uint64_t s, uint64_t) { sum = s; }));
    CHECK(sum == 80000);
    self.send(c, stop{});
  }

  // 3. ping-pong between two stateful actors, result to a scoped actor
  {
    actor_system sys{2};
    scoped_actor main_actor{sys};
    actor ponger = sys.spawn(behavior{handler_from<ping, int>([&sys](const actor& from, ping, int k) {
      sys.send(from, pong{}, k);
    })});
    actor pinger = sys.spawn<pinger_state>([&](actor_ctx<pinger_state>& self) {
      auto& s = self.state;
      return behavior{
          handler<actor, actor, int>([&](actor peer, actor done, int rounds) {
            s.peer = peer;
            s.done = done;
            s.left = rounds;
            self.send(s.peer, ping{}, s.left);
          }),
          handler<pong, int>([&](pong, int k) {
            CHECK(k == s.left);
            if (--s.left == 0) {
              self.send(s.done, std::string("finished"));
              self.quit();
            } else {
              self.send(s.peer, ping{}, s.left);
            }
          }),
      };
    });
    sys.send(pinger, ponger, main_actor.self(), 1000);
    std::string got;
    main_actor.receive(handler<std::string>([&](std::string x) { got = x; }));
    CHECK(got == "finished");
    sys.quit(ponger.get());
  }

  // 4. receive keeps messages that match no handler for a later receive,
  //    and FIFO order per sender holds
  {
    actor_system sys{2};
    scoped_actor self{sys};
    sys.send(self.self(), std::string("first"));
    sys.send(self.self(), 7);
    sys.send(self.self(), std::string("second"));
    int x = 0;
    self.receive(handler<int>([&](int v) { x = v; }));
    CHECK(x == 7);
    std::string a, b;
    self.receive(handler<std::string>([&](std::string v) { a = v; }));
    self.receive(handler<std::string>([&](std::string v) { b = v; }));
    CHECK(a == "first");
    CHECK(b == "second");
  }

  // 5. a quit actor drops later messages; await_all_actors_done returns
  {
    actor_system sys{2};
    std::atomic<int> seen{0};
    actor a = sys.spawn(behavior{handler<int>([&](int) { seen.fetch_add(1); })});
    sys.send(a, 1);
    scoped_actor self{sys};
    // let the first message through, then quit
    for (int spin = 0; spin < 1000000 && seen.load() == 0; ++spin) std::this_thread::yield();
    sys.quit(a.get());
    sys.send(a, 2);
    sys.await_all_actors_done();
    CHECK(seen.load() == 1);
  }

  if (failures) {
    std::fprintf(stderr, "actors: %d checks failed\n", failures);
    return 1;
  }
  std::printf("actors: all checks passed\n");
  return 0;
}
