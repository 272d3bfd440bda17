// actors.hpp -- a small actor runtime for the host programs.
//
// The reference drives its GPU phases from CAF actors: an actor_system with a
// scheduler, stateful actors with typed message handlers, `send`, and a
// scoped_actor that blocks in `receive` for replies (src/phases.cpp:713-1077,
// src/gpu.cpp:103-261).  CAF is not available here, so this header provides
// the same shape in plain C++17:
//
//   actor_system sys{threads};
//   auto a = sys.spawn<State>([](actor_ctx<State>& self) {
//     return behavior{handler<int, std::string>([&](int x, std::string s) {...})};
//   });
//   sys.send(a, 42, std::string("x"));          // fire and forget
//   scoped_actor self{sys};
//   self.send(a, ...); self.receive(handler<Reply>(...));  // blocking reply
//
// Messages are std::tuple values carried in std::any with the sender's
// reference; a behavior is a list of handlers tried in order (first whose
// tuple type matches wins).  Each actor processes one message at a time on the
// system's worker threads; an actor's state is touched only by its own
// handlers, so handlers need no locks.
#pragma once

#include <any>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <tuple>
#include <utility>
#include <vector>

namespace wahact {

class actor_system;
struct actor_core;

// A handle to an actor (or to a scoped_actor's mailbox).
class actor {
 public:
  actor() = default;
  explicit actor(std::shared_ptr<actor_core> c) : core_(std::move(c)) {}
  explicit operator bool() const { return static_cast<bool>(core_); }
  actor_core* get() const { return core_.get(); }
  const std::shared_ptr<actor_core>& core() const { return core_; }

 private:
  std::shared_ptr<actor_core> core_;
};

struct envelope {
  actor sender;
  std::any content;
};

// Handler: returns true when it accepted the message.
using handler_fn = std::function<bool(const actor& sender, std::any& content)>;

template <class... Ts, class F>
handler_fn handler(F f) {
  return [f = std::move(f)](const actor&, std::any& c) mutable {
    auto* t = std::any_cast<std::tuple<Ts...>>(&c);
    if (!t) return false;
    std::apply(f, std::move(*t));
    return true;
  };
}

// Like handler, but the callback also gets the sender (to reply).
template <class... Ts, class F>
handler_fn handler_from(F f) {
  return [f = std::move(f)](const actor& from, std::any& c) mutable {
    auto* t = std::any_cast<std::tuple<Ts...>>(&c);
    if (!t) return false;
    std::apply([&](auto&&... xs) { f(from, std::forward<decltype(xs)>(xs)...); }, std::move(*t));
    return true;
  };
}

struct behavior {
  std::vector<handler_fn> handlers;
  behavior() = default;
  behavior(std::initializer_list<handler_fn> hs) : handlers(hs) {}
  bool dispatch(const actor& from, std::any& content) {
    for (auto& h : handlers)
      if (h(from, content)) return true;
    return false;
  }
};

struct actor_core {
  std::mutex mu;
  std::deque<envelope> mailbox;
  bool scheduled = false;  // queued on (or running in) the system
  bool quit = false;
  behavior beh;
  actor_system* sys = nullptr;
  std::function<void()> on_quit;
  // scoped actors: a blocking mailbox instead of a behavior
  bool blocking = false;
  std::condition_variable cv;
};

class actor_system {
 public:
  explicit actor_system(unsigned threads = 0) {
    if (threads == 0) threads = std::max(2u, std::thread::hardware_concurrency() / 2);
    for (unsigned i = 0; i < threads; ++i) workers_.emplace_back([this] { run(); });
  }
  ~actor_system() {
    await_all_actors_done();
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }
  actor_system(const actor_system&) = delete;
  actor_system& operator=(const actor_system&) = delete;

  // Spawns a stateful actor: init(self) builds its behavior.
  template <class State, class Init>
  actor spawn(Init init);

  // Spawns a stateless actor from a behavior.
  actor spawn(behavior b) {
    auto core = std::make_shared<actor_core>();
    core->sys = this;
    core->beh = std::move(b);
    alive_.fetch_add(1);
    return actor(core);
  }

  template <class... Ts>
  void send(const actor& to, Ts&&... xs) {
    send_from(actor(), to, std::forward<Ts>(xs)...);
  }

  template <class... Ts>
  void send_from(const actor& from, const actor& to, Ts&&... xs) {
    enqueue(to, envelope{from, std::any(std::make_tuple(std::forward<Ts>(xs)...))});
  }

  void enqueue(const actor& to, envelope e) {
    actor_core* c = to.get();
    if (!c) return;
    bool schedule = false;
    {
      std::lock_guard<std::mutex> lk(c->mu);
      if (c->quit) return;
      c->mailbox.push_back(std::move(e));
      if (c->blocking) {
        c->cv.notify_all();
        return;
      }
      if (!c->scheduled) {
        c->scheduled = true;
        schedule = true;
      }
    }
    if (schedule) {
      std::lock_guard<std::mutex> lk(mu_);
      ready_.push_back(to.core());
      cv_.notify_one();
    }
  }

  // Ends an actor after its current message; pending messages are dropped.
  // Its behavior (whose handlers hold the actor's context, and through it
  // the actor itself) is released as soon as no handler of it runs.
  void quit(actor_core* c) {
    std::function<void()> cb;
    behavior dead;
    {
      std::lock_guard<std::mutex> lk(c->mu);
      if (c->quit) return;
      c->quit = true;
      c->mailbox.clear();
      cb = std::move(c->on_quit);
      if (!c->scheduled) dead = std::move(c->beh);  // not running nor queued
    }
    if (cb) cb();
    if (alive_.fetch_sub(1) == 1) {
      std::lock_guard<std::mutex> lk(mu_);
      done_cv_.notify_all();
    }
  }

  void await_all_actors_done() {
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [this] { return alive_.load() == 0; });
  }

 private:
  void run() {
    while (true) {
      std::shared_ptr<actor_core> c;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [this] { return stop_ || !ready_.empty(); });
        if (ready_.empty()) return;
        c = std::move(ready_.front());
        ready_.pop_front();
      }
      // one message per turn keeps actors fair
      envelope e;
      {
        behavior dead;
        std::lock_guard<std::mutex> lk(c->mu);
        if (c->mailbox.empty() || c->quit) {
          if (c->quit) dead = std::move(c->beh);
          c->scheduled = false;
          continue;
        }
        e = std::move(c->mailbox.front());
        c->mailbox.pop_front();
      }
      if (!c->beh.dispatch(e.sender, e.content)) {
        // unmatched messages are dropped, as CAF does with unexpected ones
      }
      bool again = false;
      behavior dead;  // a quit actor's behavior, released outside the lock
      {
        std::lock_guard<std::mutex> lk(c->mu);
        if (c->quit) {
          dead = std::move(c->beh);
          c->scheduled = false;
        } else if (!c->mailbox.empty()) {
          again = true;
        } else {
          c->scheduled = false;
        }
      }
      if (again) {
        std::lock_guard<std::mutex> lk(mu_);
        ready_.push_back(std::move(c));
        cv_.notify_one();
      }
    }
  }

  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<std::shared_ptr<actor_core>> ready_;
  std::vector<std::thread> workers_;
  std::atomic<int> alive_{0};
  bool stop_ = false;
};

// Context a stateful actor's handlers use: its state, its handle, send, quit.
template <class State>
class actor_ctx {
 public:
  actor_ctx(actor_system& sys, actor self) : sys_(sys), self_(std::move(self)) {}
  State state{};
  const actor& self() const { return self_; }
  actor_system& system() { return sys_; }
  template <class... Ts>
  void send(const actor& to, Ts&&... xs) {
    sys_.send_from(self_, to, std::forward<Ts>(xs)...);
  }
  void quit() { sys_.quit(self_.get()); }

 private:
  actor_system& sys_;
  actor self_;
};

template <class State, class Init>
actor actor_system::spawn(Init init) {
  auto core = std::make_shared<actor_core>();
  core->sys = this;
  actor a(core);
  // the context lives as long as the actor
  auto ctx = std::make_shared<actor_ctx<State>>(*this, a);
  core->beh = init(*ctx);
  core->beh.handlers.push_back([ctx](const actor&, std::any&) { return false; });
  alive_.fetch_add(1);
  return a;
}

// A blocking actor for the calling thread (CAF's scoped_actor).
class scoped_actor {
 public:
  explicit scoped_actor(actor_system& sys) : sys_(sys), core_(std::make_shared<actor_core>()) {
    core_->sys = &sys;
    core_->blocking = true;
  }
  const actor self() const { return actor(core_); }
  template <class... Ts>
  void send(const actor& to, Ts&&... xs) {
    sys_.send_from(self(), to, std::forward<Ts>(xs)...);
  }
  // Blocks until one message matches one of the handlers; the oldest such
  // message is taken, the others stay in the mailbox in their order.
  template <class... H>
  void receive(H... hs) {
    behavior b{hs...};
    std::unique_lock<std::mutex> lk(core_->mu);
    size_t scanned = 0;  // messages already found not to match
    while (true) {
      while (scanned < core_->mailbox.size()) {
        auto it = core_->mailbox.begin() + static_cast<std::ptrdiff_t>(scanned);
        envelope e = std::move(*it);
        core_->mailbox.erase(it);
        lk.unlock();
        if (b.dispatch(e.sender, e.content)) return;
        lk.lock();
        // not for us: put it back where it was
        core_->mailbox.insert(core_->mailbox.begin() + static_cast<std::ptrdiff_t>(scanned),
                              std::move(e));
        ++scanned;
      }
      core_->cv.wait(lk);
    }
  }

 private:
  actor_system& sys_;
  std::shared_ptr<actor_core> core_;
};

}  // namespace wahact
