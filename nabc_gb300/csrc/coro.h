// The resumable computation behind the reverse-communication routines
// (xmin.cpp, lmod.cpp): a C++20 coroutine that co_yields a request code
// each time it needs the caller to evaluate something, and co_returns a
// status at the end.
#pragma once

#include <coroutine>
#include <exception>

namespace sffg {

struct Gen {
  struct promise_type {
    int request = 0, status = 0;
    Gen get_return_object() { return Gen(std::coroutine_handle<promise_type>::from_promise(*this)); }
    std::suspend_always initial_suspend() noexcept { return {}; }
    std::suspend_always final_suspend() noexcept { return {}; }
    std::suspend_always yield_value(int r) noexcept {
      request = r;
      return {};
    }
    void return_value(int s) noexcept { status = s; }
    void unhandled_exception() { std::terminate(); }
  };
  explicit Gen(std::coroutine_handle<promise_type> h) : h_(h) {}
  Gen(Gen &&o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  Gen(const Gen &) = delete;
  ~Gen() {
    if (h_) h_.destroy();
  }
  // Runs to the next request (true) or to the end (false).
  bool next() {
    h_.resume();
    return !h_.done();
  }
  int request() const { return h_.promise().request; }
  int status() const { return h_.promise().status; }

 private:
  std::coroutine_handle<promise_type> h_;
};

}  // namespace sffg

// Inside a coroutine: passes every request of a sub-computation out and
// stores its status.
#define CORO_RUN(gen, status_out)                           \
  {                                                         \
    ::sffg::Gen sub_ = (gen);                               \
    while (sub_.next()) co_yield sub_.request();            \
    (status_out) = sub_.status();                           \
    (void)(status_out);                                     \
  }
