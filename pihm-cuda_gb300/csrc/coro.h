// Minimal C++20 coroutine task used by the integrator: a lazily started,
// awaitable Task<T> whose completion resumes its awaiter by symmetric
// transfer.  With operations that complete immediately a Task chain runs to
// completion inside the first resume(); with operations that suspend (the
// batch engine) control returns to whoever resumed the innermost coroutine.
#pragma once

#include <coroutine>
#include <exception>
#include <utility>

namespace pihm {

template <class T>
class Task;

namespace detail {

struct FinalAwaiter {
  bool await_ready() const noexcept { return false; }
  template <class P>
  std::coroutine_handle<> await_suspend(std::coroutine_handle<P> h) noexcept {
    auto c = h.promise().continuation;
    return c ? c : std::noop_coroutine();
  }
  void await_resume() const noexcept {}
};

struct PromiseBase {
  std::coroutine_handle<> continuation{};
  std::suspend_always initial_suspend() const noexcept { return {}; }
  FinalAwaiter final_suspend() const noexcept { return {}; }
  void unhandled_exception() { std::terminate(); }
};

}  // namespace detail

template <class T>
class Task {
 public:
  struct promise_type : detail::PromiseBase {
    T value{};
    Task get_return_object() { return Task(std::coroutine_handle<promise_type>::from_promise(*this)); }
    void return_value(T v) { value = std::move(v); }
  };
  explicit Task(std::coroutine_handle<promise_type> h) : h_(h) {}
  Task(Task &&o) noexcept : h_(std::exchange(o.h_, {})) {}
  Task(const Task &) = delete;
  ~Task() {
    if (h_) h_.destroy();
  }
  bool await_ready() const noexcept { return false; }
  std::coroutine_handle<> await_suspend(std::coroutine_handle<> awaiter) noexcept {
    h_.promise().continuation = awaiter;
    return h_;
  }
  T await_resume() { return std::move(h_.promise().value); }
  std::coroutine_handle<promise_type> handle() const { return h_; }
  bool done() const { return h_.done(); }
  T result() { return std::move(h_.promise().value); }

 private:
  std::coroutine_handle<promise_type> h_;
};

template <>
class Task<void> {
 public:
  struct promise_type : detail::PromiseBase {
    Task get_return_object() { return Task(std::coroutine_handle<promise_type>::from_promise(*this)); }
    void return_void() {}
  };
  explicit Task(std::coroutine_handle<promise_type> h) : h_(h) {}
  Task(Task &&o) noexcept : h_(std::exchange(o.h_, {})) {}
  Task(const Task &) = delete;
  ~Task() {
    if (h_) h_.destroy();
  }
  bool await_ready() const noexcept { return false; }
  std::coroutine_handle<> await_suspend(std::coroutine_handle<> awaiter) noexcept {
    h_.promise().continuation = awaiter;
    return h_;
  }
  void await_resume() {}
  std::coroutine_handle<promise_type> handle() const { return h_; }
  bool done() const { return h_.done(); }

 private:
  std::coroutine_handle<promise_type> h_;
};

// An operation that completed when it was issued.
template <class T>
struct Ready {
  T value;
  bool await_ready() const noexcept { return true; }
  void await_suspend(std::coroutine_handle<>) const noexcept {}
  T await_resume() const noexcept { return value; }
};

struct ReadyVoid {
  bool await_ready() const noexcept { return true; }
  void await_suspend(std::coroutine_handle<>) const noexcept {}
  void await_resume() const noexcept {}
};

// Run a task whose operations all complete immediately.
template <class T>
T run_sync(Task<T> t) {
  t.handle().resume();
  return t.result();
}

}  // namespace pihm
