/*
 * Runtime part of the host SYCL 1.2.1 subset (see CL/sycl.hpp) -- TEST INFRASTRUCTURE ONLY.
 *
 * Work-item fibers: each OS thread keeps a pool of fibers with their own stacks.  A fiber is
 * entered the first time with setcontext() and afterwards with _setjmp/_longjmp, which do
 * not touch the signal mask (no system call per switch).  A fiber runs work-items in a loop:
 * it runs the item it was given, marks it done and jumps back to the scheduler, which later
 * resumes it with the next group's item.  barrier() saves the fiber and jumps back to the
 * scheduler; the scheduler resumes the items round-robin, so every item reaches barrier k
 * before any item passes it.
 *
 * Must be compiled without _FORTIFY_SOURCE: the checked longjmp rejects jumps between
 * stacks.
 */
#include "CL/sycl.hpp"

#include <cstdio>
#include <setjmp.h>

namespace jxshim {
long long g_group_sample = 1;
long long g_group_residue = 0;
const unsigned char *g_group_mask = nullptr;
long long g_group_mask_len = 0;
}

namespace cl {
namespace sycl {
namespace detail {

thread_local char *tl_local_base = nullptr;

namespace {
constexpr size_t kStack = 64 * 1024;

struct Fiber {
  ucontext_t uc;
  jmp_buf jb;
  std::unique_ptr<char[]> stack;
  size_t index = 0;
  bool started = false;
  bool done = true;
};

struct Pool {
  std::vector<std::unique_ptr<Fiber>> fibers;
  jmp_buf sched;
  Fiber *cur = nullptr;
  const std::function<void(size_t)> *item = nullptr;
  bool barrier_called = false;
  bool in_fiber = false;
};

thread_local Pool tl_pool;

void trampoline() {
  Pool &p = tl_pool;
  for (;;) {
    Fiber *f = p.cur;
    (*p.item)(f->index);
    f->done = true;
    if (_setjmp(f->jb) == 0) _longjmp(p.sched, 1);
  }
}

void switch_to(Fiber *f) {
  Pool &p = tl_pool;
  p.cur = f;
  if (_setjmp(p.sched) == 0) {
    if (!f->started) {
      f->started = true;
      setcontext(&f->uc);
    } else {
      _longjmp(f->jb, 1);
    }
  }
}

Fiber *fiber_at(size_t k) {
  Pool &p = tl_pool;
  while (p.fibers.size() <= k) {
    auto f = std::make_unique<Fiber>();
    f->stack.reset(new char[kStack]);
    if (getcontext(&f->uc) != 0) {
      std::fprintf(stderr, "syclshim: getcontext failed\n");
      std::abort();
    }
    f->uc.uc_stack.ss_sp = f->stack.get();
    f->uc.uc_stack.ss_size = kStack;
    f->uc.uc_link = nullptr;
    makecontext(&f->uc, trampoline, 0);
    p.fibers.push_back(std::move(f));
  }
  return p.fibers[k].get();
}
} // namespace

bool in_fiber() { return tl_pool.in_fiber; }

void barrier_yield() {
  Pool &p = tl_pool;
  if (!p.in_fiber) {
    std::fprintf(stderr, "syclshim: barrier() in a kernel first run without one\n");
    std::abort();
  }
  p.barrier_called = true;
  Fiber *f = p.cur;
  if (_setjmp(f->jb) == 0) _longjmp(p.sched, 1);
}

bool run_group(size_t n_items, const std::function<void(size_t)> &item, bool use_fibers) {
  if (!use_fibers) {
    for (size_t k = 0; k < n_items; ++k) item(k);
    return false;
  }
  Pool &p = tl_pool;
  p.item = &item;
  p.barrier_called = false;
  p.in_fiber = true;
  for (size_t k = 0; k < n_items; ++k) {
    Fiber *f = fiber_at(k);
    f->index = k;
    f->done = false;
  }
  size_t remaining = n_items;
  while (remaining > 0) {
    remaining = 0;
    for (size_t k = 0; k < n_items; ++k) {
      Fiber *f = p.fibers[k].get();
      if (f->done) continue;
      switch_to(f);
      if (!f->done) ++remaining;
    }
  }
  p.in_fiber = false;
  return p.barrier_called;
}

} // namespace detail
} // namespace sycl
} // namespace cl
