/*
 * Host-only subset of SYCL 1.2.1 -- TEST INFRASTRUCTURE ONLY.
 *
 * Just enough of the SYCL 1.2.1 interface to compile the reference's `jaccard.cpp`
 * (vtsynergy/SYCL-Jaccard) unmodified and run its kernels on the host cores, so the CPU
 * oracle can be checked against the reference itself and the reference can be timed as a
 * CPU baseline.  It is written for that one purpose; it is not a general SYCL runtime.
 *
 * Execution model:
 *   - `queue::submit` runs the command group immediately and synchronously (in order).
 *   - An nd_range launch runs its work-groups in parallel on OpenMP threads.  The
 *     work-items of one group run one after another in linear-id order (dimension N-1
 *     fastest), on the thread that owns the group, which is how a CPU SYCL device without
 *     vectorisation executes them.
 *   - Work-items that call `nd_item::barrier()` run as fibers: each item runs until the
 *     barrier, then the next item runs, and the group continues past the barrier once every
 *     item has reached it.  Whether a kernel needs fibers is found out on the first group of
 *     each launch; barrier-free kernels then run as plain loops.
 *   - Buffers wrap host memory directly; accessors are raw pointers.  Local memory is a
 *     per-thread arena rebased for each work-group.
 *   - `atomic<uint32_t|uint64_t>` maps onto GCC atomic builtins.
 *
 * Sampling hooks (for a bounded CPU baseline): `jxshim::set_group_sample(K, r)` makes every
 * nd_range launch execute only the work-groups whose linear group id g has g % K == r;
 * `jxshim::set_group_mask(mask, len)` only those with g < len and mask[g] != 0.
 */
#ifndef JX_SYCLSHIM_SYCL_HPP
#define JX_SYCLSHIM_SYCL_HPP

#include <chrono>
#include <csetjmp>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <functional>
#include <memory>
#include <string>
#include <type_traits>
#include <ucontext.h>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef SYCL_EXTERNAL
#define SYCL_EXTERNAL
#endif

namespace jxshim {
/* Group sampling: run only work-groups whose linear id g has g % stride == residue.
 * stride 1 = run every work-group.  Defined in syclshim.cpp. */
extern long long g_group_sample;
extern long long g_group_residue;
extern const unsigned char *g_group_mask; /* when set, overrides the stride */
extern long long g_group_mask_len;
inline void set_group_sample(long long k, long long residue = 0) {
  g_group_sample = k > 0 ? k : 1;
  g_group_residue = residue;
}
inline void set_group_mask(const unsigned char *mask, long long len) {
  g_group_mask = len > 0 ? mask : nullptr;
  g_group_mask_len = mask ? len : 0;
}
inline bool group_selected(long long g) {
  if (g_group_mask) return g < g_group_mask_len && g_group_mask[g] != 0;
  return g % g_group_sample == g_group_residue;
}
} // namespace jxshim

namespace cl {
namespace sycl {

namespace access {
enum class mode { read, write, read_write, discard_write, discard_read_write, atomic };
enum class target { global_buffer, constant_buffer, local, host_buffer };
enum class fence_space { local_space, global_space, global_and_local };
} // namespace access

namespace info {
enum class device { name };
enum class event_profiling { command_submit, command_start, command_end };
} // namespace info

namespace property {
namespace queue {
struct enable_profiling {};
} // namespace queue
} // namespace property

class property_list {
public:
  template <typename... P> property_list(P...) {}
};

class exception : public std::exception {
  std::string msg_;

public:
  explicit exception(std::string m = "sycl exception") : msg_(std::move(m)) {}
  const char *what() const noexcept override { return msg_.c_str(); }
  int get_cl_code() const { return -1; }
};
using exception_list = std::vector<std::exception_ptr>;
using async_handler = std::function<void(exception_list)>;

template <int D> struct range {
  size_t v[D > 0 ? D : 1];
  range() { for (int i = 0; i < D; ++i) v[i] = 0; }
  template <typename... I, typename = std::enable_if_t<sizeof...(I) == D>> range(I... xs) {
    size_t t[] = {static_cast<size_t>(xs)...};
    for (int i = 0; i < D; ++i) v[i] = t[i];
  }
  size_t get(int i) const { return v[i]; }
  size_t operator[](int i) const { return v[i]; }
  size_t size() const {
    size_t s = 1;
    for (int i = 0; i < D; ++i) s *= v[i];
    return s;
  }
};

template <int D> struct id {
  size_t v[D > 0 ? D : 1];
  id() { for (int i = 0; i < D; ++i) v[i] = 0; }
  template <typename... I, typename = std::enable_if_t<sizeof...(I) == D>> id(I... xs) {
    size_t t[] = {static_cast<size_t>(xs)...};
    for (int i = 0; i < D; ++i) v[i] = t[i];
  }
  size_t get(int i) const { return v[i]; }
  size_t operator[](int i) const { return v[i]; }
  operator size_t() const { return v[0]; }
};

template <int D> struct nd_range {
  range<D> g, l;
  nd_range(range<D> global, range<D> local) : g(global), l(local) {}
  range<D> get_global_range() const { return g; }
  range<D> get_local_range() const { return l; }
};

template <int D> struct group {
  size_t gid[D];
};

namespace detail {
/* Fiber scheduler for one work-group; defined in syclshim.cpp. */
struct fiber_group;
void barrier_yield();
bool in_fiber();
} // namespace detail

template <int D> class nd_item {
public:
  size_t gid[D], lid[D], grp[D], G[D], L[D];
  size_t get_global_id(int d) const { return gid[d]; }
  size_t get_global_range(int d) const { return G[d]; }
  size_t get_local_id(int d) const { return lid[d]; }
  size_t get_local_range(int d) const { return L[d]; }
  size_t get_group_linear_id() const {
    size_t r = 0;
    for (int i = 0; i < D; ++i) r = r * (G[i] / L[i]) + grp[i];
    return r;
  }
  size_t get_local_linear_id() const {
    size_t r = 0;
    for (int i = 0; i < D; ++i) r = r * L[i] + lid[i];
    return r;
  }
  group<D> get_group() const {
    group<D> g;
    for (int i = 0; i < D; ++i) g.gid[i] = grp[i];
    return g;
  }
  void barrier(access::fence_space = access::fence_space::global_and_local) const {
    detail::barrier_yield();
  }
};

template <typename T> class global_ptr {
public:
  T *p;
  global_ptr(T *q = nullptr) : p(q) {}
  T *get() const { return p; }
  operator T *() const { return p; }
};

namespace memory_order {
enum { relaxed };
}

template <typename T> class atomic {
  T *p_;

public:
  explicit atomic(global_ptr<T> g) : p_(g.get()) {}
  T load(int = 0) const { return __atomic_load_n(p_, __ATOMIC_RELAXED); }
  void store(T v, int = 0) const { __atomic_store_n(p_, v, __ATOMIC_RELAXED); }
  bool compare_exchange_strong(T &expected, T desired, int = 0, int = 0) const {
    return __atomic_compare_exchange_n(p_, &expected, desired, false, __ATOMIC_RELAXED,
                                       __ATOMIC_RELAXED);
  }
  T fetch_add(T v, int = 0) const { return __atomic_fetch_add(p_, v, __ATOMIC_RELAXED); }
};

class device {
public:
  template <info::device P> std::string get_info() const { return "jx host SYCL subset (CPU)"; }
  bool is_host() const { return true; }
  bool is_cpu() const { return true; }
};

class platform {
public:
  static std::vector<platform> get_platforms() { return {platform()}; }
  std::vector<device> get_devices() const { return {device()}; }
};

class cpu_selector {};
class default_selector {};

class event {
public:
  uint64_t t_submit = 0, t_start = 0, t_end = 0;
  void wait() {}
  template <info::event_profiling P> uint64_t get_profiling_info() const {
    if (P == info::event_profiling::command_submit) return t_submit;
    if (P == info::event_profiling::command_start) return t_start;
    return t_end;
  }
};

class handler;

namespace detail {
/* Local-memory arena of the work-group that is currently executing on this thread. */
extern thread_local char *tl_local_base;
inline uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
/* Run `n_items` work-items of one group; item(k) runs work-item k.  Returns true when some
 * work-item called barrier() (the group then ran as fibers). */
bool run_group(size_t n_items, const std::function<void(size_t)> &item, bool use_fibers);
} // namespace detail

template <typename T, int D = 1, access::mode M = access::mode::read_write,
          access::target Tg = access::target::global_buffer>
class accessor {
public:
  T *ptr = nullptr;
  size_t count = 0;
  size_t local_off = 0; /* byte offset into the local arena (target::local) */

  accessor() = default;
  accessor(T *p, size_t n) : ptr(p), count(n) {}
  /* Local accessor: (size, handler) */
  template <access::target X = Tg, typename = std::enable_if_t<X == access::target::local>>
  accessor(size_t n, handler &cgh);

  T &operator[](size_t i) const {
    if constexpr (Tg == access::target::local)
      return reinterpret_cast<T *>(detail::tl_local_base + local_off)[i];
    else
      return ptr[i];
  }
  T &operator[](id<1> i) const { return (*this)[i.get(0)]; }
  size_t get_count() const { return count; }
  range<1> get_range() const { return range<1>(count); }
  T *get_pointer() const { return ptr; }
};

template <typename T, int D = 1> class buffer {
  struct impl {
    T *data = nullptr;
    size_t n = 0;
    std::shared_ptr<T> keep; /* shared host data, if any */
    std::unique_ptr<T[]> own;
  };
  std::shared_ptr<impl> p_;

public:
  buffer() : p_(std::make_shared<impl>()) {}
  buffer(std::nullptr_t) : p_(std::make_shared<impl>()) {}
  explicit buffer(range<1> r) : p_(std::make_shared<impl>()) {
    p_->n = r.get(0);
    p_->own.reset(new T[p_->n > 0 ? p_->n : 1]());
    p_->data = p_->own.get();
  }
  buffer(T *host, range<1> r) : p_(std::make_shared<impl>()) {
    p_->n = r.get(0);
    p_->data = host;
  }
  buffer(T *host, size_t n) : buffer(host, range<1>(n)) {}
  buffer(std::shared_ptr<T> host, range<1> r) : p_(std::make_shared<impl>()) {
    p_->n = r.get(0);
    p_->keep = host;
    p_->data = host.get();
  }
  buffer(std::shared_ptr<T> host, size_t n) : buffer(host, range<1>(n)) {}

  size_t get_count() const { return p_->n; }
  range<1> get_range() const { return range<1>(p_->n); }
  T *host_data() const { return p_->data; }

  template <access::mode M, access::target Tg = access::target::global_buffer>
  accessor<T, 1, M, Tg> get_access(handler &, range<1> r = range<1>(0)) {
    (void)r;
    return accessor<T, 1, M, Tg>(p_->data, p_->n);
  }
  template <access::mode M, access::target Tg = access::target::global_buffer>
  accessor<T, 1, M, Tg> get_access(handler &, range<1> r, id<1>) {
    (void)r;
    return accessor<T, 1, M, Tg>(p_->data, p_->n);
  }
  /* host accessor */
  template <access::mode M> accessor<T, 1, M, access::target::host_buffer> get_access(range<1> r = range<1>(0)) {
    (void)r;
    return accessor<T, 1, M, access::target::host_buffer>(p_->data, p_->n);
  }
};

class handler {
public:
  size_t local_bytes = 0;
  size_t reserve_local(size_t bytes) {
    size_t off = (local_bytes + 63) & ~size_t(63);
    local_bytes = off + bytes;
    return off;
  }

  template <typename Name = void, int D, typename K> void parallel_for(nd_range<D> r, K kernel) {
    size_t ngroups[D], total_groups = 1, items = 1;
    for (int i = 0; i < D; ++i) {
      ngroups[i] = r.g.v[i] / r.l.v[i];
      total_groups *= ngroups[i];
      items *= r.l.v[i];
    }
    const size_t arena = local_bytes > 0 ? local_bytes : 64;
    auto run_one = [&](size_t glin, bool fibers, char *base) -> bool {
      size_t grp[D];
      size_t t = glin;
      for (int i = D - 1; i >= 0; --i) {
        grp[i] = t % ngroups[i];
        t /= ngroups[i];
      }
      detail::tl_local_base = base;
      std::memset(base, 0, arena);
      auto item = [&](size_t llin) {
        nd_item<D> it;
        size_t u = llin;
        for (int i = D - 1; i >= 0; --i) {
          it.lid[i] = u % r.l.v[i];
          u /= r.l.v[i];
        }
        for (int i = 0; i < D; ++i) {
          it.grp[i] = grp[i];
          it.G[i] = r.g.v[i];
          it.L[i] = r.l.v[i];
          it.gid[i] = grp[i] * r.l.v[i] + it.lid[i];
        }
        kernel(it);
      };
      return detail::run_group(items, item, fibers);
    };
    if (total_groups == 0) return;
    /* The first executed group decides whether fibers are needed. */
    long long g0 = 0;
    while (g0 < (long long)total_groups && !jxshim::group_selected(g0)) ++g0;
    if (g0 >= (long long)total_groups) return;
    std::vector<char> first(arena);
    const bool fibers = run_one((size_t)g0, true, first.data());
#pragma omp parallel
    {
      std::vector<char> local(arena);
#pragma omp for schedule(dynamic, 1)
      for (long long g = g0 + 1; g < (long long)total_groups; ++g) {
        if (!jxshim::group_selected(g)) continue;
        run_one((size_t)g, fibers, local.data());
      }
    }
  }

  /* Basic range<1> parallel_for over a lambda taking id<1>. */
  template <typename Name = void, typename K> void parallel_for(range<1> r, K kernel) {
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)r.get(0); ++i) kernel(id<1>((size_t)i));
  }

  template <typename T, access::mode M, access::target Tg>
  void copy(accessor<T, 1, M, Tg> src, T *dst) {
    std::memcpy(dst, src.ptr, sizeof(T) * src.count);
  }
};

template <typename T, int D, access::mode M, access::target Tg>
template <access::target X, typename>
accessor<T, D, M, Tg>::accessor(size_t n, handler &cgh) : ptr(nullptr), count(n) {
  local_off = cgh.reserve_local(sizeof(T) * n);
}

class queue {
  device dev_;

public:
  queue() {}
  template <typename H, typename = std::enable_if_t<!std::is_same_v<std::decay_t<H>, device> &&
                                                    !std::is_same_v<std::decay_t<H>, property_list>>>
  explicit queue(H &&, const property_list & = property_list()) {}
  explicit queue(const property_list &) {}
  queue(const cpu_selector &) {}
  template <typename H> queue(const device &d, H &&, const property_list & = property_list()) : dev_(d) {}
  queue(const device &d) : dev_(d) {}

  template <typename CGF> event submit(CGF cgf) {
    event e;
    e.t_submit = detail::now_ns();
    handler h;
    e.t_start = detail::now_ns();
    cgf(h);
    e.t_end = detail::now_ns();
    return e;
  }
  void wait() {}
  void wait_and_throw() {}
  device get_device() const { return dev_; }
};

} // namespace sycl
} // namespace cl

namespace sycl = cl::sycl;

#endif /* JX_SYCLSHIM_SYCL_HPP */
