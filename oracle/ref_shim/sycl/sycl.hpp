// Minimal host-only stand-in for <sycl/sycl.hpp>.
//
// TEST INFRASTRUCTURE ONLY.  It exists so that the reference's own kernel
// headers (kernels/selection.hpp, projection.hpp, aggregation.hpp, join.hpp,
// common.hpp) compile unchanged with g++ and run on the CPU, one work-item at
// a time in index order.  That gives the oracle tests the reference's kernel
// functors themselves as a second checker.  Only the subset of SYCL that those
// headers use is provided: queue/handler/event, id/range, parallel_for with
// and without a reduction, atomic_ref, USM malloc/free, and the device-info
// calls that operations/memory_manager.hpp names.  All of it is written for
// this shim; none of it is SYCL implementation code.
#pragma once

#include <cctype>
#include <chrono>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace sycl {

template <int D = 1>
struct id {
    size_t v;
    id() : v(0) {}
    id(size_t x) : v(x) {}
    operator size_t() const { return v; }
    size_t operator[](int) const { return v; }
};

template <int D = 1>
struct range {
    size_t v;
    range(size_t x) : v(x) {}
    size_t size() const { return v; }
};

template <int D = 1>
struct item {
    size_t v;
    item() : v(0) {}
    item(size_t x) : v(x) {}
    item(id<D> x) : v(x.v) {}
    operator size_t() const { return v; }
    size_t operator[](int) const { return v; }
    size_t get_id(int) const { return v; }
};

struct event {
    void wait() {}
    void wait_and_throw() {}
    static void wait(const std::vector<event> &) {}
    static void wait_and_throw(const std::vector<event> &) {}
    bool operator==(const event &) const { return true; }
    bool operator!=(const event &) const { return false; }
    template <typename T>
    uint64_t get_profiling_info() const { return 0; }
};

enum class backend { host = 0, ocl = 1, omp = 2, cuda = 3, hip = 4, level_zero = 5, ext_oneapi_cuda = 3,
                     ext_oneapi_hip = 4, ext_oneapi_level_zero = 5 };

struct platform;

// Device and platform queries: each info descriptor names the type it returns.
namespace info {
namespace device {
struct name { using return_type = std::string; };
struct vendor { using return_type = std::string; };
struct global_mem_size { using return_type = uint64_t; };
struct max_compute_units { using return_type = uint32_t; };
struct platform { using return_type = sycl::platform; };
}  // namespace device
namespace platform {
struct name { using return_type = std::string; };
}  // namespace platform
namespace event_profiling {
struct command_start {};
struct command_end {};
}  // namespace event_profiling
}  // namespace info

struct platform {
    template <typename T>
    typename T::return_type get_info() const { return "host-shim"; }
};

// One device: the host, on which every work-item runs in turn.
struct device {
    template <typename T>
    typename T::return_type get_info() const
    {
        using R = typename T::return_type;
        if constexpr (std::is_same_v<R, std::string>) return "host-shim";
        else if constexpr (std::is_same_v<R, uint64_t>) return (uint64_t)1 << 34;
        else if constexpr (std::is_same_v<R, uint32_t>) return 1u;
        else return R{};
    }
    backend get_backend() const { return backend::host; }
    bool is_gpu() const { return false; }
    bool is_cpu() const { return true; }
    bool is_host() const { return true; }
    static std::vector<device> get_devices() { return {device{}}; }
};

struct default_selector_t {};
inline constexpr default_selector_t default_selector_v{};

namespace property {
namespace queue {
struct in_order {};
struct enable_profiling {};
}  // namespace queue
}  // namespace property

struct property_list {
    template <typename... P>
    property_list(P...) {}
};

template <typename T = void>
struct plus {
    T operator()(const T &a, const T &b) const { return a + b; }
};
template <>
struct plus<void> {
    template <typename A, typename B>
    auto operator()(const A &a, const B &b) const { return a + b; }
};

namespace property {
namespace reduction {
struct initialize_to_identity {};
}  // namespace reduction
}  // namespace property

template <typename T, typename Op>
struct reduction_desc {
    T *ptr;
    bool init_identity;
};

template <typename T, typename Op>
reduction_desc<T, Op> reduction(T *ptr, Op)
{
    return {ptr, false};
}

template <typename T, typename Op>
reduction_desc<T, Op> reduction(T *ptr, Op, property::reduction::initialize_to_identity)
{
    return {ptr, true};
}

// Reducer handed to a kernel: combine(x) converts x to T, as SYCL's
// reducer::combine(const T&) does, then adds.
template <typename T>
struct reducer {
    T acc;
    void combine(const T &x) { acc = acc + x; }
    reducer &operator+=(const T &x) { combine(x); return *this; }
};

class handler {
public:
    template <typename Deps>
    void depends_on(const Deps &) {}

    template <typename K>
    void parallel_for(range<1> r, K k)
    {
        for (size_t i = 0; i < r.size(); i++) invoke(k, i);
    }

    template <typename K>
    void parallel_for(size_t n, K k)
    {
        parallel_for(range<1>(n), k);
    }

    template <typename T, typename Op, typename K>
    void parallel_for(range<1> r, reduction_desc<T, Op> red, K k)
    {
        reducer<T> rd{red.init_identity ? T(0) : *red.ptr};
        for (size_t i = 0; i < r.size(); i++) {
            if constexpr (std::is_invocable_v<K &, id<1>, reducer<T> &>)
                k(id<1>(i), rd);
            else
                k(item<1>(i), rd);
        }
        *red.ptr = rd.acc;
    }

    template <typename T, typename Op, typename K>
    void parallel_for(size_t n, reduction_desc<T, Op> red, K k)
    {
        parallel_for(range<1>(n), red, k);
    }

    template <typename K>
    void single_task(K k) { k(); }

private:
    template <typename K>
    static void invoke(K &k, size_t i)
    {
        if constexpr (std::is_invocable_v<K &, id<1>>)
            k(id<1>(i));
        else
            k(item<1>{i});
    }
};

class queue {
public:
    queue() = default;
    queue(default_selector_t) {}
    queue(const device &) {}
    template <typename P>
    queue(const device &, const P &) {}
    void wait_and_throw() {}
    template <typename F>
    event submit(F f)
    {
        handler h;
        f(h);
        return event{};
    }
    template <typename T>
    event fill(T *p, const T &v, size_t n)
    {
        for (size_t i = 0; i < n; i++) p[i] = v;
        return event{};
    }
    template <typename T, typename Deps>
    event fill(T *p, const T &v, size_t n, const Deps &)
    {
        return fill(p, v, n);
    }
    template <typename Name = void, typename K>
    event single_task(K k)
    {
        k();
        return event{};
    }
    template <typename Name = void, typename Deps, typename K>
    event single_task(const Deps &, K k)
    {
        k();
        return event{};
    }
    template <typename K>
    event parallel_for(range<1> r, K k)
    {
        return submit([&](handler &h) { h.parallel_for(r, k); });
    }
    event memset(void *p, int v, size_t n)
    {
        std::memset(p, v, n);
        return event{};
    }
    event memcpy(void *d, const void *s, size_t n)
    {
        std::memcpy(d, s, n);
        return event{};
    }
    template <typename Deps>
    event memcpy(void *d, const void *s, size_t n, const Deps &)
    {
        return memcpy(d, s, n);
    }
    template <typename T>
    event copy(const T *s, T *d, size_t n)
    {
        return memcpy(d, s, n * sizeof(T));
    }
    void wait() {}
    device get_device() const { return device{}; }
};

template <typename T>
T *malloc_shared(size_t n, const queue &) { return static_cast<T *>(std::calloc(n ? n : 1, sizeof(T))); }
template <typename T>
T *malloc_device(size_t n, const queue &) { return malloc_shared<T>(n, queue{}); }
template <typename T>
T *malloc_host(size_t n, const queue &) { return malloc_shared<T>(n, queue{}); }
inline void free(void *p, const queue &) { std::free(p); }

enum class memory_order { relaxed, acquire, release, acq_rel, seq_cst };
enum class memory_scope { work_item, sub_group, work_group, device, system };
namespace access {
enum class address_space { global_space, local_space, generic_space };
}

// Work-items run one at a time, so plain loads and stores are atomic here.
template <typename T, memory_order MO = memory_order::relaxed, memory_scope MS = memory_scope::device,
          access::address_space AS = access::address_space::global_space>
class atomic_ref {
    T &r;
public:
    explicit atomic_ref(T &x) : r(x) {}
    T exchange(T v) { T o = r; r = v; return o; }
    bool compare_exchange_strong(T &expected, T desired)
    {
        if (r == expected) { r = desired; return true; }
        expected = r;
        return false;
    }
    template <typename U>
    T fetch_add(U v) { T o = r; r = r + static_cast<T>(v); return o; }
    T load() const { return r; }
    void store(T v) { r = v; }
};

}  // namespace sycl
