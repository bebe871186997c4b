// Minimal stand-in for AdaptiveCpp's <hipSYCL/sycl/jit.hpp> (test
// infrastructure).  The reference's call-sequence JIT fusion is switched off
// in its own code (models/execution.hpp: disable_fusion = true), so these
// types only need to compile: a definition wraps a function pointer and a
// config's apply returns the kernel it is given.  Written for this shim.
#pragma once

namespace sycl {
namespace AdaptiveCpp_jit {

template <typename Ret, typename... Args>
struct dynamic_function_definition {
    using fn_t = Ret (*)(Args...);
    fn_t fn = nullptr;
    dynamic_function_definition() = default;
    dynamic_function_definition(fn_t f) : fn(f) {}
};

struct dynamic_function_config {
    template <typename F, typename Defs>
    void define_as_call_sequence(F, const Defs &) {}
    template <typename K>
    K apply(K k) { return k; }
};

}  // namespace AdaptiveCpp_jit
}  // namespace sycl
