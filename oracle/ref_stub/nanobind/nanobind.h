/*
 * Stand-in for the nanobind headers, so that the reference's CUDA sources
 * (cunusht/c/pointing.cu, cunusht/c/doubling.cu) compile with nvcc alone into
 * a device-only module for the parity checks.  Only what those two files
 * name is declared: nb::ndarray (data(), size()), nb::ndim, nb::device::cuda,
 * the _a argument literal with .noconvert(), and NB_MODULE, whose body
 * becomes an ordinary host function that is never called -- it still names
 * every binding, so the kernel templates those bindings launch are
 * instantiated exactly as in the reference's own module.
 *
 * TEST INFRASTRUCTURE ONLY: used by oracle/ref_build.py, never by the product.
 */
#ifndef CUNUSHT_REF_NANOBIND_STUB_H
#define CUNUSHT_REF_NANOBIND_STUB_H
#include <cstddef>

namespace nanobind {
struct arg_stub {
    constexpr arg_stub noconvert() const { return *this; }
};
namespace literals {
constexpr arg_stub operator""_a(const char *, std::size_t) { return {}; }
}  // namespace literals
template <std::size_t N> struct ndim {};
namespace device {
struct cuda {};
}  // namespace device
template <typename T, typename... Tags> struct ndarray {
    T *ptr_ = nullptr;
    std::size_t n_ = 0;
    T *data() const { return ptr_; }
    std::size_t size() const { return n_; }
};
struct module_ {
    template <typename... A> module_ &def(const char *, A &&...) { return *this; }
};
}  // namespace nanobind

#define NB_MODULE(name, var) void cunusht_ref_stub_module_##name(::nanobind::module_ &var)
#endif
