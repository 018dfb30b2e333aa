// Minimal stand-in for the AllScale API's assertion macros (assert_true,
// assert_eq, ... with a streamed message). TEST INFRASTRUCTURE ONLY (oracle).
//
// With ALLSCALE_SHIM_CHECKS defined the conditions are evaluated and a failure
// prints the message and aborts; otherwise, as in the reference's release
// builds, the conditions are not evaluated at all.
#pragma once

#include <cstdlib>
#include <iostream>
#include <sstream>

namespace allscale {
namespace utils {
namespace detail {

struct AssertSink {
    template <typename T>
    AssertSink& operator<<(const T&) { return *this; }
};

class AssertCheck {
    bool failed_;
    std::ostringstream msg_;

  public:
    AssertCheck(bool failed, const char* file, int line, const char* what) : failed_(failed) {
        if (failed_) msg_ << file << ":" << line << ": assertion failed: " << what << " ";
    }
    ~AssertCheck() {
        if (failed_) {
            std::cerr << msg_.str() << std::endl;
            std::abort();
        }
    }
    template <typename T>
    AssertCheck& operator<<(const T& v) {
        if (failed_) msg_ << v;
        return *this;
    }
};

}  // namespace detail
}  // namespace utils
}  // namespace allscale

#ifdef ALLSCALE_SHIM_CHECKS
#define ALLSCALE_SHIM_ASSERT(cond, what) ::allscale::utils::detail::AssertCheck(!(cond), __FILE__, __LINE__, what)
#define assert_decl(...) __VA_ARGS__
#else
#define ALLSCALE_SHIM_ASSERT(cond, what) \
    if (true) {                          \
    } else                               \
        ::allscale::utils::detail::AssertSink()
#define assert_decl(...)
#endif

#define assert_true(c) ALLSCALE_SHIM_ASSERT((c), #c)
#define assert_false(c) ALLSCALE_SHIM_ASSERT(!(c), "!(" #c ")")
#define assert_eq(a, b) ALLSCALE_SHIM_ASSERT((a) == (b), #a " == " #b)
#define assert_ne(a, b) ALLSCALE_SHIM_ASSERT((a) != (b), #a " != " #b)
#define assert_lt(a, b) ALLSCALE_SHIM_ASSERT((a) < (b), #a " < " #b)
#define assert_le(a, b) ALLSCALE_SHIM_ASSERT((a) <= (b), #a " <= " #b)
#define assert_gt(a, b) ALLSCALE_SHIM_ASSERT((a) > (b), #a " > " #b)
#define assert_ge(a, b) ALLSCALE_SHIM_ASSERT((a) >= (b), #a " >= " #b)
#define assert_fail() ALLSCALE_SHIM_ASSERT(false, "fail")
#define assert_not_implemented() ALLSCALE_SHIM_ASSERT(false, "not implemented")
