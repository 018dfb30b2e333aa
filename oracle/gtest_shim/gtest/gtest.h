// A small gtest-compatible macro set, enough to compile and run the
// reference's own unit tests (code/app/test/*.cc) unmodified against the
// AllScale shim. TEST INFRASTRUCTURE ONLY (oracle): it runs the reference's
// known-answer tests on this machine, which pins the shim and the oracle.
//
// Supported: TEST, EXPECT_/ASSERT_ {EQ,NE,LT,LE,GT,GE,TRUE,FALSE,NEAR} with a
// streamed message, DISABLED_ tests (skipped), and a main() that runs every
// registered test (optionally filtered by a substring given as argv[1]).
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <sys/wait.h>
#include <unistd.h>

namespace testing {

struct TestCase {
    std::string suite, name;
    std::function<void()> fn;
};

inline std::vector<TestCase>& registry() {
    static std::vector<TestCase> r;
    return r;
}

inline int& failures() {
    static int f = 0;
    return f;
}

struct Registrar {
    Registrar(const char* s, const char* n, std::function<void()> f) { registry().push_back({s, n, std::move(f)}); }
};

// Reports a failure when destroyed, after the user's streamed message.
class Failure {
    bool active_;
    std::ostringstream msg_;

  public:
    Failure(bool failed, const char* file, int line, const std::string& what) : active_(failed) {
        if (active_) msg_ << file << ":" << line << ": Failure: " << what;
    }
    Failure(const Failure&) = delete;
    ~Failure() {
        if (active_) {
            ++failures();
            std::cout << msg_.str() << std::endl;
        }
    }
    template <typename T>
    Failure& operator<<(const T& v) {
        if (active_) msg_ << " " << v;
        return *this;
    }
    explicit operator bool() const { return active_; }
};

template <typename A, typename B>
std::string describe(const char* op, const char* ea, const char* eb, const A& a, const B& b) {
    std::ostringstream s;
    s << ea << " " << op << " " << eb << " (" << a << " vs " << b << ")";
    return s.str();
}

struct AssertHelper {
    void operator=(const Failure&) const {}
};

}  // namespace testing

#define GTS_CAT2(a, b) a##b
#define GTS_CAT(a, b) GTS_CAT2(a, b)

#define TEST(suite, name)                                                                              \
    static void GTS_CAT(gts_test_, GTS_CAT(suite, GTS_CAT(_, name)))();                                 \
    static ::testing::Registrar GTS_CAT(gts_reg_, GTS_CAT(suite, GTS_CAT(_, name)))(                    \
        #suite, #name, &GTS_CAT(gts_test_, GTS_CAT(suite, GTS_CAT(_, name))));                           \
    static void GTS_CAT(gts_test_, GTS_CAT(suite, GTS_CAT(_, name)))()

#define GTS_CHECK(cond, what) ::testing::Failure(!(cond), __FILE__, __LINE__, what)
#define GTS_CMP(op, a, b) GTS_CHECK((a)op(b), ::testing::describe(#op, #a, #b, (a), (b)))

#define EXPECT_TRUE(c) GTS_CHECK(static_cast<bool>(c), #c)
#define EXPECT_FALSE(c) GTS_CHECK(!static_cast<bool>(c), "!(" #c ")")
#define EXPECT_EQ(a, b) GTS_CMP(==, a, b)
#define EXPECT_NE(a, b) GTS_CMP(!=, a, b)
#define EXPECT_LT(a, b) GTS_CMP(<, a, b)
#define EXPECT_LE(a, b) GTS_CMP(<=, a, b)
#define EXPECT_GT(a, b) GTS_CMP(>, a, b)
#define EXPECT_GE(a, b) GTS_CMP(>=, a, b)
#define EXPECT_NEAR(a, b, tol) \
    GTS_CHECK(std::fabs((double)(a) - (double)(b)) <= (double)(tol), ::testing::describe("~=", #a, #b, (a), (b)))

// ASSERT_* return from the enclosing (void) function on failure.
#define GTS_FATAL(cond, what)                                                                  \
    for (bool gts_bad_ = !(cond); gts_bad_; gts_bad_ = false)                                  \
        for (::testing::Failure gts_f_(true, __FILE__, __LINE__, what); gts_bad_; gts_bad_ = false) \
            return ::testing::AssertHelper() = gts_f_ << ""

#define ASSERT_TRUE(c) GTS_FATAL(static_cast<bool>(c), #c)
#define ASSERT_FALSE(c) GTS_FATAL(!static_cast<bool>(c), "!(" #c ")")
#define ASSERT_EQ(a, b) GTS_FATAL((a) == (b), ::testing::describe("==", #a, #b, (a), (b)))
#define ASSERT_NE(a, b) GTS_FATAL((a) != (b), ::testing::describe("!=", #a, #b, (a), (b)))
#define ASSERT_LT(a, b) GTS_FATAL((a) < (b), ::testing::describe("<", #a, #b, (a), (b)))
#define ASSERT_LE(a, b) GTS_FATAL((a) <= (b), ::testing::describe("<=", #a, #b, (a), (b)))
#define ASSERT_GT(a, b) GTS_FATAL((a) > (b), ::testing::describe(">", #a, #b, (a), (b)))
#define ASSERT_NEAR(a, b, tol) \
    GTS_FATAL(std::fabs((double)(a) - (double)(b)) <= (double)(tol), ::testing::describe("~=", #a, #b, (a), (b)))

// The statement must end the process (exit with a non-zero status or a
// signal); it runs in a forked child so the test binary survives.
#define EXPECT_DEATH_IF_SUPPORTED(stmt, regex)                                          \
    GTS_CHECK(([&]() -> bool {                                                        \
                  std::cout.flush();                                                   \
                  pid_t gts_pid_ = fork();                                             \
                  if (gts_pid_ == 0) {                                                 \
                      { stmt; }                                                        \
                      _exit(0);                                                        \
                  }                                                                    \
                  int gts_st_ = 0;                                                     \
                  waitpid(gts_pid_, &gts_st_, 0);                                      \
                  return WIFSIGNALED(gts_st_) || (WIFEXITED(gts_st_) && WEXITSTATUS(gts_st_) != 0); \
              }()),                                                                    \
              "death expected: " #stmt)
#define EXPECT_DEATH(stmt, regex) EXPECT_DEATH_IF_SUPPORTED(stmt, regex)

#ifndef GTS_NO_MAIN
int main(int argc, char** argv) {
    const char* filter = argc > 1 ? argv[1] : nullptr;
    int run = 0, failed_tests = 0, skipped = 0;
    for (auto& t : ::testing::registry()) {
        std::string full = t.suite + "." + t.name;
        if (filter && full.find(filter) == std::string::npos) continue;
        if (t.name.rfind("DISABLED_", 0) == 0) {
            ++skipped;
            continue;
        }
        int before = ::testing::failures();
        std::cout << "[ RUN      ] " << full << std::endl;
        t.fn();
        ++run;
        bool ok = ::testing::failures() == before;
        if (!ok) ++failed_tests;
        std::cout << (ok ? "[       OK ] " : "[  FAILED  ] ") << full << std::endl;
    }
    std::cout << "[==========] " << run << " tests ran, " << failed_tests << " failed, " << skipped << " disabled"
              << std::endl;
    return failed_tests ? 1 : 0;
}
#endif
