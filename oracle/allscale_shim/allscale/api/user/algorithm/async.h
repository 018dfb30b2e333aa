// Stand-in for allscale/api/user/algorithm/async.h: runs the task at once.
// TEST INFRASTRUCTURE ONLY (oracle).
#pragma once

namespace allscale {
namespace api {
namespace user {
namespace algorithm {

struct done_task {
    void wait() const {}
    void get() const {}
};

template <typename F>
done_task async(const F& f) {
    f();
    return {};
}

}  // namespace algorithm
}  // namespace user
}  // namespace api
}  // namespace allscale
