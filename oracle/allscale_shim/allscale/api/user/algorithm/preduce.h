// Stand-in for allscale/api/user/algorithm/preduce.h: map/reduce over a box of
// grid points or over a container. Evaluated serially in row-major (container)
// order, so sums are deterministic. TEST INFRASTRUCTURE ONLY (oracle).
#pragma once

#include <cstdint>
#include <utility>

#include "allscale/api/user/algorithm/pfor.h"

namespace allscale {
namespace api {
namespace user {
namespace algorithm {

template <typename R>
struct ready_value {
    R value;
    R get() const { return value; }
    void wait() const {}
};

template <typename T, std::size_t D, typename Fold, typename Reduce, typename Init>
auto preduce(const allscale::utils::Vector<T, D>& start, const allscale::utils::Vector<T, D>& end, const Fold& fold,
             const Reduce&, const Init& init) -> ready_value<decltype(init())> {
    auto res = init();
    detail::forEach(start, end, [&](const allscale::utils::Vector<T, D>& p) { fold(p, res); });
    return {res};
}

template <typename Container, typename Map, typename Reduce, typename Init>
auto preduce(const Container& c, const Map& map, const Reduce&, const Init& init) -> ready_value<decltype(init())> {
    auto res = init();
    for (const auto& e : c) map(e, res);
    return {res};
}

}  // namespace algorithm
}  // namespace user
}  // namespace api
}  // namespace allscale
