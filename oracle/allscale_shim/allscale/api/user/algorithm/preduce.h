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

// The result of a range reduction, handed out by reference (pic_tracer's
// ParticleCount is move-only).
template <typename R>
struct ready_range {
    R value;
    const R& get() const { return value; }
    void wait() const {}
};

// preduce(a, b, map, reduce) over the integer range [a, b) with a range map
// operator map(a, b) -> R, as pic_tracer.cxx:282 uses it: the range is
// evaluated as one piece, so map runs once on [a, b) and reduce is not
// needed.
template <typename Map, typename Reduce>
auto preduce(int a, int b, const Map& map, const Reduce&) -> ready_range<decltype(map(a, b))> {
    return ready_range<decltype(map(a, b))>{map(a, b)};
}

}  // namespace algorithm
}  // namespace user
}  // namespace api
}  // namespace allscale
