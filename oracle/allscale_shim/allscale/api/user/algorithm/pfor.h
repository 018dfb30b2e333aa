// Stand-in for allscale/api/user/algorithm/pfor.h: a parallel loop over a
// box of grid points. Iterations run on OpenMP threads when compiled with
// -fopenmp (the shared-memory reading of AllScale's pfor), else serially in
// row-major order. The reference's mover/export/import phases have one writer
// per buffer, so their results do not depend on the iteration order.
// TEST INFRASTRUCTURE ONLY (oracle).
#pragma once

#include <cstdint>

#include "allscale/api/user/data/grid.h"
#include "allscale/utils/vector.h"

namespace allscale {
namespace api {
namespace user {
namespace algorithm {

namespace detail {

template <typename T, std::size_t D>
std::int64_t box_volume(const allscale::utils::Vector<T, D>& a, const allscale::utils::Vector<T, D>& b) {
    std::int64_t n = 1;
    for (std::size_t i = 0; i < D; ++i) {
        std::int64_t e = (std::int64_t)b[i] - (std::int64_t)a[i];
        if (e <= 0) return 0;
        n *= e;
    }
    return n;
}

template <typename T, std::size_t D>
allscale::utils::Vector<T, D> box_point(const allscale::utils::Vector<T, D>& a, const allscale::utils::Vector<T, D>& b,
                                        std::int64_t lin) {
    allscale::utils::Vector<T, D> p;
    for (std::size_t k = D; k-- > 0;) {
        std::int64_t e = (std::int64_t)b[k] - (std::int64_t)a[k];
        p[k] = (T)(a[k] + lin % e);
        lin /= e;
    }
    return p;
}

// serial row-major iteration over [start, end) (AllScale's detail::forEach)
template <typename T, std::size_t D, typename F>
void forEach(const allscale::utils::Vector<T, D>& start, const allscale::utils::Vector<T, D>& end, const F& f) {
    std::int64_t n = box_volume(start, end);
    for (std::int64_t i = 0; i < n; ++i) f(box_point(start, end, i));
}

}  // namespace detail

template <typename T, std::size_t D, typename F>
void pfor(const allscale::utils::Vector<T, D>& start, const allscale::utils::Vector<T, D>& end, const F& f) {
    std::int64_t n = detail::box_volume(start, end);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8)
#endif
    for (std::int64_t i = 0; i < n; ++i) f(detail::box_point(start, end, i));
}

template <typename T, std::size_t D, typename F>
void pfor(const allscale::utils::Vector<T, D>& end, const F& f) {
    pfor(allscale::utils::Vector<T, D>(T(0)), end, f);
}

}  // namespace algorithm
}  // namespace user
}  // namespace api
}  // namespace allscale
