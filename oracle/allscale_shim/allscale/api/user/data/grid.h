// Stand-in for allscale/api/user/data/grid.h: a dense 3-D (or D-D) grid in
// row-major order (x slowest), matching the flatten used by the reference at
// cell.h:521-523. GridPoint<D> is Vector<int64_t,D>. TEST INFRASTRUCTURE ONLY
// (oracle).
#pragma once

#include <cstdint>
#include <vector>

#include "allscale/utils/assert.h"
#include "allscale/utils/vector.h"

namespace allscale {
namespace api {
namespace user {
namespace data {

template <std::size_t D>
using GridPoint = allscale::utils::Vector<std::int64_t, D>;

template <typename T, std::size_t D = 3>
class Grid {
    GridPoint<D> size_;
    std::vector<T> data_;

    static std::size_t volume(const GridPoint<D>& s) {
        std::size_t n = 1;
        for (std::size_t i = 0; i < D; ++i) n *= (std::size_t)(s[i] > 0 ? s[i] : 0);
        return n;
    }

  public:
    using coordinate_type = GridPoint<D>;

    Grid(const GridPoint<D>& size) : size_(size), data_(volume(size)) {}

    const GridPoint<D>& size() const { return size_; }

    std::size_t flatten(const GridPoint<D>& p) const {
        std::size_t r = 0;
        for (std::size_t i = 0; i < D; ++i) r = r * (std::size_t)size_[i] + (std::size_t)p[i];
        return r;
    }

    T& operator[](const GridPoint<D>& p) { return data_[flatten(p)]; }
    const T& operator[](const GridPoint<D>& p) const { return data_[flatten(p)]; }

    T* raw() { return data_.data(); }
    const T* raw() const { return data_.data(); }
};

}  // namespace data
}  // namespace user
}  // namespace api
}  // namespace allscale
