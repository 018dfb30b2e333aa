// Minimal stand-in for the AllScale API's allscale/utils/vector.h.
//
// TEST INFRASTRUCTURE ONLY (oracle). It exists so that the reference's own
// headers (code/app/include/ipic3d/app/*.h) compile unmodified on this
// machine; it is written from the reference's usage of the API, not from the
// AllScale sources, which are not vendored (cmake/allscale.cmake:45-57 fetches
// allscale_api@fd12c6e5 over the network).
//
// Semantics pinned here (the reference relies on them):
//  * Vector<T,3> exposes members x, y, z and operator[] (cell.h:1105, field.h:311).
//  * operator<< prints "[x,y,z]" -- the per-cell count file header
//    (outputs/test.out line 1 is "[8,8,8]", written by cell.h:1372).
//  * dominatedBy = all components <=, strictlyDominatedBy = all components <
//    (universe_properties.h:127,141, cell.h:82).
//  * operator< = all components strictly less. The reference uses it only in
//    the field solvers' "do not update the ghost cells" guard
//    (field.h:315,366,377); the AllScale definition is not visible in the
//    tree, and "all less" is the reading that matches that comment.
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <set>
#include <string>
#include <type_traits>
#include <vector>

#include "allscale/utils/assert.h"

namespace allscale {
namespace utils {

template <typename T, std::size_t D>
struct Vector {
    std::array<T, D> data;

    Vector() : data() {}
    Vector(const T& v) { data.fill(v); }
    template <typename... Rest, typename = std::enable_if_t<sizeof...(Rest) + 2 == D>>
    Vector(const T& a, const T& b, const Rest&... rest) : data{{a, b, static_cast<T>(rest)...}} {}

    T& operator[](std::size_t i) { return data[i]; }
    const T& operator[](std::size_t i) const { return data[i]; }
    static constexpr std::size_t D_ = D;
    bool dominatedBy(const Vector& o) const {
        for (std::size_t i = 0; i < D_; ++i)
            if (!((*this)[i] <= o[i])) return false;
        return true;
    }
    bool strictlyDominatedBy(const Vector& o) const {
        for (std::size_t i = 0; i < D_; ++i)
            if (!((*this)[i] < o[i])) return false;
        return true;
    }
};

// D = 3 and D = 2 carry named members, as the reference reads .x/.y/.z.
template <typename T>
struct Vector<T, 3> {
    T x, y, z;

    Vector() : x(), y(), z() {}
    Vector(const T& v) : x(v), y(v), z(v) {}
    Vector(const T& a, const T& b, const T& c) : x(a), y(b), z(c) {}
    template <typename S, typename = std::enable_if_t<!std::is_same<S, T>::value>>
    explicit Vector(const Vector<S, 3>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}

    T& operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
    static constexpr std::size_t D_ = 3;
    bool dominatedBy(const Vector& o) const {
        for (std::size_t i = 0; i < D_; ++i)
            if (!((*this)[i] <= o[i])) return false;
        return true;
    }
    bool strictlyDominatedBy(const Vector& o) const {
        for (std::size_t i = 0; i < D_; ++i)
            if (!((*this)[i] < o[i])) return false;
        return true;
    }
};

template <typename T>
struct Vector<T, 2> {
    T x, y;

    Vector() : x(), y() {}
    Vector(const T& v) : x(v), y(v) {}
    Vector(const T& a, const T& b) : x(a), y(b) {}

    T& operator[](std::size_t i) { return i == 0 ? x : y; }
    const T& operator[](std::size_t i) const { return i == 0 ? x : y; }
    static constexpr std::size_t D_ = 2;
    bool dominatedBy(const Vector& o) const {
        for (std::size_t i = 0; i < D_; ++i)
            if (!((*this)[i] <= o[i])) return false;
        return true;
    }
    bool strictlyDominatedBy(const Vector& o) const {
        for (std::size_t i = 0; i < D_; ++i)
            if (!((*this)[i] < o[i])) return false;
        return true;
    }
};

template <typename S>
using is_scalar_t = std::enable_if_t<std::is_arithmetic<S>::value>;

// --- element-wise arithmetic -------------------------------------------------

template <typename T, std::size_t D>
Vector<T, D>& operator+=(Vector<T, D>& a, const Vector<T, D>& b) {
    for (std::size_t i = 0; i < D; ++i) a[i] += b[i];
    return a;
}
template <typename T, std::size_t D>
Vector<T, D>& operator-=(Vector<T, D>& a, const Vector<T, D>& b) {
    for (std::size_t i = 0; i < D; ++i) a[i] -= b[i];
    return a;
}
template <typename T, std::size_t D>
Vector<T, D> operator+(const Vector<T, D>& a, const Vector<T, D>& b) {
    Vector<T, D> r = a;
    r += b;
    return r;
}
template <typename T, std::size_t D>
Vector<T, D> operator-(const Vector<T, D>& a, const Vector<T, D>& b) {
    Vector<T, D> r = a;
    r -= b;
    return r;
}
template <typename T, std::size_t D>
Vector<T, D> operator-(const Vector<T, D>& a) {
    Vector<T, D> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = -a[i];
    return r;
}
template <typename T, std::size_t D, typename S, typename = is_scalar_t<S>>
Vector<T, D>& operator*=(Vector<T, D>& a, const S& s) {
    for (std::size_t i = 0; i < D; ++i) a[i] = a[i] * s;
    return a;
}
template <typename T, std::size_t D, typename S, typename = is_scalar_t<S>>
Vector<T, D>& operator/=(Vector<T, D>& a, const S& s) {
    for (std::size_t i = 0; i < D; ++i) a[i] = a[i] / s;
    return a;
}
template <typename T, std::size_t D, typename S, typename = is_scalar_t<S>>
Vector<T, D> operator*(const Vector<T, D>& a, const S& s) {
    Vector<T, D> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = a[i] * s;
    return r;
}
template <typename T, std::size_t D, typename S, typename = is_scalar_t<S>>
Vector<T, D> operator*(const S& s, const Vector<T, D>& a) {
    Vector<T, D> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = s * a[i];
    return r;
}
template <typename T, std::size_t D, typename S, typename = is_scalar_t<S>>
Vector<T, D> operator/(const Vector<T, D>& a, const S& s) {
    Vector<T, D> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = a[i] / s;
    return r;
}
template <typename T, std::size_t D>
Vector<T, D> operator%(const Vector<T, D>& a, const Vector<T, D>& b) {
    Vector<T, D> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = a[i] % b[i];
    return r;
}

template <typename T, typename S, std::size_t D>
Vector<T, D> elementwiseProduct(const Vector<T, D>& a, const Vector<S, D>& b) {
    Vector<T, D> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = a[i] * b[i];
    return r;
}
template <typename T, typename S, std::size_t D>
Vector<T, D> elementwiseDivision(const Vector<T, D>& a, const Vector<S, D>& b) {
    Vector<T, D> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = a[i] / b[i];
    return r;
}

template <typename T, std::size_t D>
T sumOfSquares(const Vector<T, D>& a) {
    T r = T();
    for (std::size_t i = 0; i < D; ++i) r += a[i] * a[i];
    return r;
}

template <typename T>
Vector<T, 3> crossProduct(const Vector<T, 3>& a, const Vector<T, 3>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// --- comparisons ---------------------------------------------------------------

template <typename T, std::size_t D>
bool operator==(const Vector<T, D>& a, const Vector<T, D>& b) {
    for (std::size_t i = 0; i < D; ++i)
        if (!(a[i] == b[i])) return false;
    return true;
}
template <typename T, std::size_t D>
bool operator!=(const Vector<T, D>& a, const Vector<T, D>& b) {
    return !(a == b);
}
template <typename T, std::size_t D>
bool operator<(const Vector<T, D>& a, const Vector<T, D>& b) {
    for (std::size_t i = 0; i < D; ++i)
        if (!(a[i] < b[i])) return false;
    return true;
}

// <=, >, >= follow the same all-components reading (cell.h:1362 asserts
// cells.size() <= {32,32,32}).
template <typename T, std::size_t D>
bool operator<=(const Vector<T, D>& a, const Vector<T, D>& b) {
    for (std::size_t i = 0; i < D; ++i)
        if (!(a[i] <= b[i])) return false;
    return true;
}
template <typename T, std::size_t D>
bool operator>(const Vector<T, D>& a, const Vector<T, D>& b) {
    return b < a;
}
template <typename T, std::size_t D>
bool operator>=(const Vector<T, D>& a, const Vector<T, D>& b) {
    return b <= a;
}

template <typename T, std::size_t D>
std::ostream& operator<<(std::ostream& out, const Vector<T, D>& v) {
    out << "[";
    for (std::size_t i = 0; i < D; ++i) {
        if (i) out << ",";
        out << v[i];
    }
    return out << "]";
}

}  // namespace utils
}  // namespace allscale
