// Stand-in for allscale/utils/printer/vectors.h: printing of std::vector
// (init_properties.h:48-49 prints vectors of Vector3). TEST INFRASTRUCTURE
// ONLY (oracle).
#pragma once

#include <iostream>
#include <vector>

#include "allscale/utils/vector.h"

namespace std {
template <typename T>
ostream& operator<<(ostream& out, const vector<T>& v) {
    out << "[";
    for (size_t i = 0; i < v.size(); ++i) {
        if (i) out << ",";
        out << v[i];
    }
    return out << "]";
}
}  // namespace std
