// Stand-in for allscale/utils/serializer.h. The reference only needs the
// trait (cell_test.cc:85-95) and the archive type names in store/load members
// (cell.h:164-300), which are never called on the path. TEST INFRASTRUCTURE
// ONLY (oracle).
#pragma once

#include <type_traits>

namespace allscale {
namespace utils {

struct trivially_serializable {};

class ArchiveWriter {
  public:
    template <typename T>
    void write(const T&);
};

class ArchiveReader {
  public:
    template <typename T>
    T read();
};

namespace detail {
template <typename T, typename = void>
struct has_store_load : std::false_type {};
template <typename T>
struct has_store_load<T, std::void_t<decltype(std::declval<const T&>().store(std::declval<ArchiveWriter&>())),
                                     decltype(T::load(std::declval<ArchiveReader&>()))>> : std::true_type {};
}  // namespace detail

template <typename T>
struct is_serializable
    : std::integral_constant<bool, std::is_base_of<trivially_serializable, T>::value || std::is_arithmetic<T>::value ||
                                       detail::has_store_load<T>::value> {};

}  // namespace utils
}  // namespace allscale
