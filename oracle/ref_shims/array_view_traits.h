/* Test-oracle stand-in for SuperDCA/include/Array_view_forward.h.
 *
 * The reference header declares its Array_view type traits with a
 * `template<> template<...>` prefix that current g++ rejects ("too many
 * template-parameter-lists").  This file declares the same traits with the
 * standard partial-specialisation syntax and claims the header's include
 * guard, so the rest of the reference headers compile unchanged.  It is
 * force-included (-include) by the oracle/_ref build only. */
#ifndef SUPERDCA_ARRAY_VIEW_FORWARD_H
#define SUPERDCA_ARRAY_VIEW_FORWARD_H

#include <cstddef>
#include "Math_utility.hpp"

namespace superdca {

template <typename T, std::size_t Extent = 0, std::size_t Rank = rank<T>::value + 1>
class Array_view;

template <typename T, std::size_t Extent>
struct rank<Array_view<T, Extent>> : std::integral_constant<std::size_t, rank<T>::value + 1> {};

template <typename T, std::size_t Extent>
struct extent<Array_view<T, Extent>, 0> : std::integral_constant<std::size_t, Extent> {};

template <typename T, std::size_t Extent, unsigned N>
struct extent<Array_view<T, Extent>, N> : std::integral_constant<std::size_t, extent<T, N - 1>::value> {};

template <typename T, std::size_t Extent>
struct scalar_type<Array_view<T, Extent>> { using type = typename scalar_type<T>::type; };

template <typename T, std::size_t Extent>
struct recursive_extent<Array_view<T, Extent>>
    : std::integral_constant<std::size_t, extent<Array_view<T, Extent>>::value * recursive_extent<T>::value> {
    enum { current_level = extent<Array_view<T, Extent>>::value };
    enum { sub_level = recursive_extent<T>::value };
};

} // namespace superdca

#endif
