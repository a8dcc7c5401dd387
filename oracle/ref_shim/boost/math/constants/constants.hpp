// Stand-in for boost/math/constants/constants.hpp with the five constants
// kazen_proto's closure math uses (pi, two_pi, half_pi, one_div_pi,
// one_div_root_pi), each the correctly rounded value of its type as Boost
// defines them. TEST INFRASTRUCTURE: used only to build the reference-code
// harness under oracle/_ref.
#pragma once

namespace boost {
namespace math {
namespace constants {
template <class T> constexpr T pi() { return static_cast<T>(3.141592653589793238462643383279502884L); }
template <class T> constexpr T two_pi() { return static_cast<T>(6.283185307179586476925286766559005768L); }
template <class T> constexpr T half_pi() { return static_cast<T>(1.570796326794896619231321691639751442L); }
template <class T> constexpr T one_div_pi() { return static_cast<T>(0.318309886183790671537767526745028724L); }
template <class T> constexpr T one_div_root_pi() { return static_cast<T>(0.564189583547756286948079451560772586L); }
}  // namespace constants
}  // namespace math
}  // namespace boost
