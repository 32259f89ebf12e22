// Stand-in for boost::math::legendre_p (oracle build only; Boost.Math is not
// part of the reference tree). Bonnet's recurrence in the order Boost.Math's
// legendre_p / legendre_next publish: P_0 = 1, P_1 = x,
// P_{n+1} = ((2n+1) x P_n - n P_{n-1}) / (n+1), P_{-l-1} = P_l, and a domain
// error outside [-1, 1].
#pragma once
#include <stdexcept>
#include <utility>

namespace boost {
namespace math {
template <class T> T legendre_p(int l, T x) {
    if (x < -1 || x > 1) throw std::domain_error("The Legendre Polynomial is defined for -1 <= x <= 1");
    if (l < 0) l = -l - 1;
    T p0 = 1, p1 = x;
    if (l == 0) return p0;
    unsigned n = 1;
    while (n < static_cast<unsigned>(l)) {
        std::swap(p0, p1);
        p1 = ((2 * n + 1) * x * p0 - n * p1) / (n + 1);
        ++n;
    }
    return p1;
}
}  // namespace math
}  // namespace boost
