// n! by repeated multiplication (exact for n <= 22 in double).
#pragma once
namespace boost { namespace math {
template <typename T> inline T factorial(unsigned n) {
    T r = 1;
    for (unsigned i = 2; i <= n; ++i) r *= static_cast<T>(i);
    return r;
}
}} // namespace boost::math
