// Inert stand-ins for Boost archives: the traced staple-move path never
// serialises; these only let the reference's translation units compile.
#pragma once
#include <algorithm>
#include <cmath>
#include <istream>
#include <ostream>
#include <stdexcept>
namespace boost { namespace archive {
struct stub_iarchive {
    explicit stub_iarchive(std::istream&) {}
    template <typename T> stub_iarchive& operator>>(T&) {
        throw std::runtime_error("archive input unavailable in the oracle build");
    }
    template <typename T> stub_iarchive& operator&(T& t) { return *this >> t; }
};
struct stub_oarchive {
    explicit stub_oarchive(std::ostream&) {}
    template <typename T> stub_oarchive& operator<<(const T&) {
        throw std::runtime_error("archive output unavailable in the oracle build");
    }
    template <typename T> stub_oarchive& operator&(const T& t) { return *this << t; }
};
using text_iarchive = stub_iarchive;
using text_oarchive = stub_oarchive;
using binary_iarchive = stub_iarchive;
using binary_oarchive = stub_oarchive;
}} // namespace boost::archive
namespace boost { namespace serialization { class access {}; } }
