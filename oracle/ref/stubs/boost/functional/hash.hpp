// Stand-in for the one Boost hashing facility the reference's headers use.
// Only unordered_map bucket order depends on it; no sampling decision does.
#pragma once
#include <cstddef>
#include <cmath>
#include <functional>
namespace boost {
template <typename T>
inline std::size_t hash_value(const T& v) { return std::hash<T>{}(v); }
template <typename T>
inline void hash_combine(std::size_t& seed, const T& v) {
    seed ^= std::hash<T>{}(v) + 0x9e3779b97f4a7c15ull + (seed << 6) + (seed >> 2);
}
} // namespace boost
