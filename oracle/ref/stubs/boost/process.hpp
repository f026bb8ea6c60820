// The live-viewer child process is never started by the oracle build.
#pragma once
#include <chrono>
#include <string>
namespace boost { namespace process {
struct child { template <typename... A> explicit child(A&&...) {} };
inline std::string search_path(const std::string& s) { return s; }
struct std_out_t { template <typename T> std_out_t operator>(const T&) const { return *this; } };
static const std_out_t std_out {};
}} // namespace boost::process
