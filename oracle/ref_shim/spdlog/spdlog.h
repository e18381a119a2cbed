// Stand-in for spdlog (test infrastructure for oracle/_ref): logging calls compile and do nothing.
#pragma once
#include <fmt/format.h>

namespace spdlog {
template <typename... A> inline void trace(A&&...) {}
template <typename... A> inline void debug(A&&...) {}
template <typename... A> inline void info(A&&...) {}
template <typename... A> inline void warn(A&&...) {}
template <typename... A> inline void error(A&&...) {}
template <typename... A> inline void critical(A&&...) {}
namespace level { enum level_enum { trace, debug, info, warn, err, critical, off }; }
inline void set_level(level::level_enum) {}
}
