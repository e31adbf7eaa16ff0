// No-op logging stand-in so the reference sources compile without spdlog.
// Test infrastructure only: the reference's LOG_* macros expand to these.
#pragma once
namespace spdlog {
namespace level { enum level_enum { trace, debug, info, warn, err, critical, off }; }
template <class... A> inline void trace(A&&...) {}
template <class... A> inline void debug(A&&...) {}
template <class... A> inline void info(A&&...) {}
template <class... A> inline void warn(A&&...) {}
template <class... A> inline void error(A&&...) {}
template <class... A> inline void critical(A&&...) {}
inline void set_level(level::level_enum) {}
}  // namespace spdlog
