// spdlog/spdlog.h stand-in - TEST INFRASTRUCTURE for oracle/_ref (see
// oracle/ref_shim/Eigen/Core): the reference's CPU sweep only logs through
// these calls; here they discard their arguments.
#pragma once

namespace spdlog {

template <typename... Args>
inline void trace(const Args &...) {}
template <typename... Args>
inline void debug(const Args &...) {}
template <typename... Args>
inline void info(const Args &...) {}
template <typename... Args>
inline void warn(const Args &...) {}
template <typename... Args>
inline void error(const Args &...) {}

}  // namespace spdlog
