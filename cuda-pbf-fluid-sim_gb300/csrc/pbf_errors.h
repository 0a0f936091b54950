// pbf_errors.h - bits of the device-side error word (host and device).
#pragma once

#include <cstdint>

namespace pbf {

// A decoupled look-back poll loop reached its iteration limit; the waiting
// block treated the predecessor as finished and returned.
constexpr uint32_t kErrLookbackTimeoutBit = 1u << 0;
// Non-finite particle state detected.
constexpr uint32_t kErrNonFiniteBit = 1u << 1;

}  // namespace pbf
