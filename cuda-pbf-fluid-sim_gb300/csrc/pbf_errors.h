// pbf_errors.h - bits of the device-side error word (host and device).
#pragma once

#include <cstdint>

namespace pbf {

// A decoupled look-back poll loop reached its iteration limit; the waiting
// block treated the predecessor as finished and returned.
constexpr uint32_t kErrLookbackTimeoutBit = 1u << 0;
// Non-finite particle state detected.
constexpr uint32_t kErrNonFiniteBit = 1u << 1;
// A tile's bulk copy into shared memory had not completed when the bounded
// wait for it gave up; that tile's results are not valid.
constexpr uint32_t kErrStageTimeoutBit = 1u << 2;
// Bits reported as a timeout.
constexpr uint32_t kErrTimeoutBits = kErrLookbackTimeoutBit | kErrStageTimeoutBit;

}  // namespace pbf
