// Device status bits, OR-ed into a context's (or model's) status word.
#pragma once
#include <cstdint>

namespace mptc {

constexpr uint32_t kDevTimeout = 1u;  // a bounded device-side wait expired; results invalid

}  // namespace mptc
