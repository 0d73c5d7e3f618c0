// gpu_sa.hpp -- suffix array of a DNA text on the GPU (gpu_sa.cu), for the index builder.
#pragma once

#include <cstdint>
#include <string>

namespace hpgbwt {

// Suffix array of X (n codes 0..3) followed by a terminator, built on
// `device`: sa gets n+1 entries and sa[0] == n.  0, or -1 with *err set.
int gpu_suffix_array(const uint8_t* X, uint64_t n, int device, uint32_t* sa, std::string* err);

}  // namespace hpgbwt
