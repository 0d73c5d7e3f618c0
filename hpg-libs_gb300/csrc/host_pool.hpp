// host_pool.hpp -- reusable page-locked host blocks for result sets (host_pool.cpp).
#pragma once

#include <cstddef>

namespace hpgbwt {

// Memory for a result array; release with host_pool_free (which also frees
// plain malloc'ed pointers).
void* host_pool_alloc(size_t bytes);
void host_pool_free(void* p);

}  // namespace hpgbwt
