// search_core.cuh -- per-thread forms of the reference search loops, used by
// the plain kernels (one thread per read and strand).
//
//   exact_bwd / exact_fwd ....... BWExactSearchBackward/Forward (search/search.h:9-65)
//   vector_bwd / vector_fwd ..... BWExactSearchVectorBackward/Forward (search/search.c:1407-1489)
//   search1_helper .............. BWSearch1VectorHelper (search/search.c:1491-1709)
//
// The helper keeps one mutable result cursor and appends copies of it, as the
// reference does, so the error fields of every hit (including the
// base/position quirk of search.c:1556) and the emission order match.
#pragma once

#include "fm_device.cuh"

namespace hpgbwt {

// Packed hit metadata: dir | nm<<1 | kind<<2 | base<<4 | (uint16)err_pos<<16.
__host__ __device__ __forceinline__ uint32_t pack_meta(uint32_t dir, uint32_t nm, uint32_t kind, uint32_t base,
                                                       int32_t err_pos) {
  return (dir & 1u) | ((nm & 1u) << 1) | ((kind & 3u) << 2) | ((base & 0xFFu) << 4) |
         ((uint32_t)(uint16_t)(int16_t)err_pos << 16);
}

struct Cursor {
  uint32_t dir, nm, kind, base;
  int32_t err_pos;
  uint32_t k, l;
  __device__ __forceinline__ uint32_t meta() const {
    return nm ? pack_meta(dir, 1, kind, base, err_pos) : pack_meta(dir, 0, 0, 0, 0);
  }
};

#ifdef __CUDACC__

// Continue a backward search over W[pos..start]; true if the interval survives.
__device__ __forceinline__ bool exact_bwd(const DevIndex& X, View v, const uint8_t* W, int pos, int start,
                                          uint32_t& k, uint32_t& l, uint32_t& sectors) {
  for (int i = pos; i >= start; --i) {
    sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
    bw_step(X, v, W[i], k, l);
    if (k > l) return false;
  }
  return k <= l;
}

__device__ __forceinline__ bool exact_fwd(const DevIndex& X, View v, const uint8_t* W, int pos, int end,
                                          uint32_t& k, uint32_t& l, uint32_t& sectors) {
  for (int i = pos; i <= end; ++i) {
    sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
    bw_step(X, v, W[i], k, l);
    if (k > l) return false;
  }
  return k <= l;
}

__device__ __forceinline__ int64_t isize(uint2 v) { return (int64_t)v.y - (int64_t)v.x; }

// Vector searches; the vector element for read position j lives at vec[j * stride].
__device__ __forceinline__ void vector_bwd(const DevIndex& X, View v, const uint8_t* W, int len, uint2* vec,
                                           size_t stride, uint32_t& sectors) {
  uint32_t k = 0, l = X.top;
  int i = len - 1;
  for (; i >= 0; --i) {
    sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
    bw_step(X, v, W[i], k, l);
    vec[(size_t)i * stride] = make_uint2(k, l);
    if (k > l) {
      --i;
      break;
    }
  }
  for (; i >= 0; --i) vec[(size_t)i * stride] = make_uint2(k, l);
}

__device__ __forceinline__ void vector_fwd(const DevIndex& X, View v, const uint8_t* W, int len, uint2* vec,
                                           size_t stride, uint32_t& sectors) {
  uint32_t k = 0, l = X.top;
  int i = 0;
  for (; i < len; ++i) {
    sectors += ((k >> 6) == (l >> 6)) ? 1u : 2u;
    bw_step(X, v, W[i], k, l);
    vec[(size_t)i * stride] = make_uint2(k, l);
    if (k > l) {
      ++i;
      break;
    }
  }
  for (; i < len; ++i) vec[(size_t)i * stride] = make_uint2(k, l);
}

// The helper for one strand.  `emit(cursor)` appends a hit and returns false
// when the list is full, which ends the helper (search/results.h:100-101).
// Returns true on overflow.
template <typename Emit>
__device__ bool search1_helper(const DevIndex& X, const uint8_t* W, int len, const uint2* vk, const uint2* vki,
                               size_t stride, View B, View F, Emit& emit, uint32_t& sectors) {
  const int start = 0, end = len - 1;
  const int n = end - start;
  int half = n / 2;
  Cursor c;
  c.dir = 0;
  c.nm = 0;
  c.kind = 0;
  c.base = 0;
  c.err_pos = 0;

  const uint2 v0 = vk[0];
  if (v0.x <= v0.y) {
    c.k = v0.x;
    c.l = v0.y;
    if (!emit(c)) return true;
  }
  c.nm = 1;
  c.kind = 0;
  c.base = 0xFF;
  c.err_pos = start;

  int64_t res = isize(v0), res_last;
  uint2 v = vk[1 * stride];
  res_last = res;
  res = isize(v);
  if (res != res_last) {
    c.k = v.x;
    c.l = v.y;
    c.kind = 1;  // DELETION
    c.base = 0xFF;
    c.err_pos = start;
    if (!emit(c)) return true;
    const uint32_t bw = W[start];
    for (uint32_t b = 0; b < 4; ++b) {
      uint32_t ka = v.x, la = v.y;
      sectors += ((ka >> 6) == (la >> 6)) ? 1u : 2u;
      bw_step(X, B, b, ka, la);
      if (ka > la) continue;
      if (b != bw) {
        c.k = ka;
        c.l = la;
        c.kind = 2;  // MISMATCH, err_pos kept
        c.base = b;
        if (!emit(c)) return true;
      }
      sectors += ((ka >> 6) == (la >> 6)) ? 1u : 2u;
      bw_step(X, B, bw, ka, la);
      if (ka <= la) {
        c.k = ka;
        c.l = la;
        c.kind = 3;  // stored as (kind 3, base INSERTION, position b) by search.c:1556
        c.base = 3;
        c.err_pos = (int32_t)b;
        if (!emit(c)) return true;
      }
    }
  }

  for (int i = start + 2, j = 2; j <= half; ++i, ++j) {
    res_last = res;
    v = vk[(size_t)j * stride];
    res = isize(v);
    if (res == res_last) continue;
    c.kind = 1;
    c.base = 0xFF;
    c.err_pos = i - 1;
    {
      uint32_t k = v.x, l = v.y;
      if (exact_bwd(X, B, W, i - 2, start, k, l, sectors)) {
        c.k = k;
        c.l = l;
        if (!emit(c)) return true;
      }
    }
    const uint32_t wi = W[i - 1];
    for (uint32_t b = 0; b < 4; ++b) {
      uint32_t ka = v.x, la = v.y;
      sectors += ((ka >> 6) == (la >> 6)) ? 1u : 2u;
      bw_step(X, B, b, ka, la);
      if (ka > la) continue;
      c.kind = 3;  // INSERTION, err_pos kept
      c.base = b;
      {
        uint32_t k = ka, l = la;
        if (exact_bwd(X, B, W, i - 1, start, k, l, sectors)) {
          c.k = k;
          c.l = l;
          if (!emit(c)) return true;
        }
      }
      if (b != wi) {
        c.kind = 2;  // MISMATCH
        uint32_t k = ka, l = la;
        if (exact_bwd(X, B, W, i - 2, start, k, l, sectors)) {
          c.k = k;
          c.l = l;
          if (!emit(c)) return true;
        }
      }
    }
  }

  half--;
  c.dir = 1;
  v = vki[(size_t)n * stride];
  res = isize(v);
  res_last = res;
  v = vki[(size_t)(n - 1) * stride];
  res = isize(v);
  if (res != res_last) {
    c.k = v.x;
    c.l = v.y;
    c.kind = 1;
    c.base = 0xFF;
    c.err_pos = end;
    if (!emit(c)) return true;
    const uint32_t bw = W[end];
    for (uint32_t b = 0; b < 4; ++b) {
      uint32_t ka = v.x, la = v.y;
      sectors += ((ka >> 6) == (la >> 6)) ? 1u : 2u;
      bw_step(X, F, b, ka, la);
      if (ka > la) continue;
      if (b != bw) {
        c.k = ka;
        c.l = la;
        c.kind = 2;
        c.base = b;
        if (!emit(c)) return true;
      }
      sectors += ((ka >> 6) == (la >> 6)) ? 1u : 2u;
      bw_step(X, F, bw, ka, la);
      if (ka <= la) {
        c.k = ka;
        c.l = la;
        c.kind = 3;
        c.base = b;
        if (!emit(c)) return true;
      }
    }
  }

  for (int i = end - 2, j = n - 2; j >= half; --i, --j) {
    res_last = res;
    v = vki[(size_t)j * stride];
    res = isize(v);
    if (res == res_last) continue;
    c.kind = 1;
    c.base = 0xFF;
    c.err_pos = i + 1;
    {
      uint32_t k = v.x, l = v.y;
      if (exact_fwd(X, F, W, i + 2, end, k, l, sectors)) {
        c.k = k;
        c.l = l;
        if (!emit(c)) return true;
      }
    }
    const uint32_t wi = W[i + 1];
    for (uint32_t b = 0; b < 4; ++b) {
      uint32_t ka = v.x, la = v.y;
      sectors += ((ka >> 6) == (la >> 6)) ? 1u : 2u;
      bw_step(X, F, b, ka, la);
      if (ka > la) continue;
      c.kind = 3;
      c.base = b;
      {
        uint32_t k = ka, l = la;
        if (exact_fwd(X, F, W, i + 1, end, k, l, sectors)) {
          c.k = k;
          c.l = l;
          if (!emit(c)) return true;
        }
      }
      if (b != wi) {
        c.kind = 2;
        uint32_t k = ka, l = la;
        if (exact_fwd(X, F, W, i + 2, end, k, l, sectors)) {
          c.k = k;
          c.l = l;
          if (!emit(c)) return true;
        }
      }
    }
  }
  return false;
}

#endif  // __CUDACC__

}  // namespace hpgbwt
