// sais.hpp -- suffix array by induced sorting (SA-IS).
//
// Own implementation of the published algorithm of G. Nong, S. Zhang and
// W. H. Chan, "Two Efficient Algorithms for Linear Time Suffix Array
// Construction", IEEE Trans. Computers 60(10), 2011.  The index builder uses
// it to obtain the suffix array of the encoded reference, from which the BWT,
// the occurrence table and the SA/ISA samples are derived; the reference
// builds the same BWT with Okanohara-Sadakane's direct induced-sorting BWT
// (c/src/aligners/bwt/dbwt/dbwt.c:357).  A suffix array is unique for a given
// text, so every correct construction yields byte-identical index files.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace hpgbwt {
namespace sais_detail {

// Suffix types: 1 = S (smaller than its successor), 0 = L.
template <typename C, typename I>
inline void classify(const C* T, I n, std::vector<uint8_t>& t) {
  t.assign((size_t)n, 0);
  t[n - 1] = 1;
  for (I i = n - 2; i >= 0; --i)
    t[i] = (T[i] < T[i + 1] || (T[i] == T[i + 1] && t[i + 1])) ? 1 : 0;
}

template <typename I>
inline bool is_lms(const std::vector<uint8_t>& t, I i) {
  return i > 0 && t[i] && !t[i - 1];
}

// Bucket boundaries per symbol: heads (first slot) or tails (one past last).
template <typename C, typename I>
inline void buckets(const C* T, I n, I K, std::vector<I>& b, bool tails) {
  b.assign((size_t)K, 0);
  for (I i = 0; i < n; ++i) b[(size_t)T[i]]++;
  I sum = 0;
  for (I c = 0; c < K; ++c) {
    I cnt = b[c];
    sum += cnt;
    b[c] = tails ? sum : sum - cnt;
  }
}

template <typename C, typename I>
inline void induce(const C* T, I* SA, I n, I K, const std::vector<uint8_t>& t, std::vector<I>& b) {
  // L-type suffixes, scanning left to right from the bucket heads.
  buckets(T, n, K, b, false);
  for (I i = 0; i < n; ++i) {
    I j = SA[i] - 1;
    if (SA[i] > 0 && !t[j]) SA[b[(size_t)T[j]]++] = j;
  }
  // S-type suffixes, scanning right to left from the bucket tails.
  buckets(T, n, K, b, true);
  for (I i = n - 1; i >= 0; --i) {
    I j = SA[i] - 1;
    if (SA[i] > 0 && t[j]) SA[--b[(size_t)T[j]]] = j;
  }
}

// T[0..n-1] over [0, K), with T[n-1] the unique smallest symbol.
template <typename C, typename I>
void sais(const C* T, I* SA, I n, I K) {
  std::vector<uint8_t> t;
  classify(T, n, t);
  std::vector<I> b;

  // 1. Sort the LMS substrings: seed their tails, then induce.
  buckets(T, n, K, b, true);
  std::fill(SA, SA + n, (I)-1);
  for (I i = 1; i < n; ++i)
    if (is_lms(t, i)) SA[--b[(size_t)T[i]]] = i;
  induce(T, SA, n, K, t, b);

  // 2. Name the sorted LMS substrings; equal substrings share a name.
  I n1 = 0;
  for (I i = 0; i < n; ++i)
    if (is_lms(t, SA[i])) SA[n1++] = SA[i];
  if (n1 < n) std::fill(SA + n1, SA + n, (I)-1);
  I name = 0, prev = -1;
  for (I i = 0; i < n1; ++i) {
    I pos = SA[i];
    bool differ = false;
    for (I d = 0; d < n; ++d) {
      if (prev == -1 || T[pos + d] != T[prev + d] || t[pos + d] != t[prev + d]) {
        differ = true;
        break;
      }
      if (d > 0 && (is_lms(t, pos + d) || is_lms(t, prev + d))) break;
    }
    if (differ) {
      ++name;
      prev = pos;
    }
    SA[n1 + pos / 2] = name - 1;
  }
  for (I i = n - 1, j = n - 1; i >= n1; --i)
    if (SA[i] >= 0) SA[j--] = SA[i];

  // 3. Sort the reduced string, recursively while names repeat.
  I* s1 = SA + n - n1;
  I* SA1 = SA;
  if (name < n1) {
    sais<I, I>(s1, SA1, n1, name);
  } else {
    for (I i = 0; i < n1; ++i) SA1[s1[i]] = i;
  }

  // 4. Place the LMS suffixes in their final order and induce the rest.
  buckets(T, n, K, b, true);
  for (I i = 1, j = 0; i < n; ++i)
    if (is_lms(t, i)) s1[j++] = i;
  for (I i = 0; i < n1; ++i) SA1[i] = s1[SA1[i]];
  if (n1 < n) std::fill(SA + n1, SA + n, (I)-1);
  for (I i = n1 - 1; i >= 0; --i) {
    I j = SA[i];
    SA[i] = -1;
    SA[--b[(size_t)T[j]]] = j;
  }
  induce(T, SA, n, K, t, b);
}

}  // namespace sais_detail

// Suffix array of codes[0..n-1] (values 0..3) followed by a unique smallest
// terminator: sa has n+1 entries and sa[0] == n.
template <typename I>
void suffix_array_dna(const uint8_t* codes, int64_t n, std::vector<I>& sa) {
  std::vector<uint8_t> T((size_t)n + 1);
  for (int64_t i = 0; i < n; ++i) T[(size_t)i] = (uint8_t)(codes[i] + 1);
  T[(size_t)n] = 0;
  sa.assign((size_t)n + 1, 0);
  sais_detail::sais<uint8_t, I>(T.data(), sa.data(), (I)(n + 1), (I)5);
}

}  // namespace hpgbwt
