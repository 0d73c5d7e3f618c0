// index_format.hpp -- the reference's on-disk FM-index format, read and
// written byte-for-byte, so that indexes built by either project load in both.
//
//   <dir>/C.vec, C1.vec          {u32 n, u32[n]}                   csafm.c:121-146, 252-276
//   <dir>/O.desp, Oi.desp        {u32 siz, n_desp, m_desp, u32[n_desp][m_desp]}  csafm.c:181-217
//   <dir>/O.count, Oi.count      {u32 n_count, m_count, u64[n_count][m_count]}   csafm.c:219-248
//   <dir>/S.vec, Si.vec, R.vec, Ri.vec {u32 siz, n, ratio, u32[n]} csafm.c:148-179
//   <dir>/X.vec, Xi.vec, B.vec, Bi.vec {u64 n, u64 dollar, u8[n]}  io.c:251-313
//   <dir>/index                  ">name start end" per chromosome  io.c:26-105
//   <dir>/config.txt             alphabet line, duplicate-strand line  io.c:317-362
//
// Occurrence-table semantics (FM_COMP_64, preprocess.c:74-130): column c of
// the table stands for BWT row c-1 (column 0 is a virtual row), the row
// holding '$' sets no bit, desp[b][q] counts b in columns < 64q and bit t of
// count[b][q] is column 64q+t.  get_O(b, m) = # of b in BWT rows 0..m-1.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace hpgbwt {

struct OccTable {              // comp_matrix (csafm.h:51-64)
  uint32_t siz = 0;            // n + 2
  uint32_t m = 0;              // blocks per symbol: ceil(siz / 64)
  std::vector<uint32_t> desp;  // [4][m]
  std::vector<uint64_t> count; // [4][m]
};

struct SampledVec {            // comp_vector (csafm.h:73-81)
  uint32_t siz = 0, n = 0, ratio = 0;
  std::vector<uint32_t> v;
};

struct Karyotype {             // exome (io.h:22-29)
  std::vector<std::string> name;
  std::vector<uint64_t> start, end, offset;  // offset has size()+1 entries
};

struct HostIndex {
  std::string alphabet;        // config.txt first line, e.g. "ACGT"
  bool duplicate_strand = false;
  uint32_t C[4] = {0, 0, 0, 0}, C1[4] = {0, 0, 0, 0};
  OccTable O, Oi;              // backward (text) and forward (reversed text)
  SampledVec S, Si;
  bool has_R = false;
  SampledVec R, Ri;
  Karyotype kar;
};

// All return "" on success, else an error message.
std::string read_host_index(const std::string& dir, bool inverse_sa, HostIndex* out);

std::string write_u32_vec(const std::string& path, const uint32_t* v, uint32_t n);
std::string write_sampled(const std::string& path, const SampledVec& s);
std::string write_occ(const std::string& dir, const std::string& name, const OccTable& o);
std::string write_text_vec(const std::string& path, const uint8_t* v, uint64_t n, uint64_t dollar);

// The alphabet order fixed by config.txt, with the complement of each code.
struct Alphabet {
  uint8_t code_of[256];  // 0xFF for characters outside the alphabet
  uint8_t comp[4];       // code -> code of the complementary base
  char chars[4];
};
std::string make_alphabet(const std::string& letters, Alphabet* a);

}  // namespace hpgbwt
