// index_format.cpp -- reader/writer of the reference's on-disk FM-index files.
#include "index_format.hpp"

#include <cctype>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <memory>

namespace hpgbwt {

namespace {

struct File {
  FILE* f = nullptr;
  explicit File(const std::string& p, const char* mode) { f = std::fopen(p.c_str(), mode); }
  ~File() {
    if (f) std::fclose(f);
  }
};

template <typename T>
bool rd(FILE* f, T* v, size_t n = 1) {
  return std::fread(v, sizeof(T), n, f) == n;
}

template <typename T>
bool wr(FILE* f, const T* v, size_t n = 1) {
  return std::fwrite(v, sizeof(T), n, f) == n;
}

std::string read_u32_vec(const std::string& path, uint32_t* out4) {
  File fp(path, "rb");
  if (!fp.f) return "Error opening file: " + path;
  uint32_t n = 0;
  if (!rd(fp.f, &n) || n != 4) return "bad vector header in " + path;
  if (!rd(fp.f, out4, 4)) return "short read in " + path;
  return "";
}

std::string read_sampled(const std::string& path, SampledVec* s) {
  File fp(path, "rb");
  if (!fp.f) return "Error opening file: " + path;
  if (!rd(fp.f, &s->siz) || !rd(fp.f, &s->n) || !rd(fp.f, &s->ratio)) return "short header in " + path;
  if (s->ratio == 0) return "zero sampling ratio in " + path;
  s->v.resize(s->n);
  if (s->n && !rd(fp.f, s->v.data(), s->n)) return "short read in " + path;
  return "";
}

std::string read_occ(const std::string& dir, const std::string& name, OccTable* o) {
  {
    std::string path = dir + "/" + name + ".desp";
    File fp(path, "rb");
    if (!fp.f) return "Error opening file: " + path;
    uint32_t n_desp = 0;
    if (!rd(fp.f, &o->siz) || !rd(fp.f, &n_desp) || !rd(fp.f, &o->m)) return "short header in " + path;
    if (n_desp != 4) return "only 4-letter alphabets are supported: " + path;
    o->desp.resize((size_t)4 * o->m);
    if (!rd(fp.f, o->desp.data(), o->desp.size())) return "short read in " + path;
  }
  {
    std::string path = dir + "/" + name + ".count";
    File fp(path, "rb");
    if (!fp.f) return "Error opening file: " + path;
    uint32_t n_count = 0, m_count = 0;
    if (!rd(fp.f, &n_count) || !rd(fp.f, &m_count)) return "short header in " + path;
    if (n_count != 4 || m_count != o->m) return "count/desp shape mismatch in " + path;
    o->count.resize((size_t)4 * o->m);
    if (!rd(fp.f, o->count.data(), o->count.size())) return "short read in " + path;
  }
  if (o->siz < 2 || o->m != (o->siz + 63) / 64) return "inconsistent occurrence table " + name;
  return "";
}

std::string read_karyotype(const std::string& dir, Karyotype* k) {
  std::string path = dir + "/index";
  File fp(path, "r");
  if (!fp.f) return "Error opening file: " + path;
  k->name.clear();
  k->start.clear();
  k->end.clear();
  k->offset.assign(1, 0);
  char line[4096];
  while (std::fgets(line, sizeof line, fp.f)) {
    if (line[0] != '>') continue;
    // Name runs from after '>' to the first blank (io.c:47-56), then "start end".
    size_t j = 1;
    while (line[j] && line[j] != ' ' && line[j] != '\n') ++j;
    std::string nm(line + 1, j - 1);
    uintmax_t s = 0, e = 0;
    if (std::sscanf(line + j, " %ju %ju", &s, &e) != 2) return "bad karyotype line in " + path;
    k->name.push_back(nm);
    k->start.push_back(s);
    k->end.push_back(e);
    k->offset.push_back(k->offset.back() + (e - s + 1));
  }
  return "";
}

}  // namespace

std::string make_alphabet(const std::string& letters, Alphabet* a) {
  if (letters.size() != 4) return "only 4-letter alphabets are supported, got '" + letters + "'";
  std::memset(a->code_of, 0xFF, sizeof a->code_of);
  int pos[4] = {-1, -1, -1, -1};  // A C G T
  const char* acgt = "ACGT";
  for (int i = 0; i < 4; ++i) {
    char u = (char)std::toupper((unsigned char)letters[i]);
    a->chars[i] = u;
    a->code_of[(unsigned char)u] = (uint8_t)i;
    a->code_of[(unsigned char)std::tolower((unsigned char)u)] = (uint8_t)i;
    const char* p = std::strchr(acgt, u);
    if (!p || !*p) return "alphabet must be a permutation of ACGT, got '" + letters + "'";
    pos[p - acgt] = i;
  }
  for (int i = 0; i < 4; ++i)
    if (pos[i] < 0) return "alphabet must be a permutation of ACGT, got '" + letters + "'";
  // A<->T, C<->G (bwt_commons.c:87-90).
  a->comp[pos[0]] = (uint8_t)pos[3];
  a->comp[pos[3]] = (uint8_t)pos[0];
  a->comp[pos[1]] = (uint8_t)pos[2];
  a->comp[pos[2]] = (uint8_t)pos[1];
  return "";
}

std::string read_host_index(const std::string& dir, bool inverse_sa, HostIndex* out) {
  {
    std::string path = dir + "/config.txt";
    File fp(path, "r");
    if (!fp.f) return "Error opening file: " + path;
    char line[256] = {0};
    if (!std::fgets(line, sizeof line, fp.f)) return "empty " + path;
    size_t len = std::strlen(line);
    if (len && line[len - 1] == '\n') line[--len] = 0;
    out->alphabet = line;
    // The reference reads the duplicate-strand flag with fgets(buf, 1, ...),
    // which never reads a character, so it is always 0 (io.c:357-358).
    out->duplicate_strand = false;
  }
  std::string e;
  if (!(e = read_u32_vec(dir + "/C.vec", out->C)).empty()) return e;
  if (!(e = read_u32_vec(dir + "/C1.vec", out->C1)).empty()) return e;
  if (!(e = read_occ(dir, "O", &out->O)).empty()) return e;
  if (!(e = read_occ(dir, "Oi", &out->Oi)).empty()) return e;
  if (!(e = read_sampled(dir + "/S.vec", &out->S)).empty()) return e;
  if (!(e = read_sampled(dir + "/Si.vec", &out->Si)).empty()) return e;
  out->has_R = inverse_sa;
  if (inverse_sa) {
    if (!(e = read_sampled(dir + "/R.vec", &out->R)).empty()) return e;
    if (!(e = read_sampled(dir + "/Ri.vec", &out->Ri)).empty()) return e;
  }
  if (!(e = read_karyotype(dir, &out->kar)).empty()) return e;
  if (out->O.siz != out->Oi.siz) return "O and Oi sizes differ";
  if (out->S.siz + 1 != out->O.siz || out->Si.siz != out->S.siz) return "S and O sizes disagree";
  return "";
}

std::string write_u32_vec(const std::string& path, const uint32_t* v, uint32_t n) {
  File fp(path, "wb");
  if (!fp.f) return "Error opening file: " + path;
  if (!wr(fp.f, &n) || !wr(fp.f, v, n)) return "write failed: " + path;
  return "";
}

std::string write_sampled(const std::string& path, const SampledVec& s) {
  File fp(path, "wb");
  if (!fp.f) return "Error opening file: " + path;
  if (!wr(fp.f, &s.siz) || !wr(fp.f, &s.n) || !wr(fp.f, &s.ratio)) return "write failed: " + path;
  if (s.n && !wr(fp.f, s.v.data(), s.n)) return "write failed: " + path;
  return "";
}

std::string write_occ(const std::string& dir, const std::string& name, const OccTable& o) {
  uint32_t four = 4;
  {
    std::string path = dir + "/" + name + ".desp";
    File fp(path, "wb");
    if (!fp.f) return "Error opening file: " + path;
    if (!wr(fp.f, &o.siz) || !wr(fp.f, &four) || !wr(fp.f, &o.m) || !wr(fp.f, o.desp.data(), o.desp.size()))
      return "write failed: " + path;
  }
  {
    std::string path = dir + "/" + name + ".count";
    File fp(path, "wb");
    if (!fp.f) return "Error opening file: " + path;
    if (!wr(fp.f, &four) || !wr(fp.f, &o.m) || !wr(fp.f, o.count.data(), o.count.size()))
      return "write failed: " + path;
  }
  return "";
}

std::string write_text_vec(const std::string& path, const uint8_t* v, uint64_t n, uint64_t dollar) {
  File fp(path, "wb");
  if (!fp.f) return "Error opening file: " + path;
  if (!wr(fp.f, &n) || !wr(fp.f, &dollar) || (n && !wr(fp.f, v, n))) return "write failed: " + path;
  return "";
}

}  // namespace hpgbwt
