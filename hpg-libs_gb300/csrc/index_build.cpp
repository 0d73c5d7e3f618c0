// index_build.cpp -- FM-index builder writing the reference's on-disk format.
//
// Replaces bwt_generate_index_files (c/src/aligners/bwt/bwt.c:744-819).  The
// reference encodes the FASTA (search/io.c:107-209), builds the BWT with dbwt
// and then derives C (preprocess.c:44-72), O (preprocess.c:74-130) and the
// S/R samples by an LF walk over the BWT (preprocess.c:7-42); the same is
// repeated on the reversed text for Oi/Si/Ri.  Here the suffix array of each
// text is built once (SA-IS) and every table is read off it directly:
//   BWT row i   = X[SA[i]-1], '$' where SA[i] == 0
//   S[i/ratio]  = SA[i]   for rows i with i % ratio == 0
//   R[p/ratio]  = ISA[p]  for text positions p with p % ratio == 0
// which are the values the reference's walk stores.  Both directions are
// built concurrently.
#include <cuda_runtime.h>
#include <omp.h>
#include <sys/stat.h>

#include <cerrno>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gpu_sa.hpp"
#include "index_format.hpp"
#include "sais.hpp"

namespace hpgbwt {

namespace {

struct Fasta {
  std::vector<uint8_t> codes;
  Karyotype kar;
};

// Sequence lines are concatenated with their trailing newline removed; a '>'
// line opens a chromosome named by its first word (io.c:131-193).
std::string parse_fasta(const std::string& path, const Alphabet& a, Fasta* fa) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return "Error opening file: " + path;
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> buf((size_t)(sz > 0 ? sz : 0));
  size_t got = buf.empty() ? 0 : std::fread(buf.data(), 1, buf.size(), f);
  std::fclose(f);
  if (got != buf.size()) return "short read of " + path;

  fa->codes.clear();
  fa->codes.reserve(buf.size());
  fa->kar = Karyotype();
  fa->kar.offset.assign(1, 0);
  uint64_t partial = 0;
  bool open = false;
  auto close_chrom = [&]() {
    fa->kar.end.push_back(partial - 1);
    fa->kar.offset.push_back(fa->kar.offset.back() + partial);
    partial = 0;
  };
  size_t i = 0, n = buf.size();
  while (i < n) {
    size_t j = i;
    while (j < n && buf[j] != '\n') ++j;
    if (buf[i] == '>') {
      if (open) close_chrom();
      size_t k = i + 1;
      while (k < j && !std::isspace((unsigned char)buf[k])) ++k;
      fa->kar.name.emplace_back(buf.data() + i + 1, k - i - 1);
      fa->kar.start.push_back(0);
      open = true;
    } else {
      if (!open) return "sequence before the first '>' header in " + path;
      for (size_t k = i; k < j; ++k) {
        uint8_t c = a.code_of[(unsigned char)buf[k]];
        if (c == 0xFF) {
          char msg[96];
          std::snprintf(msg, sizeof msg, "character 0x%02x outside the index alphabet at byte %zu of ",
                        (unsigned)(unsigned char)buf[k], k);
          return msg + path;
        }
        fa->codes.push_back(c);
      }
      partial += j - i;
    }
    i = j + 1;
  }
  if (open) close_chrom();
  if (fa->codes.empty()) return "no sequence in " + path;
  return "";
}

struct Direction {
  std::vector<uint8_t> bwt;  // n+1 rows, 4 = '$'
  uint64_t dollar = 0;       // row holding '$'
  OccTable occ;
  SampledVec S, R;
};

// Every table of one direction from its suffix array (n+1 entries, sa[0] == n).
template <typename I>
void tables_from_sa(const std::vector<uint8_t>& X, const std::vector<I>& sa, uint32_t ratio, Direction* d) {
  const int64_t n = (int64_t)X.size();
  const int64_t rows = n + 1;

  d->bwt.resize((size_t)rows);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < rows; ++i) {
    int64_t p = (int64_t)sa[(size_t)i];
    d->bwt[(size_t)i] = p == 0 ? (uint8_t)4 : X[(size_t)(p - 1)];
  }
  for (int64_t i = 0; i < rows; ++i)
    if (sa[(size_t)i] == 0) {
      d->dollar = (uint64_t)i;
      break;
    }

  // Occurrence table: column c <-> row c-1, column 0 empty (preprocess.c:78-128).
  OccTable& o = d->occ;
  o.siz = (uint32_t)(n + 2);
  o.m = (o.siz + 63) / 64;
  o.desp.assign((size_t)4 * o.m, 0);
  o.count.assign((size_t)4 * o.m, 0);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < (int64_t)o.m; ++q) {
    uint64_t bits[4] = {0, 0, 0, 0};
    for (int t = 0; t < 64; ++t) {
      int64_t col = q * 64 + t;
      if (col == 0 || col > rows) continue;
      uint8_t b = d->bwt[(size_t)(col - 1)];
      if (b < 4) bits[b] |= (uint64_t)1 << t;
    }
    for (int b = 0; b < 4; ++b) o.count[(size_t)b * o.m + q] = bits[b];
  }
  for (int b = 0; b < 4; ++b) {
    uint32_t run = 0;
    for (uint32_t q = 0; q < o.m; ++q) {
      o.desp[(size_t)b * o.m + q] = run;
      run += (uint32_t)__builtin_popcountll(o.count[(size_t)b * o.m + q]);
    }
  }

  // SA samples by row and ISA samples by text position (preprocess.c:7-42).
  d->S.siz = d->R.siz = (uint32_t)rows;
  d->S.ratio = d->R.ratio = ratio;
  d->S.n = d->R.n = (uint32_t)((rows + ratio - 1) / ratio);
  d->S.v.assign(d->S.n, 0);
  d->R.v.assign(d->R.n, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < rows; i += ratio) d->S.v[(size_t)(i / ratio)] = (uint32_t)sa[(size_t)i];
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < rows; ++i) {
    int64_t p = (int64_t)sa[(size_t)i];
    if (p % ratio == 0) d->R.v[(size_t)(p / ratio)] = (uint32_t)i;
  }
}

template <typename I>
void build_direction(const std::vector<uint8_t>& X, uint32_t ratio, Direction* d) {
  std::vector<I> sa;
  suffix_array_dna<I>(X.data(), (int64_t)X.size(), sa);
  tables_from_sa<I>(X, sa, ratio, d);
}

void build_direction_any(const std::vector<uint8_t>& X, uint32_t ratio, Direction* d) {
  if ((int64_t)X.size() + 1 < ((int64_t)1 << 31))
    build_direction<int32_t>(X, ratio, d);
  else
    build_direction<int64_t>(X, ratio, d);
}

// The same with the suffix array built on a GPU.
std::string build_direction_gpu(const std::vector<uint8_t>& X, uint32_t ratio, int device, Direction* d) {
  std::vector<uint32_t> sa(X.size() + 1);
  std::string e;
  if (gpu_suffix_array(X.data(), X.size(), device, sa.data(), &e) != 0) return e;
  tables_from_sa<uint32_t>(X, sa, ratio, d);
  return "";
}

// BWT without the '$' row, as dbwt writes it into B.vec (dbwt.c:732-763).
std::vector<uint8_t> bwt_without_dollar(const Direction& d) {
  std::vector<uint8_t> out;
  out.reserve(d.bwt.size() - 1);
  for (size_t i = 0; i < d.bwt.size(); ++i)
    if (i != d.dollar) out.push_back(d.bwt[i]);
  return out;
}

std::string mkdir_p(const std::string& dir) {
  if (mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST) return "cannot create directory " + dir;
  return "";
}

}  // namespace

std::string build_index(const std::string& fasta, const std::string& outdir, uint32_t ratio, bool duplicate_strand,
                        const std::string& bases, int device) {
  if (ratio == 0) return "sampling ratio must be positive";
  Alphabet a;
  std::string e;
  if (!(e = make_alphabet(bases, &a)).empty()) return e;
  if (!(e = mkdir_p(outdir)).empty()) return e;
  Fasta fa;
  if (!(e = parse_fasta(fasta, a, &fa)).empty()) return e;
  std::vector<uint8_t>& X = fa.codes;
  const uint64_t total = X.size();
  if (duplicate_strand) {  // the reverse complement follows the text (bwt_commons.c:140-150)
    X.resize(2 * total);
    for (uint64_t i = 0; i < total; ++i) X[2 * total - 1 - i] = a.comp[X[i]];
  }
  if ((uint64_t)X.size() + 2 > 0xFFFFFFFFull) return "genome too large for 32-bit suffix-array entries";

  {  // config.txt (io.c:317-334)
    std::string path = outdir + "/config.txt";
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return "Error opening file: " + path;
    std::fprintf(f, "%s\n%s\n", bases.c_str(), duplicate_strand ? "1" : "0");
    std::fclose(f);
  }
  {  // index (io.c:83-105)
    std::string path = outdir + "/index";
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return "Error opening file: " + path;
    const Karyotype& k = fa.kar;
    for (size_t i = 0; i < k.name.size(); ++i)
      std::fprintf(f, ">%s %" PRIu64 " %" PRIu64 "\n", k.name[i].c_str(), k.start[i], k.end[i]);
    if (duplicate_strand)
      for (size_t i = k.name.size(); i-- > 0;)
        std::fprintf(f, ">%s %" PRIu64 " %" PRIu64 "\n", k.name[i].c_str(), k.start[i], k.end[i]);
    std::fclose(f);
  }

  std::vector<uint8_t> Xi(X.rbegin(), X.rend());
  Direction fw, bw;
  if (device >= 0) {  // suffix arrays on the GPU, one direction after the other
    if (!(e = build_direction_gpu(X, ratio, device, &bw)).empty()) return e;
    if (!(e = build_direction_gpu(Xi, ratio, device, &fw)).empty()) return e;
  } else {
#pragma omp parallel sections num_threads(2)
    {
#pragma omp section
      build_direction_any(X, ratio, &bw);
#pragma omp section
      build_direction_any(Xi, ratio, &fw);
    }
  }

  // C counts symbols of B only (preprocess.c:44-72); both directions load it.
  uint32_t C[4] = {0, 0, 0, 0}, C1[4];
  {
    uint64_t cnt[4] = {0, 0, 0, 0};
    for (uint8_t c : X) cnt[c]++;
    uint64_t run = 0;
    for (int b = 0; b < 4; ++b) {
      C[b] = (uint32_t)run;
      run += cnt[b];
    }
    for (int b = 0; b < 4; ++b) C1[b] = C[b] + 1;
  }

  if (!(e = write_text_vec(outdir + "/X.vec", X.data(), X.size(), 0)).empty()) return e;
  if (!(e = write_text_vec(outdir + "/Xi.vec", Xi.data(), Xi.size(), 0)).empty()) return e;
  {
    std::vector<uint8_t> B = bwt_without_dollar(bw);
    if (!(e = write_text_vec(outdir + "/B.vec", B.data(), B.size(), bw.dollar)).empty()) return e;
  }
  {
    std::vector<uint8_t> Bi = bwt_without_dollar(fw);
    if (!(e = write_text_vec(outdir + "/Bi.vec", Bi.data(), Bi.size(), fw.dollar)).empty()) return e;
  }
  if (!(e = write_u32_vec(outdir + "/C.vec", C, 4)).empty()) return e;
  if (!(e = write_u32_vec(outdir + "/C1.vec", C1, 4)).empty()) return e;
  if (!(e = write_occ(outdir, "O", bw.occ)).empty()) return e;
  if (!(e = write_occ(outdir, "Oi", fw.occ)).empty()) return e;
  if (!(e = write_sampled(outdir + "/S.vec", bw.S)).empty()) return e;
  if (!(e = write_sampled(outdir + "/R.vec", bw.R)).empty()) return e;
  if (!(e = write_sampled(outdir + "/Si.vec", fw.S)).empty()) return e;
  if (!(e = write_sampled(outdir + "/Ri.vec", fw.R)).empty()) return e;
  return "";
}

}  // namespace hpgbwt

extern "C" {

// Status-returning builder: 0 on success, -1 with a message in errbuf.
int hpg_bwt_build_index_on(const char* ref_file, const char* output_dir, unsigned int s_ratio,
                           int duplicate_strand, const char* bases, int device, char* errbuf, size_t errlen) {
  std::string e = hpgbwt::build_index(ref_file ? ref_file : "", output_dir ? output_dir : "", s_ratio,
                                      duplicate_strand != 0, bases ? bases : "ACGT", device);
  if (e.empty()) return 0;
  if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", e.c_str());
  return -1;
}

int hpg_bwt_build_index(const char* ref_file, const char* output_dir, unsigned int s_ratio, int duplicate_strand,
                        const char* bases, char* errbuf, size_t errlen) {
  return hpg_bwt_build_index_on(ref_file, output_dir, s_ratio, duplicate_strand, bases, -1, errbuf, errlen);
}

// bwt.h:287-289.  Like the reference, an unrecoverable error ends the process.
// The suffix arrays are built on GPU 0 when one is visible, else on the host.
void bwt_generate_index_files(char* ref_file, char* output_dir, unsigned int s_ratio, bool duplicate_strand,
                              char* bases) {
  char err[512];
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess) {
    cudaGetLastError();
    ndev = 0;
  }
  if (hpg_bwt_build_index_on(ref_file, output_dir, s_ratio, duplicate_strand ? 1 : 0, bases, ndev > 0 ? 0 : -1, err,
                             sizeof err) != 0) {
    std::fprintf(stderr, "bwt_generate_index_files: %s\n", err);
    std::exit(EXIT_FAILURE);
  }
}

}  // extern "C"
