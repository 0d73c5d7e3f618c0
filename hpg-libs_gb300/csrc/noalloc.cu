// noalloc.cu -- BWSearch1 for callers that cannot allocate device memory.
//
// bwt_gpu_search1_noalloc runs the plain one-thread-per-(read, strand)
// BWSearch1 search without any device allocation of its own.  Its per-thread
// scratch (the read codes and the two interval vectors of the helper) lives in
// one file-scope __device__ array of fixed size, which every GPU that has run
// a call holds until the process exits.
//
// Host code cannot use the array's name as a device address (on the host it
// names a stand-in object), so the address is looked up with
// cudaGetSymbolAddress once per device, with that device current, on the
// first call made on that device.  Under CUDA's lazy module loading (the
// default since CUDA 12.2) the array itself comes into being at that same
// moment, when the runtime loads this file's module: the first call on a
// device is the one that reserves the 16 MiB, and later calls allocate
// nothing.  That first call should therefore come before another allocator
// takes the device's free memory, and before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "hpg_bwt.h"
#include "kernels.cuh"
#include "search_core.cuh"

namespace hpgbwt {

DevIndex engine_dev_index(void* engine);
const uint8_t* engine_code_table(void* engine);
int engine_device_of(void* engine);
void* engine_stream_of(void* engine);

namespace {

// 16 MiB per device: per-thread read codes plus the two interval vectors.
constexpr size_t kNoAllocScratchBytes = 16u << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Scratch layout for T threads with reads of at most len_cap bases:
// [codes: T * len_cap bytes, 256-aligned][vectors: 2 * len_cap * T uint2].
inline size_t scratch_need(size_t T, size_t len_cap) { return align256(T * len_cap) + 2 * len_cap * T * sizeof(uint2); }

__global__ void __launch_bounds__(128)
    search1_noalloc_kernel(DevIndex X, const uint8_t* __restrict__ table, const uint8_t* __restrict__ ascii,
                           const uint64_t* __restrict__ offs, uint32_t n_reads, uint32_t len_cap,
                           uint32_t max_results, unsigned char* __restrict__ scratch, hpg_hit_t* __restrict__ hits,
                           uint32_t* __restrict__ counts, uint8_t* __restrict__ truncated) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t T = 2 * n_reads;
  if (t >= T) return;
  const uint32_t read = t >> 1, strand = t & 1;
  const uint64_t b = offs[read], e = offs[read + 1];
  // Offsets that run backwards, or a read longer than len_cap, get no hits;
  // the length is narrowed to int only after that check.
  const bool span_ok = e >= b && e - b <= (uint64_t)len_cap;
  const int len = span_ok ? (int)(e - b) : 0;
  uint8_t* W = scratch + (size_t)t * len_cap;
  uint2* vecs = reinterpret_cast<uint2*>(scratch + align256((size_t)T * len_cap));
  bool ok = span_ok && len >= 3;
  for (int i = 0; ok && i < len; ++i) {
    const uint8_t c = table[ascii[b + i]];
    ok = c != 0xFF;
    W[i] = c;
  }
  uint32_t cnt = 0, sectors = 0;
  bool trunc = false;
  if (ok) {
    const View B = strand ? View{1, 1} : View{0, 0};
    const View F = strand ? View{0, 1} : View{1, 0};
    uint2* vB = vecs + t;
    uint2* vF = vecs + (size_t)len_cap * T + t;
    vector_bwd(X, B, W, len, vB, T, sectors);
    vector_fwd(X, F, W, len, vF, T, sectors);
    auto emit = [&](const Cursor& c) -> bool {
      if (cnt >= max_results) {
        trunc = true;
        return false;
      }
      const uint32_t m = c.meta();
      hpg_hit_t h;
      h.read = read;
      h.strand = (uint8_t)strand;
      h.dir = (uint8_t)(m & 1u);
      h.nm = (uint8_t)((m >> 1) & 1u);
      h.err_kind = (uint8_t)((m >> 2) & 3u);
      h.err_base = (uint8_t)((m >> 4) & 0xFFu);
      h.pad0 = 0;
      h.err_pos = (int16_t)(uint16_t)(m >> 16);
      h.pad1 = 0;
      h.k = (int64_t)c.k;
      h.l = (int64_t)c.l;
      hits[(size_t)t * max_results + cnt] = h;
      ++cnt;
      return true;
    };
    search1_helper(X, W, len, vB, vF, T, B, F, emit, sectors);
  }
  counts[t] = cnt;
  truncated[t] = trunc ? 1 : 0;
}

// The array's device address for `device`, looked up once per device.
void* scratch_address(int device, std::string* err) {
  if (device < 0 || device >= kMaxDevices) {
    *err = "device ordinal out of range";
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_addr[device]) {
    int prev = -1;
    cudaGetDevice(&prev);
    cudaError_t ce = cudaSetDevice(device);
    void* p = nullptr;
    if (ce == cudaSuccess) ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    if (ce != cudaSuccess || !p) {
      *err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(ce);
      return nullptr;
    }
    g_scratch_addr[device] = p;
  }
  return g_scratch_addr[device];
}

thread_local std::string g_noalloc_error;

}  // namespace

}  // namespace hpgbwt

extern "C" {

const char* bwt_gpu_noalloc_last_error(void) { return hpgbwt::g_noalloc_error.c_str(); }

size_t bwt_gpu_noalloc_scratch_bytes(void) { return hpgbwt::kNoAllocScratchBytes; }

int bwt_gpu_search1_noalloc(bwt_index_t* index, const char* d_seqs, const uint64_t* d_offsets, size_t n_reads,
                            uint32_t max_len, uint32_t max_results, hpg_hit_t* d_hits, uint32_t* d_counts,
                            uint8_t* d_truncated, void* stream) {
  using namespace hpgbwt;
  std::string& err = g_noalloc_error;
  if (!index || !index->gpu_ || (n_reads && (!d_seqs || !d_offsets || !d_counts || !d_truncated)) ||
      (n_reads && max_results && !d_hits)) {
    err = "bwt_gpu_search1_noalloc: null argument";
    return -1;
  }
  if (n_reads == 0) return 0;
  const size_t len_cap = max_len < 3 ? 3 : max_len;
  const size_t T = 2 * n_reads;
  if (max_len > 32767 || n_reads >= (1ull << 30) || scratch_need(T, len_cap) > kNoAllocScratchBytes) {
    err = "bwt_gpu_search1_noalloc: batch too large for the fixed " + std::to_string(kNoAllocScratchBytes >> 20) +
          " MiB scratch (needs 2*n_reads*max_len*17 bytes + alignment, i.e. n_reads*max_len <= ~490000)";
    return -1;
  }
  void* engine = index->gpu_;
  const int device = engine_device_of(engine);
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != device && cudaSetDevice(device) != cudaSuccess) {
    err = "bwt_gpu_search1_noalloc: cannot select the index's device";
    return -1;
  }
  int rc = 0;
  void* scratch = scratch_address(device, &err);
  if (!scratch) {
    rc = -1;
  } else {
    cudaStream_t s = stream ? (cudaStream_t)stream : (cudaStream_t)engine_stream_of(engine);
    const unsigned grid = (unsigned)((T + 127) / 128);
    search1_noalloc_kernel<<<grid, 128, 0, s>>>(engine_dev_index(engine), engine_code_table(engine),
                                                 reinterpret_cast<const uint8_t*>(d_seqs), d_offsets,
                                                 (uint32_t)n_reads, (uint32_t)len_cap, max_results,
                                                 static_cast<unsigned char*>(scratch), d_hits, d_counts, d_truncated);
    count_launches(1);
    // Peek, so that an error left pending by an earlier, unrelated call on
    // this thread is neither cleared nor reported as this launch's failure.
    const cudaError_t ce = cudaPeekAtLastError();
    if (ce != cudaSuccess) {
      err = std::string("bwt_gpu_search1_noalloc: launch failed: ") + cudaGetErrorString(ce);
      rc = -1;
    }
  }
  if (prev >= 0 && prev != device) cudaSetDevice(prev);
  return rc;
}

}  // extern "C"
