// sf_affine_noalloc: `affine` (align.rs:699-701) for callers that cannot allocate device
// memory.  It has no counterpart in the reference.
//
// Some callers of this library must not allocate on the device while they run alignments:
//  - a latency-bound serving path, where cudaMalloc / cudaFree synchronize the device and so
//    stall every other request already in flight on it;
//  - an embedding application that hands this library device memory from its own pool and
//    forbids any other device allocation.
// This entry point takes the caller's device buffers for its inputs and output and keeps
// every other byte it needs (packed sequences, the job descriptors, the pass result and the
// two DP rows of the wide-row kernel) in one file-scope device array of SF_NOALLOC_SCRATCH
// bytes.  It calls no cudaMalloc, cudaFree or allocating library routine.
//
// The array is global state: every call on a device uses the same bytes, and they keep the
// previous call's contents (each call rewrites what it reads and zeroes what must start at
// zero).  Calls whose work overlaps on one GPU -- on two streams, or from two threads --
// race on the array; the caller must order them, e.g. by issuing them on one stream.  The
// first call on a device looks the array's device address up (cudaGetSymbolAddress, with
// that device current) and keeps it; make that first call before any stream capture.  A
// cudaDeviceReset of that device invalidates the kept address (the module loads again,
// maybe elsewhere): load the library afresh before calling this again.  The pass's cells are
// not added to sf_dp_work's counters, since the call returns before the pass has run.
#include <mutex>

#include "../../include/sf_align.h"
#include "sf_internal.cuh"

namespace {

using namespace sf;

static __device__ __align__(256) unsigned char g_noalloc_scratch[SF_NOALLOC_SCRATCH];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Scratch layout (byte offsets): a header of descriptors, the result, the packed pool (two
// sequences plus zero slack), then the wide kernel's four row buffers.
struct Header {
  uint32_t counter;  // the kernel's work queue (one job)
  uint32_t order;    // job 0
  uint64_t seq_off[2], seq_woff[2];
  uint32_t seq_len[2];
  DJob job;
  DParams params;
  DRes res;
};
constexpr size_t kHeader = (sizeof(Header) + 255) & ~size_t(255);
constexpr uint32_t kSlackWords = 256;

__host__ __device__ inline uint64_t seq_words(uint64_t len) { return (len + 1 + 15) / 16; }

int fail(int code, const char* msg) { return sf_internal_set_error(code, msg); }

// One thread writes the descriptors and zeroes what must start at zero.
__global__ void noalloc_prep(unsigned char* scr, DJob job, DParams params, uint32_t m, uint32_t n,
                             uint64_t pool_words) {
  Header* h = reinterpret_cast<Header*>(scr);
  uint32_t* pool = reinterpret_cast<uint32_t*>(scr + kHeader);
  if (threadIdx.x == 0) {
    h->counter = 0;
    h->order = 0;
    h->seq_off[0] = 0;
    h->seq_off[1] = 0;
    h->seq_woff[0] = 0;
    h->seq_woff[1] = seq_words(m);
    h->seq_len[0] = m;
    h->seq_len[1] = n;
    h->job = job;
    h->params = params;
    h->res = DRes{};
  }
  // Zero the slack after the two sequences (the packing writes every sequence word).
  for (uint64_t w = pool_words - kSlackWords + threadIdx.x; w < pool_words; w += blockDim.x)
    pool[w] = 0;
}

// The pass's score to the caller's buffer.  A score-only pass has no failure outcome on the
// device (an unreachable end is NEG); launch errors come back as the return code.
__global__ void noalloc_out(const unsigned char* scr, int32_t* out) {
  if (threadIdx.x == 0) *out = reinterpret_cast<const Header*>(scr)->res.score;
}

}  // namespace

extern "C" int sf_affine_noalloc(const uint8_t* d_pattern, uint64_t m, const uint8_t* d_text,
                                 uint64_t n, int mode, const sf_affine_t* sc, uint64_t band,
                                 int32_t* d_score, void* stream) {
  if (!sc || !d_score || (m && !d_pattern) || (n && !d_text) || mode < 0 || mode > 2 ||
      sc->open < 0 || sc->ext < 0)
    return fail(SF_ERR_INVALID, "sf_affine_noalloc: bad argument");
  if (m > SF_NOALLOC_MAX_LEN || n > SF_NOALLOC_MAX_LEN)
    return fail(SF_ERR_TOO_LONG,
                "sf_affine_noalloc: pattern and text must each be at most SF_NOALLOC_MAX_LEN "
                "bases");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    (void)cudaGetLastError();
    return fail(SF_ERR_CUDA, "sf_affine_noalloc: no current CUDA device");
  }
  unsigned char* scr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        (void)cudaGetLastError();
        return fail(SF_ERR_CUDA, "sf_affine_noalloc: cudaGetSymbolAddress failed");
      }
      g_addr[dev] = p;
    }
    scr = static_cast<unsigned char*>(g_addr[dev]);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // The pass, as sf_affine describes it (geom = n, align.rs:699-701).
  DJob job{};
  job.m = (uint32_t)m;
  job.n = (uint32_t)n;
  job.p_word = 0;
  job.t_word = seq_words(m);
  const uint64_t geom = n;
  const uint64_t below = band > UINT64_MAX - (m > geom ? m - geom : 0)
                             ? UINT64_MAX
                             : band + (m > geom ? m - geom : 0);
  const uint64_t above = band > UINT64_MAX - (geom > m ? geom - m : 0)
                             ? UINT64_MAX
                             : band + (geom > m ? geom - m : 0);
  const uint64_t cap40 = uint64_t(1) << 40;
  job.below = (int64_t)(below < cap40 ? below : cap40);
  job.above = (int64_t)(above < cap40 ? above : cap40);
  job.cut = UINT64_MAX;
  DParams pr{};
  pr.flags = (uint32_t)mode | ((mode == SF_INFIX || band == SF_NOLIMIT) ? F_FULL : 0u);
  pr.mat = sc->mat;
  pr.mis = sc->mis;
  pr.open = sc->open;
  pr.ext = sc->ext;
  const uint64_t pool_words = seq_words(m) + seq_words(n) + kSlackWords;
  const uint64_t cells = (uint64_t)wide_chunks(sfk::kWideC, band_wmax(job, pr.flags)) * 32 *
                         sfk::kWideC;
  const size_t need = kHeader + ((pool_words * 4 + 255) & ~uint64_t(255)) + 4 * cells * 4;
  if (need > SF_NOALLOC_SCRATCH)
    return fail(SF_ERR_TOO_LONG, "sf_affine_noalloc: pass needs more than SF_NOALLOC_SCRATCH");
  Header* hd = reinterpret_cast<Header*>(scr);
  uint32_t* pool = reinterpret_cast<uint32_t*>(scr + kHeader);
  int32_t* rows = reinterpret_cast<int32_t*>(scr + kHeader + ((pool_words * 4 + 255) & ~uint64_t(255)));

  noalloc_prep<<<1, 256, 0, s>>>(scr, job, pr, (uint32_t)m, (uint32_t)n, pool_words);
  cudaError_t e = cudaGetLastError();
  for (int q = 0; q < 2 && e == cudaSuccess; ++q) {
    sfk::PackLaunch pl;
    pl.bytes = q == 0 ? d_pattern : d_text;
    pl.byte_off = &hd->seq_off[q];
    pl.len = &hd->seq_len[q];
    pl.word_off = &hd->seq_woff[q];
    pl.nseq = 1;
    pl.pool = pool;
    e = sfk::launch_pack(pl, s);
  }
  if (e == cudaSuccess) {
    sfk::AffLaunch al{};
    al.jobs = &hd->job;
    al.params = &hd->params;
    al.order = &hd->order;
    al.njobs = 1;
    al.counter = &hd->counter;
    al.pool = pool;
    al.bytes = d_pattern;
    al.out = &hd->res;
    al.tb = nullptr;
    al.scratch = rows;
    al.scratch_cells = cells;
    e = sfk::launch_affine(sfk::kWideC, true, false, false, al, 1, 32, s);
  }
  if (e == cudaSuccess) {
    noalloc_out<<<1, 32, 0, s>>>(scr, d_score);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail(SF_ERR_CUDA, cudaGetErrorString(e));
  return SF_OK;
}
