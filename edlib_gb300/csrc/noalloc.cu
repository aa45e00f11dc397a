// edgpu_vv_noalloc: the Storage::vv dot product <v, w> on caller-owned device arrays, for callers that
// must not allocate device memory.
//
// Who needs it: a serving loop that admitted its requests against a fixed device-memory budget and must
// not grow past it while requests are in flight; code that orders its work on streams and cannot afford
// the implicit device-wide synchronisation a cudaMalloc/cudaFree may cause; hosts whose allocator policy
// hands all device memory out up front.  Every other entry point of this library may allocate (through
// its context's caching allocator); this one never calls cudaMalloc, cudaFree or any allocating library
// routine.
//
// Scratch: the per-block partial sums live in g_vv_scratch, a file-scope __device__ array of
// kVvMaxParts doubles (16 KiB).  Every GPU that loads the library holds it until the process exits.
// Host code cannot use the symbol as a device address, so the first call on each device looks its
// address up with cudaGetSymbolAddress while that device is current and caches it; make that first call
// before any stream capture.  Every call on a device shares the same array and the array keeps the last
// call's contents: each partial is written before it is read, so nothing needs clearing, but calls that
// overlap on the GPU (on different streams, or from several host threads) race on the array and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "../../include/edgpu.h"

namespace edgpu {
void note_launch(long long n = 1);
}

namespace {

constexpr int kVvBlock = 256;
constexpr long long kVvChunk = 4096;  // elements summed by one block
constexpr int kVvMaxParts = 2048;     // EDGPU_VV_NOALLOC_MAX_N = kVvChunk * kVvMaxParts
static_assert(kVvChunk * kVvMaxParts == EDGPU_VV_NOALLOC_MAX_N, "limit must match the header");

static __device__ __align__(256) double g_vv_scratch[kVvMaxParts];

// block b sums elements [b*kVvChunk, (b+1)*kVvChunk) in a fixed order into part[b]
__global__ void __launch_bounds__(kVvBlock) k_vv_chunks(const double *v, const double *w, long long n, double *part) {
  __shared__ double red[kVvBlock];
  const long long lo = blockIdx.x * kVvChunk;
  long long hi = lo + kVvChunk;
  if (hi > n) hi = n;
  double s = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += kVvBlock) s = fma(v[i], w[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = kVvBlock / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_vv_final(const double *part, int nparts, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[b];
  *out = s;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
std::atomic<double *> g_scratch[kMaxDevices];

// address of g_vv_scratch on the current device (looked up once per device)
int scratch_ptr(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return EDGPU_ERR_CUDA;
  double *p = g_scratch[dev].load();
  if (!p) {
    std::lock_guard<std::mutex> lk(g_mu);
    p = g_scratch[dev].load();
    if (!p) {
      if (cudaGetSymbolAddress((void **)&p, g_vv_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return EDGPU_ERR_CUDA;
      }
      g_scratch[dev].store(p);
    }
  }
  *out = p;
  return EDGPU_OK;
}

}  // namespace

extern "C" int edgpu_vv_noalloc(const double *v, const double *w, long long n, double *out, void *stream) {
  if (!out || n < 0 || (n > 0 && (!v || !w))) return EDGPU_ERR_ARG;
  if (n > EDGPU_VV_NOALLOC_MAX_N) return EDGPU_ERR_CAPACITY;
  double *part = nullptr;
  int rc = scratch_ptr(&part);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int nparts = (int)((n + kVvChunk - 1) / kVvChunk);
  if (nparts > 0) {
    k_vv_chunks<<<nparts, kVvBlock, 0, st>>>(v, w, n, part); edgpu::note_launch();
  }
  k_vv_final<<<1, 32, 0, st>>>(part, nparts, out); edgpu::note_launch();
  if (cudaGetLastError() != cudaSuccess) return EDGPU_ERR_CUDA;
  return EDGPU_OK;
}
