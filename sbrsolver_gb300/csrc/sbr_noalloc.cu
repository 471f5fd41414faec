// Per-receiver field sum without any allocation.
//
// Some callers of this library cannot allocate device memory: processes whose
// device memory is already held by another framework's caching allocator
// (cudaMalloc would fail or force that pool to shrink), services that must
// keep a fixed device footprint after start-up, and latency-bound loops that
// cannot afford cudaMalloc/cudaFree, which may synchronise the whole device.
// For them, sbr_receiver_field_sum_noalloc sums per-path fields into
// per-receiver fields, in each receiver's (launch, BFS) rank order and with
// the arithmetic the solve's own per-receiver sum uses, with all of its
// working memory in one fixed array compiled into this library.
//
// The scratch array below is a file-scope __device__ array: every GPU that
// loads the library holds it (4 MiB) until the process exits.  Host code must
// not pass the symbol itself to a kernel; its device address is looked up once
// per device with cudaGetSymbolAddress, on the first call made while that
// device is current.  That first call therefore performs the set-up and
// must come before any stream capture; later calls may be captured into a
// CUDA graph (they then only enqueue kernels and report no device-side
// input errors).  Every call shares the array and
// leaves the previous call's contents behind, so the counters are cleared at
// the start of each call; calls that overlap on the GPU (for example on two
// streams at once) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/sbr.h"

namespace sbr {
namespace noalloc {

constexpr int kMaxRx = 1 << 18;     // receivers per call
constexpr int kMaxPaths = 1 << 18;  // paths per call
constexpr int kSmallRx = 32;        // paths a receiver may have to be sorted by one thread
constexpr int kMaxPerRx = 2048;     // paths per receiver (sorted by one block in shared memory)
// layout (ints): counts[kMaxRx + 1] | starts[kMaxRx + 2] | cursor[kMaxRx + 1] |
//                order[kMaxPaths] | large count | error flags
// (the list of receivers with many paths reuses cursor[], which the scatter
// is done with by then)
constexpr size_t kCounts = 0;
constexpr size_t kStarts = kCounts + kMaxRx + 1;
constexpr size_t kCursor = kStarts + kMaxRx + 2;
constexpr size_t kOrder = kCursor + kMaxRx + 1;
constexpr size_t kLarge = kCursor;
constexpr size_t kLargeCount = kOrder + kMaxPaths;
constexpr size_t kError = kLargeCount + 1;
constexpr size_t kScratchInts = kError + 1;
// error flags
constexpr int kErrReceiver = 1;  // a receiver index outside [0, n_rx)
constexpr int kErrPerRx = 2;     // a receiver with more than kMaxPerRx paths

static __device__ __align__(256) int g_scratch[kScratchInts];

__global__ void k_clear(int* s, int n_rx) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n_rx; i += gridDim.x * blockDim.x) {
    s[kCounts + i] = 0;
    s[kCursor + i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    s[kError] = 0;
    s[kLargeCount] = 0;
  }
}

__global__ void k_hist(const int* recv, int n, int n_rx, int* s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int r = recv[i];
    if (r < 0 || r >= n_rx) {
      atomicOr(&s[kError], kErrReceiver);
      continue;
    }
    atomicAdd(&s[kCounts + r], 1);
  }
}

// one block: exclusive scan of counts[0..n_rx) into starts[0..n_rx]
__global__ void k_scan(int* s, int n_rx) {
  __shared__ int part[1024];
  const int* in = s + kCounts;
  int* out = s + kStarts;
  const int t = threadIdx.x, T = blockDim.x;
  const int chunk = (n_rx + T - 1) / T;
  const int b = min(n_rx, t * chunk), e = min(n_rx, b + chunk);
  int sum = 0;
  for (int i = b; i < e; ++i) sum += in[i];
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
    const int v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = t ? part[t - 1] : 0;
  for (int i = b; i < e; ++i) {
    const int v = in[i];
    out[i] = run;
    run += v;
  }
  if (t == T - 1) out[n_rx] = part[T - 1];
}

__global__ void k_scatter(const int* recv, int n, int n_rx, int* s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int r = recv[i];
    if (r < 0 || r >= n_rx) continue;
    s[kOrder + s[kStarts + r] + atomicAdd(&s[kCursor + r], 1)] = i;
  }
}

// The sum of one receiver's paths in the given order: FP64 for
// SBR_FIELD_FP64, compensated FP32 (Neumaier) for both FP32 precisions,
// exactly as the solve's own per-receiver sum (k_rx_sum) forms it (for the
// receivers the solve's FP32 error bound certifies; it sums the others in
// FP64).
template <class Idx>
__device__ void sum_in_order(Idx idx, int n, const double* pf, int precision, double* out) {
  if (precision != SBR_FIELD_FP64) {
    float acc[6] = {0, 0, 0, 0, 0, 0}, c[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 6; ++k) {
        const float x = float(pf[6 * size_t(idx(i)) + k]);
        const float t = acc[k] + x;
        c[k] += fabsf(acc[k]) >= fabsf(x) ? (acc[k] - t) + x : (x - t) + acc[k];
        acc[k] = t;
      }
    for (int k = 0; k < 6; ++k) out[k] = double(acc[k]) + double(c[k]);
  } else {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 6; ++k) acc[k] = __dadd_rn(acc[k], pf[6 * size_t(idx(i)) + k]);
    for (int k = 0; k < 6; ++k) out[k] = acc[k];
  }
}

// Receivers with at most kSmallRx paths: insertion sort by rank (at most
// kSmallRx^2 / 2 steps) and the sum, one thread per receiver.  Larger ones
// are listed for k_sum_large; more than kMaxPerRx raises an error flag.
__global__ void k_sum(const long long* rank, const double* pf, int n_rx, int precision, int* s,
                      double* out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rx; r += gridDim.x * blockDim.x) {
    int* order = s + kOrder;
    const int b = s[kStarts + r], e = s[kStarts + r + 1];
    if (e - b > kMaxPerRx) {
      atomicOr(&s[kError], kErrPerRx);
      continue;
    }
    if (e - b > kSmallRx) {
      s[kLarge + atomicAdd(&s[kLargeCount], 1)] = r;
      continue;
    }
    for (int i = b + 1; i < e; ++i) {
      const int v = order[i];
      const long long key = rank[v];
      int j = i - 1;
      // ties (equal ranks) keep the lower path index first
      while (j >= b && (rank[order[j]] > key || (rank[order[j]] == key && order[j] > v))) {
        order[j + 1] = order[j];
        --j;
      }
      order[j + 1] = v;
    }
    sum_in_order([&](int i) { return order[b + i]; }, e - b, pf, precision, out + 6 * size_t(r));
  }
}

// Receivers with kSmallRx < paths <= kMaxPerRx, one block each: a bitonic
// sort of (rank, path) pairs in shared memory, then the ordered sum by one
// thread (the order of the additions is the result's definition).
constexpr int kLargeThreads = 256;
__global__ void __launch_bounds__(kLargeThreads) k_sum_large(const long long* rank,
                                                             const double* pf, int precision,
                                                             const int* s, double* out) {
  __shared__ long long key[kMaxPerRx];
  __shared__ int idx[kMaxPerRx];
  const int* order = s + kOrder;
  const int n_large = s[kLargeCount];
  for (int L = blockIdx.x; L < n_large; L += gridDim.x) {
    const int r = s[kLarge + L];
    const int b = s[kStarts + r], n = s[kStarts + r + 1] - b;
    int m = 1;
    while (m < n) m <<= 1;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      if (i < n) {
        idx[i] = order[b + i];
        key[i] = rank[idx[i]];
      } else {  // padding sorts after every real path, whatever its rank
        idx[i] = 0x7FFFFFFF;
        key[i] = 0x7FFFFFFFFFFFFFFFll;
      }
    }
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
          const int p = i ^ j;
          if (p > i) {
            const bool up = (i & k) == 0;
            // ties (equal ranks) keep the lower path index first
            const bool gt = key[i] > key[p] || (key[i] == key[p] && idx[i] > idx[p]);
            if (gt == up) {
              const long long tk = key[i];
              key[i] = key[p];
              key[p] = tk;
              const int ti = idx[i];
              idx[i] = idx[p];
              idx[p] = ti;
            }
          }
        }
        __syncthreads();
      }
    if (threadIdx.x == 0)
      sum_in_order([&](int i) { return idx[i]; }, n, pf, precision, out + 6 * size_t(r));
    __syncthreads();
  }
}

// Device address of g_scratch and the SM count, looked up once per device.
static std::mutex g_mu;
static int* g_addr[64] = {};
static int g_sms[64] = {};

static sbr_status scratch_for_current_device(int** out, int* sms, int* device, std::string& err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return SBR_ERR_CUDA;
  }
  if (dev < 0 || dev >= 64) {
    err = "device index out of range";
    return SBR_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return SBR_ERR_CUDA;
    }
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || n <= 0) {
      err = std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e);
      return SBR_ERR_CUDA;
    }
    g_sms[dev] = n;
    g_addr[dev] = static_cast<int*>(p);
  }
  *out = g_addr[dev];
  *sms = g_sms[dev];
  *device = dev;
  return SBR_OK;
}

}  // namespace noalloc
// Sets the message sbr_last_error() returns (defined with the other entry points).
void set_error_message(const std::string& s);
}  // namespace sbr

extern "C" {

sbr_status sbr_receiver_field_sum_noalloc(const int* path_receiver, const long long* path_rank,
                                          const double* path_field, int n_paths, int n_rx,
                                          int field_precision, double* field_out,
                                          void* stream) {
  using namespace sbr::noalloc;
  std::string g_err;
  struct Report {
    std::string& m;
    ~Report() {
      if (!m.empty()) sbr::set_error_message(m);
    }
  } report{g_err};
  if (n_rx < 1 || n_rx > kMaxRx || n_paths < 0 || n_paths > kMaxPaths) {
    g_err = "sbr_receiver_field_sum_noalloc: need 1 <= n_rx <= " + std::to_string(kMaxRx) +
            " and 0 <= n_paths <= " + std::to_string(kMaxPaths) + " (got n_rx=" +
            std::to_string(n_rx) + ", n_paths=" + std::to_string(n_paths) + ")";
    return SBR_ERR_INVALID_ARG;
  }
  if (field_precision != SBR_FIELD_FP64 && field_precision != SBR_FIELD_FP32 &&
      field_precision != SBR_FIELD_FP32_PHASE) {
    g_err = "sbr_receiver_field_sum_noalloc: field_precision must be SBR_FIELD_FP64, "
            "SBR_FIELD_FP32 or SBR_FIELD_FP32_PHASE (got " + std::to_string(field_precision) + ")";
    return SBR_ERR_INVALID_ARG;
  }
  if (!field_out || (n_paths > 0 && (!path_receiver || !path_rank || !path_field))) {
    g_err = "sbr_receiver_field_sum_noalloc: NULL device pointer";
    return SBR_ERR_INVALID_ARG;
  }
  int* s = nullptr;
  int sms = 0, dev = 0;
  sbr_status st = scratch_for_current_device(&s, &sms, &dev, g_err);
  if (st != SBR_OK) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  // While the stream is being captured into a CUDA graph the call only
  // enqueues its kernels: a capture admits neither the pageable read-back
  // nor the synchronisation (nor, in the global capture mode, queries beyond
  // the capture status).  The kernels still skip out-of-range receivers and
  // over-long receivers (those fields stay zero); their flags are not
  // reported then.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  {
    const cudaError_t e = cudaStreamIsCapturing(cs, &cap);
    if (e != cudaSuccess) {
      g_err = std::string("sbr_receiver_field_sum_noalloc: ") + cudaGetErrorString(e);
      return SBR_ERR_CUDA;
    }
  }
  if (cs && cap == cudaStreamCaptureStatusNone) {  // the scratch address is the current device's
    int sdev = -1;
    cudaError_t e = cudaStreamGetDevice(cs, &sdev);
    if (e != cudaSuccess || sdev != dev) {
      g_err = "sbr_receiver_field_sum_noalloc: the stream does not belong to the current device";
      return SBR_ERR_INVALID_ARG;
    }
  }
  if (cap == cudaStreamCaptureStatusNone)
    cudaGetLastError();  // an earlier, unrelated launch error is not this call's
  const int gb = sms * 4;
  k_clear<<<gb, 256, 0, cs>>>(s, n_rx);
  if (n_paths) k_hist<<<gb, 256, 0, cs>>>(path_receiver, n_paths, n_rx, s);
  k_scan<<<1, 1024, 0, cs>>>(s, n_rx);
  if (n_paths) k_scatter<<<gb, 256, 0, cs>>>(path_receiver, n_paths, n_rx, s);
  k_sum<<<gb, 128, 0, cs>>>(path_rank, path_field, n_rx, field_precision, s, field_out);
  k_sum_large<<<sms * 2, kLargeThreads, 0, cs>>>(path_rank, path_field, field_precision, s,
                                                 field_out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && cap != cudaStreamCaptureStatusNone) return SBR_OK;
  int bad = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&bad, s + kError, sizeof(int), cudaMemcpyDeviceToHost, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) {
    g_err = std::string("sbr_receiver_field_sum_noalloc: ") + cudaGetErrorString(e);
    return SBR_ERR_CUDA;
  }
  if (bad & kErrReceiver) {
    g_err = "sbr_receiver_field_sum_noalloc: a receiver index is outside [0, n_rx)";
    return SBR_ERR_INVALID_ARG;
  }
  if (bad & kErrPerRx) {
    g_err = "sbr_receiver_field_sum_noalloc: a receiver has more than " +
            std::to_string(kMaxPerRx) + " paths";
    return SBR_ERR_INVALID_ARG;
  }
  return SBR_OK;
}

}  // extern "C"
