// Receiver grid: receivers of every request of a solve binned into a uniform
// grid (about two per cell), so a node's capture test visits only the cells
// near its segment.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "sbr_device.h"
#include "sbr_field.cuh"
#include "sbr_kernels.cuh"
#include "sbr_common.cuh"

namespace sbr {

// ---- receiver grid ------------------------------------------------------

// Order-preserving float <-> int mapping for atomicMin/Max on floats.
__device__ __forceinline__ int f2o(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

struct GridBuild {
  int bmin[3], bmax[3];  // ordered ints
  float cmax;            // max |rx| (as float, atomicMax on ordered int below)
  int cmax_o;
  int ncell;
};

// Bounds of each request's receivers.  A receiver with a non-finite
// coordinate (possible only for receivers the caller placed on the device;
// host receivers are checked before upload) sets *bad and is left out of the
// bounds; the solve then fails with an argument error.
__global__ void k_rx_bounds(const double* rx, const TxParams* txp, int n_tx, GridBuild* gb,
                            int* bad) {
  const int r = blockIdx.y;  // request
  if (r >= n_tx) return;
  const TxParams& P = txp[r];
  int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN}, cm = INT_MIN;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_rx; i += gridDim.x * blockDim.x) {
    const double* c = rx + 3 * size_t(P.rx_first + i);
    if (!(isfinite(c[0]) && isfinite(c[1]) && isfinite(c[2]))) {
      atomicOr(bad, 1);
      continue;
    }
    float c32[3] = {float(c[0]), float(c[1]), float(c[2])};
    for (int a = 0; a < 3; ++a) {
      mn[a] = min(mn[a], f2o(c32[a]));
      mx[a] = max(mx[a], f2o(c32[a]));
    }
    cm = max(cm, f2o(float(sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]))));
  }
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o; o >>= 1) {
      mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  for (int o = 16; o; o >>= 1) cm = max(cm, __shfl_xor_sync(0xffffffffu, cm, o));
  if (lane_id() == 0) {
    for (int a = 0; a < 3; ++a) {
      atomicMin(&gb[r].bmin[a], mn[a]);
      atomicMax(&gb[r].bmax[a], mx[a]);
    }
    atomicMax(&gb[r].cmax_o, cm);
  }
}

// Receivers per cell the grid is sized for, and the minimum chunk length of a
// node's segment in capture, in cells.  Smaller cells hug a node's capture
// tube more closely (fewer candidates per node) but give more rows and chunks
// per node; for receivers on a plane (one layer of cells) a row costs less,
// and smaller cells pay.
#ifndef SBR_GRID_RX_PER_CELL
#define SBR_GRID_RX_PER_CELL 2.0
#endif
#ifndef SBR_GRID_RX_PER_CELL_FLAT
#define SBR_GRID_RX_PER_CELL_FLAT 0.5
#endif
#ifndef SBR_CAP_CHUNK_CELLS
#define SBR_CAP_CHUNK_CELLS 16
#endif
#ifndef SBR_CAP_CHUNK_CELLS_FLAT
#define SBR_CAP_CHUNK_CELLS_FLAT 24
#endif
constexpr double kMinRxPerCell =
    SBR_GRID_RX_PER_CELL < SBR_GRID_RX_PER_CELL_FLAT ? SBR_GRID_RX_PER_CELL : SBR_GRID_RX_PER_CELL_FLAT;

// Grid shape: cells of equal size over the axes with extent, sized for the
// receivers per cell above, at most max_cells cells.
__global__ void k_grid_shape(GridBuild* gb, RxGrid* grids, const TxParams* txp, int n_tx,
                             int max_cells, int* cell_base) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int base = 0;
  for (int r = 0; r < n_tx; ++r) {
    RxGrid& g = grids[r];
    float lo[3], hi[3], ext[3];
    float emax = 0;
    for (int a = 0; a < 3; ++a) {
      lo[a] = o2f(gb[r].bmin[a]);
      hi[a] = o2f(gb[r].bmax[a]);
      if (txp[r].n_rx == 0) lo[a] = hi[a] = 0;
      ext[a] = hi[a] - lo[a];
      emax = fmaxf(emax, ext[a]);
    }
    int k = 0;
    double vol = 1;
    for (int a = 0; a < 3; ++a)
      if (ext[a] > 1e-6f * emax && ext[a] > 0) {
        ++k;
        vol *= ext[a];
      }
    float cell = 1.0f;
    if (k > 0) {
      const double rpc = k < 3 ? SBR_GRID_RX_PER_CELL_FLAT : SBR_GRID_RX_PER_CELL;
      double target = fmax(1.0, txp[r].n_rx / rpc);
      cell = float(pow(vol / target, 1.0 / k));
    }
    if (cell <= 0) cell = 1.0f;
    int dim[3];
    long long tot;
    for (;;) {
      tot = 1;
      for (int a = 0; a < 3; ++a) {
        dim[a] = max(1, min(1 << 20, int(ext[a] / cell) + 1));
        tot *= dim[a];
      }
      if (tot <= max_cells) break;
      cell *= 1.25f;
    }
    for (int a = 0; a < 3; ++a) {
      g.org[a] = lo[a];
      g.dim[a] = dim[a];
      g.bmin[a] = lo[a];
      g.bmax[a] = hi[a];
    }
    g.cell = cell;
    g.inv_cell = 1.0f / cell;
    g.chunk_len = float(k < 3 ? SBR_CAP_CHUNK_CELLS_FLAT : SBR_CAP_CHUNK_CELLS) * cell;
    gb[r].ncell = int(tot);
    gb[r].cmax = o2f(gb[r].cmax_o);
    cell_base[r] = base;
    base += int(tot) + 1;
  }
  cell_base[n_tx] = base;
}

__device__ __forceinline__ int cell_of(const RxGrid& g, float x, float y, float z) {
  int ix = min(g.dim[0] - 1, max(0, int((x - g.org[0]) / g.cell)));
  int iy = min(g.dim[1] - 1, max(0, int((y - g.org[1]) / g.cell)));
  int iz = min(g.dim[2] - 1, max(0, int((z - g.org[2]) / g.cell)));
  return (iz * g.dim[1] + iy) * g.dim[0] + ix;
}

__global__ void k_rx_count(const double* rx, const TxParams* txp, int n_tx, const RxGrid* grids,
                           const int* cell_base, int* counts) {
  const int r = blockIdx.y;
  if (r >= n_tx) return;
  const RxGrid g = grids[r];
  const TxParams& P = txp[r];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_rx; i += gridDim.x * blockDim.x) {
    const double* c = rx + 3 * size_t(P.rx_first + i);
    atomicAdd(&counts[cell_base[r] + cell_of(g, float(c[0]), float(c[1]), float(c[2]))], 1);
  }
}

// Single-block exclusive scan (n up to a few million): each thread scans a
// contiguous chunk, then the chunk totals are scanned across the block.
__global__ void k_scan_exclusive(const int* in, int* out, int n) {
  __shared__ int part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int chunk = (n + T - 1) / T;
  const int b = min(n, t * chunk), e = min(n, b + chunk);
  int s = 0;
  for (int i = b; i < e; ++i) s += in[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
    int v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = t ? part[t - 1] : 0;
  for (int i = b; i < e; ++i) {
    int v = in[i];
    out[i] = run;
    run += v;
  }
  if (t == T - 1) out[n] = part[T - 1];
}

// Exclusive scan of n ints over many blocks (same result as k_scan_exclusive,
// out[n] = total): tile sums, one block scans the sums, then every tile
// scans its items from its offset.  Thread t of a tile owns kScanItems
// consecutive items.
constexpr int kScanThreads = 512, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_scan_incl(int v, int* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    int t = lane < nw ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) sh[lane] = t;
  }
  __syncthreads();
  const int r = v + (w ? sh[w - 1] : 0);
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const int* in, int n, int* sums) {
  __shared__ int sh[32];
  const long long base = (long long)blockIdx.x * kScanTile;
  int s = 0;
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
    if (base + i < n) s += in[base + i];
  s = block_scan_incl(s, sh);
  if (threadIdx.x == blockDim.x - 1) sums[blockIdx.x] = s;
}

__global__ void __launch_bounds__(1024) k_sums_scan(int* sums, int nb, int* total) {
  __shared__ int sh[32];
  __shared__ int last;
  int carry = 0;
  for (int c = 0; c < nb; c += blockDim.x) {
    const int i = c + threadIdx.x;
    const int v = i < nb ? sums[i] : 0;
    const int incl = block_scan_incl(v, sh);
    if (i < nb) sums[i] = carry + incl - v;
    if (threadIdx.x == blockDim.x - 1) last = incl;
    __syncthreads();
    carry += last;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const int* in, int n, const int* sums,
                                                            int* out) {
  __shared__ int sh[32];
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
  for (int j = 0; j < kScanItems; ++j) {
    v[j] = base + j < n ? in[base + j] : 0;
    s += v[j];
  }
  int run = sums[blockIdx.x] + block_scan_incl(s, sh) - s;
  for (int j = 0; j < kScanItems; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
}

__global__ void k_rx_scatter(const double* rx, const TxParams* txp, int n_tx, const RxGrid* grids,
                             const int* cell_base, const int* starts, int* cursor, float4* rx32) {
  const int r = blockIdx.y;
  if (r >= n_tx) return;
  const RxGrid g = grids[r];
  const TxParams& P = txp[r];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n_rx; i += gridDim.x * blockDim.x) {
    const int gi = P.rx_first + i;
    const double* c = rx + 3 * size_t(gi);
    const int cid = cell_base[r] + cell_of(g, float(c[0]), float(c[1]), float(c[2]));
    const int pos = starts[cid] + atomicAdd(&cursor[cid], 1);
    rx32[pos] = make_float4(float(c[0]), float(c[1]), float(c[2]), __int_as_float(gi));
  }
}

__global__ void k_grid_finish(RxGrid* grids, const int* starts, const int* cell_base,
                              const float4* rx32, int n_tx) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_tx) return;
  grids[r].cell_start = starts + cell_base[r];
  grids[r].rx32 = rx32;
}

}  // namespace sbr
