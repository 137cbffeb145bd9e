// dvc_knn.cu — processing order and k-nearest neighbours of the ROI points on
// the GPU (DataCloud::sort_order_neighbors, Core/DataCloud.cpp:69-144, whose
// host form is N sorts of N distances).
//
// Distances are the reference's (Point::pt_dist, Core/Point.h:47-48: the
// square root of the three squared differences summed in x, y, z order),
// formed with round-to-nearest FP64 operations and no contraction, so they are
// bit-identical to the host's. Ties are ordered by point index: a documented
// rule of this path. The reference's std::sort leaves equal distances in an
// order of its own; the drop-in programs use the host path where that order
// matters for parity.
//
// Neighbours: points are binned in a uniform grid of cell side h; for each
// point the cells within Chebyshev radius r are gathered into shared memory and
// bitonic-sorted by (distance, index). Every point outside that cube of cells
// is at least r*h away, so the first k are exact once the k-th distance is
// below r*h; otherwise the point is done again with r + 1 (up to a cap, then
// the whole cloud is scanned). Order: one global bitonic sort of (distance
// bits, index) keys.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/dvc_gpu.h"
#include "dvc_internal.h"

namespace {

constexpr int kCand = 2048;  // candidates per point held in shared memory

__device__ __forceinline__ double pdist(const double *a, const double *b) {
  const double dx = __dsub_rn(a[0], b[0]), dy = __dsub_rn(a[1], b[1]), dz = __dsub_rn(a[2], b[2]);
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// (distance, index) as one 128-bit order: distances are non-negative, so their
// bit patterns order like the values
struct Key {
  unsigned long long d;
  int i;
};
__device__ __forceinline__ bool key_less(const Key &a, const Key &b) {
  return a.d < b.d || (a.d == b.d && a.i < b.i);
}

struct Grid {
  double lo[3], h;
  int g[3];
};

__device__ __forceinline__ int cell_of(const Grid &G, const double *p, int d) {
  const int c = (int)floor((p[d] - G.lo[d]) / G.h);
  return min(max(c, 0), G.g[d] - 1);
}

__global__ void cell_count(int n, const double *pts, Grid G, int *cell, int *count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = pts + (size_t)i * 3;
  const int c = (cell_of(G, p, 2) * G.g[1] + cell_of(G, p, 1)) * G.g[0] + cell_of(G, p, 0);
  cell[i] = c;
  atomicAdd(count + c, 1);
}

// the points of each cell (in any order: candidates are sorted by (distance,
// index) afterwards)
__global__ void cell_fill(int n, const int *cell, const int *start, int *cursor, int *items) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cell[i];
  items[start[c] + atomicAdd(cursor + c, 1)] = i;
}

__device__ void bitonic_shared(Key *s, int m) {
  // m: power of two; all threads of the block take part
  for (int size = 2; size <= m; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      for (int t = threadIdx.x; t < m / 2; t += blockDim.x) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = ((lo & size) == 0);
        const Key a = s[lo], b = s[hi];
        if (key_less(b, a) == up) {
          s[lo] = b;
          s[hi] = a;
        }
      }
    }
  __syncthreads();
}

// one block per point of `todo`: candidates from the cells within radius r;
// writes the k nearest when exact, else appends the point to `redo`
__global__ void __launch_bounds__(256) knn_kernel(int n, const double *pts, Grid G, const int *start,
                                                  const int *items, int k, int r, const int *todo, int ntodo,
                                                  int *neigh, int *redo, int *nredo) {
  __shared__ Key s[kCand];
  __shared__ int cnt;
  if (blockIdx.x >= ntodo) return;
  const int q = todo ? todo[blockIdx.x] : blockIdx.x;
  const double *p = pts + (size_t)q * 3;
  const int c0[3] = {cell_of(G, p, 0), cell_of(G, p, 1), cell_of(G, p, 2)};
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  const int w = 2 * r + 1;
  const int ncube = w * w * w;
  for (int cc = threadIdx.x; cc < ncube; cc += blockDim.x) {
    const int cx = c0[0] + cc % w - r, cy = c0[1] + (cc / w) % w - r, cz = c0[2] + cc / (w * w) - r;
    if (cx < 0 || cy < 0 || cz < 0 || cx >= G.g[0] || cy >= G.g[1] || cz >= G.g[2]) continue;
    const int cell = (cz * G.g[1] + cy) * G.g[0] + cx;
    for (int a = start[cell]; a < start[cell + 1]; a++) {
      const int j = items[a];
      const int slot = atomicAdd(&cnt, 1);
      if (slot < kCand) s[slot] = Key{(unsigned long long)__double_as_longlong(pdist(p, pts + (size_t)j * 3)), j};
    }
  }
  __syncthreads();
  const int m0 = min(cnt, kCand);
  int m = 1;
  while (m < m0) m <<= 1;
  for (int t = m0 + threadIdx.x; t < m; t += blockDim.x) s[t] = Key{~0ull, 0x7fffffff};
  bitonic_shared(s, m);
  // exact when no candidate was dropped (cnt <= kCand), at least k were seen
  // and the k-th distance is below the cube's guaranteed radius (or the cube
  // holds the whole grid)
  const int kk = min(k, n);
  // the cube of cells holds the whole grid
  bool full = true;
  for (int d = 0; d < 3; d++) full = full && c0[d] - r <= 0 && c0[d] + r >= G.g[d] - 1;
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = (cnt <= kCand) && (m0 >= kk);
    if (ok && !full) ok = __longlong_as_double((long long)s[kk - 1].d) < r * G.h;
  }
  __syncthreads();
  if (ok) {
    for (int t = threadIdx.x; t < kk; t += blockDim.x) neigh[(size_t)q * kk + t] = s[t].i;
  } else if (threadIdx.x == 0) {
    redo[atomicAdd(nredo, 1)] = q;
  }
}

// the last resort for a point: every point of the cloud, in chunks, keeping the
// k best in shared memory
__global__ void __launch_bounds__(256) knn_all_kernel(int n, const double *pts, int k, const int *todo,
                                                      int *neigh) {
  __shared__ Key s[kCand];
  const int q = todo[blockIdx.x];
  const double *p = pts + (size_t)q * 3;
  const int kk = min(k, n);
  const int half = kCand / 2;  // best so far in s[0..half), new chunk in s[half..)
  for (int t = threadIdx.x; t < half; t += blockDim.x) s[t] = Key{~0ull, 0x7fffffff};
  for (int c0 = 0; c0 < n; c0 += half) {
    for (int t = threadIdx.x; t < half; t += blockDim.x) {
      const int j = c0 + t;
      s[half + t] = j < n ? Key{(unsigned long long)__double_as_longlong(pdist(p, pts + (size_t)j * 3)), j}
                          : Key{~0ull, 0x7fffffff};
    }
    bitonic_shared(s, kCand);
  }
  for (int t = threadIdx.x; t < kk; t += blockDim.x) neigh[(size_t)q * kk + t] = s[t].i;
}

__global__ void start_dist(int n, const double *pts, const double *start, Key *keys, int m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  keys[i] = i < n ? Key{(unsigned long long)__double_as_longlong(pdist(start, pts + (size_t)i * 3)), i}
                  : Key{~0ull, 0x7fffffff};
}

__global__ void bitonic_step(Key *keys, int m, int size, int stride) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m / 2) return;
  const int lo = 2 * t - (t & (stride - 1));
  const int hi = lo + stride;
  const bool up = ((lo & size) == 0);
  const Key a = keys[lo], b = keys[hi];
  if (key_less(b, a) == up) {
    keys[lo] = b;
    keys[hi] = a;
  }
}

__global__ void order_out(int n, const Key *keys, int *order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) order[i] = keys[i].i;
}

}  // namespace

extern "C" int dvc_gpu_order_neighbours(int n, const double *points, const double start[3], int k,
                                        int *order, int *neigh) try {
  if (n <= 0 || !points || !start || k <= 0 || !order || !neigh)
    return dvc_internal_set_error(DVC_E_ARG, "bad arguments");
  // grid: about k / 8 points per cell over the cloud's bounding box
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      lo[d] = std::min(lo[d], points[(size_t)i * 3 + d]);
      hi[d] = std::max(hi[d], points[(size_t)i * 3 + d]);
    }
  Grid G;
  double vol = 1.0;
  int dims = 0;
  for (int d = 0; d < 3; d++)
    if (hi[d] - lo[d] > 0) {
      vol *= hi[d] - lo[d];
      dims++;
    }
  const double per = std::max(1.0, (double)std::min(k, n) / 8.0);
  G.h = dims ? std::pow(vol * per / n, 1.0 / dims) : 1.0;
  if (!(G.h > 0)) G.h = 1.0;
  for (int d = 0; d < 3; d++) {
    G.lo[d] = lo[d];
    G.g[d] = std::max(1, std::min(1024, (int)std::floor((hi[d] - lo[d]) / G.h) + 1));
  }
  const int ncell = G.g[0] * G.g[1] * G.g[2];
  int m = 1;
  while (m < n) m <<= 1;
  const int kk = std::min(k, n);
  double *d_pts = nullptr, *d_start = nullptr;
  int *d_cell = nullptr, *d_count = nullptr, *d_items = nullptr, *d_cursor = nullptr, *d_neigh = nullptr;
  int *d_todo = nullptr, *d_redo = nullptr, *d_nredo = nullptr, *d_order = nullptr;
  Key *d_keys = nullptr;
  int rc = DVC_OK;
  auto fail = [&](const char *msg) { rc = dvc_internal_set_error(DVC_E_NOMEM, msg); };
  if (cudaMalloc(&d_pts, (size_t)n * 24) || cudaMalloc(&d_start, 24) || cudaMalloc(&d_cell, (size_t)n * 4) ||
      cudaMalloc(&d_count, ((size_t)ncell + 1) * 4) || cudaMalloc(&d_items, (size_t)n * 4) ||
      cudaMalloc(&d_cursor, (size_t)ncell * 4) || cudaMalloc(&d_neigh, (size_t)n * kk * 4) ||
      cudaMalloc(&d_todo, (size_t)n * 4) || cudaMalloc(&d_redo, (size_t)n * 4) || cudaMalloc(&d_nredo, 4) ||
      cudaMalloc(&d_order, (size_t)n * 4) || cudaMalloc(&d_keys, (size_t)m * sizeof(Key)))
    fail("neighbour search buffers");
  if (!rc) {
    cudaMemcpy(d_pts, points, (size_t)n * 24, cudaMemcpyHostToDevice);
    cudaMemcpy(d_start, start, 24, cudaMemcpyHostToDevice);
    cudaMemset(d_count, 0, ((size_t)ncell + 1) * 4);
    cudaMemset(d_cursor, 0, (size_t)ncell * 4);
    const int T = 256;
    cell_count<<<(n + T - 1) / T, T>>>(n, d_pts, G, d_cell, d_count);
    // exclusive scan of the counts on the host (cells are few)
    std::vector<int> cnt((size_t)ncell + 1, 0);
    cudaMemcpy(cnt.data(), d_count, (size_t)ncell * 4, cudaMemcpyDeviceToHost);
    int acc = 0;
    for (int c = 0; c < ncell; c++) {
      const int v = cnt[(size_t)c];
      cnt[(size_t)c] = acc;
      acc += v;
    }
    cnt[(size_t)ncell] = acc;
    cudaMemcpy(d_count, cnt.data(), ((size_t)ncell + 1) * 4, cudaMemcpyHostToDevice);
    cell_fill<<<(n + T - 1) / T, T>>>(n, d_cell, d_count, d_cursor, d_items);
    // neighbours, growing the radius for the points that need it
    int ntodo = n;
    const int *todo = nullptr;
    for (int r = 1; ntodo > 0 && r <= 6; r++) {
      cudaMemset(d_nredo, 0, 4);
      knn_kernel<<<ntodo, T>>>(n, d_pts, G, d_count, d_items, k, r, todo, ntodo, d_neigh, d_redo, d_nredo);
      cudaMemcpy(&ntodo, d_nredo, 4, cudaMemcpyDeviceToHost);
      std::swap(d_todo, d_redo);
      todo = d_todo;
    }
    if (ntodo > 0) knn_all_kernel<<<ntodo, T>>>(n, d_pts, k, d_todo, d_neigh);
    // processing order
    start_dist<<<(m + T - 1) / T, T>>>(n, d_pts, d_start, d_keys, m);
    for (int size = 2; size <= m; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1)
        bitonic_step<<<(m / 2 + T - 1) / T, T>>>(d_keys, m, size, stride);
    order_out<<<(n + T - 1) / T, T>>>(n, d_keys, d_order);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(e));
    if (!rc) {
      cudaMemcpy(order, d_order, (size_t)n * 4, cudaMemcpyDeviceToHost);
      cudaMemcpy(neigh, d_neigh, (size_t)n * kk * 4, cudaMemcpyDeviceToHost);
    }
  }
  cudaFree(d_pts); cudaFree(d_start); cudaFree(d_cell); cudaFree(d_count); cudaFree(d_items);
  cudaFree(d_cursor); cudaFree(d_neigh); cudaFree(d_todo); cudaFree(d_redo); cudaFree(d_nredo);
  cudaFree(d_order); cudaFree(d_keys);
  return rc;
} catch (...) {
  return dvc_internal_host_exception();
}
