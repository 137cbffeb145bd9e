// dvc_engine.cu — the per-point DVC search on the GPU and its C ABI.
//
// One persistent launch processes every ROI point. A CTA takes the next point
// in processing order from a device work counter, computes its start
// estimate, interpolates the reference subvolume, runs the coarse translation
// grid and the Gauss-Newton refinement, evaluates the final objective and
// publishes the result with a release flag. In the reference's seeding mode a
// point first waits (bounded) for the neighbours that precede it in the
// order, exactly the information Search::starting_param reads
// (Core/Search.cpp:277-377). Points are taken in order, so every awaited
// neighbour belongs to a CTA that is already running: progress is guaranteed,
// and each wait still gives up after a fixed number of polls.
//
// Reference map (Core/...):
//   process_point            Search.cpp:95-192     -> search_kernel (per point)
//   starting_param           Search.cpp:277-377    -> point_seed
//   search_pt_setup          Search.cpp:248-275    -> setup_point
//   trgrid_global            Search.cpp:934-1043   -> grid_search
//   min_Lev_Mar, LM_prep_at  Search.cpp:194-246,490-525 -> gauss_newton
//   obj_val_at               Search.cpp:448-488    -> eval_* functions
//   affine_to                FloatingCloud.cpp:236-286 -> sample positions
//   set_param_vect           SearchParams.cpp:53-107 -> warp_matrices
//   tri_cub_Lek etc.         Interpolate.cpp:404-567 -> interp_sample (dvc_device.cuh)
//   obj_*                    ObjectiveFunctions.cpp:24-263 -> objective sums
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>
#include <chrono>

#include "../../include/dvc_gpu.h"
#include "dvc_device.cuh"
#include "dvc_internal.h"
#include "dvc_search.cuh"

using namespace dvc;

// ============================================================ error state ===
static thread_local std::string g_last_error;
static int set_error(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
int dvc_internal_set_error(int code, const char *msg) { return set_error(code, msg); }
// Called from the catch clause of a C entry point: the exception in flight
// becomes the call's error code and message.
int dvc_internal_host_exception() {
  try {
    throw;
  } catch (const std::bad_alloc &) {
    return set_error(DVC_E_NOMEM, "host memory allocation failed");
  } catch (const std::exception &x) {
    return set_error(DVC_E_ARG, std::string("host error: ") + x.what());
  } catch (...) {
    return set_error(DVC_E_ARG, "host error");
  }
}
#define CUDA_TRY(expr)                                                                 \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess)                                                             \
      return set_error(DVC_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// ======================================================= small kernels ===
namespace {

__global__ void init_outputs_kernel(int n_points, int *status, double *objmin, double *params,
                                    int *gn_iters, int *done, int *rank) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_points) {
    status[i] = DVC_NOT_SEARCH;
    objmin[i] = 0.0;
    for (int p = 0; p < 12; p++) params[(size_t)i * 12 + p] = 0.0;
    if (gn_iters) gn_iters[i] = 0;
    done[i] = 0;
    rank[i] = 0x7fffffff;
  }
}

__global__ void rank_kernel(int n_process, const int *order, int *rank, int n_points) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_process) {
    const int p = order[i];
    if (p >= 0 && p < n_points) rank[p] = i;
  }
}

// ------------------------------------------------- interpolation entry ---
template <typename VT>
__global__ void interp_points_kernel(GSrc<VT> V, BoxGeom G, int n, const double *pts, int itype,
                                     double *out, unsigned long long *undef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  float f[3];
  const int o[3] = {G.ox, G.oy, G.oz};
  const int bext[3] = {G.bx, G.by, G.bz};
  for (int d = 0; d < 3; d++) split_d(__dsub_rn(pts[(size_t)i * 3 + d], (double)o[d]), c[d], f[d]);
  clamp_cell(c, bext);
  bool und;
  float g[3];
  float v;
  if (itype == 2) v = interp_global<VT, 2, false>(V, G, c, f, g, und);
  else if (itype == 1) v = interp_global<VT, 1, false>(V, G, c, f, g, und);
  else v = interp_global<VT, 0, false>(V, G, c, f, g, und);
  out[i] = (double)v;
  if (und) atomicAdd(undef, 1ULL);
}

// ----------------------------------------------------- objective entry ---
// FP64 two-pass objective (Core/ObjectiveFunctions.cpp:24-263), one CTA.
constexpr int kObjThreads = 256;
__global__ void objective_kernel(int fcn, int n, const double *r, const double *t, double *obj,
                                 double *res) {
  __shared__ double red[kObjThreads];
  const int tid = threadIdx.x;
  auto bsum = [&](double v) -> double {
    red[tid] = v;
    __syncthreads();
    for (int s = kObjThreads / 2; s; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    const double out = red[0];
    __syncthreads();
    return out;
  };
  double ar = 0, at = 0, sr = 0, st = 0;
  if (fcn == DVC_ZSSD || fcn == DVC_ZNSSD) {
    double a1 = 0, a2 = 0;
    for (int i = tid; i < n; i += kObjThreads) {
      a1 += r[i];
      a2 += t[i];
    }
    ar = bsum(a1) / n;
    at = bsum(a2) / n;
  }
  if (fcn == DVC_NSSD || fcn == DVC_ZNSSD) {
    double b1 = 0, b2 = 0;
    for (int i = tid; i < n; i += kObjThreads) {
      b1 += (r[i] - ar) * (r[i] - ar);
      b2 += (t[i] - at) * (t[i] - at);
    }
    sr = sqrt(bsum(b1));
    st = sqrt(bsum(b2));
  }
  double acc = 0;
  for (int i = tid; i < n; i += kObjThreads) {
    double diff;
    switch (fcn) {
      case DVC_SAD:
      case DVC_SSD: diff = t[i] - r[i]; break;
      case DVC_ZSSD: diff = (t[i] - at) - (r[i] - ar); break;
      case DVC_NSSD: diff = t[i] / st - r[i] / sr; break;
      default: diff = ((t[i] - at) / st) - ((r[i] - ar) / sr); break;
    }
    if (res) res[i] = diff;
    acc += (fcn == DVC_SAD) ? fabs(diff) : diff * diff;
  }
  double o = bsum(acc);
  if (tid == 0) {
    if (fcn == DVC_NSSD) o /= 2.0;
    if (fcn == DVC_ZNSSD) o /= 4.0;
    *obj = o;
  }
}

// ------------------------------------------- dataflow scheduling set-up ---
// Edge (i = order[r], m = neigh[i][j]) is a dependency of i when the reference
// processes m before i (rank[m] < r): Search::starting_param then reads m's
// result (Core/Search.cpp:297-356). The ranks may be cut into up to three
// windows, [0, w1), [w1, w2), [w2, n_process), searched by consecutive
// launches: only edges inside one window are kept (a predecessor in an
// earlier window has finished before the window's launch starts).
__host__ __device__ inline int rank_window(int r, int w1, int w2) { return (r >= w1) + (r >= w2); }
// the window's work counter and ready-queue tail in the control block's ints
// (int 1 is the error flag)
__host__ __device__ constexpr int window_work_int(int w) { return w == 0 ? 0 : 1 + 2 * w; }
__host__ __device__ constexpr int window_tail_int(int w) { return 2 + 2 * w; }

__global__ void dep_count_kernel(int n_process, int n_points, int nn, const int *order,
                                 const int *neigh, const int *rank, int w1, int w2, int *pend,
                                 int *succ_cnt) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)n_process * nn) return;
  const int r = (int)(k / nn), j = (int)(k % nn);
  const int i = order[r];
  if (i < 0 || i >= n_points) return;
  const int m = neigh[(size_t)i * nn + j];
  if (m < 0 || m >= n_points || rank[m] >= r) return;
  if (rank_window(rank[m], w1, w2) != rank_window(r, w1, w2)) return;
  atomicAdd(pend + i, 1);
  atomicAdd(succ_cnt + m, 1);
}

__global__ void dep_fill_kernel(int n_process, int n_points, int nn, const int *order,
                                const int *neigh, const int *rank, int w1, int w2, const int *succ_off,
                                int *cursor, int *succ) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (long long)n_process * nn) return;
  const int r = (int)(k / nn), j = (int)(k % nn);
  const int i = order[r];
  if (i < 0 || i >= n_points) return;
  const int m = neigh[(size_t)i * nn + j];
  if (m < 0 || m >= n_points || rank[m] >= r) return;
  if (rank_window(rank[m], w1, w2) != rank_window(r, w1, w2)) return;
  succ[succ_off[m] + atomicAdd(cursor + m, 1)] = i;
}

// exclusive prefix sum of in[0..n) into out[0..n], one CTA of 1024 threads
__global__ void __launch_bounds__(1024) exclusive_scan_kernel(int n, const int *in, int *out) {
  __shared__ int wsum[32];
  __shared__ int carry;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int v = base + t < n ? in[base + t] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = wsum[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    const int incl = x + (warp > 0 ? wsum[warp - 1] : 0);
    if (base + t < n) out[base + t] = carry + incl - v;
    __syncthreads();
    if (t == 1023) carry += incl;
    __syncthreads();
  }
  if (t == 0) out[n] = carry;
}

// points without predecessors in their window start that window's ready
// queue (window w's slots begin at its first rank)
__global__ void ready_kernel(int n_process, int n_points, const int *order, const int *pend, int w1,
                             int w2, int *queue, int *ctl) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_process) return;
  const int i = order[r];
  if (i < 0 || i >= n_points || pend[i] != 0) return;
  const int w = rank_window(r, w1, w2);
  const int start = w == 0 ? 0 : (w == 1 ? w1 : w2);
  queue[start + atomicAdd(ctl + window_tail_int(w), 1)] = i;
}

__global__ void byteswap16_kernel(uint16_t *v, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint16_t)((v[i] >> 8) | (v[i] << 8));
}

}  // namespace

// ================================================================ engine ===
struct dvc_engine {
  dvc_params p;
  int device;
  void *ref = nullptr, *cor = nullptr;
  bool owns_volumes = false;
  int n_sub = 0, cube_n = 0;
  double subv_rad = 0;
  double nom_mn[3], nom_mx[3], nom_cen[3];
  int bext[3];
  double morton_rad = 0.0;
  std::vector<double> h_offsets;  // stable sample offsets from the point (sample order)
  // the same split into whole voxels and FP32 fractions in [0, 1)
  int *d_off_i = nullptr;
  float *d_off_f = nullptr;
  double *d_rand_off = nullptr;  // random_global's translations (coarse_method random)
  // grow-only per-call workspace
  void *ws = nullptr;
  size_t ws_bytes = 0;
  // control block of the last search call (work counter, error flag, queue
  // tail, counters from +64): in ws, or in the allocation-free scratch
  char *last_ctl = nullptr;
  long long wait_polls = -1;  // dependency-wait bound of the search (< 0: default)
  // counters of the last call when it made several launches (the learned
  // search), summed on the host; otherwise read from last_ctl
  bool counts_host = false;
  unsigned long long host_counts[3] = {0, 0, 0};
  int num_sms = 0;
  int cluster = 0;          // CTAs per point (0 = choose per call)
  int last_cluster = 0, last_grid = 0, last_staged = 0, last_smem = 0;
  // rank windows of the last dataflow search: [0, w1) and [w2, n) at width
  // last_windows[2], the body at last_cluster
  int last_windows[3] = {0, 0, 0};
};

// Several configurations on the same volumes, one launch shape for all.
struct dvc_plan {
  std::vector<dvc_engine *> cfgs;  // not owned
  std::vector<SearchCfg> h_cfgs;   // the device table's host copy
  int cluster = 0;                 // CTAs per point
  int staging = 1;                 // staging allowed
  int n_staged = 0;
  int cap = 0;                     // per-CTA sample capacity (largest over configurations)
  size_t stage_bytes = 0, smem_dyn = 0;
  int max_clusters = 0;            // clusters resident at once
  SearchCfg *d_cfgs = nullptr;     // device: one record per configuration
  CUtensorMap *d_tmaps = nullptr;  // device: two tensor maps per configuration (correlate, reference)
};

namespace {

int validate(const dvc_params *p) {
  if (!p) return set_error(DVC_E_ARG, "null params");
  if (p->bytes_per_voxel != 1 && p->bytes_per_voxel != 2)
    return set_error(DVC_E_ARG, "bytes_per_voxel must be 1 or 2 (vol_bit_depth 8 or 16)");
  if (p->vol_wide <= 0 || p->vol_high <= 0 || p->vol_tall <= 0 || p->vol_wide > 8000 ||
      p->vol_high > 8000 || p->vol_tall > 8000)
    return set_error(DVC_E_ARG, "volume dimensions must be in 1..8000");
  if (p->subvol_geom != DVC_CUBE && p->subvol_geom != DVC_SPHERE)
    return set_error(DVC_E_ARG, "subvol_geom must be cube or sphere");
  if (p->subvol_npts < 1 || p->subvol_npts > 50000)
    return set_error(DVC_E_ARG, "subvol_npts must be in 1..50000");
  if (p->subvol_size < 1) return set_error(DVC_E_ARG, "subvol_size must be >= 1");
  if (p->subvol_thresh) {
    const double top = p->bytes_per_voxel == 1 ? 256.0 : 65536.0;  // 2^vol_bit_depth
    if (!(p->gray_thresh_min >= 0.0) || !(p->gray_thresh_max > p->gray_thresh_min) ||
        !(p->gray_thresh_max <= top))
      return set_error(DVC_E_ARG, "gray thresholds must satisfy 0 <= min < max <= 2^vol_bit_depth");
    if (!(p->min_vol_fract >= 0.0 && p->min_vol_fract <= 1.0))
      return set_error(DVC_E_ARG, "min_vol_fract must be in 0..1");
  }
  if (p->num_srch_dof != 3 && p->num_srch_dof != 6 && p->num_srch_dof != 12)
    return set_error(DVC_E_ARG, "num_srch_dof must be 3, 6 or 12");
  if (p->obj_function < 0 || p->obj_function > 4) return set_error(DVC_E_ARG, "bad obj_function");
  if (p->interp_type < 0 || p->interp_type > 2) return set_error(DVC_E_ARG, "bad interp_type");
  if (p->disp_max < 0) return set_error(DVC_E_ARG, "disp_max must be >= 0");
  if (!(p->basin_radius >= 0.0) || p->basin_radius > p->disp_max)
    return set_error(DVC_E_ARG, "basin_radius must be in [0, disp_max]");
  for (int d = 0; d < 3; d++)
    if (!(p->subvol_aspect[d] >= 0.1 && p->subvol_aspect[d] <= 10.0))
      return set_error(DVC_E_ARG, "subvol_aspect components must be in [0.1, 10]");
  if (p->coarse_method != DVC_COARSE_GRID && p->coarse_method != DVC_COARSE_RANDOM)
    return set_error(DVC_E_ARG, "coarse_method must be DVC_COARSE_GRID or DVC_COARSE_RANDOM");
  if (p->refine_method != DVC_REFINE_GAUSS_NEWTON && p->refine_method != DVC_REFINE_NELDER_MEAD)
    return set_error(DVC_E_ARG, "refine_method must be DVC_REFINE_GAUSS_NEWTON or DVC_REFINE_NELDER_MEAD");
  return DVC_OK;
}

// random_global's translations (Core/Search.cpp:1045-1098): num_pts of them,
// 3 draws each in x, y, z order, displ_max * (2 * rand()) / RAND_MAX with the
// doubled draw an int product (wrapping as two's complement above 2^30, as
// the reference's compiled code does); rand() after srand(seed) is the C
// library's generator, drawn here from a private state (initstate_r /
// random_r give the same sequence) so the caller's rand() is left alone.
std::vector<double> random_global_offsets(int num_pts, double displ_max, unsigned seed) {
  struct random_data rd;
  memset(&rd, 0, sizeof rd);
  int32_t state[32];  // the 128-byte state of srand() / rand()
  initstate_r(seed, reinterpret_cast<char *>(state), sizeof state, &rd);
  const double dbl_rand_max = RAND_MAX;
  std::vector<double> rel((size_t)num_pts * 3);
  for (size_t k = 0; k < rel.size(); k++) {
    int32_t r = 0;
    random_r(&rd, &r);
    const int twice = (int)(2u * (uint32_t)r);
    rel[k] = displ_max * (twice / dbl_rand_max);
  }
  return rel;
}

// Search::Search geometry: subvolume count and the nominal interpolation box
// (Core/Search.cpp:24-82).
void engine_geometry(dvc_engine *e) {
  const dvc_params &p = e->p;
  e->subv_rad = p.subvol_size / 2.0;
  if (p.subvol_geom == DVC_CUBE) {
    e->n_sub = (int)pow(ceil(pow((double)p.subvol_npts, 1.0 / 3.0)), 3.0);
    e->cube_n = (int)ceil(pow((double)e->n_sub, 1.0 / 3.0));
  } else {
    e->n_sub = p.subvol_npts;
    e->cube_n = 0;
  }
  for (int d = 0; d < 3; d++) {
    double mn = 0.0, mx = 2 * e->subv_rad * p.subvol_aspect[d];
    // grow_by(disp_max) then grow_by(2.0): min + (-f), max + f
    mn = mn + (-(double)p.disp_max);
    mx = mx + (double)p.disp_max;
    mn = mn + (-2.0);
    mx = mx + 2.0;
    e->nom_mn[d] = mn;
    e->nom_mx[d] = mx;
    e->nom_cen[d] = (mn + mx) / 2.0;
    e->bext[d] = (int)mx - (int)mn;
  }
}

// Sphere sample offsets: FloatingCloud's rejection sampling with
// std::mt19937 and uniform_real_distribution<double>(-r, r)
// (Core/FloatingCloud.cpp:40-82). Host code, the same library generator.
std::vector<double> sphere_offsets(double rad, int num, unsigned seed) {
  std::mt19937 mt(seed);
  std::uniform_real_distribution<double> dist(-rad, rad);
  std::vector<double> out;
  out.reserve((size_t)num * 3);
  int count = 0;
  while (count < num) {
    double rx = dist(mt);
    double ry = dist(mt);
    double rz = dist(mt);
    double radius = std::sqrt(rx * rx + ry * ry + rz * rz);
    if (radius <= rad) {
      count += 1;
      out.push_back(rx);
      out.push_back(ry);
      out.push_back(rz);
    }
  }
  return out;
}

// The samples' order only changes the order of the sums; a space-filling
// (Morton) order keeps each warp's gathers, and each cluster CTA's share of
// the subvolume, spatially compact.
std::vector<size_t> morton_perm(const std::vector<double> &rel, double rad) {
  const size_t n = rel.size() / 3;
  std::vector<std::pair<uint64_t, size_t>> key(n);
  for (size_t i = 0; i < n; i++) {
    uint64_t code = 0;
    uint32_t q[3];
    for (int d = 0; d < 3; d++) {
      double u = (rel[i * 3 + d] + rad) / (2.0 * rad + 1e-9);
      q[d] = (uint32_t)std::min(1023.0, std::max(0.0, u * 1024.0));
    }
    for (int b = 9; b >= 0; b--)
      for (int d = 2; d >= 0; d--) code = (code << 1) | ((q[d] >> b) & 1u);
    key[i] = {code, i};
  }
  std::stable_sort(key.begin(), key.end(),
                   [](const std::pair<uint64_t, size_t> &x, const std::pair<uint64_t, size_t> &y) {
                     return x.first < y.first;
                   });
  std::vector<size_t> perm(n);
  for (size_t i = 0; i < n; i++) perm[i] = key[i].second;
  return perm;
}

// Cluster rank ranges: with samples in Morton order, the first 1, 2 or 3
// code bits select the half, quarter slab or octant of the subvolume, so each
// CTA of a 2-, 4- or 8-wide cluster gets one compact piece.
void rank_ranges(const std::vector<double> &off, double rad, int C, int out[9]) {
  const size_t n = off.size() / 3;
  int bits = 0;
  while ((1 << bits) < C) bits++;
  int cnt[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (size_t i = 0; i < n; i++) {
    uint32_t top = 0;
    // same quantisation as morton_perm; top bits interleave z, y, x
    uint32_t q[3];
    for (int d = 0; d < 3; d++) {
      double u = (off[i * 3 + d] + rad) / (2.0 * rad + 1e-9);
      q[d] = (uint32_t)std::min(1023.0, std::max(0.0, u * 1024.0));
    }
    const uint32_t code3 = ((q[2] >> 9) << 2) | ((q[1] >> 9) << 1) | (q[0] >> 9);
    top = code3 >> (3 - bits);
    cnt[top + 1]++;
  }
  for (int r = 0; r < C; r++) cnt[r + 1] += cnt[r];
  for (int r = 0; r <= C; r++) out[r] = cnt[r];
  for (int r = C + 1; r < 9; r++) out[r] = out[C];
}

int engine_finish(dvc_engine *e) {
  engine_geometry(e);
  if (e->bext[0] > 1023 || e->bext[1] > 1023 || e->bext[2] > 1023)
    return set_error(DVC_E_ARG, "interpolation box larger than 1023 voxels per axis");
  const double rmax = e->subv_rad * std::max(e->p.subvol_aspect[0],
                                             std::max(e->p.subvol_aspect[1], e->p.subvol_aspect[2]));
  e->morton_rad = rmax;
  if (e->p.subvol_geom == DVC_SPHERE) {
    std::vector<double> rel0 = sphere_offsets(e->subv_rad, e->n_sub, e->p.sphere_seed);
    std::vector<double> sc(rel0.size());
    for (size_t i = 0; i < rel0.size(); i++) sc[i] = e->p.subvol_aspect[i % 3] * rel0[i];
    const std::vector<size_t> pm = morton_perm(sc, rmax);
    std::vector<double> rel(rel0.size());
    for (size_t i = 0; i < pm.size(); i++)
      for (int d = 0; d < 3; d++) rel[i * 3 + d] = rel0[pm[i] * 3 + d];
    e->h_offsets.resize(rel.size());
    for (size_t i = 0; i < rel.size(); i++) e->h_offsets[i] = e->p.subvol_aspect[i % 3] * rel[i];
  } else {
    // cube samples on the n^3 grid (FloatingCloud, Core/FloatingCloud.cpp:84-128),
    // taken in a space-filling order
    const int nn = e->cube_n;
    std::vector<double> off((size_t)e->n_sub * 3);
    for (int i = 0; i < e->n_sub; i++) {
      const int idx[3] = {i % nn, (i / nn) % nn, i / (nn * nn)};
      for (int d = 0; d < 3; d++) {
        const double r = e->subv_rad * e->p.subvol_aspect[d];
        off[(size_t)i * 3 + d] = -r + idx[d] * (2.0 * r / std::max(1, nn - 1));
      }
    }
    const std::vector<size_t> perm = morton_perm(off, rmax);
    e->h_offsets.resize(off.size());
    for (size_t i = 0; i < perm.size(); i++)
      for (int d = 0; d < 3; d++) e->h_offsets[i * 3 + d] = off[perm[i] * 3 + d];
  }
  {
    const size_t m = e->h_offsets.size();
    std::vector<int> oi(m);
    std::vector<float> of(m);
    for (size_t k = 0; k < m; k++) {
      const double fl = std::floor(e->h_offsets[k]);
      oi[k] = (int)fl;
      of[k] = (float)(e->h_offsets[k] - fl);
    }
    CUDA_TRY(cudaMalloc(&e->d_off_i, m * sizeof(int)));
    CUDA_TRY(cudaMalloc(&e->d_off_f, m * sizeof(float)));
    CUDA_TRY(cudaMemcpy(e->d_off_i, oi.data(), m * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(e->d_off_f, of.data(), m * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (e->p.coarse_method == DVC_COARSE_RANDOM && e->p.basin_radius != 0.0) {
    const int num_inc = (int)(e->p.disp_max / e->p.basin_radius);
    const int side = 2 * num_inc + 1;
    const std::vector<double> rel = random_global_offsets(side * side * side, e->p.disp_max, e->p.coarse_seed);
    CUDA_TRY(cudaMalloc(&e->d_rand_off, rel.size() * sizeof(double)));
    CUDA_TRY(cudaMemcpy(e->d_rand_off, rel.data(), rel.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  CUDA_TRY(cudaGetDevice(&e->device));
  CUDA_TRY(cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->device));
  if (const char *env = getenv("DVC_CLUSTER")) {
    const int c = atoi(env);
    if (c == 1 || c == 2 || c == 4 || c == 8) e->cluster = c;
  }
  return DVC_OK;
}

size_t state_bytes(int cap) {
  // per-CTA dynamic shared memory: packed cell base, fraction (3), reference
  // quantity, final value per local sample; Gauss-Newton chunk rows
  return (size_t)cap * 24 + (size_t)kGRows * kThreads * 4;
}

int ensure_ws(dvc_engine *e, size_t bytes) {
  if (bytes <= e->ws_bytes) return DVC_OK;
  if (e->ws) cudaFree(e->ws);
  e->ws = nullptr;
  e->ws_bytes = 0;
  if (cudaMalloc(&e->ws, bytes) != cudaSuccess) return set_error(DVC_E_NOMEM, "workspace allocation failed");
  e->ws_bytes = bytes;
  return DVC_OK;
}

template <typename VT, int IT, int MINB>
int launch_search(SearchArgs &a, const CUtensorMap &tmap, const CUtensorMap &tmap_ref, size_t smem_dyn,
                  int grid, int cluster, cudaStream_t st, int *max_clusters) {
  auto kern = search_kernel<VT, IT, MINB>;
  CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_dyn));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem_dyn;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (max_clusters) {  // occupancy query only
    cfg.gridDim = dim3(cluster, 1, 1);
    CUDA_TRY(cudaOccupancyMaxActiveClusters(max_clusters, kern, &cfg));
    return DVC_OK;
  }
  cfg.gridDim = dim3(grid, 1, 1);
  CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, a, tmap, tmap_ref));
  return DVC_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// Staging box for a cluster of C CTAs: per CTA rank, the extent of its share
// of the stable sample offsets, plus stencil, rounding and warp margins; x
// rounded so every copy starts and spans whole 16-byte units.
void stage_dims(const dvc_engine *e, int C, int esize, double reach, const int rs[9], bool odd,
                int out[3], bool zreach = true) {
  double emax[3] = {0.0, 0.0, 0.0};
  for (int r = 0; r < C; r++) {
    const int lo = rs[r], hi = rs[r + 1];
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int i = lo; i < hi; i++)
      for (int d = 0; d < 3; d++) {
        mn[d] = std::min(mn[d], e->h_offsets[(size_t)i * 3 + d]);
        mx[d] = std::max(mx[d], e->h_offsets[(size_t)i * 3 + d]);
      }
    for (int d = 0; d < 3; d++) emax[d] = std::max(emax[d], mx[d] - mn[d]);
  }
  const int al = 16 / esize;
  for (int d = 0; d < 3; d++) out[d] = (int)ceil(emax[d] + ((d < 2 || zreach) ? 2.0 * reach : 0.0)) + 6;
  // rows of an odd number of 16-byte units: consecutive rows then start in
  // all eight 16-byte bank groups, so the gathers of nearby samples spread
  // over the 32 shared-memory banks (an even count uses half of them)
  int units = (out[0] + al - 1 + al - 1) / al;
  if (odd && units % 2 == 0) units++;
  out[0] = units * al;
}

// minb 2: the kernel whose registers leave room for two CTAs per SM
// (tricubic only)
int dispatch_launch(int bpv, int it, SearchArgs &a, const CUtensorMap &tm, const CUtensorMap &tmr, size_t smem,
                    int grid, int cluster, cudaStream_t st, int *max_clusters, int minb = 1) {
  if (minb == 2 && it == 2) {
    if (bpv == 1) return launch_search<uint8_t, 2, 2>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
    return launch_search<uint16_t, 2, 2>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
  }
  if (bpv == 1) {
    if (it == 2) return launch_search<uint8_t, 2, 1>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
    if (it == 1) return launch_search<uint8_t, 1, 1>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
    return launch_search<uint8_t, 0, 1>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
  }
  if (it == 2) return launch_search<uint16_t, 2, 1>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
  if (it == 1) return launch_search<uint16_t, 1, 1>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
  return launch_search<uint16_t, 0, 1>(a, tm, tmr, smem, grid, cluster, st, max_clusters);
}

// ---- launch preparation ------------------------------------------------------
// Dynamic shared memory a search CTA may use on the current device: what a
// block may opt into, less the kernel's static CtaState and a little slack.
int dyn_budget(size_t *out) {
  static int optin[64] = {0};
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(DVC_E_ARG, "device index out of range");
  if (!optin[dev]) CUDA_TRY(cudaDeviceGetAttribute(&optin[dev], cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  *out = (size_t)optin[dev] - sizeof(CtaState) - 1024;
  return DVC_OK;
}

// TMA staging of the volumes needs 16-byte aligned rows, planes and bases.
bool tma_layout(const dvc_engine *e) {
  const dvc_params &p = e->p;
  const int esize = p.bytes_per_voxel;
  return encode_tiled_fn() != nullptr && ((size_t)p.vol_wide * esize) % 16 == 0 &&
         ((size_t)p.vol_wide * p.vol_high * esize) % 16 == 0 && ((uintptr_t)e->cor % 16) == 0 &&
         ((uintptr_t)e->ref % 16) == 0 &&
         !getenv("DVC_NO_STAGE");
}

// Engine e's settings as one search configuration at cluster width C:
// subvolume geometry, coarse grid, sample tables, each rank's sample range and
// the offset extrema over all samples and per rank (the sample clouds'
// bounding boxes follow from them: FP64 addition of the point is monotone).
// Staging is left off. Returns the largest per-rank sample count.
int fill_config(const dvc_engine *e, int C, SearchCfg &k) {
  const dvc_params &p = e->p;
  k = SearchCfg{};
  k.geom = p.subvol_geom;
  k.ndof = p.num_srch_dof;
  k.objfcn = p.obj_function;
  k.n_sub = e->n_sub;
  k.cube_n = e->cube_n;
  k.subv_rad = e->subv_rad;
  for (int d = 0; d < 3; d++) {
    k.aspect[d] = p.subvol_aspect[d];
    k.nom_mn[d] = e->nom_mn[d];
    k.nom_mx[d] = e->nom_mx[d];
    k.nom_cen[d] = e->nom_cen[d];
    k.bext[d] = e->bext[d];
    k.rigid[d] = p.rigid_trans[d];
  }
  k.do_grid = p.basin_radius != 0.0;
  if (k.do_grid) {
    const double displ_max = p.disp_max;
    k.num_inc = (int)(displ_max / p.basin_radius);
    k.inc = displ_max / k.num_inc;
    k.inc_int = (k.inc == std::floor(k.inc) && k.inc <= 64.0 && !getenv("DVC_GENERAL_GRID")) ? (int)k.inc : 0;
  }
  k.coarse_random = (k.do_grid && p.coarse_method == DVC_COARSE_RANDOM) ? 1 : 0;
  k.rand_off = e->d_rand_off;
  k.refine_nm = p.refine_method == DVC_REFINE_NELDER_MEAD ? 1 : 0;
  k.thresh_on = p.subvol_thresh ? 1 : 0;
  k.gmin = (float)p.gray_thresh_min;
  k.gmax = (float)p.gray_thresh_max;
  k.min_count = p.min_vol_fract * e->n_sub;
  k.inv_nsub = 1.0 / (double)e->n_sub;
  rank_ranges(e->h_offsets, e->morton_rad, C, k.rank_start);
  k.off_i = e->d_off_i;
  k.off_f = e->d_off_f;
  for (int d = 0; d < 3; d++) {
    k.off_min[d] = 1e300;
    k.off_max[d] = -1e300;
  }
  int cap = 0;
  for (int r = 0; r < C; r++) {
    cap = std::max(cap, k.rank_start[r + 1] - k.rank_start[r]);
    for (int d = 0; d < 3; d++) {
      double mn = 1e300, mx = -1e300;
      for (int i = k.rank_start[r]; i < k.rank_start[r + 1]; i++) {
        mn = std::min(mn, e->h_offsets[(size_t)i * 3 + d]);
        mx = std::max(mx, e->h_offsets[(size_t)i * 3 + d]);
      }
      k.rank_off_min[r][d] = mn;
      k.rank_off_max[r][d] = mx;
      k.off_min[d] = std::min(k.off_min[d], mn);
      k.off_max[d] = std::max(k.off_max[d], mx);
    }
  }
  return cap;
}

// Staging box of configuration k (filled at width C) when it fits `budget`
// together with `state` bytes of per-CTA sample state: one region per point
// covers every grid translation (reach k * inc) when the grid runs; odd row
// pitch (in 16-byte units) first, then the plain one. Returns the staging
// buffer's bytes, 0 when the box does not fit (k then stays unstaged).
size_t stage_config(const dvc_engine *e, int C, size_t budget, size_t state, bool grid, SearchCfg &k) {
  const dvc_params &p = e->p;
  const int esize = p.bytes_per_voxel;
  double reach = 0.0;
  int side = 1;
  if (grid && p.basin_radius != 0.0) {
    const int n = (int)((double)p.disp_max / p.basin_radius);
    reach = n * ((double)p.disp_max / n);
    side = 2 * n + 1;
  }
  // a slab is reduced as one chunk of side^2 translations: at most
  // kGridChunk of them (grids of side 13 and more stage the whole box or
  // nothing)
  const bool slab_ok = side * side <= kGridChunk;
  // the box covers the grid's translations in x, y and z; when that does not
  // fit, one z slab of translations at a time (the grid restages per slab)
  int stage[3] = {0, 0, 0};
  size_t bytes = 0;
  bool fits = false;
  int slab = 0;
  for (int zr = 1; zr >= 0 && !fits; zr--) {
    if (zr == 0 && (reach == 0.0 || !slab_ok)) break;
    for (int odd = 1; odd >= 0; odd--) {
      stage_dims(e, C, esize, reach, k.rank_start, odd != 0, stage, zr != 0);
      bytes = (((size_t)stage[0] * stage[1] * stage[2] * esize + 16) + 127) & ~(size_t)127;
      fits = bytes + state <= budget && stage[0] <= 256 && stage[1] <= 256 && stage[2] <= 256;
      if (fits) break;
    }
    slab = zr == 0;
  }
  if (!fits || (slab && getenv("DVC_NO_SLAB"))) return 0;
  k.stage_on = 1;
  k.stage_slab = slab;
  for (int d = 0; d < 3; d++) k.stage[d] = stage[d];
  k.stage_tx = (unsigned)((size_t)stage[0] * stage[1] * stage[2] * esize);
  // the reference region needs no grid reach: a smaller box in the same
  // buffer (odd pitch when it fits, else the plain one, else the full box)
  const size_t full = (size_t)stage[0] * stage[1] * stage[2] * esize;
  int sr[3];
  bool fit = false;
  for (int odd = 1; odd >= 0 && !fit; odd--) {
    stage_dims(e, C, esize, 0.0, k.rank_start, odd != 0, sr);
    fit = (size_t)sr[0] * sr[1] * sr[2] * esize <= full;
  }
  for (int d = 0; d < 3; d++) k.stage_ref[d] = fit ? sr[d] : stage[d];
  k.stage_ref_tx = (unsigned)((size_t)k.stage_ref[0] * k.stage_ref[1] * k.stage_ref[2] * esize);
  return bytes;
}

// Tensor map of volume `vol` (the engine's correlate or reference volume)
// with box `bx` (the configuration's correlate or reference staging box).
bool encode_stage_map(const dvc_engine *e, const int bx[3], const void *vol, CUtensorMap *tm) {
  const dvc_params &p = e->p;
  const int esize = p.bytes_per_voxel;
  memset(tm, 0, sizeof *tm);
  const cuuint64_t gdim[3] = {(cuuint64_t)p.vol_wide, (cuuint64_t)p.vol_high, (cuuint64_t)p.vol_tall};
  const cuuint64_t gstride[2] = {(cuuint64_t)p.vol_wide * esize, (cuuint64_t)p.vol_wide * p.vol_high * esize};
  const cuuint32_t box[3] = {(cuuint32_t)bx[0], (cuuint32_t)bx[1], (cuuint32_t)bx[2]};
  const cuuint32_t estride[3] = {1, 1, 1};
  return encode_tiled_fn()(tm, esize == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3,
                           const_cast<void *>(vol), gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The control block at the start of every search call's scratch: int work
// counter, int error flag, int ready-queue tail, then the 64-bit counters.
constexpr size_t kCtlBytes = 256;
constexpr size_t kCountersOff = 64;
static_assert(kCountersOff + kNumCounters * sizeof(unsigned long long) <= kCtlBytes, "control block");
static_assert((window_work_int(2) + 1) * sizeof(int) <= kCountersOff &&
                  (window_tail_int(2) + 1) * sizeof(int) <= kCountersOff,
              "window counters before the 64-bit counters");

// One search call's points, seeds and outputs (device pointers).
struct RunIO {
  int n_points;
  const double *points;
  int n_process;
  const int *order;
  int n_neigh;
  const int *neigh;
  int seed_mode;
  const double *seeds;
  int *status;
  double *objmin;
  double *params;
  int *gn_iters;
};

// Dataflow scheduling (predecessor counts, successor lists, ready queues)
// for the reference's seeding with neighbour lists, unless the scratch is the
// caller's fixed array or DVC_IN_ORDER asks for processing order.
bool uses_dataflow(const RunIO &io, const char *ws_fixed) {
  return io.seed_mode == DVC_SEED_NEIGHBOURS && io.n_neigh > 0 && !ws_fixed && !getenv("DVC_IN_ORDER");
}

int check_run(const dvc_engine *e, const RunIO &io) {
  if (!e) return set_error(DVC_E_ARG, "null engine");
  if (io.n_points < 0 || io.n_process < 0 || io.n_process > io.n_points)
    return set_error(DVC_E_ARG, "n_process must be in 0..n_points");
  if (io.seed_mode < 0 || io.seed_mode > 3) return set_error(DVC_E_ARG, "bad seed_mode");
  if (io.seed_mode == DVC_SEED_NEIGHBOURS && io.n_neigh > 0 && !io.neigh)
    return set_error(DVC_E_ARG, "neighbour list required");
  if ((io.seed_mode == DVC_SEED_GIVEN || io.seed_mode == DVC_SEED_PARAMS) && !io.seeds)
    return set_error(DVC_E_ARG, "seeds required");
  return DVC_OK;
}

// The run's scratch and per-call preparation, enqueued on `st`: scratch in
// engine e's grow-only workspace (or `ws_fixed`), outputs initialised, ranks
// of the processing order, and with dataflow scheduling the predecessor
// counts, successor lists and ready queues of the rank windows [0, w1),
// [w1, w2), [w2, n_process) (w1 = w2 = n_process: one window). Fills the run
// fields of `a` for window 0 (run_window gives the others).
int prepare_run(dvc_engine *e, const RunIO &io, cudaStream_t st, char *ws_fixed, size_t ws_fixed_bytes,
                SearchArgs &a, int w1, int w2) {
  const int n_points = io.n_points, n_process = io.n_process, n_neigh = io.n_neigh;
  w2 = std::max(0, std::min(w2, n_process));
  w1 = std::max(0, std::min(w1, w2));
  // workspace: the control block (kCtlBytes: work counter, error flag, queue
  // tail, counters from +kCountersOff), done[n], rank[n]; with dataflow
  // scheduling also the predecessor counts, successor lists and ready queue.
  // The control block comes first, so its place does not depend on the size.
  const size_t off_ctl = 0;
  const size_t off_done = kCtlBytes;
  const size_t off_rank = off_done + (size_t)n_points * 4;
  const bool dataflow = uses_dataflow(io, ws_fixed);
  const size_t off_pend = (off_rank + (size_t)n_points * 4 + 255) & ~(size_t)255;
  const size_t off_soff = off_pend + (size_t)n_points * 4;
  const size_t off_cursor = off_soff + ((size_t)n_points + 1) * 4;
  const size_t off_queue = off_cursor + (size_t)n_points * 4;
  const size_t off_succ = off_queue + (size_t)n_process * 4;
  const size_t ws_need = dataflow ? off_succ + (size_t)n_process * n_neigh * 4 : off_pend;
  char *ws = ws_fixed;
  if (ws) {
    if (ws_need > ws_fixed_bytes) return set_error(DVC_E_ARG, "search scratch larger than the fixed array");
  } else {
    const int rc = ensure_ws(e, ws_need);
    if (rc) return rc;
    ws = (char *)e->ws;
  }
  e->last_ctl = ws + off_ctl;
  e->counts_host = false;
  int *done = (int *)(ws + off_done);
  int *rank = (int *)(ws + off_rank);
  int *ctl = (int *)(ws + off_ctl);
  CUDA_TRY(cudaMemsetAsync(ws + off_ctl, 0, kCtlBytes, st));
  {
    const int T = 256;
    const int G = (n_points + T - 1) / T;
    init_outputs_kernel<<<G, T, 0, st>>>(n_points, io.status, io.objmin, io.params, io.gn_iters, done, rank);
    if (n_process > 0)
      rank_kernel<<<(n_process + T - 1) / T, T, 0, st>>>(n_process, io.order, rank, n_points);
    CUDA_TRY(cudaGetLastError());
  }
  if (dataflow && n_process > 0) {
    const int T = 256;
    int *pend = (int *)(ws + off_pend), *soff = (int *)(ws + off_soff);
    int *cursor = (int *)(ws + off_cursor), *queue = (int *)(ws + off_queue);
    CUDA_TRY(cudaMemsetAsync(ws + off_pend, 0, off_queue - off_pend, st));  // pend, counts, cursor
    CUDA_TRY(cudaMemsetAsync(queue, 0xFF, (size_t)n_process * 4, st));       // -1: slot empty
    const long long edges = (long long)n_process * n_neigh;
    const unsigned eg = (unsigned)((edges + T - 1) / T);
    dep_count_kernel<<<eg, T, 0, st>>>(n_process, n_points, n_neigh, io.order, io.neigh, rank, w1, w2, pend,
                                       soff);
    exclusive_scan_kernel<<<1, 1024, 0, st>>>(n_points, soff, soff);
    dep_fill_kernel<<<eg, T, 0, st>>>(n_process, n_points, n_neigh, io.order, io.neigh, rank, w1, w2, soff,
                                      cursor, (int *)(ws + off_succ));
    ready_kernel<<<(n_process + T - 1) / T, T, 0, st>>>(n_process, n_points, io.order, pend, w1, w2, queue, ctl);
    CUDA_TRY(cudaGetLastError());
  }
  a.ref = e->ref;
  a.cor = e->cor;
  a.nx = e->p.vol_wide;
  a.ny = e->p.vol_high;
  a.nz = e->p.vol_tall;
  a.itype = e->p.interp_type;
  a.n_points = n_points;
  a.n_process = n_process;
  a.n_neigh = (io.seed_mode == DVC_SEED_NEIGHBOURS) ? n_neigh : 0;
  a.seed_mode = io.seed_mode;
  a.pts = io.points;
  a.order = io.order;
  a.rank = rank;
  a.neigh = io.neigh;
  a.seeds = io.seeds;
  a.status = io.status;
  a.objmin = io.objmin;
  a.params = io.params;
  a.gn_iters = io.gn_iters;
  a.work_counter = ctl;
  a.error_flag = ctl + 1;
  a.dataflow = dataflow ? 1 : 0;
  if (dataflow) {
    a.pend = (int *)(ws + off_pend);
    a.succ_off = (const int *)(ws + off_soff);
    a.succ = (const int *)(ws + off_succ);
    a.queue = (int *)(ws + off_queue);
    a.queue_tail = ctl + window_tail_int(0);
    a.n_process = std::min(n_process, w1);
  }
  a.done = done;
  a.counters = (unsigned long long *)(ws + off_ctl + kCountersOff);
  a.wait_polls = e->wait_polls < 0 ? kWaitPolls : e->wait_polls;
  return DVC_OK;
}

// The run fields of prepare_run's `a0` (window 0) moved to rank window w of
// a dataflow run: its work counter, ready-queue slots and tail, its size.
SearchArgs window_args(const SearchArgs &a0, int w, int w1, int w2, int n_process) {
  SearchArgs a = a0;
  int *ctl = a0.work_counter;  // window 0's work counter is the control block's first int
  const int lo = w == 0 ? 0 : (w == 1 ? w1 : w2);
  const int hi = w == 0 ? w1 : (w == 1 ? w2 : n_process);
  a.work_counter = ctl + window_work_int(w);
  a.queue = a0.queue + lo;
  a.queue_tail = ctl + window_tail_int(w);
  a.n_process = hi - lo;
  return a;
}

// Launch shape of engine e's search at cluster width C: the configuration,
// the staging of the correlate region, tensor maps, dynamic shared memory and
// how many clusters fit at once.
struct SearchShape {
  int C = 0, cap = 0, max_clusters = 0;
  int minb = 1;  // CTAs per SM the kernel's registers are sized for
  SearchCfg k{};
  size_t stage_bytes = 0, smem = 0;
  CUtensorMap tmap, tmap_ref;
};

// With `grow`, C doubles (up to 8) while the per-CTA state does not fit or the
// correlate region cannot be staged; without it the shape is C's or none
// (DVC_E_ARG, no message).
int search_shape(dvc_engine *e, int C, bool grow, int seed_mode, size_t budget, bool tma_ok, cudaStream_t st,
                 SearchShape &s) {
  for (;;) {
    s.cap = fill_config(e, C, s.k);
    s.stage_bytes = tma_ok ? stage_config(e, C, budget, state_bytes(s.cap), seed_mode != DVC_SEED_PARAMS, s.k) : 0;
    const size_t need = s.stage_bytes + state_bytes(s.cap);
    const bool short_of = (tma_ok && !s.stage_bytes) || need > budget;
    if (short_of && grow && C < 8) {
      C *= 2;
      continue;
    }
    if (need > budget) return grow ? set_error(DVC_E_ARG, "subvolume too large for the search kernel") : DVC_E_ARG;
    if (short_of && !grow) return DVC_E_ARG;
    break;
  }
  memset(&s.tmap, 0, sizeof s.tmap);
  memset(&s.tmap_ref, 0, sizeof s.tmap_ref);
  if (s.stage_bytes && !(encode_stage_map(e, s.k.stage, e->cor, &s.tmap) &&
                         encode_stage_map(e, s.k.stage_ref, e->ref, &s.tmap_ref))) {
    if (!grow) return DVC_E_ARG;
    s.k = SearchCfg{};
    s.cap = fill_config(e, C, s.k);
    s.stage_bytes = 0;
  }
  s.C = C;
  s.smem = s.stage_bytes + state_bytes(s.cap);
  SearchArgs probe{};
  const int rc = dispatch_launch(e->p.bytes_per_voxel, e->p.interp_type, probe, s.tmap, s.tmap_ref, s.smem, 0, C,
                                 st, &s.max_clusters);
  if (rc) return rc;
  if (s.max_clusters < 1) return grow ? set_error(DVC_E_ARG, "search kernel cluster does not fit") : DVC_E_ARG;
  return DVC_OK;
}

// The shape with two CTAs resident per SM at width C, for searches without a
// coarse grid (start parameters given): the correlate region is read through
// L1 (no staging box), and the kernel's registers are sized for two CTAs, so
// one point's serial sections (reductions, the one-warp solve) overlap the
// other's sample evaluations. DVC_E_ARG (no message) when fewer than about
// two CTAs per SM fit.
int search_shape_pair(dvc_engine *e, int C, cudaStream_t st, SearchShape &s) {
  if (e->p.interp_type != DVC_TRICUBIC) return DVC_E_ARG;
  s.cap = fill_config(e, C, s.k);
  s.stage_bytes = 0;
  memset(&s.tmap, 0, sizeof s.tmap);
  memset(&s.tmap_ref, 0, sizeof s.tmap_ref);
  s.C = C;
  s.minb = 2;
  s.smem = state_bytes(s.cap);
  SearchArgs probe{};
  const int rc = dispatch_launch(e->p.bytes_per_voxel, e->p.interp_type, probe, s.tmap, s.tmap_ref, s.smem, 0, C,
                                 st, &s.max_clusters, 2);
  if (rc) return rc;
  if ((long long)s.max_clusters * C < 3LL * e->num_sms / 2) return DVC_E_ARG;
  return DVC_OK;
}

}  // namespace

// ================================================================== C API ===
extern "C" {

const char *dvc_gpu_version(void) { return "dvc-gb300 0.1 (sm_103a)"; }
const char *dvc_gpu_last_error(void) { return g_last_error.c_str(); }
int dvc_gpu_abi_version(void) { return DVC_ABI_VERSION; }

// Reads one byte of every page of a host buffer, on up to 8 threads for
// large buffers, right before the buffer is copied to the device. Measured on
// the Grace host of a GB300 (64 KiB pages): a 4 GiB upload from pinned memory
// took 20 ms when the same pages had just been copied or read by the CPU,
// but 272 ms after the process sat idle for a second and 458 ms after a
// second of GPU work; reading every page first (1.8 ms) brought it back to
// 20 ms. The pages' access state ages while untouched, and the CPU restores
// it far faster than the device's copies do page by page.
static void touch_pages(const void *buf, size_t bytes) {
  if (!buf || !bytes) return;
  const long ps = sysconf(_SC_PAGESIZE);
  const size_t step = ps > 0 ? (size_t)ps : 4096;
  const volatile unsigned char *b = static_cast<const volatile unsigned char *>(buf);
  auto run = [&](size_t lo, size_t hi) {
    unsigned acc = 0;
    for (size_t o = lo; o < hi; o += step) acc += b[o];
    if (acc == 0xFFFFFFFFu) fputc(0, stderr);  // keeps the reads
  };
  const size_t pages = (bytes + step - 1) / step;
  const int nt = bytes >= ((size_t)256 << 20) ? 8 : 1;
  if (nt == 1) {
    run(0, bytes);
    return;
  }
  // (no exception may leave a C entry point: pieces whose thread cannot be
  // started are read by the calling thread)
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++) {
    const size_t lo = pages * t / nt * step, hi = std::min(bytes, pages * (t + 1) / nt * step);
    try {
      th.emplace_back(run, lo, hi);
    } catch (...) {
      run(lo, hi);
    }
  }
  for (auto &x : th) x.join();
}

int dvc_gpu_create(dvc_engine **out, const dvc_params *p, const void *ref_vox, const void *cor_vox,
                   int big_endian) try {
  if (!out || !ref_vox || !cor_vox) return set_error(DVC_E_ARG, "null argument");
  *out = nullptr;
  int rc = validate(p);
  if (rc) return rc;
  dvc_engine *e = new dvc_engine();
  e->p = *p;
  const size_t nvox = (size_t)p->vol_wide * p->vol_high * p->vol_tall;
  const size_t bytes = nvox * p->bytes_per_voxel;
  const size_t alloc = bytes + 64;  // tail padding for aligned row over-reads
  const bool verbose = getenv("DVC_VERBOSE") != nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  if (cudaMalloc(&e->ref, alloc) != cudaSuccess || cudaMalloc(&e->cor, alloc) != cudaSuccess) {
    dvc_gpu_destroy(e);
    return set_error(DVC_E_NOMEM, "volume allocation failed");
  }
  e->owns_volumes = true;
  const auto t1 = std::chrono::steady_clock::now();
  touch_pages(ref_vox, bytes);
  touch_pages(cor_vox, bytes);
  if (cudaMemcpy(e->ref, ref_vox, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->cor, cor_vox, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset((char *)e->ref + bytes, 0, 64) != cudaSuccess ||
      cudaMemset((char *)e->cor + bytes, 0, 64) != cudaSuccess) {
    dvc_gpu_destroy(e);
    return set_error(DVC_E_CUDA, "volume upload failed");
  }
  if (verbose) {
    const auto t2 = std::chrono::steady_clock::now();
    cudaPointerAttributes pa{};
    const bool pinned = cudaPointerGetAttributes(&pa, ref_vox) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    using ms = std::chrono::duration<double, std::milli>;
    fprintf(stderr, "dvc create: allocation %.1f ms, upload of %zu bytes %.1f ms (host buffer %s)\n",
            ms(t1 - t0).count(), 2 * bytes, ms(t2 - t1).count(), pinned ? "pinned" : "pageable");
  }
  if (p->bytes_per_voxel == 2 && big_endian) {
    const int T = 256;
    const unsigned G = (unsigned)((nvox + T - 1) / T);
    byteswap16_kernel<<<G, T>>>((uint16_t *)e->ref, nvox);
    byteswap16_kernel<<<G, T>>>((uint16_t *)e->cor, nvox);
    if (cudaGetLastError() != cudaSuccess) {
      dvc_gpu_destroy(e);
      return set_error(DVC_E_CUDA, "byte swap failed");
    }
  }
  rc = engine_finish(e);
  if (rc) {
    dvc_gpu_destroy(e);
    return rc;
  }
  *out = e;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_create_from_files(dvc_engine **out, const dvc_params *p, const char *ref_path,
                              const char *cor_path, long long header_bytes, int big_endian) try {
  if (!out || !ref_path || !cor_path) return set_error(DVC_E_ARG, "null argument");
  *out = nullptr;
  int rc = validate(p);
  if (rc) return rc;
  dvc_engine *e = new dvc_engine();
  e->p = *p;
  const size_t bytes = (size_t)p->vol_wide * p->vol_high * p->vol_tall * p->bytes_per_voxel;
  if (cudaMalloc(&e->ref, bytes + 64) != cudaSuccess || cudaMalloc(&e->cor, bytes + 64) != cudaSuccess) {
    dvc_gpu_destroy(e);
    return set_error(DVC_E_NOMEM, "volume allocation failed");
  }
  e->owns_volumes = true;
  if (cudaMemset((char *)e->ref + bytes, 0, 64) != cudaSuccess ||
      cudaMemset((char *)e->cor + bytes, 0, 64) != cudaSuccess) {
    dvc_gpu_destroy(e);
    return set_error(DVC_E_CUDA, "volume padding");
  }
  rc = dvc_gpu_load_raw(e->ref, ref_path, header_bytes, p->vol_wide, p->vol_high, p->vol_tall,
                        p->bytes_per_voxel, big_endian, nullptr);
  if (!rc)
    rc = dvc_gpu_load_raw(e->cor, cor_path, header_bytes, p->vol_wide, p->vol_high, p->vol_tall,
                          p->bytes_per_voxel, big_endian, nullptr);
  if (!rc) rc = engine_finish(e);
  if (rc) {
    dvc_gpu_destroy(e);
    return rc;
  }
  *out = e;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_create_device(dvc_engine **out, const dvc_params *p, const void *ref_vox_dev,
                          const void *cor_vox_dev) try {
  if (!out || !ref_vox_dev || !cor_vox_dev) return set_error(DVC_E_ARG, "null argument");
  *out = nullptr;
  int rc = validate(p);
  if (rc) return rc;
  dvc_engine *e = new dvc_engine();
  e->p = *p;
  e->ref = const_cast<void *>(ref_vox_dev);
  e->cor = const_cast<void *>(cor_vox_dev);
  e->owns_volumes = false;
  rc = engine_finish(e);
  if (rc) {
    dvc_gpu_destroy(e);
    return rc;
  }
  *out = e;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

void dvc_gpu_destroy(dvc_engine *e) try {
  if (!e) return;
  if (e->owns_volumes) {
    if (e->ref) cudaFree(e->ref);
    if (e->cor) cudaFree(e->cor);
  }
  if (e->d_off_i) cudaFree(e->d_off_i);
  if (e->d_off_f) cudaFree(e->d_off_f);
  if (e->d_rand_off) cudaFree(e->d_rand_off);
  if (e->ws) cudaFree(e->ws);
  delete e;
} catch (...) {
  dvc_internal_host_exception();
}

// The search launch with one configuration (the engine's). Scratch (done
// flags, ranks, work counter, counters) is the engine's grow-only workspace,
// or `ws_fixed` (ws_fixed_bytes long) when the caller supplies it.
static int process_device_ws(dvc_engine *e, int n_points, const double *points_dev, int n_process,
                             const int *order_dev, int n_neigh, const int *neigh_dev, int seed_mode,
                             const double *seeds_dev, int *status_dev, double *objmin_dev,
                             double *params_dev, int *gn_iters_dev, void *stream, char *ws_fixed,
                             size_t ws_fixed_bytes = 0) {
  const RunIO io{n_points, points_dev, n_process, order_dev, n_neigh, neigh_dev, seed_mode,
                 seeds_dev, status_dev, objmin_dev, params_dev, gn_iters_dev};
  int rc = check_run(e, io);
  if (rc) return rc;
  if (n_points == 0) return DVC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const dvc_params &p = e->p;

  // launch shape: one cluster of C CTAs per point in flight, persistent grid
  // of as many clusters as fit. About 512 samples per CTA or more with the
  // reference's seeding (its points wait on neighbours, which favours shorter
  // per-point latency), 1024 for independent points; clusters of 8 place
  // only 120 CTAs on the 152 SMs, clusters of 4 place 144. Each CTA stages
  // the correlate region of its samples in shared memory (TMA) when the
  // volume's layout allows it and a box fits: one covering every grid
  // translation, else one per z slab of translations, else a wider cluster.
  size_t budget = 0;
  rc = dyn_budget(&budget);
  if (rc) return rc;
  const bool tma_ok = tma_layout(e);
  int C = e->cluster;
  if (C <= 0) {
    const int per = (seed_mode == DVC_SEED_NEIGHBOURS) ? 512 : 1024;
    C = 1;
    while (C < 8 && e->n_sub / (2 * C) >= per) C *= 2;
    // a call of a few points (the learned search's fallback) leaves most
    // SMs idle: wider clusters, as long as they take at most an eighth of
    // the SMs, cut its latency
    while (C < 8 && n_process > 0 && (long long)n_process * 2 * C * 8 <= e->num_sms) C *= 2;
  }
  SearchShape base;
  rc = search_shape(e, C, true, seed_mode, budget, tma_ok, st, base);
  if (rc) return rc;

  // With the reference's seeding the points form a dependency graph that
  // grows from the starting point: at first, and again at the end of the
  // processing order, fewer points are ready than clusters wait for them, and
  // the run follows a chain of points one after another. There clusters of
  // twice the width search a point in about 0.54 of the time (measured with
  // 4 and 8 CTAs on 4000 samples). So with the launch shape chosen here the
  // ranks are cut into three windows searched by consecutive launches: the
  // first K1 points at twice the width, the body at this width, the last R
  // at twice the width, K1 = 84 and R = 28 points per resident cluster of
  // the body's shape (a model of the scheduling over the graph of 60,800
  // grid points and their 75 neighbours puts the best cuts there: 10%
  // shorter than one launch). Each point's width is a function of its rank,
  // so results do not depend on timing. DVC_WINDOWS=K1,R sets the cuts
  // (0,0: one launch).
  int w1 = n_process, w2 = n_process;
  SearchShape wide;
  const bool dataflow = uses_dataflow(io, ws_fixed);
  if (dataflow && e->cluster <= 0 && (base.C == 2 || base.C == 4)) {
    long long K1 = 84LL * base.max_clusters, R = 28LL * base.max_clusters;
    bool forced = false;
    if (const char *v = getenv("DVC_WINDOWS")) {
      long long a1 = 0, a2 = 0;
      if (sscanf(v, "%lld,%lld", &a1, &a2) == 2 && a1 >= 0 && a2 >= 0) {
        K1 = a1;
        R = a2;
        forced = true;
      }
    }
    if ((K1 > 0 || R > 0) && (forced || n_process > K1 + R) &&
        search_shape(e, 2 * base.C, false, seed_mode, budget, tma_ok, st, wide) == DVC_OK) {
      w1 = (int)std::min<long long>(K1, n_process);
      w2 = (int)std::max<long long>(w1, n_process - R);
    }
  }

  // Independent points without a coarse grid (start parameters given, or
  // no basin) and Gauss-Newton: two CTAs per SM, at the narrowest cluster
  // width whose state fits two (no cluster at all when one CTA holds the
  // subvolume), the correlate region read through L1. The learned search of
  // 499,200 points (cube 41, 3375 samples, 12 dof, uint16): 1.46 s at width 2 with one
  // staged CTA per SM, 1.30 s with two per SM, 1.13 s with two per SM at
  // width 1. Other widths sum in another order and the kernel compiled for
  // two CTAs may fuse multiplies and adds differently, so results can differ
  // in the last FP32 bits. DVC_PAIR=0: one CTA per SM with staging; 1, 2, 4:
  // that width.
  SearchShape pair;
  bool use_pair = false;
  const bool no_grid = seed_mode == DVC_SEED_PARAMS || (seed_mode != DVC_SEED_NEIGHBOURS && p.basin_radius == 0.0);
  if (no_grid && p.refine_method == DVC_REFINE_GAUSS_NEWTON && e->cluster <= 0) {
    const char *v = getenv("DVC_PAIR");
    const int pc = v ? atoi(v) : -1;
    if (pc == 1 || pc == 2 || pc == 4 || pc == 8)
      use_pair = search_shape_pair(e, pc, st, pair) == DVC_OK;
    else if (pc != 0)
      for (int c = 1; c <= base.C && !use_pair; c *= 2) use_pair = search_shape_pair(e, c, st, pair) == DVC_OK;
  }

  SearchArgs a{};
  rc = prepare_run(e, io, st, ws_fixed, ws_fixed_bytes, a, w1, w2);
  if (rc) return rc;
  if (n_process == 0) return DVC_OK;
  a.n_cfg = 1;
  const int n_win = (w1 < n_process || w2 < n_process) ? 3 : 1;
  for (int w = 0; w < n_win; w++) {
    const SearchShape &sh = use_pair ? pair : ((n_win == 3 && w != 1) ? wide : base);
    SearchArgs aw = n_win == 3 ? window_args(a, w, w1, w2, n_process) : a;
    if (aw.n_process == 0) continue;
    aw.cfg0 = sh.k;
    aw.local_cap = sh.cap;
    aw.stage_bytes = (int)sh.stage_bytes;
    const int grid = sh.C * std::max(1, std::min(sh.max_clusters, aw.n_process));
    if (getenv("DVC_VERBOSE"))
      fprintf(stderr, "dvc search: %d points (window %d of %d), cluster %d, grid %d CTAs, staged %d "
              "(box %d x %d x %d), dynamic smem %zu of %zu, samples/CTA <= %d, grid step %s\n", aw.n_process, w,
              n_win, sh.C, grid, sh.k.stage_on ? (sh.k.stage_slab ? 2 : 1) : 0, sh.k.stage[0], sh.k.stage[1],
              sh.k.stage[2], sh.smem, budget, sh.cap,
              sh.k.inc_int ? "integral" : (sh.k.do_grid ? "general" : "none"));
    rc = dispatch_launch(p.bytes_per_voxel, p.interp_type, aw, sh.tmap, sh.tmap_ref, sh.smem, grid, sh.C, st, nullptr,
                         sh.minb);
    if (rc) return rc;
  }
  const SearchShape &body = use_pair ? pair : base;
  const int grid = body.C * std::max(1, std::min(body.max_clusters, n_process));
  e->last_cluster = body.C;
  e->last_grid = grid;
  e->last_staged = body.k.stage_on ? (body.k.stage_slab ? 2 : 1) : 0;
  e->last_smem = (int)body.smem;
  e->last_windows[0] = w1;
  e->last_windows[1] = w2;
  e->last_windows[2] = n_win == 3 ? wide.C : body.C;
  return DVC_OK;
}


int dvc_gpu_process_device(dvc_engine *e, int n_points, const double *points_dev, int n_process,
                           const int *order_dev, int n_neigh, const int *neigh_dev, int seed_mode,
                           const double *seeds_dev, int *status_dev, double *objmin_dev,
                           double *params_dev, int *gn_iters_dev, void *stream) try {
  return process_device_ws(e, n_points, points_dev, n_process, order_dev, n_neigh, neigh_dev,
                           seed_mode, seeds_dev, status_dev, objmin_dev, params_dev, gn_iters_dev,
                           stream, nullptr);
} catch (...) {
  return dvc_internal_host_exception();
}

// ---- allocation-free search -------------------------------------------------
// Some callers cannot allocate device memory at the moment they search: a host
// program that owns the device memory budget through its own pool, or one
// that records its work while device allocation is off limits. For them the
// search's scratch (per-point done flags and ranks, the work counter, the
// evaluation counters) lives in this fixed module array instead of the
// engine's workspace. It holds DVC_NOALLOC_MAX_POINTS points, belongs to every
// GPU that loads the library until the process exits, and is shared by all
// calls: each call clears the parts that must start at zero, and calls whose
// work overlaps on the GPU race on it. Layout (in-order scheduling, no
// dataflow tables): the control block, then done[n] and rank[n], the block
// after them rounded up to 256 bytes.
constexpr size_t kNoallocBytes = kCtlBytes + (size_t)DVC_NOALLOC_MAX_POINTS * 8 + 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (the host symbol is only a stand-in, never a device address).
// Host threads making a first call on the same device may both look it up;
// they store the same address.
static int noalloc_scratch(char **out) {
  static std::atomic<void *> addr[64];
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return set_error(DVC_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(err));
  if (dev < 0 || dev >= 64) return set_error(DVC_E_ARG, "device index above 63");
  void *p = addr[dev].load(std::memory_order_acquire);
  if (!p) {
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess || !p)
      return set_error(DVC_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(err));
    addr[dev].store(p, std::memory_order_release);
  }
  *out = (char *)p;
  return DVC_OK;
}

int dvc_gpu_process_device_noalloc(dvc_engine *e, int n_points, const double *points_dev,
                                   int n_process, const int *order_dev, int n_neigh,
                                   const int *neigh_dev, int seed_mode, const double *seeds_dev,
                                   int *status_dev, double *objmin_dev, double *params_dev,
                                   int *gn_iters_dev, void *stream) try {
  if (n_points > DVC_NOALLOC_MAX_POINTS)
    return set_error(DVC_E_ARG, "dvc_gpu_process_device_noalloc: n_points exceeds "
                                "DVC_NOALLOC_MAX_POINTS (" + std::to_string(DVC_NOALLOC_MAX_POINTS) +
                                    "); use dvc_gpu_process_device");
  char *ws = nullptr;
  const int rc = noalloc_scratch(&ws);
  if (rc) return rc;
  return process_device_ws(e, n_points, points_dev, n_process, order_dev, n_neigh, neigh_dev,
                           seed_mode, seeds_dev, status_dev, objmin_dev, params_dev, gn_iters_dev,
                           stream, ws, kNoallocBytes);
} catch (...) {
  return dvc_internal_host_exception();
}

// The error flag of engine e's last search launch, which has finished:
// DVC_OK, or the DVC_E_* code the launch recorded (with its message).
static int launch_error(dvc_engine *e) {
  if (!e->last_ctl) return DVC_OK;
  int ctl[2] = {0, 0};
  CUDA_TRY(cudaMemcpy(ctl, e->last_ctl, sizeof ctl, cudaMemcpyDeviceToHost));
  if (ctl[1] == DVC_E_TIMEOUT)
    return set_error(DVC_E_TIMEOUT, "a bounded device-side wait gave up; points were left unsearched "
                                     "(status DVC_NOT_SEARCH) or evaluated without staging");
  if (ctl[1] != 0) return set_error(ctl[1], "a point named no configuration of the plan; it was left unsearched");
  return DVC_OK;
}

// Host-array search: arguments checked, arrays copied in, the engine's (or
// the plan's) device search, results and counters copied out.
static int host_process(dvc_engine *e, dvc_plan *plan, const int *point_cfg, int n_points,
                        const double *points, int n_process, const int *order, int n_neigh,
                        const int *neigh, int seed_mode, const double *seeds, int *status,
                        double *objmin, double *params, int *gn_iters, dvc_stats *stats) {
  if (!e || !points || !status || !objmin || !params) return set_error(DVC_E_ARG, "null argument");
  if (n_points < 0 || n_process < 0 || n_process > n_points)
    return set_error(DVC_E_ARG, "n_process must be in 0..n_points");
  if (plan) {
    if (!point_cfg) return set_error(DVC_E_ARG, "point_cfg required");
    const int nc = (int)plan->cfgs.size();
    for (int i = 0; i < n_points; i++)
      if (point_cfg[i] < 0 || point_cfg[i] >= nc) return set_error(DVC_E_ARG, "configuration index out of range");
  }
  if (n_process > 0 && !order) return set_error(DVC_E_ARG, "order required");
  if (seed_mode == DVC_SEED_NEIGHBOURS && n_neigh > 0 && !neigh)
    return set_error(DVC_E_ARG, "neighbour list required");
  if ((seed_mode == DVC_SEED_GIVEN || seed_mode == DVC_SEED_PARAMS) && !seeds)
    return set_error(DVC_E_ARG, "seeds required");
  for (int i = 0; i < n_process; i++)
    if (order[i] < 0 || order[i] >= n_points) return set_error(DVC_E_ARG, "order index out of range");
  if (seed_mode == DVC_SEED_NEIGHBOURS && neigh)
    for (size_t i = 0; i < (size_t)n_points * n_neigh; i++)
      if (neigh[i] < 0 || neigh[i] >= n_points) return set_error(DVC_E_ARG, "neighbour index out of range");
  auto t0 = std::chrono::steady_clock::now();
  const size_t N = (size_t)n_points;
  double *d_pts = nullptr, *d_seeds = nullptr, *d_obj = nullptr, *d_par = nullptr;
  int *d_order = nullptr, *d_neigh = nullptr, *d_status = nullptr, *d_its = nullptr, *d_cfg = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int rc = DVC_OK;
  auto cleanup = [&]() {
    cudaFree(d_pts); cudaFree(d_seeds); cudaFree(d_obj); cudaFree(d_par);
    cudaFree(d_order); cudaFree(d_neigh); cudaFree(d_status); cudaFree(d_its); cudaFree(d_cfg);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  };
#define TRYC(x)                                                                          \
  do {                                                                                   \
    cudaError_t _e = (x);                                                                \
    if (_e != cudaSuccess) {                                                             \
      cleanup();                                                                         \
      return set_error(DVC_E_CUDA, std::string(#x) + ": " + cudaGetErrorString(_e));     \
    }                                                                                    \
  } while (0)
  TRYC(cudaMalloc(&d_pts, N * 3 * sizeof(double)));
  TRYC(cudaMalloc(&d_order, std::max<size_t>(1, n_process) * sizeof(int)));
  TRYC(cudaMalloc(&d_status, N * sizeof(int)));
  TRYC(cudaMalloc(&d_obj, N * sizeof(double)));
  TRYC(cudaMalloc(&d_par, N * 12 * sizeof(double)));
  TRYC(cudaMalloc(&d_its, N * sizeof(int)));
  TRYC(cudaMemcpy(d_pts, points, N * 3 * sizeof(double), cudaMemcpyHostToDevice));
  if (n_process) TRYC(cudaMemcpy(d_order, order, n_process * sizeof(int), cudaMemcpyHostToDevice));
  if (seed_mode == DVC_SEED_NEIGHBOURS && n_neigh > 0) {
    TRYC(cudaMalloc(&d_neigh, N * n_neigh * sizeof(int)));
    TRYC(cudaMemcpy(d_neigh, neigh, N * n_neigh * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (seed_mode == DVC_SEED_GIVEN || seed_mode == DVC_SEED_PARAMS) {
    const size_t per = seed_mode == DVC_SEED_GIVEN ? 3 : 12;
    TRYC(cudaMalloc(&d_seeds, N * per * sizeof(double)));
    TRYC(cudaMemcpy(d_seeds, seeds, N * per * sizeof(double), cudaMemcpyHostToDevice));
  }
  if (plan) {
    TRYC(cudaMalloc(&d_cfg, std::max<size_t>(1, N) * sizeof(int)));
    TRYC(cudaMemcpy(d_cfg, point_cfg, N * sizeof(int), cudaMemcpyHostToDevice));
  }
  TRYC(cudaEventCreate(&ev0));
  TRYC(cudaEventCreate(&ev1));
  TRYC(cudaEventRecord(ev0, 0));
  rc = plan ? dvc_gpu_plan_process_device(plan, d_cfg, n_points, d_pts, n_process, d_order, n_neigh, d_neigh,
                                          seed_mode, d_seeds, d_status, d_obj, d_par, d_its, nullptr)
            : dvc_gpu_process_device(e, n_points, d_pts, n_process, d_order, n_neigh, d_neigh, seed_mode,
                                     d_seeds, d_status, d_obj, d_par, d_its, nullptr);
  if (rc) {
    cleanup();
    return rc;
  }
  TRYC(cudaEventRecord(ev1, 0));
  TRYC(cudaEventSynchronize(ev1));
  TRYC(cudaGetLastError());
  unsigned long long counters[3] = {0, 0, 0};
  if (n_process > 0 && e->last_ctl)
    TRYC(cudaMemcpy(counters, e->last_ctl + kCountersOff, sizeof counters, cudaMemcpyDeviceToHost));
  TRYC(cudaMemcpy(status, d_status, N * sizeof(int), cudaMemcpyDeviceToHost));
  TRYC(cudaMemcpy(objmin, d_obj, N * sizeof(double), cudaMemcpyDeviceToHost));
  TRYC(cudaMemcpy(params, d_par, N * 12 * sizeof(double), cudaMemcpyDeviceToHost));
  if (gn_iters) TRYC(cudaMemcpy(gn_iters, d_its, N * sizeof(int), cudaMemcpyDeviceToHost));
  float kms = 0.f;
  cudaEventElapsedTime(&kms, ev0, ev1);
  cleanup();
#undef TRYC
  if (n_process > 0) {
    rc = launch_error(e);
    if (rc) return rc;
  }
  if (stats) {
    memset(stats, 0, sizeof *stats);
    stats->n_processed = n_process;
    for (int i = 0; i < n_points; i++) {
      if (status[i] == DVC_POINT_GOOD) stats->n_good++;
      if (status[i] == DVC_RANGE_FAIL) stats->n_range_fail++;
      if (status[i] == DVC_CONVG_FAIL) stats->n_convg_fail++;
    }
    stats->n_evaluations = (long long)counters[0];
    stats->n_gn_iterations = (long long)counters[1];
    stats->kernel_ms = kms;
    stats->total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return DVC_OK;
}

int dvc_gpu_process(dvc_engine *e, int n_points, const double *points, int n_process,
                    const int *order, int n_neigh, const int *neigh, int seed_mode,
                    const double *seeds, int *status, double *objmin, double *params, int *gn_iters,
                    dvc_stats *stats) try {
  return host_process(e, nullptr, nullptr, n_points, points, n_process, order, n_neigh, neigh, seed_mode,
                      seeds, status, objmin, params, gn_iters, stats);
} catch (...) {
  return dvc_internal_host_exception();
}

// ---- several configurations in one launch ------------------------------------
// Lay out plan `pl` at cluster width C: per configuration its rank ranges and
// offset extrema, then, with staging, its box when it fits beside the largest
// per-CTA sample state. The configuration table and tensor maps are uploaded
// only once the shape is known to fit, so a failed call leaves the plan as it
// was.
static int plan_build(dvc_plan *pl, int C, int staging) {
  if (C != 1 && C != 2 && C != 4 && C != 8) return set_error(DVC_E_ARG, "cluster width must be 1, 2, 4 or 8");
  size_t budget = 0;
  int rc = dyn_budget(&budget);
  if (rc) return rc;
  const int n = (int)pl->cfgs.size();
  std::vector<SearchCfg> ks((size_t)n);
  int cap = 0;
  for (int i = 0; i < n; i++) cap = std::max(cap, fill_config(pl->cfgs[i], C, ks[i]));
  if (state_bytes(cap) > budget)
    return set_error(DVC_E_ARG, "the largest subvolume does not fit the search kernel at cluster width " +
                                    std::to_string(C));
  const bool tma_ok = staging && tma_layout(pl->cfgs[0]);
  std::vector<CUtensorMap> maps((size_t)n * 2);  // per configuration: correlate, reference
  size_t sb = 0;
  int n_staged = 0;
  for (int i = 0; i < n; i++) {
    memset(&maps[(size_t)i * 2], 0, 2 * sizeof(CUtensorMap));
    if (!tma_ok) continue;
    const size_t b = stage_config(pl->cfgs[i], C, budget, state_bytes(cap), true, ks[(size_t)i]);
    if (b && encode_stage_map(pl->cfgs[i], ks[(size_t)i].stage, pl->cfgs[i]->cor, &maps[(size_t)i * 2]) &&
        encode_stage_map(pl->cfgs[i], ks[(size_t)i].stage_ref, pl->cfgs[i]->ref, &maps[(size_t)i * 2 + 1])) {
      sb = std::max(sb, b);
      n_staged++;
    } else {
      ks[(size_t)i].stage_on = 0;
      for (int d = 0; d < 3; d++) ks[(size_t)i].stage[d] = 0;
      ks[(size_t)i].stage_tx = 0;
    }
  }
  const size_t smem = sb + state_bytes(cap);
  const dvc_params &p = pl->cfgs[0]->p;
  int mc = 0;
  SearchArgs probe{};
  CUtensorMap tm0;
  memset(&tm0, 0, sizeof tm0);
  rc = dispatch_launch(p.bytes_per_voxel, p.interp_type, probe, tm0, tm0, smem, 0, C, 0, &mc);
  if (rc) return rc;
  if (mc < 1) return set_error(DVC_E_ARG, "search kernel cluster does not fit");
  if (!pl->d_cfgs) {
    CUDA_TRY(cudaMalloc(&pl->d_cfgs, (size_t)n * sizeof(SearchCfg)));
    CUDA_TRY(cudaMalloc(&pl->d_tmaps, (size_t)n * 2 * sizeof(CUtensorMap)));
  }
  for (int i = 0; i < n; i++) {
    ks[(size_t)i].tmap = ks[(size_t)i].stage_on ? pl->d_tmaps + 2 * i : nullptr;
    ks[(size_t)i].tmap_ref = ks[(size_t)i].stage_on ? pl->d_tmaps + 2 * i + 1 : nullptr;
  }
  CUDA_TRY(cudaDeviceSynchronize());  // no launch still reads the old table
  CUDA_TRY(cudaMemcpy(pl->d_tmaps, maps.data(), (size_t)n * 2 * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(pl->d_cfgs, ks.data(), (size_t)n * sizeof(SearchCfg), cudaMemcpyHostToDevice));
  pl->h_cfgs = ks;
  pl->cluster = C;
  pl->staging = staging;
  pl->n_staged = n_staged;
  pl->cap = cap;
  pl->stage_bytes = sb;
  pl->smem_dyn = smem;
  pl->max_clusters = mc;
  return DVC_OK;
}

int dvc_gpu_plan_create(dvc_plan **out, dvc_engine *const *configs, int n_configs, int cluster) try {
  if (!out || !configs) return set_error(DVC_E_ARG, "null argument");
  *out = nullptr;
  if (n_configs < 1) return set_error(DVC_E_ARG, "a plan needs at least one configuration");
  const dvc_engine *e0 = configs[0];
  for (int i = 0; i < n_configs; i++) {
    const dvc_engine *e = configs[i];
    if (!e) return set_error(DVC_E_ARG, "null configuration");
    if (e->ref != e0->ref || e->cor != e0->cor || e->p.vol_wide != e0->p.vol_wide ||
        e->p.vol_high != e0->p.vol_high || e->p.vol_tall != e0->p.vol_tall ||
        e->p.bytes_per_voxel != e0->p.bytes_per_voxel || e->p.interp_type != e0->p.interp_type)
      return set_error(DVC_E_ARG, "the configurations of a plan must share volumes, voxel type and interpolation");
  }
  if (cluster != 0 && cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8)
    return set_error(DVC_E_ARG, "cluster must be 0, 1, 2, 4 or 8");
  dvc_plan *pl = new dvc_plan();
  pl->cfgs.assign(configs, configs + n_configs);
  int rc = DVC_OK;
  if (cluster > 0) {
    rc = plan_build(pl, cluster, 1);
  } else {
    // from the largest sample count (about 512 samples per CTA and up), then
    // wider while the largest subvolume does not fit
    int nmax = 0;
    for (const dvc_engine *e : pl->cfgs) nmax = std::max(nmax, e->n_sub);
    int C = 1;
    while (C < 8 && nmax / (2 * C) >= 512) C *= 2;
    for (;; C *= 2) {
      rc = plan_build(pl, C, 1);
      if (rc == DVC_OK || C == 8) break;
    }
  }
  if (rc) {
    dvc_gpu_plan_destroy(pl);
    return rc;
  }
  *out = pl;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

void dvc_gpu_plan_destroy(dvc_plan *plan) try {
  if (!plan) return;
  if (plan->d_cfgs) cudaFree(plan->d_cfgs);
  if (plan->d_tmaps) cudaFree(plan->d_tmaps);
  delete plan;
} catch (...) {
  dvc_internal_host_exception();
}

int dvc_gpu_plan_info(const dvc_plan *plan, int *cluster, int *staging, int *n_staged, long long *smem_bytes) try {
  if (!plan) return set_error(DVC_E_ARG, "null plan");
  if (cluster) *cluster = plan->cluster;
  if (staging) *staging = plan->staging;
  if (n_staged) *n_staged = plan->n_staged;
  if (smem_bytes) *smem_bytes = (long long)plan->smem_dyn;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_plan_set_shape(dvc_plan *plan, int cluster, int staging) try {
  if (!plan) return set_error(DVC_E_ARG, "null plan");
  return plan_build(plan, cluster, staging ? 1 : 0);
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_plan_process_device(dvc_plan *plan, const int *point_cfg_dev, int n_points,
                                const double *points_dev, int n_process, const int *order_dev,
                                int n_neigh, const int *neigh_dev, int seed_mode,
                                const double *seeds_dev, int *status_dev, double *objmin_dev,
                                double *params_dev, int *gn_iters_dev, void *stream) try {
  if (!plan) return set_error(DVC_E_ARG, "null plan");
  dvc_engine *e = plan->cfgs[0];
  const RunIO io{n_points, points_dev, n_process, order_dev, n_neigh, neigh_dev, seed_mode,
                 seeds_dev, status_dev, objmin_dev, params_dev, gn_iters_dev};
  int rc = check_run(e, io);
  if (rc) return rc;
  if (n_process > 0 && !point_cfg_dev) return set_error(DVC_E_ARG, "point_cfg required");
  if (n_points == 0) return DVC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  SearchArgs a{};
  rc = prepare_run(e, io, st, nullptr, 0, a, n_process, n_process);
  if (rc) return rc;
  if (n_process == 0) return DVC_OK;
  const int n = (int)plan->cfgs.size();
  if (n == 1) {
    a.cfg0 = plan->h_cfgs[0];
    a.n_cfg = 1;
  } else {
    a.cfgs = plan->d_cfgs;
    a.point_cfg = point_cfg_dev;
    a.n_cfg = n;
  }
  a.local_cap = plan->cap;
  a.stage_bytes = (int)plan->stage_bytes;
  const int C = plan->cluster;
  const int grid = C * std::max(1, std::min(plan->max_clusters, n_process));
  if (getenv("DVC_VERBOSE"))
    fprintf(stderr, "dvc plan search: %d points, %d configurations (%d staged), cluster %d, grid %d CTAs, "
            "dynamic smem %zu, samples/CTA <= %d\n", n_process, n, plan->n_staged, C, grid, plan->smem_dyn,
            plan->cap);
  e->last_cluster = C;
  e->last_grid = grid;
  e->last_staged = plan->n_staged > 0;
  e->last_smem = (int)plan->smem_dyn;
  CUtensorMap tm0;
  memset(&tm0, 0, sizeof tm0);
  return dispatch_launch(e->p.bytes_per_voxel, e->p.interp_type, a, tm0, tm0, plan->smem_dyn, grid, C, st, nullptr);
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_plan_process(dvc_plan *plan, const int *point_cfg, int n_points, const double *points,
                         int n_process, const int *order, int n_neigh, const int *neigh,
                         int seed_mode, const double *seeds, int *status, double *objmin,
                         double *params, int *gn_iters, dvc_stats *stats) try {
  if (!plan) return set_error(DVC_E_ARG, "null plan");
  return host_process(plan->cfgs[0], plan, point_cfg, n_points, points, n_process, order, n_neigh, neigh,
                      seed_mode, seeds, status, objmin, params, gn_iters, stats);
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_plan_autotune(dvc_plan *plan, const int *point_cfg_dev, int n_points,
                          const double *points_dev, int n_process, const int *order_dev,
                          int n_neigh, const int *neigh_dev, int seed_mode,
                          const double *seeds_dev, int *status_dev, double *objmin_dev,
                          double *params_dev, int reps, double ms_out[8]) try {
  if (!plan) return set_error(DVC_E_ARG, "null plan");
  if (reps < 1) return set_error(DVC_E_ARG, "reps must be >= 1");
  const int C0 = plan->cluster, S0 = plan->staging;
  double best = -1.0;
  int bestC = C0, bestS = S0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  CUDA_TRY(cudaEventCreate(&ev0));
  CUDA_TRY(cudaEventCreate(&ev1));
  int rc = DVC_OK;
  for (int j = 0; j < 4 && rc == DVC_OK; j++)
    for (int s = 0; s < 2 && rc == DVC_OK; s++) {
      if (ms_out) ms_out[2 * j + s] = -1.0;
      if (plan_build(plan, 1 << j, s) != DVC_OK) continue;  // this shape does not fit
      if (s == 1 && plan->n_staged == 0) continue;         // same as without staging
      auto run = [&]() {
        return dvc_gpu_plan_process_device(plan, point_cfg_dev, n_points, points_dev, n_process, order_dev,
                                           n_neigh, neigh_dev, seed_mode, seeds_dev, status_dev, objmin_dev,
                                           params_dev, nullptr, nullptr);
      };
      rc = run();
      if (rc) break;
      if (cudaEventRecord(ev0, 0) != cudaSuccess) { rc = set_error(DVC_E_CUDA, "event record"); break; }
      for (int r = 0; r < reps && rc == DVC_OK; r++) rc = run();
      if (rc) break;
      float ms = 0.f;
      if (cudaEventRecord(ev1, 0) != cudaSuccess || cudaEventSynchronize(ev1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess) {
        rc = set_error(DVC_E_CUDA, "autotune timing failed");
        break;
      }
      const double mean = ms / reps;
      if (ms_out) ms_out[2 * j + s] = mean;
      if (best < 0 || mean < best) {
        best = mean;
        bestC = 1 << j;
        bestS = s;
      }
    }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  const int rc2 = plan_build(plan, rc == DVC_OK ? bestC : C0, rc == DVC_OK ? bestS : S0);
  return rc ? rc : rc2;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_last_launch(dvc_engine *e, int out[4]) try {
  if (!e || !out) return set_error(DVC_E_ARG, "null argument");
  out[0] = e->last_cluster;
  out[1] = e->last_grid;
  out[2] = e->last_staged;
  out[3] = e->last_smem;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_last_windows(dvc_engine *e, int out[3]) try {
  if (!e || !out) return set_error(DVC_E_ARG, "null argument");
  for (int k = 0; k < 3; k++) out[k] = e->last_windows[k];
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_set_cluster(dvc_engine *e, int cluster) try {
  if (!e) return set_error(DVC_E_ARG, "null engine");
  if (cluster != 0 && cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8)
    return set_error(DVC_E_ARG, "cluster must be 0, 1, 2, 4 or 8");
  e->cluster = cluster;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_last_counters(dvc_engine *e, long long out[3]) try {
  if (!e || !out) return set_error(DVC_E_ARG, "null argument");
  out[0] = out[1] = out[2] = 0;
  if (e->counts_host) {
    for (int k = 0; k < 3; k++) out[k] = (long long)e->host_counts[k];
    return DVC_OK;
  }
  if (!e->last_ctl) return DVC_OK;
  unsigned long long c[3];
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(c, e->last_ctl + kCountersOff, sizeof c, cudaMemcpyDeviceToHost));
  for (int k = 0; k < 3; k++) out[k] = (long long)c[k];
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_set_wait_limit(dvc_engine *e, long long polls) try {
  if (!e) return set_error(DVC_E_ARG, "null engine");
  e->wait_polls = polls < 0 ? -1 : polls;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_last_status(dvc_engine *e) try {
  if (!e) return set_error(DVC_E_ARG, "null engine");
  if (!e->last_ctl) return DVC_OK;
  CUDA_TRY(cudaDeviceSynchronize());
  return launch_error(e);
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_last_phase_cycles(dvc_engine *e, long long out[DVC_N_PHASES]) try {
  if (!e || !out) return set_error(DVC_E_ARG, "null argument");
  for (int k = 0; k < DVC_N_PHASES; k++) out[k] = 0;
  if (!e->last_ctl) return DVC_OK;
  static_assert(DVC_N_PHASES == kPhases, "phase count");
  unsigned long long c[DVC_N_PHASES];
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(c, e->last_ctl + kCountersOff + 4 * sizeof(unsigned long long), sizeof c,
                      cudaMemcpyDeviceToHost));
  for (int k = 0; k < DVC_N_PHASES; k++) out[k] = (long long)c[k];
  if (getenv("DVC_VERBOSE")) {
    unsigned long long slow = 0, fp64 = 0;
    CUDA_TRY(cudaMemcpy(&slow, e->last_ctl + kCountersOff + 3 * sizeof(unsigned long long),
                        sizeof slow, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(&fp64, e->last_ctl + kCountersOff + kCounterFp64Solves * sizeof(unsigned long long),
                        sizeof fp64, cudaMemcpyDeviceToHost));
    fprintf(stderr, "dvc search: %llu integral-grid evaluations took the general path, "
            "%llu Gauss-Newton systems used the FP64 factorisation\n", slow, fp64);
  }
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

// ------------------------------------------------------ learned search ---
namespace {
// points of `order` whose search failed or whose objective exceeds thr
__global__ void fallback_kernel(int n_process, const int *order, const int *status, const double *objmin,
                                double thr, int *list, int *count) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_process) return;
  const int i = order[r];
  if (status[i] != DVC_POINT_GOOD || objmin[i] > thr) list[atomicAdd(count, 1)] = i;
}
// translations of the start parameters, [n][3]
__global__ void seeds3_kernel(int n, const double *p12, double *p3) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n * 3) p3[t] = p12[(size_t)(t / 3) * 12 + t % 3];
}
// Locality order for independent points: each point's bucket is the Morton
// code of its cell (cells of `cell` voxels, `bits` bits per axis), counted,
// scanned and scattered. Points whose searches run at the same time then
// read overlapping volume regions (L1 and L2 reuse); within a bucket the
// order is that of the atomic scatter.
__device__ __forceinline__ unsigned spread3(unsigned v) {  // bit k -> bit 3k (v < 2^10)
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__global__ void cell_key_kernel(int n, const int *order, const double *pts, double cell, int bits, int *key,
                                int *count) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int i = order[r];
  const unsigned lim = (1u << bits) - 1u;
  unsigned c[3];
  for (int d = 0; d < 3; d++) {
    const double v = floor(pts[(size_t)i * 3 + d] / cell);
    c[d] = !(v >= 0.0) ? 0u : (v > (double)lim ? lim : (unsigned)v);  // NaN: cell 0
  }
  const int k = (int)(spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2));
  key[r] = k;
  atomicAdd(count + k, 1);
}
__global__ void cell_scatter_kernel(int n, const int *order, const int *key, const int *start, int *cursor,
                                    int *out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int k = key[r];
  out[start[k] + atomicAdd(cursor + k, 1)] = order[r];
}
// results of the points in list, from the second search's arrays
__global__ void merge_kernel(int n, const int *list, const int *st2, const double *ob2, const double *pa2,
                             const int *it2, int *st, double *ob, double *pa, int *it) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int i = list[r];
  st[i] = st2[i];
  ob[i] = ob2[i];
  for (int k = 0; k < 12; k++) pa[(size_t)i * 12 + k] = pa2[(size_t)i * 12 + k];
  if (it) it[i] += it2[i];
}
}  // namespace

int dvc_cnn_patches(dvc_engine *e, int n, const double *points_dev, const int *idx_dev, float *patches_dev,
                    void *stream) try {
  if (!e || n < 0 || (n > 0 && (!points_dev || !patches_dev))) return set_error(DVC_E_ARG, "bad arguments");
  return dvc_internal_patches(e->ref, e->cor, e->p.bytes_per_voxel, e->p.vol_wide, e->p.vol_high,
                              e->p.vol_tall, n, points_dev, idx_dev, patches_dev, (cudaStream_t)stream);
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_process_learned(dvc_engine *e, dvc_cnn *net, int n_points, const double *points_dev, int n_process,
                            const int *order_dev, double obj_threshold, int *status_dev, double *objmin_dev,
                            double *params_dev, int *gn_iters_dev, int *n_fallback, void *stream) try {
  if (!e || !net) return set_error(DVC_E_ARG, "null engine or network");
  if (n_points < 0 || n_process < 0 || n_process > n_points) return set_error(DVC_E_ARG, "bad sizes");
  if (n_fallback) *n_fallback = 0;
  if (n_process == 0) return DVC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t N = (size_t)n_points;
  double *p12 = nullptr, *p3 = nullptr, *ob2 = nullptr, *pa2 = nullptr;
  int *list = nullptr, *cnt = nullptr, *st2 = nullptr, *it2 = nullptr;
  int *lord = nullptr, *lkey = nullptr, *lcount = nullptr;
  int rc = DVC_OK, nfb = 0;
  auto cleanup = [&]() {
    cudaFree(p12); cudaFree(p3); cudaFree(ob2); cudaFree(pa2);
    cudaFree(list); cudaFree(cnt); cudaFree(st2); cudaFree(it2);
    cudaFree(lord); cudaFree(lkey); cudaFree(lcount);
  };
  // the points' cells: 32 voxels or more, at most 64 per axis (Morton keys
  // of 18 bits)
  const int vmax = std::max(e->p.vol_wide, std::max(e->p.vol_high, e->p.vol_tall));
  double cell = 32.0;
  while (vmax / cell > 64.0) cell *= 2.0;
  int bits = 0;
  while ((1 << bits) < (int)std::ceil(vmax / cell)) bits++;
  const int nb = 1 << (3 * bits);
  if (cudaMalloc(&p12, N * 12 * 8) != cudaSuccess || cudaMalloc(&p3, N * 3 * 8) != cudaSuccess ||
      cudaMalloc(&list, (size_t)n_process * 4) != cudaSuccess || cudaMalloc(&cnt, 4) != cudaSuccess ||
      cudaMalloc(&lord, (size_t)n_process * 4) != cudaSuccess ||
      cudaMalloc(&lkey, (size_t)n_process * 4) != cudaSuccess ||
      cudaMalloc(&lcount, (size_t)(2 * nb + 1) * 4) != cudaSuccess) {
    cleanup();
    return set_error(DVC_E_NOMEM, "learned search buffers");
  }
  // the points in locality order: the network passes and the search take them
  // in it (every point's result is independent of the order)
  {
    int *start = lcount + nb, *cursor = lcount;
    const unsigned g = (unsigned)((n_process + 255) / 256);
    cudaMemsetAsync(lcount, 0, (size_t)nb * 4, st);
    cell_key_kernel<<<g, 256, 0, st>>>(n_process, order_dev, points_dev, cell, bits, lkey, lcount);
    exclusive_scan_kernel<<<1, 1024, 0, st>>>(nb, lcount, start);
    cudaMemsetAsync(cursor, 0, (size_t)nb * 4, st);
    cell_scatter_kernel<<<g, 256, 0, st>>>(n_process, order_dev, lkey, start, cursor, lord);
    if (cudaGetLastError() != cudaSuccess) {
      cleanup();
      return set_error(DVC_E_CUDA, "locality order");
    }
    order_dev = lord;
  }
  // DVC_VERBOSE: device time of the network passes, the search and the fallback
  const bool verbose = getenv("DVC_VERBOSE") != nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  if (verbose)
    for (auto &x : ev) cudaEventCreate(&x);
  if (verbose) cudaEventRecord(ev[0], st);
  cudaMemsetAsync(p12, 0, N * 12 * 8, st);
  rc = dvc_internal_cnn_seed(net, e->ref, e->cor, e->p.bytes_per_voxel, e->p.vol_wide, e->p.vol_high,
                             e->p.vol_tall, n_process, points_dev, order_dev, p12, st);
  if (verbose) cudaEventRecord(ev[1], st);
  if (!rc)
    rc = process_device_ws(e, n_points, points_dev, n_process, order_dev, 0, nullptr, DVC_SEED_PARAMS, p12,
                           status_dev, objmin_dev, params_dev, gn_iters_dev, stream, nullptr);
  if (verbose) cudaEventRecord(ev[2], st);
  if (!rc) {
    cudaMemsetAsync(cnt, 0, 4, st);
    fallback_kernel<<<(n_process + 255) / 256, 256, 0, st>>>(n_process, order_dev, status_dev, objmin_dev,
                                                             obj_threshold, list, cnt);
    if (cudaMemcpyAsync(&nfb, cnt, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = set_error(DVC_E_CUDA, "fallback count");
    if (!rc) rc = dvc_internal_cnn_status();
    if (!rc) rc = launch_error(e);
  }
  unsigned long long counts[3] = {0, 0, 0};
  if (!rc && cudaMemcpy(counts, e->last_ctl + kCountersOff, sizeof counts, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = set_error(DVC_E_CUDA, "learned search counters");
  if (!rc && nfb > 0) {
    if (cudaMalloc(&ob2, N * 8) != cudaSuccess || cudaMalloc(&pa2, N * 96) != cudaSuccess ||
        cudaMalloc(&st2, N * 4) != cudaSuccess || cudaMalloc(&it2, N * 4) != cudaSuccess) {
      cleanup();
      return set_error(DVC_E_NOMEM, "learned search buffers");
    }
    seeds3_kernel<<<(int)((N * 3 + 255) / 256), 256, 0, st>>>(n_points, p12, p3);
    rc = process_device_ws(e, n_points, points_dev, nfb, list, 0, nullptr, DVC_SEED_GIVEN, p3, st2, ob2, pa2,
                           it2, stream, nullptr);
    if (!rc)
      merge_kernel<<<(nfb + 255) / 256, 256, 0, st>>>(nfb, list, st2, ob2, pa2, it2, status_dev, objmin_dev,
                                                      params_dev, gn_iters_dev);
  }
  if (verbose) cudaEventRecord(ev[3], st);
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = set_error(DVC_E_CUDA, "learned search");
  if (verbose && !rc) {
    float ms[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < 3; k++) cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]);
    fprintf(stderr, "dvc learned search: %d points, network %.2f ms, search %.2f ms, fallback (%d points) %.2f ms\n",
            n_process, ms[0], ms[1], nfb, ms[2]);
  }
  if (verbose)
    for (auto &x : ev) cudaEventDestroy(x);
  if (!rc && nfb > 0) rc = launch_error(e);
  if (!rc && nfb > 0) {
    unsigned long long c2[3];
    if (cudaMemcpy(c2, e->last_ctl + kCountersOff, sizeof c2, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = set_error(DVC_E_CUDA, "learned search counters");
    for (int k = 0; k < 3; k++) counts[k] += c2[k];
  }
  if (!rc) {
    for (int k = 0; k < 3; k++) e->host_counts[k] = counts[k];
    e->counts_host = true;
  }
  if (!rc && n_fallback) *n_fallback = nfb;
  cleanup();
  return rc;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_interpolate(dvc_engine *e, int volume, const double center[3], int n, const double *pts,
                        int interp_type, double *out) try {
  if (!e || !center || (n > 0 && (!pts || !out))) return set_error(DVC_E_ARG, "null argument");
  if (interp_type < 0 || interp_type > 2) return set_error(DVC_E_ARG, "bad interp_type");
  if (n <= 0) return DVC_OK;
  // boxes as Interpolate::center_on; range check as tri_cub_Lek (FP64, host)
  double est_mn[3], act_mn[3], act_mx[3];
  int o[3];
  for (int d = 0; d < 3; d++) {
    est_mn[d] = e->nom_mn[d] + (center[d] - e->nom_cen[d]);
    const double amn = e->nom_mn[d] + 1.0, amx = e->nom_mx[d] + (-1.0);
    const double acen = (amn + amx) / 2.0;
    act_mn[d] = amn + (center[d] - acen);
    act_mx[d] = amx + (center[d] - acen);
    o[d] = (int)est_mn[d];
  }
  double bmn[3] = {9999.99, 9999.99, 9999.99}, bmx[3] = {-9999.99, -9999.99, -9999.99};
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      bmn[d] = std::min(bmn[d], pts[(size_t)i * 3 + d]);
      bmx[d] = std::max(bmx[d], pts[(size_t)i * 3 + d]);
    }
  for (int d = 0; d < 3; d++)
    if (bmn[d] < act_mn[d] || bmx[d] > act_mx[d])
      return set_error(DVC_E_RANGE, "points outside the active interpolation box");
  const int vol[3] = {e->p.vol_wide, e->p.vol_high, e->p.vol_tall};
  bool checked = false;
  for (int d = 0; d < 3; d++)
    if (o[d] - 1 < 0 || o[d] + e->bext[d] > vol[d] - 1) checked = true;
  double *d_pts = nullptr, *d_out = nullptr;
  unsigned long long *d_und = nullptr;
  CUDA_TRY(cudaMalloc(&d_pts, (size_t)n * 3 * sizeof(double)));
  CUDA_TRY(cudaMalloc(&d_out, (size_t)n * sizeof(double)));
  CUDA_TRY(cudaMalloc(&d_und, sizeof(unsigned long long)));
  CUDA_TRY(cudaMemset(d_und, 0, sizeof(unsigned long long)));
  CUDA_TRY(cudaMemcpy(d_pts, pts, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice));
  const void *vp = volume == 0 ? e->ref : e->cor;
  const BoxGeom Gm{o[0], o[1], o[2], e->bext[0], e->bext[1], e->bext[2]};
  const int T = 256, G = (n + T - 1) / T;
  if (e->p.bytes_per_voxel == 1) {
    GSrc<uint8_t> V{(const uint8_t *)vp, vol[0], vol[1], vol[2], checked};
    interp_points_kernel<uint8_t><<<G, T>>>(V, Gm, n, d_pts, interp_type, d_out, d_und);
  } else {
    GSrc<uint16_t> V{(const uint16_t *)vp, vol[0], vol[1], vol[2], checked};
    interp_points_kernel<uint16_t><<<G, T>>>(V, Gm, n, d_pts, interp_type, d_out, d_und);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpy(out, d_out, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(d_pts);
  cudaFree(d_out);
  cudaFree(d_und);
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_objective(int obj_function, int n, const double *ref, const double *tar, double *obj,
                      double *residual) try {
  if (obj_function < 0 || obj_function > 4) return set_error(DVC_E_ARG, "bad obj_function");
  if (n <= 0 || !ref || !tar || !obj) return set_error(DVC_E_ARG, "bad arguments");
  double *d_r = nullptr, *d_t = nullptr, *d_o = nullptr, *d_res = nullptr;
  CUDA_TRY(cudaMalloc(&d_r, (size_t)n * sizeof(double)));
  CUDA_TRY(cudaMalloc(&d_t, (size_t)n * sizeof(double)));
  CUDA_TRY(cudaMalloc(&d_o, sizeof(double)));
  if (residual) CUDA_TRY(cudaMalloc(&d_res, (size_t)n * sizeof(double)));
  CUDA_TRY(cudaMemcpy(d_r, ref, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(d_t, tar, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  objective_kernel<<<1, kObjThreads>>>(obj_function, n, d_r, d_t, d_o, d_res);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpy(obj, d_o, sizeof(double), cudaMemcpyDeviceToHost));
  if (residual) CUDA_TRY(cudaMemcpy(residual, d_res, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(d_r);
  cudaFree(d_t);
  cudaFree(d_o);
  cudaFree(d_res);
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

}  // extern "C"
