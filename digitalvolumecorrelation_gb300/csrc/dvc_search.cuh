// dvc_search.cuh — the per-point DVC search kernel.
//
// One persistent launch processes every ROI point. A thread-block cluster of
// C CTAs (C = 1..8, on C SMs) cooperates on one point at a time: the point's
// subvolume samples are split into C contiguous ranges, each CTA evaluates
// its range, and every sum the search needs (objective statistics, grid
// objectives, Gauss-Newton normal equations, bounding boxes) is reduced
// CTA-locally and then across the cluster through distributed shared memory,
// in a fixed order, so every CTA of the cluster holds identical totals and
// takes identical decisions. The cluster's leader CTA takes the next point in
// processing order from a device work counter, waits (bounded) for the
// neighbours that precede it when the reference's seeding is used, and
// publishes the result with a release flag. Points are handed out in order,
// so every awaited neighbour is owned by a cluster that is already running.
//
// Reference map (Core/...):
//   process_point            Search.cpp:95-192       -> search_kernel (per point)
//   starting_param           Search.cpp:277-377      -> point_seed
//   search_pt_setup          Search.cpp:248-275      -> point_seed + set-up phase
//   trgrid_global            Search.cpp:934-1043     -> grid phase
//   min_Lev_Mar, LM_prep_at  Search.cpp:194-246,490-525 -> Gauss-Newton phase
//   obj_val_at               Search.cpp:448-488      -> the evaluation loops
//   affine_to                FloatingCloud.cpp:236-286 -> sample_pos + warp_matrices
//   set_param_vect           SearchParams.cpp:53-107  -> warp_matrices
//   tri_cub_Lek / tri_lin / nearest Interpolate.cpp:404-567 -> interp_sample
//   obj_SAD .. obj_ZNSSD     ObjectiveFunctions.cpp:24-263 -> objective sums
#pragma once
#include <cooperative_groups.h>
#include <cuda.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "../../include/dvc_gpu.h"
#include "dvc_device.cuh"

namespace dvc {
namespace cg = cooperative_groups;

constexpr int kGridChunk = 128;               // grid offsets reduced together
constexpr long long kWaitPolls = 1LL << 25;   // default bound of a dependency wait (~seconds)
constexpr int kCB = 384;                      // cluster reduction buffer length
constexpr int kGRows = kMaxDof + 3;           // Gauss-Newton chunk rows: g[12], 1, t', q

// One search configuration (the settings of one `dvc` input file that shape a
// point's search): a launch holds one, or one per group of points.
struct SearchCfg {
  int geom, ndof, objfcn;
  int n_sub, cube_n;
  double subv_rad, aspect[3];
  double nom_mn[3], nom_mx[3], nom_cen[3];  // nominal interpolation box (Search::Search)
  int bext[3];                              // its integer extents
  int do_grid, num_inc;
  int inc_int;  // the grid step when it is a whole number of voxels, else 0
  double inc;
  double rigid[3];
  // the search's stages: coarse_random, random_global's translations
  // (rand_off, (2 num_inc + 1)^3 x 3 offsets from the estimate, in draw
  // order) in place of the grid; refine_nm, Nelder-Mead in place of
  // Gauss-Newton
  int coarse_random, refine_nm;
  const double *rand_off;
  // subvolume pre-check: searched only when at least min_count reference
  // samples lie in [gmin, gmax]
  int thresh_on;
  float gmin, gmax;
  double min_count;
  double inv_nsub;  // 1 / n_sub
  // staging of the correlate volume: box of stage[0] x stage[1] x stage[2]
  // voxels (stage_tx bytes), TMA-loaded into the staging buffer
  int stage_on;
  int stage_slab;  // the box covers one z slab of the grid's translations
  int stage[3];
  unsigned stage_tx;
  // the reference region's box (no grid reach; fits the same buffer)
  int stage_ref[3];
  unsigned stage_ref_tx;
  const CUtensorMap *tmap;       // this configuration's tensor map, or null: the kernel's
  const CUtensorMap *tmap_ref;   // the same box over the reference volume
  int rank_start[9];             // sample range of each cluster rank
  // stable offsets of the samples from their point: whole voxels and FP32
  // fractions; their extrema over all samples and over each rank's samples
  const int *off_i;
  const float *off_f;
  double off_min[3], off_max[3];
  double rank_off_min[8][3], rank_off_max[8][3];
};

struct SearchArgs {
  const void *ref, *cor;
  int nx, ny, nz;
  int itype;
  // the configuration of every point (n_cfg == 1), or per point
  // cfgs[point_cfg[point]] (n_cfg > 1)
  SearchCfg cfg0;
  const SearchCfg *cfgs;
  const int *point_cfg;
  int n_cfg;
  int n_points, n_process, n_neigh, seed_mode;
  const double *pts;
  const int *order, *rank, *neigh;
  const double *seeds;
  int *status;
  double *objmin, *params;
  int *gn_iters;
  int *work_counter, *done, *error_flag;
  // dataflow scheduling of the reference's seeding (Search::starting_param
  // reads the neighbours processed before a point): pend[i] counts point i's
  // unfinished predecessors; succ[succ_off[j] .. succ_off[j + 1]) lists the
  // points that have j as a predecessor; ready points are appended to queue
  // (queue_tail) as their last predecessor finishes and taken in queue order
  int dataflow;
  int *pend;
  const int *succ_off, *succ;
  int *queue, *queue_tail;
  // polls before a dependency wait (a neighbour's done flag, a ready-queue
  // slot) gives up and records DVC_E_TIMEOUT
  long long wait_polls;
  unsigned long long *counters;  // [0] evaluations, [1] GN iterations, [2] undefined evals,
                                 // [3] sample evaluations of the integral grid that took the
                                 // general path, [4 + k] SM cycles of phase k summed over
                                 // CTAs (PhaseClock), [16] Gauss-Newton systems solved by
                                 // the FP64 factorisation
  int local_cap;                 // per-CTA sample capacity of the dynamic arrays
  int stage_bytes;               // staging buffer (0: none), padded
};

struct DBox {
  double mn[3], mx[3];
};

// Point description broadcast by the cluster's leader CTA.
struct PointHeader {
  int rank, n, flag;  // flag 0: search, 1: no more work, 2: dependency wait gave up
  int pad;
  double pt[3], seed[3];
  DBox act_cor;
  int o_ref[3], o_cor[3];
  int chk_ref, chk_cor;
};

struct Region {
  int r0[3];  // global voxel coordinates of the staged box's first element (x aligned)
  int ok;     // the staged box covers this CTA's samples for the evaluation
};

struct CtaState {
  SearchCfg cfg;  // the current point's configuration
  PointHeader H;
  unsigned long long wkey[kWarps][6];  // per-warp position keys (range checks)
  double sref[3], sbmn[3], sbmx[3];
  double lbmn[3], lbmx[3];  // this CTA's share of the stable cloud: bbox
  Region reg[2];
  unsigned long long bar[2];
  int kint[3];        // s_ref + seed - O_cor: integer part
  float kfrac[3];     //                       fractional part
  float shift;        // value shift of the objective sums
  double rsum2;       // sum of squared reference quantities
  double par[kMaxDof];
  double upd[3];
  int iu[3];
  float fu[3];
  float M[9], R[9], N[27];  // (I+S)R - I, R, (I+S) dR/dangle
  int use_rot, fail, stop, best;
  int nm_act;    // Nelder-Mead: the next step (thread 0's decision)
  int tma_dead;  // a staging copy did not land in time: this CTA stages no more
  int lrange;                  // lpmn/lpmx hold the last evaluation's positions of this CTA
  double lpmn[3], lpmx[3];
  int pi[3], qi[3];            // point - reference box origin, point + seed - correlate box
  float pf[3], qf[3];          // origin: whole voxels and fractions
  double best_obj, obj, obj_old;
  int giu[kGridChunk][3];
  float gfu[kGridChunk][3];
  double objv[kGridChunk];
  double cbuf[2][kCB];
  double red[kCB];
  float wred[kWarps][2 * 8];
  double wredd[kWarps][8];
  double A[kMaxDof * kMaxDof], b[kMaxDof], x[kMaxDof], v[kMaxDof], diag[kMaxDof], vv;
  double ut[kMaxDof], jte[kMaxDof], scal[6];
  int perm[kMaxDof];
};

struct Cl {
  cg::cluster_group g;
  unsigned rank, size;
  int parity;
};

__device__ __forceinline__ int itrunc_d(double v) { return (int)v; }

__device__ __forceinline__ void split_d(double v, int &i, float &f) {
  const double fl = floor(v);
  i = (int)fl;
  f = (float)(v - fl);
}

// ------------------------------------------------------------ reductions ---
// The CTA's values are in S.cbuf[parity][0..K); entries [0, nmin) combine with
// min, the rest with +, over the cluster's CTAs in rank order. Result: S.red.
__device__ __forceinline__ void cluster_reduce(Cl &c, CtaState &S, int K, int nmin) {
  c.g.sync();
  for (int k = threadIdx.x; k < K; k += kThreads) {
    double t = k < nmin ? 1e300 : 0.0;
    for (unsigned r = 0; r < c.size; r++) {
      const double *rem = c.g.map_shared_rank(&S.cbuf[c.parity][0], r);
      const double v = rem[k];
      t = k < nmin ? fmin(t, v) : t + v;
    }
    S.red[k] = t;
  }
  c.parity ^= 1;
  __syncthreads();
}

// Position keys: (c + 2^20) << 32 | bits(f) orders exactly as c + f does for a
// cell c and a non-negative fraction f < 1. v[0..2] track the minima of the
// three axes, v[3..5] the minima of the complements (the maxima).
__device__ __forceinline__ void key_update(unsigned long long v[6], const int c[3], const float f[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const unsigned long long key =
        ((unsigned long long)(unsigned)(c[d] + (1 << 20)) << 32) | __float_as_uint(f[d]);
    v[d] = min(v[d], key);
    v[3 + d] = min(v[3 + d], ~key);
  }
}

__device__ __forceinline__ double key_pos(unsigned long long k) {
  return (double)((int)(k >> 32) - (1 << 20)) + (double)__uint_as_float((unsigned)k);
}

// CTA minima of the six key words into dst[0..6) (one barrier)
__device__ __forceinline__ void cta_keys(unsigned long long v[6], CtaState &S, unsigned long long *dst) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; k++)
#pragma unroll
    for (int o = 16; o; o >>= 1) v[k] = min(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 6; k++) S.wkey[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 6) {
    unsigned long long m = ~0ull;
    for (int w = 0; w < kWarps; w++) m = min(m, S.wkey[w][threadIdx.x]);
    dst[threadIdx.x] = m;
  }
}

// cluster_reduce with key words: FP64 sums of entries [0, nsum), minima of the
// unsigned 64-bit words stored in entries [nsum, nsum + nkey)
__device__ __forceinline__ void cluster_reduce_keys(Cl &c, CtaState &S, int nsum, int nkey) {
  c.g.sync();
  for (int k = threadIdx.x; k < nsum + nkey; k += kThreads) {
    if (k < nsum) {
      double t = 0.0;
      for (unsigned r = 0; r < c.size; r++) t += c.g.map_shared_rank(&S.cbuf[c.parity][0], r)[k];
      S.red[k] = t;
    } else {
      unsigned long long m = ~0ull;
      for (unsigned r = 0; r < c.size; r++)
        m = min(m, reinterpret_cast<const unsigned long long *>(c.g.map_shared_rank(&S.cbuf[c.parity][0], r))[k]);
      reinterpret_cast<unsigned long long *>(S.red)[k] = m;
    }
  }
  c.parity ^= 1;
  __syncthreads();
}

// CTA-level compensated sum of K (<= 8) Kahan partials into dst[0..K) (FP64):
// warp partials merged by FP32 TwoSum (about 48 significant bits), one FP64
// add at the end (each FP64 instruction occupies the narrow FP64 pipe for
// ~64 cycles, so a serial FP64 sum over the warps cost ~2k cycles).
template <int K>
__device__ __forceinline__ void cta_sum_comp(KSum (&v)[K], CtaState &S, double *dst) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float hi[K], lo[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    hi[k] = v[k].s;
    lo[k] = -v[k].c;
  }
#pragma unroll
  for (int k = 0; k < K; k++)
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const float bh = __shfl_xor_sync(0xffffffffu, hi[k], o);
      const float bl = __shfl_xor_sync(0xffffffffu, lo[k], o);
      two_sum_merge(hi[k], lo[k], bh, bl);
    }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; k++) {
      S.wred[warp][2 * k] = hi[k];
      S.wred[warp][2 * k + 1] = lo[k];
    }
  __syncthreads();
  if (threadIdx.x < K) {
    float h = S.wred[0][2 * threadIdx.x], l = S.wred[0][2 * threadIdx.x + 1];
    for (int w = 1; w < kWarps; w++) two_sum_merge(h, l, S.wred[w][2 * threadIdx.x], S.wred[w][2 * threadIdx.x + 1]);
    dst[threadIdx.x] = (double)h + (double)l;
  }
  __syncthreads();
}

// CTA-level min of K (<= 8) doubles into dst.
template <int K>
__device__ __forceinline__ void cta_min(double (&v)[K], CtaState &S, double *dst) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++)
#pragma unroll
    for (int o = 16; o; o >>= 1) v[k] = fmin(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; k++) S.wredd[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x < K) {
    double m = 1e300;
    for (int w = 0; w < kWarps; w++) m = fmin(m, S.wredd[w][threadIdx.x]);
    dst[threadIdx.x] = m;
  }
  __syncthreads();
}

// ------------------------------------------------------- sample geometry ---
// Box-local cell and fraction of local sample i for the translation (iu, fu)
// relative to the seed, plus the warp M d (d = offset from the stable
// reference point) when `rot`.
__device__ __forceinline__ void sample_pos(const int *s_ip, const float *s_fp, int i,
                                           const CtaState &S, const int iu[3], const float fu[3],
                                           bool rot, int c[3], float f[3]) {
  const int packed = s_ip[i];
  const int ip[3] = {packed & 1023, (packed >> 10) & 1023, (packed >> 20) & 1023};
  float F[3];
#pragma unroll
  for (int d = 0; d < 3; d++) F[d] = s_fp[i * 3 + d] + fu[d];
  if (rot) {
    float dv[3];
#pragma unroll
    for (int d = 0; d < 3; d++) dv[d] = (float)(ip[d] - S.kint[d]) + (s_fp[i * 3 + d] - S.kfrac[d]);
#pragma unroll
    for (int r = 0; r < 3; r++) F[r] += S.M[r * 3 + 0] * dv[0] + S.M[r * 3 + 1] * dv[1] + S.M[r * 3 + 2] * dv[2];
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float fl = floorf(F[d]);
    c[d] = ip[d] + iu[d] + (int)fl;
    f[d] = F[d] - fl;
  }
}

__device__ __forceinline__ float dvec(const int *s_ip, const float *s_fp, int i, const CtaState &S,
                                      int d) {
  const int ip = (s_ip[i] >> (10 * d)) & 1023;
  return (float)(ip - S.kint[d]) + (s_fp[i * 3 + d] - S.kfrac[d]);
}

// keep gathers inside the interpolation box whatever the position (NaN
// parameters, positions the range check already rejected)
__device__ __forceinline__ void clamp_cell(int c[3], const int bext[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++) c[d] = min(max(c[d], 0), bext[d] - 1);
}

// Objective from one-pass sums: S1 = sum t', S2 = sum t'^2, S3 = sum t' q,
// S4 = sum |t' - q|, t' = t - shift, q the per-sample reference quantity,
// rs2 = sum q^2, n samples.
// (inv_n = 1/n; FP64 division and square root cost ~440 and ~680 cycles
// here, so the mean is a product and 1/sigma one reciprocal square root)
__device__ __forceinline__ double objective_from_sums(int fcn, double S1, double S2, double S3,
                                                      double S4, double rs2, int n, double inv_n) {
  switch (fcn) {
    case DVC_SAD: return S4;
    case DVC_SSD: return S2 - 2.0 * S3 + rs2;
    case DVC_ZSSD: {
      const double m = S1 * inv_n;
      return (S2 - n * m * m) - 2.0 * S3 + rs2;
    }
    case DVC_NSSD: return 1.0 - S3 * rsqrt(S2);
    default: {
      const double m = S1 * inv_n;
      return 0.5 * (1.0 - S3 * rsqrt(S2 - n * m * m));
    }
  }
}

// ---------------------------------------------------- seed and boxes ---
// Search::starting_param (Core/Search.cpp:277-377) and the boxes of
// search_pt_setup (Core/Search.cpp:248-275), on the leader CTA's first warp.
// The lanes read the neighbour list (entries lane, lane + 32, ...), wait
// (bounded) for the neighbours the reference processes before this point
// and sum the displacements of the converged ones: per lane in list order,
// then a fixed shuffle tree, where the reference keeps one running sum (the
// two differ only in FP64 rounding). H.n and H.rank are set by lane 0.
__device__ bool point_seed(const SearchArgs &a, const SearchCfg &K, PointHeader &H) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int n = H.n;
  double sum[3] = {0.0, 0.0, 0.0};
  int good = 0;
  if (a.seed_mode == DVC_SEED_NEIGHBOURS) {
    int fail = 0;
    for (int j = lane; j < a.n_neigh && !fail; j += 32) {
      const int m = a.neigh[(size_t)n * a.n_neigh + j];
      if (m < 0 || m >= a.n_points) continue;
      if (a.rank[m] >= H.rank) continue;  // not yet processed when the reference reaches n
      long long polls = 0;
      volatile int *flag = a.done + m;
      while (*flag == 0) {
        if (++polls > a.wait_polls) {
          fail = 1;
          break;
        }
        __nanosleep(128);
      }
      if (fail) break;
      __threadfence();
      const volatile int *st = a.status;
      if (st[m] == DVC_POINT_GOOD) {
        const volatile double *pm = a.params + (size_t)m * 12;
        sum[0] += pm[0];
        sum[1] += pm[1];
        sum[2] += pm[2];
        good += 1;
      }
    }
    if (__any_sync(FULL, fail)) {
      if (lane == 0) atomicExch(a.error_flag, DVC_E_TIMEOUT);
      return false;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      for (int d = 0; d < 3; d++) sum[d] += __shfl_xor_sync(FULL, sum[d], o);
      good += __shfl_xor_sync(FULL, good, o);
    }
  }
  // lanes 0..2: the seed and the boxes of one axis each: the nominal box
  // centred on the point (reference volume) and on point + seed (correlate
  // volume); act box one voxel inside
  if (lane < 3) {
    const int d = lane;
    double sd;
    if (a.seed_mode == DVC_SEED_GIVEN) sd = a.seeds[(size_t)n * 3 + d];
    else if (a.seed_mode == DVC_SEED_PARAMS) sd = a.seeds[(size_t)n * 12 + d];
    else if (good != 0) sd = sum[d] / good;
    else sd = K.rigid[d];
    H.seed[d] = sd;
    const double cref = H.pt[d];
    const double ccor = __dadd_rn(H.pt[d], sd);  // Point::move_by
    const double ref_mn = __dadd_rn(K.nom_mn[d], __dsub_rn(cref, K.nom_cen[d]));
    const double cor_mn = __dadd_rn(K.nom_mn[d], __dsub_rn(ccor, K.nom_cen[d]));
    const double amn = __dadd_rn(K.nom_mn[d], 1.0), amx = __dadd_rn(K.nom_mx[d], -1.0);
    const double acen = __ddiv_rn(__dadd_rn(amn, amx), 2.0);
    const double dact = __dsub_rn(ccor, acen);
    H.act_cor.mn[d] = __dadd_rn(amn, dact);
    H.act_cor.mx[d] = __dadd_rn(amx, dact);
    H.o_ref[d] = itrunc_d(ref_mn);
    H.o_cor[d] = itrunc_d(cor_mn);
  }
  __syncwarp();
  if (lane == 0) {
    const int vol[3] = {a.nx, a.ny, a.nz};
    H.chk_ref = 0;
    H.chk_cor = 0;
    for (int d = 0; d < 3; d++) {
      if (H.o_ref[d] - 1 < 0 || H.o_ref[d] + K.bext[d] > vol[d] - 1) H.chk_ref = 1;
      if (H.o_cor[d] - 1 < 0 || H.o_cor[d] + K.bext[d] > vol[d] - 1) H.chk_cor = 1;
    }
  }
  __syncwarp();
  return true;
}

// The leader CTA's first warp, after point n's result is published: one
// predecessor fewer for every successor; those left with none become ready.
__device__ __forceinline__ void release_successors(const SearchArgs &a, int n) {
  const int lane = threadIdx.x & 31;
  for (int k = a.succ_off[n] + lane; k < a.succ_off[n + 1]; k += 32) {
    const int sp = a.succ[k];
    if (atomicSub(a.pend + sp, 1) == 1) {
      const int slot = atomicAdd(a.queue_tail, 1);
      atomicExch(a.queue + slot, sp);
    }
  }
}

// SearchParams::set_param_vect (Core/SearchParams.cpp:53-107) and the
// derivatives used by the analytic Jacobian. One thread.
__device__ void warp_matrices(const double *x, int ndof, CtaState &S) {
  if (ndof <= 3) {
    S.use_rot = 0;
    return;
  }
  S.use_rot = 1;
  // FP32: the matrices are consumed in FP32 by the sample positions. Cosines
  // enter M = (I+S)R - I through cos(a) - 1 = -2 sin^2(a/2), so M keeps its
  // full relative accuracy for small angles.
  float sf, cf, st, ct, sp, cp;
  sincosf((float)x[3], &sf, &cf);
  sincosf((float)x[4], &st, &ct);
  sincosf((float)x[5], &sp, &cp);
  const float s2 = sinf(0.5f * (float)x[3]), t2 = sinf(0.5f * (float)x[4]),
              p2 = sinf(0.5f * (float)x[5]);
  const float hf = -2.f * s2 * s2, ht = -2.f * t2 * t2, hp = -2.f * p2 * p2;  // cos - 1
  const float R[9] = {ct * cf, ct * sf, -st,
                      sp * st * cf - cp * sf, sp * st * sf + cp * cf, ct * sp,
                      cp * st * cf + sp * sf, cp * st * sf - sp * cf, ct * cp};
  // R - I with the diagonal formed from the cos - 1 terms
  float Rm[9] = {ht * cf + hf, R[1], R[2],
                 R[3], sp * st * sf + hp * cf + hf, R[5],
                 R[6], R[7], ht * cp + hp};
  const float dR[3][9] = {
      {-ct * sf, ct * cf, 0.f, -sp * st * sf - cp * cf, sp * st * cf - cp * sf, 0.f,
       -cp * st * sf + sp * cf, cp * st * cf + sp * sf, 0.f},
      {-st * cf, -st * sf, -ct, sp * ct * cf, sp * ct * sf, -st * sp, cp * ct * cf, cp * ct * sf,
       -st * cp},
      {0.f, 0.f, 0.f, cp * st * cf + sp * sf, cp * st * sf - sp * cf, ct * cp,
       -sp * st * cf + cp * sf, -sp * st * sf - cp * cf, -ct * sp}};
  float Sm[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (ndof > 6) {
    Sm[0] = (float)x[6]; Sm[1] = (float)x[9]; Sm[2] = (float)x[11];
    Sm[3] = (float)x[9]; Sm[4] = (float)x[7]; Sm[5] = (float)x[10];
    Sm[6] = (float)x[11]; Sm[7] = (float)x[10]; Sm[8] = (float)x[8];
  }
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      // M = (R - I) + S R ; N_q = (I + S) dR_q
      float m = Rm[r * 3 + c];
      for (int k = 0; k < 3; k++) m += Sm[r * 3 + k] * R[k * 3 + c];
      S.M[r * 3 + c] = m;
      S.R[r * 3 + c] = R[r * 3 + c];
      for (int q = 0; q < 3; q++) {
        float s = dR[q][r * 3 + c];
        for (int k = 0; k < 3; k++) s += Sm[r * 3 + k] * dR[q][k * 3 + c];
        S.N[q * 9 + r * 3 + c] = s;
      }
    }
}

// Householder QR with column pivoting solving A x = b (n <= 12, FP64) on one
// warp: the algorithm the reference reaches through
// colPivHouseholderQr().solve (Core/Search.cpp:234). Unknowns beyond the
// numerical rank are 0.
__device__ void warp_qr_solve(CtaState &S, int n) {
  const int lane = threadIdx.x & 31;
  double *A = S.A;  // row-major n x n
  if (lane < n) S.perm[lane] = lane;
  __syncwarp();
  for (int k = 0; k < n; k++) {
    double s = -1.0;
    if (lane >= k && lane < n) {
      s = 0.0;
      for (int i = k; i < n; i++) s += A[i * n + lane] * A[i * n + lane];
    }
    int pc = lane;
    double best = s;
    for (int o = 16; o; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, pc, o);
      if (ob > best || (ob == best && oi < pc)) {
        best = ob;
        pc = oi;
      }
    }
    if (pc != k) {
      if (lane < n) {
        const double t = A[lane * n + k];
        A[lane * n + k] = A[lane * n + pc];
        A[lane * n + pc] = t;
      }
      if (lane == 0) {
        const int t = S.perm[k];
        S.perm[k] = S.perm[pc];
        S.perm[pc] = t;
      }
    }
    __syncwarp();
    if (lane == 0) {
      double norm = 0.0;
      for (int i = k; i < n; i++) norm += A[i * n + k] * A[i * n + k];
      norm = sqrt(norm);
      S.vv = 0.0;
      if (norm != 0.0) {
        const double alpha = A[k * n + k] > 0 ? -norm : norm;
        double vv = 0.0;
        for (int i = k; i < n; i++) {
          S.v[i - k] = A[i * n + k] - (i == k ? alpha : 0.0);
          vv += S.v[i - k] * S.v[i - k];
        }
        S.vv = vv;
      }
    }
    __syncwarp();
    const double vv = S.vv;
    if (vv != 0.0 && lane >= k && lane <= n) {  // lane n applies the reflector to b
      double s2 = 0.0;
      for (int i = k; i < n; i++) s2 += S.v[i - k] * (lane < n ? A[i * n + lane] : S.b[i]);
      s2 = 2.0 * s2 / vv;
      for (int i = k; i < n; i++) {
        if (lane < n) A[i * n + lane] -= s2 * S.v[i - k];
        else S.b[i] -= s2 * S.v[i - k];
      }
    }
    __syncwarp();
    if (lane == 0) S.diag[k] = A[k * n + k];
    __syncwarp();
  }
  if (lane == 0) {
    int rank = 0;
    const double thr = 2.220446049250313e-16 * (double)n * fabs(S.diag[0]);
    for (int k = 0; k < n; k++) {
      if (fabs(S.diag[k]) > thr) rank = k + 1;
      else break;
    }
    double y[kMaxDof];
    for (int k = 0; k < n; k++) y[k] = 0.0;
    for (int k = rank - 1; k >= 0; k--) {
      double s2 = S.b[k];
      for (int j = k + 1; j < rank; j++) s2 -= A[k * n + j] * y[j];
      y[k] = s2 / A[k * n + k];
    }
    for (int k = 0; k < n; k++) S.x[S.perm[k]] = y[k];
  }
  __syncwarp();
}

// The solve used by the search: J'J is symmetric positive definite, so the
// Jacobi-scaled system D A D y = D b (D = diag(A)^-1/2) is factored by a
// Cholesky factorisation in FP32 across one warp (lane i holds row i of L,
// the columns' entries reach the other rows by shuffles), and three solves
// with FP64 residuals r = b - A x (iterative refinement) bring x to FP64
// accuracy. A pivoted Householder QR of the same system in FP32 took 100k
// cycles per 12-dof solve inside the search kernel (its serial shuffle
// chains dominated the iteration); this takes 18k. A pivot below 1e-4
// (condition number above about 10^4, where two refinements no longer reach
// FP64 accuracy, or a rank-deficient system) returns false and the caller
// uses the FP64 factorisation, which also decides the numerical rank.
// Scratch: S.red, free once A and b are assembled.
__device__ bool warp_solve_chol(CtaState &S, int n) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int M = kMaxDof;
  const int lane = threadIdx.x & 31;
  float *sL = reinterpret_cast<float *>(S.red);  // [M][M] L, row i columns <= i
  float *sAf = sL + M * M;                        // [M * M] A in FP32
  double *sX = reinterpret_cast<double *>(sAf + M * M);  // [M] current x
  for (int e = lane; e < n * n; e += 32) sAf[e] = (float)S.A[e];
  __syncwarp();
  const float di = (lane < n && sAf[lane * n + lane] > 0.f) ? rsqrtf(sAf[lane * n + lane]) : 1.f;
  float a[M], rinv[M];
#pragma unroll
  for (int j = 0; j < M; j++) {
    const float dj = __shfl_sync(FULL, di, j);
    a[j] = (lane < n && j < n) ? sAf[lane * n + j] * di * dj : 0.f;
  }
  bool ok = true;
#pragma unroll
  for (int k = 0; k < M; k++) {
    rinv[k] = 0.f;
    if (k < n) {
      const float piv = __shfl_sync(FULL, a[k], k);  // Schur complement diagonal
      ok = ok && (piv > 1e-4f);                      // also NaN
      const float r = rsqrtf(fmaxf(piv, 1e-30f));    // 1 / L_kk
      rinv[k] = r;
      const float l = a[k] * r;                      // lane i: L_ik
      a[k] = l;
#pragma unroll
      for (int j = k + 1; j < M; j++) {
        if (j < n) {
          const float lj = __shfl_sync(FULL, l, j);  // L_jk
          if (lane >= j) a[j] = fmaf(-l, lj, a[j]);
        }
      }
    }
  }
  if (!ok) return false;
  if (lane < n) {
#pragma unroll
    for (int j = 0; j < M; j++)
      if (j <= lane) sL[lane * M + j] = a[j];
  }
  __syncwarp();
  double xi = 0.0;  // lane i: x_i
#pragma unroll 1
  for (int pass = 0; pass < 3; pass++) {
    float z = 0.f;
    if (lane < n) {
      double r = S.b[lane];
      if (pass > 0)
        for (int j = 0; j < n; j++) r = fma(-S.A[lane * n + j], sX[j], r);
      z = (float)r * di;
    }
    // L y = z: lane k finishes y_k, the rows below take it off
#pragma unroll
    for (int k = 0; k < M; k++) {
      if (k < n) {
        const float yk = __shfl_sync(FULL, z, k) * rinv[k];
        if (lane == k) z = yk;
        else if (lane > k) z = fmaf(-a[k], yk, z);
      }
    }
    // L' w = y: lane k finishes w_k, the rows above take it off (L_ki from
    // shared memory)
#pragma unroll
    for (int k = M - 1; k >= 0; k--) {
      if (k < n) {
        const float wk = __shfl_sync(FULL, z, k) * rinv[k];
        if (lane == k) z = wk;
        else if (lane < k) z = fmaf(-sL[k * M + lane], wk, z);
      }
    }
    if (lane < n) {
      xi += (double)(z * di);
      sX[lane] = xi;
    }
    __syncwarp();
  }
  if (lane < n) S.x[lane] = xi;
  __syncwarp();
  return true;
}

// ----------------------------------------------------------- TMA staging ---
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

// One elected thread: order earlier generic-proxy reads of the buffer before
// the asynchronous write, arm the barrier with the byte count, start the
// 3D tiled copy (coordinates x, y, z in voxels; out-of-volume parts read 0).
__device__ __forceinline__ void tma_load_3d(const CUtensorMap *tm, uint32_t dst, uint32_t bar,
                                            int x, int y, int z, uint32_t bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// Bounded wait for the barrier's phase; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  for (long long i = 0; i < (1LL << 24); i++) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    if (ok) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

// Every thread of the block waits for the staging copy on barrier `bar`. A
// thread whose wait gives up marks the CTA (tma_dead) and records
// DVC_E_TIMEOUT; after the block barrier every thread sees the mark, so the
// evaluation path chosen from the region stays block-uniform: a dead CTA
// evaluates from global memory and starts no further copies (a late copy
// could land on a later one). The phase of a copy that never landed is not
// flipped, so the exit can wait for it once more. Block-uniform call sites.
__device__ __forceinline__ bool stage_wait(const SearchArgs &a, CtaState &S, uint32_t bar,
                                           uint32_t &phase) {
  if (!mbar_wait(bar, phase)) {
    S.tma_dead = 1;
    atomicExch(a.error_flag, DVC_E_TIMEOUT);
  }
  __syncthreads();
  if (S.tma_dead) return false;
  phase ^= 1u;
  return true;
}

// Staged region covering positions [pmin, pmax] (global voxel coordinates)
// with the stencil margin; ok = 0 when it does not fit the staging box.
__device__ __forceinline__ Region make_region_box(int on, const int box[3], const double pmin[3],
                                                  const double pmax[3], int esize) {
  Region r;
  r.ok = on;
  const int al = 16 / esize;
  for (int d = 0; d < 3; d++) {
    const double lo = floor(pmin[d]) - 2.0, hi = floor(pmax[d]) + 3.0;
    if (!(lo > -1e9 && hi < 1e9)) {  // NaN or absurd positions: do not stage
      r.ok = 0;
      r.r0[d] = 0;
      continue;
    }
    int l = (int)lo;
    if (d == 0) l = (l >= 0) ? (l / al) * al : -(((-l) + al - 1) / al) * al;
    r.r0[d] = l;
    if ((int)hi - l + 1 > box[d]) r.ok = 0;
  }
  return r;
}

__device__ __forceinline__ Region make_region(const SearchCfg &a, const double pmin[3],
                                              const double pmax[3], int esize) {
  return make_region_box(a.stage_on, a.stage, pmin, pmax, esize);
}

template <typename VT, int IT, bool GRAD>
__device__ __noinline__ float interp_gsrc(const GSrc<VT> src, int l0, int l1, int l2, int k0, int k1,
                                          int k2, float f0, float f1, float f2, float *g) {
  const int lo[3] = {l0, l1, l2}, kind[3] = {k0, k1, k2};
  const float f[3] = {f0, f1, f2};
  float gg[3];
  const float v = interp_at<GSrc<VT>, IT, GRAD>(src, lo, kind, f, gg);
  if (GRAD)
    for (int d = 0; d < 3; d++) g[d] = gg[d];
  return v;
}

// One sample of the correlate volume: from the staged box when its stencil
// lies inside, otherwise from global memory.
template <typename VT, int IT, bool GRAD>
__device__ __forceinline__ float eval_sample(bool staged, const SSrc<VT> &ss, const int r0[3],
                                             const int B[3], const GSrc<VT> &gs, const BoxGeom &G,
                                             int c[3], float f[3], float g[3], bool &undef) {
  int lo[3], kind[3];
  undef = prep_cell<IT>(G, c, f, lo, kind);
  const int w = IT == 0 ? 1 : 4;
  const bool in = staged && lo[0] >= r0[0] && lo[0] + w <= r0[0] + B[0] && lo[1] >= r0[1] &&
                  lo[1] + w <= r0[1] + B[1] && lo[2] >= r0[2] && lo[2] + w <= r0[2] + B[2];
  if (in) return interp_at<SSrc<VT>, IT, GRAD>(ss, lo, kind, f, g);
  return interp_gsrc<VT, IT, GRAD>(gs, lo[0], lo[1], lo[2], kind[0], kind[1], kind[2], f[0], f[1],
                                   f[2], g);
}

// The same with a compile-time choice: STAGED uses the staged box (and the
// out-of-line global path for the rare samples outside it); otherwise the
// global path is inlined.
template <typename VT, int IT, bool GRAD, bool STAGED>
__device__ __forceinline__ float eval_sample_t(const SSrc<VT> &ss, const int r0[3], const int B[3],
                                               const GSrc<VT> &gs, const BoxGeom &G, int c[3],
                                               float f[3], float g[3], bool &undef) {
  if (STAGED) return eval_sample<VT, IT, GRAD>(true, ss, r0, B, gs, G, c, f, g, undef);
  int lo[3], kind[3];
  undef = prep_cell<IT>(G, c, f, lo, kind);
  return interp_at<GSrc<VT>, IT, GRAD>(gs, lo, kind, f, g);
}

// ---------------------------------------------------- integral-step grid ---
// When the grid step inc is a whole number of voxels, every translation of
// the coarse grid (trgrid_global, Core/Search.cpp:934-1043) moves a sample by
// whole voxels: its cell fraction, and so its interpolation weights, are those
// of the centre translation. The CTA's threads are split into groups of
// `span` lanes; lane j of a group evaluates translation j of the chunk for the
// group's share of the samples. A warp thus gathers the stencils of ONE
// sample under 32 translations: addresses a fixed lattice apart, spread over
// the shared-memory banks (lanes that read the same word share it), where
// 32 different samples would hit the banks at random. Sample data reaches
// the lanes by shuffles, 32 samples per round. A (sample, translation) whose
// stencil leaves the staged box, or lies on a face cell or the undefined last
// plane, takes the general evaluation in its lane. Sums: FP32 over a round,
// compensated across rounds, then over the groups.
template <typename VT, int IT>
__device__ __forceinline__ void grid_chunk_lanes(
    const SearchArgs &a, CtaState &S, const int *s_ip, const float *s_fp, const float *s_r, int nl,
    float *s_scr, const SSrc<VT> &ss, const int r0[3], const int B[3], const GSrc<VT> &gsc,
    const BoxGeom &G, int o0, int nch, int side, int k, int parity, bool sad,
    unsigned long long &n_undef, unsigned long long &n_slow) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int esize = (int)sizeof(VT);
  const int tid = threadIdx.x, lane = tid & 31;
  int span = 32;
  while (span < nch) span *= 2;  // nch <= kGridChunk = 128
  const int groups = kThreads / span;
  const int j = tid % span, grp = tid / span;
  const bool live = j < nch;
  // this lane's translation
  const int step = S.cfg.inc_int;
  const int o = o0 + min(j, nch - 1);
  const int dc[3] = {(o % side - k) * step, ((o / side) % side - k) * step, (o / (side * side) - k) * step};
  const int dbytes = ((dc[2] * B[1] + dc[1]) * B[0] + dc[0]) * esize;
  const int n3[3] = {G.bx, G.by, G.bz};
  const int o3[3] = {G.ox, G.oy, G.oz};
  int lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    lo[d] = max(IT == 2 ? 1 : 0, r0[d] + 1 - o3[d]) - dc[d];
    hi[d] = min(min(n3[d] - (IT == 2 ? 3 : 2), S.cfg.bext[d] - 1), r0[d] + B[d] - 3 - o3[d]) - dc[d];
  }
  int iu0[3];
  float fu0[3];
#pragma unroll
  for (int d = 0; d < 3; d++) split_d(__dsub_rn(S.par[d], S.H.seed[d]), iu0[d], fu0[d]);
  // this group's samples
  const int s_lo = (int)(((long long)nl * grp) / groups), s_hi = (int)(((long long)nl * (grp + 1)) / groups);
  KSum k0, k1, k2;
  for (int ib = s_lo; ib < s_hi; ib += 32) {
    const int nb = min(32, s_hi - ib);
    // lane l prepares sample ib + l
    int c[3] = {0, 0, 0};
    float f[3] = {0.f, 0.f, 0.f}, qv = 0.f;
    uint32_t off0 = 0;
    if (lane < nb) {
      sample_pos(s_ip, s_fp, ib + lane, S, iu0, fu0, false, c, f);
      qv = s_r[ib + lane];
      off0 = ss.boff(o3[0] + c[0] - 1, o3[1] + c[1] - 1, o3[2] + c[2] - 1);
    }
    float p0 = 0.f, p1 = 0.f, p2 = 0.f;
#pragma unroll 2
    for (int m = 0; m < nb; m++) {
      const int cx = __shfl_sync(FULL, c[0], m), cy = __shfl_sync(FULL, c[1], m),
                cz = __shfl_sync(FULL, c[2], m);
      float fm[3] = {__shfl_sync(FULL, f[0], m), __shfl_sync(FULL, f[1], m), __shfl_sync(FULL, f[2], m)};
      const float q = __shfl_sync(FULL, qv, m);
      const uint32_t ob = __shfl_sync(FULL, off0, m);
      if (!live) continue;
      float t;
      if (cx >= lo[0] && cx <= hi[0] && cy >= lo[1] && cy <= hi[1] && cz >= lo[2] && cz <= hi[2]) {
        float w[3][4], dw[4];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          if (IT == 2) {
            cr_weights(fm[d], w[d], dw);
          } else {
            w[d][0] = 0.f; w[d][1] = 1.f - fm[d]; w[d][2] = fm[d]; w[d][3] = 0.f;
          }
        }
        float g[3];
        t = contract_h<SSrc<VT>, false>(ss, ss.stencil_at(ob + (uint32_t)dbytes), w[0], w[1], w[2],
                                        w[0], w[1], w[2], g);
      } else {
        int cc[3] = {cx + dc[0], cy + dc[1], cz + dc[2]};
        clamp_cell(cc, S.cfg.bext);
        float g[3];
        bool und;
        t = eval_sample_t<VT, IT, false, true>(ss, r0, B, gsc, G, cc, fm, g, und);
        n_undef += und;
        n_slow++;
      }
      t -= S.shift;
      if (sad) {
        p0 += fabsf(t - q);
      } else {
        p0 += t;
        p1 += t * t;
        p2 += t * q;
      }
    }
    k0.add(p0);
    k1.add(p1);
    k2.add(p2);
  }
  // groups -> chunk sums (FP32 pairs in scratch, FP64 in cbuf)
  float *part = s_scr;  // [groups][span][6]
  {
    float *my = part + ((size_t)grp * span + j) * 6;
    my[0] = k0.s; my[1] = -k0.c;
    my[2] = k1.s; my[3] = -k1.c;
    my[4] = k2.s; my[5] = -k2.c;
  }
  __syncthreads();
  if (tid < nch) {
    double acc[3] = {0.0, 0.0, 0.0};
    for (int g2 = 0; g2 < groups; g2++) {
      const float *pp = part + ((size_t)g2 * span + tid) * 6;
#pragma unroll
      for (int m = 0; m < 3; m++) acc[m] += (double)pp[2 * m] + (double)pp[2 * m + 1];
    }
#pragma unroll
    for (int m = 0; m < 3; m++) S.cbuf[parity][3 * tid + m] = acc[m];
  }
}

// The same evaluation with groups of exactly nch threads (any nch <= 128, so a
// slab of 25 translations keeps 250 of 256 threads busy where groups of 32
// lanes keep 200): thread j of a group evaluates translation o0 + j. A group
// may straddle two warps, so per round each thread prepares one sample of its
// group into a shared record (interpolation weights, reference quantity,
// stencil offset, packed cell) that every thread of the group then reads as
// a broadcast. `rec` holds 16 floats per thread (16-byte aligned), `s_scr`
// the group partial sums afterwards.
template <typename VT, int IT>
__device__ __forceinline__ void grid_chunk_groups(
    CtaState &S, const int *s_ip, const float *s_fp, const float *s_r, int nl, float *rec, float *s_scr,
    const SSrc<VT> &ss, const int r0[3], const int B[3], const GSrc<VT> &gsc, const BoxGeom &G, int o0,
    int nch, int side, int k, int parity, bool sad, unsigned long long &n_undef, unsigned long long &n_slow) {
  constexpr int esize = (int)sizeof(VT);
  const int tid = threadIdx.x;
  const int groups = kThreads / nch;
  const int grp = tid / nch, j = tid % nch;
  const bool in = grp < groups;
  // this thread's translation
  const int step = S.cfg.inc_int;
  const int o = o0 + j;
  const int dc[3] = {(o % side - k) * step, ((o / side) % side - k) * step, (o / (side * side) - k) * step};
  const int dbytes = ((dc[2] * B[1] + dc[1]) * B[0] + dc[0]) * esize;
  const int n3[3] = {G.bx, G.by, G.bz};
  const int o3[3] = {G.ox, G.oy, G.oz};
  int lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    lo[d] = max(IT == 2 ? 1 : 0, r0[d] + 1 - o3[d]) - dc[d];
    hi[d] = min(min(n3[d] - (IT == 2 ? 3 : 2), S.cfg.bext[d] - 1), r0[d] + B[d] - 3 - o3[d]) - dc[d];
  }
  int iu0[3];
  float fu0[3];
#pragma unroll
  for (int d = 0; d < 3; d++) split_d(__dsub_rn(S.par[d], S.H.seed[d]), iu0[d], fu0[d]);
  // this group's samples, in rounds of nch (one per thread)
  const int s_lo = in ? (int)(((long long)nl * grp) / groups) : 0;
  const int s_hi = in ? (int)(((long long)nl * (grp + 1)) / groups) : 0;
  const int per = (nl + groups - 1) / groups;
  const int rounds = (per + nch - 1) / nch;
  const uint32_t rg_addr = smem_addr(rec + (size_t)(in ? grp : 0) * nch * 16);
  KSum k0, k1, k2;
  for (int r = 0; r < rounds; r++) {
    const int sb0 = s_lo + r * nch;
    const int cnt = in ? max(0, min(nch, s_hi - sb0)) : 0;
    if (in && j < cnt) {
      int c[3];
      float f[3];
      sample_pos(s_ip, s_fp, sb0 + j, S, iu0, fu0, false, c, f);
      float w[3][4], dw[4];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        if (IT == 2) {
          cr_weights(f[d], w[d], dw);
        } else {
          w[d][0] = 0.f; w[d][1] = 1.f - f[d]; w[d][2] = f[d]; w[d][3] = 0.f;
        }
      }
      float4 *my = reinterpret_cast<float4 *>(rec) + (size_t)tid * 4;
      my[0] = make_float4(w[0][0], w[0][1], w[0][2], w[0][3]);
      my[1] = make_float4(w[1][0], w[1][1], w[1][2], w[1][3]);
      my[2] = make_float4(w[2][0], w[2][1], w[2][2], w[2][3]);
      // cells as signed 16-bit pairs (box-local, so far inside that range)
      my[3] = make_float4(s_r[sb0 + j],
                          __uint_as_float(ss.boff(o3[0] + c[0] - 1, o3[1] + c[1] - 1, o3[2] + c[2] - 1)),
                          __int_as_float((c[0] & 0xffff) | (c[1] << 16)), __int_as_float(c[2]));
    }
    __syncthreads();
    float p0 = 0.f, p1 = 0.f, p2 = 0.f;
#pragma unroll 1
    for (int m = 0; m < cnt; m++) {
      // the record by 8-byte loads, the weights only on the fast path
      const uint32_t ra = rg_addr + (uint32_t)m * 64u;
      const uint2 h0 = lds64(ra + 48), h1 = lds64(ra + 56);
      const float q = __uint_as_float(h0.x);
      const uint32_t obv = h0.y;
      const int cp = (int)h1.x, cz = (int)h1.y;
      const int cx = (cp << 16) >> 16, cy = cp >> 16;
      float t;
      if (cx >= lo[0] && cx <= hi[0] && cy >= lo[1] && cy <= hi[1] && cz >= lo[2] && cz <= hi[2]) {
        float wx[4], wy[4], wz[4];
#pragma unroll
        for (int a2 = 0; a2 < 2; a2++) {
          const uint2 ux = lds64(ra + 8 * a2), uy = lds64(ra + 16 + 8 * a2), uz = lds64(ra + 32 + 8 * a2);
          wx[2 * a2] = __uint_as_float(ux.x); wx[2 * a2 + 1] = __uint_as_float(ux.y);
          wy[2 * a2] = __uint_as_float(uy.x); wy[2 * a2 + 1] = __uint_as_float(uy.y);
          wz[2 * a2] = __uint_as_float(uz.x); wz[2 * a2 + 1] = __uint_as_float(uz.y);
        }
        float g[3];
        t = contract_h<SSrc<VT>, false>(ss, ss.stencil_at(obv + (uint32_t)dbytes), wx, wy, wz,
                                        wx, wy, wz, g);
      } else {
        int c[3];
        float f[3];
        sample_pos(s_ip, s_fp, sb0 + m, S, iu0, fu0, false, c, f);
        int cc[3] = {c[0] + dc[0], c[1] + dc[1], c[2] + dc[2]};
        clamp_cell(cc, S.cfg.bext);
        float g[3];
        bool und;
        t = eval_sample_t<VT, IT, false, true>(ss, r0, B, gsc, G, cc, f, g, und);
        n_undef += und;
        n_slow++;
      }
      t -= S.shift;
      if (sad) {
        p0 += fabsf(t - q);
      } else {
        p0 += t;
        p1 += t * t;
        p2 += t * q;
      }
    }
    k0.add(p0);
    k1.add(p1);
    k2.add(p2);
    __syncthreads();  // the records are rewritten next round
  }
  // groups -> chunk sums (FP32 pairs in scratch, merged by TwoSum, FP64 in cbuf)
  float *part = s_scr;  // [groups][nch][6]
  if (in) {
    float *my = part + ((size_t)grp * nch + j) * 6;
    my[0] = k0.s; my[1] = -k0.c;
    my[2] = k1.s; my[3] = -k1.c;
    my[4] = k2.s; my[5] = -k2.c;
  }
  __syncthreads();
  if (tid < nch) {
    float h[3], l[3];
#pragma unroll
    for (int m = 0; m < 3; m++) {
      h[m] = part[(size_t)tid * 6 + 2 * m];
      l[m] = part[(size_t)tid * 6 + 2 * m + 1];
    }
    for (int g2 = 1; g2 < groups; g2++) {
      const float *pp = part + ((size_t)g2 * nch + tid) * 6;
#pragma unroll
      for (int m = 0; m < 3; m++) two_sum_merge(h[m], l[m], pp[2 * m], pp[2 * m + 1]);
    }
#pragma unroll
    for (int m = 0; m < 3; m++) S.cbuf[parity][3 * tid + m] = (double)h[m] + (double)l[m];
  }
}

// Offset of coarse-stage translation o along axis d from the current
// estimate: the grid's (o in z, y, x loop order, steps of inc) or
// random_global's o-th draw.
__device__ __forceinline__ double coarse_off(const SearchCfg &K, int o, int d, int side, int k,
                                             double inc) {
  if (K.coarse_random) return K.rand_off[(size_t)o * 3 + d];
  const int off = d == 0 ? o % side - k : (d == 1 ? (o / side) % side - k : o / (side * side) - k);
  return __dmul_rn((double)off, inc);
}

// Keep the staged region when it covers positions [pmn, pmx] with the stencil
// margin; otherwise stage a new one into the same buffer. One thread; returns
// 1 when a copy was started (the block then waits for it).
__device__ __forceinline__ int restage(const SearchArgs &a, CtaState &S, const double pmn[3],
                                       const double pmx[3], int esize, const CUtensorMap *tm,
                                       uint32_t buf, uint32_t bar, uint32_t tx) {
  if (S.tma_dead) {
    S.reg[0].ok = 0;
    return 0;
  }
  const Region cur = S.reg[0];
  if (cur.ok) {
    bool in = true;
    for (int d = 0; d < 3; d++) {
      const double lo = floor(pmn[d]) - 2.0, hi = floor(pmx[d]) + 3.0;
      if (!(lo >= cur.r0[d] && hi < cur.r0[d] + S.cfg.stage[d])) in = false;
    }
    if (in) return 0;
  }
  const Region r = make_region(S.cfg, pmn, pmx, esize);
  S.reg[0] = r;
  if (!r.ok) return 0;
  tma_load_3d(tm, buf, bar, r.r0[0], r.r0[1], r.r0[2], tx);
  return 1;
}

// Range check of the moving sample cloud against the correlate act box
// (BoundBox::contains in tri_cub_Lek, Core/Interpolate.cpp:474-481).
// Translation only: the exact FP64 bbox (stable bbox + u, affine_to). With a
// rotation/strain: min/max of the warped samples over the cluster. Thread 0
// also gets this CTA's own position range in pmn/pmx (global voxel frame),
// which only it uses (staging).
__device__ __forceinline__ void range_check(Cl &cl, const int *s_ip, const float *s_fp, int nl,
                                            CtaState &S, bool rot, double pmn[3], double pmx[3]) {
  if (!rot) {
    if (threadIdx.x == 0) {
      int fail = 0;
      for (int d = 0; d < 3; d++) {
        const double bmn = __dadd_rn(S.sbmn[d], S.par[d]);
        const double bmx = __dadd_rn(S.sbmx[d], S.par[d]);
        if (!(bmn >= S.H.act_cor.mn[d]) || !(bmx <= S.H.act_cor.mx[d])) fail = 1;
        pmn[d] = S.lbmn[d] + S.par[d];
        pmx[d] = S.lbmx[d] + S.par[d];
      }
      S.fail = fail;
    }
    __syncthreads();
    return;
  }
  // Exact min / max of the warped positions c + f without FP64 per sample:
  // the key (c + 2^20) << 32 | bits(f) orders exactly as c + f does, f being
  // a non-negative float below 1. Mins of the keys and of their complements
  // (the maxima) over the CTA, then over the cluster.
  constexpr unsigned FULL = 0xffffffffu;
  unsigned long long v[6] = {~0ull, ~0ull, ~0ull, ~0ull, ~0ull, ~0ull};
  for (int i = threadIdx.x; i < nl; i += kThreads) {
    int c[3];
    float f[3];
    sample_pos(s_ip, s_fp, i, S, S.iu, S.fu, true, c, f);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const unsigned long long key =
          ((unsigned long long)(unsigned)(c[d] + (1 << 20)) << 32) | __float_as_uint(f[d]);
      v[d] = min(v[d], key);
      v[3 + d] = min(v[3 + d], ~key);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; k++)
#pragma unroll
    for (int o = 16; o; o >>= 1) v[k] = min(v[k], __shfl_xor_sync(FULL, v[k], o));
  unsigned long long *wk = reinterpret_cast<unsigned long long *>(S.red);  // [kWarps][6]
  unsigned long long *out = wk + 64;                                       // [6]
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 6; k++) wk[warp * 6 + k] = v[k];
  __syncthreads();
  unsigned long long *cb = reinterpret_cast<unsigned long long *>(S.cbuf[cl.parity]);
  if (threadIdx.x < 6) {
    unsigned long long m = ~0ull;
    for (int w = 0; w < kWarps; w++) m = min(m, wk[w * 6 + threadIdx.x]);
    cb[threadIdx.x] = m;
  }
  cl.g.sync();
  if (threadIdx.x < 6) {
    unsigned long long m = ~0ull;
    for (unsigned r = 0; r < cl.size; r++) {
      const unsigned long long *rem = cl.g.map_shared_rank(cb, r);
      m = min(m, rem[threadIdx.x]);
    }
    out[threadIdx.x] = m;
  }
  cl.parity ^= 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    // this CTA's own range (staging) and the cluster's (range check)
    int fail = 0;
    for (int d = 0; d < 3; d++) {
      const unsigned long long kl = cb[d], kh = ~cb[3 + d];
      const unsigned long long gl = out[d], gh = ~out[3 + d];
      const double o = (double)S.H.o_cor[d];
      pmn[d] = o + ((double)((int)(kl >> 32) - (1 << 20)) + (double)__uint_as_float((unsigned)kl));
      pmx[d] = o + ((double)((int)(kh >> 32) - (1 << 20)) + (double)__uint_as_float((unsigned)kh));
      const double bmn = o + ((double)((int)(gl >> 32) - (1 << 20)) + (double)__uint_as_float((unsigned)gl));
      const double bmx = o + ((double)((int)(gh >> 32) - (1 << 20)) + (double)__uint_as_float((unsigned)gh));
      if (!(bmn >= S.H.act_cor.mn[d]) || !(bmx <= S.H.act_cor.mx[d])) fail = 1;
    }
    S.fail = fail;
  }
  __syncthreads();
}

// Time per phase of the point loop, kept by thread 0 of each CTA from the SM
// clock and added to the call's counters once at exit: 0 take work and seed
// (dependency waits included), 1 reference subvolume and samples, 2 coarse
// grid, 3 Gauss-Newton entry and exit, 4 final objective and result; inside
// each Gauss-Newton iteration 5 warp matrices, 6 range check and staging,
// 7 sample evaluation and G'G chunks, 8 block and cluster reductions,
// 9 objective, assembly, solve and update, 10 G'G accumulation (inside 7).
constexpr int kPhases = 11;
// counters[]: 0..3 as listed in SearchArgs, 4 + k phase k's cycles, then the
// Gauss-Newton systems solved by the FP64 factorisation
constexpr int kCounterFp64Solves = 16;
constexpr int kNumCounters = kCounterFp64Solves + 1;
static_assert(4 + kPhases <= kCounterFp64Solves, "counter layout");
struct PhaseClock {
  long long acc[kPhases] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  long long prev = 0;
  int cur = 0;
  __device__ __forceinline__ void start() {
    if (threadIdx.x == 0) prev = clock64();
  }
  __device__ __forceinline__ void to(int ph) {
    if (threadIdx.x == 0) {
      const long long t = clock64();
      acc[cur] += t - prev;
      prev = t;
      cur = ph;
    }
  }
  __device__ __forceinline__ void flush(unsigned long long *counters) {
    to(0);
    if (threadIdx.x == 0)
      for (int k = 0; k < kPhases; k++) atomicAdd(counters + 4 + k, (unsigned long long)acc[k]);
  }
};

// ================================================================ kernel ===
// MINB: CTAs resident per SM the registers are sized for (1, or 2 for the
// searches without coarse grid that run two points per SM side by side)
template <typename VT, int IT, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
    search_kernel(const __grid_constant__ SearchArgs a, const __grid_constant__ CUtensorMap tmap,
                  const __grid_constant__ CUtensorMap tmap_ref) {
  extern __shared__ __align__(128) unsigned char dsm[];
  __shared__ CtaState S;
  Cl cl{cg::this_cluster(), 0u, 1u, 0};
  cl.rank = cl.g.block_rank();
  cl.size = cl.g.num_blocks();
  const int tid = threadIdx.x;
  constexpr int esize = (int)sizeof(VT);

  // dynamic shared memory: two staging buffers, then the per-CTA sample
  // state (packed cell base, fraction x3, reference quantity, final value)
  // and the Gauss-Newton chunk rows
  const int sb = a.stage_bytes;
  unsigned char *stage_buf[2] = {dsm, dsm};
  const int cap = a.local_cap;
  int *s_ip = reinterpret_cast<int *>(dsm + sb);
  float *s_fp = reinterpret_cast<float *>(s_ip + cap);
  float *s_r = s_fp + 3 * cap;
  float *s_t = s_r + cap;
  float *s_G = s_t + cap;  // [kGRows][kThreads]
  // the grid's shared sample records (16 floats per thread, 16-byte aligned)
  // reuse the final values and chunk rows, free during the grid phase
  float *grid_rec = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(s_t) + 15) & ~(uintptr_t)15);
  const bool grid_groups = grid_rec + 16 * kThreads <= s_G + kGRows * kThreads;
  const uint32_t bar_addr[2] = {smem_addr(&S.bar[0]), smem_addr(&S.bar[1])};
  const uint32_t buf_addr[2] = {smem_addr(stage_buf[0]), smem_addr(stage_buf[1])};
  uint32_t phase[2] = {0u, 0u};
  if (tid == 0) {
    S.tma_dead = 0;
    mbar_init(bar_addr[0]);
    mbar_init(bar_addr[1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the configuration of every point, when there is one
  if (a.n_cfg <= 1)
    for (int k = tid; k < (int)(sizeof(SearchCfg) / 4); k += kThreads)
      reinterpret_cast<int *>(&S.cfg)[k] = reinterpret_cast<const int *>(&a.cfg0)[k];
  __syncthreads();

  const GSrc<VT> gref{reinterpret_cast<const VT *>(a.ref), a.nx, a.ny, a.nz, false};
  const GSrc<VT> gcor0{reinterpret_cast<const VT *>(a.cor), a.nx, a.ny, a.nz, false};
  PhaseClock pc;
  pc.start();

  for (;;) {
    // --------------------------------------------- take work (leader) ---
    // In processing order, or with dataflow scheduling the next point whose
    // predecessors have all finished (the ready queue's next entry).
    if (cl.rank == 0 && tid < 32) {
      PointHeader &H = S.H;
      if (tid == 0) {
        H.flag = 0;
        const int h = atomicAdd(a.work_counter, 1);
        if (h >= a.n_process) {
          H.flag = 1;
        } else if (a.dataflow) {
          volatile int *slot = a.queue + h;
          long long polls = 0;
          int n;
          while ((n = *slot) < 0 && ++polls <= a.wait_polls) __nanosleep(256);
          if (n < 0) {
            atomicExch(a.error_flag, DVC_E_TIMEOUT);
            H.flag = 1;
          } else {
            __threadfence();
            H.n = n;
            H.rank = a.rank[n];
          }
        } else {
          H.rank = h;
          H.n = a.order[h];
        }
        if (H.flag == 0)
          for (int d = 0; d < 3; d++) H.pt[d] = a.pts[(size_t)H.n * 3 + d];
      }
      __syncwarp();
      if (a.n_cfg > 1 && H.flag == 0) {  // this point's configuration
        const int ci = a.point_cfg[H.n];
        if ((unsigned)ci >= (unsigned)a.n_cfg) {
          // no such configuration: the point is left unsearched, the call fails
          if (tid == 0) {
            atomicExch(a.error_flag, DVC_E_ARG);
            H.flag = 2;
          }
        } else {
          const int *src = reinterpret_cast<const int *>(a.cfgs + ci);
          for (int k = tid; k < (int)(sizeof(SearchCfg) / 4); k += 32) reinterpret_cast<int *>(&S.cfg)[k] = src[k];
        }
        __syncwarp();
      }
      if (H.flag == 0 && !point_seed(a, S.cfg, H) && tid == 0) H.flag = 2;
    }
    cl.g.sync();
    if (cl.rank != 0) {
      const int *src = reinterpret_cast<const int *>(cl.g.map_shared_rank(&S.H, 0));
      int *dst = reinterpret_cast<int *>(&S.H);
      for (int k = tid; k < (int)(sizeof(PointHeader) / 4); k += kThreads) dst[k] = src[k];
    }
    __syncthreads();
    if (S.H.flag == 1) break;
    if (S.H.flag == 2) {
      if (cl.rank == 0 && tid == 0) {
        a.status[S.H.n] = DVC_NOT_SEARCH;
        __threadfence();
        atomicExch(a.done + S.H.n, 1);
      }
      if (a.dataflow && cl.rank == 0 && tid < 32) {
        __syncwarp();
        release_successors(a, S.H.n);
      }
      cl.g.sync();
      continue;
    }
    if (a.n_cfg > 1) {
      if (cl.rank != 0) {
        const int *src = reinterpret_cast<const int *>(a.cfgs + a.point_cfg[S.H.n]);
        for (int k = tid; k < (int)(sizeof(SearchCfg) / 4); k += kThreads) reinterpret_cast<int *>(&S.cfg)[k] = src[k];
      }
      __syncthreads();
    }
    const SearchCfg &K = S.cfg;
    const int nsub = K.n_sub;
    const int lo = K.rank_start[cl.rank];
    const int nl = K.rank_start[cl.rank + 1] - lo;
    const int B[3] = {K.stage[0], K.stage[1], K.stage[2]};
    const uint32_t stage_tx = K.stage_tx;
    const CUtensorMap *tmp = K.tmap ? K.tmap : &tmap;
    const CUtensorMap *tmp_ref = K.tmap_ref ? K.tmap_ref : &tmap_ref;
    if (K.tmap && tid == 0) {  // tensor maps in global memory: their latest contents for the TMA unit
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                       reinterpret_cast<unsigned long long>(tmp))
                   : "memory");
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                       reinterpret_cast<unsigned long long>(tmp_ref))
                   : "memory");
    }
    const int ndof = K.ndof;
    const int fcn = K.objfcn;
    const bool sad = (fcn == DVC_SAD);
    const double inv_nsub = K.inv_nsub;
    GSrc<VT> gsr = gref, gsc = gcor0;
    gsr.checked = S.H.chk_ref;
    gsc.checked = S.H.chk_cor;
    const BoxGeom Gref{S.H.o_ref[0], S.H.o_ref[1], S.H.o_ref[2], K.bext[0], K.bext[1], K.bext[2]};
    const BoxGeom Gcor{S.H.o_cor[0], S.H.o_cor[1], S.H.o_cor[2], K.bext[0], K.bext[1], K.bext[2]};
    unsigned long long n_eval = 0, n_undef = 0, n_slow = 0;
    bool gn_last;                 // set before Gauss-Newton
    unsigned long long und_last;  // undefined-cell evaluations of its last evaluation
    if (tid == 0) S.fail = 0;
    pc.to(1);

    // ------------------------------- reference subvolume and samples ---
    // (search_pt_setup: the stable cloud interpolated in the reference box)
    // Sample positions relative to the boxes: the point's offset from each box
    // origin (FP64, once) plus the sample's stable offset, each split into
    // whole voxels and an FP32 fraction. The clouds' bounding boxes are the
    // point plus the offset extrema (FP64 rounding is monotone, so this is the
    // bounding box of the rounded FP64 positions); for cubes the reference's
    // own grid ends (FloatingCloud, Core/FloatingCloud.cpp:84-128).
    if (tid == 0) {
      for (int d = 0; d < 3; d++) {
        split_d(__dsub_rn(S.H.pt[d], (double)S.H.o_ref[d]), S.pi[d], S.pf[d]);
        split_d(__dsub_rn(__dadd_rn(S.H.pt[d], S.H.seed[d]), (double)S.H.o_cor[d]), S.qi[d], S.qf[d]);
        if (K.geom == DVC_SPHERE) {
          S.sbmn[d] = __dadd_rn(S.H.pt[d], K.off_min[d]);
          S.sbmx[d] = __dadd_rn(S.H.pt[d], K.off_max[d]);
        } else {
          const double r = __dmul_rn(K.subv_rad, K.aspect[d]);
          const double bmin = __dadd_rn(S.H.pt[d], -r);
          const double bmax = __dadd_rn(S.H.pt[d], r);
          const double inc = __ddiv_rn(__dsub_rn(bmax, bmin), (double)(K.cube_n - 1));
          S.sbmn[d] = bmin;
          S.sbmx[d] = __dadd_rn(bmin, __dmul_rn((double)(K.cube_n - 1), inc));
        }
        S.lbmn[d] = __dadd_rn(S.H.pt[d], K.rank_off_min[cl.rank][d]);  // this CTA's share
        S.lbmx[d] = __dadd_rn(S.H.pt[d], K.rank_off_max[cl.rank][d]);
      }
    }
    __syncthreads();
    // the reference region of this CTA's samples, staged by TMA into the
    // buffer that later holds the correlate region (same box)
    if (K.stage_on) {
      if (tid == 0) {
        const Region r = make_region_box(!S.tma_dead, K.stage_ref, S.lbmn, S.lbmx, esize);
        S.reg[0] = r;
        if (r.ok) tma_load_3d(tmp_ref, buf_addr[0], bar_addr[0], r.r0[0], r.r0[1], r.r0[2], K.stage_ref_tx);
      }
      __syncthreads();
      if (S.reg[0].ok) stage_wait(a, S, bar_addr[0], phase[0]);
    }
    {
      Region rr = S.reg[0];
      if (S.tma_dead) rr.ok = 0;
      const bool rstaged = K.stage_on && rr.ok;
      const int Br[3] = {K.stage_ref[0], K.stage_ref[1], K.stage_ref[2]};
      const SSrc<VT> ssr{buf_addr[0], rr.r0[0], rr.r0[1], rr.r0[2], Br[0], Br[1]};
      KSum rk[2];
      for (int i = tid; i < nl; i += kThreads) {
        int c[3], ip[3];
        float f[3], fp[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const int oi = K.off_i[(size_t)(lo + i) * 3 + d];
          const float of = K.off_f[(size_t)(lo + i) * 3 + d];
          const float F = S.pf[d] + of, G = S.qf[d] + of;
          const float fl = floorf(F), gl = floorf(G);
          c[d] = S.pi[d] + oi + (int)fl;
          f[d] = F - fl;
          ip[d] = min(max(S.qi[d] + oi + (int)gl, 0), 1023);
          fp[d] = G - gl;
        }
        clamp_cell(c, K.bext);
        bool und;
        float g[3];
        const float r = rstaged ? eval_sample_t<VT, IT, false, true>(ssr, rr.r0, Br, gsr, Gref, c, f, g, und)
                                : interp_global<VT, IT, false>(gsr, Gref, c, f, g, und);
        n_undef += und;
        s_r[i] = r;
        s_ip[i] = ip[0] | (ip[1] << 10) | (ip[2] << 20);
        s_fp[i * 3 + 0] = fp[0];
        s_fp[i * 3 + 1] = fp[1];
        s_fp[i * 3 + 2] = fp[2];
        rk[0].add(r);
        rk[1].add((r >= K.gmin && r <= K.gmax) ? 1.f : 0.f);
      }
      cta_sum_comp<2>(rk, S, S.cbuf[cl.parity]);
      cluster_reduce(cl, S, 2, 0);
    }
    // subvolume pre-check (subvol_thresh, documented in Core/InputRead.cpp:
    // 282-323): too few reference samples in the gray range, not searched
    if (K.thresh_on) {
      if (tid == 0 && S.red[1] < K.min_count) S.fail = 3;
      __syncthreads();
      if (S.fail) goto point_done;
    }
    {
    if (tid == 0) {
      for (int d = 0; d < 3; d++) {
        // stable reference point (FloatingCloud: centre, or middle of the cube box)
        if (K.geom == DVC_SPHERE) {
          S.sref[d] = S.H.pt[d];
        } else {
          const double r = __dmul_rn(K.subv_rad, K.aspect[d]);
          S.sref[d] = __ddiv_rn(__dadd_rn(__dadd_rn(S.H.pt[d], r), __dadd_rn(S.H.pt[d], -r)), 2.0);
        }
        int ki;
        float kf;
        split_d(__dsub_rn(__dadd_rn(S.sref[d], S.H.seed[d]), (double)S.H.o_cor[d]), ki, kf);
        S.kint[d] = ki;
        S.kfrac[d] = kf;
      }
      S.scal[0] = S.red[0] / nsub;  // reference mean
    }
    __syncthreads();
    const double rmean = S.scal[0];
    {
      KSum v[2];
      const float m = (float)rmean;
      for (int i = tid; i < nl; i += kThreads) {
        const float dv = s_r[i] - m;
        v[0].add(dv * dv);
        v[1].add(s_r[i] * s_r[i]);
      }
      cta_sum_comp<2>(v, S, S.cbuf[cl.parity]);
      cluster_reduce(cl, S, 2, 0);
    }
    const double rc2 = S.red[0], rraw2 = S.red[1];
    // per-sample reference quantity q and the value shift:
    //   SAD/SSD q = r - mean (shift = mean), ZSSD q = r - mean,
    //   NSSD q = r / |r| (no shift), ZNSSD q = (r - mean) / |r - mean|
    const float shift = (fcn == DVC_NSSD) ? 0.f : (float)rmean;
    const float qs = fcn == DVC_NSSD ? rsqrtf((float)rraw2) : (fcn == DVC_ZNSSD ? rsqrtf((float)rc2) : 1.f);
    for (int i = tid; i < nl; i += kThreads) s_r[i] = (s_r[i] - shift) * qs;
    if (tid == 0) {
      S.shift = shift;
      S.rsum2 = (fcn == DVC_NSSD || fcn == DVC_ZNSSD) ? 1.0 : rc2;
      for (int d = 0; d < 3; d++) S.par[d] = S.H.seed[d];
      for (int d = 3; d < kMaxDof; d++)
        S.par[d] = (a.seed_mode == DVC_SEED_PARAMS && d < ndof) ? a.seeds[(size_t)S.H.n * 12 + d] : 0.0;
      S.best = -1;
      S.best_obj = 1.7976931348623157e308;
      S.lrange = 0;
    }
    n_eval += 1;
    __syncthreads();
    }

    pc.to(2);
    // ---------------------------------------------------- grid search ---
    // trgrid_global (Core/Search.cpp:934-1043): (2k+1)^3 translations; the
    // first strictly smaller objective in z, y, x loop order wins. Any
    // translation whose sample box leaves the active box fails the point.
    // random_global (:1045-1098) is the same over its drawn translations
    // (the general evaluation path: their steps are not whole voxels).
    // The correlate region of each translation is staged by TMA into one of
    // two buffers while the previous translation is evaluated.
    if (K.do_grid && a.seed_mode != DVC_SEED_PARAMS) {
      const int k = K.num_inc;
      const int side = 2 * k + 1;
      const int total = side * side * side;
      const double inc = K.inc;
      // range check of every translation first (exact FP64; one thread each)
      {
        int bad = 0;
        for (int o = tid; o < total; o += kThreads) {
          for (int d = 0; d < 3; d++) {
            const double pc = __dadd_rn(S.par[d], coarse_off(K, o, d, side, k, inc));
            if (!(__dadd_rn(S.sbmn[d], pc) >= S.H.act_cor.mn[d]) ||
                !(__dadd_rn(S.sbmx[d], pc) <= S.H.act_cor.mx[d]))
              bad = 1;
          }
        }
        if (__syncthreads_or(bad)) {
          if (tid == 0) S.fail = 1;
          __syncthreads();
        }
      }
      if (S.fail) goto point_done;
      // one staged region covering this CTA's samples under every
      // translation, or (slab boxes) under the translations of one z offset,
      // restaged per chunk of side^2 translations (z-major order, so the
      // first strict minimum is the same)
      const bool slab = K.stage_slab != 0 && !K.coarse_random;
      const int chunk = slab ? side * side : kGridChunk;
      const int lane = tid & 31, warp = tid >> 5;
      for (int o0 = 0; o0 < total; o0 += chunk) {
        const int nch = min(chunk, total - o0);
        if (o0 == 0 || slab) {
          if (tid == 0) {
            const double zo = slab ? (double)(o0 / (side * side) - k) * inc : 0.0;
            double pmn[3], pmx[3];
            for (int d = 0; d < 3; d++) {
              const bool zs = slab && d == 2;
              pmn[d] = S.lbmn[d] + S.par[d] + (zs ? zo : -k * inc);
              pmx[d] = S.lbmx[d] + S.par[d] + (zs ? zo : k * inc);
            }
            Region r = make_region(K, pmn, pmx, esize);
            if (S.tma_dead) r.ok = 0;
            S.reg[0] = r;
            if (r.ok) tma_load_3d(tmp, buf_addr[0], bar_addr[0], r.r0[0], r.r0[1], r.r0[2], stage_tx);
          }
          __syncthreads();
          if (S.reg[0].ok) stage_wait(a, S, bar_addr[0], phase[0]);
        }
        Region rg = S.reg[0];
        if (S.tma_dead) rg.ok = 0;
        const SSrc<VT> ss{buf_addr[0], rg.r0[0], rg.r0[1], rg.r0[2], B[0], B[1]};
        if (tid < nch) {
          const int o = o0 + tid;
          for (int d = 0; d < 3; d++) {
            const double pc = __dadd_rn(S.par[d], coarse_off(K, o, d, side, k, inc));
            split_d(__dsub_rn(pc, S.H.seed[d]), S.giu[tid][d], S.gfu[tid][d]);
          }
        }
        __syncthreads();
        const bool integral = K.inc_int > 0 && !K.coarse_random;
        if (IT != 0 && rg.ok && integral && grid_groups) {
          grid_chunk_groups<VT, IT>(S, s_ip, s_fp, s_r, nl, grid_rec, grid_rec, ss, rg.r0, B, gsc, Gcor, o0, nch,
                                    side, k, cl.parity, sad, n_undef, n_slow);
        } else if (IT != 0 && rg.ok && integral) {
          grid_chunk_lanes<VT, IT>(a, S, s_ip, s_fp, s_r, nl, s_G, ss, rg.r0, B, gsc, Gcor, o0, nch,
                                   side, k, cl.parity, sad, n_undef, n_slow);
        } else {
        // each warp evaluates whole translations: its lanes cover this CTA's
        // samples, one shuffle reduction per translation, no block barrier
#pragma unroll 1
        for (int j = warp; j < nch; j += kWarps) {
          const int iu[3] = {S.giu[j][0], S.giu[j][1], S.giu[j][2]};
          const float fu[3] = {S.gfu[j][0], S.gfu[j][1], S.gfu[j][2]};
          float p0 = 0.f, p1 = 0.f, p2 = 0.f;
          auto body = [&](auto staged_tag) {
            constexpr bool ST = decltype(staged_tag)::value;
#pragma unroll (ST ? 2 : 1)
            for (int i = lane; i < nl; i += 32) {
              int c[3];
              float f[3], g[3];
              sample_pos(s_ip, s_fp, i, S, iu, fu, false, c, f);
              clamp_cell(c, K.bext);
              bool und;
              const float t = eval_sample_t<VT, IT, false, ST>(ss, rg.r0, B, gsc, Gcor, c, f, g, und) - S.shift;
              n_undef += und;
              const float q = s_r[i];
              if (sad) {
                p0 += fabsf(t - q);
              } else {
                p0 += t;
                p1 += t * t;
                p2 += t * q;
              }
            }
          };
          if (rg.ok) body(std::true_type{});
          else body(std::false_type{});
          // compensated warp reduction (TwoSum tree)
          float l0 = 0.f, l1 = 0.f, l2 = 0.f;
#pragma unroll
          for (int sh = 16; sh; sh >>= 1) {
            two_sum_merge(p0, l0, __shfl_xor_sync(0xffffffffu, p0, sh), __shfl_xor_sync(0xffffffffu, l0, sh));
            two_sum_merge(p1, l1, __shfl_xor_sync(0xffffffffu, p1, sh), __shfl_xor_sync(0xffffffffu, l1, sh));
            two_sum_merge(p2, l2, __shfl_xor_sync(0xffffffffu, p2, sh), __shfl_xor_sync(0xffffffffu, l2, sh));
          }
          if (lane == 0) {
            S.cbuf[cl.parity][3 * j + 0] = (double)p0 + (double)l0;
            S.cbuf[cl.parity][3 * j + 1] = (double)p1 + (double)l1;
            S.cbuf[cl.parity][3 * j + 2] = (double)p2 + (double)l2;
          }
        }
        }
        cluster_reduce(cl, S, 3 * nch, 0);
        if (tid < nch)
          S.objv[tid] = sad ? S.red[3 * tid]
                            : objective_from_sums(fcn, S.red[3 * tid], S.red[3 * tid + 1],
                                                  S.red[3 * tid + 2], 0.0, S.rsum2, nsub, inv_nsub);
        __syncthreads();
        if (tid == 0)
          for (int j = 0; j < nch; j++)
            if (S.objv[j] < S.best_obj) {  // first strictly smaller value wins
              S.best_obj = S.objv[j];
              S.best = o0 + j;
            }
        __syncthreads();
        n_eval += nch;
      }
      if (tid == 0 && S.best >= 0) {
        const int o = S.best;
        if (K.coarse_random) {
          for (int d = 0; d < 3; d++) S.par[d] = __dadd_rn(S.par[d], K.rand_off[(size_t)o * 3 + d]);
        } else {
          const int off[3] = {o % side - k, (o / side) % side - k, o / (side * side) - k};
          for (int d = 0; d < 3; d++) S.par[d] += (double)off[d] * inc;
        }
      }
      __syncthreads();
    } else if (tid == 0) {
      S.reg[0].ok = 0;
    }

    // ------------------------------------------- objective at S.par ---
    // obj_val_at(x) (Core/Search.cpp:448-488) at the parameters in S.par
    // (thread 0 sets them before the call): warp, range check (false: the
    // cloud left the active box, S.fail = 1), staging, the samples' values
    // (s_t) and the objective by explicit residuals, the reference's own
    // two-pass formulation (S.obj). reuse: s_t and their sum (S.red[0]) are
    // already those of these parameters (the last Gauss-Newton evaluation:
    // the same values summed in the same order), and its range check passed.
    {
    auto objective_at_par = [&](bool reuse) -> bool {
      if (reuse) {
        n_undef += und_last;
      } else {
        if (tid == 0) {
          warp_matrices(S.par, ndof, S);
          for (int d = 0; d < 3; d++) split_d(__dsub_rn(S.par[d], S.H.seed[d]), S.iu[d], S.fu[d]);
        }
        __syncthreads();
        const bool rot = S.use_rot;
        double pmn[3], pmx[3];
        range_check(cl, s_ip, s_fp, nl, S, rot, pmn, pmx);
        if (S.fail) return false;
        if (tid == 0) S.stop = restage(a, S, pmn, pmx, esize, tmp, buf_addr[0], bar_addr[0], stage_tx);
        __syncthreads();
        if (S.stop) stage_wait(a, S, bar_addr[0], phase[0]);
        Region rg = S.reg[0];
        if (S.tma_dead) rg.ok = 0;
        const SSrc<VT> ss{buf_addr[0], rg.r0[0], rg.r0[1], rg.r0[2], B[0], B[1]};
        {
          KSum v[1];
          for (int i = tid; i < nl; i += kThreads) {
            int c[3];
            float f[3], g[3];
            sample_pos(s_ip, s_fp, i, S, S.iu, S.fu, rot, c, f);
            clamp_cell(c, K.bext);
            bool und;
            const float t = (rg.ok ? eval_sample_t<VT, IT, false, true>(ss, rg.r0, B, gsc, Gcor, c, f, g, und)
                                   : eval_sample_t<VT, IT, false, false>(ss, rg.r0, B, gsc, Gcor, c, f, g, und)) -
                            S.shift;
            n_undef += und;
            s_t[i] = t;
            v[0].add(t);
          }
          cta_sum_comp<1>(v, S, S.cbuf[cl.parity]);
          cluster_reduce(cl, S, 1, 0);
        }
      }
      {
        const float tm = (float)(S.red[0] / nsub);
        {
          KSum v[2];
          for (int i = tid; i < nl; i += kThreads) {
            const float t = s_t[i];
            v[0].add((t - tm) * (t - tm));
            v[1].add(t * t);
          }
          cta_sum_comp<2>(v, S, S.cbuf[cl.parity]);
          cluster_reduce(cl, S, 2, 0);
        }
        const float inv_sig = rsqrtf((float)S.red[0]);
        const float inv_T = rsqrtf((float)S.red[1]);
        {
          KSum v[2];
          for (int i = tid; i < nl; i += kThreads) {
            const float t = s_t[i], q = s_r[i];
            float e;
            switch (fcn) {
              case DVC_SAD:
              case DVC_SSD: e = t - q; break;
              case DVC_ZSSD: e = (t - tm) - q; break;
              case DVC_NSSD: e = t * inv_T - q; break;
              default: e = (t - tm) * inv_sig - q; break;
            }
            v[0].add(e * e);
            v[1].add(fabsf(e));
          }
          cta_sum_comp<2>(v, S, S.cbuf[cl.parity]);
          cluster_reduce(cl, S, 2, 0);
        }
        if (tid == 0) {
          double obj = S.red[0];
          if (fcn == DVC_SAD) obj = S.red[1];
          if (fcn == DVC_NSSD) obj /= 2.0;
          if (fcn == DVC_ZNSSD) obj /= 4.0;
          S.obj = obj;
        }
        __syncthreads();
      }
      return true;
    };
    bool have_obj = false;  // S.obj holds the objective at the final parameters

    pc.to(3);
    // ------------------------------------------------- Gauss-Newton ---
    // min_Lev_Mar(start, 1e-6, 0.01) (Core/Search.cpp:194-246): undamped
    // Gauss-Newton on the residual vector of the objective, at most 20
    // iterations, stop when |obj - obj_old| < 1e-6 or |du| < 0.01. The
    // reference differentiates the residuals by forward differences
    // (h = 1e-10, LM_prep_at); here J is the analytic gradient of the
    // interpolant chained through the warp and the objective's normalisation:
    //   g_i = dt_i/dp (per sample), G = [g_i], t' = t - shift, q_i reference
    //   SSD/SAD: e = t - r,            J = G
    //   ZSSD:    e = t - tbar - q,     J = (I - 11'/n) G
    //   NSSD:    e = t/T - q,          J = (I - tt'/T^2) G / T
    //   ZNSSD:   e = (t-tbar)/sig - q, J = (I - 11'/n - that that') G / sig
    // so J'J and J'e follow from G'G, G'1, G't' and G'q: chunks of kThreads
    // samples pass through shared memory, one thread per matrix entry.
    gn_last = false;  // the last Gauss-Newton evaluation was at the final parameters
    und_last = 0;
    if (K.refine_nm) {
      // ----------------------------------------------- Nelder-Mead ---
      // look_with(amoeba, ndof, ftol) (Core/Search.cpp:379-440) with
      // min_Nelder_Mead (:680-932): simplex steps 0.2 in every parameter,
      // ftol 1e-5 for 3 dof and 1e-7 otherwise; reflection 1, expansion 2,
      // contraction -0.5 (kept only when it beats the best vertex, as the
      // reference has it), shrink 0.5 towards the best vertex; Convg_Fail
      // after 2000 evaluations; an evaluation outside the active box fails
      // the point. The simplex logic runs on thread 0 of every CTA in FP64
      // (the objectives are cluster totals, so all CTAs decide alike); each
      // objective is evaluated by the whole cluster. The simplex lives in the
      // Gauss-Newton chunk rows, which this mode leaves unused.
      double *nm = reinterpret_cast<double *>(s_G);  // [13][12] vertices
      double *nmv = nm + 13 * kMaxDof;              // [13] their objectives
      double *xref = nmv + 13;                       // [12] the reflected vertex
      const int nvrt = ndof + 1;
      const double tol = ndof == 3 ? 1e-5 : 1e-7;
      int nfunc = 0;
      int wrst = 0, best = 0, poor = 0;  // thread 0's
      double cen[kMaxDof], del[kMaxDof], yref = 0.0;
      if (tid == 0)
        for (int i = 0; i < nvrt; i++)
          for (int j = 0; j < ndof; j++)
            nm[i * kMaxDof + j] = (i > 0 && j == i - 1) ? __dadd_rn(S.par[j], 0.2) : S.par[j];
      for (int i = 0; i < nvrt; i++) {
        if (tid == 0)
          for (int j = 0; j < ndof; j++) S.par[j] = nm[i * kMaxDof + j];
        n_eval += 1;
        if (!objective_at_par(false)) goto point_done;
        if (tid == 0) nmv[i] = S.obj;
      }
      nfunc = nvrt;
      for (;;) {
        if (tid == 0) {
          wrst = 0;
          best = 0;
          for (int i = 1; i < nvrt; i++) {
            if (nmv[i] > nmv[wrst]) wrst = i;
            if (nmv[i] < nmv[best]) best = i;
          }
          poor = best;
          for (int i = 0; i < nvrt; i++)
            if (i != wrst && i != best && nmv[i] > nmv[poor]) poor = i;
          S.best = best;
          const double rel = __ddiv_rn(2.0 * fabs(nmv[wrst] - nmv[best]),
                                       fabs(nmv[wrst]) + fabs(nmv[best]) + 1.0e-10);
          if (rel < tol) {
            S.nm_act = 1;  // converged
          } else if (nfunc > 2000) {
            S.nm_act = 2;  // Convg_Fail
          } else {
            S.nm_act = 0;
            for (int j = 0; j < ndof; j++) {
              double c = 0.0;
              for (int i = 0; i < nvrt; i++)
                if (i != wrst) c = __dadd_rn(c, nm[i * kMaxDof + j]);
              c = __ddiv_rn(c, (double)ndof);
              cen[j] = c;
              del[j] = __dsub_rn(c, nm[wrst * kMaxDof + j]);
              xref[j] = __dadd_rn(c, del[j]);
              S.par[j] = xref[j];
            }
          }
        }
        __syncthreads();
        if (S.nm_act == 1) break;
        if (S.nm_act == 2) {
          if (tid == 0) S.fail = 2;
          __syncthreads();
          goto point_done;
        }
        n_eval += 1;
        if (!objective_at_par(false)) goto point_done;
        nfunc += 1;
        if (tid == 0) {
          yref = S.obj;
          if (yref <= nmv[poor] && yref >= nmv[best]) {  // keep the reflection
            for (int j = 0; j < ndof; j++) nm[wrst * kMaxDof + j] = xref[j];
            nmv[wrst] = yref;
            S.nm_act = 0;
          } else if (yref < nmv[best]) {  // try the expansion
            for (int j = 0; j < ndof; j++) S.par[j] = __dadd_rn(cen[j], __dmul_rn(2.0, del[j]));
            S.nm_act = 3;
          } else {  // the contraction
            for (int j = 0; j < ndof; j++) S.par[j] = __dadd_rn(cen[j], __dmul_rn(-0.5, del[j]));
            S.nm_act = 4;
          }
        }
        __syncthreads();
        if (S.nm_act == 0) continue;
        n_eval += 1;
        if (!objective_at_par(false)) goto point_done;
        nfunc += 1;
        if (tid == 0) {
          const double y = S.obj;
          if (S.nm_act == 3) {  // the expansion if better than the best, else the reflection
            const bool e = y < nmv[best];
            for (int j = 0; j < ndof; j++) nm[wrst * kMaxDof + j] = e ? S.par[j] : xref[j];
            nmv[wrst] = e ? y : yref;
            S.nm_act = 0;
          } else if (y < nmv[best]) {  // the contraction beats the best vertex
            for (int j = 0; j < ndof; j++) nm[wrst * kMaxDof + j] = S.par[j];
            nmv[wrst] = y;
            S.nm_act = 0;
          } else {
            S.nm_act = 5;  // shrink towards the best vertex
          }
        }
        __syncthreads();
        if (S.nm_act == 0) continue;
        for (int i = 0; i < nvrt; i++) {
          if (i == S.best) continue;
          if (tid == 0) {
            const int b = S.best;
            for (int j = 0; j < ndof; j++) {
              const double v = __dadd_rn(nm[b * kMaxDof + j],
                                         __dmul_rn(0.5, __dsub_rn(nm[i * kMaxDof + j], nm[b * kMaxDof + j])));
              nm[i * kMaxDof + j] = v;
              S.par[j] = v;
            }
          }
          n_eval += 1;
          if (!objective_at_par(false)) goto point_done;
          nfunc += 1;
          if (tid == 0) nmv[i] = S.obj;
        }
      }
      // the best vertex; its objective is the final one (obj_val_at there
      // evaluates the same values again)
      if (tid == 0) {
        const int b = S.best;
        for (int j = 0; j < ndof; j++) S.par[j] = nm[b * kMaxDof + j];
        S.obj = nmv[b];
        if (cl.rank == 0) {
          if (a.gn_iters) a.gn_iters[S.H.n] = nfunc;
          atomicAdd(a.counters + 1, (unsigned long long)nfunc);
        }
      }
      __syncthreads();
      have_obj = true;
    } else {
      int it_done = 20;
      unsigned long long und_it = 0;
      const int ntri = ndof * (ndof + 1) / 2;
      const int nent = ntri + 3 * ndof;
      // G'G in 3x3 register tiles: row blocks of the ndof gradient
      // components, column blocks of the components plus one block of the
      // (1, t, q) columns; tiles on or above the diagonal. Each tile is summed
      // by `parts` threads over interleaved samples (consecutive lanes read
      // consecutive samples: no bank conflicts), the parts are combined at
      // the end of the iteration.
      const int R = ndof / 3;
      const int ntile = R * (R + 1) / 2 + R;
      const int parts = kThreads / ntile;
      const int tile = tid / parts, part = tid % parts;
      const bool gact = tile < ntile;
      int row0 = 0, col0 = 0;
      if (gact) {
        int b = tile, rb = 0;
        while (b >= R + 1 - rb) {
          b -= R + 1 - rb;
          rb++;
        }
        const int cb = rb + b;
        row0 = 3 * rb;
        col0 = cb == R ? kMaxDof : 3 * cb;
      }
      for (int it = 0; it < 20; it++) {
        pc.to(5);
        if (tid == 0) {
          warp_matrices(S.par, ndof, S);
          for (int d = 0; d < 3; d++) split_d(__dsub_rn(S.par[d], S.H.seed[d]), S.iu[d], S.fu[d]);
        }
        __syncthreads();
        const bool rot = S.use_rot;
        double pmn[3], pmx[3];
        pc.to(6);
        // Translation only: the exact bbox check before the evaluation. With
        // rotation/strain the check rides on this iteration's evaluation
        // (position keys reduced with the sums; a failed check discards the
        // evaluation); a region is staged here only when none is, otherwise
        // the previous iteration restaged it if its positions left it.
        if (!rot || !S.reg[0].ok) {
          if (!rot) {
            range_check(cl, s_ip, s_fp, nl, S, rot, pmn, pmx);
            if (S.fail) goto point_done;
          } else {
            unsigned long long kv[6] = {~0ull, ~0ull, ~0ull, ~0ull, ~0ull, ~0ull};
            for (int i = tid; i < nl; i += kThreads) {
              int c[3];
              float f[3];
              sample_pos(s_ip, s_fp, i, S, S.iu, S.fu, true, c, f);
              key_update(kv, c, f);
            }
            cta_keys(kv, S, reinterpret_cast<unsigned long long *>(S.ut));
            __syncthreads();
            if (tid == 0) {
              const unsigned long long *k6 = reinterpret_cast<const unsigned long long *>(S.ut);
              for (int d = 0; d < 3; d++) {
                pmn[d] = (double)S.H.o_cor[d] + key_pos(k6[d]);
                pmx[d] = (double)S.H.o_cor[d] + key_pos(~k6[3 + d]);
              }
            }
          }
          if (tid == 0) S.stop = restage(a, S, pmn, pmx, esize, tmp, buf_addr[0], bar_addr[0], stage_tx);
          __syncthreads();
        } else if (tid == 0) {
          // restage when the last evaluation's positions left the region
          S.stop = S.lrange ? restage(a, S, S.lpmn, S.lpmx, esize, tmp, buf_addr[0], bar_addr[0],
                                      stage_tx)
                            : 0;
          S.lrange = 0;
        }
        __syncthreads();
        if (S.stop) stage_wait(a, S, bar_addr[0], phase[0]);
        Region rg = S.reg[0];
        if (S.tma_dead) rg.ok = 0;
        const SSrc<VT> ss{buf_addr[0], rg.r0[0], rg.r0[1], rg.r0[2], B[0], B[1]};
        pc.to(7);

        KSum v[4];
        float acc[9];
#pragma unroll
        for (int q = 0; q < 9; q++) acc[q] = 0.f;
        unsigned long long kv[6] = {~0ull, ~0ull, ~0ull, ~0ull, ~0ull, ~0ull};
        for (int base = 0; base < nl; base += kThreads) {
          const int i = base + tid;
          float g[kMaxDof];
#pragma unroll
          for (int p = 0; p < kMaxDof; p++) g[p] = 0.f;
          float t = 0.f, q = 0.f, one = 0.f;
          if (i < nl) {
            int c[3];
            float f[3], gv[3];
            sample_pos(s_ip, s_fp, i, S, S.iu, S.fu, rot, c, f);
            if (rot) key_update(kv, c, f);
            clamp_cell(c, K.bext);
            bool und;
            t = (rg.ok ? eval_sample_t<VT, IT, true, true>(ss, rg.r0, B, gsc, Gcor, c, f, gv, und)
                       : eval_sample_t<VT, IT, true, false>(ss, rg.r0, B, gsc, Gcor, c, f, gv, und)) -
                S.shift;
            n_undef += und;
            und_it += und;
            s_t[i] = t;
            q = s_r[i];
            one = 1.f;
            v[0].add(t);
            v[1].add(t * t);
            v[2].add(t * q);
            v[3].add(fabsf(t - q));
            g[0] = gv[0];
            g[1] = gv[1];
            g[2] = gv[2];
            if (ndof > 3) {
              float dv[3];
              for (int d = 0; d < 3; d++) dv[d] = dvec(s_ip, s_fp, i, S, d);
#pragma unroll
              for (int an = 0; an < 3; an++) {
                float acc = 0.f;
#pragma unroll
                for (int r = 0; r < 3; r++)
                  acc += gv[r] * (S.N[an * 9 + r * 3 + 0] * dv[0] + S.N[an * 9 + r * 3 + 1] * dv[1] +
                                  S.N[an * 9 + r * 3 + 2] * dv[2]);
                g[3 + an] = acc;
              }
              if (ndof > 6) {
                float Rd[3];
#pragma unroll
                for (int r = 0; r < 3; r++)
                  Rd[r] = S.R[r * 3 + 0] * dv[0] + S.R[r * 3 + 1] * dv[1] + S.R[r * 3 + 2] * dv[2];
                g[6] = gv[0] * Rd[0];
                g[7] = gv[1] * Rd[1];
                g[8] = gv[2] * Rd[2];
                g[9] = gv[0] * Rd[1] + gv[1] * Rd[0];
                g[10] = gv[1] * Rd[2] + gv[2] * Rd[1];
                g[11] = gv[0] * Rd[2] + gv[2] * Rd[0];
              }
            }
          }
#pragma unroll
          for (int p = 0; p < kMaxDof; p++) s_G[p * kThreads + tid] = g[p];
          s_G[(kMaxDof + 0) * kThreads + tid] = one;
          s_G[(kMaxDof + 1) * kThreads + tid] = t;
          s_G[(kMaxDof + 2) * kThreads + tid] = q;
          __syncthreads();
          pc.to(10);
          if (gact) {
            const int cnt = min(kThreads, nl - base);
            for (int s2 = part; s2 < cnt; s2 += parts) {
              float ga[3], gb[3];
#pragma unroll
              for (int q = 0; q < 3; q++) {
                ga[q] = s_G[(row0 + q) * kThreads + s2];
                gb[q] = s_G[(col0 + q) * kThreads + s2];
              }
#pragma unroll
              for (int q = 0; q < 9; q++) acc[q] = fmaf(ga[q / 3], gb[q % 3], acc[q]);
            }
          }
          __syncthreads();
          pc.to(7);
        }
        n_eval += 1;
        pc.to(8);
        cta_sum_comp<4>(v, S, S.cbuf[cl.parity]);
        // tile parts -> entries after the 4 value sums: each (part, entry)
        // is written by exactly one thread (the lower half of diagonal tiles
        // is left out), then summed over the parts with TwoSum
        {
          float *pe = s_G;  // [parts][nent], free after the last chunk
          if (gact) {
#pragma unroll
            for (int q = 0; q < 9; q++) {
              const int ra = row0 + q / 3, cb2 = col0 + q % 3;
              int e = -1;
              if (cb2 >= kMaxDof) e = ntri + (cb2 - kMaxDof) * ndof + ra;
              else if (ra <= cb2) e = ra * ndof - ra * (ra - 1) / 2 + (cb2 - ra);
              if (e >= 0) pe[part * nent + e] = acc[q];
            }
          }
          __syncthreads();
          if (tid < nent) {
            float hi = 0.f, lo = 0.f;
            for (int pp = 0; pp < parts; pp++) two_sum_merge(hi, lo, pe[pp * nent + tid], 0.f);
            S.cbuf[cl.parity][4 + tid] = (double)hi + (double)lo;
          }
        }
        if (rot) {
          cta_keys(kv, S, reinterpret_cast<unsigned long long *>(&S.cbuf[cl.parity][4 + nent]));
          cluster_reduce_keys(cl, S, 4 + nent, 6);
          // the range check of this evaluation (BoundBox::contains,
          // Core/Interpolate.cpp:474-481); this CTA's position range is kept
          // for the staging decision of the next iteration
          if (tid == 0) {
            const unsigned long long *g6 = reinterpret_cast<const unsigned long long *>(&S.red[4 + nent]);
            const unsigned long long *l6 =
                reinterpret_cast<const unsigned long long *>(&S.cbuf[cl.parity ^ 1][4 + nent]);
            int fail = 0;
            for (int d = 0; d < 3; d++) {
              const double o = (double)S.H.o_cor[d];
              if (!(o + key_pos(g6[d]) >= S.H.act_cor.mn[d]) || !(o + key_pos(~g6[3 + d]) <= S.H.act_cor.mx[d]))
                fail = 1;
              S.lpmn[d] = o + key_pos(l6[d]);
              S.lpmx[d] = o + key_pos(~l6[3 + d]);
            }
            S.fail = fail;
            S.lrange = 1;
          }
          __syncthreads();
          if (S.fail) goto point_done;
        } else {
          cluster_reduce(cl, S, 4 + nent, 0);
        }
        pc.to(9);
        // assemble J'J and -J'e (FP64)
        if (tid == 0) {
          // FP64 division and square root cost ~440 and ~680 cycles here: one
          // reciprocal square root gives 1/sigma, sigma and the scales
          const double S1 = S.red[0], S2 = S.red[1], S3 = S.red[2], S4 = S.red[3];
          const double n = nsub, mean = S1 * inv_nsub;
          double obj, sc = 1.0, rho = 0.0, den = 1.0, rden = 1.0;
          switch (fcn) {
            case DVC_SAD:
            case DVC_SSD:
            case DVC_ZSSD: obj = objective_from_sums(fcn, S1, S2, S3, S4, S.rsum2, nsub, inv_nsub); break;
            case DVC_NSSD:
              rden = rsqrt(S2);  // 1 / T
              den = S2 * rden;
              rho = S3 * rden;
              obj = 1.0 - rho;
              sc = rden * rden;
              break;
            default: {
              const double var = S2 - n * mean * mean;
              rden = rsqrt(var);  // 1 / sigma
              den = var * rden;
              rho = S3 * rden;
              obj = 0.5 * (1.0 - rho);
              sc = rden * rden;
              break;
            }
          }
          S.scal[0] = mean;
          S.scal[1] = sc;
          S.scal[2] = den;
          S.scal[3] = rho;
          S.scal[4] = rden;
          S.obj = obj;
          int stop = 0;
          if (it > 0) {
            // |obj - obj_old| < 1e-6 or |du| < 0.01 (min_Lev_Mar); |du|^2 is
            // compared first, the square root only near the threshold
            const double del_obj = fabs(obj - S.obj_old);
            const double m2 = S.upd[0] * S.upd[0] + S.upd[1] * S.upd[1] + S.upd[2] * S.upd[2];
            const bool small_du = m2 < 0.99999e-4 || (m2 <= 1.00001e-4 && sqrt(m2) < 0.01);
            if ((del_obj < 0.000001) || small_du) stop = 1;
          }
          S.stop = stop;
        }
        __syncthreads();
        if (S.stop) {
          it_done = it;
          gn_last = true;
          und_last = und_it;
          break;
        }
        {
          const double *GG = &S.red[4];
          const double *Gs = GG + ntri, *Gt = GG + ntri + ndof, *Gq = GG + ntri + 2 * ndof;
          const double mean = S.scal[0], sc = S.scal[1], rden = S.scal[4], rr = S.scal[3];
          const bool sub_mean = (fcn == DVC_ZSSD || fcn == DVC_ZNSSD);
          const bool sub_t = (fcn == DVC_NSSD || fcn == DVC_ZNSSD);
          if (tid < ndof) {
            const int p = tid;
            double ut = 0.0, jte;
            if (fcn == DVC_SAD || fcn == DVC_SSD) {
              jte = Gt[p] - Gq[p];
            } else if (fcn == DVC_ZSSD) {
              jte = Gt[p] - mean * Gs[p] - Gq[p];
            } else if (fcn == DVC_NSSD) {
              ut = Gt[p] * rden;
              jte = (rr * ut - Gq[p]) * rden;
            } else {
              ut = (Gt[p] - mean * Gs[p]) * rden;
              jte = (rr * ut - Gq[p]) * rden;
            }
            S.ut[p] = ut;
            S.b[p] = -jte;
          }
          __syncthreads();
          if (tid < ntri) {
            int e = tid, r = 0;
            while (e >= ndof - r) {
              e -= ndof - r;
              r++;
            }
            const int c2 = r + e;
            double v2 = GG[tid];
            if (sub_mean) v2 -= Gs[r] * Gs[c2] * inv_nsub;
            if (sub_t) v2 -= S.ut[r] * S.ut[c2];
            v2 *= sc;
            S.A[r * ndof + c2] = v2;
            S.A[c2 * ndof + r] = v2;
          }
          __syncthreads();
        }
        if (tid < 32) {
          if (!warp_solve_chol(S, ndof)) {
            warp_qr_solve(S, ndof);
            if (tid == 0) atomicAdd(a.counters + kCounterFp64Solves, 1ull);
          }
          if (tid < ndof) S.par[tid] += S.x[tid];
          if (tid < 3) S.upd[tid] = S.x[tid];
          if (tid == 0) S.obj_old = S.obj;
        }
        __syncthreads();
      }
      pc.to(3);
      if (cl.rank == 0 && tid == 0) {
        if (a.gn_iters) a.gn_iters[S.H.n] = it_done;
        atomicAdd(a.counters + 1, (unsigned long long)it_done);
      }
    }

    pc.to(4);
    // ------------------------------------------------ final objective ---
    // obj_val_at(par_min) (Core/Search.cpp:187); after Gauss-Newton stopped
    // by its rule the final parameters are those of its last evaluation
    if (!have_obj) {
      n_eval += 1;
      if (!objective_at_par(gn_last)) goto point_done;
    }
    }

  point_done:
    if (cl.rank == 0 && tid == 0) {
      const int n = S.H.n;
      if (S.fail) {
        a.status[n] = S.fail == 3 ? DVC_NOT_SEARCH : (S.fail == 2 ? DVC_CONVG_FAIL : DVC_RANGE_FAIL);
        a.objmin[n] = 0.0;
        for (int p = 0; p < 12; p++) a.params[(size_t)n * 12 + p] = 0.0;
      } else {
        a.status[n] = DVC_POINT_GOOD;
        a.objmin[n] = S.obj;
        for (int p = 0; p < 12; p++) a.params[(size_t)n * 12 + p] = p < ndof ? S.par[p] : 0.0;
      }
      __threadfence();
      atomicExch(a.done + n, 1);
      atomicAdd(a.counters + 0, n_eval);
    }
    if (a.dataflow && cl.rank == 0 && tid < 32) {
      __syncwarp();
      release_successors(a, S.H.n);
    }
    {
      unsigned long long u = n_undef;
      for (int o = 16; o; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
      if ((tid & 31) == 0 && u) atomicAdd(a.counters + 2, u);
      unsigned long long w = n_slow;
      for (int o = 16; o; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
      if ((tid & 31) == 0 && w) atomicAdd(a.counters + 3, w);
    }
    // the leader may overwrite its header only after every CTA copied it
    cl.g.sync();
    pc.to(0);
  }
  pc.flush(a.counters);
  // a copy that did not land in time: one more bounded wait before the
  // shared memory it writes is released
  if (S.tma_dead && tid == 0) mbar_wait(bar_addr[0], phase[0]);
  // no CTA leaves while another may still read its shared memory
  cl.g.sync();
}

}  // namespace dvc
