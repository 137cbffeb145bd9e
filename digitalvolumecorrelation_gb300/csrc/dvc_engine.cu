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
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include <chrono>

#include "../../include/dvc_gpu.h"
#include "dvc_device.cuh"
#include "dvc_internal.h"

using namespace dvc;

// ============================================================ error state ===
static thread_local std::string g_last_error;
static int set_error(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
int dvc_internal_set_error(int code, const char *msg) { return set_error(code, msg); }
#define CUDA_TRY(expr)                                                                 \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess)                                                             \
      return set_error(DVC_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// ======================================================= search constants ===
namespace {

constexpr int kMaxGridX = 8;         // x offsets of one grid row evaluated together
constexpr long long kWaitPolls = 1LL << 25;  // bounded dependency wait (~seconds)

struct SearchArgs {
  const void *ref, *cor;
  int nx, ny, nz;
  int geom, ndof, objfcn, itype;
  int n_sub, cube_n;
  double subv_rad, aspect[3];
  double nom_mn[3], nom_mx[3], nom_cen[3];  // nominal interpolation box (Search::Search)
  int bext[3];                              // its integer extents
  int do_grid, num_inc;
  double inc;
  double rigid[3];
  const double *sphere_rel;  // n_sub*3 uniform offsets (sphere)
  int n_points, n_process, n_neigh, seed_mode;
  const double *pts;
  const int *order, *rank, *neigh;
  const double *seeds;
  int *status;
  double *objmin, *params;
  int *gn_iters;
  int *work_counter, *done, *error_flag;
  unsigned long long *counters;  // [0] evaluations, [1] GN iterations, [2] undefined evals
  float *scratch;                // per-CTA sample state when it does not fit in shared memory
  long long scratch_floats_per_cta;
  int state_in_smem;
};

// FP64 box with BoundBox semantics (Core/BoundBox.cpp)
struct DBox {
  double mn[3], mx[3];
};

// State of the point a CTA is working on (shared memory).
struct PointState {
  int rank, n, fail;
  double pt[3], seed[3];
  DBox act_cor;
  int o_ref[3], o_cor[3];
  int chk_ref, chk_cor;
  double sref[3];                  // stable reference point
  double sbmn[3], sbmx[3];         // stable bbox
  int kint[3];                     // s_ref + seed - O_cor, integer part
  float kfrac[3];                  //                       fractional part
  float shift;                     // value shift for the objective sums
  double rsum2;                    // sum of squared reference quantities
  double par[kMaxDof];             // current parameters
  double jump_prev_update[3];
  // per-evaluation broadcast
  int iu[3];
  float fu[3];
  float M[9], R[9], N[27];         // (I+S)R - I, R, (I+S) dR/dangle
  int use_rot;
  // grid row broadcast
  int giu[kMaxGridX][3];
  float gfu[kMaxGridX][3];
  // reductions
  double red[256];
  float wred[kWarps][64];
  long long bbred[kWarps][6];
  double A[kMaxDof * kMaxDof], b[kMaxDof], x[kMaxDof], v[kMaxDof], diag[kMaxDof];
  int perm[kMaxDof];
  double obj;
  int grid_best[3];
  double grid_obj_min;
};

__device__ __forceinline__ int itrunc_d(double v) { return (int)v; }

// Block-wide sum of K floats per thread (warp shuffles, FP64 across warps).
template <int K>
__device__ __forceinline__ void block_sum(float (&v)[K], PointState &S) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++)
#pragma unroll
    for (int o = 16; o; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; k++) S.wred[warp][k] = v[k];
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double s = 0.0;
    for (int w = 0; w < kWarps; w++) s += (double)S.wred[w][k];
    S.red[k] = s;
  }
  __syncthreads();
}

// Block-wide compensated sum of K (hi, lo) pairs: TwoSum in the warp tree,
// FP64 across warps. Results in S.red[0..K).
template <int K>
__device__ __forceinline__ void block_sum_comp(KSum (&v)[K], PointState &S) {
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
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double s = 0.0;
    for (int w = 0; w < kWarps; w++) s += (double)S.wred[w][2 * k] + (double)S.wred[w][2 * k + 1];
    S.red[k] = s;
  }
  __syncthreads();
}

// Split a double into floor (int) and remainder (float).
__device__ __forceinline__ void split_d(double v, int &i, float &f) {
  const double fl = floor(v);
  i = (int)fl;
  f = (float)(v - fl);
}

// Box-local cell and fraction of sample i for translation (iu, fu) and
// optional warp M d (d = offset from the stable reference point).
__device__ __forceinline__ void sample_pos(const int *s_ip, const float *s_fp, int i,
                                           const PointState &S, const int iu[3],
                                           const float fu[3], bool rot, int c[3], float f[3]) {
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

__device__ __forceinline__ float dvec(const int *s_ip, const float *s_fp, int i, const PointState &S,
                                      int d) {
  const int packed = s_ip[i];
  const int ip = (packed >> (10 * d)) & 1023;
  return (float)(ip - S.kint[d]) + (s_fp[i * 3 + d] - S.kfrac[d]);
}

// keep gathers inside the interpolation box whatever the position (NaN
// parameters, positions the range check already rejected)
__device__ __forceinline__ void clamp_cell(int c[3], const int bext[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++) c[d] = min(max(c[d], 0), bext[d] - 1);
}

// Objective from the one-pass sums (see gauss_newton for the residual forms).
// S1 = sum t', S2 = sum t'^2, S3 = sum t' q, S4 = sum |t' - q|, t' = t - shift,
// q the per-sample reference quantity, rs2 = sum q^2, n samples.
__device__ __forceinline__ double objective_from_sums(int fcn, double S1, double S2, double S3,
                                                      double S4, double rs2, int n) {
  switch (fcn) {
    case DVC_SAD: return S4;
    case DVC_SSD: return S2 - 2.0 * S3 + rs2;
    case DVC_ZSSD: {
      const double m = S1 / n;
      return (S2 - n * m * m) - 2.0 * S3 + rs2;
    }
    case DVC_NSSD: return 1.0 - S3 / sqrt(S2);
    default: {
      const double m = S1 / n;
      const double sig = sqrt(S2 - n * m * m);
      return 0.5 * (1.0 - S3 / sig);
    }
  }
}

// ---------------------------------------------------- point set-up phase ---
// Seed (Search::starting_param, Core/Search.cpp:277-377) and boxes
// (search_pt_setup, Core/Search.cpp:248-275). Thread 0 only.
__device__ bool point_seed(const SearchArgs &a, PointState &S) {
  const int n = S.n;
  double sd[3];
  if (a.seed_mode == DVC_SEED_GIVEN) {
    for (int d = 0; d < 3; d++) sd[d] = a.seeds[(size_t)n * 3 + d];
  } else {
    double sx = 0.0, sy = 0.0, sz = 0.0;
    int good = 0;
    if (a.seed_mode == DVC_SEED_NEIGHBOURS) {
      for (int j = 0; j < a.n_neigh; j++) {
        const int m = a.neigh[(size_t)n * a.n_neigh + j];
        if (m < 0 || m >= a.n_points) continue;
        const int rk = a.rank[m];
        if (rk >= S.rank) continue;  // not yet processed when the reference reaches n
        // bounded wait for the neighbour's result
        long long polls = 0;
        volatile int *flag = a.done + m;
        while (*flag == 0) {
          if (++polls > kWaitPolls) {
            atomicExch(a.error_flag, DVC_E_TIMEOUT);
            return false;
          }
          __nanosleep(200);
        }
        __threadfence();
        const volatile int *st = a.status;
        if (st[m] == DVC_POINT_GOOD) {
          const volatile double *pm = a.params + (size_t)m * 12;
          sx += pm[0];
          sy += pm[1];
          sz += pm[2];
          good += 1;
        }
      }
    }
    if (good != 0) {
      sd[0] = sx / good;
      sd[1] = sy / good;
      sd[2] = sz / good;
    } else {
      for (int d = 0; d < 3; d++) sd[d] = a.rigid[d];
    }
  }
  for (int d = 0; d < 3; d++) S.seed[d] = sd[d];
  // interpolation boxes: the nominal box centred on the point (reference
  // volume) and on point + seed (correlate volume), act box one voxel inside
  for (int d = 0; d < 3; d++) {
    const double cref = S.pt[d];
    const double ccor = __dadd_rn(S.pt[d], sd[d]);  // Point::move_by
    const double dref = __dsub_rn(cref, a.nom_cen[d]);
    const double dcor = __dsub_rn(ccor, a.nom_cen[d]);
    const double ref_mn = __dadd_rn(a.nom_mn[d], dref);
    const double cor_mn = __dadd_rn(a.nom_mn[d], dcor);
    // act box: nominal box grown by -1, then centred with its own centre
    const double amn = __dadd_rn(a.nom_mn[d], 1.0), amx = __dadd_rn(a.nom_mx[d], -1.0);
    const double acen = __ddiv_rn(__dadd_rn(amn, amx), 2.0);
    const double dact = __dsub_rn(ccor, acen);
    S.act_cor.mn[d] = __dadd_rn(amn, dact);
    S.act_cor.mx[d] = __dadd_rn(amx, dact);
    S.o_ref[d] = itrunc_d(ref_mn);
    S.o_cor[d] = itrunc_d(cor_mn);
  }
  const int vol[3] = {a.nx, a.ny, a.nz};
  S.chk_ref = 0;
  S.chk_cor = 0;
  for (int d = 0; d < 3; d++) {
    if (S.o_ref[d] - 1 < 0 || S.o_ref[d] + a.bext[d] > vol[d] - 1) S.chk_ref = 1;
    if (S.o_cor[d] - 1 < 0 || S.o_cor[d] + a.bext[d] > vol[d] - 1) S.chk_cor = 1;
  }
  return true;
}

// Stable sample position (FloatingCloud constructors, Core/FloatingCloud.cpp:40-128)
__device__ __forceinline__ void stable_pos(const SearchArgs &a, const PointState &S, int i,
                                           double p[3]) {
  if (a.geom == DVC_SPHERE) {
    for (int d = 0; d < 3; d++)
      p[d] = __dadd_rn(S.pt[d], __dmul_rn(a.aspect[d], a.sphere_rel[(size_t)i * 3 + d]));
  } else {
    const int nn = a.cube_n;
    const int k = i % nn, j = (i / nn) % nn, l = i / (nn * nn);
    const int idx[3] = {k, j, l};
    for (int d = 0; d < 3; d++) {
      const double r = __dmul_rn(a.subv_rad, a.aspect[d]);
      const double bmin = __dadd_rn(S.pt[d], -r);
      const double bmax = __dadd_rn(S.pt[d], r);
      const double inc = __ddiv_rn(__dsub_rn(bmax, bmin), (double)(nn - 1));
      p[d] = __dadd_rn(bmin, __dmul_rn((double)idx[d], inc));
    }
  }
}

// ---------------------------------------------------------- warp matrices ---
// SearchParams::set_param_vect (Core/SearchParams.cpp:53-107) and the
// derivatives used by the analytic Jacobian. Thread 0.
__device__ void warp_matrices(const double *x, int ndof, PointState &S) {
  if (ndof <= 3) {
    S.use_rot = 0;
    return;
  }
  S.use_rot = 1;
  const double phi = x[3], the = x[4], psi = x[5];
  const double cf = cos(phi), sf = sin(phi), ct = cos(the), st = sin(the), cp = cos(psi), sp = sin(psi);
  double R[9] = {ct * cf, ct * sf, -st,
                 sp * st * cf - cp * sf, sp * st * sf + cp * cf, ct * sp,
                 cp * st * cf + sp * sf, cp * st * sf - sp * cf, ct * cp};
  double dR[3][9] = {
      {-ct * sf, ct * cf, 0.0, -sp * st * sf - cp * cf, sp * st * cf - cp * sf, 0.0,
       -cp * st * sf + sp * cf, cp * st * cf + sp * sf, 0.0},
      {-st * cf, -st * sf, -ct, sp * ct * cf, sp * ct * sf, -st * sp, cp * ct * cf, cp * ct * sf,
       -st * cp},
      {0.0, 0.0, 0.0, cp * st * cf + sp * sf, cp * st * sf - sp * cf, ct * cp,
       -sp * st * cf + cp * sf, -sp * st * sf - cp * cf, -ct * sp}};
  double IS[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (ndof > 6) {
    IS[0] += x[6]; IS[1] += x[9]; IS[2] += x[11];
    IS[3] += x[9]; IS[4] += x[7]; IS[5] += x[10];
    IS[6] += x[11]; IS[7] += x[10]; IS[8] += x[8];
  }
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      double m = 0.0;
      for (int k = 0; k < 3; k++) m += IS[r * 3 + k] * R[k * 3 + c];
      S.M[r * 3 + c] = (float)(m - (r == c ? 1.0 : 0.0));
      S.R[r * 3 + c] = (float)R[r * 3 + c];
      for (int a = 0; a < 3; a++) {
        double q = 0.0;
        for (int k = 0; k < 3; k++) q += IS[r * 3 + k] * dR[a][k * 3 + c];
        S.N[a * 9 + r * 3 + c] = (float)q;
      }
    }
}

// ---------------------------------------------------- warp-parallel solve ---
// Householder QR with column pivoting solving A x = b (n <= 12, FP64), the
// algorithm the reference reaches through colPivHouseholderQr().solve
// (Core/Search.cpp:234). Trailing unknowns beyond the numerical rank are 0.
__device__ void warp_qr_solve(PointState &S, int n) {
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
      S.v[0] = 0.0;
      S.obj = 0.0;
      if (norm != 0.0) {
        const double alpha = A[k * n + k] > 0 ? -norm : norm;
        double vv = 0.0;
        for (int i = k; i < n; i++) {
          S.v[i - k] = A[i * n + k] - (i == k ? alpha : 0.0);
          vv += S.v[i - k] * S.v[i - k];
        }
        S.obj = vv;  // scratch: v.v (0 = no reflection)
      }
    }
    __syncwarp();
    const double vv = S.obj;
    if (vv != 0.0) {
      if (lane >= k && lane <= n) {  // lane n applies the reflector to b
        double s2 = 0.0;
        for (int i = k; i < n; i++) s2 += S.v[i - k] * (lane < n ? A[i * n + lane] : S.b[i]);
        s2 = 2.0 * s2 / vv;
        for (int i = k; i < n; i++) {
          if (lane < n)
            A[i * n + lane] -= s2 * S.v[i - k];
          else
            S.b[i] -= s2 * S.v[i - k];
        }
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

// ================================================================ kernel ===
// Range check of the moving sample cloud against the correlate act box
// (BoundBox::contains inside tri_cub_Lek, Core/Interpolate.cpp:474-481).
// Translation only: the exact FP64 bbox (stable bbox + u, affine_to). With a
// rotation/strain: min/max of the warped samples (fixed point, 2^-24 voxel).
__device__ __forceinline__ void range_check(const int *s_ip, const float *s_fp, int nsub,
                                            PointState &S, bool rot) {
  const int tid = threadIdx.x;
  if (!rot) {
    if (tid == 0) {
      int fail = 0;
      for (int d = 0; d < 3; d++) {
        const double bmn = __dadd_rn(S.sbmn[d], S.par[d]);
        const double bmx = __dadd_rn(S.sbmx[d], S.par[d]);
        if (!(bmn >= S.act_cor.mn[d]) || !(bmx <= S.act_cor.mx[d])) fail = 1;
      }
      S.fail = fail;
    }
    __syncthreads();
    return;
  }
  long long mn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, mx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
  for (int i = tid; i < nsub; i += kThreads) {
    int c[3];
    float f[3];
    sample_pos(s_ip, s_fp, i, S, S.iu, S.fu, true, c, f);
    for (int d = 0; d < 3; d++) {
      const long long key = (long long)c[d] * 16777216LL + (long long)(f[d] * 16777216.0f);
      mn[d] = min(mn[d], key);
      mx[d] = max(mx[d], key);
    }
  }
  const int lane = tid & 31, warp = tid >> 5;
  for (int d = 0; d < 3; d++)
    for (int o = 16; o; o >>= 1) {
      mn[d] = min(mn[d], (long long)__shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = max(mx[d], (long long)__shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  if (lane == 0)
    for (int d = 0; d < 3; d++) {
      S.bbred[warp][d] = mn[d];
      S.bbred[warp][3 + d] = mx[d];
    }
  __syncthreads();
  if (tid == 0) {
    int fail = 0;
    for (int d = 0; d < 3; d++) {
      long long m0 = LLONG_MAX, m1 = LLONG_MIN;
      for (int w = 0; w < kWarps; w++) {
        m0 = min(m0, S.bbred[w][d]);
        m1 = max(m1, S.bbred[w][3 + d]);
      }
      const double bmn = (double)S.o_cor[d] + (double)m0 / 16777216.0;
      const double bmx = (double)S.o_cor[d] + (double)m1 / 16777216.0;
      if (!(bmn >= S.act_cor.mn[d]) || !(bmx <= S.act_cor.mx[d])) fail = 1;
    }
    S.fail = fail;
  }
  __syncthreads();
}

// Column sums of a [K][kThreads] float array in shared memory, compensated
// within each column, FP64 result in S.red[0..K).
__device__ __forceinline__ void column_sums(const float *buf, int K, PointState &S) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = warp; k < K; k += kWarps) {
    float hi = 0.f, lo = 0.f;
    for (int j = lane; j < kThreads; j += 32) two_sum_merge(hi, lo, buf[k * kThreads + j], 0.f);
    for (int o = 16; o; o >>= 1) {
      const float bh = __shfl_xor_sync(0xffffffffu, hi, o);
      const float bl = __shfl_xor_sync(0xffffffffu, lo, o);
      two_sum_merge(hi, lo, bh, bl);
    }
    if (lane == 0) S.red[k] = (double)hi + (double)lo;
  }
  __syncthreads();
}

template <typename VT, int IT>
__global__ void __launch_bounds__(kThreads, 2) search_kernel(SearchArgs a) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ PointState S;
  const int tid = threadIdx.x;
  const int nsub = a.n_sub;

  // sample state: packed cell base (int), cell fraction (3 floats), reference
  // quantity (float), and an auxiliary array (grid partials, GN gradient
  // chunks, final values)
  int *s_ip;
  float *s_fp, *s_r, *s_aux;
  if (a.state_in_smem) {
    s_ip = reinterpret_cast<int *>(dsm);
    s_fp = reinterpret_cast<float *>(s_ip + nsub);
    s_r = s_fp + 3 * nsub;
    s_aux = s_r + nsub;
  } else {
    float *base = a.scratch + (long long)blockIdx.x * a.scratch_floats_per_cta;
    s_ip = reinterpret_cast<int *>(base);
    s_fp = base + nsub;
    s_r = s_fp + 3 * nsub;
    s_aux = s_r + nsub;
  }

  const VolView<VT> base_ref{reinterpret_cast<const VT *>(a.ref), a.nx, a.ny, a.nz, 0, 0, 0,
                             a.bext[0], a.bext[1], a.bext[2], false};
  const VolView<VT> base_cor{reinterpret_cast<const VT *>(a.cor), a.nx, a.ny, a.nz, 0, 0, 0,
                             a.bext[0], a.bext[1], a.bext[2], false};

  for (;;) {
    // ------------------------------------------------------- take work ---
    if (tid == 0) {
      S.rank = atomicAdd(a.work_counter, 1);
      S.fail = 0;
    }
    __syncthreads();
    if (S.rank >= a.n_process) return;
    if (tid == 0) {
      S.n = a.order[S.rank];
      for (int d = 0; d < 3; d++) S.pt[d] = a.pts[(size_t)S.n * 3 + d];
      if (!point_seed(a, S)) S.fail = 2;
    }
    __syncthreads();
    if (S.fail == 2) {
      if (tid == 0) {
        a.status[S.n] = DVC_NOT_SEARCH;
        __threadfence();
        atomicExch(a.done + S.n, 1);
      }
      __syncthreads();
      continue;
    }
    VolView<VT> Vref = base_ref, Vcor = base_cor;
    Vref.ox = S.o_ref[0]; Vref.oy = S.o_ref[1]; Vref.oz = S.o_ref[2]; Vref.checked = S.chk_ref;
    Vcor.ox = S.o_cor[0]; Vcor.oy = S.o_cor[1]; Vcor.oz = S.o_cor[2]; Vcor.checked = S.chk_cor;
    const int ndof = a.ndof;
    const int fcn = a.objfcn;
    unsigned long long n_eval = 0, n_undef = 0;

    // ------------------------------------ reference subvolume + samples ---
    // (search_pt_setup: tri_cub_Lek of the stable cloud in the reference box)
    double lmn[3] = {1e300, 1e300, 1e300}, lmx[3] = {-1e300, -1e300, -1e300};
    KSum rk;
    for (int i = tid; i < nsub; i += kThreads) {
      double p[3];
      stable_pos(a, S, i, p);
      int c[3], ip[3];
      float f[3], fp[3];
      for (int d = 0; d < 3; d++) {
        lmn[d] = fmin(lmn[d], p[d]);
        lmx[d] = fmax(lmx[d], p[d]);
        split_d(__dsub_rn(p[d], (double)S.o_ref[d]), c[d], f[d]);
        split_d(__dsub_rn(__dadd_rn(p[d], S.seed[d]), (double)S.o_cor[d]), ip[d], fp[d]);
        ip[d] = min(max(ip[d], 0), 1023);
      }
      clamp_cell(c, a.bext);
      bool und;
      float g[3];
      const float r = interp_sample<VT, IT, false>(Vref, c, f, g, und);
      n_undef += und;
      s_r[i] = r;
      s_ip[i] = ip[0] | (ip[1] << 10) | (ip[2] << 20);
      s_fp[i * 3 + 0] = fp[0];
      s_fp[i * 3 + 1] = fp[1];
      s_fp[i * 3 + 2] = fp[2];
      rk.add(r);
    }
    // stable bbox (exact FP64 min/max)
    {
      const int lane = tid & 31, warp = tid >> 5;
      for (int d = 0; d < 3; d++)
        for (int o = 16; o; o >>= 1) {
          lmn[d] = fmin(lmn[d], __shfl_xor_sync(0xffffffffu, lmn[d], o));
          lmx[d] = fmax(lmx[d], __shfl_xor_sync(0xffffffffu, lmx[d], o));
        }
      if (lane == 0)
        for (int d = 0; d < 3; d++) {
          S.red[warp * 6 + d] = lmn[d];
          S.red[warp * 6 + 3 + d] = lmx[d];
        }
      __syncthreads();
      if (tid == 0) {
        for (int d = 0; d < 3; d++) {
          double mn = 1e300, mx = -1e300;
          for (int w = 0; w < kWarps; w++) {
            mn = fmin(mn, S.red[w * 6 + d]);
            mx = fmax(mx, S.red[w * 6 + 3 + d]);
          }
          S.sbmn[d] = mn;
          S.sbmx[d] = mx;
        }
        // stable reference point (FloatingCloud: centre, or middle of the cube box)
        for (int d = 0; d < 3; d++) {
          if (a.geom == DVC_SPHERE) {
            S.sref[d] = S.pt[d];
          } else {
            const double r = __dmul_rn(a.subv_rad, a.aspect[d]);
            S.sref[d] = __ddiv_rn(__dadd_rn(__dadd_rn(S.pt[d], r), __dadd_rn(S.pt[d], -r)), 2.0);
          }
          int ki;
          float kf;
          split_d(__dsub_rn(__dadd_rn(S.sref[d], S.seed[d]), (double)S.o_cor[d]), ki, kf);
          S.kint[d] = ki;
          S.kfrac[d] = kf;
        }
      }
      __syncthreads();
    }
    // reference statistics: mean, centred and raw sums of squares
    {
      KSum v1[1] = {rk};
      block_sum_comp<1>(v1, S);
    }
    const double rmean = S.red[0] / nsub;
    {
      KSum c2, q2;
      const float m = (float)rmean;
      for (int i = tid; i < nsub; i += kThreads) {
        const float dv = s_r[i] - m;
        c2.add(dv * dv);
        q2.add(s_r[i] * s_r[i]);
      }
      KSum v2[2] = {c2, q2};
      block_sum_comp<2>(v2, S);
    }
    const double rc2 = S.red[0], rraw2 = S.red[1];
    // per-sample reference quantity q and the value shift:
    //   SAD/SSD q = r - mean (shift = mean), ZSSD q = r - mean,
    //   NSSD q = r / |r| (no shift), ZNSSD q = (r - mean) / |r - mean|
    const float shift = (fcn == DVC_NSSD) ? 0.f : (float)rmean;
    const float qs = (float)(fcn == DVC_NSSD ? 1.0 / sqrt(rraw2) : (fcn == DVC_ZNSSD ? 1.0 / sqrt(rc2) : 1.0));
    for (int i = tid; i < nsub; i += kThreads) s_r[i] = (s_r[i] - shift) * qs;
    if (tid == 0) {
      S.shift = shift;
      S.rsum2 = (fcn == DVC_NSSD || fcn == DVC_ZNSSD) ? 1.0 : rc2;
      for (int d = 0; d < 3; d++) S.par[d] = S.seed[d];
      for (int d = 3; d < kMaxDof; d++) S.par[d] = 0.0;
    }
    n_eval += 1;
    __syncthreads();

    // ---------------------------------------------------- grid search ---
    // trgrid_global (Core/Search.cpp:934-1043): (2k+1)^3 translations, first
    // strictly smaller objective wins in z, y, x loop order. Any translation
    // whose sample box leaves the active box fails the point.
    if (a.do_grid) {
      const int k = a.num_inc;
      const double inc = a.inc;
      if (tid == 0) {
        int fail = 0;
        for (int z = -k; z <= k && !fail; z++)
          for (int y = -k; y <= k && !fail; y++)
            for (int x = -k; x <= k && !fail; x++) {
              const int o[3] = {x, y, z};
              for (int d = 0; d < 3; d++) {
                const double pc = __dadd_rn(S.par[d], __dmul_rn((double)o[d], inc));
                const double bmn = __dadd_rn(S.sbmn[d], pc), bmx = __dadd_rn(S.sbmx[d], pc);
                if (!(bmn >= S.act_cor.mn[d]) || !(bmx <= S.act_cor.mx[d])) fail = 1;
              }
            }
        S.fail = fail;
        S.grid_obj_min = 1.7976931348623157e308;
        S.grid_best[0] = S.grid_best[1] = S.grid_best[2] = 0;
      }
      __syncthreads();
      if (S.fail) goto point_done;
      const bool sad = (fcn == DVC_SAD);
      for (int z = -k; z <= k; z++)
        for (int y = -k; y <= k; y++)
          for (int x0 = -k; x0 <= k; x0 += kMaxGridX) {
            const int nxo = min(kMaxGridX, k - x0 + 1);
            if (tid < nxo) {
              const int o[3] = {x0 + tid, y, z};
              for (int d = 0; d < 3; d++) {
                // translation relative to the seed, added to the per-sample base
                const double pc = __dadd_rn(S.par[d], __dmul_rn((double)o[d], inc));
                split_d(__dsub_rn(pc, S.seed[d]), S.giu[tid][d], S.gfu[tid][d]);
              }
            }
            __syncthreads();
#pragma unroll 1
            for (int j = 0; j < nxo; j++) {
              const int iu[3] = {S.giu[j][0], S.giu[j][1], S.giu[j][2]};
              const float fu[3] = {S.gfu[j][0], S.gfu[j][1], S.gfu[j][2]};
              float p0 = 0.f, p1 = 0.f, p2 = 0.f;
              for (int i = tid; i < nsub; i += kThreads) {
                int c[3];
                float f[3], g[3];
                sample_pos(s_ip, s_fp, i, S, iu, fu, false, c, f);
                clamp_cell(c, a.bext);
                bool und;
                const float t = interp_sample<VT, IT, false>(Vcor, c, f, g, und) - S.shift;
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
              s_aux[(3 * j + 0) * kThreads + tid] = p0;
              s_aux[(3 * j + 1) * kThreads + tid] = p1;
              s_aux[(3 * j + 2) * kThreads + tid] = p2;
            }
            __syncthreads();
            column_sums(s_aux, 3 * nxo, S);
            if (tid == 0) {
              for (int j = 0; j < nxo; j++) {
                const double o =
                    sad ? S.red[3 * j]
                        : objective_from_sums(fcn, S.red[3 * j], S.red[3 * j + 1], S.red[3 * j + 2],
                                              0.0, S.rsum2, nsub);
                if (o < S.grid_obj_min) {  // first strictly smaller value wins
                  S.grid_obj_min = o;
                  S.grid_best[0] = x0 + j;
                  S.grid_best[1] = y;
                  S.grid_best[2] = z;
                }
              }
            }
            __syncthreads();
            n_eval += nxo;
          }
      if (tid == 0)
        for (int d = 0; d < 3; d++) S.par[d] += (double)S.grid_best[d] * inc;
      __syncthreads();
    }

    // ------------------------------------------------- Gauss-Newton ---
    // min_Lev_Mar(start, 1e-6, 0.01) (Core/Search.cpp:194-246): undamped
    // Gauss-Newton on the residual vector of the objective, at most 20
    // iterations, stop when |obj - obj_old| < 1e-6 or |du| < 0.01. The
    // reference differentiates the residuals by forward differences
    // (h = 1e-10, LM_prep_at); here J comes from the analytic gradient of the
    // interpolant chained through the warp and the objective's normalisation:
    //   g_i = dt_i/dp (per sample), G = [g_i], t' = t - shift, q_i reference
    //   SSD/SAD: e = t - r,            J = G
    //   ZSSD:    e = t - tbar - q,     J = (I - 11'/n) G
    //   NSSD:    e = t/T - q,          J = (I - tt'/T^2) G / T
    //   ZNSSD:   e = (t-tbar)/sig - q, J = (I - 11'/n - that that') G / sig
    // so J'J and J'e follow from G'G, G'1, G't' and G'q, accumulated per
    // chunk of kThreads samples through shared memory.
    {
      int it_done = 20;
      double obj_old = 0.0;
      const int ntri = ndof * (ndof + 1) / 2;
      const int nent = ntri + 3 * ndof;
      const int nparts = kThreads / nent;
      const int my_e = tid % nent, my_part = tid / nent;
      int ea = 0, eb = 0;
      if (my_e < ntri) {
        int e = my_e, r = 0;
        while (e >= ndof - r) {
          e -= ndof - r;
          r++;
        }
        ea = r;
        eb = r + e;
      } else {
        ea = (my_e - ntri) % ndof;
        eb = kMaxDof + (my_e - ntri) / ndof;  // rows 12 (ones), 13 (t'), 14 (q)
      }
      for (int it = 0; it < 20; it++) {
        if (tid == 0) {
          warp_matrices(S.par, ndof, S);
          for (int d = 0; d < 3; d++) split_d(__dsub_rn(S.par[d], S.seed[d]), S.iu[d], S.fu[d]);
        }
        __syncthreads();
        const bool rot = S.use_rot;
        range_check(s_ip, s_fp, nsub, S, rot);
        if (S.fail) goto point_done;

        KSum v1, v2, v3;
        float v4 = 0.f;
        float gg = 0.f;  // this thread's entry partial
        for (int base = 0; base < nsub; base += kThreads) {
          const int i = base + tid;
          float g[kMaxDof];
#pragma unroll
          for (int p = 0; p < kMaxDof; p++) g[p] = 0.f;
          float t = 0.f, q = 0.f, one = 0.f;
          if (i < nsub) {
            int c[3];
            float f[3], gv[3];
            sample_pos(s_ip, s_fp, i, S, S.iu, S.fu, rot, c, f);
            clamp_cell(c, a.bext);
            bool und;
            t = interp_sample<VT, IT, true>(Vcor, c, f, gv, und) - S.shift;
            n_undef += und;
            q = s_r[i];
            one = 1.f;
            v1.add(t);
            v2.add(t * t);
            v3.add(t * q);
            v4 += fabsf(t - q);
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
          for (int p = 0; p < kMaxDof; p++) s_aux[p * kThreads + tid] = g[p];
          s_aux[(kMaxDof + 0) * kThreads + tid] = one;
          s_aux[(kMaxDof + 1) * kThreads + tid] = t;
          s_aux[(kMaxDof + 2) * kThreads + tid] = q;
          __syncthreads();
          if (my_part < nparts) {
            const int lo = (my_part * kThreads) / nparts, hi = ((my_part + 1) * kThreads) / nparts;
            const float *ga = s_aux + ea * kThreads, *gb = s_aux + eb * kThreads;
            for (int s2 = lo; s2 < hi; s2++) gg += ga[s2] * gb[s2];
          }
          __syncthreads();
        }
        n_eval += 1;
        {
          KSum vv[3] = {v1, v2, v3};
          block_sum_comp<3>(vv, S);
        }
        const double S1 = S.red[0], S2 = S.red[1], S3 = S.red[2];
        __syncthreads();
        {
          float f1[1] = {v4};
          block_sum<1>(f1, S);
        }
        const double S4 = S.red[0];
        __syncthreads();
        // entry parts -> FP64 entries in S.red[128 ..]
        {
          __shared__ double ggpart[kThreads];
          ggpart[tid] = (my_part < nparts) ? (double)gg : 0.0;
          __syncthreads();
          if (tid < nent) {
            double s = 0.0;
            for (int pp = 0; pp < nparts; pp++) s += ggpart[pp * nent + tid];
            S.red[128 + tid] = s;
          }
          __syncthreads();
        }
        // assemble J'J and -J'e (FP64), objective value
        if (tid == 0) {
          const double *GG = &S.red[128];
          const double *Gsd = GG + ntri, *Gtd = GG + ntri + ndof, *Gqd = GG + ntri + 2 * ndof;
          const int n = nsub;
          const double mean = S1 / n;
          double ut[kMaxDof], jte[kMaxDof];
          double obj;
          double scale2 = 1.0;
          bool sub_mean = false, sub_t = false;
          switch (fcn) {
            case DVC_SAD:
            case DVC_SSD:
              for (int p = 0; p < ndof; p++) jte[p] = Gtd[p] - Gqd[p];
              obj = objective_from_sums(fcn, S1, S2, S3, S4, S.rsum2, n);
              break;
            case DVC_ZSSD:
              for (int p = 0; p < ndof; p++) jte[p] = Gtd[p] - mean * Gsd[p] - Gqd[p];
              sub_mean = true;
              obj = objective_from_sums(fcn, S1, S2, S3, S4, S.rsum2, n);
              break;
            case DVC_NSSD: {
              const double T = sqrt(S2);
              for (int p = 0; p < ndof; p++) {
                ut[p] = Gtd[p] / T;
                jte[p] = ((S3 / T) * ut[p] - Gqd[p]) / T;
              }
              sub_t = true;
              scale2 = 1.0 / (T * T);
              obj = 1.0 - S3 / T;
              break;
            }
            default: {
              const double sig = sqrt(S2 - n * mean * mean);
              const double rho = S3 / sig;
              for (int p = 0; p < ndof; p++) {
                ut[p] = (Gtd[p] - mean * Gsd[p]) / sig;
                jte[p] = (rho * ut[p] - Gqd[p]) / sig;
              }
              sub_mean = true;
              sub_t = true;
              scale2 = 1.0 / (sig * sig);
              obj = 0.5 * (1.0 - rho);
              break;
            }
          }
          int e = 0;
          for (int r = 0; r < ndof; r++)
            for (int c2 = r; c2 < ndof; c2++, e++) {
              double v = GG[e];
              if (sub_mean) v -= Gsd[r] * Gsd[c2] / n;
              if (sub_t) v -= ut[r] * ut[c2];
              v *= scale2;
              S.A[r * ndof + c2] = v;
              S.A[c2 * ndof + r] = v;
            }
          for (int p = 0; p < ndof; p++) S.b[p] = -jte[p];
          // stop rule of min_Lev_Mar
          int stop = 0;
          if (it > 0) {
            const double del_obj = fabs(obj - obj_old);
            const double *u = S.jump_prev_update;
            const double del_mag = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
            if ((del_obj < 0.000001) || (del_mag < 0.01)) stop = 1;
          }
          S.fail = stop ? 3 : 0;
          S.red[250] = obj;
        }
        __syncthreads();
        if (S.fail == 3) {
          it_done = it;
          break;
        }
        obj_old = S.red[250];
        // solve and update (warp 0)
        if (tid < 32) {
          warp_qr_solve(S, ndof);
          if (tid == 0) {
            for (int p = 0; p < ndof; p++) S.par[p] += S.x[p];
            for (int d = 0; d < 3; d++) S.jump_prev_update[d] = S.x[d];
          }
        }
        __syncthreads();
      }
      if (tid == 0) {
        S.fail = 0;
        if (a.gn_iters) a.gn_iters[S.n] = it_done;
        atomicAdd(a.counters + 1, (unsigned long long)it_done);
      }
      __syncthreads();
    }

    // ------------------------------------------------ final objective ---
    // obj_val_at(par_min) (Core/Search.cpp:187), explicit residuals over
    // stored values (the reference's own two-pass formulation)
    {
      if (tid == 0) {
        warp_matrices(S.par, ndof, S);
        for (int d = 0; d < 3; d++) split_d(__dsub_rn(S.par[d], S.seed[d]), S.iu[d], S.fu[d]);
      }
      __syncthreads();
      const bool rot = S.use_rot;
      range_check(s_ip, s_fp, nsub, S, rot);
      n_eval += 1;
      if (S.fail) goto point_done;
      KSum t1;
      for (int i = tid; i < nsub; i += kThreads) {
        int c[3];
        float f[3], g[3];
        sample_pos(s_ip, s_fp, i, S, S.iu, S.fu, rot, c, f);
        clamp_cell(c, a.bext);
        bool und;
        const float t = interp_sample<VT, IT, false>(Vcor, c, f, g, und) - S.shift;
        n_undef += und;
        s_aux[i] = t;
        t1.add(t);
      }
      {
        KSum v[1] = {t1};
        block_sum_comp<1>(v, S);
      }
      const float tm = (float)(S.red[0] / nsub);
      KSum c2, r2;
      for (int i = tid; i < nsub; i += kThreads) {
        const float t = s_aux[i];
        c2.add((t - tm) * (t - tm));
        r2.add(t * t);
      }
      {
        KSum v[2] = {c2, r2};
        block_sum_comp<2>(v, S);
      }
      const double tc2 = S.red[0], traw2 = S.red[1];
      const float inv_sig = (float)(1.0 / sqrt(tc2));
      const float inv_T = (float)(1.0 / sqrt(traw2));
      KSum e2, ea1;
      for (int i = tid; i < nsub; i += kThreads) {
        const float t = s_aux[i], q = s_r[i];
        float e;
        switch (fcn) {
          case DVC_SAD:
          case DVC_SSD: e = t - q; break;
          case DVC_ZSSD: e = (t - tm) - q; break;
          case DVC_NSSD: e = t * inv_T - q; break;
          default: e = (t - tm) * inv_sig - q; break;
        }
        e2.add(e * e);
        ea1.add(fabsf(e));
      }
      {
        KSum v[2] = {e2, ea1};
        block_sum_comp<2>(v, S);
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

  point_done:
    if (tid == 0) {
      const int n = S.n;
      if (S.fail) {
        a.status[n] = DVC_RANGE_FAIL;
        a.objmin[n] = 0.0;
        for (int p = 0; p < 12; p++) a.params[(size_t)n * 12 + p] = 0.0;
      } else {
        a.status[n] = DVC_POINT_GOOD;
        a.objmin[n] = S.obj;
        for (int p = 0; p < 12; p++) a.params[(size_t)n * 12 + p] = p < ndof ? S.par[p] : 0.0;
      }
      __threadfence();
      atomicExch(a.done + n, 1);
    }
    {
      unsigned long long u = n_undef;
      for (int o = 16; o; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
      if ((tid & 31) == 0 && u) atomicAdd(a.counters + 2, u);
      if (tid == 0) atomicAdd(a.counters + 0, n_eval);
    }
    __syncthreads();
  }
}

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
__global__ void interp_points_kernel(VolView<VT> V, int n, const double *pts, int itype,
                                     double *out, unsigned long long *undef) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  float f[3];
  const int o[3] = {V.ox, V.oy, V.oz};
  const int bext[3] = {V.bx, V.by, V.bz};
  for (int d = 0; d < 3; d++) split_d(__dsub_rn(pts[(size_t)i * 3 + d], (double)o[d]), c[d], f[d]);
  clamp_cell(c, bext);
  bool und;
  float g[3];
  float v;
  if (itype == 2) v = interp_sample<VT, 2, false>(V, c, f, g, und);
  else if (itype == 1) v = interp_sample<VT, 1, false>(V, c, f, g, und);
  else v = interp_sample<VT, 0, false>(V, c, f, g, und);
  out[i] = (double)v;
  if (und) atomicAdd(undef, 1ULL);
}

// ----------------------------------------------------- objective entry ---
// FP64 two-pass objective (Core/ObjectiveFunctions.cpp:24-263), one CTA.
__global__ void objective_kernel(int fcn, int n, const double *r, const double *t, double *obj,
                                 double *res) {
  __shared__ double red[kThreads];
  const int tid = threadIdx.x;
  auto bsum = [&](double v) -> double {
    red[tid] = v;
    __syncthreads();
    for (int s = kThreads / 2; s; s >>= 1) {
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
    for (int i = tid; i < n; i += kThreads) {
      a1 += r[i];
      a2 += t[i];
    }
    ar = bsum(a1) / n;
    at = bsum(a2) / n;
  }
  if (fcn == DVC_NSSD || fcn == DVC_ZNSSD) {
    double b1 = 0, b2 = 0;
    for (int i = tid; i < n; i += kThreads) {
      b1 += (r[i] - ar) * (r[i] - ar);
      b2 += (t[i] - at) * (t[i] - at);
    }
    sr = sqrt(bsum(b1));
    st = sqrt(bsum(b2));
  }
  double acc = 0;
  for (int i = tid; i < n; i += kThreads) {
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
  double *d_sphere = nullptr;
  // grow-only per-call workspace
  void *ws = nullptr;
  size_t ws_bytes = 0;
  size_t counters_off = 0;  // offset of the last call's counters in ws
  int num_sms = 0;
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
  return DVC_OK;
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

int engine_finish(dvc_engine *e) {
  engine_geometry(e);
  if (e->bext[0] > 1023 || e->bext[1] > 1023 || e->bext[2] > 1023)
    return set_error(DVC_E_ARG, "interpolation box larger than 1023 voxels per axis");
  if (e->p.subvol_geom == DVC_SPHERE) {
    std::vector<double> rel = sphere_offsets(e->subv_rad, e->n_sub, e->p.sphere_seed);
    CUDA_TRY(cudaMalloc(&e->d_sphere, rel.size() * sizeof(double)));
    CUDA_TRY(cudaMemcpy(e->d_sphere, rel.data(), rel.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  CUDA_TRY(cudaGetDevice(&e->device));
  CUDA_TRY(cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->device));
  return DVC_OK;
}

size_t state_bytes(int n_sub) {
  const size_t aux = (size_t)std::max(n_sub, kThreads * std::max(kMaxDof + 3, 3 * kMaxGridX));
  return (size_t)n_sub * 4 /*ip*/ + (size_t)n_sub * 12 /*fp*/ + (size_t)n_sub * 4 /*r*/ + aux * 4;
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

template <typename VT, int IT>
int launch_search(dvc_engine *e, SearchArgs &a, size_t smem_dyn, int grid, cudaStream_t st) {
  auto kern = search_kernel<VT, IT>;
  // static + dynamic shared memory may exceed the 48 KB default: opt in
  CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_dyn));
  kern<<<grid, kThreads, smem_dyn, st>>>(a);
  CUDA_TRY(cudaGetLastError());
  return DVC_OK;
}

template <typename VT, int IT>
int occupancy(size_t smem_dyn, int *blocks) {
  auto kern = search_kernel<VT, IT>;
  CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_dyn));
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, kern, kThreads, smem_dyn));
  return DVC_OK;
}

int dispatch_occupancy(int bpv, int it, size_t smem, int *blocks) {
  if (bpv == 1) {
    if (it == 2) return occupancy<uint8_t, 2>(smem, blocks);
    if (it == 1) return occupancy<uint8_t, 1>(smem, blocks);
    return occupancy<uint8_t, 0>(smem, blocks);
  }
  if (it == 2) return occupancy<uint16_t, 2>(smem, blocks);
  if (it == 1) return occupancy<uint16_t, 1>(smem, blocks);
  return occupancy<uint16_t, 0>(smem, blocks);
}

int dispatch_launch(int bpv, int it, dvc_engine *e, SearchArgs &a, size_t smem, int grid,
                    cudaStream_t st) {
  if (bpv == 1) {
    if (it == 2) return launch_search<uint8_t, 2>(e, a, smem, grid, st);
    if (it == 1) return launch_search<uint8_t, 1>(e, a, smem, grid, st);
    return launch_search<uint8_t, 0>(e, a, smem, grid, st);
  }
  if (it == 2) return launch_search<uint16_t, 2>(e, a, smem, grid, st);
  if (it == 1) return launch_search<uint16_t, 1>(e, a, smem, grid, st);
  return launch_search<uint16_t, 0>(e, a, smem, grid, st);
}

}  // namespace

// ================================================================== C API ===
extern "C" {

const char *dvc_gpu_version(void) { return "dvc-gb300 0.1 (sm_103a)"; }
const char *dvc_gpu_last_error(void) { return g_last_error.c_str(); }
int dvc_gpu_abi_version(void) { return DVC_ABI_VERSION; }

int dvc_gpu_create(dvc_engine **out, const dvc_params *p, const void *ref_vox, const void *cor_vox,
                   int big_endian) {
  if (!out || !ref_vox || !cor_vox) return set_error(DVC_E_ARG, "null argument");
  *out = nullptr;
  int rc = validate(p);
  if (rc) return rc;
  dvc_engine *e = new dvc_engine();
  e->p = *p;
  const size_t nvox = (size_t)p->vol_wide * p->vol_high * p->vol_tall;
  const size_t bytes = nvox * p->bytes_per_voxel;
  const size_t alloc = bytes + 64;  // tail padding for aligned row over-reads
  if (cudaMalloc(&e->ref, alloc) != cudaSuccess || cudaMalloc(&e->cor, alloc) != cudaSuccess) {
    dvc_gpu_destroy(e);
    return set_error(DVC_E_NOMEM, "volume allocation failed");
  }
  e->owns_volumes = true;
  if (cudaMemcpy(e->ref, ref_vox, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->cor, cor_vox, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset((char *)e->ref + bytes, 0, 64) != cudaSuccess ||
      cudaMemset((char *)e->cor + bytes, 0, 64) != cudaSuccess) {
    dvc_gpu_destroy(e);
    return set_error(DVC_E_CUDA, "volume upload failed");
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
}

int dvc_gpu_create_device(dvc_engine **out, const dvc_params *p, const void *ref_vox_dev,
                          const void *cor_vox_dev) {
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
}

void dvc_gpu_destroy(dvc_engine *e) {
  if (!e) return;
  if (e->owns_volumes) {
    if (e->ref) cudaFree(e->ref);
    if (e->cor) cudaFree(e->cor);
  }
  if (e->d_sphere) cudaFree(e->d_sphere);
  if (e->ws) cudaFree(e->ws);
  delete e;
}

int dvc_gpu_process_device(dvc_engine *e, int n_points, const double *points_dev, int n_process,
                           const int *order_dev, int n_neigh, const int *neigh_dev, int seed_mode,
                           const double *seeds_dev, int *status_dev, double *objmin_dev,
                           double *params_dev, int *gn_iters_dev, void *stream) {
  if (!e) return set_error(DVC_E_ARG, "null engine");
  if (n_points < 0 || n_process < 0 || n_process > n_points)
    return set_error(DVC_E_ARG, "n_process must be in 0..n_points");
  if (seed_mode < 0 || seed_mode > 2) return set_error(DVC_E_ARG, "bad seed_mode");
  if (seed_mode == DVC_SEED_NEIGHBOURS && n_neigh > 0 && !neigh_dev)
    return set_error(DVC_E_ARG, "neighbour list required");
  if (seed_mode == DVC_SEED_GIVEN && !seeds_dev) return set_error(DVC_E_ARG, "seeds required");
  if (n_points == 0) return DVC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const dvc_params &p = e->p;

  // launch shape: persistent grid, occupancy-limited
  const size_t sbytes = state_bytes(e->n_sub);
  const bool in_smem = sbytes <= 160 * 1024;
  const size_t smem_dyn = in_smem ? sbytes : 0;
  int blocks = 0;
  int rc = dispatch_occupancy(p.bytes_per_voxel, p.interp_type, smem_dyn, &blocks);
  if (rc) return rc;
  if (blocks < 1) return set_error(DVC_E_ARG, "search kernel does not fit on an SM");
  const int grid = std::max(1, std::min(blocks * e->num_sms, n_process));

  // workspace: done[n], rank[n], counter/error/counters, per-CTA state
  const size_t off_done = 0;
  const size_t off_rank = off_done + (size_t)n_points * 4;
  const size_t off_ctl = (off_rank + (size_t)n_points * 4 + 255) & ~(size_t)255;
  const size_t off_state = off_ctl + 256;
  const size_t state_per_cta = in_smem ? 0 : ((sbytes + 255) & ~(size_t)255);
  rc = ensure_ws(e, off_state + state_per_cta * grid);
  if (rc) return rc;
  char *ws = (char *)e->ws;
  int *done = (int *)(ws + off_done);
  int *rank = (int *)(ws + off_rank);
  int *ctl = (int *)(ws + off_ctl);
  unsigned long long *counters = (unsigned long long *)(ws + off_ctl + 64);
  CUDA_TRY(cudaMemsetAsync(ws + off_ctl, 0, 256, st));
  e->counters_off = off_ctl + 64;
  {
    const int T = 256;
    const int G = (n_points + T - 1) / T;
    init_outputs_kernel<<<G, T, 0, st>>>(n_points, status_dev, objmin_dev, params_dev, gn_iters_dev,
                                         done, rank);
    if (n_process > 0) rank_kernel<<<(n_process + T - 1) / T, T, 0, st>>>(n_process, order_dev, rank, n_points);
    CUDA_TRY(cudaGetLastError());
  }
  if (n_process == 0) return DVC_OK;

  SearchArgs a{};
  a.ref = e->ref;
  a.cor = e->cor;
  a.nx = p.vol_wide;
  a.ny = p.vol_high;
  a.nz = p.vol_tall;
  a.geom = p.subvol_geom;
  a.ndof = p.num_srch_dof;
  a.objfcn = p.obj_function;
  a.itype = p.interp_type;
  a.n_sub = e->n_sub;
  a.cube_n = e->cube_n;
  a.subv_rad = e->subv_rad;
  for (int d = 0; d < 3; d++) {
    a.aspect[d] = p.subvol_aspect[d];
    a.nom_mn[d] = e->nom_mn[d];
    a.nom_mx[d] = e->nom_mx[d];
    a.nom_cen[d] = e->nom_cen[d];
    a.bext[d] = e->bext[d];
    a.rigid[d] = p.rigid_trans[d];
  }
  a.do_grid = p.basin_radius != 0.0;
  if (a.do_grid) {
    const double displ_max = p.disp_max;
    a.num_inc = (int)(displ_max / p.basin_radius);
    a.inc = displ_max / a.num_inc;
  }
  a.sphere_rel = e->d_sphere;
  a.n_points = n_points;
  a.n_process = n_process;
  a.n_neigh = (seed_mode == DVC_SEED_NEIGHBOURS) ? n_neigh : 0;
  a.seed_mode = seed_mode;
  a.pts = points_dev;
  a.order = order_dev;
  a.rank = rank;
  a.neigh = neigh_dev;
  a.seeds = seeds_dev;
  a.status = status_dev;
  a.objmin = objmin_dev;
  a.params = params_dev;
  a.gn_iters = gn_iters_dev;
  a.work_counter = ctl;
  a.error_flag = ctl + 1;
  a.done = done;
  a.counters = counters;
  a.state_in_smem = in_smem;
  a.scratch = in_smem ? nullptr : (float *)(ws + off_state);
  a.scratch_floats_per_cta = (long long)(state_per_cta / 4);
  return dispatch_launch(p.bytes_per_voxel, p.interp_type, e, a, smem_dyn, grid, st);
}

int dvc_gpu_process(dvc_engine *e, int n_points, const double *points, int n_process,
                    const int *order, int n_neigh, const int *neigh, int seed_mode,
                    const double *seeds, int *status, double *objmin, double *params, int *gn_iters,
                    dvc_stats *stats) {
  if (!e || !points || !status || !objmin || !params) return set_error(DVC_E_ARG, "null argument");
  if (n_points < 0 || n_process < 0 || n_process > n_points)
    return set_error(DVC_E_ARG, "n_process must be in 0..n_points");
  if (n_process > 0 && !order) return set_error(DVC_E_ARG, "order required");
  if (seed_mode == DVC_SEED_NEIGHBOURS && n_neigh > 0 && !neigh)
    return set_error(DVC_E_ARG, "neighbour list required");
  if (seed_mode == DVC_SEED_GIVEN && !seeds) return set_error(DVC_E_ARG, "seeds required");
  for (int i = 0; i < n_process; i++)
    if (order[i] < 0 || order[i] >= n_points) return set_error(DVC_E_ARG, "order index out of range");
  if (seed_mode == DVC_SEED_NEIGHBOURS && neigh)
    for (size_t i = 0; i < (size_t)n_points * n_neigh; i++)
      if (neigh[i] < 0 || neigh[i] >= n_points) return set_error(DVC_E_ARG, "neighbour index out of range");
  auto t0 = std::chrono::steady_clock::now();
  const size_t N = (size_t)n_points;
  double *d_pts = nullptr, *d_seeds = nullptr, *d_obj = nullptr, *d_par = nullptr;
  int *d_order = nullptr, *d_neigh = nullptr, *d_status = nullptr, *d_its = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int rc = DVC_OK;
  auto cleanup = [&]() {
    cudaFree(d_pts); cudaFree(d_seeds); cudaFree(d_obj); cudaFree(d_par);
    cudaFree(d_order); cudaFree(d_neigh); cudaFree(d_status); cudaFree(d_its);
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
  if (seed_mode == DVC_SEED_GIVEN) {
    TRYC(cudaMalloc(&d_seeds, N * 3 * sizeof(double)));
    TRYC(cudaMemcpy(d_seeds, seeds, N * 3 * sizeof(double), cudaMemcpyHostToDevice));
  }
  TRYC(cudaEventCreate(&ev0));
  TRYC(cudaEventCreate(&ev1));
  TRYC(cudaEventRecord(ev0, 0));
  rc = dvc_gpu_process_device(e, n_points, d_pts, n_process, d_order, n_neigh, d_neigh, seed_mode,
                              d_seeds, d_status, d_obj, d_par, d_its, nullptr);
  if (rc) {
    cleanup();
    return rc;
  }
  TRYC(cudaEventRecord(ev1, 0));
  TRYC(cudaEventSynchronize(ev1));
  TRYC(cudaGetLastError());
  int ctl[2] = {0, 0};
  unsigned long long counters[3] = {0, 0, 0};
  if (n_process > 0) {
    const size_t off_ctl = ((size_t)n_points * 8 + 255) & ~(size_t)255;
    TRYC(cudaMemcpy(ctl, (char *)e->ws + off_ctl, sizeof ctl, cudaMemcpyDeviceToHost));
    TRYC(cudaMemcpy(counters, (char *)e->ws + off_ctl + 64, sizeof counters, cudaMemcpyDeviceToHost));
  }
  TRYC(cudaMemcpy(status, d_status, N * sizeof(int), cudaMemcpyDeviceToHost));
  TRYC(cudaMemcpy(objmin, d_obj, N * sizeof(double), cudaMemcpyDeviceToHost));
  TRYC(cudaMemcpy(params, d_par, N * 12 * sizeof(double), cudaMemcpyDeviceToHost));
  if (gn_iters) TRYC(cudaMemcpy(gn_iters, d_its, N * sizeof(int), cudaMemcpyDeviceToHost));
  float kms = 0.f;
  cudaEventElapsedTime(&kms, ev0, ev1);
  cleanup();
#undef TRYC
  if (ctl[1] != 0) return set_error(ctl[1], "a bounded dependency wait gave up; points left unsearched");
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

int dvc_gpu_last_counters(dvc_engine *e, long long out[3]) {
  if (!e || !out) return set_error(DVC_E_ARG, "null argument");
  out[0] = out[1] = out[2] = 0;
  if (!e->ws) return DVC_OK;
  unsigned long long c[3];
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(c, (char *)e->ws + e->counters_off, sizeof c, cudaMemcpyDeviceToHost));
  for (int k = 0; k < 3; k++) out[k] = (long long)c[k];
  return DVC_OK;
}

int dvc_gpu_interpolate(dvc_engine *e, int volume, const double center[3], int n, const double *pts,
                        int interp_type, double *out) {
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
  const int T = 256, G = (n + T - 1) / T;
  if (e->p.bytes_per_voxel == 1) {
    VolView<uint8_t> V{(const uint8_t *)vp, vol[0], vol[1], vol[2], o[0], o[1], o[2],
                       e->bext[0], e->bext[1], e->bext[2], checked};
    interp_points_kernel<uint8_t><<<G, T>>>(V, n, d_pts, interp_type, d_out, d_und);
  } else {
    VolView<uint16_t> V{(const uint16_t *)vp, vol[0], vol[1], vol[2], o[0], o[1], o[2],
                        e->bext[0], e->bext[1], e->bext[2], checked};
    interp_points_kernel<uint16_t><<<G, T>>>(V, n, d_pts, interp_type, d_out, d_und);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpy(out, d_out, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(d_pts);
  cudaFree(d_out);
  cudaFree(d_und);
  return DVC_OK;
}

int dvc_gpu_objective(int obj_function, int n, const double *ref, const double *tar, double *obj,
                      double *residual) {
  if (obj_function < 0 || obj_function > 4) return set_error(DVC_E_ARG, "bad obj_function");
  if (n <= 0 || !ref || !tar || !obj) return set_error(DVC_E_ARG, "bad arguments");
  double *d_r = nullptr, *d_t = nullptr, *d_o = nullptr, *d_res = nullptr;
  CUDA_TRY(cudaMalloc(&d_r, (size_t)n * sizeof(double)));
  CUDA_TRY(cudaMalloc(&d_t, (size_t)n * sizeof(double)));
  CUDA_TRY(cudaMalloc(&d_o, sizeof(double)));
  if (residual) CUDA_TRY(cudaMalloc(&d_res, (size_t)n * sizeof(double)));
  CUDA_TRY(cudaMemcpy(d_r, ref, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(d_t, tar, (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  objective_kernel<<<1, kThreads>>>(obj_function, n, d_r, d_t, d_o, d_res);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpy(obj, d_o, sizeof(double), cudaMemcpyDeviceToHost));
  if (residual) CUDA_TRY(cudaMemcpy(residual, d_res, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(d_r);
  cudaFree(d_t);
  cudaFree(d_o);
  cudaFree(d_res);
  return DVC_OK;
}

}  // extern "C"
