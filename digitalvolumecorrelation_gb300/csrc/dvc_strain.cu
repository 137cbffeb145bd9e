// dvc_strain.cu — strain-window least-squares fit on the GPU (FP64).
//
// Replaces the per-point loop of the reference `strain` executable
// (Core/strain.cpp:402-591): for each point, up to `ndp` neighbours from its
// sorted neighbour list that converged (status 0) with objmin <= threshold,
// coordinates scaled by 1/|p| (distance of the point from the origin), a
// 10-term quadratic polynomial fitted to u, v and w through the normal
// equations solved by Householder QR with complete pivoting
// (fullPivHouseholderQr in the reference), the deformation gradient at the
// point, the engineering and Lagrangian strain tensors and their principal
// values (sorted descending; planar special cases as :556-568).
// One thread per point; every quantity in double precision.
#include <cuda_runtime.h>

#include <string>

#include "../../include/dvc_gpu.h"
#include "dvc_internal.h"

namespace {

constexpr int kNmp = 10;

// A x = b for a 10x10 system (row-major, in place), complete pivoting, the
// trailing unknowns beyond the numerical rank set to zero.
__device__ void qr_solve_full(double *A, double *b, double *x) {
  const int n = kNmp;
  int perm[kNmp];
  double diag[kNmp];
  for (int j = 0; j < n; j++) perm[j] = j;
  for (int k = 0; k < n; k++) {
    int pc = k, pr = k;
    double best = -1.0;
    for (int j = k; j < n; j++)
      for (int i = k; i < n; i++)
        if (fabs(A[i * n + j]) > best) {
          best = fabs(A[i * n + j]);
          pc = j;
          pr = i;
        }
    if (pc != k) {
      for (int i = 0; i < n; i++) {
        const double t = A[i * n + k];
        A[i * n + k] = A[i * n + pc];
        A[i * n + pc] = t;
      }
      const int t = perm[k];
      perm[k] = perm[pc];
      perm[pc] = t;
    }
    if (pr != k) {
      for (int j = 0; j < n; j++) {
        const double t = A[k * n + j];
        A[k * n + j] = A[pr * n + j];
        A[pr * n + j] = t;
      }
      const double t = b[k];
      b[k] = b[pr];
      b[pr] = t;
    }
    double norm = 0.0;
    for (int i = k; i < n; i++) norm += A[i * n + k] * A[i * n + k];
    norm = sqrt(norm);
    if (norm == 0.0) {
      diag[k] = 0.0;
      continue;
    }
    const double alpha = A[k * n + k] > 0 ? -norm : norm;
    double v[kNmp];
    double vv = 0.0;
    for (int i = k; i < n; i++) {
      v[i - k] = A[i * n + k] - (i == k ? alpha : 0.0);
      vv += v[i - k] * v[i - k];
    }
    if (vv == 0.0) {
      diag[k] = A[k * n + k];
      continue;
    }
    for (int j = k; j < n; j++) {
      double s = 0.0;
      for (int i = k; i < n; i++) s += v[i - k] * A[i * n + j];
      s = 2.0 * s / vv;
      for (int i = k; i < n; i++) A[i * n + j] -= s * v[i - k];
    }
    double s = 0.0;
    for (int i = k; i < n; i++) s += v[i - k] * b[i];
    s = 2.0 * s / vv;
    for (int i = k; i < n; i++) b[i] -= s * v[i - k];
    diag[k] = A[k * n + k];
  }
  int rank = 0;
  const double thr = 2.220446049250313e-16 * (double)n * fabs(diag[0]);
  for (int k = 0; k < n; k++) {
    if (fabs(diag[k]) > thr) rank = k + 1;
    else break;
  }
  double y[kNmp];
  for (int k = 0; k < n; k++) y[k] = 0.0;
  for (int k = rank - 1; k >= 0; k--) {
    double s = b[k];
    for (int j = k + 1; j < rank; j++) s -= A[k * n + j] * y[j];
    y[k] = s / A[k * n + k];
  }
  for (int k = 0; k < n; k++) x[perm[k]] = y[k];
}

// principal values of a symmetric 3x3 matrix by cyclic Jacobi rotations
__device__ void sym3_eigenvalues(const double ST[9], double lam[3]) {
  double s[9];
  for (int i = 0; i < 9; i++) s[i] = ST[i];
  for (int sweep = 0; sweep < 64; sweep++) {
    const double off = s[1] * s[1] + s[2] * s[2] + s[5] * s[5];
    if (off == 0.0) break;
    for (int p = 0; p < 3; p++)
      for (int q = p + 1; q < 3; q++) {
        const double apq = s[p * 3 + q];
        if (apq == 0.0) continue;
        const double theta = (s[q * 3 + q] - s[p * 3 + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 3; k++) {
          const double skp = s[k * 3 + p], skq = s[k * 3 + q];
          s[k * 3 + p] = c * skp - sn * skq;
          s[k * 3 + q] = sn * skp + c * skq;
        }
        for (int k = 0; k < 3; k++) {
          const double spk = s[p * 3 + k], sqk = s[q * 3 + k];
          s[p * 3 + k] = c * spk - sn * sqk;
          s[q * 3 + k] = sn * spk + c * sqk;
        }
      }
  }
  lam[0] = s[0];
  lam[1] = s[4];
  lam[2] = s[8];
  // sort descending (Core/strain.cpp:555-556)
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2 - i; j++)
      if (lam[j] < lam[j + 1]) {
        const double t = lam[j];
        lam[j] = lam[j + 1];
        lam[j + 1] = t;
      }
}

__device__ __forceinline__ double dist3(const double *a, const double *b) {
  const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return sqrt(dx * dx + dy * dy + dz * dz);
}

__global__ void strain_kernel(int n, const double *__restrict__ pts, const int *__restrict__ status,
                              const double *__restrict__ objmin, const double *__restrict__ disp,
                              int n_neigh, const int *__restrict__ neigh, int ndp, double objt,
                              int refill, int planar, double *u_fit, int *pts_in_sw,
                              double *sw_radius, double *e_strain, double *l_strain,
                              double *dgrad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool yz_only = planar & 1, zx_only = planar & 2, xy_only = planar & 4;
  const int *nb = neigh + (size_t)i * n_neigh;
  const double origin[3] = {0.0, 0.0, 0.0};
  const double distance = dist3(pts + (size_t)i * 3, origin);
  const double scale = 1.0 / distance;
  const double base[3] = {scale * pts[(size_t)i * 3], scale * pts[(size_t)i * 3 + 1],
                          scale * pts[(size_t)i * 3 + 2]};
  // normal equations X'X and X'd accumulated over the window's good points
  double XtX[kNmp * kNmp], Xtd[3][kNmp];
  for (int k = 0; k < kNmp * kNmp; k++) XtX[k] = 0.0;
  for (int c = 0; c < 3; c++)
    for (int k = 0; k < kNmp; k++) Xtd[c][k] = 0.0;
  int ngp = 0;
  double last[3] = {0.0, 0.0, 0.0};
  int indx = 0, np = 0;
  const int limit = refill ? n_neigh : min(ndp, n_neigh);
  while (indx < limit && (!refill || np < ndp)) {
    const int m = nb[indx];
    indx++;
    if (m < 0 || m >= n) continue;
    if (!(status[m] == 0 && objmin[m] <= objt)) continue;
    np++;
    const double q[3] = {scale * pts[(size_t)m * 3], scale * pts[(size_t)m * 3 + 1],
                         scale * pts[(size_t)m * 3 + 2]};
    double dv[3] = {scale * disp[(size_t)m * 3], scale * disp[(size_t)m * 3 + 1],
                    scale * disp[(size_t)m * 3 + 2]};
    double X[kNmp] = {1.0, q[0], q[1], q[2], q[0] * q[0], q[1] * q[1], q[2] * q[2],
                      q[0] * q[1], q[1] * q[2], q[0] * q[2]};
    if (yz_only) {
      X[1] = X[4] = X[7] = X[9] = 0.0;
      dv[0] = 0.0;
    }
    if (zx_only) {
      X[2] = X[5] = X[7] = X[8] = 0.0;
      dv[1] = 0.0;
    }
    if (xy_only) {
      X[3] = X[6] = X[8] = X[9] = 0.0;
      dv[2] = 0.0;
    }
    for (int a = 0; a < kNmp; a++) {
      for (int b = 0; b < kNmp; b++) XtX[a * kNmp + b] += X[a] * X[b];
      for (int c = 0; c < 3; c++) Xtd[c][a] += X[a] * dv[c];
    }
    last[0] = q[0];
    last[1] = q[1];
    last[2] = q[2];
    ngp++;
  }
  pts_in_sw[i] = ngp;
  sw_radius[i] = ngp == 0 ? 0.0 : distance * dist3(base, last);
  double DG[9], displ[3];
  for (int c = 0; c < 3; c++) {
    double A[kNmp * kNmp], b[kNmp], par[kNmp];
    for (int k = 0; k < kNmp * kNmp; k++) A[k] = XtX[k];
    for (int k = 0; k < kNmp; k++) b[k] = Xtd[c][k];
    qr_solve_full(A, b, par);
    DG[c * 3 + 0] = par[1] + 2 * par[4] * base[0] + par[7] * base[1] + par[9] * base[2];
    DG[c * 3 + 1] = par[2] + 2 * par[5] * base[1] + par[7] * base[0] + par[8] * base[2];
    DG[c * 3 + 2] = par[3] + 2 * par[6] * base[2] + par[8] * base[1] + par[9] * base[0];
    displ[c] = distance * (par[0] + par[1] * base[0] + par[2] * base[1] + par[3] * base[2] +
                           par[4] * base[0] * base[0] + par[5] * base[1] * base[1] +
                           par[6] * base[2] * base[2] + par[7] * base[0] * base[1] +
                           par[8] * base[1] * base[2] + par[9] * base[0] * base[2]);
  }
  for (int c = 0; c < 3; c++) u_fit[(size_t)i * 3 + c] = displ[c];
  for (int k = 0; k < 9; k++) dgrad[(size_t)i * 9 + k] = DG[k];
  for (int which = 0; which < 2; which++) {
    double ST[9];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        double v = 0.5 * (DG[a * 3 + b] + DG[b * 3 + a]);
        if (which == 1) {
          double s = 0.0;
          for (int k = 0; k < 3; k++) s += DG[k * 3 + a] * DG[k * 3 + b];
          v = 0.5 * (DG[a * 3 + b] + DG[b * 3 + a] + s);
        }
        ST[a * 3 + b] = v;
      }
    double lam[3];
    sym3_eigenvalues(ST, lam);
    if (xy_only || yz_only || zx_only) {
      if (lam[0] == 0.0) {
        lam[0] = lam[1];
        lam[1] = lam[2];
      }
      if (lam[1] == 0.0) lam[1] = lam[2];
      lam[2] = 0.0;
    }
    double *o = (which == 0 ? e_strain : l_strain) + (size_t)i * 9;
    o[0] = ST[0];
    o[1] = ST[4];
    o[2] = ST[8];
    o[3] = ST[1];
    o[4] = ST[5];
    o[5] = ST[2];
    o[6] = lam[0];
    o[7] = lam[1];
    o[8] = lam[2];
  }
}

}  // namespace

extern "C" int dvc_gpu_strain(int n, const double *pts, const int *status, const double *objmin,
                              const double *disp, int n_neigh, const int *neigh, int ndp,
                              double objt, int refill, int planar, double *u_fit, int *pts_in_sw,
                              double *sw_radius, double *e_strain, double *l_strain,
                              double *dgrad) try {
  if (n < 0 || n_neigh < 0 || ndp < 0) return dvc_internal_set_error(DVC_E_ARG, "bad sizes");
  if (n == 0) return DVC_OK;
  if (!pts || !status || !objmin || !disp || !neigh || !u_fit || !pts_in_sw || !sw_radius ||
      !e_strain || !l_strain || !dgrad)
    return dvc_internal_set_error(DVC_E_ARG, "null argument");
  const size_t N = (size_t)n;
  char *buf = nullptr;
  // inputs: pts 24N, status 4N, objmin 8N, disp 24N, neigh 4N*nn;
  // outputs: ufit 24N, pisw 4N, swr 8N, e 72N, l 72N, dg 72N
  const size_t sz[] = {24 * N, 4 * N, 8 * N, 24 * N, 4 * N * (size_t)n_neigh,
                       24 * N, 4 * N, 8 * N, 72 * N, 72 * N, 72 * N};
  size_t off[12];
  off[0] = 0;
  for (int k = 0; k < 11; k++) off[k + 1] = off[k] + ((sz[k] + 255) & ~(size_t)255);
  if (cudaMalloc(&buf, off[11]) != cudaSuccess)
    return dvc_internal_set_error(DVC_E_NOMEM, "strain buffers");
  const void *in[5] = {pts, status, objmin, disp, neigh};
  cudaError_t err = cudaSuccess;
  for (int k = 0; k < 5 && err == cudaSuccess; k++)
    err = cudaMemcpy(buf + off[k], in[k], sz[k], cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    const int T = 128;
    strain_kernel<<<(n + T - 1) / T, T>>>(
        n, (const double *)(buf + off[0]), (const int *)(buf + off[1]),
        (const double *)(buf + off[2]), (const double *)(buf + off[3]), n_neigh,
        (const int *)(buf + off[4]), ndp, objt, refill, planar, (double *)(buf + off[5]),
        (int *)(buf + off[6]), (double *)(buf + off[7]), (double *)(buf + off[8]),
        (double *)(buf + off[9]), (double *)(buf + off[10]));
    err = cudaGetLastError();
  }
  void *out[6] = {u_fit, pts_in_sw, sw_radius, e_strain, l_strain, dgrad};
  for (int k = 0; k < 6 && err == cudaSuccess; k++)
    err = cudaMemcpy(out[k], buf + off[5 + k], sz[5 + k], cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (err != cudaSuccess) return dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(err));
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}
