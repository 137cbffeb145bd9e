// dvc_synth.cu — synthetic speckle volumes on the device (benchmark and test
// data; no reference counterpart).
//
// value(x) = background + sum_b amp_b exp(-|X(x) - c_b|^2 / (2 sigma_b^2)) + noise
// where X(x) is the reference position of voxel x under the deformation
// (X + u(X) = x; affine: solved, sinusoid and bump field: fixed-point
// iteration, their gradients being well below 1; two affine pieces split by
// the plane X_x = split: piece 1's solution where it lies left of the plane,
// else piece 2's), blobs contribute within 4 sigma, noise ~ N(0, noise_sigma)
// from a counter-based hash of (seed, voxel index), then the value is rounded
// and clipped to [0, vmax]. Blobs are binned on the host by their deformed
// centre so each voxel visits only the blobs of its 27 neighbouring bins.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/dvc_gpu.h"
#include "dvc_internal.h"

namespace {

constexpr int kBin = 16;
constexpr int kMaxBumps = 32;

struct SynthArgs {
  void *vol;
  int nx, ny, nz, bpv;
  int gx, gy, gz;             // bin grid
  const float4 *blobs;        // x y z 1/(2 sigma^2), sorted by bin
  const float2 *amp_r2;       // amplitude, (4 sigma)^2; split field: negative amplitude
                              // for the copy binned by piece 2
  const int *bin_start;       // gx*gy*gz + 1
  int deform;
  float Ainv[9], t[3], c[3];  // affine: X = c + Ainv (x - t - c)
  float amp, len;             // sinusoid
  // bump field: affine t + E (X - c) plus sum_k a_k exp(-|X - p_k|^2 / (2 s_k^2))
  float E[9];
  int nbump;
  float bump[kMaxBumps][7];   // p (3), 1/(2 s^2), a (3)
  // split field: piece 2's X = c2 + Ainv2 (x - t2 - c2), the plane X_x = split
  float Ainv2[9], t2[3], c2[3], split;
  // bending and jump: kappa, xc, h, J, z0, 1/w
  float bend[6];
  float background, noise_sigma, vmax;
  unsigned long long seed;
};

__device__ __forceinline__ unsigned long long splitmix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__global__ void synth_kernel(SynthArgs a) {
  const long long nvox = (long long)a.nx * a.ny * a.nz;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < nvox;
       idx += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(idx % a.nx);
    const int y = (int)((idx / a.nx) % a.ny);
    const int z = (int)(idx / ((long long)a.nx * a.ny));
    float X[3] = {(float)x, (float)y, (float)z};
    bool piece2 = false;
    if (a.deform == 1 || a.deform == 4) {
      const float x0[3] = {X[0], X[1], X[2]};
      const float r[3] = {X[0] - a.t[0] - a.c[0], X[1] - a.t[1] - a.c[1], X[2] - a.t[2] - a.c[2]};
      for (int i = 0; i < 3; i++)
        X[i] = a.c[i] + a.Ainv[i * 3 + 0] * r[0] + a.Ainv[i * 3 + 1] * r[1] + a.Ainv[i * 3 + 2] * r[2];
      if (a.deform == 4 && !(X[0] < a.split)) {
        piece2 = true;
        const float q[3] = {x0[0] - a.t2[0] - a.c2[0], x0[1] - a.t2[1] - a.c2[1], x0[2] - a.t2[2] - a.c2[2]};
        for (int i = 0; i < 3; i++)
          X[i] = a.c2[i] + a.Ainv2[i * 3 + 0] * q[0] + a.Ainv2[i * 3 + 1] * q[1] + a.Ainv2[i * 3 + 2] * q[2];
      }
    } else if (a.deform == 3) {
      const float x0[3] = {X[0], X[1], X[2]};
      for (int it = 0; it < 12; it++) {
        float u[3];
        const float r[3] = {X[0] - a.c[0], X[1] - a.c[1], X[2] - a.c[2]};
        for (int i = 0; i < 3; i++) u[i] = a.t[i] + a.E[i * 3] * r[0] + a.E[i * 3 + 1] * r[1] + a.E[i * 3 + 2] * r[2];
        for (int k = 0; k < a.nbump; k++) {
          const float dx = X[0] - a.bump[k][0], dy = X[1] - a.bump[k][1], dz = X[2] - a.bump[k][2];
          const float g = __expf(-(dx * dx + dy * dy + dz * dz) * a.bump[k][3]);
          u[0] += a.bump[k][4] * g;
          u[1] += a.bump[k][5] * g;
          u[2] += a.bump[k][6] * g;
        }
        X[0] = x0[0] - u[0];
        X[1] = x0[1] - u[1];
        X[2] = x0[2] - u[2];
      }
    } else if (a.deform == 5) {
      const float x0[3] = {X[0], X[1], X[2]};
      for (int it = 0; it < 20; it++) {
        const float dx = X[0] - a.bend[1];
        const float ux = 0.5f * a.bend[3] * tanhf((X[2] - a.bend[4]) * a.bend[5]);
        const float uz = 0.5f * a.bend[0] * (dx * dx - a.bend[2]);
        X[0] = x0[0] - ux;
        X[2] = x0[2] - uz;
      }
    } else if (a.deform == 2) {
      const float x0[3] = {X[0], X[1], X[2]};
      const float w = 6.283185307179586f / a.len;
      for (int it = 0; it < 30; it++) {
        const float u0 = a.amp * sinf(w * X[1]), u1 = a.amp * sinf(w * X[2]), u2 = a.amp * sinf(w * X[0]);
        X[0] = x0[0] - u0;
        X[1] = x0[1] - u1;
        X[2] = x0[2] - u2;
      }
    }
    float v = a.background;
    const int bx = x / kBin, by = y / kBin, bz = z / kBin;
    for (int dz = -1; dz <= 1; dz++) {
      const int cz = bz + dz;
      if (cz < 0 || cz >= a.gz) continue;
      for (int dy = -1; dy <= 1; dy++) {
        const int cy = by + dy;
        if (cy < 0 || cy >= a.gy) continue;
        for (int dx = -1; dx <= 1; dx++) {
          const int cx = bx + dx;
          if (cx < 0 || cx >= a.gx) continue;
          const int b = (cz * a.gy + cy) * a.gx + cx;
          for (int k = a.bin_start[b]; k < a.bin_start[b + 1]; k++) {
            const float4 bl = a.blobs[k];
            const float ex = X[0] - bl.x, ey = X[1] - bl.y, ez = X[2] - bl.z;
            const float d2 = ex * ex + ey * ey + ez * ez;
            const float2 ar = a.amp_r2[k];
            if (a.deform == 4 && ((ar.x < 0.f) != piece2)) continue;  // the other piece's copy
            if (d2 <= ar.y) v += (a.deform == 4 ? fabsf(ar.x) : ar.x) * __expf(-d2 * bl.w);
          }
        }
      }
    }
    if (a.noise_sigma > 0.f) {
      const unsigned long long h = splitmix(a.seed ^ splitmix((unsigned long long)idx));
      const float u1 = ((h >> 40) + 1.0f) * (1.0f / 16777217.0f);
      const float u2 = ((h >> 16) & 0xFFFFFF) * (1.0f / 16777216.0f);
      v += a.noise_sigma * sqrtf(-2.f * logf(u1)) * cosf(6.283185307179586f * u2);
    }
    v = fminf(fmaxf(rintf(v), 0.f), a.vmax);
    if (a.bpv == 1)
      reinterpret_cast<unsigned char *>(a.vol)[idx] = (unsigned char)v;
    else
      reinterpret_cast<unsigned short *>(a.vol)[idx] = (unsigned short)v;
  }
}

}  // namespace

extern "C" int dvc_gpu_synth_volume(void *vol_dev, int nx, int ny, int nz, int bytes_per_voxel,
                                    int n_blobs, const float *blobs, int deform,
                                    const double *coef, float background, float noise_sigma,
                                    unsigned long long noise_seed, float vmax, void *stream) try {
  if (!vol_dev || nx <= 0 || ny <= 0 || nz <= 0 || (bytes_per_voxel != 1 && bytes_per_voxel != 2) ||
      n_blobs < 0 || (n_blobs > 0 && !blobs) || deform < 0 || deform > 5 || (deform && !coef))
    return dvc_internal_set_error(DVC_E_ARG, "bad synth arguments");
  SynthArgs a{};
  a.vol = vol_dev;
  a.nx = nx;
  a.ny = ny;
  a.nz = nz;
  a.bpv = bytes_per_voxel;
  a.gx = (nx + kBin - 1) / kBin;
  a.gy = (ny + kBin - 1) / kBin;
  a.gz = (nz + kBin - 1) / kBin;
  a.deform = deform;
  a.background = background;
  a.noise_sigma = noise_sigma;
  a.vmax = vmax;
  a.seed = noise_seed;
  // deformed blob centres and bins (host)
  // inverse of I + E (E row-major)
  auto inverse = [](const double *E, float out[9]) {
    const double A[9] = {1 + E[0], E[1], E[2], E[3], 1 + E[4], E[5], E[6], E[7], 1 + E[8]};
    const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                       A[2] * (A[3] * A[7] - A[4] * A[6]);
    const double inv[9] = {(A[4] * A[8] - A[5] * A[7]) / det, (A[2] * A[7] - A[1] * A[8]) / det,
                           (A[1] * A[5] - A[2] * A[4]) / det, (A[5] * A[6] - A[3] * A[8]) / det,
                           (A[0] * A[8] - A[2] * A[6]) / det, (A[2] * A[3] - A[0] * A[5]) / det,
                           (A[3] * A[7] - A[4] * A[6]) / det, (A[1] * A[6] - A[0] * A[7]) / det,
                           (A[0] * A[4] - A[1] * A[3]) / det};
    for (int i = 0; i < 9; i++) out[i] = (float)inv[i];
  };
  if (deform == 1 || deform == 4) {
    // coef: t (3), E (9), c (3); split field: then piece 2's t, E, c and the plane
    inverse(coef + 3, a.Ainv);
    for (int i = 0; i < 3; i++) {
      a.t[i] = (float)coef[i];
      a.c[i] = (float)coef[12 + i];
    }
    if (deform == 4) {
      inverse(coef + 18, a.Ainv2);
      for (int i = 0; i < 3; i++) {
        a.t2[i] = (float)coef[15 + i];
        a.c2[i] = (float)coef[27 + i];
      }
      a.split = (float)coef[30];
      for (int k = 0; k < n_blobs; k++)
        if (!(blobs[(size_t)k * 5 + 4] >= 0.f))
          return dvc_internal_set_error(DVC_E_ARG, "a split field needs blob amplitudes >= 0");
    }
  } else if (deform == 2) {
    a.amp = (float)coef[0];
    a.len = (float)coef[1];
  } else if (deform == 5) {
    // coef: kappa, xc, h, J, z0, w
    if (!(coef[5] > 0.0)) return dvc_internal_set_error(DVC_E_ARG, "jump width must be > 0");
    for (int i = 0; i < 5; i++) a.bend[i] = (float)coef[i];
    a.bend[5] = (float)(1.0 / coef[5]);
  } else if (deform == 3) {
    // coef: t (3), E (9), c (3), n, then n x (p (3), s, a (3))
    const int nb = (int)coef[15];
    if (nb < 0 || nb > kMaxBumps) return dvc_internal_set_error(DVC_E_ARG, "at most 32 bumps");
    for (int i = 0; i < 3; i++) {
      a.t[i] = (float)coef[i];
      a.c[i] = (float)coef[12 + i];
    }
    for (int i = 0; i < 9; i++) a.E[i] = (float)coef[3 + i];
    a.nbump = nb;
    for (int k = 0; k < nb; k++) {
      const double *b = coef + 16 + 7 * k;
      a.bump[k][0] = (float)b[0];
      a.bump[k][1] = (float)b[1];
      a.bump[k][2] = (float)b[2];
      a.bump[k][3] = (float)(1.0 / (2.0 * b[3] * b[3]));
      a.bump[k][4] = (float)b[4];
      a.bump[k][5] = (float)b[5];
      a.bump[k][6] = (float)b[6];
    }
  }
  const int nbins = a.gx * a.gy * a.gz;
  // one entry per blob; a split field has two, each binned by one piece's
  // map (entry k + n_blobs: piece 2's, stored with a negative amplitude)
  const int n_entries = deform == 4 ? 2 * n_blobs : n_blobs;
  std::vector<int> bin_of((size_t)n_entries), count((size_t)nbins + 1, 0);
  for (int e = 0; e < n_entries; e++) {
    const int k = e % std::max(n_blobs, 1);
    const float *b = blobs + (size_t)k * 5;
    double X[3] = {b[0], b[1], b[2]}, x[3] = {b[0], b[1], b[2]};
    if (deform == 1 || deform == 4) {
      const double *P = coef + (e >= n_blobs ? 15 : 0);  // t (3), E (9), c (3)
      const double *E = P + 3;
      for (int i = 0; i < 3; i++)
        x[i] = X[i] + P[i] + E[i * 3 + 0] * (X[0] - P[12]) + E[i * 3 + 1] * (X[1] - P[13]) +
               E[i * 3 + 2] * (X[2] - P[14]);
    } else if (deform == 5) {
      x[0] = X[0] + 0.5 * coef[3] * tanh((X[2] - coef[4]) / coef[5]);
      x[2] = X[2] + 0.5 * coef[0] * ((X[0] - coef[1]) * (X[0] - coef[1]) - coef[2]);
    } else if (deform == 2) {
      const double w = 2.0 * M_PI / coef[1];
      x[0] = X[0] + coef[0] * sin(w * X[1]);
      x[1] = X[1] + coef[0] * sin(w * X[2]);
      x[2] = X[2] + coef[0] * sin(w * X[0]);
    } else if (deform == 3) {
      const double *E = coef + 3;
      for (int i = 0; i < 3; i++)
        x[i] = X[i] + coef[i] + E[i * 3 + 0] * (X[0] - coef[12]) + E[i * 3 + 1] * (X[1] - coef[13]) +
               E[i * 3 + 2] * (X[2] - coef[14]);
      for (int q = 0; q < (int)coef[15]; q++) {
        const double *bp = coef + 16 + 7 * q;
        const double d2 = (X[0] - bp[0]) * (X[0] - bp[0]) + (X[1] - bp[1]) * (X[1] - bp[1]) +
                          (X[2] - bp[2]) * (X[2] - bp[2]);
        const double g = exp(-d2 / (2.0 * bp[3] * bp[3]));
        for (int i = 0; i < 3; i++) x[i] += bp[4 + i] * g;
      }
    }
    int bx = std::min(std::max((int)floor(x[0] / kBin), 0), a.gx - 1);
    int by = std::min(std::max((int)floor(x[1] / kBin), 0), a.gy - 1);
    int bz = std::min(std::max((int)floor(x[2] / kBin), 0), a.gz - 1);
    bin_of[(size_t)e] = (bz * a.gy + by) * a.gx + bx;
    count[(size_t)bin_of[(size_t)e] + 1]++;
  }
  for (int b = 0; b < nbins; b++) count[(size_t)b + 1] += count[(size_t)b];
  std::vector<int> fill(count.begin(), count.end() - 1);
  std::vector<float> h_blob((size_t)std::max(n_entries, 1) * 4), h_ar((size_t)std::max(n_entries, 1) * 2);
  for (int e = 0; e < n_entries; e++) {
    const int k = e % std::max(n_blobs, 1);
    const float *b = blobs + (size_t)k * 5;
    const int pos = fill[(size_t)bin_of[(size_t)e]]++;
    h_blob[(size_t)pos * 4 + 0] = b[0];
    h_blob[(size_t)pos * 4 + 1] = b[1];
    h_blob[(size_t)pos * 4 + 2] = b[2];
    h_blob[(size_t)pos * 4 + 3] = 1.0f / (2.0f * b[3] * b[3]);
    h_ar[(size_t)pos * 2 + 0] = e >= n_blobs ? -b[4] : b[4];
    h_ar[(size_t)pos * 2 + 1] = 16.0f * b[3] * b[3];
  }
  // blobs reach 4 sigma; bins are 16 voxels and neighbours one bin away, so
  // sigma may not exceed 3.5 voxels (plus the deformation's local stretch)
  for (int k = 0; k < n_blobs; k++)
    if (blobs[(size_t)k * 5 + 3] > 3.5f) return dvc_internal_set_error(DVC_E_ARG, "blob sigma > 3.5");
  void *d_blob = nullptr, *d_ar = nullptr, *d_start = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMalloc(&d_blob, h_blob.size() * 4) != cudaSuccess || cudaMalloc(&d_ar, h_ar.size() * 4) != cudaSuccess ||
      cudaMalloc(&d_start, count.size() * 4) != cudaSuccess) {
    cudaFree(d_blob);
    cudaFree(d_ar);
    cudaFree(d_start);
    return dvc_internal_set_error(DVC_E_NOMEM, "synth buffers");
  }
  cudaMemcpy(d_blob, h_blob.data(), h_blob.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(d_ar, h_ar.data(), h_ar.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(d_start, count.data(), count.size() * 4, cudaMemcpyHostToDevice);
  a.blobs = (const float4 *)d_blob;
  a.amp_r2 = (const float2 *)d_ar;
  a.bin_start = (const int *)d_start;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  synth_kernel<<<sms * 8, 256, 0, st>>>(a);
  cudaError_t err = cudaGetLastError();
  if (err == cudaSuccess) err = cudaStreamSynchronize(st);
  cudaFree(d_blob);
  cudaFree(d_ar);
  cudaFree(d_start);
  if (err != cudaSuccess) return dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(err));
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}
