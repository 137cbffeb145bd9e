// dvc_device.cuh — device building blocks of the DVC engine.
//
// Interpolation. The reference builds, per touched cell, the 64 Lekien-Marsden
// tricubic coefficients a = BI * vb from the values and central-difference
// derivatives (f, fx, fy, fz, fxy, fxz, fyz, fxyz) at the cell's 8 corners
// (Core/Interpolate.cpp:377-402, Core/Matrix_4d.h:108-133), then evaluates
// sum a_ijk x^i y^j z^k (Core/Interpolate.cpp:539-561). The corner
// constraints are the tensor product of the 1D Hermite constraints, and the
// central differences are the tensor product of 1D differences, so inside the
// interpolation box that interpolant is exactly the tensor product of 1D cubic
// Hermite interpolation with central-difference slopes (Catmull-Rom):
//   val = sum_{a,b,c} wx_a wy_b wz_c V[x-1+a, y-1+b, z-1+c]
// with per-axis weights of the cell fraction f
//   w_-1 = (-f^3 + 2f^2 - f)/2, w_0 = (3f^3 - 5f^2 + 2)/2,
//   w_1  = (-3f^3 + 4f^2 + f)/2, w_2 = (f^3 - f^2)/2.
// That is 84 FMAs per sample instead of a 64x64 coefficient product.
//
// Box faces. The reference computes derivatives only inside its interpolation
// box and copies them outward on the faces (Core/Interpolate.cpp:293-335): the
// derivative quantities of a corner on a face equal those of the nearest
// interior voxel, while the value f stays the corner's own. Per axis this
// gives three 1D weight sets for a cell of box-local index c (n voxels):
//   A: values and slopes at the clamped corners (Catmull-Rom inside),
//   B: values only, at the clamped corners,
//   C: values only, at the true corners,
// and the interpolant is  A(x)A(y)A(z) - B(x)B(y)B(z) + C(x)C(y)C(z).
// Inside the box B == C on every axis and it reduces to the separable form.
// A cell with c = n-1 (the reference reads past its arrays) is evaluated as
// the cubic of cell n-2 continued past its end; the FP64 oracle does the same.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dvc {

// threads per search CTA (DVC_THREADS: a multiple of 32, for experiments)
#ifndef DVC_THREADS
#define DVC_THREADS 256
#endif
constexpr int kThreads = DVC_THREADS;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxDof = 12;

// ------------------------------------------------------------ 1D weights ---
struct W4 {
  float w[4];
};

// Catmull-Rom (interior) weights and their derivative in f.
__device__ __forceinline__ void cr_weights(float f, float w[4], float dw[4]) {
  const float f2 = f * f, f3 = f2 * f;
  w[0] = 0.5f * (-f3 + 2.f * f2 - f);
  w[1] = 0.5f * (3.f * f3 - 5.f * f2 + 2.f);
  w[2] = 0.5f * (-3.f * f3 + 4.f * f2 + f);
  w[3] = 0.5f * (f3 - f2);
  dw[0] = 0.5f * (-3.f * f2 + 4.f * f - 1.f);
  dw[1] = 0.5f * (9.f * f2 - 10.f * f);
  dw[2] = 0.5f * (-9.f * f2 + 8.f * f + 1.f);
  dw[3] = 0.5f * (3.f * f2 - 2.f * f);
}

// Face weight sets (A, B, C) for one axis; kind 1 = max face (c == n-2),
// kind 2 = min face (c == 0). See the file header.
__device__ __forceinline__ void face_weights(int kind, float f, float A[4], float dA[4], float B[4],
                                             float dB[4], float Cc[4], float dC[4]) {
  const float f2 = f * f, f3 = f2 * f;
  const float h00 = 2.f * f3 - 3.f * f2 + 1.f, dh00 = 6.f * f2 - 6.f * f;
  const float h01 = 1.f - h00, dh01 = -dh00;
  const float hs = 2.f * f3 - 3.f * f2 + f, dhs = 6.f * f2 - 6.f * f + 1.f;  // h10 + h11
  Cc[0] = 0.f; Cc[1] = h00; Cc[2] = h01; Cc[3] = 0.f;
  dC[0] = 0.f; dC[1] = dh00; dC[2] = dh01; dC[3] = 0.f;
  if (kind == 1) {
    A[0] = -0.5f * hs; A[1] = 1.f; A[2] = 0.5f * hs; A[3] = 0.f;
    dA[0] = -0.5f * dhs; dA[1] = 0.f; dA[2] = 0.5f * dhs; dA[3] = 0.f;
    B[0] = 0.f; B[1] = 1.f; B[2] = 0.f; B[3] = 0.f;
  } else {
    A[0] = 0.f; A[1] = -0.5f * hs; A[2] = 1.f; A[3] = 0.5f * hs;
    dA[0] = 0.f; dA[1] = -0.5f * dhs; dA[2] = 0.f; dA[3] = 0.5f * dhs;
    B[0] = 0.f; B[1] = 0.f; B[2] = 1.f; B[3] = 0.f;
  }
  dB[0] = dB[1] = dB[2] = dB[3] = 0.f;
}

// ------------------------------------------------------------- row loads ---
// Four consecutive voxels along x starting at linear index `idx`, as floats.
// Volumes are allocated with >= 16 bytes of tail padding, so the aligned
// over-read past the last row stays inside the allocation.
__device__ __forceinline__ float u8f(uint32_t b) {  // exact uint8 -> float
  return __int_as_float(0x4B000000u | b) - 8388608.0f;
}

__device__ __forceinline__ void load_row4(const uint8_t *__restrict__ vol, long long idx,
                                          float v[4]) {
  const uint32_t *p = reinterpret_cast<const uint32_t *>(vol + (idx & ~3LL));
  const uint32_t w0 = __ldg(p), w1 = __ldg(p + 1);
  const uint32_t s = (uint32_t)(idx & 3);
  const uint32_t sel = (s) | ((s + 1) << 4) | ((s + 2) << 8) | ((s + 3) << 12);
  const uint32_t w = __byte_perm(w0, w1, sel);
  v[0] = u8f(__byte_perm(w, 0, 0x4440));
  v[1] = u8f(__byte_perm(w, 0, 0x4441));
  v[2] = u8f(__byte_perm(w, 0, 0x4442));
  v[3] = u8f(__byte_perm(w, 0, 0x4443));
}

__device__ __forceinline__ void load_row4(const uint16_t *__restrict__ vol, long long idx,
                                          float v[4]) {
  const char *base = reinterpret_cast<const char *>(vol);
  const long long a = idx * 2;
  const uint2 *p = reinterpret_cast<const uint2 *>(base + (a & ~7LL));
  const uint2 q01 = __ldg(p), q23 = __ldg(p + 1);
  const uint32_t s = (uint32_t)(a & 7);  // 0, 2, 4 or 6 bytes
  const bool hi = s >= 4;
  const uint32_t lo = hi ? q01.y : q01.x, mid = hi ? q23.x : q01.y, top = hi ? q23.y : q23.x;
  const uint32_t sh = (s & 3) * 8;
  const uint32_t r0 = __funnelshift_r(lo, mid, sh), r1 = __funnelshift_r(mid, top, sh);
  v[0] = __int_as_float(0x4B000000u | (r0 & 0xFFFFu)) - 8388608.0f;
  v[1] = __int_as_float(0x4B000000u | (r0 >> 16)) - 8388608.0f;
  v[2] = __int_as_float(0x4B000000u | (r1 & 0xFFFFu)) - 8388608.0f;
  v[3] = __int_as_float(0x4B000000u | (r1 >> 16)) - 8388608.0f;
}

template <typename VT>
__device__ __forceinline__ float load_voxel_checked(const VT *__restrict__ vol, int x, int y, int z,
                                                    int nx, int ny, int nz) {
  if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return 0.f;
  return (float)__ldg(vol + ((long long)z * ny + y) * nx + x);
}

// Voxel sources. A source returns rows of four consecutive voxels along x
// (and single voxels) at global voxel coordinates.
//   GSrc: the volume in global memory (read-only path), optionally with
//         bounds checks (boxes reaching the volume edge read 0 outside);
//   SSrc: a box-shaped region of the volume staged in shared memory by TMA.
template <typename VT>
struct GSrc {
  const VT *vol;
  int nx, ny, nz;
  bool checked;
  __device__ __forceinline__ void row4(int x, int y, int z, float v[4]) const {
    if (!checked) {
      load_row4(vol, ((long long)z * ny + y) * nx + x, v);
    } else {
#pragma unroll
      for (int a = 0; a < 4; a++) v[a] = load_voxel_checked(vol, x + a, y, z, nx, ny, nz);
    }
  }
  __device__ __forceinline__ float voxel(int x, int y, int z) const {
    if (checked) return load_voxel_checked(vol, x, y, z, nx, ny, nz);
    return (float)__ldg(vol + ((long long)z * ny + y) * nx + x);
  }
  // rows of the 4x4x4 stencil with low corner (x0, y0, z0): row (b, c) is at
  // y0 + b, z0 + c
  struct Stencil {
    int x0, y0, z0;
  };
  __device__ __forceinline__ Stencil stencil(int x0, int y0, int z0) const { return {x0, y0, z0}; }
  __device__ __forceinline__ void srow(const Stencil &h, int b, int c, float v[4]) const {
    row4(h.x0, h.y0 + b, h.z0 + c, v);
  }
};

__device__ __forceinline__ uint32_t lds32(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ uint2 lds64(uint32_t addr) {
  uint2 v;
  asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(addr));
  return v;
}

template <typename VT>
struct SSrc {
  uint32_t base;       // shared-memory address of the staged box
  int r0x, r0y, r0z;   // global voxel coordinates of the box's first element
  int bx, by;          // box pitch (elements per row, rows per slice); a row is
                       // a whole number of 16-byte units
  __device__ __forceinline__ uint32_t boff(int x, int y, int z) const {
    return (uint32_t)(((z - r0z) * by + (y - r0y)) * bx + (x - r0x)) * (uint32_t)sizeof(VT);
  }
  // A stencil's rows all start at the same position inside their 4-byte
  // word (row pitches are multiples of 16 bytes): keep the word address of
  // the first row and the byte shift, each row is then one address add.
  struct Stencil {
    uint32_t al;  // shared-memory address of the 4-byte word holding the first voxel
    uint32_t sh;  // byte position of the first voxel in that word
  };
  __device__ __forceinline__ Stencil stencil_at(uint32_t off) const { return {base + (off & ~3u), off & 3u}; }
  __device__ __forceinline__ Stencil stencil(int x0, int y0, int z0) const {
    return stencil_at(boff(x0, y0, z0));
  }
  // four voxels from word address `al`, byte shift `sh`; the byte permutes
  // build 2^23 + voxel directly as a float (exact), one subtraction each
  __device__ __forceinline__ void row_al(uint32_t al, uint32_t sh, float v[4]) const {
    if (sizeof(VT) == 1) {
      const uint32_t w = __byte_perm(lds32(al), lds32(al + 4), 0x3210u + sh * 0x1111u);
      v[0] = __int_as_float(__byte_perm(w, 0x4B00u, 0x5440u)) - 8388608.0f;
      v[1] = __int_as_float(__byte_perm(w, 0x4B00u, 0x5441u)) - 8388608.0f;
      v[2] = __int_as_float(__byte_perm(w, 0x4B00u, 0x5442u)) - 8388608.0f;
      v[3] = __int_as_float(__byte_perm(w, 0x4B00u, 0x5443u)) - 8388608.0f;
    } else {
      const uint32_t w0 = lds32(al), w1 = lds32(al + 4), w2 = lds32(al + 8);
      const uint32_t r0 = __funnelshift_r(w0, w1, sh * 8), r1 = __funnelshift_r(w1, w2, sh * 8);
      v[0] = __int_as_float(__byte_perm(r0, 0x4B00u, 0x5410u)) - 8388608.0f;
      v[1] = __int_as_float(__byte_perm(r0, 0x4B00u, 0x5432u)) - 8388608.0f;
      v[2] = __int_as_float(__byte_perm(r1, 0x4B00u, 0x5410u)) - 8388608.0f;
      v[3] = __int_as_float(__byte_perm(r1, 0x4B00u, 0x5432u)) - 8388608.0f;
    }
  }
  __device__ __forceinline__ void row4(int x, int y, int z, float v[4]) const {
    const Stencil h = stencil(x, y, z);
    row_al(h.al, h.sh, v);
  }
  __device__ __forceinline__ float voxel(int x, int y, int z) const {
    const uint32_t off = boff(x, y, z);
    const uint32_t w = lds32(base + (off & ~3u));
    if (sizeof(VT) == 1) return __int_as_float(__byte_perm(w, 0x4B00u, 0x5440u | (off & 3u))) - 8388608.0f;
    return __int_as_float(__byte_perm(w, 0x4B00u, (off & 2u) ? 0x5432u : 0x5410u)) - 8388608.0f;
  }
  // byte distance between stencil rows (b, c) and (0, 0)
  __device__ __forceinline__ uint32_t row_step(int b, int c) const {
    return (uint32_t)((c * by + b) * bx) * (uint32_t)sizeof(VT);
  }
  __device__ __forceinline__ void srow(const Stencil &h, int b, int c, float v[4]) const {
    row_al(h.al + row_step(b, c), h.sh, v);
  }
};

// Interpolation box of the current point: global voxel origin and extents.
struct BoxGeom {
  int ox, oy, oz;  // global voxel index of box voxel (0,0,0)
  int bx, by, bz;  // box extents (voxels)
};

// Separable contraction of the 4x4x4 stencil whose low corner is at global
// voxel (x0, y0, z0), with value weights w* and (when GRAD) slope weights d*.
template <typename Src, bool GRAD>
__device__ __forceinline__ float contract_h(const Src &src, const typename Src::Stencil &h,
                                            const float wx[4], const float wy[4], const float wz[4],
                                            const float dx[4], const float dy[4], const float dz[4],
                                            float g[3]) {
  float val = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float s = 0.f, sdx = 0.f, sdy = 0.f;
#pragma unroll
    for (int b = 0; b < 4; b++) {
      float v[4];
      src.srow(h, b, c, v);
      const float r = wx[0] * v[0] + wx[1] * v[1] + wx[2] * v[2] + wx[3] * v[3];
      s += wy[b] * r;
      if (GRAD) {
        const float rdx = dx[0] * v[0] + dx[1] * v[1] + dx[2] * v[2] + dx[3] * v[3];
        sdx += wy[b] * rdx;
        sdy += dy[b] * r;
      }
    }
    val += wz[c] * s;
    if (GRAD) {
      gx += wz[c] * sdx;
      gy += wz[c] * sdy;
      gz += dz[c] * s;
    }
  }
  if (GRAD) {
    g[0] = gx;
    g[1] = gy;
    g[2] = gz;
  }
  return val;
}

template <typename Src, bool GRAD>
__device__ __forceinline__ float contract(const Src &src, int x0, int y0, int z0,
                                          const float wx[4], const float wy[4], const float wz[4],
                                          const float dx[4], const float dy[4], const float dz[4],
                                          float g[3]) {
  return contract_h<Src, GRAD>(src, src.stencil(x0, y0, z0), wx, wy, wz, dx, dy, dz, g);
}

// Face cells (rare): A A A - B B B + C C C, out of line to keep the hot
// interior path small.
template <typename Src, bool GRAD>
__device__ __noinline__ float interp_face(const Src src, int x0, int y0, int z0, int k0, int k1,
                                          int k2, float f0, float f1, float f2, float *gout) {
  const int kind[3] = {k0, k1, k2};
  const float f[3] = {f0, f1, f2};
  float A[3][4], dA[3][4], B[3][4], dB[3][4], Cc[3][4], dC[3][4];
  for (int d = 0; d < 3; d++) {
    if (kind[d] == 0) {
      cr_weights(f[d], A[d], dA[d]);
      const float f2 = f[d] * f[d], f3 = f2 * f[d];
      const float h00 = 2.f * f3 - 3.f * f2 + 1.f, dh00 = 6.f * f2 - 6.f * f[d];
      B[d][0] = 0.f; B[d][1] = h00; B[d][2] = 1.f - h00; B[d][3] = 0.f;
      dB[d][0] = 0.f; dB[d][1] = dh00; dB[d][2] = -dh00; dB[d][3] = 0.f;
      for (int k = 0; k < 4; k++) {
        Cc[d][k] = B[d][k];
        dC[d][k] = dB[d][k];
      }
    } else {
      face_weights(kind[d], f[d], A[d], dA[d], B[d], dB[d], Cc[d], dC[d]);
    }
  }
  float g1[3], g2[3], g3[3];
  float v = contract<Src, GRAD>(src, x0, y0, z0, A[0], A[1], A[2], dA[0], dA[1], dA[2], g1);
  v -= contract<Src, GRAD>(src, x0, y0, z0, B[0], B[1], B[2], dB[0], dB[1], dB[2], g2);
  v += contract<Src, GRAD>(src, x0, y0, z0, Cc[0], Cc[1], Cc[2], dC[0], dC[1], dC[2], g3);
  if (GRAD)
    for (int d = 0; d < 3; d++) gout[d] = g1[d] - g2[d] + g3[d];
  return v;
}

// Cell adjustment shared by all sources: the reference-undefined last plane
// (c = n-1) is evaluated as cell n-2 continued past its end. Returns the
// stencil's low corner (global) and the per-axis face kinds.
template <int ITYPE>
__device__ __forceinline__ bool prep_cell(const BoxGeom &G, int c[3], float f[3], int lo[3],
                                          int kind[3]) {
  const int n[3] = {G.bx, G.by, G.bz};
  const int o[3] = {G.ox, G.oy, G.oz};
  bool undef = false;
  bool face = false;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (ITYPE == 0) {
      if (c[d] > n[d] - 1) {
        undef = true;
        c[d] = n[d] - 1;
      }
      lo[d] = o[d] + c[d];
      kind[d] = 0;
    } else {
      if (c[d] > n[d] - 2) {
        undef = true;
        f[d] += (float)(c[d] - (n[d] - 2));
        c[d] = n[d] - 2;
      }
      lo[d] = o[d] + c[d] - 1;
      kind[d] = ITYPE == 2 ? ((c[d] == n[d] - 2) ? 1 : (c[d] <= 0 ? 2 : 0)) : 0;
      face |= kind[d] != 0;
    }
  }
  (void)face;
  return undef;
}

// Interpolation of one sample at box-local cell c and fraction f from source
// `src`; the stencil's global low corner `lo` and face kinds come from
// prep_cell. ITYPE: 0 nearest, 1 trilinear, 2 tricubic.
template <typename Src, int ITYPE, bool GRAD>
__device__ __forceinline__ float interp_at(const Src &src, const int lo[3], const int kind[3],
                                           const float f[3], float g[3]) {
  if (ITYPE == 0) {
    if (GRAD) g[0] = g[1] = g[2] = 0.f;
    return src.voxel(lo[0], lo[1], lo[2]);
  }
  float w[3][4], dw[3][4];
  if (ITYPE == 1) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
      w[d][0] = 0.f; w[d][1] = 1.f - f[d]; w[d][2] = f[d]; w[d][3] = 0.f;
      dw[d][0] = 0.f; dw[d][1] = -1.f; dw[d][2] = 1.f; dw[d][3] = 0.f;
    }
    return contract<Src, GRAD>(src, lo[0], lo[1], lo[2], w[0], w[1], w[2], dw[0], dw[1], dw[2], g);
  }
  if ((kind[0] | kind[1] | kind[2]) == 0) {
#pragma unroll
    for (int d = 0; d < 3; d++) cr_weights(f[d], w[d], dw[d]);
    return contract<Src, GRAD>(src, lo[0], lo[1], lo[2], w[0], w[1], w[2], dw[0], dw[1], dw[2], g);
  }
  return interp_face<Src, GRAD>(src, lo[0], lo[1], lo[2], kind[0], kind[1], kind[2], f[0], f[1],
                                f[2], g);
}

// Global-memory interpolation in the point's box (cell clamping included).
template <typename VT, int ITYPE, bool GRAD>
__device__ __forceinline__ float interp_global(const GSrc<VT> &src, const BoxGeom &G, int c[3],
                                               float f[3], float g[3], bool &undef) {
  int lo[3], kind[3];
  undef = prep_cell<ITYPE>(G, c, f, lo, kind);
  return interp_at<GSrc<VT>, ITYPE, GRAD>(src, lo, kind, f, g);
}

// ------------------------------------------------------------ reductions ---
// Compensated (Kahan) FP32 accumulator.
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// TwoSum merge of two compensated partials (hi, lo).
__device__ __forceinline__ void two_sum_merge(float &hi, float &lo, float bhi, float blo) {
  const float s = hi + bhi;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (bhi - bb);
  hi = s;
  lo = lo + blo + err;
}

}  // namespace dvc
