// dvc_oracle.cpp — FP64 CPU restatement of the reference DVC hot path.
//
// TEST INFRASTRUCTURE ONLY. The product (libdvcgpu.so, the dvc/strain host
// programs) never links, loads or calls this file. tests/, the smoke check in
// __graft_entry__.py and the cpu_baseline leg of bench.py use it as the
// checker: a plain restatement of what the reference computes, step by step,
// in double precision, with the reference's own control flow.
//
// Each function cites the reference source it follows. The restatement is
// pinned against the reference itself: oracle/build_ref.sh compiles the
// reference's own Core/*.cpp into oracle/_ref/libdvcref.so (against the
// project-written Eigen subset in oracle/eigen_shim) and tests/test_oracle_vs_ref.py
// compares the two on the same inputs.
//
// Behaviour the reference leaves undefined, and the rule used here instead
// (the GPU engine uses the same rules):
//  * voxels outside the volume (the reference reads past the file and keeps an
//    uninitialised buffer, Core/Interpolate.cpp:171-192) read as 0;
//  * a sample whose interpolation cell touches the last plane of the
//    interpolation box (Core/Interpolate.cpp:377-402 then reads past the
//    Matrix_4d allocation in x, or wraps into the next row in y/z) is
//    evaluated as the cubic of the previous cell extended past its end; such
//    evaluations are counted in `undefined_evals` so tests can exclude them.
#include "../include/dvc_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- volume ---
struct Volume {
  const void *data;
  long nx, ny, nz;
  int bpv;
  double at(long x, long y, long z) const {
    if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return 0.0;
    size_t i = (size_t)((z * ny + y) * nx + x);
    if (bpv == 1) return (double)((const uint8_t *)data)[i];
    return (double)((const uint16_t *)data)[i];
  }
};

// Point::parse_point (Core/Point.cpp:57-66): integer part by truncation
inline int itrunc(double v) { return (int)(v / 1); }

// --------------------------------------------------------------- BoundBox ---
// Core/BoundBox.cpp / BoundBox.h: min, max, centre; integer extents from the
// truncated corners.
struct Box {
  double mn[3], mx[3], cen[3];
  void set(const double a[3], const double b[3]) {
    for (int d = 0; d < 3; d++) {
      mn[d] = a[d];
      mx[d] = b[d];
      cen[d] = (a[d] + b[d]) / 2.0;
    }
  }
  void grow_by(double f) {  // Core/BoundBox.cpp:45-53
    for (int d = 0; d < 3; d++) {
      mn[d] = mn[d] + (-f);
      mx[d] = mx[d] + f;
      cen[d] = (mn[d] + mx[d]) / 2.0;
    }
  }
  void center_on(const double c[3]) {  // Core/BoundBox.cpp:55-65
    for (int d = 0; d < 3; d++) {
      double del = c[d] - cen[d];
      mn[d] = mn[d] + del;
      mx[d] = mx[d] + del;
      cen[d] = cen[d] + del;
    }
  }
  int iext(int d) const { return itrunc(mx[d]) - itrunc(mn[d]); }
  // BoundBox::contains (Core/BoundBox.cpp:67-79): true when b lies inside
  bool contains(const double bmn[3], const double bmx[3]) const {
    return !(bmn[0] < mn[0] || bmn[1] < mn[1] || bmn[2] < mn[2] || bmx[0] > mx[0] ||
             bmx[1] > mx[1] || bmx[2] > mx[2]);
  }
};

// ------------------------------------------------------ Lekien inverse BI ---
// The 64x64 Lekien-Marsden matrix maps the 64 corner quantities
// vb[k*8+c] (k: f, fx, fy, fz, fxy, fxz, fyz, fxyz; corner c = dx+2dy+4dz,
// Core/Matrix_4d.cpp:48-56,65-77) to the tricubic coefficients a[i+4j+16k] of
// x^i y^j z^k (Core/Interpolate.cpp:539-561). The constraint set is the
// tensor product of the 1D Hermite constraints {p(0), p(1), p'(0), p'(1)}, so
// the inverse is the tensor product of the 1D Hermite inverse
//   H = [[1,0,0,0],[0,0,1,0],[-3,3,-2,-1],[2,-2,1,1]]
// acting on (p0, p1, m0, m1). Built here from that definition; it equals the
// literal table of Core/Interpolate.cpp:63-127 entry for entry (checked in
// tests/test_oracle_vs_ref.py through interpolated values).
struct LekienBI {
  double m[64][64];
  LekienBI() {
    const int H[4][4] = {{1, 0, 0, 0}, {0, 0, 1, 0}, {-3, 3, -2, -1}, {2, -2, 1, 1}};
    // quantity k -> derivative flags per axis
    const int dflag[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                             {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    for (int r = 0; r < 64; r++)
      for (int c = 0; c < 64; c++) m[r][c] = 0.0;
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++)
        for (int kz = 0; kz < 4; kz++) {
          int row = i + 4 * j + 16 * kz;
          for (int q = 0; q < 8; q++)
            for (int c = 0; c < 8; c++) {
              int cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
              // 1D input index: value at corner 0/1 -> 0/1, derivative -> 2/3
              int ix = dflag[q][0] * 2 + cx, iy = dflag[q][1] * 2 + cy, iz = dflag[q][2] * 2 + cz;
              m[row][q * 8 + c] = (double)(H[i][ix] * H[j][iy] * H[kz][iz]);
            }
        }
  }
};
const LekienBI &bi() {
  static LekienBI b;
  return b;
}

// ------------------------------------------------------------ Interpolate ---
// One interpolation region: est_box of the search's nominal size, the
// active box one voxel inside it (Core/Interpolate.cpp:34-56), voxel values,
// the 7 finite-difference derivatives per voxel and lazily built Lekien
// coefficients per cell (Core/Matrix_4d.h:22-48).
struct Interp {
  Box est, act;
  int n[3];  // allocated extents (Core/Interpolate.cpp:58)
  std::vector<double> q;   // 8 quantities per voxel, x slowest like Matrix_4d
  std::vector<double> co;  // 64 coefficients per voxel cell
  std::vector<char> avail;
  long undefined_evals = 0;

  Interp(const Box &nom) {
    est = nom;
    act = nom;
    act.grow_by(-1.0);
    for (int d = 0; d < 3; d++) n[d] = est.iext(d);
    size_t nv = (size_t)n[0] * n[1] * n[2];
    q.assign(nv * 8, 0.0);
    co.assign(nv * 64, 0.0);
    avail.assign(nv, 0);
  }
  size_t vi(int x, int y, int z) const { return ((size_t)x * n[1] + y) * n[2] + z; }
  void center_on(const double c[3]) {
    est.center_on(c);
    act.center_on(c);
  }

  // Interpolate::kernels (Core/Interpolate.cpp:144-258) + kernels_derivs
  // (:260-337): load the est_box voxels, then central differences inside the
  // box (Core/Matrix_4d.h:108-133). The face passes of kernels_derivs copy
  // x, then y, then z faces from their inner neighbours; the net effect is
  // that the derivatives of every voxel equal those of the nearest interior
  // voxel (each index clamped to [1, n-2]).
  void load(const Volume &v) {
    const int x0 = itrunc(est.mn[0]), y0 = itrunc(est.mn[1]), z0 = itrunc(est.mn[2]);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n[0]; x++)
      for (int y = 0; y < n[1]; y++)
        for (int z = 0; z < n[2]; z++) {
          q[vi(x, y, z) * 8 + 0] = v.at(x0 + x, y0 + y, z0 + z);
          avail[vi(x, y, z)] = 0;
        }
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n[0]; x++) {
      int cx = std::min(std::max(x, 1), n[0] - 2);
      for (int y = 0; y < n[1]; y++) {
        int cy = std::min(std::max(y, 1), n[1] - 2);
        for (int z = 0; z < n[2]; z++) {
          int cz = std::min(std::max(z, 1), n[2] - 2);
          auto F = [&](int dx, int dy, int dz) { return q[vi(cx + dx, cy + dy, cz + dz) * 8]; };
          double *o = &q[vi(x, y, z) * 8];
          o[1] = (F(1, 0, 0) - F(-1, 0, 0)) / 2.0;
          o[2] = (F(0, 1, 0) - F(0, -1, 0)) / 2.0;
          o[3] = (F(0, 0, 1) - F(0, 0, -1)) / 2.0;
          o[4] = (F(1, 1, 0) - F(-1, 1, 0) + F(-1, -1, 0) - F(1, -1, 0)) / 4.0;
          o[5] = (F(1, 0, 1) - F(-1, 0, 1) + F(-1, 0, -1) - F(1, 0, -1)) / 4.0;
          o[6] = (F(0, 1, 1) - F(0, -1, 1) + F(0, -1, -1) - F(0, 1, -1)) / 4.0;
          double t1 = (F(1, 1, -1) - F(-1, 1, -1) + F(-1, -1, -1) - F(1, -1, -1)) / 4.0;
          double t2 = (F(1, 1, 1) - F(-1, 1, 1) + F(-1, -1, 1) - F(1, -1, 1)) / 4.0;
          o[7] = (t2 - t1) / 2.0;
        }
      }
    }
  }

  // Interpolate::kernels_Lekien_one (Core/Interpolate.cpp:377-402):
  // va = BI * vb over the 8 corners of cell (x,y,z).
  void lekien_one(int x, int y, int z) {
    double vb[64];
    for (int k = 0; k < 8; k++)
      for (int c = 0; c < 8; c++) {
        int xx = x + (c & 1), yy = y + ((c >> 1) & 1), zz = z + ((c >> 2) & 1);
        vb[k * 8 + c] = q[vi(xx, yy, zz) * 8 + k];
      }
    const auto &B = bi().m;
    // sparse column-major product order of the reference: y(i) += A(i,j) x(j)
    // for columns j ascending (exact here: integer BI, dyadic vb). Built in a
    // local array and stored whole, so two threads filling the same cell
    // store identical values (the reference's lazy fill races the same way).
    double va[64];
    for (int r = 0; r < 64; r++) va[r] = 0.0;
    for (int c = 0; c < 64; c++)
      for (int r = 0; r < 64; r++)
        if (B[r][c] != 0.0) va[r] += B[r][c] * vb[c];
    double *a = &co[vi(x, y, z) * 64];
    for (int r = 0; r < 64; r++) a[r] = va[r];
  }

  // cell + remainder of one point relative to est_box (Core/Interpolate.cpp:494-496,517-524)
  // with the extension rule for the last cell plane (see file header).
  bool cell_of(const double p[3], int c[3], double r[3]) {
    bool undefined = false;
    for (int d = 0; d < 3; d++) {
      int ip = itrunc(p[d]);
      c[d] = ip - itrunc(est.mn[d]);
      r[d] = p[d] - ip;
      if (c[d] > n[d] - 2) {
        undefined = true;
        r[d] += (double)(c[d] - (n[d] - 2));
        c[d] = n[d] - 2;
      }
    }
    return undefined;
  }

  // Interpolate::tri_cub_Lek (Core/Interpolate.cpp:472-567)
  bool tricubic(const std::vector<double> &P, const double bmn[3], const double bmx[3],
                std::vector<double> &out) {
    if (!act.contains(bmn, bmx)) return false;
    const long np = (long)P.size() / 3;
    long undef = 0;
#pragma omp parallel for schedule(static) reduction(+ : undef)
    for (long s = 0; s < np; s++) {
      int c[3];
      double r[3];
      if (cell_of(&P[s * 3], c, r)) undef++;
      size_t cell = vi(c[0], c[1], c[2]);
      if (!avail[cell]) {  // benign race as in the reference: same values
        lekien_one(c[0], c[1], c[2]);
        avail[cell] = 1;
      }
    }
    undefined_evals += undef;
#pragma omp parallel for schedule(static)
    for (long s = 0; s < np; s++) {
      int c[3];
      double r[3];
      cell_of(&P[s * 3], c, r);
      const double *a = &co[vi(c[0], c[1], c[2]) * 64];
      double prx[4] = {1.0, r[0], r[0] * r[0], r[0] * r[0] * r[0]};
      double pry[4] = {1.0, r[1], r[1] * r[1], r[1] * r[1] * r[1]};
      double prz[4] = {1.0, r[2], r[2] * r[2], r[2] * r[2] * r[2]};
      double val = 0;
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
          double pxy = prx[i] * pry[j];
          int k = i + 4 * j;
          val += a[k] * pxy;
          val += a[k + 16] * pxy * prz[1];
          val += a[k + 32] * pxy * prz[2];
          val += a[k + 48] * pxy * prz[3];
        }
      out[(size_t)s] = val;
    }
    return true;
  }

  // Interpolate::tri_lin (Core/Interpolate.cpp:429-470)
  bool trilinear(const std::vector<double> &P, const double bmn[3], const double bmx[3],
                 std::vector<double> &out) {
    if (!act.contains(bmn, bmx)) return false;
    const long np = (long)P.size() / 3;
    for (long s = 0; s < np; s++) {
      int c[3];
      double r[3];
      if (cell_of(&P[s * 3], c, r)) undefined_evals++;
      auto G = [&](int dx, int dy, int dz) { return q[vi(c[0] + dx, c[1] + dy, c[2] + dz) * 8]; };
      double rx = r[0], ry = r[1], rz = r[2];
      out[(size_t)s] = G(0, 0, 0) * (1.0 - rx) * (1.0 - ry) * (1.0 - rz) +
                       G(1, 0, 0) * (rx) * (1.0 - ry) * (1.0 - rz) +
                       G(0, 1, 0) * (1.0 - rx) * (ry) * (1.0 - rz) +
                       G(0, 0, 1) * (1.0 - rx) * (1.0 - ry) * (rz) +
                       G(1, 0, 1) * (rx) * (1.0 - ry) * (rz) +
                       G(0, 1, 1) * (1.0 - rx) * (ry) * (rz) +
                       G(1, 1, 0) * (rx) * (ry) * (1.0 - rz) +
                       G(1, 1, 1) * (rx) * (ry) * (rz);
    }
    return true;
  }

  // Interpolate::nearest (Core/Interpolate.cpp:404-427): the voxel at the
  // truncated position (the cell's low corner).
  bool nearest(const std::vector<double> &P, const double bmn[3], const double bmx[3],
               std::vector<double> &out) {
    if (!act.contains(bmn, bmx)) return false;
    const long np = (long)P.size() / 3;
    for (long s = 0; s < np; s++) {
      int c[3];
      for (int d = 0; d < 3; d++) c[d] = itrunc(P[s * 3 + d]) - itrunc(est.mn[d]);
      if (c[0] > n[0] - 1 || c[1] > n[1] - 1 || c[2] > n[2] - 1) {
        undefined_evals++;
        for (int d = 0; d < 3; d++) c[d] = std::min(c[d], n[d] - 1);
      }
      out[(size_t)s] = q[vi(c[0], c[1], c[2]) * 8];
    }
    return true;
  }

  bool interp(int type, const std::vector<double> &P, const double bmn[3], const double bmx[3],
              std::vector<double> &out) {
    if (type == DVC_NEAREST) return nearest(P, bmn, bmx, out);
    if (type == DVC_TRILINEAR) return trilinear(P, bmn, bmx, out);
    return tricubic(P, bmn, bmx, out);
  }
};

// ----------------------------------------------------- objective functions ---
// Core/ObjectiveFunctions.cpp:24-263, two-pass FP64. The residual overloads
// return the bracketed per-sample difference (SAD: signed difference).
double objective(int fcn, const std::vector<double> &r, const std::vector<double> &t,
                 std::vector<double> *res) {
  const size_t n = r.size();
  double obj = 0.0;
  if (fcn == DVC_SAD || fcn == DVC_SSD) {
    for (size_t i = 0; i < n; i++) {
      double diff = t[i] - r[i];
      if (res) (*res)[i] = diff;
      obj += (fcn == DVC_SAD) ? std::fabs(diff) : diff * diff;
    }
    return obj;
  }
  if (fcn == DVC_ZSSD) {
    double ar = 0.0, at = 0.0;
    for (size_t i = 0; i < n; i++) {
      ar += r[i];
      at += t[i];
    }
    ar = ar / (int)n;
    at = at / (int)n;
    for (size_t i = 0; i < n; i++) {
      double diff = (t[i] - at) - (r[i] - ar);
      if (res) (*res)[i] = diff;
      obj += diff * diff;
    }
    return obj;
  }
  if (fcn == DVC_NSSD) {
    double sr = 0.0, st = 0.0;
    for (size_t i = 0; i < n; i++) {
      sr += r[i] * r[i];
      st += t[i] * t[i];
    }
    sr = std::sqrt(sr);
    st = std::sqrt(st);
    for (size_t i = 0; i < n; i++) {
      double diff = t[i] / st - r[i] / sr;
      if (res) (*res)[i] = diff;
      obj += diff * diff;
    }
    return obj / 2.0;
  }
  // ZNSSD
  double ar = 0.0, at = 0.0;
  for (size_t i = 0; i < n; i++) {
    ar += r[i];
    at += t[i];
  }
  ar = ar / (int)n;
  at = at / (int)n;
  double sr = 0.0, st = 0.0;
  for (size_t i = 0; i < n; i++) {
    sr += (r[i] - ar) * (r[i] - ar);
    st += (t[i] - at) * (t[i] - at);
  }
  sr = std::sqrt(sr);
  st = std::sqrt(st);
  for (size_t i = 0; i < n; i++) {
    double diff = ((t[i] - at) / st) - ((r[i] - ar) / sr);
    if (res) (*res)[i] = diff;
    obj += diff * diff;
  }
  return obj / 4.0;
}

// ----------------------------------------------------------- FloatingCloud ---
struct Cloud {
  std::vector<double> stable;  // n*3
  std::vector<double> moving;  // n*3
  double sref[3];              // stable_refpt
  double sbmn[3], sbmx[3];     // stable bbox (Cloud::AddPoint, Core/Cloud.cpp:28-56)
  double mbmn[3], mbmx[3];     // moving bbox

  void finish() {
    for (int d = 0; d < 3; d++) {
      sbmn[d] = 9999.99;
      sbmx[d] = -9999.99;
    }
    for (size_t s = 0; s < stable.size() / 3; s++)
      for (int d = 0; d < 3; d++) {
        sbmn[d] = std::min(sbmn[d], stable[s * 3 + d]);
        sbmx[d] = std::max(sbmx[d], stable[s * 3 + d]);
      }
    moving = stable;
  }
  // sphere: FloatingCloud(cen, rad, num, aspect.., seed) (Core/FloatingCloud.cpp:40-82)
  void sphere(const double cen[3], double rad, int num, const double asp[3], unsigned seed) {
    std::mt19937 mt(seed);
    std::uniform_real_distribution<double> dist(-rad, rad);
    stable.clear();
    for (int d = 0; d < 3; d++) sref[d] = cen[d];
    int count = 0;
    while (count < num) {
      double rx = dist(mt);
      double ry = dist(mt);
      double rz = dist(mt);
      double radius = std::sqrt(rx * rx + ry * ry + rz * rz);
      if (radius <= rad) {
        count += 1;
        stable.push_back(cen[0] + asp[0] * (rx));
        stable.push_back(cen[1] + asp[1] * (ry));
        stable.push_back(cen[2] + asp[2] * (rz));
      }
    }
    finish();
  }
  // cube: FloatingCloud(box_min, box_max, nx, ny, nz) (Core/FloatingCloud.cpp:84-128)
  void cube(const double bmin[3], const double bmax[3], int nn) {
    stable.clear();
    for (int d = 0; d < 3; d++) sref[d] = (bmax[d] + bmin[d]) / 2.0;
    double inc[3];
    for (int d = 0; d < 3; d++) inc[d] = (bmax[d] - bmin[d]) / (nn - 1);
    for (int i = 0; i < nn; i++) {
      double pz = bmin[2] + i * inc[2];
      for (int j = 0; j < nn; j++) {
        double py = bmin[1] + j * inc[1];
        for (int k = 0; k < nn; k++) {
          double px = bmin[0] + k * inc[0];
          stable.push_back(px);
          stable.push_back(py);
          stable.push_back(pz);
        }
      }
    }
    finish();
  }

  // FloatingCloud::affine_to (Core/FloatingCloud.cpp:236-286) with
  // SearchParams::set_param_vect (Core/SearchParams.cpp:53-107)
  void affine_to(const double *x, int ndof) {
    double mref[3];
    for (int d = 0; d < 3; d++) {
      mref[d] = sref[d] + x[d];
      mbmn[d] = sbmn[d] + x[d];
      mbmx[d] = sbmx[d] + x[d];
    }
    const size_t np = stable.size() / 3;
    for (size_t s = 0; s < np; s++)
      for (int d = 0; d < 3; d++) moving[s * 3 + d] = stable[s * 3 + d] + x[d];
    if (ndof > 3) {
      double phi = x[3], the = x[4], psi = x[5];
      double A[3][3];
      A[0][0] = cos(the) * cos(phi);
      A[0][1] = cos(the) * sin(phi);
      A[0][2] = -sin(the);
      A[1][0] = sin(psi) * sin(the) * cos(phi) - cos(psi) * sin(phi);
      A[1][1] = sin(psi) * sin(the) * sin(phi) + cos(psi) * cos(phi);
      A[1][2] = cos(the) * sin(psi);
      A[2][0] = cos(psi) * sin(the) * cos(phi) + sin(psi) * sin(phi);
      A[2][1] = cos(psi) * sin(the) * sin(phi) - sin(psi) * cos(phi);
      A[2][2] = cos(the) * cos(psi);
      // rotate_ptvect (Core/FloatingCloud.cpp:160-190)
      for (size_t s = 0; s < np; s++) {
        double *p = &moving[s * 3];
        double rel[3] = {p[0] - mref[0], p[1] - mref[1], p[2] - mref[2]};
        double rot[3];
        for (int i = 0; i < 3; i++) rot[i] = A[i][0] * rel[0] + A[i][1] * rel[1] + A[i][2] * rel[2];
        for (int i = 0; i < 3; i++) p[i] = p[i] + (rot[i] - rel[i]);
      }
      if (ndof > 6) {
        // strain_ptvect (Core/FloatingCloud.cpp:130-158)
        double S[3][3] = {{x[6], x[9], x[11]}, {x[9], x[7], x[10]}, {x[11], x[10], x[8]}};
        for (size_t s = 0; s < np; s++) {
          double *p = &moving[s * 3];
          double rel[3] = {p[0] - mref[0], p[1] - mref[1], p[2] - mref[2]};
          double st[3];
          for (int i = 0; i < 3; i++) st[i] = S[i][0] * rel[0] + S[i][1] * rel[1] + S[i][2] * rel[2];
          for (int i = 0; i < 3; i++) p[i] = p[i] + st[i];
        }
      }
      // resize_bbox (Core/FloatingCloud.cpp:192-233)
      double mn[3] = {9999.9, 9999.9, 9999.9}, mx[3] = {-9999.9, -9999.9, -9999.9};
      bool reset = false;
      for (size_t s = 0; s < np; s++)
        for (int d = 0; d < 3; d++) {
          if (moving[s * 3 + d] < mn[d]) {
            mn[d] = moving[s * 3 + d];
            reset = true;
          }
          if (moving[s * 3 + d] > mx[d]) {
            mx[d] = moving[s * 3 + d];
            reset = true;
          }
        }
      if (reset)
        for (int d = 0; d < 3; d++) {
          mbmn[d] = mn[d];
          mbmx[d] = mx[d];
        }
    }
  }
};

// --------------------------------------------------- pivoted QR least squares ---
// Householder QR with column pivoting (Golub & Van Loan Alg. 5.4.1), or
// complete pivoting, solving A x = b with the trailing rank-deficient unknowns
// set to zero. Used where the reference calls colPivHouseholderQr().solve
// (Core/Search.cpp:234) and fullPivHouseholderQr().solve (Core/strain.cpp:533).
void qr_solve(int m, int n, const double *A0 /* row-major m x n */, const double *b0, double *x,
              bool full_pivot) {
  std::vector<double> A(A0, A0 + (size_t)m * n), b(b0, b0 + m);
  auto a = [&](int i, int j) -> double & { return A[(size_t)i * n + j]; };
  std::vector<int> perm(n);
  for (int j = 0; j < n; j++) perm[j] = j;
  const int kmax = std::min(m, n);
  std::vector<double> diag(kmax, 0.0);
  for (int k = 0; k < kmax; k++) {
    int pc = k, pr = k;
    double best = -1.0;
    for (int j = k; j < n; j++) {
      if (full_pivot) {
        for (int i = k; i < m; i++)
          if (std::fabs(a(i, j)) > best) {
            best = std::fabs(a(i, j));
            pc = j;
            pr = i;
          }
      } else {
        double s = 0.0;
        for (int i = k; i < m; i++) s += a(i, j) * a(i, j);
        if (s > best) {
          best = s;
          pc = j;
        }
      }
    }
    if (pc != k) {
      for (int i = 0; i < m; i++) std::swap(a(i, k), a(i, pc));
      std::swap(perm[k], perm[pc]);
    }
    if (full_pivot && pr != k) {
      for (int j = 0; j < n; j++) std::swap(a(k, j), a(pr, j));
      std::swap(b[k], b[pr]);
    }
    double norm = 0.0;
    for (int i = k; i < m; i++) norm += a(i, k) * a(i, k);
    norm = std::sqrt(norm);
    if (norm == 0.0) {
      diag[k] = 0.0;
      continue;
    }
    double alpha = a(k, k) > 0 ? -norm : norm;
    std::vector<double> v(m - k);
    for (int i = k; i < m; i++) v[i - k] = a(i, k);
    v[0] -= alpha;
    double vv = 0.0;
    for (double t : v) vv += t * t;
    if (vv == 0.0) {
      diag[k] = a(k, k);
      continue;
    }
    for (int j = k; j < n; j++) {
      double s = 0.0;
      for (int i = k; i < m; i++) s += v[i - k] * a(i, j);
      s = 2.0 * s / vv;
      for (int i = k; i < m; i++) a(i, j) -= s * v[i - k];
    }
    double s = 0.0;
    for (int i = k; i < m; i++) s += v[i - k] * b[i];
    s = 2.0 * s / vv;
    for (int i = k; i < m; i++) b[i] -= s * v[i - k];
    diag[k] = a(k, k);
  }
  int rank = 0;
  double r00 = kmax > 0 ? std::fabs(diag[0]) : 0.0;
  double thr = std::numeric_limits<double>::epsilon() * (double)std::max(m, n) * r00;
  for (int k = 0; k < kmax; k++) {
    if (std::fabs(diag[k]) > thr)
      rank = k + 1;
    else
      break;
  }
  std::vector<double> y(n, 0.0);
  for (int k = rank - 1; k >= 0; k--) {
    double s = b[k];
    for (int j = k + 1; j < rank; j++) s -= a(k, j) * y[j];
    y[k] = s / a(k, k);
  }
  for (int k = 0; k < n; k++) x[perm[k]] = y[k];
}

// ------------------------------------------------------------------ Search ---
// random_global's translations (Core/Search.cpp:1045-1098): 3 draws per
// translation from the C library's rand() after srand(seed), each
// displ_max * (2 * rand()) / RAND_MAX with the doubled draw an int product
// (wrapping as two's complement above 2^30).
std::vector<double> random_offsets(int num_pts, double displ_max, unsigned seed) {
  srand(seed);
  const double dbl_rand_max = RAND_MAX;
  std::vector<double> rel((size_t)num_pts * 3);
  for (size_t k = 0; k < rel.size(); k++) {
    const int twice = (int)(2u * (unsigned)rand());
    rel[k] = displ_max * (twice / dbl_rand_max);
  }
  return rel;
}

struct Search {
  dvc_params p;
  Volume ref, cor;
  double subv_rad;
  int subv_num;
  Box est_nom;
  Interp *interp_ref, *interp_cor;
  std::vector<double> ref_sub, tar_sub;
  Cloud fc;
  long evals = 0;
  long gn_iters = 0;

  // Search::Search (Core/Search.cpp:24-82)
  explicit Search(const dvc_params &pp, const void *rv, const void *cv) : p(pp) {
    ref = Volume{rv, p.vol_wide, p.vol_high, p.vol_tall, p.bytes_per_voxel};
    cor = Volume{cv, p.vol_wide, p.vol_high, p.vol_tall, p.bytes_per_voxel};
    subv_rad = (p.subvol_size) / 2.0;
    if (p.subvol_geom == DVC_CUBE)
      subv_num = (int)pow(ceil(pow((double)p.subvol_npts, 1.0 / 3.0)), 3.0);
    else
      subv_num = p.subvol_npts;
    double mn[3] = {0.0, 0.0, 0.0};
    double mx[3] = {2 * subv_rad * p.subvol_aspect[0], 2 * subv_rad * p.subvol_aspect[1],
                    2 * subv_rad * p.subvol_aspect[2]};
    est_nom.set(mn, mx);
    est_nom.grow_by(p.disp_max);
    est_nom.grow_by(2.0);
    interp_ref = new Interp(est_nom);
    interp_cor = new Interp(est_nom);
    ref_sub.assign(subv_num, 0.0);
    tar_sub.assign(subv_num, 0.0);
  }
  ~Search() {
    delete interp_ref;
    delete interp_cor;
  }

  // min_Nelder_Mead (Core/Search.cpp:680-932): the reference's simplex rules
  // (reflection 1, expansion 2, contraction -0.5 towards the worst vertex,
  // shrink 0.5 towards the best; a contraction is kept only when it beats
  // the best vertex), its convergence test and its limit of 2000 objective
  // evaluations (Convg_Fail). Returns the status; out = the best vertex.
  int nelder_mead(const double *start, int ndof, double conv_tol, double *out, int &num_func) {
    const int MAX_FUNC = 2000;
    const double NOT_ZERO = 1.0e-10, ALPHA = 1.0, GAMMA = 2.0, DELTA = -0.5, OMEGA = 0.5;
    const int nvrt = ndof + 1;
    std::vector<std::vector<double>> simplex((size_t)nvrt, std::vector<double>(start, start + ndof));
    for (int i = 1; i < nvrt; i++) simplex[(size_t)i][(size_t)i - 1] += 0.2;  // del_tra = del_rot = del_str
    std::vector<double> val((size_t)nvrt), centroid((size_t)ndof), del((size_t)ndof), xref((size_t)ndof),
        xexp((size_t)ndof), xcon((size_t)ndof);
    num_func = 0;
    for (int i = 0; i < nvrt; i++)
      if (!obj_val_at(simplex[(size_t)i].data(), ndof, val[(size_t)i], nullptr)) return DVC_RANGE_FAIL;
    num_func += nvrt;
    for (;;) {
      int wrst = 0, best = 0;
      for (int i = 1; i < nvrt; i++) {
        if (val[(size_t)i] > val[(size_t)wrst]) wrst = i;
        if (val[(size_t)i] < val[(size_t)best]) best = i;
      }
      int poor = best;
      for (int i = 0; i < nvrt; i++)
        if (i != wrst && i != best && val[(size_t)i] > val[(size_t)poor]) poor = i;
      const double rel_diff = 2.0 * std::fabs(val[(size_t)wrst] - val[(size_t)best]) /
                              (std::fabs(val[(size_t)wrst]) + std::fabs(val[(size_t)best]) + NOT_ZERO);
      if (rel_diff < conv_tol) {
        for (int j = 0; j < ndof; j++) out[j] = simplex[(size_t)best][(size_t)j];
        return DVC_POINT_GOOD;
      }
      if (num_func > MAX_FUNC) return DVC_CONVG_FAIL;
      for (int j = 0; j < ndof; j++) {
        double c = 0.0;
        for (int i = 0; i < nvrt; i++)
          if (i != wrst) c += simplex[(size_t)i][(size_t)j];
        c /= ndof;
        centroid[(size_t)j] = c;
        del[(size_t)j] = c - simplex[(size_t)wrst][(size_t)j];
      }
      for (int j = 0; j < ndof; j++) xref[(size_t)j] = centroid[(size_t)j] + ALPHA * del[(size_t)j];
      double yref, yexp, ycon;
      if (!obj_val_at(xref.data(), ndof, yref, nullptr)) return DVC_RANGE_FAIL;
      num_func += 1;
      if (yref <= val[(size_t)poor] && yref >= val[(size_t)best]) {
        simplex[(size_t)wrst] = xref;
        val[(size_t)wrst] = yref;
        continue;
      }
      if (yref < val[(size_t)best]) {
        for (int j = 0; j < ndof; j++) xexp[(size_t)j] = centroid[(size_t)j] + GAMMA * del[(size_t)j];
        if (!obj_val_at(xexp.data(), ndof, yexp, nullptr)) return DVC_RANGE_FAIL;
        num_func += 1;
        if (yexp < val[(size_t)best]) {
          simplex[(size_t)wrst] = xexp;
          val[(size_t)wrst] = yexp;
        } else {
          simplex[(size_t)wrst] = xref;
          val[(size_t)wrst] = yref;
        }
        continue;
      }
      for (int j = 0; j < ndof; j++) xcon[(size_t)j] = centroid[(size_t)j] + DELTA * del[(size_t)j];
      if (!obj_val_at(xcon.data(), ndof, ycon, nullptr)) return DVC_RANGE_FAIL;
      num_func += 1;
      if (ycon < val[(size_t)best]) {
        simplex[(size_t)wrst] = xcon;
        val[(size_t)wrst] = ycon;
        continue;
      }
      for (int i = 0; i < nvrt; i++) {
        if (i == best) continue;
        for (int j = 0; j < ndof; j++)
          simplex[(size_t)i][(size_t)j] =
              simplex[(size_t)best][(size_t)j] + OMEGA * (simplex[(size_t)i][(size_t)j] - simplex[(size_t)best][(size_t)j]);
        if (!obj_val_at(simplex[(size_t)i].data(), ndof, val[(size_t)i], nullptr)) return DVC_RANGE_FAIL;
        num_func += 1;
      }
    }
  }

  // Search::obj_val_at (Core/Search.cpp:448-488); false = Range_Fail
  bool obj_val_at(const double *x, int nd, double &obj, std::vector<double> *res) {
    fc.affine_to(x, nd);
    evals++;
    if (!interp_cor->interp(p.interp_type, fc.moving, fc.mbmn, fc.mbmx, tar_sub)) return false;
    obj = objective(p.obj_function, ref_sub, tar_sub, res);
    return true;
  }

  // Search::process_point (Core/Search.cpp:95-192); returns the status and
  // fills par_min/obj_min. `seed` is the starting_param translation.
  int process_point(const double pt[3], const double seed[3], double *par_out, double &obj_out,
                    int *iters_out) {
    // subvolume sample cloud (Core/Search.cpp:100-119)
    if (p.subvol_geom == DVC_SPHERE) {
      fc.sphere(pt, subv_rad, subv_num, p.subvol_aspect, p.sphere_seed);
    } else {
      double smn[3], smx[3];
      for (int d = 0; d < 3; d++) {
        smn[d] = pt[d] + (-subv_rad * p.subvol_aspect[d]);
        smx[d] = pt[d] + (subv_rad * p.subvol_aspect[d]);
      }
      int grid_inc = (int)ceil(pow((double)subv_num, 1.0 / 3.0));
      fc.cube(smn, smx, grid_inc);
    }
    // search_pt_setup (Core/Search.cpp:248-275)
    interp_ref->center_on(pt);
    interp_ref->load(ref);
    interp_ref->interp(p.interp_type, fc.stable, fc.sbmn, fc.sbmx, ref_sub);
    // subvolume pre-check as the reference's manual documents it
    // (Core/InputRead.cpp:282-323; parsed there, never applied by its search):
    // fewer than min_vol_fract of the reference samples in the gray range
    if (p.subvol_thresh) {
      int cnt = 0;
      for (double v : ref_sub)
        if (v >= p.gray_thresh_min && v <= p.gray_thresh_max) cnt++;
      if ((double)cnt < p.min_vol_fract * subv_num) {
        evals++;
        return DVC_NOT_SEARCH;
      }
    }
    const int ndof = p.num_srch_dof;
    std::vector<double> par(ndof, 0.0);
    for (int d = 0; d < 3; d++) par[d] = seed[d];
    double off[3] = {pt[0], pt[1], pt[2]};
    // Point::move_by
    for (int d = 0; d < 3; d++) off[d] = off[d] + par[d];
    interp_cor->center_on(off);
    interp_cor->load(cor);
    evals++;  // the reference-subvolume interpolation counts as one evaluation

    // random_global (Core/Search.cpp:1045-1098): as many random translations
    // as the grid has points, each component displ_max * (2 rand()) /
    // RAND_MAX from the C library's generator seeded with coarse_seed (the
    // reference seeds it from the clock); the doubled draw is an int product
    // that wraps for draws above 2^30 (two's complement), which spreads the
    // components over [-displ_max, displ_max)
    if (p.coarse_method == DVC_COARSE_RANDOM && p.basin_radius != 0.0) {
      double displ_max = p.disp_max;
      int num_inc = (int)(displ_max / p.basin_radius);
      int num_pts = (2 * num_inc + 1) * (2 * num_inc + 1) * (2 * num_inc + 1);
      std::vector<double> rel = random_offsets(num_pts, displ_max, p.coarse_seed);
      double obj_min = std::numeric_limits<double>::max();
      double mn[3] = {0.0, 0.0, 0.0};
      for (int i = 0; i < num_pts; i++) {
        double pc[3] = {par[0] + rel[(size_t)i * 3], par[1] + rel[(size_t)i * 3 + 1], par[2] + rel[(size_t)i * 3 + 2]};
        double o;
        if (!obj_val_at(pc, 3, o, nullptr)) return DVC_RANGE_FAIL;
        if (o < obj_min) {
          obj_min = o;
          for (int d = 0; d < 3; d++) mn[d] = rel[(size_t)i * 3 + d];
        }
      }
      for (int d = 0; d < 3; d++) par[d] += mn[d];
    } else
    // trgrid_global (Core/Search.cpp:934-1043)
    if (p.basin_radius != 0.0) {
      double displ_max = p.disp_max;
      int num_inc = (int)(displ_max / p.basin_radius);
      double inc = displ_max / num_inc;
      double obj_min = std::numeric_limits<double>::max();
      int mnx = 0, mny = 0, mnz = 0;
      double pc[3];
      for (int z = -num_inc; z <= num_inc; z++)
        for (int y = -num_inc; y <= num_inc; y++)
          for (int x = -num_inc; x <= num_inc; x++) {
            pc[0] = par[0] + (double)x * inc;
            pc[1] = par[1] + (double)y * inc;
            pc[2] = par[2] + (double)z * inc;
            double o;
            if (!obj_val_at(pc, 3, o, nullptr)) return DVC_RANGE_FAIL;
            if (o < obj_min) {
              obj_min = o;
              mnx = x;
              mny = y;
              mnz = z;
            }
          }
      par[0] += (double)mnx * inc;
      par[1] += (double)mny * inc;
      par[2] += (double)mnz * inc;
    }

    if (p.refine_method == DVC_REFINE_NELDER_MEAD) {
      // look_with(amoeba, ndof, ftol) (Core/Search.cpp:379-440): simplex
      // steps 0.2 in every parameter; ftol 1e-5 for 3 dof, else 1e-7
      double best[12], objf;
      int nf = 0;
      const int st = nelder_mead(par.data(), ndof, ndof == 3 ? 0.00001 : 0.0000001, best, nf);
      if (iters_out) *iters_out = nf;
      if (st != DVC_POINT_GOOD) return st;
      // final objective (Core/Search.cpp:187)
      if (!obj_val_at(best, ndof, objf, nullptr)) return DVC_RANGE_FAIL;
      for (int i = 0; i < 12; i++) par_out[i] = i < ndof ? best[i] : 0.0;
      obj_out = objf;
      return DVC_POINT_GOOD;
    }

    // min_Lev_Mar(par, 1e-6, 0.01) (Core/Search.cpp:194-246) with the
    // forward-difference Jacobian of LM_prep_at (:490-525)
    const int npts = subv_num;
    std::vector<double> jump(par), base_res(npts), step_res(npts), J((size_t)npts * ndof),
        step(ndof);
    double update[12] = {0}, obj_old = 0.0;
    int nits = 20;
    for (int it = 0; it < 20; it++) {
      double obj;
      if (!obj_val_at(jump.data(), ndof, obj, &base_res)) return DVC_RANGE_FAIL;
      const double h = 1E-10;
      for (int i = 0; i < ndof; i++) {
        step = jump;
        step[i] += h;
        double o2;
        if (!obj_val_at(step.data(), ndof, o2, &step_res)) return DVC_RANGE_FAIL;
        for (int j = 0; j < npts; j++) J[(size_t)j * ndof + i] = (step_res[j] - base_res[j]) / h;
      }
      if (it > 0) {
        double del_obj = std::fabs(obj - obj_old);
        double del_mag =
            std::sqrt(update[0] * update[0] + update[1] * update[1] + update[2] * update[2]);
        if ((del_obj < 1e-6) || (del_mag < 0.01)) {
          nits = it;
          break;
        }
      }
      // JTJ = J^T J, JTe = J^T e (column-major product order of the shim:
      // sum over samples ascending), update = QR solve of JTJ u = -JTe
      std::vector<double> JTJ((size_t)ndof * ndof, 0.0), mJTe(ndof, 0.0);
      for (int a = 0; a < ndof; a++)
        for (int b = 0; b < ndof; b++) {
          double s = 0.0;
          for (int j = 0; j < npts; j++) s += J[(size_t)j * ndof + a] * J[(size_t)j * ndof + b];
          JTJ[(size_t)a * ndof + b] = s;
        }
      for (int a = 0; a < ndof; a++) {
        double s = 0.0;
        for (int j = 0; j < npts; j++) s += J[(size_t)j * ndof + a] * base_res[j];
        mJTe[a] = -s;
      }
      qr_solve(ndof, ndof, JTJ.data(), mJTe.data(), update, false);
      for (int i = 0; i < ndof; i++) jump[i] += update[i];
      obj_old = obj;
    }
    gn_iters += nits;
    if (iters_out) *iters_out = nits;
    // final objective (Core/Search.cpp:187)
    double objf;
    if (!obj_val_at(jump.data(), ndof, objf, nullptr)) return DVC_RANGE_FAIL;
    for (int i = 0; i < 12; i++) par_out[i] = i < ndof ? jump[i] : 0.0;
    obj_out = objf;
    return DVC_POINT_GOOD;
  }
};

}  // namespace

// ================================================================ C API ====
extern "C" {

// Search::process_point over points in `order` (Core/dvc.cpp:233-303), with
// starting_param (Core/Search.cpp:277-377) in DVC_SEED_NEIGHBOURS mode.
int oracle_process(const dvc_params *p, const void *ref_vox, const void *cor_vox, int n_points,
                   const double *points, int n_process, const int *order, int n_neigh,
                   const int *neigh, int seed_mode, const double *seeds, int *status,
                   double *objmin, double *params, int *gn_iters, long long *n_evals,
                   long long *undefined_evals, int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  Search S(*p, ref_vox, cor_vox);
  for (int i = 0; i < n_points; i++) {
    status[i] = DVC_NOT_SEARCH;
    objmin[i] = 0.0;
    for (int k = 0; k < 12; k++) params[(size_t)i * 12 + k] = 0.0;
    if (gn_iters) gn_iters[i] = 0;
  }
  for (int i = 0; i < n_process; i++) {
    const int n = order ? order[i] : i;
    double seed[3];
    if (seed_mode == DVC_SEED_GIVEN) {
      for (int d = 0; d < 3; d++) seed[d] = seeds[(size_t)n * 3 + d];
    } else {
      double sx = 0.0, sy = 0.0, sz = 0.0;
      int good = 0;
      if (seed_mode == DVC_SEED_NEIGHBOURS)
        for (int j = 0; j < n_neigh; j++) {
          int m = neigh[(size_t)n * n_neigh + j];
          if (status[m] == DVC_POINT_GOOD) {
            sx += params[(size_t)m * 12 + 0];
            sy += params[(size_t)m * 12 + 1];
            sz += params[(size_t)m * 12 + 2];
            good += 1;
          }
        }
      if (good != 0) {
        seed[0] = sx / good;
        seed[1] = sy / good;
        seed[2] = sz / good;
      } else {
        for (int d = 0; d < 3; d++) seed[d] = p->rigid_trans[d];
      }
    }
    double par[12], obj = 0.0;
    int it = 0;
    int st = S.process_point(&points[(size_t)n * 3], seed, par, obj, &it);
    status[n] = st;
    if (st == DVC_POINT_GOOD) {
      objmin[n] = obj;
      for (int k = 0; k < 12; k++) params[(size_t)n * 12 + k] = par[k];
      if (gn_iters) gn_iters[n] = it;
    }
  }
  if (n_evals) *n_evals = S.evals;
  if (undefined_evals) *undefined_evals = S.interp_ref->undefined_evals + S.interp_cor->undefined_evals;
  return 0;
}

// Interpolate::center_on + kernels + nearest/tri_lin/tri_cub_Lek for one
// volume, with the interpolation box of the search (Core/Search.cpp:66-80).
// Returns 0, or DVC_E_RANGE on Intrp_Fail.
int oracle_interpolate(const dvc_params *p, const void *vox, const double center[3], int n,
                       const double *pts, int interp_type, double *out,
                       long long *undefined_evals) {
  Search S(*p, vox, vox);
  Interp &I = *S.interp_ref;
  I.center_on(center);
  I.load(S.ref);
  std::vector<double> P(pts, pts + (size_t)n * 3), o((size_t)n);
  double mn[3] = {9999.99, 9999.99, 9999.99}, mx[3] = {-9999.99, -9999.99, -9999.99};
  for (int s = 0; s < n; s++)
    for (int d = 0; d < 3; d++) {
      mn[d] = std::min(mn[d], P[(size_t)s * 3 + d]);
      mx[d] = std::max(mx[d], P[(size_t)s * 3 + d]);
    }
  if (!I.interp(interp_type, P, mn, mx, o)) return DVC_E_RANGE;
  for (int s = 0; s < n; s++) out[s] = o[(size_t)s];
  if (undefined_evals) *undefined_evals = I.undefined_evals;
  return 0;
}

double oracle_objective(int fcn, int n, const double *ref, const double *tar, double *residual) {
  std::vector<double> r(ref, ref + n), t(tar, tar + n), res((size_t)n);
  double o = objective(fcn, r, t, residual ? &res : nullptr);
  if (residual)
    for (int i = 0; i < n; i++) residual[i] = res[(size_t)i];
  return o;
}

// The 64x64 Lekien inverse as built above (row-major), for tests.
void oracle_lekien_matrix(double *out) {
  for (int r = 0; r < 64; r++)
    for (int c = 0; c < 64; c++) out[r * 64 + c] = bi().m[r][c];
}

// Lekien coefficients of cells of the interpolation box centred on `center`
// (Interpolate::kernels_Lekien_one). cells [n*3] box-local cell indices.
int oracle_lekien_coefficients(const dvc_params *p, const void *vox, const double center[3], int n,
                               const int *cells, double *coef) {
  Search S(*p, vox, vox);
  Interp &I = *S.interp_ref;
  I.center_on(center);
  I.load(S.ref);
  for (int s = 0; s < n; s++) {
    int x = cells[s * 3], y = cells[s * 3 + 1], z = cells[s * 3 + 2];
    if (x < 0 || y < 0 || z < 0 || x > I.n[0] - 2 || y > I.n[1] - 2 || z > I.n[2] - 2)
      return DVC_E_ARG;
    I.lekien_one(x, y, z);
    for (int k = 0; k < 64; k++) coef[(size_t)s * 64 + k] = I.co[I.vi(x, y, z) * 64 + k];
  }
  return 0;
}

// Sample cloud of one point (Core/Search.cpp:100-119 + FloatingCloud ctors):
// positions [subv_num*3]. Returns subv_num.
int oracle_sample_cloud(const dvc_params *p, const double pt[3], double *out) {
  Search S(*p, nullptr, nullptr);
  if (p->subvol_geom == DVC_SPHERE) {
    S.fc.sphere(pt, S.subv_rad, S.subv_num, p->subvol_aspect, p->sphere_seed);
  } else {
    double smn[3], smx[3];
    for (int d = 0; d < 3; d++) {
      smn[d] = pt[d] + (-S.subv_rad * p->subvol_aspect[d]);
      smx[d] = pt[d] + (S.subv_rad * p->subvol_aspect[d]);
    }
    S.fc.cube(smn, smx, (int)ceil(pow((double)S.subv_num, 1.0 / 3.0)));
  }
  if (out)
    for (size_t i = 0; i < S.fc.stable.size(); i++) out[i] = S.fc.stable[i];
  return (int)(S.fc.stable.size() / 3);
}

// FloatingCloud::affine_to for one parameter vector: moved positions and bbox.
void oracle_affine(const dvc_params *p, const double pt[3], const double *x, int ndof,
                   double *moved, double *bbox6) {
  Search S(*p, nullptr, nullptr);
  int n = oracle_sample_cloud(p, pt, nullptr);
  (void)n;
  if (p->subvol_geom == DVC_SPHERE) {
    S.fc.sphere(pt, S.subv_rad, S.subv_num, p->subvol_aspect, p->sphere_seed);
  } else {
    double smn[3], smx[3];
    for (int d = 0; d < 3; d++) {
      smn[d] = pt[d] + (-S.subv_rad * p->subvol_aspect[d]);
      smx[d] = pt[d] + (S.subv_rad * p->subvol_aspect[d]);
    }
    S.fc.cube(smn, smx, (int)ceil(pow((double)S.subv_num, 1.0 / 3.0)));
  }
  S.fc.affine_to(x, ndof);
  for (size_t i = 0; i < S.fc.moving.size(); i++) moved[i] = S.fc.moving[i];
  for (int d = 0; d < 3; d++) {
    bbox6[d] = S.fc.mbmn[d];
    bbox6[3 + d] = S.fc.mbmx[d];
  }
}

// DataCloud::sort_order_neighbors (Core/DataCloud.cpp:69-144): processing
// order by distance from `start`, and the n_neigh nearest points of every
// point, both by std::sort on (index, distance) records as the reference.
struct DualSortRec {
  int index;
  double value;
};
static bool by_value(const DualSortRec &a, const DualSortRec &b) { return a.value < b.value; }
static double pt_dist(const double *a, const double *b) {
  return sqrt(pow(a[0] - b[0], 2) + pow(a[1] - b[1], 2) + pow(a[2] - b[2], 2));
}
int oracle_order_neighbours(int n, const double *pts, const double start[3], int n_neigh,
                            int *order, int *neigh) {
  std::vector<DualSortRec> rec((size_t)n);
  for (int i = 0; i < n; i++) {
    rec[(size_t)i].index = i;
    rec[(size_t)i].value = pt_dist(start, &pts[(size_t)i * 3]);
  }
  std::sort(rec.begin(), rec.end(), by_value);
  for (int i = 0; i < n; i++) order[i] = rec[(size_t)i].index;
  const int keep = std::min(n_neigh, n);
#pragma omp parallel
  {
    std::vector<DualSortRec> r2((size_t)n);
#pragma omp for
    for (int i = 0; i < n; i++) {
      for (int j = 0; j < n; j++) {
        r2[(size_t)j].index = j;
        r2[(size_t)j].value = pt_dist(&pts[(size_t)i * 3], &pts[(size_t)j * 3]);
      }
      std::sort(r2.begin(), r2.end(), by_value);
      for (int j = 0; j < keep; j++) neigh[(size_t)i * keep + j] = r2[(size_t)j].index;
    }
  }
  return keep;
}

// Strain-window fit of the `strain` executable (Core/strain.cpp:402-591).
int oracle_strain(int n, const double *pts, const int *status, const double *objmin,
                  const double *disp, int n_neigh, const int *neigh, int ndp, double objt,
                  int refill, int planar, double *u_fit, int *pts_in_sw, double *sw_radius,
                  double *e_strain, double *l_strain, double *dgrad) {
  const bool yz_only = planar & 1, zx_only = planar & 2, xy_only = planar & 4;
  const int nmp = 10;
  for (int i = 0; i < n; i++) {
    const int *nb = &neigh[(size_t)i * n_neigh];
    const double origin[3] = {0.0, 0.0, 0.0};
    double distance = pt_dist(&pts[(size_t)i * 3], origin);
    double scale = 1.0 / distance;
    double base[3] = {scale * pts[(size_t)i * 3], scale * pts[(size_t)i * 3 + 1],
                      scale * pts[(size_t)i * 3 + 2]};
    std::vector<double> npos, ndis;
    auto take = [&](int m) {
      for (int d = 0; d < 3; d++) npos.push_back(scale * pts[(size_t)m * 3 + d]);
      for (int d = 0; d < 3; d++) ndis.push_back(scale * disp[(size_t)m * 3 + d]);
    };
    if (!refill) {
      for (int j = 0; j < ndp && j < n_neigh; j++) {
        int m = nb[j];
        if (status[m] == 0 && objmin[m] <= objt) take(m);
      }
    } else {
      int indx = 0, np = 0;
      while (np < ndp && indx < n_neigh) {
        int m = nb[indx];
        if (status[m] == 0 && objmin[m] <= objt) {
          take(m);
          np += 1;
        }
        indx += 1;
      }
    }
    const int ngp = (int)(npos.size() / 3);
    pts_in_sw[i] = ngp;
    if (ngp == 0) {
      sw_radius[i] = 0.0;
    } else {
      sw_radius[i] = distance * pt_dist(base, &npos[(size_t)(ngp - 1) * 3]);
    }
    std::vector<double> Xm((size_t)ngp * nmp), dvs((size_t)ngp * 3);
    for (int j = 0; j < ngp; j++) {
      const double *q = &npos[(size_t)j * 3];
      double *X = &Xm[(size_t)j * nmp];
      X[0] = 1;
      X[1] = q[0];
      X[2] = q[1];
      X[3] = q[2];
      X[4] = q[0] * q[0];
      X[5] = q[1] * q[1];
      X[6] = q[2] * q[2];
      X[7] = q[0] * q[1];
      X[8] = q[1] * q[2];
      X[9] = q[0] * q[2];
      for (int d = 0; d < 3; d++) dvs[(size_t)j * 3 + d] = ndis[(size_t)j * 3 + d];
      if (yz_only) {
        X[1] = X[4] = X[7] = X[9] = 0.0;
        dvs[(size_t)j * 3 + 0] = 0.0;
      }
      if (zx_only) {
        X[2] = X[5] = X[7] = X[8] = 0.0;
        dvs[(size_t)j * 3 + 1] = 0.0;
      }
      if (xy_only) {
        X[3] = X[6] = X[8] = X[9] = 0.0;
        dvs[(size_t)j * 3 + 2] = 0.0;
      }
    }
    double XtX[100];
    for (int a = 0; a < nmp; a++)
      for (int b = 0; b < nmp; b++) {
        double s = 0.0;
        for (int j = 0; j < ngp; j++) s += Xm[(size_t)j * nmp + a] * Xm[(size_t)j * nmp + b];
        XtX[a * nmp + b] = s;
      }
    double DG[3][3], displ[3];
    for (int c = 0; c < 3; c++) {
      double rhs[10], par[10];
      for (int a = 0; a < nmp; a++) {
        double s = 0.0;
        for (int j = 0; j < ngp; j++) s += Xm[(size_t)j * nmp + a] * dvs[(size_t)j * 3 + c];
        rhs[a] = s;
      }
      qr_solve(nmp, nmp, XtX, rhs, par, true);
      DG[c][0] = par[1] + 2 * par[4] * base[0] + par[7] * base[1] + par[9] * base[2];
      DG[c][1] = par[2] + 2 * par[5] * base[1] + par[7] * base[0] + par[8] * base[2];
      DG[c][2] = par[3] + 2 * par[6] * base[2] + par[8] * base[1] + par[9] * base[0];
      displ[c] = distance * (par[0] + par[1] * base[0] + par[2] * base[1] + par[3] * base[2] +
                             par[4] * base[0] * base[0] + par[5] * base[1] * base[1] +
                             par[6] * base[2] * base[2] + par[7] * base[0] * base[1] +
                             par[8] * base[1] * base[2] + par[9] * base[0] * base[2]);
    }
    for (int c = 0; c < 3; c++) u_fit[(size_t)i * 3 + c] = displ[c];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) dgrad[(size_t)i * 9 + a * 3 + b] = DG[a][b];
    // engineering and Lagrangian strain, principal values sorted descending
    // (Core/strain.cpp:550-590); symmetric 3x3 eigenvalues by cyclic Jacobi
    for (int which = 0; which < 2; which++) {
      double ST[3][3];
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
          ST[a][b] = 0.5 * (DG[a][b] + DG[b][a]);
          if (which == 1) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += DG[k][a] * DG[k][b];
            ST[a][b] = 0.5 * (DG[a][b] + DG[b][a] + s);
          }
        }
      double s[3][3];
      std::memcpy(s, ST, sizeof s);
      for (int sweep = 0; sweep < 64; sweep++) {
        double off = s[0][1] * s[0][1] + s[0][2] * s[0][2] + s[1][2] * s[1][2];
        if (off == 0.0) break;
        for (int pp = 0; pp < 3; pp++)
          for (int qq = pp + 1; qq < 3; qq++) {
            double apq = s[pp][qq];
            if (apq == 0.0) continue;
            double theta = (s[qq][qq] - s[pp][pp]) / (2.0 * apq);
            double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
            double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
            for (int k = 0; k < 3; k++) {
              double skp = s[k][pp], skq = s[k][qq];
              s[k][pp] = c * skp - sn * skq;
              s[k][qq] = sn * skp + c * skq;
            }
            for (int k = 0; k < 3; k++) {
              double spk = s[pp][k], sqk = s[qq][k];
              s[pp][k] = c * spk - sn * sqk;
              s[qq][k] = sn * spk + c * sqk;
            }
          }
      }
      double lam[3] = {s[0][0], s[1][1], s[2][2]};
      std::sort(lam, lam + 3);
      std::reverse(lam, lam + 3);
      if (xy_only || yz_only || zx_only) {
        if (lam[0] == 0.0) {
          lam[0] = lam[1];
          lam[1] = lam[2];
        }
        if (lam[1] == 0.0) lam[1] = lam[2];
        lam[2] = 0.0;
      }
      double *o = (which == 0 ? e_strain : l_strain) + (size_t)i * 9;
      o[0] = ST[0][0];
      o[1] = ST[1][1];
      o[2] = ST[2][2];
      o[3] = ST[0][1];
      o[4] = ST[1][2];
      o[5] = ST[0][2];
      o[6] = lam[0];
      o[7] = lam[1];
      o[8] = lam[2];
    }
  }
  return 0;
}

}  // extern "C"
