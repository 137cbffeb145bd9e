// The binding a maintainer of the reference adds to its programs: in `dvc`
// (Core/dvc.cpp, after data.organize_cloud(&run) at :150) every point of the
// run searched by the GPU engine, data.results filled as the catch blocks of
// :250-283 fill them; in `strain` (Core/strain.cpp) the per-point loop of
// :402-591 replaced by the GPU fit, its results stored where the loop stores
// them. Compiled against the reference's own headers (Utility.h,
// DataCloud.h) by the CPU tests where those are present; it is not part of
// this library's build.
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

#include <Eigen/Dense>

#include "DataCloud.h"
#include "Utility.h"
#include "dvc_gpu.h"

// a raw volume file, its header skipped
static std::vector<char> read_raw(const std::string &fname, int header_bytes) {
  std::ifstream s(fname, std::ios::binary);
  s.seekg(header_bytes);
  return std::vector<char>((std::istreambuf_iterator<char>(s)), std::istreambuf_iterator<char>());
}

// N: the points to process (the reference's num_points_to_process rule);
// returns 0 after printing the engine's message when the engine cannot be
// created, as the reference's input errors do
int dvc_search_on_gpu(RunControl &run, DataCloud &data, int N) {
  // RunControl -> dvc_params (field meaning as Core/Utility.h:90-134)
  dvc_params p = {};
  p.vol_wide = run.vol_wide; p.vol_high = run.vol_high; p.vol_tall = run.vol_tall;
  p.bytes_per_voxel = run.vol_bit_depth / 8;
  p.subvol_geom = run.sub_geo;            // cube 0, sphere 1 (Core/Utility.h:61)
  p.subvol_size = run.subvol_size;  p.subvol_npts = run.subvol_npts;
  for (int d = 0; d < 3; d++) { p.subvol_aspect[d] = run.subvol_aspect[d]; p.rigid_trans[d] = run.rigid_trans[d]; }
  p.disp_max = run.disp_max;  p.num_srch_dof = run.num_srch_dof;
  p.obj_function = run.obj_fcn;  p.interp_type = run.int_typ;
  p.basin_radius = run.basin_radius;  p.sphere_seed = 1;   // the reference's reproducible test seed

  std::vector<char> ref = read_raw(run.ref_fname, run.vol_hdr_lngth), cor = read_raw(run.cor_fname, run.vol_hdr_lngth);
  dvc_engine *eng = nullptr;
  if (dvc_gpu_create(&eng, &p, ref.data(), cor.data(), run.vol_endian == "big") != DVC_OK)
    { std::cout << dvc_gpu_last_error() << "\n"; return 0; }

  const int n = data.points.size();
  std::vector<double> pts(3 * n);
  for (int i = 0; i < n; i++) { pts[3*i] = data.points[i].x(); pts[3*i+1] = data.points[i].y(); pts[3*i+2] = data.points[i].z(); }
  std::vector<int> neigh; const int nn = data.neigh[0].size();
  for (auto &row : data.neigh) neigh.insert(neigh.end(), row.begin(), row.end());
  std::vector<int> status(n); std::vector<double> objmin(n), par(12 * n);
  dvc_gpu_process(eng, n, pts.data(), N /* points to process */, data.order.data(), nn, neigh.data(),
                  DVC_SEED_NEIGHBOURS, nullptr, status.data(), objmin.data(), par.data(), nullptr, nullptr);
  for (int i = 0; i < N; i++) {                       // what the catch blocks of :250-283 record
    int m = data.order[i];
    data.results[0][m].status = status[m];
    if (status[m] == DVC_POINT_GOOD) {
      data.results[0][m].obj_min = objmin[m];
      for (int j = 0; j < run.num_srch_dof; j++) data.results[0][m].par_min[j] = par[12 * m + j];
    }
  }
  dvc_gpu_destroy(eng);
  return 1;
}

// The strain program's per-point loop on the GPU (dvc_gpu_strain: the same
// window rules and fit). status, objmin, dis: the .disp columns as the
// program reads them (:298-300); planar: bit 0 yz_only, bit 1 zx_only, bit 2
// xy_only. Fills data.pts_in_sw, data.sw_rad, data.dis_vfit, data.Estrain,
// data.Lstrain and DG_all_pts as the loop does, so the output code of
// :593-656 runs unchanged.
int dvc_strain_on_gpu(DataCloud &data, const std::vector<int> &status, const std::vector<double> &objmin,
                      const std::vector<Point> &dis, int ndp, double objt, bool refill, int planar,
                      std::vector<Eigen::MatrixXd> &DG_all_pts) {
  const int n = data.points.size();
  const int nn = data.neigh[0].size();
  std::vector<double> pts(3 * n), disp(3 * n);
  for (int i = 0; i < n; i++) {
    pts[3 * i] = data.points[i].x(); pts[3 * i + 1] = data.points[i].y(); pts[3 * i + 2] = data.points[i].z();
    disp[3 * i] = dis[i].x(); disp[3 * i + 1] = dis[i].y(); disp[3 * i + 2] = dis[i].z();
  }
  std::vector<int> neigh;
  for (auto &row : data.neigh) neigh.insert(neigh.end(), row.begin(), row.end());
  std::vector<double> u(3 * n), rad(n), E(9 * n), L(9 * n), D(9 * n);
  std::vector<int> pis(n);
  if (dvc_gpu_strain(n, pts.data(), status.data(), objmin.data(), disp.data(), nn, neigh.data(), ndp, objt,
                     refill ? 1 : 0, planar, u.data(), pis.data(), rad.data(), E.data(), L.data(), D.data()) != DVC_OK)
    { std::cout << dvc_gpu_last_error() << "\n"; return 0; }
  for (int i = 0; i < n; i++) {
    data.pts_in_sw.push_back(pis[i]);
    data.sw_rad.push_back(rad[i]);
    data.dis_vfit.push_back({u[3 * i], u[3 * i + 1], u[3 * i + 2]});
    data.Estrain.push_back(std::vector<double>(E.begin() + 9 * i, E.begin() + 9 * i + 9));
    data.Lstrain.push_back(std::vector<double>(L.begin() + 9 * i, L.begin() + 9 * i + 9));
    Eigen::MatrixXd DG(3, 3);
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) DG(r, c) = D[9 * i + 3 * r + c];  // row-major du_r / dx_c
    DG_all_pts.push_back(DG);
  }
  return 1;
}
