// The binding a maintainer of the reference adds to its `dvc` program
// (Core/dvc.cpp, after data.organize_cloud(&run) at :150): every point of the
// run searched by the GPU engine, data.results filled as the catch blocks of
// :250-283 fill them. Compiled against the reference's own headers
// (Utility.h, DataCloud.h) by the CPU tests where those are present; it is
// not part of this library's build.
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

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
