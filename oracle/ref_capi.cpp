// ref_capi.cpp — C entry points that drive the reference's own classes.
//
// TEST INFRASTRUCTURE ONLY. oracle/build_ref.sh compiles this file together
// with the reference sources (Core/*.cpp, unmodified, read where they lie)
// into oracle/_ref/libdvcref.so, so tests can run the reference itself on the
// same inputs as the oracle restatement and the GPU engine. The reference
// reads volumes from raw files (Interpolate::kernels, Core/Interpolate.cpp:144),
// so these functions take file names.
#include "DataCloud.h"
#include "InputRead.h"
#include "ObjectiveFunctions.h"
#include "Search.h"

#include <time.h>

#include "../include/dvc_gpu.h"

// Search::random_global seeds the C library's generator from the clock
// (srand(time(NULL)), Core/Search.cpp:1060). While g_fixed_clock >= 0 this
// library's time() returns it instead, so the reference's own draws are
// reproducible; build_ref.sh links libdvcref.so with -Bsymbolic-functions,
// which binds the reference's call to this definition (the reference's own
// `dvc` and `strain` programs do not contain this file).
static long long g_fixed_clock = -1;
extern "C" time_t time(time_t *t) noexcept {
  time_t v;
  if (g_fixed_clock >= 0) {
    v = (time_t)g_fixed_clock;
  } else {
    struct timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    v = ts.tv_sec;
  }
  if (t) *t = v;
  return v;
}

namespace {
void fill_run(RunControl &run, const dvc_params *p, const char *ref_file, const char *cor_file,
              int hdr, const char *endian) {
  run.ref_fname = ref_file ? ref_file : "";
  run.cor_fname = cor_file ? cor_file : "";
  run.vol_bit_depth = 8 * p->bytes_per_voxel;
  run.vol_endian = endian ? endian : "little";
  run.vol_hdr_lngth = hdr;
  run.vol_wide = p->vol_wide;
  run.vol_high = p->vol_high;
  run.vol_tall = p->vol_tall;
  run.sub_geo = (Subvol_Type)p->subvol_geom;
  run.subvol_geom = p->subvol_geom == 0 ? "cube" : "sphere";
  run.subvol_size = p->subvol_size;
  run.subvol_npts = p->subvol_npts;
  run.subvol_thresh = "off";
  run.disp_max = p->disp_max;
  run.num_srch_dof = p->num_srch_dof;
  run.num_points_to_process = 0;
  run.obj_fcn = (Objfcn_Type)p->obj_function;
  run.int_typ = (Interp_Type)p->interp_type;
  run.rigid_trans = {p->rigid_trans[0], p->rigid_trans[1], p->rigid_trans[2]};
  run.basin_radius = p->basin_radius;
  run.subvol_aspect = {p->subvol_aspect[0], p->subvol_aspect[1], p->subvol_aspect[2]};
  run.starting_point = {std::nan(""), std::nan(""), std::nan("")};
}
}  // namespace

extern "C" {

int ref_interpolate(const dvc_params *p, const char *vol_file, int hdr, const char *endian,
                    const double center[3], int n, const double *pts, int interp_type,
                    double *out) {
  RunControl run;
  fill_run(run, p, vol_file, vol_file, hdr, endian);
  run.int_typ = (Interp_Type)interp_type;
  Search S(&run);
  Point c(center[0], center[1], center[2]);
  S.interp->center_on(c);
  S.interp->kernels(vol_file, S.vox_box, S.bytes_per, run.vol_endian, (unsigned)hdr);
  Cloud cl;
  for (int i = 0; i < n; i++) cl.AddPoint(Point(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]));
  std::vector<double> vals((size_t)n, 0.0);
  try {
    if (interp_type == 0) S.interp->nearest(cl.ptvect, cl.bbox(), vals);
    if (interp_type == 1) S.interp->tri_lin(cl.ptvect, cl.bbox(), vals);
    if (interp_type == 2) S.interp->tri_cub_Lek(cl.ptvect, cl.bbox(), vals);
  } catch (Intrp_Fail) {
    return DVC_E_RANGE;
  }
  for (int i = 0; i < n; i++) out[i] = vals[(size_t)i];
  return 0;
}

double ref_objective(int fcn, int n, const double *ref, const double *tar, double *residual) {
  std::vector<double> r(ref, ref + n), t(tar, tar + n), res((size_t)n, 0.0);
  double (*f)(const std::vector<double> &, const std::vector<double> &, std::vector<double> &) =
      nullptr;
  if (fcn == 0) f = &obj_SAD;
  if (fcn == 1) f = &obj_SSD;
  if (fcn == 2) f = &obj_ZSSD;
  if (fcn == 3) f = &obj_NSSD;
  if (fcn == 4) f = &obj_ZNSSD;
  double o = f(r, t, res);
  if (residual)
    for (int i = 0; i < n; i++) residual[i] = res[(size_t)i];
  return o;
}

// The loop of Core/dvc.cpp:233-303 with Search::process_point(..., test=1)
// (fixed sphere seed, Core/Search.cpp:102-105).
int ref_process(const dvc_params *p, const char *ref_file, const char *cor_file, int hdr,
                const char *endian, int n_points, const double *points, int n_process,
                const int *order, int n_neigh, const int *neigh, int *status, double *objmin,
                double *params) {
  RunControl run;
  fill_run(run, p, ref_file, cor_file, hdr, endian);
  DataCloud data;
  for (int i = 0; i < n_points; i++) {
    data.points.push_back(Point(points[i * 3], points[i * 3 + 1], points[i * 3 + 2]));
    data.labels.push_back(i + 1);
  }
  data.order.assign(order, order + n_process);
  data.neigh.resize((size_t)n_points);
  for (int i = 0; i < n_points; i++)
    data.neigh[(size_t)i].assign(neigh + (size_t)i * n_neigh, neigh + (size_t)(i + 1) * n_neigh);
  data.results.resize(1);
  data.results[0].resize((size_t)n_points);
  for (auto &r : data.results[0]) {
    r.status = not_search;
    r.obj_min = 0.0;
    r.par_min.assign((size_t)run.num_srch_dof, 0.0);
  }
  std::streambuf *old = std::cout.rdbuf(nullptr);  // silence per-point chatter
  Search optimize(&run);
  for (int i = 0; i < n_process; i++) {
    int n = data.order[(size_t)i];
    try {
      optimize.process_point(0, n, &data, 1);
    } catch (Point_Good) {
      data.results[0][(size_t)n].status = point_good;
      data.results[0][(size_t)n].obj_min = optimize.obj_min;
      for (int j = 0; j < run.num_srch_dof; j++)
        data.results[0][(size_t)n].par_min[(size_t)j] = optimize.par_min[(size_t)j];
    } catch (Range_Fail) {
      data.results[0][(size_t)n].status = range_fail;
    } catch (Convg_Fail) {
      data.results[0][(size_t)n].status = convg_fail;
    }
  }
  std::cout.rdbuf(old);
  for (int i = 0; i < n_points; i++) {
    const ResultRecord &r = data.results[0][(size_t)i];
    status[i] = r.status;
    objmin[i] = r.obj_min;
    for (int k = 0; k < 12; k++)
      params[(size_t)i * 12 + k] = k < (int)r.par_min.size() ? r.par_min[(size_t)k] : 0.0;
  }
  return 0;
}

// The body of Search::process_point (Core/Search.cpp:95-192, test seed 1 for
// spheres) with the stages its source holds but never selects switched in:
// random_global (:1045-1098) in place of trgrid_global when
// p->coarse_method is DVC_COARSE_RANDOM (the clock fixed at p->coarse_seed),
// and look_with(amoeba, ndof, ftol) with the ftol of :163-165 in place of
// min_Lev_Mar when p->refine_method is DVC_REFINE_NELDER_MEAD. Throws the
// reference's status exceptions as process_point does.
static void run_point(Search &S, const dvc_params *p, int n, DataCloud *data) {
  RunControl *rc = S.rc;
  Point srch_pt = data->points[(size_t)n];
  if (rc->sub_geo == sphere)
    S.fcld = new FloatingCloud(srch_pt, S.subv_rad, S.subv_num, rc->subvol_aspect[0], rc->subvol_aspect[1],
                               rc->subvol_aspect[2], 1);
  if (rc->sub_geo == Subvol_Type::cube) {
    Point sub_min = srch_pt, sub_max = srch_pt;
    sub_min.move_by(-S.subv_rad * rc->subvol_aspect[0], -S.subv_rad * rc->subvol_aspect[1],
                    -S.subv_rad * rc->subvol_aspect[2]);
    sub_max.move_by(S.subv_rad * rc->subvol_aspect[0], S.subv_rad * rc->subvol_aspect[1],
                    S.subv_rad * rc->subvol_aspect[2]);
    int grid_inc = ceil(pow((double)S.subv_num, 1.0 / 3.0));
    S.fcld = new FloatingCloud(sub_min, sub_max, grid_inc, grid_inc, grid_inc);
  }
  std::vector<ResultRecord> neigh_res;
  for (size_t i = 0; i < data->neigh[(size_t)n].size(); i++)
    neigh_res.push_back(data->results[0][(size_t)data->neigh[(size_t)n][i]]);
  S.search_pt_setup(srch_pt, neigh_res);
  if (p->coarse_method == DVC_COARSE_RANDOM) {
    g_fixed_clock = p->coarse_seed;
    try {
      S.random_global(rc->disp_max, rc->basin_radius);
    } catch (...) {
      g_fixed_clock = -1;
      throw;
    }
    g_fixed_clock = -1;
  } else {
    S.trgrid_global(rc->disp_max, rc->basin_radius, n);
  }
  const int ndof = (int)S.par_min.size();
  if (p->refine_method == DVC_REFINE_NELDER_MEAD) {
    S.look_with(amoeba, ndof, ndof == 3 ? 0.00001 : 0.0000001);
  } else {
    std::vector<double> jump = S.min_Lev_Mar(S.par_min, 0.000001, 0.01);
    for (int i = 0; i < ndof; i++) S.par_min[(size_t)i] = jump[(size_t)i];
  }
  S.obj_min = S.obj_val_at(S.par_min);
  delete S.fcld;
  throw Point_Good();
}

// ref_process with the search stages of p->coarse_method / p->refine_method
int ref_process_stages(const dvc_params *p, const char *ref_file, const char *cor_file, int hdr,
                       const char *endian, int n_points, const double *points, int n_process,
                       const int *order, int n_neigh, const int *neigh, int *status, double *objmin,
                       double *params) {
  RunControl run;
  fill_run(run, p, ref_file, cor_file, hdr, endian);
  DataCloud data;
  for (int i = 0; i < n_points; i++) {
    data.points.push_back(Point(points[i * 3], points[i * 3 + 1], points[i * 3 + 2]));
    data.labels.push_back(i + 1);
  }
  data.order.assign(order, order + n_process);
  data.neigh.resize((size_t)n_points);
  for (int i = 0; i < n_points; i++)
    data.neigh[(size_t)i].assign(neigh + (size_t)i * n_neigh, neigh + (size_t)(i + 1) * n_neigh);
  data.results.resize(1);
  data.results[0].resize((size_t)n_points);
  for (auto &r : data.results[0]) {
    r.status = not_search;
    r.obj_min = 0.0;
    r.par_min.assign((size_t)run.num_srch_dof, 0.0);
  }
  std::streambuf *old = std::cout.rdbuf(nullptr);
  Search optimize(&run);
  for (int i = 0; i < n_process; i++) {
    int n = data.order[(size_t)i];
    try {
      run_point(optimize, p, n, &data);
    } catch (Point_Good) {
      data.results[0][(size_t)n].status = point_good;
      data.results[0][(size_t)n].obj_min = optimize.obj_min;
      for (int j = 0; j < run.num_srch_dof; j++)
        data.results[0][(size_t)n].par_min[(size_t)j] = optimize.par_min[(size_t)j];
    } catch (Range_Fail) {
      data.results[0][(size_t)n].status = range_fail;
    } catch (Convg_Fail) {
      data.results[0][(size_t)n].status = convg_fail;
    }
  }
  std::cout.rdbuf(old);
  for (int i = 0; i < n_points; i++) {
    const ResultRecord &r = data.results[0][(size_t)i];
    status[i] = r.status;
    objmin[i] = r.obj_min;
    for (int k = 0; k < 12; k++)
      params[(size_t)i * 12 + k] = k < (int)r.par_min.size() ? r.par_min[(size_t)k] : 0.0;
  }
  return 0;
}

// DataCloud::sort_order_neighbors (Core/DataCloud.cpp:69-144)
int ref_order_neighbours(int n, const double *pts, const double start[3], int *order,
                         int *neigh) {
  DataCloud data;
  for (int i = 0; i < n; i++) data.points.push_back(Point(pts[i * 3], pts[i * 3 + 1], pts[i * 3 + 2]));
  std::streambuf *old = std::cout.rdbuf(nullptr);
  data.sort_order_neighbors(Point(start[0], start[1], start[2]));
  std::cout.rdbuf(old);
  for (int i = 0; i < n; i++) order[i] = data.order[(size_t)i];
  int keep = (int)data.neigh[0].size();
  for (int i = 0; i < n; i++)
    for (int j = 0; j < keep; j++) neigh[(size_t)i * keep + j] = data.neigh[(size_t)i][(size_t)j];
  return keep;
}

}  // extern "C"
