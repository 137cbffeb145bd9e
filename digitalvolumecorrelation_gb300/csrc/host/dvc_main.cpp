// dvc_main.cpp — the drop-in `dvc` program: same command line, input file,
// point cloud and output files as the reference's `dvc` (Core/dvc.cpp), with
// the per-point search loop (Core/dvc.cpp:233-303) replaced by one call of the
// GPU engine (include/dvc_gpu.h).
//
// Differences from the reference, by design:
//  * sphere subvolumes use one sample set drawn from mt19937 with seed
//    DVC_SPHERE_SEED (default 1, the reference's reproducible test seed) for
//    every point; the reference's normal runs draw a clock-seeded set per point
//    (Core/Search.cpp:100-110), which no two runs reproduce;
//  * `.disp` rows are written once, after the search (the reference appends
//    each row as it goes, then rewrites the file in the same order);
//  * a file name may end its line (the reference needs a tab after it);
//  * with DVC_GPU_NEIGHBOURS set, order and neighbour lists come from the GPU
//    (same distances, ties by point index instead of std::sort's order);
//  * with DVC_SUBVOL_THRESH set, `subvol_thresh on` is applied as the manual
//    documents it (points with too little of the gray range are not searched,
//    status -3); the reference only parses and echoes the keywords, and so
//    does this program without the variable.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "dvc_gpu.h"
#include "host_io.h"

using namespace dvchost;

static const char *kVersion = "dvc-gb300 0.1";

static void usage() {
  std::cout << "\nOptions:\n"
            << "dvc dvc_in\t\t// run the correlation described by the input file dvc_in\n"
            << "dvc help\t\t// what a run needs and what it writes\n"
            << "dvc example\t\t// write dvc_in_example, an input file with every keyword\n"
            << "dvc manual\t\t// write dvc_manual, the keyword reference\n"
            << "dvc version\t\t// print the program version\n\n";
}

int main(int argc, char *argv[]) {
  if (argc == 1) {
    usage();
    return 0;
  }
  const std::string a1(argv[1]);
  if (a1 == "help") {
    std::cout << "\nA run is controlled by a keyword input file: dvc <input file>.\n"
              << "The file names the two raw image volumes, the point cloud and the output base\n"
              << "name, describes the volume layout, the subvolumes and the search; see\n"
              << "`dvc example` and `dvc manual`. The file is checked first and the run stops\n"
              << "with a message at the first problem. The search runs on the GPU; results go to\n"
              << "<output>.disp and run information to <output>.stat.\n\n";
    return 0;
  }
  if (a1 == "example") {
    std::cout << "\ndvc_in_example printed in the current working directory\n\n";
    std::ofstream f("dvc_in_example");
    write_example(f);
    return 0;
  }
  if (a1 == "manual") {
    std::cout << "\ndvc_manual printed in the current working directory\n\n";
    std::ofstream f("dvc_manual");
    write_manual(f);
    return 0;
  }
  if (a1 == "version") {
    std::cout << "CCPi Digital Volume Correlation (GB300 engine) version: " << kVersion << " ("
              << dvc_gpu_version() << ")" << std::endl;
    return 0;
  }

  InputFile in;
  if (!in.open(a1)) return 0;
  RunConfig run;
  if (!in.read(run)) return 0;

  std::vector<int> labels;
  std::vector<double> pts;
  double bmin[3], bmax[3];
  if (!read_roi(run.pts_fname, labels, pts, bmin, bmax)) return 0;
  const int n = (int)labels.size();

  // organize_cloud (Core/DataCloud.cpp:148-174): its test of the
  // starting_point keyword compares the NaN default with NaN, which is never
  // equal, so the keyword's values are used whether given or not (all
  // distances NaN when it is absent, and the order is std::sort's)
  std::vector<int> order;
  std::vector<std::vector<int>> neigh;
  if (std::getenv("DVC_GPU_NEIGHBOURS")) {
    // the GPU path: same distances, ties by point index
    const int kk = std::min(75, n);
    std::vector<int> flat((size_t)n * kk);
    order.resize((size_t)n);
    if (dvc_gpu_order_neighbours(n, pts.data(), run.starting_point, 75, order.data(), flat.data()) != DVC_OK) {
      std::cout << "\nNeighbour search on the GPU failed: " << dvc_gpu_last_error() << "\n\n";
      return 0;
    }
    neigh.assign((size_t)n, std::vector<int>());
    for (int i = 0; i < n; i++) neigh[(size_t)i].assign(flat.begin() + (size_t)i * kk, flat.begin() + (size_t)(i + 1) * kk);
  } else {
    order_neighbours(pts, run.starting_point, 75, order, neigh);
  }
  std::cout << "sorting finished" << std::endl;
  write_sort_csv(run.pts_fname, neigh);

  const long long t_start = (long long)std::time(nullptr);
  write_stat_echo(run, (size_t)n, bmin, bmax, kVersion);
  append_stat_time(run.sta_fname, "Run start: ", t_start);

  const int bpv = run.vol_bit_depth / 8;

  dvc_params p{};
  p.vol_wide = run.vol_wide;
  p.vol_high = run.vol_high;
  p.vol_tall = run.vol_tall;
  p.bytes_per_voxel = bpv;
  p.subvol_geom = run.sub_geo;
  p.subvol_size = run.subvol_size;
  p.subvol_npts = run.subvol_npts;
  for (int d = 0; d < 3; d++) {
    p.subvol_aspect[d] = run.subvol_aspect[d];
    p.rigid_trans[d] = run.rigid_trans[d];
  }
  p.disp_max = run.disp_max;
  p.num_srch_dof = run.num_srch_dof;
  p.obj_function = run.obj_fcn;
  p.interp_type = run.int_typ;
  p.basin_radius = run.basin_radius;
  if (run.subvol_thresh == "on" && std::getenv("DVC_SUBVOL_THRESH")) {
    p.subvol_thresh = 1;
    p.gray_thresh_min = run.gray_thresh_min;
    p.gray_thresh_max = run.gray_thresh_max;
    p.min_vol_fract = run.min_vol_fract;
  }
  const char *seed = std::getenv("DVC_SPHERE_SEED");
  p.sphere_seed = seed ? (unsigned)std::strtoul(seed, nullptr, 10) : 1u;

  // both volumes streamed from their files straight to device memory
  dvc_engine *eng = nullptr;
  if (dvc_gpu_create_from_files(&eng, &p, run.ref_fname.c_str(), run.cor_fname.c_str(), run.vol_hdr_lngth,
                                run.vol_endian == "big" ? 1 : 0) != DVC_OK) {
    std::cout << "\nThe GPU engine could not be set up: " << dvc_gpu_last_error() << "\n\n";
    return 0;
  }

  const char *fcn_names[5] = {"SAD", "SSD", "ZSSD", "NSSD", "ZNSSD"};
  std::cout << "\n\n*************************\nSearch: ( \nSearch(\nbytes_per " << bpv
            << "\nsubv_rad " << run.subvol_size / 2.0 << "\nsubv_num " << run.subvol_npts
            << "\nobj_fun objective function " << fcn_names[run.obj_fcn] << "\ninput shape "
            << run.vol_wide << " " << run.vol_high << " " << run.vol_tall << "\nsubvol aspect "
            << run.subvol_aspect[0] << " " << run.subvol_aspect[1] << " " << run.subvol_aspect[2]
            << "\nnumr_search_dof " << run.num_srch_dof << "\ndisp max " << run.disp_max
            << "\n)\n) \n\n";

  write_disp_header(run.res_fname);
  int N = n;
  if (run.num_points_to_process > 1 && run.num_points_to_process < (unsigned)N)
    N = (int)run.num_points_to_process;

  const int nn = neigh.empty() ? 0 : (int)neigh[0].size();
  std::vector<int> nflat((size_t)n * nn);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < nn; j++) nflat[(size_t)i * nn + j] = neigh[(size_t)i][(size_t)j];
  std::vector<int> status((size_t)n), iters((size_t)n);
  std::vector<double> objmin((size_t)n), par((size_t)n * 12);
  dvc_stats st{};
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = dvc_gpu_process(eng, n, pts.data(), N, order.data(), nn, nflat.data(),
                                 DVC_SEED_NEIGHBOURS, nullptr, status.data(), objmin.data(),
                                 par.data(), iters.data(), &st);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rc != DVC_OK) {
    std::cout << "\nThe GPU search failed: " << dvc_gpu_last_error() << "\n\n";
    dvc_gpu_destroy(eng);
    return 0;
  }
  dvc_gpu_destroy(eng);

  int good = 0, rfail = 0, cfail = 0;
  for (int i = 0; i < N; i++) {
    const int m = order[(size_t)i];
    std::cout << i << "/" << N << " " << labels[(size_t)m] << "\t" << std::setprecision(3)
              << std::fixed << pts[(size_t)m * 3] << " " << pts[(size_t)m * 3 + 1] << " "
              << pts[(size_t)m * 3 + 2] << " \t";
    if (status[(size_t)m] == DVC_POINT_GOOD) {
      good++;
      std::cout << "Point_Good\t" << std::setprecision(6) << "obj= " << objmin[(size_t)m]
                << std::setw(12) << "dx= " << par[(size_t)m * 12] << std::setw(12) << "dy= "
                << par[(size_t)m * 12 + 1] << std::setw(12) << "dz= " << par[(size_t)m * 12 + 2];
    } else if (status[(size_t)m] == DVC_RANGE_FAIL) {
      rfail++;
      std::cout << "Range_Fail";
    } else if (status[(size_t)m] == DVC_NOT_SEARCH) {
      std::cout << "Not_Searched";
    } else {
      cfail++;
      std::cout << "Convg_Fail";
    }
    std::cout << "\n";
  }
  std::cout << N / secs << " pt/sec average" << std::endl;
  std::cout.unsetf(std::ios::floatfield);

  const long long t_finish = (long long)std::time(nullptr);
  // rows in processing order from the stored results, as the reference's final
  // rewrite (Core/dvc.cpp:314-320): a failed point keeps its initial objmin 0
  // and zero displacements
  write_disp_header(run.res_fname);
  write_par_header(run.par_fname, run.num_srch_dof);
  for (int i = 0; i < N; i++) {
    const int m = order[(size_t)i];
    append_disp_row(run.res_fname, labels[(size_t)m], &pts[(size_t)m * 3], status[(size_t)m],
                    objmin[(size_t)m], &par[(size_t)m * 12]);
    append_par_row(run.par_fname, labels[(size_t)m], &pts[(size_t)m * 3], status[(size_t)m],
                   objmin[(size_t)m], &par[(size_t)m * 12], run.num_srch_dof);
  }
  write_stat_echo(run, (size_t)n, bmin, bmax, kVersion);
  append_stat_time(run.sta_fname, "Run start:\t", t_start);
  append_stat_time(run.sta_fname, "Run finish:\t", t_finish);
  append_stat_totals(run.sta_fname, N, secs, good, rfail, cfail);
  return 0;
}
