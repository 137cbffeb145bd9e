// strain_main.cpp — the drop-in `strain` program: same command line flags,
// input files (.disp, optional .sort.csv) and CSV outputs as the reference's
// `strain` (Core/strain.cpp:166-661); the per-point strain-window fits run on
// the GPU (dvc_gpu_strain, FP64).
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "dvc_gpu.h"
#include "host_io.h"

using namespace dvchost;

namespace {

const int kNdpMin = 10, kNdpDef = 25, kNdpMax = 75;  // Core/strain.cpp:24-31, DataCloud.cpp:34
const double kObjtMin = 0.0001, kObjtMax = 1.0, kObjtDef = 1.0;

void drop(int &argc, char *argv[], int i, int k) {
  for (int j = i; j + k < argc; j++) argv[j] = argv[j + k];
  argc -= k;
}

// flag without a value: remove it and report whether it was there
bool find_flag(const std::string &flag, int &argc, char *argv[]) {
  for (int i = 0; i < argc; i++)
    if (flag == argv[i]) {
      drop(argc, argv, i, 1);
      return true;
    }
  return false;
}

// flag with a value: both removed when the value converts; a value that does
// not convert is left in place (the flag is removed); a missing value is
// reported (Core/strain.cpp:48-110)
template <typename T>
bool find_flag(const std::string &flag, int &argc, char *argv[], T &val) {
  for (int i = 0; i < argc; i++) {
    if (flag != argv[i]) continue;
    if (argc > i + 1) {
      try {
        const T v = std::is_same<T, int>::value ? (T)std::stoi(argv[i + 1]) : (T)std::stod(argv[i + 1]);
        val = v;
        drop(argc, argv, i, 2);
        return true;
      } catch (const std::exception &) {
        drop(argc, argv, i, 1);
        std::cout << "argument after " << flag << " not valid" << std::endl;
        return false;
      }
    }
    std::cout << "no argument after " << flag << " flag" << std::endl;
    argc -= 1;
  }
  return false;
}

// the first remaining argument that starts with '-' is dropped with a note
void drop_unknown_flag(int &argc, char *argv[]) {
  for (int i = 0; i < argc; i++)
    if (argv[i][0] == '-') {
      std::cout << "-> unused flag " << argv[i] << " found, ignored" << std::endl;
      drop(argc, argv, i, 1);
      return;
    }
}

void usage() {
  std::cout << "strain needs a .disp file.\n\nCommand line:\n"
            << "strain run.disp\n"
            << "  - strain windows from run.disp; the neighbour lists are computed and written\n"
            << "    to <base>.sort.csv (slow for large point clouds)\n"
            << "strain run.disp run.sort.csv\n"
            << "  - reuse the neighbour lists written by dvc or by an earlier strain run\n\n"
            << "Defaults:\n"
            << "strain window = " << kNdpDef << " points (min = " << kNdpMin << ", max = " << kNdpMax
            << "), set with -sw\n"
            << "objmin threshold = " << kObjtDef << " (min = " << kObjtMin << ", max = " << kObjtMax
            << "): points with objmin above it are left out of the windows, set with -t\n"
            << "output: Lagrangian strain (<base>-sw<n>.Lstr.csv)\n\n"
            << "Flags:\n"
            << "-sw 30\t\t strain window size in points\n"
            << "-t 0.01\t\t objmin threshold\n"
            << "-r\t\t refill windows past points that fail the threshold\n"
            << "-E\t\t also write engineering strain (.Estr.csv)\n"
            << "-D\t\t also write the displacement gradient (.dgrd.csv)\n"
            << "-A\t\t write every output\n"
            << "-xy -yz -zx\t plane-only analysis (found automatically for planar clouds)\n\n";
}

}  // namespace

int main(int argc, char *argv[]) {
  std::cout << std::endl;
  if (argc == 1) {
    usage();
    return 0;
  }
  int ndp = kNdpDef;
  double objt = kObjtDef;
  bool refill = false, xy = false, yz = false, zx = false, out_e = false, out_d = false;
  if (find_flag("-sw", argc, argv, ndp)) ndp = std::min(std::max(ndp, kNdpMin), kNdpMax);
  if (find_flag("-t", argc, argv, objt)) objt = std::min(std::max(objt, kObjtMin), kObjtMax);
  if (find_flag("-r", argc, argv)) refill = true;
  if (find_flag("-xy", argc, argv)) xy = true;
  if (find_flag("-yz", argc, argv)) yz = true;
  if (find_flag("-zx", argc, argv)) zx = true;
  if (find_flag("-E", argc, argv)) out_e = true;
  if (find_flag("-D", argc, argv)) out_d = true;
  if (find_flag("-A", argc, argv)) out_e = out_d = true;
  drop_unknown_flag(argc, argv);
  if (argc < 2) {
    usage();
    return 0;
  }

  const std::string fdisp(argv[1]);
  if (!std::ifstream(fdisp.c_str()).good()) {
    std::cout << "-> cannot find .disp file '" << fdisp << std::endl;
    return 0;
  }
  std::cout << "using disp file: " << fdisp << std::endl;
  // the base name ends before the first '.' of the argument
  const size_t dot = fdisp.find_first_of('.');
  const std::string base = dot == std::string::npos ? fdisp : fdisp.substr(0, dot);

  std::string fsort;
  bool sort_read = false;
  if (argc > 2) {
    fsort = argv[2];
    sort_read = std::ifstream(fsort.c_str()).good();
    if (!sort_read) std::cout << "-> cannot find .sort file " << fsort << std::endl;
  }

  std::vector<int> labels, status;
  std::vector<double> pts, objmin, disp;
  if (!read_disp(fdisp, labels, pts, status, objmin, disp)) return 0;
  const int n = (int)labels.size();
  if (n == 0) {
    std::cout << "-> no points read from " << fdisp << std::endl;
    return 0;
  }
  std::vector<std::vector<int>> neigh;
  if (sort_read) {
    read_sort_csv(fsort, neigh);
    std::cout << "using sort file: " << fsort << std::endl;
  }
  const int nsort = (int)neigh.size();
  if (sort_read && nsort != n) {
    sort_read = false;
    neigh.clear();
    std::cout << "-> different number of points in .disp and .sort" << std::endl;
  }
  if (!sort_read) {
    std::cout << "-> creating a new sort file: " << base + ".sort.csv" << std::endl;
    std::vector<int> order;
    if (std::getenv("DVC_GPU_NEIGHBOURS")) {  // GPU path: ties by point index
      const int kk = std::min(kNdpMax, n);
      std::vector<int> flat((size_t)n * kk);
      order.resize((size_t)n);
      if (dvc_gpu_order_neighbours(n, pts.data(), &pts[0], kNdpMax, order.data(), flat.data()) != DVC_OK) {
        std::cout << "-> neighbour search on the GPU failed: " << dvc_gpu_last_error() << std::endl;
        return 0;
      }
      neigh.assign((size_t)n, std::vector<int>());
      for (int i = 0; i < n; i++)
        neigh[(size_t)i].assign(flat.begin() + (size_t)i * kk, flat.begin() + (size_t)(i + 1) * kk);
    } else {
      order_neighbours(pts, &pts[0], kNdpMax, order, neigh);
    }
    std::cout << "sorting finished" << std::endl;
    write_sort_csv(base, neigh);
  }

  // a point cloud in a coordinate plane gets the plane analysis
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = hi[d] = pts[(size_t)d];
    for (int i = 0; i < n; i++) {
      lo[d] = std::min(lo[d], pts[(size_t)i * 3 + d]);
      hi[d] = std::max(hi[d], pts[(size_t)i * 3 + d]);
    }
  }
  if (std::fabs(hi[0] - lo[0]) < 0.001) yz = true;
  if (std::fabs(hi[1] - lo[1]) < 0.001) zx = true;
  if (std::fabs(hi[2] - lo[2]) < 0.001) xy = true;
  if (yz) std::cout << "using 2d yz coordinate plane analsis" << std::endl;
  if (zx) std::cout << "using 2d zx coordinate plane analsis" << std::endl;
  if (xy) std::cout << "using 2d xy coordinate plane analsis" << std::endl;
  std::cout << "using strain window: " << ndp << std::endl;
  if (objt == kObjtMin)
    std::cout << "using objmin thresh: " << objt << " (use only highly matched points)" << std::endl;
  else if (objt == kObjtMax)
    std::cout << "using objmin thresh: " << objt << " (use all convergent points)" << std::endl;
  else
    std::cout << "using objmin thresh: " << objt << " " << std::endl;
  if (refill) std::cout << "using strain window refill " << std::endl;
  std::cout << "nsort_pts =" << nsort << std::endl;
  std::cout << "ndisp_pts =" << n << std::endl;

  int nn = 0;
  for (const auto &row : neigh) nn = std::max(nn, (int)row.size());
  std::vector<int> nflat((size_t)n * nn, -1);
  for (int i = 0; i < n; i++)
    for (size_t j = 0; j < neigh[(size_t)i].size(); j++) nflat[(size_t)i * nn + j] = neigh[(size_t)i][j];
  std::vector<double> ufit((size_t)n * 3), swr((size_t)n), es((size_t)n * 9), ls((size_t)n * 9),
      dg((size_t)n * 9);
  std::vector<int> pin((size_t)n);
  const int planar = (yz ? 1 : 0) | (zx ? 2 : 0) | (xy ? 4 : 0);
  if (dvc_gpu_strain(n, pts.data(), status.data(), objmin.data(), disp.data(), nn, nflat.data(), ndp,
                     objt, refill ? 1 : 0, planar, ufit.data(), pin.data(), swr.data(), es.data(),
                     ls.data(), dg.data()) != DVC_OK) {
    std::cout << "-> strain calculation failed: " << dvc_gpu_last_error() << std::endl;
    return 0;
  }

  const std::string hdr = "n,x,y,z,u_fit,v_fit,w_fit,pts_in_sw,sw_radius,exx,eyy,ezz,exy,eyz,exz,ep1,ep2,ep3";
  auto write = [&](const char *ext, const std::string &header, const std::vector<double> &v) {
    const std::string name = base + "-sw" + std::to_string(ndp) + ext;
    std::cout << "output file: " << name << std::endl;
    std::ofstream f(name);
    f << header << std::endl;
    for (int i = 0; i < n; i++) {
      f << labels[(size_t)i] << "," << pts[(size_t)i * 3] << "," << pts[(size_t)i * 3 + 1] << ","
        << pts[(size_t)i * 3 + 2];
      for (int k = 0; k < 3; k++) f << "," << ufit[(size_t)i * 3 + k];
      f << "," << pin[(size_t)i] << "," << swr[(size_t)i];
      for (int k = 0; k < 9; k++) f << "," << v[(size_t)i * 9 + k];
      f << std::endl;
    }
  };
  if (out_e) write(".Estr.csv", hdr, es);
  write(".Lstr.csv", hdr, ls);
  if (out_d)
    write(".dgrd.csv", "n,x,y,z,u_fit,v_fit,w_fit,pts_in_sw,sw_radius,ux,uy,uz,vx,vy,vz,wx,wy,wz", dg);
  std::cout << std::endl;
  return 0;
}
