// data_cloud.cpp — processing order and neighbour lists of the point cloud
// (the reference's DataCloud::sort_order_neighbors / write_sort_file,
// Core/DataCloud.cpp:38-144).
//
// Both are std::sort over {index, distance} records with a strict
// less-than on the distance, started in index order, so points at equal
// distance come out in the order this standard library's std::sort leaves
// them, exactly as in the reference built with the same library. The
// neighbour lists cost O(N^2 log N), as in the reference; the per-point sorts
// are spread over the host threads.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>

#include "host_io.h"

namespace dvchost {

namespace {
struct Rec {
  int index;
  double value;
};
bool by_value(const Rec &a, const Rec &b) { return a.value < b.value; }
// Point::pt_dist (Core/Point.h:47-48), same operations
double pt_dist(const double *a, const double *b) {
  return std::sqrt(std::pow(a[0] - b[0], 2) + std::pow(a[1] - b[1], 2) + std::pow(a[2] - b[2], 2));
}
}  // namespace

void order_neighbours(const std::vector<double> &pts, const double start[3], int keep,
                      std::vector<int> &order, std::vector<std::vector<int>> &neigh) {
  const int n = (int)(pts.size() / 3);
  keep = std::min(keep, n);
  std::vector<Rec> rec((size_t)n);
  for (int i = 0; i < n; i++) rec[(size_t)i] = {i, pt_dist(start, &pts[(size_t)i * 3])};
  std::sort(rec.begin(), rec.end(), by_value);
  order.resize((size_t)n);
  for (int i = 0; i < n; i++) order[(size_t)i] = rec[(size_t)i].index;
  neigh.assign((size_t)n, std::vector<int>());
#pragma omp parallel
  {
    std::vector<Rec> r2((size_t)n);
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < n; i++) {
      for (int j = 0; j < n; j++) r2[(size_t)j] = {j, pt_dist(&pts[(size_t)i * 3], &pts[(size_t)j * 3])};
      std::sort(r2.begin(), r2.end(), by_value);
      std::vector<int> &row = neigh[(size_t)i];
      row.resize((size_t)keep);
      for (int j = 0; j < keep; j++) row[(size_t)j] = r2[(size_t)j].index;
    }
  }
}

void write_sort_csv(const std::string &base, const std::vector<std::vector<int>> &neigh) {
  std::cout << "Saving sorted pointcloud" << std::endl;
  std::ofstream f(base + ".sort.csv");
  for (const std::vector<int> &row : neigh) {
    for (size_t j = 0; j < row.size(); j++) {
      if (j) f << ",";
      f << row[j];
    }
    f << std::endl;
  }
}

}  // namespace dvchost
