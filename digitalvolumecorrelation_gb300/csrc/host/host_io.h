// host_io.h — input, point-cloud and result files of the drop-in `dvc` and
// `strain` programs (host C++17 over the C ABI of include/dvc_gpu.h).
//
// The reference reads a keyword input file (Core/InputRead.cpp:519-631), a
// "label x y z" point cloud (:666-730) and writes `<out>.disp`, `<out>.stat`
// (:1033-1196) and `<roi>.sort.csv` (Core/DataCloud.cpp:38-64); its `strain`
// program reads `.disp` / `.sort.csv` back (Core/InputRead.cpp:720-863). The
// functions here follow those rules: which line a keyword is taken from, how
// each value is extracted and range-checked, the order of the checks (the
// first failing one aborts the run), and the number formats of every output.
#pragma once

#include <cmath>
#include <cstdint>
#include <ostream>
#include <string>
#include <vector>

namespace dvchost {

// Settings of one run (the reference's RunControl, Core/Utility.h:90-134).
struct RunConfig {
  std::string ref_fname, cor_fname, pts_fname, out_fname, res_fname, sta_fname;
  std::string par_fname;  // <output_filename>.par: every search parameter (no reference counterpart)
  unsigned long ref_bytes = 0, cor_bytes = 0;  // file sizes found while checking the names
  int vol_bit_depth = 8;
  std::string vol_endian = "little";
  int vol_hdr_lngth = 0, vol_wide = 0, vol_high = 0, vol_tall = 0;
  std::string subvol_geom;
  int sub_geo = 0;  // 0 cube, 1 sphere
  int subvol_size = 0, subvol_npts = 0;
  std::string subvol_thresh;
  double gray_thresh_min = 0.0, gray_thresh_max = 0.0, min_vol_fract = 0.0;
  int disp_max = 0, num_srch_dof = 0;
  std::string obj_function, interp_type;
  int obj_fcn = 0, int_typ = 0;  // enum positions in the option lists
  double basin_radius = 0.0;
  double rigid_trans[3] = {0.0, 0.0, 0.0};
  double subvol_aspect[3] = {1.0, 1.0, 1.0};
  double starting_point[3] = {NAN, NAN, NAN};
  unsigned int num_points_to_process = 0;
};

// One keyword of the input file: its group, whether it is required, an
// example value and what values are suitable.
struct Keyword {
  const char *word, *group, *required, *example, *suitable;
};
const std::vector<Keyword> &keywords();

// The input file, split into lines the way the reference splits it: the line
// terminator is '\n' unless the file has more '\r'-separated pieces.
class InputFile {
 public:
  // false (with the message) when the file cannot be opened
  bool open(const std::string &fname);
  // parse and check every keyword in the reference's order; prints the
  // reference's kind of message and returns false at the first problem
  bool read(RunConfig &run);

 private:
  std::vector<std::string> lines_;  // each with "\n" appended
  // first line not starting with '#' that contains `word` anywhere
  bool find(const std::string &word, std::string &line, bool required) const;
  int old_file(const char *word, std::string &out, unsigned long &bytes);
  int new_file(const char *word, std::string &out);
  int int_in(const char *word, const std::vector<int> &ok, int &out);
  int str_in(const char *word, const std::vector<std::string> &ok, std::string &out);
  int int_range(const char *word, int lo, int hi, int &out, bool required);
  int uint_range(const char *word, unsigned lo, unsigned hi, unsigned &out, bool required);
  int dbl_range(const char *word, double lo, double hi, double &out, bool required);
  int vec_abs(const char *word, const double lim[3], double out[3]);
  int vec_range(const char *word, double lo, double hi, double out[3]);
  void invalid(const char *word) const;
};

// Point cloud: whitespace separated "label x y z" lines; any other line is
// skipped (Core/InputRead.cpp:666-696). bmin/bmax: the cloud's bounding box,
// started as the reference starts it (max from the smallest positive double).
bool read_roi(const std::string &fname, std::vector<int> &labels, std::vector<double> &pts,
              double bmin[3], double bmax[3]);

// `dvc example` / `dvc manual` texts (own wording, same keyword set)
void write_example(std::ostream &os);
void write_manual(std::ostream &os);

// Results. `.disp`: header, then label, x, y, z, status, objmin with six
// significant digits and u, v, w fixed to six decimals, tab separated.
void write_disp_header(const std::string &fname);
void append_disp_row(const std::string &fname, int label, const double pt[3], int status,
                     double objmin, const double uvw[3]);
// `.par` (no reference counterpart; the reference's .disp keeps u, v, w
// only, Core/InputRead.cpp:1133-1196): the .disp columns label, x, y, z,
// status, objmin, then all num_srch_dof parameters (u v w phi the psi exx
// eyy ezz exy eyz exz) in scientific notation with 9 decimals, so the
// rotations and strains of 6- and 12-dof searches are kept.
void write_par_header(const std::string &fname, int ndof);
void append_par_row(const std::string &fname, int label, const double pt[3], int status,
                    double objmin, const double *par, int ndof);
// `.stat`: the input echo (truncates the file), a time stamp line, run totals
void write_stat_echo(const RunConfig &run, size_t n_points, const double bmin[3],
                     const double bmax[3], const char *version);
void append_stat_time(const std::string &fname, const std::string &label, long long unix_time);
void append_stat_line(const std::string &fname, const std::string &text);
void append_stat_totals(const std::string &fname, int count, double seconds, int good,
                        int range_fail, int convg_fail);

// `.disp` reader of the `strain` program: the first line must start with
// 'n'; rows with all nine columns are kept (Core/InputRead.cpp:796-863).
bool read_disp(const std::string &fname, std::vector<int> &labels, std::vector<double> &pts,
               std::vector<int> &status, std::vector<double> &objmin, std::vector<double> &disp);
// `.sort.csv` reader: integers separated by ',' (or blank / tab) per line
void read_sort_csv(const std::string &fname, std::vector<std::vector<int>> &neigh);

// Processing order and neighbour lists (Core/DataCloud.cpp:69-144): order by
// distance from `start` and, per point, the `keep` nearest points, each from
// std::sort of all distances so ties come out as they do in the reference.
void order_neighbours(const std::vector<double> &pts, const double start[3], int keep,
                      std::vector<int> &order, std::vector<std::vector<int>> &neigh);
// `<base>.sort.csv`, comma separated, one line per point
void write_sort_csv(const std::string &base, const std::vector<std::vector<int>> &neigh);

}  // namespace dvchost
