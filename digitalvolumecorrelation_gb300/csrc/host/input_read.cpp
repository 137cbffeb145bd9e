// input_read.cpp — keyword input file, point cloud and result files of the
// drop-in `dvc` / `strain` programs. Behaviour follows the reference's
// InputRead (Core/InputRead.cpp); messages are worded here.
#include <algorithm>
#include <cstdio>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>

#include "host_io.h"

namespace dvchost {

const std::vector<Keyword> &keywords() {
  // group, required, example value, suitable values (Core/InputRead.cpp:45-455)
  static const std::vector<Keyword> k = {
      {"reference_filename", "fio_name", "yes", "reference_volume.raw",
       "existing raw volume file (tab after the keyword)"},
      {"correlate_filename", "fio_name", "yes", "correlate_volume.raw",
       "existing raw volume file, same layout as the reference volume"},
      {"point_cloud_filename", "fio_name", "yes", "ROI_points_nxyz.txt",
       "existing text file of 'label x y z' lines"},
      {"output_filename", "fio_name", "yes", "myproject_results",
       "base name of the .disp and .stat files (a writeable location)"},
      {"vol_bit_depth", "vox_data", "yes", "8", "8, 16"},
      {"vol_endian", "vox_data", "if vol_bit_depth is not 8", "little", "little, big"},
      {"vol_hdr_lngth", "vox_data", "yes", "0", "0 <= int <= 4096"},
      {"vol_wide", "vox_data", "yes", "512", "0 <= int <= 8000 (x, voxels per row)"},
      {"vol_high", "vox_data", "yes", "512", "0 <= int <= 8000 (y, rows per slice)"},
      {"vol_tall", "vox_data", "yes", "512", "0 <= int <= 8000 (z, slices)"},
      {"subvol_geom", "sub_vols", "yes", "cube", "cube, sphere"},
      {"subvol_size", "sub_vols", "yes", "30", "0 <= int <= smallest volume dimension"},
      {"subvol_npts", "sub_vols", "yes", "5000", "0 <= int <= 50000"},
      {"subvol_thresh", "sub_vols", "yes", "off", "on, off"},
      {"gray_thresh_min", "sub_vols", "if subvol_thresh is on", "25",
       "0 <= double <= 2^vol_bit_depth"},
      {"gray_thresh_max", "sub_vols", "if subvol_thresh is on", "125",
       "gray_thresh_min <= double <= 2^vol_bit_depth"},
      {"min_vol_fract", "sub_vols", "if subvol_thresh is on", "0.2", "0.0 <= double <= 1.0"},
      {"disp_max", "opt_mthd", "yes", "15", "0 <= int <= smallest volume dimension"},
      {"num_srch_dof", "opt_mthd", "yes", "6", "3, 6, 12"},
      {"obj_function", "opt_mthd", "yes", "znssd", "sad, ssd, zssd, nssd, znssd"},
      {"interp_type", "opt_mthd", "yes", "tricubic", "nearest, trilinear, tricubic"},
      {"rigid_trans", "opt_tune", "no", "0.0 0.0 0.0",
       "three doubles, |x|,|y|,|z| <= the volume dimensions"},
      {"basin_radius", "opt_tune", "no", "0.0", "0.0 <= double <= disp_max (0 = no coarse grid)"},
      {"subvol_aspect", "opt_tune", "no", "1.0 1.0 1.0", "three doubles in [0.1, 10.0]"},
      {"num_points_to_process", "opt_tune", "yes", "0",
       "0 <= int; 0 or 1 = every point, otherwise the first n in processing order"},
      {"starting_point", "opt_tune", "no", "0.0 0.0 0.0",
       "three doubles, |x|,|y|,|z| <= the volume dimensions"},
  };
  return k;
}

static const Keyword *kw(const char *word) {
  for (const Keyword &k : keywords())
    if (std::string(k.word) == word) return &k;
  return nullptr;
}

// return codes of the parse helpers (Core/Utility.h:33-35)
static const int kOk = 1, kMissing = -1, kInvalid = -2;

bool InputFile::open(const std::string &fname) {
  std::ifstream f(fname.c_str(), std::ios::binary);
  if (!f.good()) {
    std::cout << "\nCannot find input file '" << fname << "'\n\n";
    return false;
  }
  std::string all((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  // the terminator is whichever of '\n' / '\r' splits the file into more
  // pieces, '\n' on a tie (Core/InputRead.cpp:492-517)
  auto pieces = [&](char c) {
    std::istringstream s(all);
    std::string l;
    size_t n = 0;
    while (std::getline(s, l, c)) n++;
    return n;
  };
  const char eol = pieces('\n') >= pieces('\r') ? '\n' : '\r';
  std::istringstream s(all);
  std::string l;
  lines_.clear();
  while (std::getline(s, l, eol)) lines_.push_back(l + "\n");
  return true;
}

bool InputFile::find(const std::string &word, std::string &line, bool required) const {
  for (const std::string &l : lines_) {
    if (l[0] == '#') continue;
    if (l.find(word) != std::string::npos) {
      line = l;
      return true;
    }
  }
  if (required) std::cout << "\n\nInput Error: keyword '" << word << "' not found in input file.\n\n";
  return false;
}

void InputFile::invalid(const char *word) const {
  const Keyword *k = kw(word);
  std::cout << "\nInput Error: " << word << " contains an invalid parameter.\n\n";
  if (k) std::cout << "   suitable: " << k->suitable << "\n\n";
}

// tab-separated fields: the keyword, then the file name (trailing line
// terminators are not part of the name)
static bool second_tab_field(const std::string &line, std::string &name) {
  std::istringstream io(line);
  std::string field;
  int seen = 0;
  while (std::getline(io, field, '\t')) {
    if (field.empty()) continue;
    if (++seen == 2) {
      while (!field.empty() && (field.back() == '\n' || field.back() == '\r')) field.pop_back();
      name = field;
      return !name.empty();
    }
  }
  return false;
}

int InputFile::old_file(const char *word, std::string &out, unsigned long &bytes) {
  std::string line, name;
  if (!find(word, line, true)) return kMissing;
  if (!second_tab_field(line, name)) {
    invalid(word);
    return kInvalid;
  }
  std::ifstream f(name.c_str(), std::ios::binary);
  if (f.good()) {
    out = name;
    f.seekg(0, f.end);
    bytes = (unsigned long)f.tellg();
    return kOk;
  }
  std::cout << "\nInput Error: " << word << " cannot find file: " << name << "\n\n";
  return kInvalid;
}

int InputFile::new_file(const char *word, std::string &out) {
  std::string line, name;
  if (!find(word, line, true)) return kMissing;
  if (second_tab_field(line, name)) {
    std::ofstream f(name.c_str());
    if (f.is_open()) {
      f.close();
      std::remove(name.c_str());
      out = name;
      return kOk;
    }
  }
  invalid(word);
  return kInvalid;
}

// values are read with stream extraction after the keyword token: a value
// that does not parse reads as 0 and is then range checked
int InputFile::int_in(const char *word, const std::vector<int> &ok, int &out) {
  std::string line, w;
  if (!find(word, line, true)) return kMissing;
  std::istringstream io(line);
  double v = 0.0;
  io >> w >> v;
  for (int o : ok)
    if (v == o) {
      out = (int)v;
      return kOk;
    }
  invalid(word);
  return kInvalid;
}

int InputFile::str_in(const char *word, const std::vector<std::string> &ok, std::string &out) {
  std::string line, w, v;
  if (!find(word, line, true)) return kMissing;
  std::istringstream io(line);
  io >> w >> v;
  for (const std::string &o : ok)
    if (v == o) {
      out = v;
      return kOk;
    }
  invalid(word);
  return kInvalid;
}

int InputFile::int_range(const char *word, int lo, int hi, int &out, bool required) {
  std::string line, w;
  if (!find(word, line, required)) return kMissing;
  std::istringstream io(line);
  int v = 0;
  io >> w >> v;
  if (v >= lo && v <= hi) {
    out = v;
    return kOk;
  }
  invalid(word);
  return kInvalid;
}

int InputFile::uint_range(const char *word, unsigned lo, unsigned hi, unsigned &out, bool required) {
  std::string line, w;
  if (!find(word, line, required)) return kMissing;
  std::istringstream io(line);
  unsigned v = 0;
  io >> w >> v;
  if (v >= lo && v <= hi) {
    out = v;
    return kOk;
  }
  invalid(word);
  return kInvalid;
}

int InputFile::dbl_range(const char *word, double lo, double hi, double &out, bool required) {
  std::string line, w;
  if (!find(word, line, required)) return kMissing;
  std::istringstream io(line);
  double v = 0.0;
  io >> w >> v;
  if (v >= lo && v <= hi) {
    out = v;
    return kOk;
  }
  invalid(word);
  return kInvalid;
}

int InputFile::vec_abs(const char *word, const double lim[3], double out[3]) {
  std::string line, w;
  if (!find(word, line, false)) return kMissing;
  std::istringstream io(line);
  io >> w;
  int ok = 0;
  for (int i = 0; i < 3; i++) {
    double v = 0.0;
    io >> v;
    if (std::fabs(v) > std::fabs(lim[i])) break;
    out[i] = v;
    ok++;
  }
  if (ok == 3) return kOk;
  invalid(word);
  return kInvalid;
}

int InputFile::vec_range(const char *word, double lo, double hi, double out[3]) {
  std::string line, w;
  if (!find(word, line, false)) return kMissing;
  std::istringstream io(line);
  io >> w;
  int ok = 0;
  for (int i = 0; i < 3; i++) {
    double v = 0.0;
    io >> v;
    if (v < lo || v > hi) break;
    out[i] = v;
    ok++;
  }
  if (ok == 3) return kOk;
  invalid(word);
  return kInvalid;
}

bool InputFile::read(RunConfig &r) {
  // order and limits of Core/InputRead.cpp:519-631
  if (old_file("reference_filename", r.ref_fname, r.ref_bytes) != kOk) return false;
  if (old_file("correlate_filename", r.cor_fname, r.cor_bytes) != kOk) return false;
  unsigned long pts_bytes = 0;
  if (old_file("point_cloud_filename", r.pts_fname, pts_bytes) != kOk) return false;
  if (new_file("output_filename", r.out_fname) != kOk) return false;
  r.res_fname = r.out_fname + ".disp";
  r.sta_fname = r.out_fname + ".stat";
  r.par_fname = r.out_fname + ".par";

  if (int_in("vol_bit_depth", {8, 16}, r.vol_bit_depth) != kOk) return false;
  if (r.vol_bit_depth != 8 && str_in("vol_endian", {"little", "big"}, r.vol_endian) != kOk) return false;
  if (int_range("vol_hdr_lngth", 0, 4096, r.vol_hdr_lngth, true) != kOk) return false;
  if (int_range("vol_wide", 0, 8000, r.vol_wide, true) != kOk) return false;
  if (int_range("vol_high", 0, 8000, r.vol_high, true) != kOk) return false;
  if (int_range("vol_tall", 0, 8000, r.vol_tall, true) != kOk) return false;
  const int size_max = std::min(r.vol_wide, std::min(r.vol_high, r.vol_tall));

  if (str_in("subvol_geom", {"cube", "sphere"}, r.subvol_geom) != kOk) return false;
  r.sub_geo = r.subvol_geom == "sphere" ? 1 : 0;
  if (int_range("subvol_size", 0, size_max, r.subvol_size, true) != kOk) return false;
  if (int_range("subvol_npts", 0, 50000, r.subvol_npts, true) != kOk) return false;
  if (str_in("subvol_thresh", {"on", "off"}, r.subvol_thresh) != kOk) return false;
  if (r.subvol_thresh == "on") {
    const double top = std::pow(2.0, (double)r.vol_bit_depth);
    if (dbl_range("gray_thresh_min", 0.0, top, r.gray_thresh_min, true) != kOk) return false;
    if (dbl_range("gray_thresh_max", r.gray_thresh_min, top, r.gray_thresh_max, true) != kOk) return false;
    if (dbl_range("min_vol_fract", 0.0, 1.0, r.min_vol_fract, true) != kOk) return false;
  }

  if (int_range("disp_max", 0, size_max, r.disp_max, true) != kOk) return false;
  if (int_in("num_srch_dof", {3, 6, 12}, r.num_srch_dof) != kOk) return false;
  const std::vector<std::string> fcn = {"sad", "ssd", "zssd", "nssd", "znssd"};
  if (str_in("obj_function", fcn, r.obj_function) != kOk) return false;
  r.obj_fcn = (int)(std::find(fcn.begin(), fcn.end(), r.obj_function) - fcn.begin());
  const std::vector<std::string> itp = {"nearest", "trilinear", "tricubic"};
  if (str_in("interp_type", itp, r.interp_type) != kOk) return false;
  r.int_typ = (int)(std::find(itp.begin(), itp.end(), r.interp_type) - itp.begin());

  // optional tuning keywords: absent keeps the default, a bad value aborts
  r.basin_radius = 0.0;
  if (dbl_range("basin_radius", 0.0, (double)r.disp_max, r.basin_radius, false) == kInvalid) return false;
  const double dims[3] = {(double)r.vol_wide, (double)r.vol_high, (double)r.vol_tall};
  if (vec_abs("rigid_trans", dims, r.rigid_trans) == kInvalid) return false;
  if (vec_range("subvol_aspect", 0.1, 10.0, r.subvol_aspect) == kInvalid) return false;
  if (vec_abs("starting_point", dims, r.starting_point) == kInvalid) return false;
  // parsed as required by the reference (Core/InputRead.cpp:604)
  if (uint_range("num_points_to_process", 0u, std::numeric_limits<unsigned>::max(),
                 r.num_points_to_process, true) != kOk)
    return false;
  std::cout << "Max points to process is " << r.num_points_to_process << std::endl;

  const unsigned long expect = (unsigned long)r.vol_hdr_lngth + (unsigned long)r.vol_wide *
                                                                    (unsigned long)r.vol_high *
                                                                    (unsigned long)r.vol_tall *
                                                                    (unsigned long)(r.vol_bit_depth / 8);
  const char *which[2] = {"Reference", "Correlate"};
  const unsigned long got[2] = {r.ref_bytes, r.cor_bytes};
  for (int v = 0; v < 2; v++)
    if (got[v] != expect) {
      std::cout << "\n" << which[v] << " volume file size (" << got[v]
                << " bytes) does not match the volume description (" << expect << " bytes).\n"
                << "Check vol_bit_depth, vol_hdr_lngth, vol_wide, vol_high and vol_tall.\n\n";
      return false;
    }
  return true;
}

bool read_roi(const std::string &fname, std::vector<int> &labels, std::vector<double> &pts,
              double bmin[3], double bmax[3]) {
  std::ifstream f(fname.c_str(), std::ios::binary);
  std::string all((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  auto pieces = [&](char c) {
    std::istringstream s(all);
    std::string l;
    size_t n = 0;
    while (std::getline(s, l, c)) n++;
    return n;
  };
  const char eol = pieces('\n') >= pieces('\r') ? '\n' : '\r';
  for (int d = 0; d < 3; d++) {
    bmin[d] = std::numeric_limits<double>::max();
    bmax[d] = std::numeric_limits<double>::min();
  }
  std::istringstream s(all);
  std::string line;
  while (std::getline(s, line, eol)) {
    std::istringstream ss(line + "\n");
    int label;
    double x, y, z;
    // an integer label not followed by '.' or 'E', then three numbers
    if (!(ss >> label)) continue;
    const int c = ss.peek();
    if (c == '.' || c == 'E') continue;
    if (!(ss >> x) || !(ss >> y) || !(ss >> z)) continue;
    labels.push_back(label);
    pts.push_back(x);
    pts.push_back(y);
    pts.push_back(z);
    const double p[3] = {x, y, z};
    for (int d = 0; d < 3; d++) {
      if (p[d] < bmin[d]) bmin[d] = p[d];
      if (p[d] > bmax[d]) bmax[d] = p[d];
    }
  }
  if (labels.empty()) {
    std::cout << "\nNo points were read from the point cloud file '" << fname << "'.\n"
              << "Each point is one line of plain text: an integer label and the x y z\n"
              << "coordinates, separated by tabs or blanks, e.g.\n\n5\t10.72\t15.87\t23.45\n\n"
              << "Other lines (headers, comments) are skipped.\n\n";
    return false;
  }
  return true;
}

static const char *kGroups[5][2] = {
    {"fio_name", "files read and written by the run"},
    {"vox_data", "layout of the two raw image volumes"},
    {"sub_vols", "the subvolume (template) built around every point"},
    {"opt_mthd", "the search: range, degrees of freedom, objective, interpolation"},
    {"opt_tune", "optional tuning of the search"},
};

void write_example(std::ostream &os) {
  for (const auto &g : kGroups) {
    os << "###\n###\t keywords of group " << g[0] << ": " << g[1] << "\n###\n\n";
    for (const Keyword &k : keywords())
      if (std::string(k.group) == g[0])
        os << (std::string(k.required) == "yes" ? "" : "# ") << k.word << "\t" << k.example
           << "\t### " << k.suitable << "\n";
    os << "\n";
  }
}

void write_manual(std::ostream &os) {
  os << "dvc: digital volume correlation of a reference and a correlate image volume\n\n"
     << "   dvc              list the command line options\n"
     << "   dvc help         short description of a run\n"
     << "   dvc example      write dvc_in_example, an input file with every keyword\n"
     << "   dvc manual       write this manual\n"
     << "   dvc version      print the program version\n"
     << "   dvc <input>      run the correlation described by the input file\n\n"
     << "The input file holds one keyword per line followed by its value(s). Lines starting\n"
     << "with # are ignored; the first other line that contains a keyword supplies it.\n"
     << "File names follow their keyword after a tab. Keywords by group:\n\n";
  for (const auto &g : kGroups) {
    os << "group " << g[0] << " (" << g[1] << ")\n\n";
    for (const Keyword &k : keywords())
      if (std::string(k.group) == g[0])
        os << "   " << k.word << "\n      example:  " << k.word << "\t" << k.example
           << "\n      required: " << k.required << "\n      suitable: " << k.suitable << "\n\n";
  }
  os << "Output\n\n"
     << "   <output_filename>.disp  tab separated: n x y z status objmin u v w, one line per\n"
     << "                           point in processing order; status 0 = converged,\n"
     << "                           -1 = range fail (the search left the disp_max range),\n"
     << "                           -2 = convergence fail; u v w = target - reference position\n"
     << "   <output_filename>.stat  echo of the input, the point cloud, run times and totals\n"
     << "   <point_cloud_filename>.sort.csv  the 75 nearest points of every point (for strain)\n"
     << "   <output_filename>.par   the .disp columns with every search parameter: u v w, and\n"
     << "                           phi the psi (6 dof), exx eyy ezz exy eyz exz (12 dof)\n\n";
}

void write_disp_header(const std::string &fname) {
  std::ofstream f(fname.c_str(), std::ios_base::out);
  f << "n\tx\ty\tz\tstatus\tobjmin\tu\tv\tw\n";
}

void append_disp_row(const std::string &fname, int label, const double pt[3], int status,
                     double objmin, const double uvw[3]) {
  std::ofstream f(fname.c_str(), std::ios_base::out | std::ios_base::app);
  f << label << "\t" << pt[0] << "\t" << pt[1] << "\t" << pt[2] << "\t" << status << "\t" << objmin;
  f << std::fixed << std::setprecision(6);
  for (int i = 0; i < 3; i++) f << "\t" << uvw[i];
  f << "\n";
}

void write_par_header(const std::string &fname, int ndof) {
  static const char *names[12] = {"u", "v", "w", "phi", "the", "psi", "exx", "eyy", "ezz", "exy", "eyz", "exz"};
  std::ofstream f(fname.c_str(), std::ios_base::out);
  f << "n\tx\ty\tz\tstatus\tobjmin";
  for (int i = 0; i < ndof; i++) f << "\t" << names[i];
  f << "\n";
}

void append_par_row(const std::string &fname, int label, const double pt[3], int status,
                    double objmin, const double *par, int ndof) {
  std::ofstream f(fname.c_str(), std::ios_base::out | std::ios_base::app);
  f << label << "\t" << pt[0] << "\t" << pt[1] << "\t" << pt[2] << "\t" << status << "\t" << objmin;
  f << std::scientific << std::setprecision(9);
  for (int i = 0; i < ndof; i++) f << "\t" << par[i];
  f << "\n";
}

void write_stat_echo(const RunConfig &r, size_t n_points, const double bmin[3],
                     const double bmax[3], const char *version) {
  // layout of Core/InputRead.cpp:1033-1100
  std::ofstream f(r.sta_fname.c_str(), std::ios_base::out);
  f << "\n### echo of the input file for this run\n\n";
  f << "reference_filename\t" << r.ref_fname << "\n";
  f << "correlate_filename\t" << r.cor_fname << "\n";
  f << "point_cloud_filename\t" << r.pts_fname << "\n";
  f << "output_filename\t" << r.out_fname << "\n\n";
  f << "vol_bit_depth\t" << r.vol_bit_depth << "\n";
  if (r.vol_bit_depth != 8) f << "vol_endian\t" << r.vol_endian << "\n";
  f << "vol_hdr_lngth\t" << r.vol_hdr_lngth << "\n";
  f << "vol_wide\t" << r.vol_wide << "\n";
  f << "vol_high\t" << r.vol_high << "\n";
  f << "vol_tall\t" << r.vol_tall << "\n\n";
  f << "subvol_geom\t" << r.subvol_geom << "\n";
  f << "subvol_size\t" << r.subvol_size << "\n";
  f << "subvol_npts\t" << r.subvol_npts << "\n\n";
  f << "subvol_thresh\t" << r.subvol_thresh << "\n";
  if (r.subvol_thresh == "on") {
    f << "gray_thresh_min\t" << r.gray_thresh_min << "\n";
    f << "gray_thresh_max\t" << r.gray_thresh_max << "\n";
    f << "min_vol_fract\t" << r.min_vol_fract << "\n";
  }
  f << "\n";
  f << "disp_max\t" << r.disp_max << "\n";
  f << "num_srch_dof\t" << r.num_srch_dof << "\n";
  f << "obj_function\t" << r.obj_function << "\n";
  f << "interp_type\t" << r.interp_type << "\n\n";
  f << "rigid_trans\t" << r.rigid_trans[0] << "\t" << r.rigid_trans[1] << "\t" << r.rigid_trans[2] << "\n";
  f << "basin_radius\t" << r.basin_radius << "\n";
  f << "subvol_aspect\t" << r.subvol_aspect[0] << "\t" << r.subvol_aspect[1] << "\t"
    << r.subvol_aspect[2] << "\n";
  f << "\n### end of input file echo\n";
  f << "\nPoint Cloud contains " << n_points << " points\n\n";
  f << "\tbounding box min = [" << bmin[0] << " " << bmin[1] << " " << bmin[2] << "]\n";
  f << "\tbounding box max = [" << bmax[0] << " " << bmax[1] << " " << bmax[2] << "]\n";
  f << "\nrunning under dvc code version: " << version << "\n\n";
}

void append_stat_time(const std::string &fname, const std::string &label, long long unix_time) {
  std::ofstream f(fname.c_str(), std::ios_base::out | std::ios_base::app);
  const time_t t = (time_t)unix_time;
  char buf[32];
  std::strftime(buf, sizeof buf, "%Y-%m-%d %H:%M:%S", std::localtime(&t));
  f << label << buf << "\n";
}

void append_stat_line(const std::string &fname, const std::string &text) {
  std::ofstream f(fname.c_str(), std::ios_base::out | std::ios_base::app);
  f << text;
}

void append_stat_totals(const std::string &fname, int count, double seconds, int good,
                        int range_fail, int convg_fail) {
  // Core/dvc.cpp:322-338
  std::ofstream f(fname.c_str(), std::ios_base::out | std::ios_base::app);
  f << std::setprecision(0) << std::fixed;
  f << count << " points processed in " << seconds << " seconds\n";
  f << std::setprecision(3) << std::fixed;
  f << seconds / count << " sec/pt\n";
  f << count / seconds << " pt/sec\n\n";
  f << "number successful = " << good << "\t(" << 100 * ((double)good / (double)count) << "%)\n";
  f << "number range fail = " << range_fail << "\t(" << 100 * ((double)range_fail / (double)count) << "%)\n";
  f << "number convg fail = " << convg_fail << "\t(" << 100 * ((double)convg_fail / (double)count) << "%)\n\n";
}

// one value followed by at most one ',', one ' ' and one '\t' separator
template <typename T>
static bool get_val(std::stringstream &ss, T &v) {
  if (!(ss >> v)) return false;
  if (ss.peek() == ',') ss.ignore();
  if (ss.peek() == ' ') ss.ignore();
  if (ss.peek() == '\t') ss.ignore();
  return true;
}

bool read_disp(const std::string &fname, std::vector<int> &labels, std::vector<double> &pts,
               std::vector<int> &status, std::vector<double> &objmin, std::vector<double> &disp) {
  std::ifstream f(fname.c_str());
  std::string line;
  bool first = true;
  while (std::getline(f, line)) {
    std::stringstream ss(line);
    if (first) {
      first = false;
      if (ss.peek() != 'n') {
        std::cout << "-> .disp file lacks the header line (n x y z ...): check the command line"
                  << std::endl;
        return false;
      }
    }
    int n = 0, st = 0;
    double p[3], ob = 0.0, u[3];
    int cols = 0;
    if (get_val(ss, n)) cols += 1;
    if (get_val(ss, p[0]) && get_val(ss, p[1]) && get_val(ss, p[2])) cols += 3;
    if (get_val(ss, st)) cols += 1;
    if (get_val(ss, ob)) cols += 1;
    if (get_val(ss, u[0]) && get_val(ss, u[1]) && get_val(ss, u[2])) cols += 3;
    if (cols != 9) continue;
    labels.push_back(n);
    pts.insert(pts.end(), p, p + 3);
    status.push_back(st);
    objmin.push_back(ob);
    disp.insert(disp.end(), u, u + 3);
  }
  return true;
}

void read_sort_csv(const std::string &fname, std::vector<std::vector<int>> &neigh) {
  std::ifstream f(fname.c_str());
  std::string line;
  while (std::getline(f, line)) {
    std::stringstream ss(line);
    std::vector<int> row;
    int v;
    while (ss >> v) {
      row.push_back(v);
      if (ss.peek() == ',') ss.ignore();
      if (ss.peek() == ' ') ss.ignore();
      if (ss.peek() == '\t') ss.ignore();
    }
    if (!row.empty()) neigh.push_back(row);
  }
}

}  // namespace dvchost
