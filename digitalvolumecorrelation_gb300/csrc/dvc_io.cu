// dvc_io.cu — volume files straight to device memory, and MetaImage headers.
//
// The reference reads its raw volumes piecewise for every point: per z-slice
// and y-row of the interpolation box one seekg + read (Interpolate::kernels,
// Core/Interpolate.cpp:144-258), with the 16-bit endian swap done on the host
// by every OpenMP thread. Here each file is streamed once into HBM: chunks are
// read into two pinned host buffers in turn and copied asynchronously, so the
// file read of one chunk overlaps the copy of the previous one; big-endian
// 16-bit data is swapped on the device after each chunk lands. The `.mhd`
// (MetaImage) header is what users of the reference hold next to their raw
// files (its test data, `dvc_test/*/*.mhd`); dvc_gpu_read_mhd reads the keys
// that locate and describe the raw data.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/dvc_gpu.h"
#include "dvc_internal.h"

namespace {

constexpr size_t kChunk = 64ull << 20;  // bytes per staged chunk

__global__ void swap16_kernel(uint16_t *v, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint16_t x = v[i];
    v[i] = (uint16_t)((x >> 8) | (x << 8));
  }
}

int io_error(int code, const std::string &msg) { return dvc_internal_set_error(code, msg.c_str()); }

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

}  // namespace

extern "C" {

int dvc_gpu_load_raw(void *vol_dev, const char *path, long long header_bytes, int nx, int ny, int nz,
                     int bytes_per_voxel, int big_endian, void *stream) try {
  if (!vol_dev || !path || header_bytes < 0 || nx <= 0 || ny <= 0 || nz <= 0 ||
      (bytes_per_voxel != 1 && bytes_per_voxel != 2))
    return io_error(DVC_E_ARG, "dvc_gpu_load_raw: bad arguments");
  const size_t bytes = (size_t)nx * ny * nz * bytes_per_voxel;
  std::FILE *f = std::fopen(path, "rb");
  if (!f) return io_error(DVC_E_ARG, std::string("cannot open ") + path);
  if (fseeko(f, 0, SEEK_END) != 0) {
    std::fclose(f);
    return io_error(DVC_E_ARG, std::string("cannot seek in ") + path);
  }
  const long long fsize = (long long)ftello(f);
  if (fsize < header_bytes + (long long)bytes) {
    std::fclose(f);
    return io_error(DVC_E_ARG, std::string(path) + " is shorter than header + volume");
  }
  if (fseeko(f, (off_t)header_bytes, SEEK_SET) != 0) {
    std::fclose(f);
    return io_error(DVC_E_ARG, std::string("cannot seek in ") + path);
  }
  cudaStream_t st = (cudaStream_t)stream;
  void *hbuf[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  std::string err;
  int rc = DVC_OK;
  const size_t chunk = std::min(kChunk, bytes);
  for (int b = 0; b < 2 && rc == DVC_OK; b++) {
    if (cudaHostAlloc(&hbuf[b], chunk, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming) != cudaSuccess) {
      rc = DVC_E_NOMEM;
      err = "pinned staging buffers";
    }
  }
  size_t off = 0;
  for (int k = 0; rc == DVC_OK && off < bytes; k++) {
    const int b = k & 1;
    const size_t n = std::min(chunk, bytes - off);
    // the copy that last used this buffer must have finished
    if (k >= 2 && cudaEventSynchronize(done[b]) != cudaSuccess) {
      rc = DVC_E_CUDA;
      err = "waiting for a staged copy";
      break;
    }
    if (std::fread(hbuf[b], 1, n, f) != n) {
      rc = DVC_E_ARG;
      err = std::string("short read from ") + path;
      break;
    }
    char *dst = (char *)vol_dev + off;
    if (cudaMemcpyAsync(dst, hbuf[b], n, cudaMemcpyHostToDevice, st) != cudaSuccess) {
      rc = DVC_E_CUDA;
      err = "chunk copy";
      break;
    }
    if (bytes_per_voxel == 2 && big_endian) {
      const size_t nv = n / 2;  // chunks hold whole voxels (even sizes, even offsets)
      swap16_kernel<<<(unsigned)std::min<size_t>((nv + 255) / 256, 4096), 256, 0, st>>>((uint16_t *)dst, nv);
    }
    if (cudaEventRecord(done[b], st) != cudaSuccess) {
      rc = DVC_E_CUDA;
      err = "event record";
      break;
    }
    off += n;
  }
  if (rc == DVC_OK) {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      rc = DVC_E_CUDA;
      err = cudaGetErrorString(e);
    }
  } else {
    cudaStreamSynchronize(st);
  }
  for (int b = 0; b < 2; b++) {
    if (done[b]) cudaEventDestroy(done[b]);
    if (hbuf[b]) cudaFreeHost(hbuf[b]);
  }
  std::fclose(f);
  if (rc != DVC_OK) return io_error(rc, "dvc_gpu_load_raw: " + err);
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_gpu_read_mhd(const char *mhd_path, dvc_volume_info *out) try {
  if (!mhd_path || !out) return io_error(DVC_E_ARG, "null argument");
  std::memset(out, 0, sizeof *out);
  std::ifstream f(mhd_path);
  if (!f.good()) return io_error(DVC_E_ARG, std::string("cannot open ") + mhd_path);
  int ndims = 3, dims[3] = {0, 0, 0}, have_dims = 0, esize = 0;
  long long header = 0;
  int msb = 0;
  std::string data;
  std::string line;
  while (std::getline(f, line)) {
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    const std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
    std::istringstream vs(val);
    if (key == "NDims") {
      vs >> ndims;
    } else if (key == "DimSize") {
      have_dims = 0;
      while (have_dims < 3 && (vs >> dims[have_dims])) have_dims++;
    } else if (key == "ElementType") {
      if (val == "MET_UCHAR" || val == "MET_CHAR") esize = 1;
      else if (val == "MET_USHORT" || val == "MET_SHORT") esize = 2;
      else return io_error(DVC_E_ARG, "ElementType " + val + " is not 8 or 16 bit");
    } else if (key == "HeaderSize") {
      vs >> header;
    } else if (key == "BinaryDataByteOrderMSB" || key == "ElementByteOrderMSB") {
      msb = (val == "True" || val == "true" || val == "1") ? 1 : 0;
    } else if (key == "ElementDataFile") {
      data = val;
    } else if (key == "CompressedData") {
      if (val == "True" || val == "true") return io_error(DVC_E_ARG, "compressed MetaImage data");
    }
  }
  if (ndims != 3 || have_dims != 3 || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
    return io_error(DVC_E_ARG, "MetaImage header needs NDims = 3 and three DimSize values");
  if (!esize) return io_error(DVC_E_ARG, "MetaImage header has no ElementType");
  if (data.empty() || data == "LIST") return io_error(DVC_E_ARG, "MetaImage header has no single ElementDataFile");
  if (header < 0) return io_error(DVC_E_ARG, "HeaderSize -1 (computed from the end) is not supported");
  std::string path;
  if (data == "LOCAL") {
    // data follows the header in the same file
    path = mhd_path;
    std::ifstream g(mhd_path, std::ios::binary);
    std::string l;
    long long pos = 0;
    while (std::getline(g, l)) {
      pos = (long long)g.tellg();
      if (l.compare(0, 15, "ElementDataFile") == 0) break;
    }
    header += pos;
  } else if (data[0] == '/') {
    path = data;
  } else {
    const std::string m(mhd_path);
    const size_t slash = m.find_last_of('/');
    path = (slash == std::string::npos ? std::string() : m.substr(0, slash + 1)) + data;
  }
  if (path.size() >= sizeof out->data_file) return io_error(DVC_E_ARG, "data file path too long");
  out->nx = dims[0];
  out->ny = dims[1];
  out->nz = dims[2];
  out->bytes_per_voxel = esize;
  out->big_endian = esize == 2 ? msb : 0;
  out->header_bytes = header;
  std::strcpy(out->data_file, path.c_str());
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

}  // extern "C"
