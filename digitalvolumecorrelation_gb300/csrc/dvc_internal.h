// dvc_internal.h — helpers shared by the translation units of libdvcgpu.so
// (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include "../../include/dvc_gpu.h"

int dvc_internal_set_error(int code, const char *msg);
// No C++ exception leaves an entry point of the C ABI: each is a function
// try block whose catch clause returns this (the exception in flight as an
// error code: DVC_E_NOMEM for a failed allocation, else DVC_E_ARG, with its
// message for dvc_gpu_last_error)
int dvc_internal_host_exception();

// patches [n][2][32^3] of points idx[0..n) (or 0..n) of a volume pair
int dvc_internal_patches(const void *ref, const void *cor, int bpv, int nx, int ny, int nz, int n,
                         const double *pts_dev, const int *idx_dev, float *out_dev, cudaStream_t st);
// the network's start parameters of points idx[0..n) into params_dev [point][12]
int dvc_internal_cnn_seed(dvc_cnn *c, const void *ref, const void *cor, int bpv, int nx, int ny, int nz,
                          int n, const double *pts_dev, const int *idx_dev, double *params_dev,
                          cudaStream_t st);
// DVC_E_TIMEOUT when a tensor-core convolution's bounded wait gave up since
// the last check (call after synchronising), else DVC_OK
int dvc_internal_cnn_status();
