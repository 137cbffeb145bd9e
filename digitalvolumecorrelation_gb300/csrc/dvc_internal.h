// dvc_internal.h — helpers shared by the translation units of libdvcgpu.so
// (not part of the C ABI).
#pragma once
int dvc_internal_set_error(int code, const char *msg);
