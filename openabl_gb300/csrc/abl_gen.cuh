// Common includes of files generated by `-b cuda`.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "abl_device.cuh"
#ifdef ABL_PERSIST
#include "abl_persist.cuh"
#endif
#include "abl_host.h"
#include "abl_model.h"
#include "openabl_cuda.h"

// save() of the reference runtime (asset/c/libabl.h:217), bound to the
// generated program's float width.
#define save(agents, info, path, type) abl_save(agents, info, path, type, (int) sizeof(abl_float))

// Builtins of sequential steps (src/main.cpp:104-130) over the C ABI.  A
// failing runtime call is recorded on the context (abl_seq_record_error) and
// returned by the timestep; the builtin's value is then 0.
static inline int abl_seq_count(abl_ctx *c, int type) {
  int v = 0;
  abl_seq_record_error(c, abl_reduce(c, ABL_REDUCE_COUNT, type, 0, &v));
  return v;
}
template <typename T>
static inline T abl_seq_sum(abl_ctx *c, int type, int member) {
  T v{};
  abl_seq_record_error(c, abl_reduce(c, ABL_REDUCE_SUM, type, member, &v));
  return v;
}
template <typename T>
static inline int abl_seq_count_eq(abl_ctx *c, int type, int member, T value) {
  union {
    T v;
    int n;
    unsigned char b[24];
  } u;
  std::memset(&u, 0, sizeof u);
  u.v = value;
  abl_seq_record_error(c, abl_reduce(c, ABL_REDUCE_COUNT_EQ, type, member, &u));
  return u.n;
}
static inline double abl_seq_exec_time(abl_ctx *c) {
  double s = 0.0;
  abl_seq_record_error(c, abl_last_timestep_time(c, &s));
  return s;
}
