// Common includes of files generated by `-b cuda`.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>

#include "abl_device.cuh"
#include "abl_host.h"
#include "abl_model.h"
#include "openabl_cuda.h"

// Entry points the reference runtime exposes under these names
// (asset/c/libabl.h:177-217), bound to the generated program's float width.
#define random_float(lo, hi) abl_random_float(lo, hi)
#define save(agents, info, path, type) abl_save(agents, info, path, type, (int) sizeof(abl_float))
