// catalog.hpp -- catalog ingestion on device columns (catalog.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tcgpu.h"

namespace tc {

// Catalog._finish_input's column work on device columns (see catalog.cu).  cols: ncols
// device pointers (host array); w: device, length n (filled with 1 when !w_given); wpos,
// flag: device or NULL.  Compacts the columns in place when rows are removed.
int catalog_finish_device(int64_t n, int ncols, double* const* cols, double* w, double* wpos,
                          const int64_t* flag, int64_t ignore_flag, int w_given,
                          int keep_zero_weight, cudaStream_t st, tc_catalog_info* out);

// Catalog._get_center_size on device columns (z may be NULL): out = (mean x, y, z, size).
int catalog_center_size_device(int64_t n, const double* x, const double* y, const double* z,
                               cudaStream_t st, double out[4]);

}  // namespace tc
