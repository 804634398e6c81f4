// SHP kernel arguments and host launchers shared with the phase-linking pipeline.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/dpl.h"

namespace dpl {

struct GlrtArgs {
    int rows, cols, hy, hx, sy, sx, out_rows, out_cols, nslc;
    float thr;
    int tile_r, tile_c;  // output pixels per CTA
    int box_w, box_h;    // TMA box (floats x rows)
    uint8_t* is_shp;     // (out_rows, out_cols, wy, wx) bytes, or
    uint32_t* bits;      // (out_rows, out_cols, wy, words_per_row) packed masks
    int words_per_row;   // 1 (wx <= 32) or 2 (wx <= 64)
    int* status;         // set to DPL_ERR_TIMEOUT if a bounded wait gives up
};

struct KsArgs {
    const float* sorted;  // (n, rows, cols)
    const int* lo;
    const int* hi;
    int n, rows, cols, hy, hx, sy, sx, out_rows, out_cols;
    int tile_r, tile_c;
    uint8_t* is_shp;
};

int64_t glrt_pitch(int64_t cols);
size_t glrt_workspace_size(int64_t rows, int64_t cols);
size_t ks_workspace_size(int64_t nslc, int64_t rows, int64_t cols);

// scale2: rows x glrt_pitch(cols) floats.  Exactly one of is_shp / bits is non-null.
dpl_status launch_glrt(const float* mean, const float* var, int64_t rows, int64_t cols, int hy, int hx, int sy,
                       int sx, int nslc, float threshold, uint8_t* is_shp, uint32_t* bits, int* status,
                       float* scale2, cudaStream_t s);

}  // namespace dpl
