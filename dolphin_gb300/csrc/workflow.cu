// Output-raster helper of the wrapped-phase workflow: grow_nodata_region
// (utils.py:613-660), which the block loop applies to the strided outputs before
// writing them (workflows/single.py:352-362).
//
// k_grow_nodata<T> -- one thread per pixel: the pixel becomes `nodata` if any pixel of
// the (2n + 1) x (2n + 1) square around it (clipped to the image: scipy's
// binary_dilation pads with False) is nodata.  A pixel is nodata where it equals the
// nodata value, or, for a NaN nodata value, where it is NaN (integer arrays then have
// none).  Out of place: `out` must not alias `in`.  HBM-bound on the output rasters,
// which are small next to the stack.
#include <cstdio>
#include <limits>
#include <type_traits>

#include "dpl_common.cuh"

namespace dpl {

template <class T>
__device__ __forceinline__ bool is_nodata(T v, double nodata, bool nan_nodata) {
    if (nan_nodata) return false;
    return (double)v == nodata;
}
template <>
__device__ __forceinline__ bool is_nodata<float>(float v, double nodata, bool nan_nodata) {
    if (nan_nodata) return isnan(v);
    return (double)v == nodata;
}

template <class T>
__global__ void __launch_bounds__(256) k_grow_nodata(const T* in, T* out, int rows, int cols, double nodata,
                                                      int nan_nodata, int n, T fill) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (int64_t)rows * cols) return;
    const int r = (int)(p / cols), c = (int)(p - (int64_t)r * cols);
    bool hit = false;
    for (int dr = -n; dr <= n && !hit; ++dr) {
        const int rr = r + dr;
        if (rr < 0 || rr >= rows) continue;
        for (int dc = -n; dc <= n; ++dc) {
            const int cc = c + dc;
            if (cc < 0 || cc >= cols) continue;
            if (is_nodata<T>(in[(int64_t)rr * cols + cc], nodata, nan_nodata != 0)) {
                hit = true;
                break;
            }
        }
    }
    out[p] = hit ? fill : in[p];
}

template <class T>
static dpl_status grow_launch(const void* in, void* out, int64_t rows, int64_t cols, double nodata, int nan_nodata,
                              int n, cudaStream_t st) {
    if (((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) % alignof(T)) != 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_grow_nodata_region: arrays must be aligned to their element size");
    // the value written over grown pixels; where no pixel can be nodata (a NaN nodata
    // on integers, or a value the type cannot hold) it is never written
    T fill = T(0);
    if (std::is_floating_point<T>::value) {
        fill = nan_nodata ? std::numeric_limits<T>::quiet_NaN() : (T)nodata;
    } else if (!nan_nodata && nodata >= (double)std::numeric_limits<T>::lowest() &&
               nodata <= (double)std::numeric_limits<T>::max()) {
        fill = (T)nodata;
    }
    const int64_t npix = rows * cols;
    k_grow_nodata<T><<<(unsigned)ceil_div(npix, 256), 256, 0, st>>>(static_cast<const T*>(in), static_cast<T*>(out),
                                                                     (int)rows, (int)cols, nodata, nan_nodata, n, fill);
    return check_launch("k_grow_nodata");
}

}  // namespace dpl

using namespace dpl;

extern "C" dpl_status dpl_grow_nodata_region(const void* in, void* out, int dtype, int64_t rows, int64_t cols,
                                             double nodata, int nodata_is_nan, int n_pixels, dpl_stream_t stream) {
    if (rows < 0 || cols < 0 || n_pixels < 0)
        return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_grow_nodata_region: bad shape or n_pixels");
    if (rows > INT32_MAX || cols > INT32_MAX) return fail(DPL_ERR_UNSUPPORTED, "dpl_grow_nodata_region: too large");
    if (rows * cols == 0) return DPL_OK;
    if (!in || !out) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_grow_nodata_region: null pointer");
    if (in == out) return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_grow_nodata_region: out must not alias in");
    cudaStream_t st = (cudaStream_t)stream;
    const int nan = nodata_is_nan != 0;
    switch (dtype) {
        case DPL_DTYPE_F32: return grow_launch<float>(in, out, rows, cols, nodata, nan, n_pixels, st);
        case DPL_DTYPE_U8: return grow_launch<uint8_t>(in, out, rows, cols, nodata, nan, n_pixels, st);
        case DPL_DTYPE_I8: return grow_launch<int8_t>(in, out, rows, cols, nodata, nan, n_pixels, st);
        case DPL_DTYPE_I16: return grow_launch<int16_t>(in, out, rows, cols, nodata, nan, n_pixels, st);
        case DPL_DTYPE_U16: return grow_launch<uint16_t>(in, out, rows, cols, nodata, nan, n_pixels, st);
        case DPL_DTYPE_I32: return grow_launch<int32_t>(in, out, rows, cols, nodata, nan, n_pixels, st);
        default: return fail(DPL_ERR_INVALID_ARGUMENT, "dpl_grow_nodata_region: unknown dtype");
    }
}
