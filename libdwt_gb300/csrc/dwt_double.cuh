// Double-precision transforms (libdwt's _d API): declarations of the kernels'
// launchers (see dwt_double.cu).
#pragma once

#include "dwt_common.cuh"

namespace dwt {

// Lifting parameters in double, as libdwt's _d variants apply them: the same
// step order and layout as Wavelet, constants rounded to double, 1/zeta the
// double division (src/libdwt.c:536-574, 1467-1571, 5673-5777).
struct WaveletD {
    double c[4];
    double zeta_e, zeta_o;
    double n1_fwd, n1_inv;
    int nsteps;
};

WaveletD make_wavelet_d(int id, bool inverse);

// Byte-strided frame <-> compact row-major double frame (pitch in doubles).
cudaError_t launch_repack_d(const void *src, long long sx, long long sy, int ox, int oy, double *dst,
                            long long dpitch, cudaStream_t s);
cudaError_t launch_unpack_d(const double *src, long long spitch, void *dst, long long sx, long long sy, int ox,
                            int oy, cudaStream_t s);

// One level of the reference's in-place 2D sequence on a compact double
// frame (rows then columns, L to [0, ceil/2), H from the outer midpoint,
// optional zero padding), as sparse_forward_level / sparse_inverse_level.
// tmp holds max(lines) * max(length) doubles.
cudaError_t level_forward_d(double *f, long long pitch, int osx, int osy, int odx, int ody, int isx, int isy,
                            int zero_padding, int wavelet, double *tmp, cudaStream_t s);
cudaError_t level_inverse_d(double *f, long long pitch, int osx, int osy, int odx, int ody, int idx, int idy,
                            int zero_padding, int wavelet, double *tmp, cudaStream_t s);

// One compact line of N doubles in place: forward writes L to [0, ceil(N/2))
// and H from ceil(N/2); inverse reads them there and writes the N samples.
cudaError_t line_d(bool inverse, double *line, int N, int wavelet, double *tmp, cudaStream_t s);

}  // namespace dwt
