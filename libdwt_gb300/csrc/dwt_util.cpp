// Coefficient-layout helpers of the libdwt C API (host only): where each
// subband of a decomposition lives in the transformed frame, the frame sizes
// and strides of the array layouts, and the "optimal" (prime) row stride.
// Callers use these to consume the in-place coefficient layout the 2D
// transforms produce; they touch no device state.
#include <cstdint>

#include "../../include/libdwt.h"

namespace {

int ceil_half(int x) { return (x + 1) >> 1; }
int floor_half(int x) { return x >> 1; }

// 2^e mod n by repeated squaring (n odd, >= 3).
uint64_t pow2_mod(uint64_t e, uint64_t n)
{
    uint64_t r = 1 % n, b = 2 % n;
    while (e) {
        if (e & 1) r = (r * b) % n;
        b = (b * b) % n;
        e >>= 1;
    }
    return r;
}

// Subband geometry after j_max levels: the subband sits at the halved OUTER
// frame size (the row / column where the H half of the enclosing LL band
// starts), its extent follows the halved INNER size.
void subband(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y, int size_i_big_x,
             int size_i_big_y, int j_max, enum dwt_subbands band, void **dst_ptr, int *dst_size_x, int *dst_size_y)
{
    int hx = 0, hy = 0, lx = size_i_big_x, ly = size_i_big_y, ox = size_o_big_x, oy = size_o_big_y;
    for (int j = 1; j <= j_max; ++j) {
        hx = floor_half(lx);
        hy = floor_half(ly);
        lx = ceil_half(lx);
        ly = ceil_half(ly);
        ox = ceil_half(ox);
        oy = ceil_half(oy);
    }
    char *base = static_cast<char *>(ptr);
    int row = 0, col = 0, sx = lx, sy = ly;
    switch (band) {
    case DWT_LL:
        break;
    case DWT_HL:
        col = ox;
        sx = hx;
        break;
    case DWT_LH:
        row = oy;
        sy = hy;
        break;
    case DWT_HH:
        row = oy;
        col = ox;
        sx = hx;
        sy = hy;
        break;
    }
    *dst_ptr = base + (long long)row * stride_x + (long long)col * stride_y;
    *dst_size_x = sx;
    *dst_size_y = sy;
}

void get_sizes(enum dwt_array array_type, int size_x, int size_y, int opt_stride, int elem, int *stride_x,
               int *stride_y, int *size_o_big_x, int *size_o_big_y, int *size_i_big_x, int *size_i_big_y)
{
    *stride_x = dwt_util_get_stride(dwt_util_pow2_ceil_log2(size_x) * elem, opt_stride);
    *stride_y = elem;
    *size_o_big_x = size_x;
    *size_o_big_y = size_y;
    *size_i_big_x = size_x;
    *size_i_big_y = size_y;
    // the sparse and simple layouts place the image in a power-of-two frame
    if (array_type == DWT_ARR_SPARSE || array_type == DWT_ARR_SIMPLE) {
        *size_o_big_x = dwt_util_pow2_ceil_log2(size_x);
        *size_o_big_y = dwt_util_pow2_ceil_log2(size_y);
    }
}

}  // namespace

extern "C" {

int dwt_util_is_prime(int n)
{
    // the reference's test: 2 is prime, other even numbers and n < 2 are
    // not, and an odd n is accepted when 2^(n-1) = 1 (mod n) (Fermat's test
    // to base 2, so base-2 pseudoprimes such as 341 pass)
    if (n == 2) return 1;
    if (n < 2 || (n & 1) == 0) return 0;
    return pow2_mod(uint64_t(n) - 1, uint64_t(n)) == 1 ? 1 : 0;
}

int dwt_util_next_prime(int n)
{
    if (n <= 2) return 2;
    n |= 1;
    while (!dwt_util_is_prime(n)) n += 2;
    return n;
}

int dwt_util_get_opt_stride(int min_stride) { return dwt_util_next_prime(min_stride); }

int dwt_util_get_stride(int min_stride, int opt) { return opt ? dwt_util_get_opt_stride(min_stride) : min_stride; }

void dwt_util_subband(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y, int size_i_big_x,
                      int size_i_big_y, int j_max, enum dwt_subbands band, void **dst_ptr, int *dst_size_x,
                      int *dst_size_y)
{
    subband(ptr, stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x, size_i_big_y, j_max, band, dst_ptr,
            dst_size_x, dst_size_y);
}

void dwt_util_subband_s(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y, int size_i_big_x,
                        int size_i_big_y, int j_max, enum dwt_subbands band, void **dst_ptr, int *dst_size_x,
                        int *dst_size_y)
{
    subband(ptr, stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x, size_i_big_y, j_max, band, dst_ptr,
            dst_size_x, dst_size_y);
}

void dwt_util_subband_d(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y, int size_i_big_x,
                        int size_i_big_y, int j_max, enum dwt_subbands band, void **dst_ptr, int *dst_size_x,
                        int *dst_size_y)
{
    subband(ptr, stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x, size_i_big_y, j_max, band, dst_ptr,
            dst_size_x, dst_size_y);
}

void dwt_util_get_sizes_s(enum dwt_array array_type, int size_x, int size_y, int opt_stride, int *stride_x,
                          int *stride_y, int *size_o_big_x, int *size_o_big_y, int *size_i_big_x, int *size_i_big_y)
{
    get_sizes(array_type, size_x, size_y, opt_stride, int(sizeof(float)), stride_x, stride_y, size_o_big_x,
              size_o_big_y, size_i_big_x, size_i_big_y);
}

void dwt_util_get_sizes_d(enum dwt_array array_type, int size_x, int size_y, int opt_stride, int *stride_x,
                          int *stride_y, int *size_o_big_x, int *size_o_big_y, int *size_i_big_x, int *size_i_big_y)
{
    get_sizes(array_type, size_x, size_y, opt_stride, int(sizeof(double)), stride_x, stride_y, size_o_big_x,
              size_o_big_y, size_i_big_x, size_i_big_y);
}

}  // extern "C"
