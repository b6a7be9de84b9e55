/* The reference's calling pattern for a bank of strided signals, driven from
 * native code against this library: an OpenMP loop over the signals, one
 * dwt_cdf97_f_ex_stride_s (or _i_) call per signal (src/libdwt.c:5512-5557
 * are the calls; the loop is how the reference's callers and its perf
 * harness drive them).  Signal s of the bank lives at base + (s / lanes) *
 * group_stride + (s % lanes) * 4 bytes, samples `stride` bytes apart, in
 * place: L at the signal's start, H ceil(n/2) samples later.  Built by
 * bench.py (gcc -fopenmp) against libdwt_gb300.so; returns the seconds the
 * loop took. */
#include <omp.h>
#include <stddef.h>

void dwt_cdf97_f_ex_stride_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N, int stride);
void dwt_cdf97_i_ex_stride_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N, int stride);

double calls_1d(int inverse, char *base, int n, int stride, int lanes, long long group_stride, long long count,
                int threads)
{
    const long long off_h = (long long)((n + 1) / 2) * stride;
    const double t0 = omp_get_wtime();
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long s = 0; s < count; ++s) {
        float *a = (float *)(base + (s / lanes) * group_stride + (s % lanes) * 4);
        float *h = (float *)((char *)a + off_h);
        if (inverse)
            dwt_cdf97_i_ex_stride_s(a, h, a, NULL, n, stride);
        else
            dwt_cdf97_f_ex_stride_s(a, a, h, NULL, n, stride);
    }
    return omp_get_wtime() - t0;
}
