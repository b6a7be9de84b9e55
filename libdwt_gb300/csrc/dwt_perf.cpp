// libdwt's performance harness and the host utilities its callers use
// (host only): image allocation, the test pattern, result comparison, the
// timers, and dwt_util_perf_* / dwt_util_measure_perf_*, which time the
// transforms of this library (the GPU path) and print gnuplot-ready data
// exactly as the reference does, so examples/perf-plot and
// examples/simple-perf run unchanged against the GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <sys/resource.h>
#include <sys/time.h>
#include <sys/times.h>
#include <unistd.h>
#include <vector>

#include "../../include/libdwt.h"

namespace {

// The test pattern, type 0 (src/libdwt.c:1051-1134): x is shifted right by
// `rand`, the value is 2xy / (x^2 + y^2 + 1) evaluated in the target type.
template <typename T>
void fill_pattern(void *ptr, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y, int rand)
{
    char *base = static_cast<char *>(ptr);
    for (int y = 0; y < size_i_big_y; ++y)
        for (int x0 = 0; x0 < size_i_big_x; ++x0) {
            const int x = x0 >> rand;
            T *p = reinterpret_cast<T *>(base + (long long)y * stride_x + (long long)x0 * stride_y);
            *p = T(2 * x * y) / T(x * x + y * y + 1);
        }
}

template <typename T>
int compare(void *p1, void *p2, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y, T eps)
{
    const char *a = static_cast<const char *>(p1), *b = static_cast<const char *>(p2);
    for (int y = 0; y < size_i_big_y; ++y)
        for (int x = 0; x < size_i_big_x; ++x) {
            const long long o = (long long)y * stride_x + (long long)x * stride_y;
            const T u = *reinterpret_cast<const T *>(a + o), v = *reinterpret_cast<const T *>(b + o);
            if (std::isnan(u) || std::isinf(u) || std::isnan(v) || std::isinf(v)) return 1;
            if (std::fabs(u - v) > eps) return 1;
        }
    return 0;
}

int resolve(int type) { return type == DWT_TIME_AUTOSELECT ? dwt_util_clock_autoselect() : type; }

dwt_clock_t ts_ns(clockid_t id)
{
    timespec t;
    clock_gettime(id, &t);
    return dwt_clock_t(t.tv_sec) * 1000000000LL + t.tv_nsec;
}

// Times M forward and M inverse transforms of M test images, N times; the
// minimum over the N loops of the per-transform average (src/libdwt.c:8386-8617).
template <typename T, typename Fwd, typename Inv>
void perf_2(int stride_x, int stride_y, int size_o_big_x, int size_o_big_y, int size_i_big_x, int size_i_big_y,
            int j_max, int decompose_one, int zero_padding, int M, int N, int clock_type, T *fwd_secs, T *inv_secs,
            Fwd fwd, Inv inv)
{
    if (M <= 0 || N <= 0 || !fwd_secs || !inv_secs) {
        std::fprintf(stderr, "ERROR: dwt_util_perf: invalid arguments\n");
        std::abort();
    }
    std::vector<void *> img(M);
    std::vector<int> j(M, j_max);
    for (int m = 0; m < M; ++m) {
        dwt_util_alloc_image(&img[m], stride_x, stride_y, size_o_big_x, size_o_big_y);
        fill_pattern<T>(img[m], stride_x, stride_y, size_i_big_x, size_i_big_y, 0);
    }
    *fwd_secs = T(INFINITY);
    *inv_secs = T(INFINITY);
    const T freq = T(dwt_util_get_frequency(clock_type));
    for (int n = 0; n < N; ++n) {
        const dwt_clock_t f0 = dwt_util_get_clock(clock_type);
        for (int m = 0; m < M; ++m)
            fwd(img[m], stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x, size_i_big_y, &j[m],
                decompose_one, zero_padding);
        const dwt_clock_t f1 = dwt_util_get_clock(clock_type);
        const T tf = T(f1 - f0) / M / freq;
        if (tf < *fwd_secs) *fwd_secs = tf;
        const dwt_clock_t i0 = dwt_util_get_clock(clock_type);
        for (int m = 0; m < M; ++m)
            inv(img[m], stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x, size_i_big_y, j[m],
                decompose_one, zero_padding);
        const dwt_clock_t i1 = dwt_util_get_clock(clock_type);
        const T ti = T(i1 - i0) / M / freq;
        if (ti < *inv_secs) *inv_secs = ti;
    }
    for (int m = 0; m < M; ++m) dwt_util_free_image(&img[m]);
}

// Sizes x = min_x, ceil(x * 1.28), ... up to max_x; square images (2D) or
// single rows (1D); one "pixels<TAB>seconds" line per size and direction
// (src/libdwt.c:8703-9036).
template <typename T, typename Sizes, typename Perf>
void measure(enum dwt_array array_type, int min_x, int max_x, int opt_stride, int j_max, int decompose_one,
             int zero_padding, int M, int N, int clock_type, FILE *fwd_plot_data, FILE *inv_plot_data, bool rows,
             Sizes sizes, Perf perf)
{
    if (min_x <= 0 || min_x >= max_x || M <= 0 || N <= 0 || !fwd_plot_data || !inv_plot_data) {
        std::fprintf(stderr, "ERROR: dwt_util_measure_perf: invalid arguments\n");
        std::abort();
    }
    const T growth = T(1.28);
    for (int x = min_x; x <= max_x; x = int(std::ceil(x * growth))) {
        const int y = rows ? 1 : x;
        int sx, sy, ox, oy, ix, iy;
        sizes(array_type, x, y, opt_stride, &sx, &sy, &ox, &oy, &ix, &iy);
        T fs, is;
        perf(sx, sy, ox, oy, ix, iy, j_max, decompose_one, zero_padding, M, N, clock_type, &fs, &is);
        std::fprintf(fwd_plot_data, "%i\t%.10f\n", x * y, double(fs));
        std::fprintf(inv_plot_data, "%i\t%.10f\n", x * y, double(is));
    }
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------ timers

int dwt_util_clock_autoselect(void) { return DWT_TIME_CLOCK_GETTIME; }

dwt_clock_t dwt_util_get_clock(int type)
{
    switch (resolve(type)) {
    case DWT_TIME_CLOCK_GETTIME_REALTIME:
        return ts_ns(CLOCK_REALTIME);
    case DWT_TIME_CLOCK_GETTIME_MONOTONIC_RAW:
        return ts_ns(CLOCK_MONOTONIC_RAW);
    case DWT_TIME_CLOCK_GETTIME_PROCESS_CPUTIME_ID:
        return ts_ns(CLOCK_PROCESS_CPUTIME_ID);
    case DWT_TIME_CLOCK_GETTIME_THREAD_CPUTIME_ID:
        return ts_ns(CLOCK_THREAD_CPUTIME_ID);
    case DWT_TIME_CLOCK:
        return dwt_clock_t(clock());
    case DWT_TIME_TIMES: {
        tms t;
        times(&t);
        return dwt_clock_t(t.tms_utime);
    }
    case DWT_TIME_GETRUSAGE:
    case DWT_TIME_GETRUSAGE_SELF:
    case DWT_TIME_GETRUSAGE_CHILDREN:
    case DWT_TIME_GETRUSAGE_THREAD: {
        rusage u;
        getrusage(RUSAGE_SELF, &u);
        return dwt_clock_t(u.ru_utime.tv_sec) * 1000000 + u.ru_utime.tv_usec;
    }
    case DWT_TIME_GETTIMEOFDAY: {
        timeval t;
        gettimeofday(&t, nullptr);
        return dwt_clock_t(t.tv_sec) * 1000000 + t.tv_usec;
    }
    case DWT_TIME_IOCTL_RTC:
        return dwt_clock_t(time(nullptr));
    default:  // DWT_TIME_CLOCK_GETTIME, _MONOTONIC
        return ts_ns(CLOCK_MONOTONIC);
    }
}

dwt_clock_t dwt_util_get_frequency(int type)
{
    switch (resolve(type)) {
    case DWT_TIME_CLOCK:
        return CLOCKS_PER_SEC;
    case DWT_TIME_TIMES:
        return sysconf(_SC_CLK_TCK);
    case DWT_TIME_GETRUSAGE:
    case DWT_TIME_GETRUSAGE_SELF:
    case DWT_TIME_GETRUSAGE_CHILDREN:
    case DWT_TIME_GETRUSAGE_THREAD:
    case DWT_TIME_GETTIMEOFDAY:
        return 1000000;
    case DWT_TIME_IOCTL_RTC:
        return 1;
    default:
        return 1000000000LL;
    }
}

// ------------------------------------------------------- images and checks

void dwt_util_alloc_image(void **pptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y)
{
    (void)stride_y;
    (void)size_o_big_x;
    *pptr = std::malloc(size_t(stride_x) * size_t(size_o_big_y));
    if (!*pptr) {
        std::fprintf(stderr, "ERROR: Unable to allocate memory.\n");
        std::abort();
    }
}

void dwt_util_free_image(void **pptr)
{
    std::free(*pptr);
    *pptr = nullptr;
}

void dwt_util_test_image_fill_s(void *ptr, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y, int rand)
{
    fill_pattern<float>(ptr, stride_x, stride_y, size_i_big_x, size_i_big_y, rand);
}

void dwt_util_test_image_fill_d(void *ptr, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y, int rand)
{
    fill_pattern<double>(ptr, stride_x, stride_y, size_i_big_x, size_i_big_y, rand);
}

int dwt_util_compare_s(void *ptr1, void *ptr2, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y)
{
    return compare<float>(ptr1, ptr2, stride_x, stride_y, size_i_big_x, size_i_big_y, 1e-3f);
}

int dwt_util_compare_d(void *ptr1, void *ptr2, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y)
{
    return compare<double>(ptr1, ptr2, stride_x, stride_y, size_i_big_x, size_i_big_y, 1e-6);
}

// Host threads: the transforms run on the GPU, one host thread drives them.
int dwt_util_get_max_threads(void) { return 1; }
int dwt_util_get_num_threads(void) { return 1; }
int dwt_util_get_num_workers(void) { return 1; }
void dwt_util_set_num_threads(int num_threads) { (void)num_threads; }

// --------------------------------------------------------------- harness

void dwt_util_perf_cdf97_2_s(int stride_x, int stride_y, int size_o_big_x, int size_o_big_y, int size_i_big_x,
                             int size_i_big_y, int j_max, int decompose_one, int zero_padding, int M, int N,
                             int clock_type, float *fwd_secs, float *inv_secs)
{
    perf_2<float>(stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x, size_i_big_y, j_max, decompose_one,
                  zero_padding, M, N, clock_type, fwd_secs, inv_secs, dwt_cdf97_2f_s, dwt_cdf97_2i_s);
}

void dwt_util_perf_cdf97_2_d(int stride_x, int stride_y, int size_o_big_x, int size_o_big_y, int size_i_big_x,
                             int size_i_big_y, int j_max, int decompose_one, int zero_padding, int M, int N,
                             int clock_type, double *fwd_secs, double *inv_secs)
{
    perf_2<double>(stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x, size_i_big_y, j_max,
                   decompose_one, zero_padding, M, N, clock_type, fwd_secs, inv_secs, dwt_cdf97_2f_d,
                   dwt_cdf97_2i_d);
}

void dwt_util_measure_perf_cdf97_2_s(enum dwt_array array_type, int min_x, int max_x, int opt_stride, int j_max,
                                     int decompose_one, int zero_padding, int M, int N, int clock_type,
                                     FILE *fwd_plot_data, FILE *inv_plot_data)
{
    measure<float>(array_type, min_x, max_x, opt_stride, j_max, decompose_one, zero_padding, M, N, clock_type,
                   fwd_plot_data, inv_plot_data, false, dwt_util_get_sizes_s, dwt_util_perf_cdf97_2_s);
}

void dwt_util_measure_perf_cdf97_2_d(enum dwt_array array_type, int min_x, int max_x, int opt_stride, int j_max,
                                     int decompose_one, int zero_padding, int M, int N, int clock_type,
                                     FILE *fwd_plot_data, FILE *inv_plot_data)
{
    measure<double>(array_type, min_x, max_x, opt_stride, j_max, decompose_one, zero_padding, M, N, clock_type,
                    fwd_plot_data, inv_plot_data, false, dwt_util_get_sizes_d, dwt_util_perf_cdf97_2_d);
}

void dwt_util_measure_perf_cdf97_1_s(enum dwt_array array_type, int min_x, int max_x, int opt_stride, int j_max,
                                     int decompose_one, int zero_padding, int M, int N, int clock_type,
                                     FILE *fwd_plot_data, FILE *inv_plot_data)
{
    measure<float>(array_type, min_x, max_x, opt_stride, j_max, decompose_one, zero_padding, M, N, clock_type,
                   fwd_plot_data, inv_plot_data, true, dwt_util_get_sizes_s, dwt_util_perf_cdf97_2_s);
}

void dwt_util_measure_perf_cdf97_1_d(enum dwt_array array_type, int min_x, int max_x, int opt_stride, int j_max,
                                     int decompose_one, int zero_padding, int M, int N, int clock_type,
                                     FILE *fwd_plot_data, FILE *inv_plot_data)
{
    measure<double>(array_type, min_x, max_x, opt_stride, j_max, decompose_one, zero_padding, M, N, clock_type,
                    fwd_plot_data, inv_plot_data, true, dwt_util_get_sizes_d, dwt_util_perf_cdf97_2_d);
}

}  // extern "C"
