/*
 * libdwt_gb300 -- GB300 (sm_103a) drop-in for the lifting-scheme wavelet hot
 * path of libdwt (slchen/libdwt, VERSION 2013-01-29-dev).
 *
 * The first group of declarations is libdwt's own C API for the path, with
 * the same names, argument meaning, memory model (byte strides, in place,
 * outer/inner frame) and error behaviour (log, then abort).  Each one cites
 * the reference declaration it replaces.  Pointers may be host memory
 * (pageable or pinned) or device/managed memory of the current device; every
 * call is synchronous on return, like the reference.
 *
 * The second group (dwt_gpu_*) is this library's extension: non-aborting
 * variants that return an error code, device-resident out-of-place forms with
 * an explicit stream, the batched strided 1D form, the batched 2D form and
 * the serving loop.
 */
#ifndef LIBDWT_GB300_H
#define LIBDWT_GB300_H

#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#if defined(__GNUC__)
#define DWT_EXPORT __attribute__((visibility("default")))
#else
#define DWT_EXPORT
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ 2D, float */

/* src/libdwt.h:491-502 (src/libdwt.c:6286-6408): in-place forward CDF 9/7,
 * *j_max_ptr levels (clamped to the limit and written back). */
DWT_EXPORT void dwt_cdf97_2f_s(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                    int size_i_big_x, int size_i_big_y, int *j_max_ptr, int decompose_one,
                    int zero_padding);

/* src/libdwt.h:509-520 (src/libdwt.c:6410-6491): in-place forward CDF 5/3. */
DWT_EXPORT void dwt_cdf53_2f_s(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                    int size_i_big_x, int size_i_big_y, int *j_max_ptr, int decompose_one,
                    int zero_padding);

/* src/libdwt.h:563-574 (src/libdwt.c:6647-6755): in-place inverse CDF 9/7. */
DWT_EXPORT void dwt_cdf97_2i_s(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                    int size_i_big_x, int size_i_big_y, int j_max, int decompose_one,
                    int zero_padding);

/* src/libdwt.h:581-592 (src/libdwt.c:6757-6832): in-place inverse CDF 5/3. */
DWT_EXPORT void dwt_cdf53_2i_s(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                    int size_i_big_x, int size_i_big_y, int j_max, int decompose_one,
                    int zero_padding);

/* ------------------------------------------------------------------ 1D, float */

/* src/libdwt.h:219-226 (src/libdwt.c:5512-5557): one forward CDF 9/7 level of
 * N samples `stride` bytes apart; L to dst_l, H to dst_h (same stride).
 * tmp is accepted and not used. */
DWT_EXPORT void dwt_cdf97_f_ex_stride_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N,
                             int stride);

/* src/libdwt.h:327-334 (src/libdwt.c:5779-5824): one inverse CDF 9/7 level. */
DWT_EXPORT void dwt_cdf97_i_ex_stride_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N,
                             int stride);

/* src/libdwt.h:233-240 (src/libdwt.c:5559-5603): one forward CDF 5/3 level. */
DWT_EXPORT void dwt_cdf53_f_ex_stride_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N,
                             int stride);

/* src/libdwt.h:341-348 (src/libdwt.c:5826-5870): one inverse CDF 5/3 level. */
DWT_EXPORT void dwt_cdf53_i_ex_stride_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N,
                             int stride);

/* src/libdwt.h:165-184, 273-292 (src/libdwt.c:1433-1465, 5639-5671): the
 * contiguous forms, stride = sizeof(float). */
DWT_EXPORT void dwt_cdf97_f_ex_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N);
DWT_EXPORT void dwt_cdf53_f_ex_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N);
DWT_EXPORT void dwt_cdf97_i_ex_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N);
DWT_EXPORT void dwt_cdf53_i_ex_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N);

/* src/libdwt.h:57-134 (src/libdwt.c:1309-1337, 1369-1397): the deprecated
 * forms with L and H concatenated in one array. */
DWT_EXPORT void dwt_cdf97_f_s(const float *src, float *dst, float *tmp, int N);
DWT_EXPORT void dwt_cdf53_f_s(const float *src, float *dst, float *tmp, int N);
DWT_EXPORT void dwt_cdf97_i_s(const float *src, float *dst, float *tmp, int N);
DWT_EXPORT void dwt_cdf53_i_s(const float *src, float *dst, float *tmp, int N);

/* --------------------------------------------------------- double precision */

/* src/libdwt.h:455-486, 527-558 (src/libdwt.c:6120-6284, 6493-6645): the
 * 2D drivers in double, same frame and level semantics as the float ones.
 * Run on the GPU's FP64 units through the general per-line path: for
 * completeness and FP64 checks, not throughput. */
DWT_EXPORT void dwt_cdf97_2f_d(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                               int size_i_big_x, int size_i_big_y, int *j_max_ptr, int decompose_one,
                               int zero_padding);
DWT_EXPORT void dwt_cdf53_2f_d(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                               int size_i_big_x, int size_i_big_y, int *j_max_ptr, int decompose_one,
                               int zero_padding);
DWT_EXPORT void dwt_cdf97_2i_d(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                               int size_i_big_x, int size_i_big_y, int j_max, int decompose_one,
                               int zero_padding);
DWT_EXPORT void dwt_cdf53_2i_d(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                               int size_i_big_x, int size_i_big_y, int j_max, int decompose_one,
                               int zero_padding);

/* src/libdwt.h:191-212, 299-320 (src/libdwt.c:1467-1571, 5673-5777): one
 * 1D level in double, samples `stride` bytes apart; tmp is not used. */
DWT_EXPORT void dwt_cdf97_f_ex_stride_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N,
                                        int stride);
DWT_EXPORT void dwt_cdf53_f_ex_stride_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N,
                                        int stride);
DWT_EXPORT void dwt_cdf97_i_ex_stride_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N,
                                        int stride);
DWT_EXPORT void dwt_cdf53_i_ex_stride_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N,
                                        int stride);

/* src/libdwt.h:139-158, 247-266, 29-106: the contiguous and the
 * concatenated (deprecated) forms in double. */
DWT_EXPORT void dwt_cdf97_f_ex_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N);
DWT_EXPORT void dwt_cdf53_f_ex_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N);
DWT_EXPORT void dwt_cdf97_i_ex_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N);
DWT_EXPORT void dwt_cdf53_i_ex_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N);
DWT_EXPORT void dwt_cdf97_f_d(const double *src, double *dst, double *tmp, int N);
DWT_EXPORT void dwt_cdf53_f_d(const double *src, double *dst, double *tmp, int N);
DWT_EXPORT void dwt_cdf97_i_d(const double *src, double *dst, double *tmp, int N);
DWT_EXPORT void dwt_cdf53_i_d(const double *src, double *dst, double *tmp, int N);

/* ----------------------------------------------------------------- lifecycle */

/* src/libdwt.h:851 (src/libdwt.c:7466-7490): bring up the GPU context, the
 * buffer pool and the call lanes (streams, events and device error word of
 * one call each, so that calls from several host threads overlap); also done
 * lazily by the first call. */
DWT_EXPORT void dwt_util_init(void);

/* src/libdwt.h:856 (src/libdwt.c:7492-7510): release the pool, the lanes and
 * the context's streams. */
DWT_EXPORT void dwt_util_finish(void);

/* src/libdwt.h:845 (src/libdwt.c:7668-7672): selects a CPU lifting kernel in
 * the reference; recorded and ignored here (every value computes the same
 * bits on the GPU). */
DWT_EXPORT void dwt_util_set_accel(int accel_type);

/* src/libdwt.h:606-618 (src/libdwt.c:624-634). */
DWT_EXPORT int dwt_util_ceil_log2(int x);
DWT_EXPORT int dwt_util_pow2_ceil_log2(int x);

/* ------------------------------------------------- coefficient layout helpers */

/* src/libdwt.h:1124-1129: the four subbands of one decomposition level. */
enum dwt_subbands { DWT_LL, DWT_HL, DWT_LH, DWT_HH };

/* src/libdwt.h:1295-1300: how an image is placed in its frame. */
enum dwt_array { DWT_ARR_SIMPLE, DWT_ARR_SPARSE, DWT_ARR_PACKED };

/* src/libdwt.h:1134-1187 (src/libdwt.c:8153-8262): pointer to and size of
 * subband `band` of level j_max in a transformed frame (the subband starts
 * at the halved outer size, its extent is the halved inner size). */
DWT_EXPORT void dwt_util_subband(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                                 int size_i_big_x, int size_i_big_y, int j_max, enum dwt_subbands band,
                                 void **dst_ptr, int *dst_size_x, int *dst_size_y);
DWT_EXPORT void dwt_util_subband_s(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                                   int size_i_big_x, int size_i_big_y, int j_max, enum dwt_subbands band,
                                   void **dst_ptr, int *dst_size_x, int *dst_size_y);
DWT_EXPORT void dwt_util_subband_d(void *ptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                                   int size_i_big_x, int size_i_big_y, int j_max, enum dwt_subbands band,
                                   void **dst_ptr, int *dst_size_x, int *dst_size_y);

/* src/libdwt.h:1307-1340 (src/libdwt.c:8620-8701): row stride (bytes, a
 * power-of-two row, made prime when opt_stride), element stride and the
 * outer / inner frame of an image of size_x x size_y in layout array_type. */
DWT_EXPORT void dwt_util_get_sizes_s(enum dwt_array array_type, int size_x, int size_y, int opt_stride,
                                     int *stride_x, int *stride_y, int *size_o_big_x, int *size_o_big_y,
                                     int *size_i_big_x, int *size_i_big_y);
DWT_EXPORT void dwt_util_get_sizes_d(enum dwt_array array_type, int size_x, int size_y, int opt_stride,
                                     int *stride_x, int *stride_y, int *size_o_big_x, int *size_o_big_y,
                                     int *size_i_big_x, int *size_i_big_y);

/* ------------------------------------------ performance harness and helpers */

/* src/libdwt.h:720-737, 753: timer types and their tick counter. */
enum dwt_timer_types {
    DWT_TIME_CLOCK_GETTIME,
    DWT_TIME_CLOCK_GETTIME_REALTIME,
    DWT_TIME_CLOCK_GETTIME_MONOTONIC,
    DWT_TIME_CLOCK_GETTIME_MONOTONIC_RAW,
    DWT_TIME_CLOCK_GETTIME_PROCESS_CPUTIME_ID,
    DWT_TIME_CLOCK_GETTIME_THREAD_CPUTIME_ID,
    DWT_TIME_CLOCK,
    DWT_TIME_TIMES,
    DWT_TIME_GETRUSAGE,
    DWT_TIME_GETRUSAGE_SELF,
    DWT_TIME_GETRUSAGE_CHILDREN,
    DWT_TIME_GETRUSAGE_THREAD,
    DWT_TIME_GETTIMEOFDAY,
    DWT_TIME_IOCTL_RTC,
    DWT_TIME_AUTOSELECT
};
typedef int64_t dwt_clock_t;

/* src/libdwt.c:6834-7120: the timer the harness uses by default, a tick
 * count and the ticks per second. */
DWT_EXPORT int dwt_util_clock_autoselect(void);
DWT_EXPORT dwt_clock_t dwt_util_get_clock(int type);
DWT_EXPORT dwt_clock_t dwt_util_get_frequency(int type);

/* src/libdwt.c:1140-1212: test pattern (type 0) and image allocation
 * (malloc(stride_x * size_o_big_y), abort when it fails). */
DWT_EXPORT void dwt_util_test_image_fill_s(void *ptr, int stride_x, int stride_y, int size_i_big_x,
                                           int size_i_big_y, int rand);
DWT_EXPORT void dwt_util_test_image_fill_d(void *ptr, int stride_x, int stride_y, int size_i_big_x,
                                           int size_i_big_y, int rand);
DWT_EXPORT void dwt_util_alloc_image(void **pptr, int stride_x, int stride_y, int size_o_big_x, int size_o_big_y);
DWT_EXPORT void dwt_util_free_image(void **pptr);

/* src/libdwt.c:1223-1277: 0 when two frames agree within 1e-3 (float) /
 * 1e-6 (double) and hold no NaN or infinity, else 1. */
DWT_EXPORT int dwt_util_compare_s(void *ptr1, void *ptr2, int stride_x, int stride_y, int size_i_big_x,
                                  int size_i_big_y);
DWT_EXPORT int dwt_util_compare_d(void *ptr1, void *ptr2, int stride_x, int stride_y, int size_i_big_x,
                                  int size_i_big_y);

/* src/libdwt.h:798-915: host thread controls of the CPU library; the GPU
 * path is driven by one host thread (1, setting is accepted). */
DWT_EXPORT int dwt_util_get_max_threads(void);
DWT_EXPORT int dwt_util_get_num_threads(void);
DWT_EXPORT int dwt_util_get_num_workers(void);
DWT_EXPORT void dwt_util_set_num_threads(int num_threads);

/* src/libdwt.c:8386-8617: M forward and M inverse transforms of M test
 * images (this library's GPU path), N loops, the minimum of the
 * per-transform averages in seconds. */
DWT_EXPORT void dwt_util_perf_cdf97_2_s(int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                                        int size_i_big_x, int size_i_big_y, int j_max, int decompose_one,
                                        int zero_padding, int M, int N, int clock_type, float *fwd_secs,
                                        float *inv_secs);
DWT_EXPORT void dwt_util_perf_cdf97_2_d(int stride_x, int stride_y, int size_o_big_x, int size_o_big_y,
                                        int size_i_big_x, int size_i_big_y, int j_max, int decompose_one,
                                        int zero_padding, int M, int N, int clock_type, double *fwd_secs,
                                        double *inv_secs);

/* src/libdwt.c:8703-9036: the harness over sizes min_x, ceil(1.28 x), ...,
 * max_x (square images, or single rows for _1_), one "pixels<TAB>seconds"
 * line per size into each file (gnuplot data, the reference's format). */
DWT_EXPORT void dwt_util_measure_perf_cdf97_2_s(enum dwt_array array_type, int min_x, int max_x, int opt_stride,
                                                int j_max, int decompose_one, int zero_padding, int M, int N,
                                                int clock_type, FILE *fwd_plot_data, FILE *inv_plot_data);
DWT_EXPORT void dwt_util_measure_perf_cdf97_2_d(enum dwt_array array_type, int min_x, int max_x, int opt_stride,
                                                int j_max, int decompose_one, int zero_padding, int M, int N,
                                                int clock_type, FILE *fwd_plot_data, FILE *inv_plot_data);
DWT_EXPORT void dwt_util_measure_perf_cdf97_1_s(enum dwt_array array_type, int min_x, int max_x, int opt_stride,
                                                int j_max, int decompose_one, int zero_padding, int M, int N,
                                                int clock_type, FILE *fwd_plot_data, FILE *inv_plot_data);
DWT_EXPORT void dwt_util_measure_perf_cdf97_1_d(enum dwt_array array_type, int min_x, int max_x, int opt_stride,
                                                int j_max, int decompose_one, int zero_padding, int M, int N,
                                                int clock_type, FILE *fwd_plot_data, FILE *inv_plot_data);

/* src/libdwt.c:8072-8151: the "optimal" stride is the smallest number at
 * least min_stride that passes the reference's base-2 Fermat test (so it
 * may be a base-2 pseudoprime, as in the reference). */
DWT_EXPORT int dwt_util_is_prime(int n);
DWT_EXPORT int dwt_util_next_prime(int n);
DWT_EXPORT int dwt_util_get_opt_stride(int min_stride);
DWT_EXPORT int dwt_util_get_stride(int min_stride, int opt);

/* ---------------------------------------------------- zero padding, stand-alone */

/* src/libdwt.h:355-406 (src/libdwt.c:5872-5942): zeros in L at samples
 * [ceil(N/2), N_dst_L) and in H at [floor(N/2), N_dst_H), `stride` bytes
 * apart (sizeof the element for the unstrided forms).  Host, device or
 * managed memory.  A destination shorter than its half writes nothing. */
DWT_EXPORT void dwt_zero_padding_f_s(float *dst_l, float *dst_h, int N, int N_dst_L, int N_dst_H);
DWT_EXPORT void dwt_zero_padding_f_d(double *dst_l, double *dst_h, int N, int N_dst_L, int N_dst_H);
DWT_EXPORT void dwt_zero_padding_f_stride_s(float *dst_l, float *dst_h, int N, int N_dst_L, int N_dst_H,
                                            int stride);
DWT_EXPORT void dwt_zero_padding_f_stride_d(double *dst_l, double *dst_h, int N, int N_dst_L, int N_dst_H,
                                            int stride);

/* src/libdwt.h:409-453 (src/libdwt.c:5944-6004): zeros at samples [N, N_dst). */
DWT_EXPORT void dwt_zero_padding_i_s(float *dst_l, int N, int N_dst);
DWT_EXPORT void dwt_zero_padding_i_d(double *dst_l, int N, int N_dst);
DWT_EXPORT void dwt_zero_padding_i_stride_s(float *dst_l, int N, int N_dst, int stride);
DWT_EXPORT void dwt_zero_padding_i_stride_d(double *dst_l, int N, int N_dst, int stride);

/* ------------------------------------------------ images, vectors, platform */

/* src/libdwt.h:1190-1222 (src/libdwt.c:958-986): ptr + y*stride_x + x*stride_y. */
DWT_EXPORT void *dwt_util_addr_coeff(void *ptr, int y, int x, int stride_x, int stride_y);
DWT_EXPORT float *dwt_util_addr_coeff_s(void *ptr, int y, int x, int stride_x, int stride_y);
DWT_EXPORT double *dwt_util_addr_coeff_d(void *ptr, int y, int x, int stride_x, int stride_y);

/* src/libdwt.h:645 (src/libdwt.c:1180-1192): zero the inner frame (host memory). */
DWT_EXPORT void dwt_util_test_image_zero_s(void *ptr, int stride_x, int stride_y, int size_i_big_x,
                                           int size_i_big_y);

/* src/libdwt.h:866-892 (src/libdwt.c:7532-7668): plain PGM ("P2", maxval
 * 255) of the inner frame, pixel = 255 * px / max_value truncated, clamped
 * to [0, 255]; 0 on success, 1 when the file cannot be written. */
DWT_EXPORT int dwt_util_save_to_pgm_s(const char *filename, float max_value, const void *ptr, int stride_x,
                                      int stride_y, int size_i_big_x, int size_i_big_y);
DWT_EXPORT int dwt_util_save_to_pgm_d(const char *filename, double max_value, const void *ptr, int stride_x,
                                      int stride_y, int size_i_big_x, int size_i_big_y);

/* src/libdwt.h:1227-1250 (src/libdwt.c:8326-8384): dst = log(1 + 100|src|) / 10. */
DWT_EXPORT void dwt_util_conv_show_s(const void *src, void *dst, int stride_x, int stride_y, int size_i_big_x,
                                     int size_i_big_y);
DWT_EXPORT void dwt_util_conv_show_d(const void *src, void *dst, int stride_x, int stride_y, int size_i_big_x,
                                     int size_i_big_y);

/* src/libdwt.h:961-1005 (src/libdwt.c:7716-7833): 8-byte aligned vector of an
 * even number of floats; fill with 0, 1, ...; zero; copy; compare.  The int
 * results are 0 when every element checks (normal or zero, within 1e-4). */
DWT_EXPORT float *dwt_util_allocate_vec_s(int size);
DWT_EXPORT int dwt_util_generate_vec_s(float *addr, int size);
DWT_EXPORT int dwt_util_zero_vec_s(float *addr, int size);
DWT_EXPORT int dwt_util_copy_vec_s(const float *src, float *dst, int size);
DWT_EXPORT int dwt_util_cmp_vec_s(const float *a, const float *b, int size);

/* src/libdwt.h:1010-1060 (src/libdwt.c:7921-7985): printf wrappers, and a
 * log line to stderr behind the level's prefix ("DEBUG: ", "INFO: ",
 * "WARNING: ", "ERROR: ", "TEST: "). */
enum dwt_util_loglevel { LOG_NONE = 0, LOG_DBG, LOG_INFO, LOG_WARN, LOG_ERR, LOG_TEST };
DWT_EXPORT int dwt_util_vfprintf(FILE *stream, const char *format, va_list ap);
DWT_EXPORT int dwt_util_vprintf(const char *format, va_list ap);
DWT_EXPORT int dwt_util_fprintf(FILE *stream, const char *format, ...);
DWT_EXPORT int dwt_util_printf(const char *format, ...);
DWT_EXPORT int dwt_util_log(enum dwt_util_loglevel level, const char *format, ...);

/* src/libdwt.h:708-713, 1067-1083 (src/libdwt.c:507-520, 4918, 8014-8058):
 * library version, architecture, 8-byte alignment test, host name and
 * program name. */
DWT_EXPORT const char *dwt_util_version(void);
DWT_EXPORT const char *dwt_util_arch(void);
DWT_EXPORT int dwt_util_is_aligned_8(const void *ptr);
DWT_EXPORT const char *dwt_util_node(void);
DWT_EXPORT const char *dwt_util_appname(void);

/* src/libdwt.h:744-747 (src/libdwt.c:7259-7373): 0 when the timer type is
 * available, else -1.  src/libdwt.h:950-955 (7375-7387): busy wait. */
DWT_EXPORT int dwt_util_clock_available(int type);
DWT_EXPORT void dwt_util_wait(int ms);

/* src/libdwt.h:803-823, 899, 918-945 (src/libdwt.c:6006-6060, 7389-7436,
 * 7512-7530, 7835-7919): worker and firmware controls of the reference's
 * embedded accelerator (one worker here, the firmware switch is accepted),
 * the OpenMP thread number (0: calls are not in a parallel region), abort,
 * and the platform self-test (host vectors, then a device round trip). */
enum dwt_op { DWT_OP_NONE, DWT_OP_LIFT4SA, DWT_OP_LIFT4SB };
DWT_EXPORT int dwt_util_get_max_workers(void);
DWT_EXPORT void dwt_util_set_num_workers(int num_workers);
DWT_EXPORT int dwt_util_get_thread_num(void);
DWT_EXPORT void dwt_util_switch_op(enum dwt_op op);
DWT_EXPORT void dwt_util_abort(void);
DWT_EXPORT void dwt_util_test(void);

/* ------------------------------------------------------------- extensions */

/* Error codes of the dwt_gpu_* functions (0 = success). */
#define DWT_GPU_OK 0
#define DWT_GPU_EINVAL (-1)      /* invalid arguments */
#define DWT_GPU_ECUDA (-2)       /* a CUDA call failed */
#define DWT_GPU_ENOMEM (-3)      /* device memory exhausted */
#define DWT_GPU_EDEVICE (-4)     /* a device-side wait gave up (error word set) */
#define DWT_GPU_EBUSY (-5)       /* admission refused (serving budget) */
#define DWT_GPU_ENOTFOUND (-6)   /* unknown request id */

/* Wavelet / direction selectors of the extension API. */
#define DWT_GPU_CDF97 0
#define DWT_GPU_CDF53 1

/* Last error of this thread (0 if none) and its text. */
DWT_EXPORT int dwt_gpu_get_last_error(void);
DWT_EXPORT const char *dwt_gpu_error_string(int code);

/* Non-aborting forms of the four 2D drop-ins: same arguments, wavelet and
 * direction as parameters, return an error code. */
DWT_EXPORT int dwt_gpu_2f_s(int wavelet, void *ptr, int stride_x, int stride_y, int size_o_big_x,
                 int size_o_big_y, int size_i_big_x, int size_i_big_y, int *j_max_ptr,
                 int decompose_one, int zero_padding);
DWT_EXPORT int dwt_gpu_2i_s(int wavelet, void *ptr, int stride_x, int stride_y, int size_o_big_x,
                 int size_o_big_y, int size_i_big_x, int size_i_big_y, int j_max,
                 int decompose_one, int zero_padding);

/* Non-aborting strided 1D level.  Forward (inverse = 0): a = src, b unused,
 * c_or_l = dst_l, h_or_null = dst_h.  Inverse (inverse = 1): a = src_l,
 * b = src_h, c_or_l = dst, h_or_null unused. */
DWT_EXPORT int dwt_gpu_1_s(int wavelet, int inverse, const float *a, const float *b, float *c_or_l,
                float *h_or_null, int N, int stride);

/* Every channel of a dense interleaved float image (pixel = `channels`
 * floats, rows stride_x bytes apart: the layout the reference's OpenCV
 * wrapper transforms channel by channel, src/cvdwt.cpp:67-147), in place, in
 * one call with one copy of the image each way.  The same result as
 * dwt_cdf{97,53}_2{f,i}_s on each channel (ptr + 4c, stride_y = 4 *
 * channels, outer = inner = w x h).  *j_levels: levels (< 0: the limit);
 * the forward writes back the levels it ran. */
DWT_EXPORT int dwt_gpu_2_channels_s(int wavelet, int inverse, void *ptr, int stride_x, int channels, int w, int h,
                                    int *j_levels, int decompose_one);

/* The double-precision forms of the three calls above, returning an error
 * code (dwt_cdf97_2f_d and friends abort instead, like libdwt). */
DWT_EXPORT int dwt_gpu_2f_d(int wavelet, void *ptr, int stride_x, int stride_y, int size_o_big_x,
                            int size_o_big_y, int size_i_big_x, int size_i_big_y, int *j_max_ptr,
                            int decompose_one, int zero_padding);
DWT_EXPORT int dwt_gpu_2i_d(int wavelet, void *ptr, int stride_x, int stride_y, int size_o_big_x,
                            int size_o_big_y, int size_i_big_x, int size_i_big_y, int j_max, int decompose_one,
                            int zero_padding);
DWT_EXPORT int dwt_gpu_1_d(int wavelet, int inverse, const double *a, const double *b, double *c_or_l,
                           double *h_or_null, int N, int stride);

/* Device-resident, out-of-place, asynchronous dense 2D transform of a w x h
 * image (outer == inner): src and dst are device pointers with row pitches in
 * bytes; src rows must be 16-byte aligned (pitch a multiple of 16, base
 * 16-byte aligned).  The result is the reference's in-place layout written to
 * dst.  j_levels < 0 means the full depth; the achieved depth is returned
 * (>= 0) or an error code (< 0).  stream is a cudaStream_t (0 = default).
 * Out of place only: frames whose byte spans intersect return DWT_GPU_EINVAL
 * (unless j_levels resolves to 0).  Work is enqueued; the call does not
 * synchronize; dwt_gpu_sync_check reports a device-side error of it. */
DWT_EXPORT int dwt_gpu_2_dev(int wavelet, int inverse, const float *src, long long src_pitch_bytes,
                  float *dst, long long dst_pitch_bytes, int w, int h, int j_levels,
                  int decompose_one, void *stream);

/* One decomposition level, device-resident and out of place, enqueued on
 * `stream`.  Forward: in[0] is the interleaved w x h image, out[0..3] receive
 * LL, HL, LH, HH.  Inverse: in[0..3] are LL, HL, LH, HH of a w x h image,
 * out[0] receives it.  Source pitches must be multiples of 16 bytes (and the
 * forward source 16-byte aligned); destinations need 4-byte alignment. */
DWT_EXPORT int dwt_gpu_level_dev(int wavelet, int inverse, int w, int h, const float *const in[4],
                                 const long long in_pitch_bytes[4], float *const out[4],
                                 const long long out_pitch_bytes[4], void *stream);

/* Kernel launches of one dense transform of a w x h image to j_levels
 * levels (< 0: the full depth of the smaller side), the same in either
 * direction: one level kernel per level down to the band the single-CTA
 * coarse kernel takes, then one coarse launch for the rest. */
DWT_EXPORT int dwt_gpu_dense_launches(int w, int h, int j_levels);

/* Failure detection without a fault: a one-warp kernel waits on an mbarrier
 * that nothing completes, through the same bounded wait the level kernels
 * use, limited to `iterations` tries.  The wait gives up, sets the device
 * error word and returns; the call reports DWT_GPU_EDEVICE (and logs the
 * code), and the context stays usable.  DWT_GPU_EINVAL for iterations <= 0. */
DWT_EXPORT int dwt_gpu_selftest_wait_timeout(int iterations);

/* No counterpart in the reference.  Test hook of the ordered in-place level
 * (the drop-in 2D calls on device frames): one warp waits, through the same
 * bounded wait, for segments of a level that nothing finishes, limited to
 * `iterations` polls; the wait gives up, sets the device error word and
 * returns.  The call reports DWT_GPU_EDEVICE (and logs the code); the context
 * stays usable.  DWT_GPU_EINVAL for iterations <= 0. */
DWT_EXPORT int dwt_gpu_selftest_inplace_wait_timeout(int iterations);

/* No counterpart in the reference.  The plan of level 0 of an in-place
 * transform of a w x h image in a device frame whose LH / HH bands start at
 * frame row detail_row ((h + 1) / 2 when negative: a dense frame; the outer
 * midpoint of a zero-padded sparse frame), host only, no device work:
 * segments of *seg_pairs row pairs, *n_segs of them, handed out bottom-up
 * (forward) or top-down (inverse); segments >= *stage_seg pass their LH / HH
 * rows through the staging frame.  When `readers` is not null it receives,
 * per segment s, the inclusive range readers[2s] .. readers[2s+1] of the
 * segments that must finish before s writes into the frame (empty when the
 * second is smaller).  For tests and tuning; DWT_GPU_EINVAL for w or h < 2
 * or 0 <= detail_row < (h + 1) / 2. */
DWT_EXPORT int dwt_gpu_inplace_plan(int wavelet, int inverse, int w, int h, int detail_row, int *seg_pairs,
                                    int *n_segs, int *stage_seg, int *readers);

/* Waits for all device work and reports (and clears) a device-side error:
 * DWT_GPU_EDEVICE when a bounded device-side wait of the library's own
 * context or of dwt_gpu_2_dev_noalloc (on any device it ran on) gave up.
 * Creates nothing: a process that only ever called dwt_gpu_2_dev_noalloc
 * can check its work without the pooled context being set up. */
DWT_EXPORT int dwt_gpu_sync_check(void);

/* No counterpart in the reference.  dwt_gpu_2_dev without any device
 * allocation, for callers that may not allocate device memory: plugins whose
 * host application owns every device allocation, services that budget every
 * byte, and latency-critical loops that cannot risk cudaMalloc/cudaFree (which
 * may synchronize the device).  Its inter-level scratch is a fixed ~5.2 MB
 * array inside the library (held by every GPU that loads it, until exit);
 * images up to 2048 x 2048 fit, larger ones return DWT_GPU_EINVAL, and so do
 * overlapping source and destination frames (out of place only).  The first
 * call on a device looks the array up (make it before any stream capture); a
 * cudaDeviceReset invalidates that address, so make no further call after
 * one.  All calls share the array: calls whose GPU work overlaps race.  The
 * call enqueues and returns; dwt_gpu_sync_check reports a device-side wait
 * that gave up (DWT_GPU_EDEVICE). */
DWT_EXPORT int dwt_gpu_2_dev_noalloc(int wavelet, int inverse, const float *src,
                                     long long src_pitch_bytes, float *dst,
                                     long long dst_pitch_bytes, int w, int h, int j_levels,
                                     int decompose_one, void *stream);

/* No counterpart in the reference.  Test hook of the error path above: a
 * one-warp kernel on the default stream waits (bounded, `iterations` tries)
 * on an mbarrier that nothing completes and sets the error word of
 * dwt_gpu_2_dev_noalloc on the current device, as a level kernel does when its
 * staged data never arrives; no fault, no allocation.  Enqueues and returns;
 * dwt_gpu_sync_check then reports DWT_GPU_EDEVICE.  DWT_GPU_EINVAL for
 * iterations <= 0. */
DWT_EXPORT int dwt_gpu_selftest_noalloc_wait_timeout(int iterations);

/* Batched strided 1D level, in place, device or host memory: `count`
 * signals of N samples, signal s at base + (s / group) * group_stride +
 * (s % group) * lane_stride bytes, samples `stride` bytes apart; L to samples
 * [0, ceil(N/2)), H to [ceil(N/2), N) of each signal (the layout of a caller
 * running dwt_cdf97_f_ex_stride_s with dst_l = src, dst_h = src +
 * ceil(N/2)*stride on every signal).  One launch for the whole bank. */
DWT_EXPORT int dwt_gpu_1_batch_s(int wavelet, int inverse, void *base, int N, int stride, long long count,
                      int group, long long group_stride, int lane_stride);

/* ------------------------------------------------------------- batches */

/* One image of a batch: device frames, out of place (src rows 16-byte
 * aligned), a w x h dense image, j_levels < 0 for the full depth, wavelet
 * DWT_GPU_CDF97 / DWT_GPU_CDF53, inverse 0 / 1. */
typedef struct {
    const float *src;
    long long src_pitch_bytes;
    float *dst;
    long long dst_pitch_bytes;
    int w, h;
    int j_levels;
    int decompose_one;
    int wavelet;
    int inverse;
} dwt_gpu_batch_image;

/* Tunables of the batched kernel: rows pairs per work unit (tile height),
 * side of the band from which one warp runs all remaining levels (the
 * fused-level depth; 0 = none), resident CTAs per SM. */
typedef struct {
    int seg_pairs;
    int tail_side;
    int ctas_per_sm;
} dwt_gpu_batch_params;

typedef struct dwt_gpu_batch dwt_gpu_batch;

/* Plans a batch: descriptors, work queue, scratch, and a CUDA graph of one
 * persistent launch.  params = NULL runs the autotuner (times candidate
 * settings on this batch, caches the winner by batch signature in
 * $DWT_GPU_TUNE_CACHE or ~/.cache/libdwt_gb300_batch_tune.txt).  While
 * tuning, dst frames are written. */
DWT_EXPORT int dwt_gpu_batch_create(dwt_gpu_batch **out, int n, const dwt_gpu_batch_image *images,
                                    const dwt_gpu_batch_params *params);
/* Replays the batch's graph on `stream` (asynchronous). */
DWT_EXPORT int dwt_gpu_batch_run(dwt_gpu_batch *b, void *stream);
DWT_EXPORT int dwt_gpu_batch_params_get(const dwt_gpu_batch *b, dwt_gpu_batch_params *p);
/* Work items of the planned batch. */
DWT_EXPORT int dwt_gpu_batch_items(const dwt_gpu_batch *b);
DWT_EXPORT void dwt_gpu_batch_destroy(dwt_gpu_batch *b);

/* --------------------------------------------------------------- serving */

/* One transform request: src a device frame (rows 16-byte aligned), dst a
 * device frame or NULL (the server then writes into a pooled buffer it
 * releases on completion), w x h, j_levels < 0 for the full depth. */
typedef struct {
    const float *src;
    long long src_pitch_bytes;
    float *dst;
    long long dst_pitch_bytes;
    int w, h;
    int j_levels;
    int decompose_one;
    int wavelet;
    int inverse;
    long long tag; /* returned with the completion */
} dwt_gpu_request;

/* A finished request; times in seconds on the steady clock. */
typedef struct {
    long long id;
    long long tag;
    int status;
    double t_submit;
    double t_admit;
    double t_complete;
} dwt_gpu_completion;

typedef struct {
    long long submitted, completed, launches, pending;
    long long bytes_in_use, peak_bytes, budget_bytes;
    long long arena_bytes;     /* device memory the server's arena holds */
    long long device_allocs;   /* cudaMalloc / cudaHostAlloc calls of the server since it started */
    long long max_dispatch_ns; /* longest dispatcher iteration since the last reserve / replay */
} dwt_gpu_server_stats_t;

typedef struct dwt_gpu_server dwt_gpu_server;

/* Starts a server: requests are admitted in arrival order while their device
 * memory (scratch + pooled output) fits `budget_bytes`, grouped into
 * micro-batches of the batched kernel and run on `n_streams` streams that
 * overlap on the device.  params = NULL uses (32, 32, 4). */
DWT_EXPORT int dwt_gpu_server_create(dwt_gpu_server **out, long long budget_bytes, int n_streams,
                                     const dwt_gpu_batch_params *params);
/* Reserves `bytes` (at most the budget) of device memory for the server's
 * arena, out of which every request's output and scratch are carved, and runs
 * one small and one large request of each wavelet and direction so that every
 * kernel is loaded and configured.  Call it once after create, before the
 * first client request: afterwards no cudaMalloc / cudaFree runs while
 * requests are served unless a request fits nowhere in the reserved slabs
 * (the arena then grows by one slab, up to the budget).  Without it the
 * arena grows on demand, 1 GiB at a time. */
DWT_EXPORT int dwt_gpu_server_reserve(dwt_gpu_server *s, long long bytes);
/* Queues a request (never blocks); DWT_GPU_EBUSY if it alone exceeds the budget. */
DWT_EXPORT int dwt_gpu_server_submit(dwt_gpu_server *s, const dwt_gpu_request *r, long long *id);
/* Takes up to `max` completions. */
DWT_EXPORT int dwt_gpu_server_poll(dwt_gpu_server *s, dwt_gpu_completion *out, int max, int *n);
/* Waits until every submitted request completed (DWT_GPU_EBUSY on timeout). */
DWT_EXPORT int dwt_gpu_server_drain(dwt_gpu_server *s, double timeout_s);
DWT_EXPORT int dwt_gpu_server_stats(dwt_gpu_server *s, dwt_gpu_server_stats_t *st);
/* Submits reqs[i] at arrival_s[i] seconds after the call (real time, from
 * the calling thread), drains, and writes each request's arrival-to-
 * completion latency. */
DWT_EXPORT int dwt_gpu_server_replay(dwt_gpu_server *s, int n, const double *arrival_s,
                                     const dwt_gpu_request *reqs, double *latency_s, double timeout_s);
DWT_EXPORT void dwt_gpu_server_destroy(dwt_gpu_server *s);

#ifdef __cplusplus
}
#endif

#endif /* LIBDWT_GB300_H */
