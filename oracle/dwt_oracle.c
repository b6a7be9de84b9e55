/*
 * CPU oracle for the libdwt lifting hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C99, the algorithm of libdwt (slchen/libdwt,
 * VERSION 2013-01-29-dev) for the functions the GPU library replaces.  It is the
 * checker for the CUDA path and the timed CPU baseline ("port") of bench.py; the
 * product library never links, loads or calls it.
 *
 * Parity is pinned two ways (see tests/test_oracle_pin.py):
 *   - bit-exact against golden vectors produced by the reference itself
 *     (tests/golden/make_golden.py runs src/libdwt.c compiled by the `ref`
 *     target of oracle/Makefile), and
 *   - bit-exact against the compiled reference directly where it is present.
 *
 * Arithmetic rules that make the float path bit-identical to the reference:
 *   - every lifting update is x + c*(l + r) with three separately rounded float
 *     operations (no FMA: build with -ffp-contract=off);
 *   - whole-sample symmetric extension: the missing neighbour of an end sample
 *     is its only neighbour, so x[0] + c*(x[1]+x[1]) == x[0] + (2c)*x[1] as in
 *     accel_lift_op4s_prolog_s / _epilog_s / _short_s (src/libdwt.c:5036-5377);
 *   - CDF 9/7 float scaling multiplies by zeta and by (1/zeta) computed as a
 *     float division (accel_lift_op4s_main_s, src/libdwt.c:1584-1643), except
 *     that the N==1 inverse multiplies by the separately rounded constant
 *     dwt_cdf97_s2_s (src/libdwt.c:5790-5794);
 *   - CDF 5/3 float scaling uses the two constants s1 and s2
 *     (src/libdwt.c:5589-5592, 5850-5853).
 */
#include <stddef.h>
#include <string.h>
#include <stdlib.h>
#include <math.h>

#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdint.h>

/* Lifting constants, src/libdwt.c:541-573. */
static const float  cdf97_p1_s =  1.58613434342059;
static const float  cdf97_u1_s = -0.0529801185729;
static const float  cdf97_p2_s = -0.8829110755309;
static const float  cdf97_u2_s =  0.4435068520439;
static const float  cdf97_s1_s =  1.1496043988602;
static const float  cdf97_s2_s =  1/1.1496043988602;

static const double cdf97_p1_d =  1.58613434342059;
static const double cdf97_u1_d = -0.0529801185729;
static const double cdf97_p2_d = -0.8829110755309;
static const double cdf97_u2_d =  0.4435068520439;
static const double cdf97_s1_d =  1.1496043988602;
static const double cdf97_s2_d =  1/1.1496043988602;

static const float  cdf53_p1_s = 0.5;
static const float  cdf53_u1_s = 0.25;
static const float  cdf53_s1_s = 1.41421356237309504880;
static const float  cdf53_s2_s = 0.70710678118654752440;

static const double cdf53_p1_d = 0.5;
static const double cdf53_u1_d = 0.25;
static const double cdf53_s1_d = 1.41421356237309504880;
static const double cdf53_s2_d = 0.70710678118654752440;

/* Level geometry, src/libdwt.c:576-672. */
static int ceil_div_pow2(int i, int j) { return (i + (1 << j) - 1) >> j; }
static int ceil_div2(int x) { return (x + 1) >> 1; }
static int floor_div2(int x) { return x >> 1; }
static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

int oracle_ceil_log2(int x)
{
	/* ceil(log2(x)) for x > 0, the value of ceil_log2() at src/libdwt.c:617-622 */
	int r = 0;
	while ((1L << r) < (long)x)
		r++;
	return r;
}

#define ADDR_S(p, y, x, sx, sy) ((float *)((char *)(p) + (ptrdiff_t)(y) * (sx) + (ptrdiff_t)(x) * (sy)))
#define ADDR_D(p, y, x, sx, sy) ((double *)((char *)(p) + (ptrdiff_t)(y) * (sx) + (ptrdiff_t)(x) * (sy)))
#define AT_S(p, i, st) (*(float *)((char *)(p) + (ptrdiff_t)(i) * (st)))
#define AT_D(p, i, st) (*(double *)((char *)(p) + (ptrdiff_t)(i) * (st)))

/* One lifting step on every sample of the given parity of x[0..N), N >= 2,
 * with whole-sample symmetric extension at both ends. */
static void lift_s(float *x, int N, int parity, float c)
{
	for (int i = parity; i < N; i += 2) {
		const float l = (i > 0) ? x[i - 1] : x[i + 1];
		const float r = (i + 1 < N) ? x[i + 1] : x[i - 1];
		x[i] = x[i] + c * (l + r);
	}
}

static void lift_d(double *x, int N, int parity, double c)
{
	for (int i = parity; i < N; i += 2) {
		const double l = (i > 0) ? x[i - 1] : x[i + 1];
		const double r = (i + 1 < N) ? x[i + 1] : x[i - 1];
		x[i] = x[i] - c * (l + r);
	}
}

static void scale_s(float *x, int N, float even, float odd)
{
	for (int i = 0; i < N; i += 2) x[i] = x[i] * even;
	for (int i = 1; i < N; i += 2) x[i] = x[i] * odd;
}

static void scale_d(double *x, int N, double even, double odd)
{
	for (int i = 0; i < N; i += 2) x[i] = x[i] * even;
	for (int i = 1; i < N; i += 2) x[i] = x[i] * odd;
}

/* ---------------------------------------------------------------- float 1D */

/* dwt_cdf97_f_ex_stride_s, src/libdwt.c:5512-5557: gather, lift with
 * (alpha,beta,gamma,delta) = (-p1,u1,-p2,u2), scale, deinterleave. */
void oracle_cdf97_f_ex_stride_s(const float *src, float *dst_l, float *dst_h,
                                float *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst_l[0] = src[0] * cdf97_s1_s;
		return;
	}
	for (int i = 0; i < N; i++) tmp[i] = AT_S(src, i, stride);
	lift_s(tmp, N, 1, -cdf97_p1_s);
	lift_s(tmp, N, 0, cdf97_u1_s);
	lift_s(tmp, N, 1, -cdf97_p2_s);
	lift_s(tmp, N, 0, cdf97_u2_s);
	scale_s(tmp, N, cdf97_s1_s, 1 / cdf97_s1_s);
	for (int i = 0; i < ceil_div2(N); i++) AT_S(dst_l, i, stride) = tmp[2 * i];
	for (int i = 0; i < floor_div2(N); i++) AT_S(dst_h, i, stride) = tmp[2 * i + 1];
}

/* dwt_cdf97_i_ex_stride_s, src/libdwt.c:5779-5824: interleave, pre-scale,
 * lift with (alpha,beta,gamma,delta) = (-u2,p2,-u1,p1), scatter. */
void oracle_cdf97_i_ex_stride_s(const float *src_l, const float *src_h, float *dst,
                                float *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst[0] = src_l[0] * cdf97_s2_s;
		return;
	}
	for (int i = 0; i < ceil_div2(N); i++) tmp[2 * i] = AT_S(src_l, i, stride);
	for (int i = 0; i < floor_div2(N); i++) tmp[2 * i + 1] = AT_S(src_h, i, stride);
	scale_s(tmp, N, 1 / cdf97_s1_s, cdf97_s1_s);
	lift_s(tmp, N, 0, -cdf97_u2_s);
	lift_s(tmp, N, 1, cdf97_p2_s);
	lift_s(tmp, N, 0, -cdf97_u1_s);
	lift_s(tmp, N, 1, cdf97_p1_s);
	for (int i = 0; i < N; i++) AT_S(dst, i, stride) = tmp[i];
}

/* dwt_cdf53_f_ex_stride_s, src/libdwt.c:5559-5603. */
void oracle_cdf53_f_ex_stride_s(const float *src, float *dst_l, float *dst_h,
                                float *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst_l[0] = src[0] * cdf53_s1_s;
		return;
	}
	for (int i = 0; i < N; i++) tmp[i] = AT_S(src, i, stride);
	lift_s(tmp, N, 1, -cdf53_p1_s);
	lift_s(tmp, N, 0, cdf53_u1_s);
	scale_s(tmp, N, cdf53_s1_s, cdf53_s2_s);
	for (int i = 0; i < ceil_div2(N); i++) AT_S(dst_l, i, stride) = tmp[2 * i];
	for (int i = 0; i < floor_div2(N); i++) AT_S(dst_h, i, stride) = tmp[2 * i + 1];
}

/* dwt_cdf53_i_ex_stride_s, src/libdwt.c:5826-5870. */
void oracle_cdf53_i_ex_stride_s(const float *src_l, const float *src_h, float *dst,
                                float *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst[0] = src_l[0] * cdf53_s2_s;
		return;
	}
	for (int i = 0; i < ceil_div2(N); i++) tmp[2 * i] = AT_S(src_l, i, stride);
	for (int i = 0; i < floor_div2(N); i++) tmp[2 * i + 1] = AT_S(src_h, i, stride);
	scale_s(tmp, N, cdf53_s2_s, cdf53_s1_s);
	lift_s(tmp, N, 0, -cdf53_u1_s);
	lift_s(tmp, N, 1, cdf53_p1_s);
	for (int i = 0; i < N; i++) AT_S(dst, i, stride) = tmp[i];
}

/* --------------------------------------------------------------- double 1D */

/* dwt_cdf97_f_ex_stride_d, src/libdwt.c:1467-1525 (lift_d subtracts c*(l+r)). */
void oracle_cdf97_f_ex_stride_d(const double *src, double *dst_l, double *dst_h,
                                double *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst_l[0] = src[0] * cdf97_s1_d;
		return;
	}
	for (int i = 0; i < N; i++) tmp[i] = AT_D(src, i, stride);
	lift_d(tmp, N, 1, cdf97_p1_d);
	lift_d(tmp, N, 0, -cdf97_u1_d);
	lift_d(tmp, N, 1, cdf97_p2_d);
	lift_d(tmp, N, 0, -cdf97_u2_d);
	scale_d(tmp, N, cdf97_s1_d, cdf97_s2_d);
	for (int i = 0; i < ceil_div2(N); i++) AT_D(dst_l, i, stride) = tmp[2 * i];
	for (int i = 0; i < floor_div2(N); i++) AT_D(dst_h, i, stride) = tmp[2 * i + 1];
}

/* dwt_cdf97_i_ex_stride_d, src/libdwt.c:5673-5731. */
void oracle_cdf97_i_ex_stride_d(const double *src_l, const double *src_h, double *dst,
                                double *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst[0] = src_l[0] * cdf97_s2_d;
		return;
	}
	for (int i = 0; i < ceil_div2(N); i++) tmp[2 * i] = AT_D(src_l, i, stride);
	for (int i = 0; i < floor_div2(N); i++) tmp[2 * i + 1] = AT_D(src_h, i, stride);
	scale_d(tmp, N, cdf97_s2_d, cdf97_s1_d);
	lift_d(tmp, N, 0, cdf97_u2_d);
	lift_d(tmp, N, 1, -cdf97_p2_d);
	lift_d(tmp, N, 0, cdf97_u1_d);
	lift_d(tmp, N, 1, -cdf97_p1_d);
	for (int i = 0; i < N; i++) AT_D(dst, i, stride) = tmp[i];
}

/* dwt_cdf53_f_ex_stride_d, src/libdwt.c:1527-1571. */
void oracle_cdf53_f_ex_stride_d(const double *src, double *dst_l, double *dst_h,
                                double *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst_l[0] = src[0] * cdf53_s1_d;
		return;
	}
	for (int i = 0; i < N; i++) tmp[i] = AT_D(src, i, stride);
	lift_d(tmp, N, 1, cdf53_p1_d);
	lift_d(tmp, N, 0, -cdf53_u1_d);
	scale_d(tmp, N, cdf53_s1_d, cdf53_s2_d);
	for (int i = 0; i < ceil_div2(N); i++) AT_D(dst_l, i, stride) = tmp[2 * i];
	for (int i = 0; i < floor_div2(N); i++) AT_D(dst_h, i, stride) = tmp[2 * i + 1];
}

/* dwt_cdf53_i_ex_stride_d, src/libdwt.c:5733-5777. */
void oracle_cdf53_i_ex_stride_d(const double *src_l, const double *src_h, double *dst,
                                double *tmp, int N, int stride)
{
	if (N < 2) {
		if (N == 1)
			dst[0] = src_l[0] * cdf53_s2_d;
		return;
	}
	for (int i = 0; i < ceil_div2(N); i++) tmp[2 * i] = AT_D(src_l, i, stride);
	for (int i = 0; i < floor_div2(N); i++) tmp[2 * i + 1] = AT_D(src_h, i, stride);
	scale_d(tmp, N, cdf53_s2_d, cdf53_s1_d);
	lift_d(tmp, N, 0, cdf53_u1_d);
	lift_d(tmp, N, 1, -cdf53_p1_d);
	for (int i = 0; i < N; i++) AT_D(dst, i, stride) = tmp[i];
}

/* ------------------------------------------------------------ zero padding */

/* dwt_zero_padding_f_stride_s, src/libdwt.c:5925-5942. */
static void zero_padding_f_s(float *dst_l, float *dst_h, int N, int N_dst_L, int N_dst_H, int stride)
{
	if (N_dst_L || N_dst_H) {
		for (int i = ceil_div2(N); i < N_dst_L; i++) AT_S(dst_l, i, stride) = 0.0f;
		for (int i = floor_div2(N); i < N_dst_H; i++) AT_S(dst_h, i, stride) = 0.0f;
	}
}

/* dwt_zero_padding_i_stride_s, src/libdwt.c:5988-6004. */
static void zero_padding_i_s(float *dst, int N, int N_dst, int stride)
{
	for (int i = N; i < N_dst; i++) AT_S(dst, i, stride) = 0.0f;
}

static void zero_padding_f_d(double *dst_l, double *dst_h, int N, int N_dst_L, int N_dst_H, int stride)
{
	if (N_dst_L || N_dst_H) {
		for (int i = ceil_div2(N); i < N_dst_L; i++) AT_D(dst_l, i, stride) = 0.0;
		for (int i = floor_div2(N); i < N_dst_H; i++) AT_D(dst_h, i, stride) = 0.0;
	}
}

static void zero_padding_i_d(double *dst, int N, int N_dst, int stride)
{
	for (int i = N; i < N_dst; i++) AT_D(dst, i, stride) = 0.0;
}

/* ---------------------------------------------------------------- float 2D */

typedef void (*fwd1_s_t)(const float *, float *, float *, float *, int, int);
typedef void (*inv1_s_t)(const float *, const float *, float *, float *, int, int);
typedef void (*fwd1_d_t)(const double *, double *, double *, double *, int, int);
typedef void (*inv1_d_t)(const double *, const double *, double *, double *, int, int);

/* Multi-level in-place forward driver, the structure of dwt_cdf97_2f_s
 * (src/libdwt.c:6286-6408) and dwt_cdf53_2f_s (6410-6491): per level, rows
 * y < outer height get an inner-width transform, then columns x < outer width
 * get an inner-height transform, then optional zero padding.  `threads` > 1
 * runs the row and column loops with OpenMP, as the reference does. */
static void fwd2_s(fwd1_s_t f, void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                   int *j_max_ptr, int decompose_one, int zero_padding, int threads)
{
	const int j_limit = oracle_ceil_log2(decompose_one ? imax(ox, oy) : imin(ox, oy));
	if (*j_max_ptr < 0 || *j_max_ptr > j_limit)
		*j_max_ptr = j_limit;
	const int tmp_len = imax(imax(ox, oy), imax(ix, iy)) + 4;
	(void)threads;

	for (int j = 0; j < *j_max_ptr; j++) {
		const int osx = ceil_div_pow2(ox, j), osy = ceil_div_pow2(oy, j);
		const int odx = ceil_div_pow2(ox, j + 1), ody = ceil_div_pow2(oy, j + 1);
		const int isx = ceil_div_pow2(ix, j), isy = ceil_div_pow2(iy, j);

		#pragma omp parallel num_threads(threads) if(threads > 1)
		{
			float *tmp = (float *)malloc(sizeof(float) * tmp_len);
			#pragma omp for schedule(static)
			for (int y = 0; y < osy; y++)
				f(ADDR_S(ptr, y, 0, sx, sy), ADDR_S(ptr, y, 0, sx, sy),
				  ADDR_S(ptr, y, odx, sx, sy), tmp, isx, sy);
			#pragma omp for schedule(static)
			for (int x = 0; x < osx; x++)
				f(ADDR_S(ptr, 0, x, sx, sy), ADDR_S(ptr, 0, x, sx, sy),
				  ADDR_S(ptr, ody, x, sx, sy), tmp, isy, sx);
			free(tmp);
		}
		if (zero_padding) {
			for (int y = 0; y < osy; y++)
				zero_padding_f_s(ADDR_S(ptr, y, 0, sx, sy), ADDR_S(ptr, y, odx, sx, sy),
				                 isx, odx, osx - odx, sy);
			for (int x = 0; x < osx; x++)
				zero_padding_f_s(ADDR_S(ptr, 0, x, sx, sy), ADDR_S(ptr, ody, x, sx, sy),
				                 isy, ody, osy - ody, sx);
		}
	}
}

/* Multi-level in-place inverse driver, dwt_cdf97_2i_s (src/libdwt.c:6647-6755)
 * and dwt_cdf53_2i_s (6757-6832): levels j..1, rows first, then columns. */
static void inv2_s(inv1_s_t f, void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                   int j_max, int decompose_one, int zero_padding, int threads)
{
	int j = oracle_ceil_log2(decompose_one ? imax(ox, oy) : imin(ox, oy));
	if (j_max >= 0 && j_max < j)
		j = j_max;
	const int tmp_len = imax(imax(ox, oy), imax(ix, iy)) + 4;
	(void)threads;

	for (; j > 0; j--) {
		const int osx = ceil_div_pow2(ox, j), osy = ceil_div_pow2(oy, j);
		const int odx = ceil_div_pow2(ox, j - 1), ody = ceil_div_pow2(oy, j - 1);
		const int idx = ceil_div_pow2(ix, j - 1), idy = ceil_div_pow2(iy, j - 1);

		#pragma omp parallel num_threads(threads) if(threads > 1)
		{
			float *tmp = (float *)malloc(sizeof(float) * tmp_len);
			#pragma omp for schedule(static)
			for (int y = 0; y < ody; y++)
				f(ADDR_S(ptr, y, 0, sx, sy), ADDR_S(ptr, y, osx, sx, sy),
				  ADDR_S(ptr, y, 0, sx, sy), tmp, idx, sy);
			#pragma omp for schedule(static)
			for (int x = 0; x < odx; x++)
				f(ADDR_S(ptr, 0, x, sx, sy), ADDR_S(ptr, osy, x, sx, sy),
				  ADDR_S(ptr, 0, x, sx, sy), tmp, idy, sx);
			free(tmp);
		}
		if (zero_padding) {
			for (int y = 0; y < ody; y++)
				zero_padding_i_s(ADDR_S(ptr, y, 0, sx, sy), idx, odx, sy);
			for (int x = 0; x < odx; x++)
				zero_padding_i_s(ADDR_S(ptr, 0, x, sx, sy), idy, ody, sx);
		}
	}
}

static void fwd2_d(fwd1_d_t f, void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                   int *j_max_ptr, int decompose_one, int zero_padding, int threads)
{
	const int j_limit = oracle_ceil_log2(decompose_one ? imax(ox, oy) : imin(ox, oy));
	if (*j_max_ptr < 0 || *j_max_ptr > j_limit)
		*j_max_ptr = j_limit;
	const int tmp_len = imax(imax(ox, oy), imax(ix, iy)) + 4;
	(void)threads;

	for (int j = 0; j < *j_max_ptr; j++) {
		const int osx = ceil_div_pow2(ox, j), osy = ceil_div_pow2(oy, j);
		const int odx = ceil_div_pow2(ox, j + 1), ody = ceil_div_pow2(oy, j + 1);
		const int isx = ceil_div_pow2(ix, j), isy = ceil_div_pow2(iy, j);

		#pragma omp parallel num_threads(threads) if(threads > 1)
		{
			double *tmp = (double *)malloc(sizeof(double) * tmp_len);
			#pragma omp for schedule(static)
			for (int y = 0; y < osy; y++)
				f(ADDR_D(ptr, y, 0, sx, sy), ADDR_D(ptr, y, 0, sx, sy),
				  ADDR_D(ptr, y, odx, sx, sy), tmp, isx, sy);
			#pragma omp for schedule(static)
			for (int x = 0; x < osx; x++)
				f(ADDR_D(ptr, 0, x, sx, sy), ADDR_D(ptr, 0, x, sx, sy),
				  ADDR_D(ptr, ody, x, sx, sy), tmp, isy, sx);
			free(tmp);
		}
		if (zero_padding) {
			for (int y = 0; y < osy; y++)
				zero_padding_f_d(ADDR_D(ptr, y, 0, sx, sy), ADDR_D(ptr, y, odx, sx, sy),
				                 isx, odx, osx - odx, sy);
			for (int x = 0; x < osx; x++)
				zero_padding_f_d(ADDR_D(ptr, 0, x, sx, sy), ADDR_D(ptr, ody, x, sx, sy),
				                 isy, ody, osy - ody, sx);
		}
	}
}

static void inv2_d(inv1_d_t f, void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                   int j_max, int decompose_one, int zero_padding, int threads)
{
	int j = oracle_ceil_log2(decompose_one ? imax(ox, oy) : imin(ox, oy));
	if (j_max >= 0 && j_max < j)
		j = j_max;
	const int tmp_len = imax(imax(ox, oy), imax(ix, iy)) + 4;
	(void)threads;

	for (; j > 0; j--) {
		const int osx = ceil_div_pow2(ox, j), osy = ceil_div_pow2(oy, j);
		const int odx = ceil_div_pow2(ox, j - 1), ody = ceil_div_pow2(oy, j - 1);
		const int idx = ceil_div_pow2(ix, j - 1), idy = ceil_div_pow2(iy, j - 1);

		#pragma omp parallel num_threads(threads) if(threads > 1)
		{
			double *tmp = (double *)malloc(sizeof(double) * tmp_len);
			#pragma omp for schedule(static)
			for (int y = 0; y < ody; y++)
				f(ADDR_D(ptr, y, 0, sx, sy), ADDR_D(ptr, y, osx, sx, sy),
				  ADDR_D(ptr, y, 0, sx, sy), tmp, idx, sy);
			#pragma omp for schedule(static)
			for (int x = 0; x < odx; x++)
				f(ADDR_D(ptr, 0, x, sx, sy), ADDR_D(ptr, osy, x, sx, sy),
				  ADDR_D(ptr, 0, x, sx, sy), tmp, idy, sx);
			free(tmp);
		}
		if (zero_padding) {
			for (int y = 0; y < ody; y++)
				zero_padding_i_d(ADDR_D(ptr, y, 0, sx, sy), idx, odx, sy);
			for (int x = 0; x < odx; x++)
				zero_padding_i_d(ADDR_D(ptr, 0, x, sx, sy), idy, ody, sx);
		}
	}
}

/* Exported 2D entry points.  Same arguments as the reference functions plus the
 * OpenMP thread count (1 = serial). */
void oracle_cdf97_2f_s(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int *j_max_ptr, int decompose_one, int zero_padding, int threads)
{ fwd2_s(oracle_cdf97_f_ex_stride_s, ptr, sx, sy, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding, threads); }

void oracle_cdf53_2f_s(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int *j_max_ptr, int decompose_one, int zero_padding, int threads)
{ fwd2_s(oracle_cdf53_f_ex_stride_s, ptr, sx, sy, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding, threads); }

void oracle_cdf97_2i_s(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int j_max, int decompose_one, int zero_padding, int threads)
{ inv2_s(oracle_cdf97_i_ex_stride_s, ptr, sx, sy, ox, oy, ix, iy, j_max, decompose_one, zero_padding, threads); }

void oracle_cdf53_2i_s(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int j_max, int decompose_one, int zero_padding, int threads)
{ inv2_s(oracle_cdf53_i_ex_stride_s, ptr, sx, sy, ox, oy, ix, iy, j_max, decompose_one, zero_padding, threads); }

void oracle_cdf97_2f_d(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int *j_max_ptr, int decompose_one, int zero_padding, int threads)
{ fwd2_d(oracle_cdf97_f_ex_stride_d, ptr, sx, sy, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding, threads); }

void oracle_cdf53_2f_d(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int *j_max_ptr, int decompose_one, int zero_padding, int threads)
{ fwd2_d(oracle_cdf53_f_ex_stride_d, ptr, sx, sy, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding, threads); }

void oracle_cdf97_2i_d(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int j_max, int decompose_one, int zero_padding, int threads)
{ inv2_d(oracle_cdf97_i_ex_stride_d, ptr, sx, sy, ox, oy, ix, iy, j_max, decompose_one, zero_padding, threads); }

void oracle_cdf53_2i_d(void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                       int j_max, int decompose_one, int zero_padding, int threads)
{ inv2_d(oracle_cdf53_i_ex_stride_d, ptr, sx, sy, ox, oy, ix, iy, j_max, decompose_one, zero_padding, threads); }

/* Batched strided 1D: `count` signals, signal s starting at byte offset
 * (s / group) * group_stride + (s % group) * lane_stride from `base`, samples
 * `stride` bytes apart, transformed in place (L to samples [0, ceil(N/2)),
 * H to [ceil(N/2), N)) with the float 1D functions above.  This is the loop
 * a caller of dwt_cdf97_{f,i}_ex_stride_s runs over a bank of signals. */
void oracle_cdf97_1_batch_s(void *base, int N, int stride, long count, int group,
                            long group_stride, int lane_stride, int inverse, int threads)
{
	(void)threads;
	#pragma omp parallel num_threads(threads) if(threads > 1)
	{
		float *tmp = (float *)malloc(sizeof(float) * (N + 4));
		#pragma omp for schedule(static)
		for (long s = 0; s < count; s++) {
			float *sig = (float *)((char *)base + (s / group) * group_stride + (s % group) * (long)lane_stride);
			float *h = (float *)((char *)sig + (ptrdiff_t)ceil_div2(N) * stride);
			if (inverse)
				oracle_cdf97_i_ex_stride_s(sig, h, sig, tmp, N, stride);
			else
				oracle_cdf97_f_ex_stride_s(sig, sig, h, tmp, N, stride);
		}
		free(tmp);
	}
}

/* The reference's own calling pattern for a bank of strided signals (the
 * OpenMP loop its callers write around dwt_cdf97_f_ex_stride_s,
 * src/libdwt.c:5512-5557): one call of `fn` per signal, in place (L at the
 * signal's start, H ceil(N/2) samples later), with a per-thread 16-byte
 * aligned tmp (forward gets tmp + 3, so that the lifting array tmp + 4 the
 * SSE kernels use is aligned; inverse gets tmp).  `fn` is the forward or
 * inverse strided function of any library with the reference's signature:
 * the compiled reference itself (timed as the CPU baseline), or the oracle. */
typedef void (*oracle_fwd1_fn)(const float *, float *, float *, float *, int, int);
typedef void (*oracle_inv1_fn)(const float *, const float *, float *, float *, int, int);

void oracle_call_1_batch_s(void *fn, void *base, int N, int stride, long count, int group,
                           long group_stride, int lane_stride, int inverse, int threads)
{
	#pragma omp parallel num_threads(threads) if(threads > 1)
	{
		void *raw = malloc(sizeof(float) * (N + 16) + 16);
		float *tmp = (float *)(((uintptr_t)raw + 15) & ~(uintptr_t)15);
		#pragma omp for schedule(static)
		for (long s = 0; s < count; s++) {
			float *sig = (float *)((char *)base + (s / group) * group_stride + (s % group) * (long)lane_stride);
			float *h = (float *)((char *)sig + (ptrdiff_t)ceil_div2(N) * stride);
			if (inverse)
				((oracle_inv1_fn)fn)(sig, h, sig, tmp, N, stride);
			else
				((oracle_fwd1_fn)fn)(sig, sig, h, tmp + 3, N, stride);
		}
		free(raw);
	}
}

/* dwt_util_test_image_fill_s, src/libdwt.c:1108-1178 (type 0 pattern). */
void oracle_test_image_fill_s(void *ptr, int sx, int sy, int ix, int iy, int rand)
{
	for (int y = 0; y < iy; y++)
		for (int x = 0; x < ix; x++) {
			const int xx = x >> rand;
			*ADDR_S(ptr, y, x, sx, sy) = 2 * xx * y / (float)(xx * xx + y * y + 1);
		}
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}
