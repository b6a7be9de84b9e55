// The rest of libdwt's public C API: the zero-padding steps of the
// transforms as stand-alone calls (host or device memory), coefficient
// addressing, image export (PGM) and the log-magnitude view of a transform,
// the float vector helpers, logging, and the platform queries.  Apart from
// the zero padding on device memory these are host code; the image and
// vector helpers take host memory, as the reference's do.
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/libdwt.h"
#include "dwt_capi_internal.h"

namespace {

// ---------------------------------------------------------------- zero padding

__global__ void zero_strided_kernel(char *base, long long stride, int n, int elem)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        char *p = base + (long long)i * stride;
        if (elem == 8)
            *reinterpret_cast<double *>(p) = 0.0;
        else
            *reinterpret_cast<float *>(p) = 0.0f;
    }
}

// Stores n zeros of `elem` bytes, `stride` bytes apart, from `base`: a loop on
// host memory, one small kernel on device or managed memory.
void zero_strided(void *base, long long stride, int n, int elem)
{
    if (n <= 0) return;
    const dwt::MemKind kind = dwt::classify(base);
    if (kind != dwt::MemKind::Device && kind != dwt::MemKind::Managed) {
        char *p = static_cast<char *>(base);
        for (int i = 0; i < n; ++i, p += stride) {
            if (elem == 8)
                *reinterpret_cast<double *>(p) = 0.0;
            else
                *reinterpret_cast<float *>(p) = 0.0f;
        }
        return;
    }
    dwt::LaneGuard lane(dwt::ctx());
    const cudaStream_t s = lane.get().stream;
    const int block = 256, grid = (n + block - 1) / block < 1024 ? (n + block - 1) / block : 1024;
    zero_strided_kernel<<<grid, block, 0, s>>>(static_cast<char *>(base), stride, n, elem);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        dwt::log_error("zero padding on device memory failed: %s\n", cudaGetErrorString(e));
        abort();
    }
}

// The reference states its preconditions as assertions (log-free abort);
// this library logs the failed condition, then aborts.
void require(bool ok, const char *fn, const char *what)
{
    if (ok) return;
    dwt::log_error("%s: precondition failed: %s\n", fn, what);
    abort();
}

int ceil_half(int n) { return (n + 1) >> 1; }
int floor_half(int n) { return n >> 1; }

// Forward padding (src/libdwt.c:5906-5942): L gets zeros at samples
// [ceil(N/2), N_dst_L), H at [floor(N/2), N_dst_H).  A destination shorter
// than the decomposed half writes nothing.
void pad_forward(void *dst_l, void *dst_h, int N, int N_dst_L, int N_dst_H, int stride, int elem, const char *fn)
{
    require(N >= 0 && N_dst_L >= 0 && N_dst_H >= 0 && dst_l && dst_h && stride != 0, fn,
            "N >= 0 && N_dst_L >= 0 && N_dst_H >= 0 && dst_l && dst_h && stride != 0");
    if (!N_dst_L && !N_dst_H) return;
    zero_strided(static_cast<char *>(dst_l) + (long long)ceil_half(N) * stride, stride, N_dst_L - ceil_half(N), elem);
    zero_strided(static_cast<char *>(dst_h) + (long long)floor_half(N) * stride, stride, N_dst_H - floor_half(N),
                 elem);
}

// Inverse padding (src/libdwt.c:5970-6004): zeros at samples [N, N_dst).
void pad_inverse(void *dst, int N, int N_dst, int stride, int elem, const char *fn)
{
    require(N >= 0 && N_dst >= 0 && dst && stride != 0, fn, "N >= 0 && N_dst >= 0 && dst && stride != 0");
    zero_strided(static_cast<char *>(dst) + (long long)N * stride, stride, N_dst - N, elem);
}

// ------------------------------------------------------------- image export

char *pixel(const void *ptr, int y, int x, int stride_x, int stride_y)
{
    return const_cast<char *>(static_cast<const char *>(ptr)) + (long long)y * stride_x + (long long)x * stride_y;
}

// Plain ("P2") PGM with maxval 255 (src/libdwt.c:7532-7668): each pixel is
// 255 * px / max_value in T, truncated toward zero; values above max_value
// give 255, negative values 0.  The first value more than `tol` outside
// [0, max_value] is reported once, and the number of such values at the end.
template <typename T>
int save_pgm(const char *fn, const char *filename, T max_value, T tol, const void *ptr, int stride_x, int stride_y,
             int size_x, int size_y)
{
    require(max_value != T(0) && size_x >= 0 && size_y >= 0, fn, "max_value != 0 && size_x >= 0 && size_y >= 0");
    const int target = 255;
    FILE *f = fopen(filename, "w");
    if (!f) return 1;
    fprintf(f, "P2\n%i %i\n%i\n", size_x, size_y, target);
    int err = 0;
    for (int y = 0; y < size_y; ++y)
        for (int x = 0; x < size_x; ++x) {
            const T px = *reinterpret_cast<const T *>(pixel(ptr, y, x, stride_x, stride_y));
            const T scaled = T(target) * px / max_value;
            // truncation toward zero; NaN and out-of-range quotients map to 0
            int val = (scaled > T(-2147483648.0) && scaled < T(2147483647.0)) ? int(scaled) : 0;
            if (px - tol > max_value && !err++)
                dwt_util_log(LOG_WARN,
                             "%s: Maximum pixel intensity exceeded (%f > %f). Such an incident will be reported "
                             "only once.\n",
                             fn, double(px), double(max_value));
            if (px > max_value) val = target;
            if (px + tol < T(0) && !err++)
                dwt_util_log(LOG_WARN,
                             "%s: Minimum pixel intensity exceeded (%f < %f). Such an incident will be reported "
                             "only once.\n",
                             fn, double(px), 0.0);
            if (px < T(0)) val = 0;
            if (fprintf(f, "%i\n", val) < 0) {
                dwt_util_log(LOG_WARN, "%s: error writing into file.\n", fn);
                fclose(f);
                return 1;
            }
        }
    fclose(f);
    if (err) dwt_util_log(LOG_WARN, "%s: %i errors ocurred while saving a file.\n", fn, err);
    return 0;
}

// ------------------------------------------------------------ vector helpers

// The reference's scalar check (src/libdwt.c:7676-7714): both values normal
// or zero, and within 1e-4 of each other.
int cmp_value(float a, float b)
{
    const bool ok_a = std::isnormal(a) || a == 0.0f, ok_b = std::isnormal(b) || b == 0.0f;
    if (!ok_a || !ok_b) {
        dwt_util_log(LOG_ERR, "%f or %f is not normal nor zero!\n", double(a), double(b));
        return 1;
    }
    if (std::fabs(a - b) > 1e-4f) {
        dwt_util_log(LOG_ERR, "%f should be %f!\n", double(a), double(b));
        return 1;
    }
    return 0;
}

// First line of a /proc file (up to `n` - 1 bytes) into buf; false if absent.
bool read_proc_line(const char *path, char *buf, int n)
{
    FILE *f = fopen(path, "r");
    if (!f) return false;
    const char *r = fgets(buf, n, f);
    fclose(f);
    return r != nullptr;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- zero padding

void dwt_zero_padding_f_stride_s(float *dst_l, float *dst_h, int N, int N_dst_L, int N_dst_H, int stride)
{
    pad_forward(dst_l, dst_h, N, N_dst_L, N_dst_H, stride, 4, "dwt_zero_padding_f_stride_s");
}

void dwt_zero_padding_f_stride_d(double *dst_l, double *dst_h, int N, int N_dst_L, int N_dst_H, int stride)
{
    pad_forward(dst_l, dst_h, N, N_dst_L, N_dst_H, stride, 8, "dwt_zero_padding_f_stride_d");
}

void dwt_zero_padding_f_s(float *dst_l, float *dst_h, int N, int N_dst_L, int N_dst_H)
{
    pad_forward(dst_l, dst_h, N, N_dst_L, N_dst_H, int(sizeof(float)), 4, "dwt_zero_padding_f_s");
}

void dwt_zero_padding_f_d(double *dst_l, double *dst_h, int N, int N_dst_L, int N_dst_H)
{
    pad_forward(dst_l, dst_h, N, N_dst_L, N_dst_H, int(sizeof(double)), 8, "dwt_zero_padding_f_d");
}

void dwt_zero_padding_i_stride_s(float *dst_l, int N, int N_dst, int stride)
{
    pad_inverse(dst_l, N, N_dst, stride, 4, "dwt_zero_padding_i_stride_s");
}

void dwt_zero_padding_i_stride_d(double *dst_l, int N, int N_dst, int stride)
{
    pad_inverse(dst_l, N, N_dst, stride, 8, "dwt_zero_padding_i_stride_d");
}

void dwt_zero_padding_i_s(float *dst_l, int N, int N_dst)
{
    pad_inverse(dst_l, N, N_dst, int(sizeof(float)), 4, "dwt_zero_padding_i_s");
}

void dwt_zero_padding_i_d(double *dst_l, int N, int N_dst)
{
    pad_inverse(dst_l, N, N_dst, int(sizeof(double)), 8, "dwt_zero_padding_i_d");
}

// ------------------------------------------------------ coefficient addressing

void *dwt_util_addr_coeff(void *ptr, int y, int x, int stride_x, int stride_y)
{
    return pixel(ptr, y, x, stride_x, stride_y);
}

float *dwt_util_addr_coeff_s(void *ptr, int y, int x, int stride_x, int stride_y)
{
    return reinterpret_cast<float *>(pixel(ptr, y, x, stride_x, stride_y));
}

double *dwt_util_addr_coeff_d(void *ptr, int y, int x, int stride_x, int stride_y)
{
    return reinterpret_cast<double *>(pixel(ptr, y, x, stride_x, stride_y));
}

void dwt_util_test_image_zero_s(void *ptr, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y)
{
    require(ptr != nullptr, "dwt_util_test_image_zero_s", "ptr != NULL");
    for (int y = 0; y < size_i_big_y; ++y)
        for (int x = 0; x < size_i_big_x; ++x) *reinterpret_cast<float *>(pixel(ptr, y, x, stride_x, stride_y)) = 0.0f;
}

// ------------------------------------------------------------- image export

int dwt_util_save_to_pgm_s(const char *filename, float max_value, const void *ptr, int stride_x, int stride_y,
                           int size_i_big_x, int size_i_big_y)
{
    return save_pgm<float>("dwt_util_save_to_pgm_s", filename, max_value, 1e-3f, ptr, stride_x, stride_y,
                           size_i_big_x, size_i_big_y);
}

int dwt_util_save_to_pgm_d(const char *filename, double max_value, const void *ptr, int stride_x, int stride_y,
                           int size_i_big_x, int size_i_big_y)
{
    return save_pgm<double>("dwt_util_save_to_pgm_d", filename, max_value, 1e-6, ptr, stride_x, stride_y,
                            size_i_big_x, size_i_big_y);
}

// log(1 + 100 |c|) / 10 per coefficient (src/libdwt.c:8326-8384), each
// operation rounded in the element type.
void dwt_util_conv_show_s(const void *src, void *dst, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y)
{
    require(src && dst && size_i_big_x >= 0 && size_i_big_y >= 0, "dwt_util_conv_show_s",
            "src && dst && size_x >= 0 && size_y >= 0");
    for (int y = 0; y < size_i_big_y; ++y)
        for (int x = 0; x < size_i_big_x; ++x) {
            const float c = *reinterpret_cast<const float *>(pixel(src, y, x, stride_x, stride_y));
            const float m = std::fabs(c) * 100.f;
            const float t = logf(1.f + m);
            *reinterpret_cast<float *>(pixel(dst, y, x, stride_x, stride_y)) = t / 10.f;
        }
}

void dwt_util_conv_show_d(const void *src, void *dst, int stride_x, int stride_y, int size_i_big_x, int size_i_big_y)
{
    require(src && dst && size_i_big_x >= 0 && size_i_big_y >= 0, "dwt_util_conv_show_d",
            "src && dst && size_x >= 0 && size_y >= 0");
    for (int y = 0; y < size_i_big_y; ++y)
        for (int x = 0; x < size_i_big_x; ++x) {
            const double c = *reinterpret_cast<const double *>(pixel(src, y, x, stride_x, stride_y));
            const double m = std::fabs(c) * 100.;
            const double t = log(1. + m);
            *reinterpret_cast<double *>(pixel(dst, y, x, stride_x, stride_y)) = t / 10.;
        }
}

// ------------------------------------------------------------ vector helpers

float *dwt_util_allocate_vec_s(int size)
{
    require(size >= 0 && (size & 1) == 0, "dwt_util_allocate_vec_s", "size is even");
    void *p = nullptr;
    if (posix_memalign(&p, 8, sizeof(float) * size_t(size > 0 ? size : 1)) != 0) return nullptr;
    return static_cast<float *>(p);
}

int dwt_util_generate_vec_s(float *addr, int size)
{
    for (int i = 0; i < size; ++i) addr[i] = float(i);
    for (int i = 0; i < size; ++i)
        if (cmp_value(addr[i], float(i))) return 1;
    return 0;
}

int dwt_util_zero_vec_s(float *addr, int size)
{
    for (int i = 0; i < size; ++i) addr[i] = 0.0f;
    for (int i = 0; i < size; ++i)
        if (cmp_value(addr[i], 0.0f)) return 1;
    return 0;
}

int dwt_util_copy_vec_s(const float *src, float *dst, int size)
{
    if (size > 0) memcpy(dst, src, sizeof(float) * size_t(size));
    for (int i = 0; i < size; ++i)
        if (cmp_value(dst[i], src[i])) return 1;
    return 0;
}

int dwt_util_cmp_vec_s(const float *a, const float *b, int size)
{
    for (int i = size - 1; i >= 0; --i)
        if (cmp_value(a[i], b[i])) return 1;
    return 0;
}

// ------------------------------------------------------------------ logging

int dwt_util_vfprintf(FILE *stream, const char *format, va_list ap) { return vfprintf(stream, format, ap); }

int dwt_util_vprintf(const char *format, va_list ap) { return vfprintf(stdout, format, ap); }

int dwt_util_fprintf(FILE *stream, const char *format, ...)
{
    va_list ap;
    va_start(ap, format);
    const int r = vfprintf(stream, format, ap);
    va_end(ap);
    return r;
}

int dwt_util_printf(const char *format, ...)
{
    va_list ap;
    va_start(ap, format);
    const int r = vfprintf(stdout, format, ap);
    va_end(ap);
    return r;
}

// One message to stderr behind the level's prefix, written under the
// stream's lock and flushed (src/libdwt.c:7953-7985).
int dwt_util_log(enum dwt_util_loglevel level, const char *format, ...)
{
    static const char *const prefix[] = {"", "DEBUG: ", "INFO: ", "WARNING: ", "ERROR: ", "TEST: "};
    const int l = (int(level) >= 0 && int(level) <= int(LOG_TEST)) ? int(level) : 0;
    flockfile(stderr);
    int r = fputs(prefix[l], stderr) >= 0 ? int(strlen(prefix[l])) : 0;
    va_list ap;
    va_start(ap, format);
    r += vfprintf(stderr, format, ap);
    va_end(ap);
    fflush(stderr);
    funlockfile(stderr);
    return r;
}

// ----------------------------------------------------------- platform queries

const char *dwt_util_version(void) { return "libdwt_gb300 (libdwt 2013-01-29-dev API)"; }

const char *dwt_util_arch(void)
{
#if defined(__aarch64__)
    return "aarch64";
#elif defined(__x86_64__)
    return "x86_64";
#else
    return "unknown";
#endif
}

const char *dwt_util_node(void)
{
    static char buf[256];
    if (!read_proc_line("/proc/sys/kernel/hostname", buf, int(sizeof buf))) return "unknown";
    if (char *nl = strchr(buf, '\n')) *nl = 0;
    return buf;
}

const char *dwt_util_appname(void)
{
    // argv[0] (the first NUL-terminated field of the command line), without
    // its directory
    static char buf[4096];
    if (!read_proc_line("/proc/self/cmdline", buf, int(sizeof buf))) return "unknown";
    const char *slash = strrchr(buf, '/');
    return slash ? slash + 1 : buf;
}

int dwt_util_is_aligned_8(const void *ptr) { return (reinterpret_cast<uintptr_t>(ptr) & 7) == 0 ? 1 : 0; }

int dwt_util_clock_available(int type)
{
    // every timer of the enumeration up to gettimeofday(); the RTC ioctl
    // (it needs /dev/rtc) and the autoselect pseudo-type are not clocks here
    return (type >= DWT_TIME_CLOCK_GETTIME && type <= DWT_TIME_GETTIMEOFDAY) ? 0 : -1;
}

void dwt_util_wait(int ms)
{
    require(ms > 0, "dwt_util_wait", "ms > 0");
    const int type = dwt_util_clock_autoselect();
    const dwt_clock_t freq = dwt_util_get_frequency(type), start = dwt_util_get_clock(type);
    while (1000.0 * double(dwt_util_get_clock(type) - start) / double(freq) < double(ms)) {
    }
}

void dwt_util_abort(void) { abort(); }

// Workers are the accelerator cores of the reference's embedded platform;
// here the GPU is one worker and host threads are not split further.
int dwt_util_get_thread_num(void) { return 0; }
int dwt_util_get_max_workers(void) { return 1; }

void dwt_util_set_num_workers(int num_workers)
{
    require(num_workers > 0, "dwt_util_set_num_workers", "num_workers > 0");
}

// Selects the embedded platform's accelerator firmware; there is none to
// switch on this platform, the call is accepted.
void dwt_util_switch_op(enum dwt_op op) { (void)op; }

// Self-test of the platform: host vectors of 2 .. 4096 floats as the
// reference allocates them, then (when a CUDA device is present) a 64 x 64
// forward and inverse CDF 9/7 round trip through this library on the device,
// which must reproduce the image within 1e-3.  A failure logs and aborts.
void dwt_util_test(void)
{
    for (int i = 2; i <= 4096; i *= 2) {
        dwt_util_log(LOG_TEST, "allocate vector of %i floats...\n", i);
        float *v = dwt_util_allocate_vec_s(i);
        if (!v) {
            dwt_util_log(LOG_ERR, "Failed to allocate vector of %i floats.\n", i);
            abort();
        }
        free(v);
        dwt_util_log(LOG_TEST, "ok\n");
    }
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        dwt_util_log(LOG_TEST, "no CUDA device: GPU round trip skipped\n");
        return;
    }
    dwt_util_log(LOG_TEST, "GPU round trip of a 64x64 image...\n");
    const int S = 64, sx = S * 4;
    float *a = nullptr, *b = nullptr;
    dwt_util_alloc_image(reinterpret_cast<void **>(&a), sx, 4, S, S);
    dwt_util_alloc_image(reinterpret_cast<void **>(&b), sx, 4, S, S);
    dwt_util_test_image_fill_s(a, sx, 4, S, S, 0);
    dwt_util_test_image_fill_s(b, sx, 4, S, S, 0);
    int j = -1;
    dwt_cdf97_2f_s(b, sx, 4, S, S, S, S, &j, 0, 0);
    dwt_cdf97_2i_s(b, sx, 4, S, S, S, S, j, 0, 0);
    const int bad = dwt_util_compare_s(a, b, sx, 4, S, S);
    dwt_util_free_image(reinterpret_cast<void **>(&a));
    dwt_util_free_image(reinterpret_cast<void **>(&b));
    if (bad) {
        dwt_util_log(LOG_ERR, "GPU round trip does not reproduce the image.\n");
        abort();
    }
    dwt_util_log(LOG_TEST, "ok\n");
}

}  // extern "C"
