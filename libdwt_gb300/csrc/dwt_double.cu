// Double-precision transforms (libdwt's _d API) on the GPU.
//
// libdwt's double variants lift as x - c*(l + r) with the positive
// constants (src/libdwt.c:1489-1520, 5696-5727); negation is exact, so this
// equals x + (-c)*(l + r) bit for bit, which is the form used here with the
// constants of WaveletD.  Every operation is an explicitly rounded double
// add or multiply (no contraction).  The path is the general per-line one:
// one thread per line, the line gathered into an interleaved scratch so a
// warp's accesses coalesce, in place on a compact frame.  Double arithmetic
// runs at a small fraction of the float rate on this GPU; these calls are
// for API completeness and FP64 checking, not throughput.
#include "dwt_double.cuh"

namespace dwt {

WaveletD make_wavelet_d(int id, bool inverse)
{
    WaveletD w{};
    if (id == CDF97) {
        // src/libdwt.c:541-547, in double
        const double p1 = 1.58613434342059, u1 = -0.0529801185729;
        const double p2 = -0.8829110755309, u2 = 0.4435068520439;
        const double s1 = 1.1496043988602, s2 = 1 / 1.1496043988602;
        w.nsteps = 4;
        w.zeta_e = s1;
        w.zeta_o = s2;
        w.n1_fwd = s1;
        w.n1_inv = s2;
        if (!inverse) {
            w.c[0] = -p1; w.c[1] = u1; w.c[2] = -p2; w.c[3] = u2;
        } else {
            w.c[0] = -u2; w.c[1] = p2; w.c[2] = -u1; w.c[3] = p1;
        }
    } else {
        // src/libdwt.c:566-569, in double
        const double p1 = 0.5, u1 = 0.25;
        const double s1 = 1.41421356237309504880, s2 = 0.70710678118654752440;
        w.nsteps = 2;
        w.zeta_e = s1;
        w.zeta_o = s2;
        w.n1_fwd = s1;
        w.n1_inv = s2;
        if (!inverse) {
            w.c[0] = -p1; w.c[1] = u1;
        } else {
            w.c[0] = -u1; w.c[1] = p1;
        }
    }
    return w;
}

namespace {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dlift(double x, double c, double l, double r)
{
    return __dadd_rn(x, __dmul_rn(c, __dadd_rn(l, r)));
}

__device__ __forceinline__ double load_any_d(const unsigned char *p)
{
    if ((reinterpret_cast<uintptr_t>(p) & 7) == 0) return *reinterpret_cast<const double *>(p);
    unsigned long long u = 0;
    for (int b = 7; b >= 0; --b) u = (u << 8) | p[b];
    return __longlong_as_double(static_cast<long long>(u));
}

__device__ __forceinline__ void store_any_d(unsigned char *p, double v)
{
    if ((reinterpret_cast<uintptr_t>(p) & 7) == 0) {
        *reinterpret_cast<double *>(p) = v;
        return;
    }
    unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v));
    for (int b = 0; b < 8; ++b, u >>= 8) p[b] = static_cast<unsigned char>(u & 0xff);
}

__global__ void repack_d_kernel(const unsigned char *src, long long sx, long long sy, int ox, int oy, double *dst,
                                long long dpitch)
{
    const long long n = (long long)ox * oy;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int y = int(k / ox), x = int(k % ox);
        dst[y * dpitch + x] = load_any_d(src + y * sx + x * sy);
    }
}

__global__ void unpack_d_kernel(const double *src, long long spitch, unsigned char *dst, long long sx, long long sy,
                                int ox, int oy)
{
    const long long n = (long long)ox * oy;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int y = int(k / ox), x = int(k % ox);
        store_any_d(dst + y * sx + x * sy, src[y * spitch + x]);
    }
}

// One lifting step on the samples of `parity`, whole-sample symmetric
// extension at both ends.
__device__ __forceinline__ void step_d(double *x, long long ts, int N, int parity, double c)
{
    for (int i = parity; i < N; i += 2) {
        const double l = (i > 0) ? x[(i - 1) * ts] : x[(i + 1) * ts];
        const double r = (i + 1 < N) ? x[(i + 1) * ts] : x[(i - 1) * ts];
        x[i * ts] = dlift(x[i * ts], c, l, r);
    }
}

__device__ __forceinline__ void scale_d(double *x, long long ts, int N, double even, double odd)
{
    for (int i = 0; i < N; i += 2) x[i * ts] = dmul(x[i * ts], even);
    for (int i = 1; i < N; i += 2) x[i * ts] = dmul(x[i * ts], odd);
}

// Line k at base + k*ls, samples es apart: N samples in, L to
// [0, ceil(N/2)), H to [hoff, hoff + floor(N/2)).  One thread per line.
__global__ void lines_forward_d(double *base, long long ls, long long es, int nlines, int N, int hoff, double *tmp,
                                const WaveletD W)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines || N <= 0) return;
    double *line = base + k * ls;
    if (N == 1) {
        line[0] = dmul(line[0], W.n1_fwd);
        return;
    }
    double *x = tmp + k;
    const long long ts = nlines;
    for (int i = 0; i < N; ++i) x[i * ts] = line[i * es];
    for (int s = 0; s < W.nsteps; ++s) step_d(x, ts, N, (s & 1) ? 0 : 1, W.c[s]);
    scale_d(x, ts, N, W.zeta_e, W.zeta_o);
    for (int i = 0; 2 * i < N; ++i) line[i * es] = x[(2 * i) * ts];
    for (int i = 0; 2 * i + 1 < N; ++i) line[(hoff + i) * es] = x[(2 * i + 1) * ts];
}

__global__ void lines_inverse_d(double *base, long long ls, long long es, int nlines, int N, int hoff, double *tmp,
                                const WaveletD W)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines || N <= 0) return;
    double *line = base + k * ls;
    if (N == 1) {
        line[0] = dmul(line[0], W.n1_inv);
        return;
    }
    double *x = tmp + k;
    const long long ts = nlines;
    for (int i = 0; 2 * i < N; ++i) x[(2 * i) * ts] = line[i * es];
    for (int i = 0; 2 * i + 1 < N; ++i) x[(2 * i + 1) * ts] = line[(hoff + i) * es];
    scale_d(x, ts, N, W.zeta_o, W.zeta_e);
    for (int s = 0; s < W.nsteps; ++s) step_d(x, ts, N, (s & 1) ? 1 : 0, W.c[s]);
    for (int i = 0; i < N; ++i) line[i * es] = x[i * ts];
}

// Zero padding (dwt_zero_padding_f_stride_d / _i_stride_d semantics).
__global__ void zero_forward_d(double *base, long long ls, long long es, int nlines, int N, int nL, int nH, int hoff)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines || (nL == 0 && nH == 0)) return;
    double *line = base + k * ls;
    for (int i = (N + 1) / 2; i < nL; ++i) line[i * es] = 0.0;
    for (int i = N / 2; i < nH; ++i) line[(hoff + i) * es] = 0.0;
}

__global__ void zero_inverse_d(double *base, long long ls, long long es, int nlines, int N, int n_dst)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines) return;
    double *line = base + k * ls;
    for (int i = N; i < n_dst; ++i) line[i * es] = 0.0;
}

int grid_for(long long n, int block)
{
    long long g = (n + block - 1) / block;
    if (g > 152LL * 32) g = 152LL * 32;
    if (g < 1) g = 1;
    return int(g);
}

}  // namespace

cudaError_t launch_repack_d(const void *src, long long sx, long long sy, int ox, int oy, double *dst,
                            long long dpitch, cudaStream_t s)
{
    if ((long long)ox * oy == 0) return cudaSuccess;
    repack_d_kernel<<<grid_for((long long)ox * oy, 256), 256, 0, s>>>(static_cast<const unsigned char *>(src), sx,
                                                                       sy, ox, oy, dst, dpitch);
    return cudaGetLastError();
}

cudaError_t launch_unpack_d(const double *src, long long spitch, void *dst, long long sx, long long sy, int ox,
                            int oy, cudaStream_t s)
{
    if ((long long)ox * oy == 0) return cudaSuccess;
    unpack_d_kernel<<<grid_for((long long)ox * oy, 256), 256, 0, s>>>(src, spitch, static_cast<unsigned char *>(dst),
                                                                       sx, sy, ox, oy);
    return cudaGetLastError();
}

cudaError_t level_forward_d(double *f, long long pitch, int osx, int osy, int odx, int ody, int isx, int isy,
                            int zero_padding, int wavelet, double *tmp, cudaStream_t s)
{
    const WaveletD W = make_wavelet_d(wavelet, false);
    lines_forward_d<<<ceil_div(osy, 128), 128, 0, s>>>(f, pitch, 1, osy, isx, odx, tmp, W);
    lines_forward_d<<<ceil_div(osx, 128), 128, 0, s>>>(f, 1, pitch, osx, isy, ody, tmp, W);
    if (zero_padding) {
        zero_forward_d<<<ceil_div(osy, 128), 128, 0, s>>>(f, pitch, 1, osy, isx, odx, osx - odx, odx);
        zero_forward_d<<<ceil_div(osx, 128), 128, 0, s>>>(f, 1, pitch, osx, isy, ody, osy - ody, ody);
    }
    return cudaGetLastError();
}

cudaError_t level_inverse_d(double *f, long long pitch, int osx, int osy, int odx, int ody, int idx, int idy,
                            int zero_padding, int wavelet, double *tmp, cudaStream_t s)
{
    const WaveletD W = make_wavelet_d(wavelet, true);
    lines_inverse_d<<<ceil_div(ody, 128), 128, 0, s>>>(f, pitch, 1, ody, idx, osx, tmp, W);
    lines_inverse_d<<<ceil_div(odx, 128), 128, 0, s>>>(f, 1, pitch, odx, idy, osy, tmp, W);
    if (zero_padding) {
        zero_inverse_d<<<ceil_div(ody, 128), 128, 0, s>>>(f, pitch, 1, ody, idx, odx);
        zero_inverse_d<<<ceil_div(odx, 128), 128, 0, s>>>(f, 1, pitch, odx, idy, ody);
    }
    return cudaGetLastError();
}

cudaError_t line_d(bool inverse, double *line, int N, int wavelet, double *tmp, cudaStream_t s)
{
    if (N <= 0) return cudaSuccess;
    const int hoff = (N + 1) / 2;
    if (inverse)
        lines_inverse_d<<<1, 32, 0, s>>>(line, 0, 1, 1, N, hoff, tmp, make_wavelet_d(wavelet, true));
    else
        lines_forward_d<<<1, 32, 0, s>>>(line, 0, 1, 1, N, hoff, tmp, make_wavelet_d(wavelet, false));
    return cudaGetLastError();
}

}  // namespace dwt
