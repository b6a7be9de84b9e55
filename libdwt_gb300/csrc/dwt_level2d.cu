// Fused row + column lifting level for GB300 (sm_103a): the per-level kernel
// over the warp work units of dwt_units.cuh, the level planner and the
// wavelet constants.
#include "dwt_level2d.cuh"
#include "dwt_units.cuh"

#include <algorithm>
#include <cstdlib>

namespace dwt {

bool pdl_enabled()
{
    static const bool on = [] {
        const char *v = getenv("DWT_GPU_PDL");
        return !(v && v[0] == '0');
    }();
    return on;
}

Wavelet make_wavelet(int id, bool inverse)
{
    const Wavelet w = make_wavelet_dev(id, inverse);
    // 1/zeta must be the float division 1.0f / s1 (src/libdwt.c:1637-1640),
    // one ulp away from the separately rounded constant s2
    volatile float one = 1.0f;
    Wavelet r = w;
    if (id == CDF97) r.zeta_o = one / w.zeta_e;
    return r;
}

namespace {

template <int NS, bool INV>
__global__ void __launch_bounds__(kWarpsPerCta * 32)
level_kernel(const LevelDesc D, const Wavelet W, int *err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *ring = units::warp_ring(smem, warp);
    uint64_t *bars = units::warp_bars(smem, warp, kWarpsPerCta);
    units::init_bars(bars, lane);
    pdl_release();
    pdl_wait();
    const bool fast_launch = units::fast_ok<INV>(D);
    uint32_t tick = 0;
    const int n = D.n_strips * D.n_segs;
    for (int u = blockIdx.x * kWarpsPerCta + warp; u < n; u += gridDim.x * kWarpsPerCta) {
        const int strip = u % D.n_strips, seg = D.seg_base + u / D.n_strips;
        if (!units::run_unit<NS, INV>(D, W, strip, seg, ring, bars, tick, lane, err, fast_launch)) break;
    }
}

template <int NS, bool INV>
cudaError_t launch_t(const LevelDesc &d, const Wavelet &W, cudaStream_t stream, int *err)
{
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(level_kernel<NS, INV>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    const int units = d.n_strips * d.n_segs;
    const int grid = ceil_div(units, kWarpsPerCta);
    return launch_pdl(level_kernel<NS, INV>, dim3(grid), dim3(kWarpsPerCta * 32), kSmemBytes, stream, d, W, err);
}

}  // namespace

void plan_level(LevelDesc &d, int seg_pairs_hint)
{
    const bool one_row = (d.h == 1) || d.rows_only;
    const int npairs = one_row ? d.h : (d.h + 1) / 2;
    d.n_strips = ceil_div(d.w, kStripOut);
    int seg = seg_pairs_hint;
    if (seg <= 0) {
        // About 1.5 units per resident warp (152 SMs x 24 warps): long
        // segments on large levels keep the 2*LAT warm-up pairs a few percent
        // of the work; small levels get short segments for parallelism.
        const long long target_units = 152LL * 24 * 3 / 2;
        seg = int(((long long)npairs * d.n_strips + target_units - 1) / target_units);
        seg = std::max(seg, one_row ? 1 : 4);
        seg = std::min(seg, 256);
    }
    seg = std::min(seg, std::max(npairs, 1));
    d.seg_pairs = seg;
    d.n_segs = ceil_div(npairs, seg);
}

cudaError_t launch_level(const LevelDesc &d, int wavelet, bool inverse, cudaStream_t stream, int *err)
{
    const Wavelet W = make_wavelet(wavelet, inverse);
    if (wavelet == CDF97)
        return inverse ? launch_t<4, true>(d, W, stream, err) : launch_t<4, false>(d, W, stream, err);
    return inverse ? launch_t<2, true>(d, W, stream, err) : launch_t<2, false>(d, W, stream, err);
}

}  // namespace dwt
