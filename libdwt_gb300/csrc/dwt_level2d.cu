// Fused row + column lifting level for GB300 (sm_103a): the per-level kernel
// over the warp work units of dwt_units.cuh, the level planner and the
// wavelet constants.
#include "dwt_level2d.cuh"
#include "dwt_units.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace dwt {

// Box copies for the inverse levels (default on; DWT_GPU_TMAP=0 turns them
// off).
bool tensor_copies_enabled()
{
    static const bool on = [] {
        const char *v = getenv("DWT_GPU_TMAP");
        return !(v && v[0] == '0');
    }();
    return on;
}

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

// Test hook: one warp runs the ordered wait of segment 0 of a forward
// 1024 x 1024 level whose counters (order, zeroed by the caller) nothing
// advances; the wait gives up after `limit` polls and raises the error word.
__global__ void order_wait_timeout_kernel(LevelDesc D, uint32_t limit, int *err)
{
    units::order_wait(D, false, 2, 0, threadIdx.x & 31, err, limit);
}

template <int NS, bool INV, bool ORD, bool VST = true>
__global__ void __launch_bounds__(kWarpsPerCta * 32, ORD ? 5 : 0)
level_kernel(const LevelDesc D, const Wavelet W, int *err, const __grid_constant__ LevelMaps M)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *ring = units::warp_ring(smem, warp);
    uint64_t *bars = units::warp_bars(smem, warp, kWarpsPerCta);
    units::init_bars(bars, lane);
    pdl_release();
    pdl_wait();
    const bool fast_launch = units::fast_ok<INV>(D);
    // tensor copies need 128-byte aligned slots
    const bool maps = INV && D.tmap && (smem_addr(smem) & 127) == 0;
    const LevelMaps *mp = maps ? &M : nullptr;
    uint32_t tick = 0;
    const int n = D.n_strips * D.n_segs;
    if constexpr (ORD) {
        // ordered in-place launch: tickets in segment order, one per group of
        // kWarpsPerCta consecutive units (adjacent strips of a segment, as a
        // CTA of the plain launch holds them); a unit waits (after issuing its
        // first loads, before its first store) only for units of earlier
        // tickets, which are running.  Warp 0 takes the next ticket a few
        // stages before the end of its unit.
        __shared__ int s_group[2];
        if (threadIdx.x == 0) s_group[0] = atomicAdd(D.order, 1);
        __syncthreads();
        bool alive = true;
        for (int k = 0;; k ^= 1) {
            const int g = s_group[k];
            if (g >= ceil_div(n, kWarpsPerCta)) break;  // the same for the whole CTA
            const int u = g * kWarpsPerCta + warp;
            int next = warp == 0 ? -1 : 0;
            if (alive && u < n) {
                const int q = u / D.n_strips;
                const int strip = u % D.n_strips, seg = D.seg_base + (D.reverse ? D.n_segs - 1 - q : q);
                alive = units::run_unit<NS, INV, true>(D, W, strip, seg, ring, bars, tick, lane, err, fast_launch,
                                                       mp, next);
                if (alive) units::order_done(D, seg, lane);
            }
            if (warp == 0 && lane == 0) s_group[k ^ 1] = next >= 0 ? next : atomicAdd(D.order, 1);
            __syncthreads();
        }
    } else {
        for (int u = blockIdx.x * kWarpsPerCta + warp; u < n; u += gridDim.x * kWarpsPerCta) {
            const int q = u / D.n_strips;
            const int strip = u % D.n_strips, seg = D.seg_base + (D.reverse ? D.n_segs - 1 - q : q);
            int unused = 0;
            if (!units::run_unit<NS, INV, false, VST>(D, W, strip, seg, ring, bars, tick, lane, err, fast_launch, mp,
                                                      unused))
                break;
        }
    }
}

// The driver's tensor-map encoder (resolved once through the runtime).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        cudaGetLastError();
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// A w x h float region at `base` (pitch in floats) with boxes of box_w x 2;
// false if the geometry does not qualify (16-byte aligned base and pitch).
bool encode_band_map(CUtensorMap *m, const float *base, long long w, long long h, long long pitch, int box_w)
{
    const auto enc = tensor_map_encoder();
    if (!enc || !base || w <= 0 || h <= 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0 || (pitch & 3) != 0)
        return false;
    cuuint64_t dims[2] = {cuuint64_t(w), cuuint64_t(h)};
    cuuint64_t strides[1] = {cuuint64_t(pitch) * 4};
    cuuint32_t box[2] = {cuuint32_t(box_w), 2};
    cuuint32_t es[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of an inverse level: LL from in[0], and the frame the other
// three bands live in -- HL at column dx, LH at row dy, HH at both, as the
// level pipeline lays them out (dx, dy = the band's half sizes) or as a
// zero-padded sparse frame does (the outer midpoints); an ordered in-place
// level reads HL and the staged LH / HH rows from one frame and the other
// LH / HH rows from the caller's (`lower`).  Fills dx, dy.
bool encode_inverse_maps(const LevelDesc &d, LevelMaps &M, int box_w, int &dx, int &dy)
{
    if (d.rows_only || d.h < 2 || d.w < 2) return false;
    const long long ws = (d.w + 1) / 2, hs = (d.h + 1) / 2, hx = d.w / 2, hy = d.h / 2;
    // the H columns' offset: HH sits dx floats right of LH in the same rows
    const long long sx = d.order ? d.alt[1] - d.alt[0] : d.in[3] - d.in[2];
    if (sx < ws || (d.order && d.in[3] - d.in[2] != sx)) return false;
    const long long p = d.in_pitch[1];
    const float *frame = d.in[1] - sx;
    const float *lh = d.order ? d.alt[0] : d.in[2];
    if ((d.order ? d.alt_pitch : d.in_pitch[2]) != p || (!d.order && d.in_pitch[3] != p)) return false;
    const long long off = lh - frame;
    if (off < 0 || off % p != 0 || off / p < hs) return false;
    const long long sy = off / p;
    if (sx + hx > INT32_MAX || sy + hy > INT32_MAX) return false;
    const long long fw = sx + hx, fh = sy + hy;
    bool ok = encode_band_map(&M.ll, d.in[0], ws, hs, d.in_pitch[0], box_w) &&
              encode_band_map(&M.frame, frame, fw, fh, p, box_w);
    if (ok && d.order) {
        const long long q = d.in_pitch[2];
        if (d.in_pitch[3] != q) return false;
        const float *lower = d.in[2] - sy * q;
        ok = encode_band_map(&M.lower, lower, fw, fh, q, box_w);
    }
    dx = int(sx);
    dy = int(sy);
    return ok;
}

template <int NS, bool INV, bool ORD, bool VST = true>
cudaError_t launch_o(const LevelDesc &d, const Wavelet &W, cudaStream_t stream, int *err)
{
    // once per instantiation, safe from several host threads
    static const cudaError_t configured =
        cudaFuncSetAttribute(level_kernel<NS, INV, ORD, VST>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (configured != cudaSuccess) return configured;
    const int units = d.n_strips * d.n_segs;
    const int grid = ceil_div(units, kWarpsPerCta);
    LevelMaps M;
    memset(&M, 0, sizeof(M));
    LevelDesc dd = d;
    int dx = 0, dy = 0;
    dd.tmap = (INV && tensor_copies_enabled() && encode_inverse_maps(d, M, kBandRowF, dx, dy)) ? 1 : 0;
    dd.map_dx = dx;
    dd.map_dy = dy;
    return launch_pdl(level_kernel<NS, INV, ORD, VST>, dim3(grid), dim3(kWarpsPerCta * 32), kSmemBytes, stream, dd,
                      W, err, M);
}

// Whether the forward level's band rows take 8-byte stores (the device-side
// check of units::fast_ok, on the host).
bool forward_stores_aligned(const LevelDesc &d)
{
    for (int k = 0; k < 4; ++k)
        if ((reinterpret_cast<uintptr_t>(d.out[k]) & 7) != 0 || (d.out_pitch[k] & 1) != 0) return false;
    return true;
}

template <int NS, bool INV>
cudaError_t launch_t(const LevelDesc &d, const Wavelet &W, cudaStream_t stream, int *err)
{
    if (d.order) return launch_o<NS, INV, true>(d, W, stream, err);
    // forward levels whose bands cannot take 8-byte stores: a kernel whose
    // interior strips keep the fast loads and store one by one
    if constexpr (!INV)
        if (!d.rows_only && d.h > 1 && !forward_stores_aligned(d))
            return launch_o<NS, INV, false, false>(d, W, stream, err);
    return launch_o<NS, INV, false>(d, W, stream, err);
}

}  // namespace

namespace {

// Segment length of a 2D level, measured on 16384^2 (level kernel times and
// the whole forward + inverse step, CUDA events): the forward is fastest with
// about 176 segments per level (none shorter than 4 pairs from 1024 row
// pairs up, 2 below); the inverse with about 384 on large levels, none
// shorter than 16 pairs (88 segments: inverse level 0 in 0.361 ms, 176:
// 0.350, 256: 0.342, 384: 0.337; the step 1.052 / 1.022 / 1.009 ms at 88 /
// 256 / 384-and-16) and 128 (at least 2 pairs) from 1024 row pairs down.
constexpr int kSegsForward = 176;
constexpr int kSegsInverse = 384;
constexpr int kSegsInverseSmall = 128;
constexpr int kSmallPairs = 1024;
// Below kSmallPairs the levels are latency-bound: segments as short as 2
// pairs (more, shorter units) measured 5 us faster per 16384^2 forward +
// inverse than a 4-pair minimum.
constexpr int kSegMinSmall = 2;
// Shortest forward / inverse segment above kSmallPairs row pairs.
constexpr int kSegMinForward = 4;
constexpr int kSegMinInverse = 16;

int env_int(const char *name, int dflt)
{
    const char *v = getenv(name);
    return (v && *v) ? atoi(v) : dflt;
}

}  // namespace

void plan_level(LevelDesc &d, int seg_pairs_hint, bool inverse)
{
    const bool one_row = (d.h == 1) || d.rows_only;
    const int npairs = one_row ? d.h : (d.h + 1) / 2;
    d.n_strips = ceil_div(d.w, kStripOut);
    int seg = seg_pairs_hint;
    if (seg <= 0) {
        if (one_row) {
            // rows are independent: about 1.5 units per resident warp
            const long long target_units = 152LL * 20 * 3 / 2;
            seg = int(std::max(1LL, ((long long)npairs * d.n_strips + target_units - 1) / target_units));
            seg = std::min(seg, 256);
        } else {
            static const int segs_f = std::max(1, env_int("DWT_GPU_SEGS_FWD", kSegsForward));
            static const int segs_i = std::max(1, env_int("DWT_GPU_SEGS_INV", kSegsInverse));
            static const int segs_is = std::max(1, env_int("DWT_GPU_SEGS_INV_SMALL", kSegsInverseSmall));
            static const int fwd_min = std::max(1, env_int("DWT_GPU_SEG_MIN_FWD", kSegMinForward));
            static const int inv_min = std::max(1, env_int("DWT_GPU_SEG_MIN_INV", kSegMinInverse));
            if (!inverse)
                seg = std::max(ceil_div(npairs, segs_f), npairs >= kSmallPairs ? fwd_min : kSegMinSmall);
            else if (npairs > kSmallPairs)
                seg = std::max(ceil_div(npairs, segs_i), inv_min);
            else
                seg = std::max(ceil_div(npairs, segs_is), kSegMinSmall);
        }
    }
    seg = std::min(seg, std::max(npairs, 1));
    d.seg_pairs = seg;
    d.n_segs = ceil_div(npairs, seg);
}

int order_wait_timeout_words()
{
    LevelDesc d{};
    d.w = d.h = 1024;
    plan_level(d, 0, false);
    return d.n_segs + 1;
}

cudaError_t launch_order_wait_timeout(uint32_t limit, int *order, int *err, cudaStream_t stream)
{
    LevelDesc d{};
    d.w = d.h = 1024;
    plan_level(d, 0, false);
    d.order = order;
    d.stage_seg = d.n_segs;
    d.order_dy = (d.h + 1) / 2;
    d.reverse = 1;
    order_wait_timeout_kernel<<<1, 32, 0, stream>>>(d, limit, err);
    return cudaGetLastError();
}

cudaError_t launch_level(const LevelDesc &d, int wavelet, bool inverse, cudaStream_t stream, int *err)
{
    const Wavelet W = make_wavelet(wavelet, inverse);
    if (wavelet == CDF97)
        return inverse ? launch_t<4, true>(d, W, stream, err) : launch_t<4, false>(d, W, stream, err);
    return inverse ? launch_t<2, true>(d, W, stream, err) : launch_t<2, false>(d, W, stream, err);
}

}  // namespace dwt
