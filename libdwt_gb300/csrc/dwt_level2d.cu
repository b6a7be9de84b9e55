// Fused row + column lifting level for GB300 (sm_103a).
//
// Each warp owns one work unit: a strip of 128 interleaved columns (4 per
// lane) by a segment of row pairs.  Its rows (forward) or band rows (inverse)
// are streamed into a private shared-memory ring by the TMA bulk-copy engine
// (cp.async.bulk + mbarrier complete_tx), one stage per row pair, kStages
// stages deep.  For every row pair the warp
//   1. reads its 4 columns of each row from shared memory,
//   2. runs the horizontal lifting steps in registers, exchanging the one
//      neighbour value per step with warp shuffles,
//   3. advances the vertical lifting as a per-column register recurrence that
//      emits one finished output row pair per input row pair, and
//   4. stores the finished pair with coalesced vector stores.
// Symmetric extension at the image borders is applied by reading mirrored
// columns (lane offsets) and mirrored rows (the producer's row choice), which
// reproduces the reference's boundary formulas bit for bit
// (accel_lift_op4s_prolog_s / _epilog_s / _short_s, src/libdwt.c:5036-5377).
//
// Arithmetic follows the reference's float path operation by operation
// (x + c*(l + r) with three roundings, scaling afterwards / beforehand), so
// every output equals the reference's to the last bit.
#include "dwt_level2d.cuh"

#include <algorithm>

namespace dwt {

Wavelet make_wavelet(int id, bool inverse)
{
    Wavelet w{};
    if (id == CDF97) {
        // src/libdwt.c:541-547
        const float p1 = 1.58613434342059f, u1 = -0.0529801185729f;
        const float p2 = -0.8829110755309f, u2 = 0.4435068520439f;
        const float s1 = 1.1496043988602f;
        const float s2 = (float)(1 / 1.1496043988602);
        volatile float one = 1.0f;  // 1/zeta as a float division, as the reference computes it
        w.nsteps = 4;
        w.zeta_e = s1;
        w.zeta_o = one / s1;
        w.n1_fwd = s1;
        w.n1_inv = s2;
        if (!inverse) {
            w.c[0] = -p1; w.c[1] = u1; w.c[2] = -p2; w.c[3] = u2;
        } else {
            w.c[0] = -u2; w.c[1] = p2; w.c[2] = -u1; w.c[3] = p1;
        }
    } else {
        // src/libdwt.c:566-569
        const float p1 = 0.5f, u1 = 0.25f;
        const float s1 = (float)1.41421356237309504880, s2 = (float)0.70710678118654752440;
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
        w.c[2] = w.c[3] = 0.0f;
    }
    return w;
}

namespace {

constexpr unsigned kFull = 0xffffffffu;

// Forward horizontal lifting of the lane's 4 interleaved samples
// (even, odd, even, odd), neighbours from lanes l-1 / l+1.
template <int NS>
__device__ __forceinline__ void h_forward(float v[4], const Wavelet &W)
{
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
        const float nx = __shfl_down_sync(kFull, v[0], 1);
        v[1] = lift(v[1], W.c[s], v[0], v[2]);
        v[3] = lift(v[3], W.c[s], v[2], nx);
        const float pv = __shfl_up_sync(kFull, v[3], 1);
        v[0] = lift(v[0], W.c[s + 1], pv, v[1]);
        v[2] = lift(v[2], W.c[s + 1], v[1], v[3]);
    }
    v[0] = fmul(v[0], W.zeta_e);
    v[1] = fmul(v[1], W.zeta_o);
    v[2] = fmul(v[2], W.zeta_e);
    v[3] = fmul(v[3], W.zeta_o);
}

template <int NS>
__device__ __forceinline__ void h_inverse(float v[4], const Wavelet &W)
{
    v[0] = fmul(v[0], W.zeta_o);
    v[1] = fmul(v[1], W.zeta_e);
    v[2] = fmul(v[2], W.zeta_o);
    v[3] = fmul(v[3], W.zeta_e);
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
        const float pv = __shfl_up_sync(kFull, v[3], 1);
        v[0] = lift(v[0], W.c[s], pv, v[1]);
        v[2] = lift(v[2], W.c[s], v[1], v[3]);
        const float nx = __shfl_down_sync(kFull, v[0], 1);
        v[1] = lift(v[1], W.c[s + 1], v[0], v[2]);
        v[3] = lift(v[3], W.c[s + 1], v[2], nx);
    }
}

__device__ __forceinline__ void store2(float *p, float a, float b, bool va, bool vb)
{
    if (va && vb && ((reinterpret_cast<uintptr_t>(p) & 7) == 0)) {
        *reinterpret_cast<float2 *>(p) = make_float2(a, b);
    } else {
        if (va) p[0] = a;
        if (vb) p[1] = b;
    }
}

__device__ __forceinline__ void store4(float *p, const float v[4], const bool ok[4])
{
    if (ok[0] && ok[1] && ok[2] && ok[3] && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (ok[i]) p[i] = v[i];
    }
}

__device__ __forceinline__ void raise_error(int *err, int code)
{
    if (err) atomicCAS(err, 0, code);
}

// A 16-byte aligned bulk copy covering floats [src, src + n): returns the
// aligned start, the byte count and the float shift of src within it.
struct Span {
    const float *start;
    uint32_t bytes;
    int shift;
};

__device__ __forceinline__ Span aligned_span(const float *src, int n)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(src);
    const uintptr_t a0 = a & ~uintptr_t(15);
    const uintptr_t e = (a + uintptr_t(n) * 4 + 15) & ~uintptr_t(15);
    return Span{reinterpret_cast<const float *>(a0), uint32_t(e - a0), int((a - a0) >> 2)};
}

// ------------------------------------------------------------------ forward

template <int NS>
__device__ bool forward_unit(const LevelDesc &D, const Wavelet &W, int strip, int seg,
                             float *ring, uint64_t *bars, uint32_t &tick, int lane, int *err)
{
    constexpr int LAT = NS / 2;
    const int w = D.w, h = D.h;
    const bool one_row = (h == 1) || D.rows_only;
    const int b = strip * kStripOut - 4;  // interleaved column held by lane 0, value 0
    const int npairs = one_row ? h : (h + 1) >> 1;
    const int k0 = seg * D.seg_pairs;
    const int k1 = min(k0 + D.seg_pairs, npairs);
    const int m0 = one_row ? k0 : k0 - LAT;
    const int total = one_row ? (k1 - k0) : (k1 - k0 + 2 * LAT);

    // staged column window [lo, hi) of every row
    const int w4 = (w + 3) & ~3;
    const int lo = max(b, 0), hi = min(b + kStripIn, w4);
    const uint32_t bytes = uint32_t(hi - lo) * 4u;
    const int dst_off = lo - b;

    // this lane's 4 shared-memory offsets (mirrored at the borders)
    int off[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int c = b + 4 * lane + i;
        int o = mirror(c, w) - b;
        o = min(max(o, lo - b), hi - b - 1);
        off[i] = o;
    }
    const bool fast = ((off[0] & 3) == 0) && off[1] == off[0] + 1 && off[2] == off[0] + 2 &&
                      off[3] == off[0] + 3;

    const float *src = D.in[0];
    const long long pitch = D.in_pitch[0];

    auto issue = [&](int t) {
        const int m = m0 + t;
        const uint32_t st = (tick + t) % kStages;
        float *slot = ring + st * kStageFloats;
        int ra, rb;
        if (one_row) {
            ra = m; rb = -1;
        } else {
            ra = mirror(2 * m, h);
            rb = mirror(2 * m + 1, h);
        }
        mbar_arrive_expect_tx(&bars[st], rb >= 0 ? 2 * bytes : bytes);
        bulk_g2s(slot + dst_off, src + ra * pitch + lo, bytes, &bars[st]);
        if (rb >= 0) bulk_g2s(slot + kSlotF + dst_off, src + rb * pitch + lo, bytes, &bars[st]);
    };

    if (lane == 0) {
        fence_proxy_async_smem();
        for (int t = 0; t < min(total, kStages); ++t) issue(t);
    }
    __syncwarp();

    // output geometry of this lane
    const int c0 = b + 4 * lane;
    const bool lane_ok = lane >= 1 && lane <= kLanes - 2;
    const bool vL0 = lane_ok && c0 < w, vH0 = lane_ok && c0 + 1 < w;
    const bool vL1 = lane_ok && c0 + 2 < w, vH1 = lane_ok && c0 + 3 < w;
    const int q = (b >> 1) + 2 * lane;  // band column of this lane's first value

    float e[4] = {0, 0, 0, 0}, o[4] = {0, 0, 0, 0}, o1[4] = {0, 0, 0, 0};
    float e1[4] = {0, 0, 0, 0}, o2[4] = {0, 0, 0, 0};

    for (int t = 0; t < total; ++t) {
        const uint32_t st = (tick + t) % kStages;
        const uint32_t par = ((tick + t) / kStages) & 1u;
        if (!mbar_wait_bounded(&bars[st], par)) {
            if (lane == 0) raise_error(err, kErrWaitTimeout);
            return false;
        }
        const float *slot = ring + st * kStageFloats;
        float A[4], B[4];
        if (fast) {
            const float4 a4 = *reinterpret_cast<const float4 *>(slot + off[0]);
            A[0] = a4.x; A[1] = a4.y; A[2] = a4.z; A[3] = a4.w;
            if (!one_row) {
                const float4 b4 = *reinterpret_cast<const float4 *>(slot + kSlotF + off[0]);
                B[0] = b4.x; B[1] = b4.y; B[2] = b4.z; B[3] = b4.w;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                A[i] = slot[off[i]];
                B[i] = one_row ? 0.0f : slot[kSlotF + off[i]];
            }
        }
        __syncwarp();
        if (lane == 0 && t + kStages < total) {
            fence_proxy_async_smem();
            issue(t + kStages);
        }

        // rows: horizontal lifting (a single-sample row is only scaled)
        if (w == 1) {
            A[0] = fmul(A[0], W.n1_fwd);
            B[0] = fmul(B[0], W.n1_fwd);
        } else {
            h_forward<NS>(A, W);
            if (!one_row) h_forward<NS>(B, W);
        }

        if (one_row) {
            const int p = m0 + t;
            if (!D.rows_only) {  // a single-row image: the column step only scales
#pragma unroll
                for (int i = 0; i < 4; ++i) A[i] = fmul(A[i], W.n1_fwd);
            }
            store2(D.out[0] + p * D.out_pitch[0] + q, A[0], A[2], vL0, vL1);
            store2(D.out[1] + p * D.out_pitch[1] + q, A[1], A[3], vH0, vH1);
            continue;
        }

        // columns: one step of the vertical recurrence per column
        float Lv[4], Hv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (NS == 4) {
                const float o1n = lift(o[i], W.c[0], e[i], A[i]);    // o'(m-1)
                const float e1n = lift(e[i], W.c[1], o1[i], o1n);    // e'(m-1)
                const float o2n = lift(o1[i], W.c[2], e1[i], e1n);   // o''(m-2)
                const float e2n = lift(e1[i], W.c[3], o2[i], o2n);   // e''(m-2)
                Lv[i] = fmul(e2n, W.zeta_e);
                Hv[i] = fmul(o2n, W.zeta_o);
                o1[i] = o1n; e1[i] = e1n; o2[i] = o2n;
            } else {
                const float o1n = lift(o[i], W.c[0], e[i], A[i]);    // o'(m-1)
                const float e1n = lift(e[i], W.c[1], o1[i], o1n);    // e'(m-1)
                Lv[i] = fmul(e1n, W.zeta_e);
                Hv[i] = fmul(o1n, W.zeta_o);
                o1[i] = o1n;
            }
            e[i] = A[i];
            o[i] = B[i];
        }
        const int p = m0 + t - LAT;
        if (p >= k0) {
            store2(D.out[0] + p * D.out_pitch[0] + q, Lv[0], Lv[2], vL0, vL1);
            store2(D.out[1] + p * D.out_pitch[1] + q, Lv[1], Lv[3], vH0, vH1);
            if (2 * p + 1 < h) {
                store2(D.out[2] + p * D.out_pitch[2] + q, Hv[0], Hv[2], vL0, vL1);
                store2(D.out[3] + p * D.out_pitch[3] + q, Hv[1], Hv[3], vH0, vH1);
            }
        }
    }
    tick += total;
    return true;
}

// ------------------------------------------------------------------ inverse

template <int NS>
__device__ bool inverse_unit(const LevelDesc &D, const Wavelet &W, int strip, int seg,
                             float *ring, uint64_t *bars, uint32_t &tick, int lane, int *err)
{
    constexpr int LAT = NS / 2;
    const int w = D.w, h = D.h;
    const bool one_row = (h == 1) || D.rows_only;
    const int b = strip * kStripOut - 4;
    const int bq = b >> 1;                 // band column of lane 0's first value
    const int Lw = (w + 1) >> 1, Hw = w >> 1;
    const int npairs = one_row ? h : (h + 1) >> 1;
    const int k0 = seg * D.seg_pairs;
    const int k1 = min(k0 + D.seg_pairs, npairs);
    const int m0 = one_row ? k0 : k0 - LAT;
    const int total = one_row ? (k1 - k0) : (k1 - k0 + 2 * LAT);

    // staged band column windows
    const int loL = max(bq, 0), hiL = min(bq + 64, Lw);
    const int loH = max(bq, 0), hiH = min(bq + 64, Hw);
    const int nL = hiL - loL, nH = hiH - loH;  // nL > 0 always, nH may be <= 0

    // float shift of each band row start inside its 16-byte aligned copy;
    // the same for every row because pitches are multiples of 4 floats
    int shift[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int lo_k = (k & 1) ? loH : loL;
        shift[k] = int((reinterpret_cast<uintptr_t>(D.in[k] + lo_k) & 15) >> 2);
    }

    // this lane's offsets: even samples come from the L band, odd from H
    int offA[4], offB[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int c = b + 4 * lane + i;
        int bi, k;
        if (w == 1) {
            bi = 0; k = 0;
        } else {
            const int mc = mirror(c, w);
            bi = mc >> 1;
            k = mc & 1;
        }
        const int lo_k = k ? loH : loL;
        int oa = bi - lo_k + shift[k];
        int ob = bi - lo_k + shift[k + 2];
        oa = min(max(oa, 0), kSlotI - 1);
        ob = min(max(ob, 0), kSlotI - 1);
        offA[i] = k * kSlotI + oa;        // slot 0 = LL row, slot 1 = HL row
        offB[i] = (2 + k) * kSlotI + ob;  // slot 2 = LH row, slot 3 = HH row
    }

    auto issue = [&](int t) {
        const int m = m0 + t;
        const uint32_t st = (tick + t) % kStages;
        float *slot = ring + st * kStageFloats;
        int qa, qb;
        if (one_row) {
            qa = m; qb = -1;
        } else {
            qa = mirror(2 * m, h) >> 1;
            qb = mirror(2 * m + 1, h) >> 1;
        }
        Span s[4];
        uint32_t total_bytes = 0;
        s[0] = aligned_span(D.in[0] + qa * D.in_pitch[0] + loL, nL);
        total_bytes += s[0].bytes;
        if (nH > 0) {
            s[1] = aligned_span(D.in[1] + qa * D.in_pitch[1] + loH, nH);
            total_bytes += s[1].bytes;
        }
        if (qb >= 0) {
            s[2] = aligned_span(D.in[2] + qb * D.in_pitch[2] + loL, nL);
            total_bytes += s[2].bytes;
            if (nH > 0) {
                s[3] = aligned_span(D.in[3] + qb * D.in_pitch[3] + loH, nH);
                total_bytes += s[3].bytes;
            }
        }
        mbar_arrive_expect_tx(&bars[st], total_bytes);
        bulk_g2s(slot, s[0].start, s[0].bytes, &bars[st]);
        if (nH > 0) bulk_g2s(slot + kSlotI, s[1].start, s[1].bytes, &bars[st]);
        if (qb >= 0) {
            bulk_g2s(slot + 2 * kSlotI, s[2].start, s[2].bytes, &bars[st]);
            if (nH > 0) bulk_g2s(slot + 3 * kSlotI, s[3].start, s[3].bytes, &bars[st]);
        }
    };

    if (lane == 0) {
        fence_proxy_async_smem();
        for (int t = 0; t < min(total, kStages); ++t) issue(t);
    }
    __syncwarp();

    const int c0 = b + 4 * lane;
    const bool lane_ok = lane >= 1 && lane <= kLanes - 2;
    bool ok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) ok[i] = lane_ok && (c0 + i < w);

    float o[4] = {0, 0, 0, 0}, e1[4] = {0, 0, 0, 0}, o1[4] = {0, 0, 0, 0}, e2[4] = {0, 0, 0, 0};

    for (int t = 0; t < total; ++t) {
        const uint32_t st = (tick + t) % kStages;
        const uint32_t par = ((tick + t) / kStages) & 1u;
        if (!mbar_wait_bounded(&bars[st], par)) {
            if (lane == 0) raise_error(err, kErrWaitTimeout);
            return false;
        }
        const float *slot = ring + st * kStageFloats;
        float A[4], B[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            A[i] = slot[offA[i]];
            B[i] = one_row ? 0.0f : slot[offB[i]];
        }
        __syncwarp();
        if (lane == 0 && t + kStages < total) {
            fence_proxy_async_smem();
            issue(t + kStages);
        }

        // rows first (src/libdwt.c:6706-6717), then columns
        if (w == 1) {
            A[0] = fmul(A[0], W.n1_inv);
            B[0] = fmul(B[0], W.n1_inv);
        } else {
            h_inverse<NS>(A, W);
            if (!one_row) h_inverse<NS>(B, W);
        }

        if (one_row) {
            const int p = m0 + t;
            if (!D.rows_only) {
#pragma unroll
                for (int i = 0; i < 4; ++i) A[i] = fmul(A[i], W.n1_inv);
            }
            store4(D.out[0] + p * D.out_pitch[0] + c0, A, ok);
            continue;
        }

        float Ev[4], Ov[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float E = fmul(A[i], W.zeta_o);   // pre-scale: even x (1/zeta)
            const float O = fmul(B[i], W.zeta_e);   //            odd  x zeta
            if (NS == 4) {
                const float e1n = lift(E, W.c[0], o[i], O);        // e'(m)
                const float o1n = lift(o[i], W.c[1], e1[i], e1n);  // o'(m-1)
                const float e2n = lift(e1[i], W.c[2], o1[i], o1n); // e''(m-1)
                const float o2n = lift(o1[i], W.c[3], e2[i], e2n); // o''(m-2)
                Ev[i] = e2[i];                                     // e''(m-2)
                Ov[i] = o2n;
                e1[i] = e1n; o1[i] = o1n; e2[i] = e2n;
            } else {
                const float e1n = lift(E, W.c[0], o[i], O);        // e'(m)
                const float o1n = lift(o[i], W.c[1], e1[i], e1n);  // o'(m-1)
                Ev[i] = e1[i];                                     // e'(m-1)
                Ov[i] = o1n;
                e1[i] = e1n;
            }
            o[i] = O;
        }
        const int p = m0 + t - LAT;
        if (p >= k0) {
            store4(D.out[0] + (2 * p) * D.out_pitch[0] + c0, Ev, ok);
            if (2 * p + 1 < h) store4(D.out[0] + (2 * p + 1) * D.out_pitch[0] + c0, Ov, ok);
        }
    }
    tick += total;
    return true;
}

template <int NS, bool INV>
__global__ void __launch_bounds__(kWarpsPerCta * 32)
level_kernel(const LevelDesc D, const Wavelet W, int *err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *ring = reinterpret_cast<float *>(smem) + warp * kStages * kStageFloats;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kWarpsPerCta * kStages * kStageFloats * 4) +
                     warp * kStages;
    if (lane == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncwarp();

    uint32_t tick = 0;
    const int units = D.n_strips * D.n_segs;
    for (int u = blockIdx.x * kWarpsPerCta + warp; u < units; u += gridDim.x * kWarpsPerCta) {
        const int strip = u % D.n_strips, seg = u / D.n_strips;
        const bool ok = INV ? inverse_unit<NS>(D, W, strip, seg, ring, bars, tick, lane, err)
                            : forward_unit<NS>(D, W, strip, seg, ring, bars, tick, lane, err);
        if (!ok) break;
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
    level_kernel<NS, INV><<<grid, kWarpsPerCta * 32, kSmemBytes, stream>>>(d, W, err);
    return cudaGetLastError();
}

}  // namespace

void plan_level(LevelDesc &d, int seg_pairs_hint)
{
    const bool one_row = (d.h == 1) || d.rows_only;
    const int npairs = one_row ? d.h : (d.h + 1) / 2;
    d.n_strips = ceil_div(d.w, kStripOut);
    int seg = seg_pairs_hint;
    if (seg <= 0) {
        // aim for about 3 units per resident warp slot, segments of 16..256 pairs
        const long long target_units = 152LL * 48 * 3;
        const long long per_strip = std::max<long long>(1, target_units / d.n_strips);
        seg = int((npairs + per_strip - 1) / per_strip);
        seg = std::max(seg, one_row ? 1 : 16);
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
