// Warp work units of the fused lifting level (device code shared by the
// per-level kernel and the batched persistent kernel).
//
// A unit is a strip of 128 interleaved columns (4 per lane) by a segment of
// row pairs of one level of one image.  Its rows (forward) or band rows
// (inverse) are streamed into the warp's private shared-memory ring by the
// TMA bulk-copy engine (cp.async.bulk + mbarrier complete_tx), two row pairs
// per stage, kStages stages deep.  For every row pair the warp
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
// Arithmetic follows the reference's float path operation by operation
// (x + c*(l + r) with three roundings, scaling afterwards / beforehand).
#pragma once

#include "dwt_level2d.cuh"

namespace dwt {
namespace units {

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

// Stage ring cursor: stage index and mbarrier phase parity, advanced per use.
struct Cursor {
    uint32_t st, par;
    __device__ __forceinline__ void next()
    {
        if (++st == kStages) {
            st = 0;
            par ^= 1u;
        }
    }
};

__device__ __forceinline__ Cursor cursor_at(uint32_t tick)
{
    return Cursor{tick % kStages, (tick / kStages) & 1u};
}

// Row pair m of a column of height h: the two source rows, mirrored only at
// the image borders.
__device__ __forceinline__ void pair_rows(int m, int h, int &ra, int &rb)
{
    ra = 2 * m;
    rb = ra + 1;
    if (ra < 0 || rb >= h) {
        ra = mirror(2 * m, h);
        rb = mirror(2 * m + 1, h);
    }
}

// Per-lane store pointer for one band row stream: base + column, advanced by
// the pitch per output row; vector stores when the band base is 8-byte
// aligned and the pitch even (then every lane's pair is aligned: its band
// column is even).
struct BandOut {
    float *p;
    long long pitch;
    bool vec;
    __device__ __forceinline__ void init(float *base, long long pit, int q, int row0)
    {
        vec = ((reinterpret_cast<uintptr_t>(base) & 7) == 0) && ((pit & 1) == 0);
        pitch = pit;
        p = base + q + row0 * pit;
    }
    __device__ __forceinline__ void put(float a, float b, bool va, bool vb) const
    {
        if (vec && va && vb) {
            *reinterpret_cast<float2 *>(p) = make_float2(a, b);
        } else {
            if (va) p[0] = a;
            if (vb) p[1] = b;
        }
    }
    __device__ __forceinline__ void advance() { p += pitch; }
};

// ------------------------------------------------------------ forward, rows

// A unit of single rows: the rows of a one-row image (then the column step
// only scales by n1), or independent 1D signals stored as rows (rows_only).
template <int NS>
__device__ bool forward_rows_unit(const LevelDesc &D, const Wavelet &W, int strip, int seg, float *ring,
                                  uint64_t *bars, uint32_t &tick, int lane, int *err)
{
    const int w = D.w;
    const int b = strip * kStripOut - 4;
    const int k0 = seg * D.seg_pairs;
    const int k1 = min(k0 + D.seg_pairs, D.h);
    const int total = k1 - k0;
    const int w4 = (w + 3) & ~3;
    const int lo = max(b, 0), hi = min(b + kStripIn, w4);
    const uint32_t bytes = uint32_t(hi - lo) * 4u;
    const int dst_off = lo - b;
    int off[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) off[i] = min(max(mirror(b + 4 * lane + i, w) - b, lo - b), hi - b - 1);
    const float *srow = D.in[0] + lo;
    const long long pitch = D.in_pitch[0];
    const float scale = D.rows_only ? 1.0f : W.n1_fwd;

    Cursor pc = cursor_at(tick);
    if (lane == 0) {
        fence_proxy_async_smem();
        for (int t = 0; t < min(total, kStages); ++t) {
            mbar_arrive_expect_tx(&bars[pc.st], bytes);
            bulk_g2s(ring + pc.st * kStageFloats + dst_off, srow + (long long)(k0 + t) * pitch, bytes,
                     &bars[pc.st]);
            pc.next();
        }
    }
    __syncwarp();
    const int c0 = b + 4 * lane;
    const bool lane_ok = lane >= 1 && lane <= kLanes - 2;
    const bool vL0 = lane_ok && c0 < w, vH0 = lane_ok && c0 + 1 < w;
    const bool vL1 = lane_ok && c0 + 2 < w, vH1 = lane_ok && c0 + 3 < w;
    const int q = (b >> 1) + 2 * lane;
    BandOut oL, oH;
    oL.init(D.out[0], D.out_pitch[0], q, k0);
    oH.init(D.out[1], D.out_pitch[1], q, k0);

    Cursor c = cursor_at(tick);
#pragma unroll 1
    for (int t = 0; t < total; ++t) {
        if (!mbar_wait_bounded(&bars[c.st], c.par)) {
            if (lane == 0) raise_error(err, kErrWaitTimeout);
            return false;
        }
        const float *slot = ring + c.st * kStageFloats;
        float A[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) A[i] = slot[off[i]];
        if (w == 1) {
            A[0] = fmul(A[0], W.n1_fwd);
        } else {
            h_forward<NS>(A, W);
        }
        __syncwarp();
        if (lane == 0 && t + kStages < total) {
            mbar_arrive_expect_tx(&bars[c.st], bytes);
            bulk_g2s(ring + c.st * kStageFloats + dst_off, srow + (long long)(k0 + t + kStages) * pitch,
                     bytes, &bars[c.st]);
        }
        c.next();
        if (!D.rows_only) {
#pragma unroll
            for (int i = 0; i < 4; ++i) A[i] = fmul(A[i], scale);
        }
        oL.put(A[0], A[2], vL0, vL1);
        oH.put(A[1], A[3], vH0, vH1);
        oL.advance();
        oH.advance();
    }
    tick += total;
    return true;
}

// --------------------------------------------------------------- forward, 2D

// Horizontal forward lifting of one row held as E = (v0, v2) and O = (v1, v3)
// (the lane's even and odd columns), packed two-wide.
template <int NS>
__device__ __forceinline__ void h_forward2(f2 &E, f2 &O, const f2 *C, f2 ZE, f2 ZO)
{
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
        const float nx = __shfl_down_sync(kFull, f2lo(E), 1);  // next lane's v0
        O = lift2(O, C[s], E, pk(f2hi(E), nx));                // (v1,v3) += c((v0,v2) + (v2,nx))
        const float pv = __shfl_up_sync(kFull, f2hi(O), 1);    // previous lane's v3
        E = lift2(E, C[s + 1], pk(pv, f2lo(O)), O);            // (v0,v2) += c((pv,v1) + (v1,v3))
    }
    E = mul2(E, ZE);
    O = mul2(O, ZO);
}

template <int NS>
__device__ __forceinline__ void h_inverse2(f2 &E, f2 &O, const f2 *C, f2 ZE, f2 ZO)
{
    E = mul2(E, ZO);
    O = mul2(O, ZE);
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
        const float pv = __shfl_up_sync(kFull, f2hi(O), 1);
        E = lift2(E, C[s], pk(pv, f2lo(O)), O);
        const float nx = __shfl_down_sync(kFull, f2lo(E), 1);
        O = lift2(O, C[s + 1], E, pk(f2hi(E), nx));
    }
}

// Vertical forward recurrence of one packed column pair (see forward_unit).
template <int NS>
__device__ __forceinline__ void v_forward2(f2 A, f2 B, f2 &e, f2 &o, f2 &o1, f2 &e1, f2 &o2, const f2 *C,
                                           f2 ZE, f2 ZO, f2 &L, f2 &H)
{
    if (NS == 4) {
        const f2 o1n = lift2(o, C[0], e, A);    // o'(m-1)
        const f2 e1n = lift2(e, C[1], o1, o1n); // e'(m-1)
        const f2 o2n = lift2(o1, C[2], e1, e1n); // o''(m-2)
        const f2 e2n = lift2(e1, C[3], o2, o2n); // e''(m-2)
        L = mul2(e2n, ZE);
        H = mul2(o2n, ZO);
        o1 = o1n; e1 = e1n; o2 = o2n;
    } else {
        const f2 o1n = lift2(o, C[0], e, A);    // o'(m-1)
        const f2 e1n = lift2(e, C[1], o1, o1n); // e'(m-1)
        L = mul2(e1n, ZE);
        H = mul2(o1n, ZO);
        o1 = o1n;
    }
    e = A;
    o = B;
}

// ------------------------------------------------------------ staging pipes
//
// A 2D unit streams `iters` stages (two row pairs each) through a ring of
// shared-memory slots; the pipe owns the slots and their barriers, the unit
// says what a stage holds.  Iterations are numbered by a running tick, so a
// ring carries on across the units a warp takes in turn.
//
// WarpPipe: a warp's private ring.  Its lane 0 issues every stage and
// refills a slot as soon as the warp has read it (the warp's own program
// order orders the reuse).
struct WarpPipe {
    float *ring;
    uint64_t *full;
    static constexpr int kDepth = kStages;
    static constexpr int kLag = 0;  // after reading iteration u, issue u + kDepth - kLag
    __device__ __forceinline__ float *slot(uint32_t t) const { return ring + (t % kDepth) * kStageFloats; }
    __device__ __forceinline__ uint64_t *bar(uint32_t t) const { return &full[t % kDepth]; }
    __device__ __forceinline__ bool wait(uint32_t t) const
    {
        return mbar_wait_bounded(&full[t % kDepth], (t / kDepth) & 1u);
    }
    __device__ __forceinline__ bool producer(int lane) const { return lane == 0; }
    __device__ __forceinline__ bool acquire(uint32_t) const { return true; }
    __device__ __forceinline__ void release(uint32_t, int) const { __syncwarp(); }
};

// Ordered in-place launches (LevelDesc::order).  order_wait: the warp waits
// (at most `limit` polls, 128 ns apart, each lane polling one segment; it
// gives up early when another warp has raised an error) until every strip
// of the segments that must finish before segment `seg` writes into the
// frame is done.  order_done: counts a
// finished strip of `seg`; every read of the unit has completed (its stages
// were waited for), which is all a later writer of those rows needs.
// order_ticket: lane 0 takes the next ticket, when `next` is armed (< 0).
constexpr uint32_t kOrderWaitLimit = 1u << 24;

__device__ __forceinline__ bool order_wait(const LevelDesc &D, bool inverse, int lat, int seg, int lane, int *err,
                                           uint32_t limit = kOrderWaitLimit)
{
    int a, b;
    inplace_readers(D.h, D.seg_pairs, D.n_segs, lat, inverse, seg, D.stage_seg, D.order_dy, a, b);
    if (b < a) return true;
    // one segment per lane (ranges span a few segments; longer ones loop)
    bool ok = true;
    for (int r0 = a; r0 <= b; r0 += 32) {
        const int r = r0 + lane;
        bool mine = r > b || r == seg;  // the host's stage_seg excludes seg itself
        uint32_t spins = 0;
        while (!__all_sync(0xffffffffu, mine)) {
            if (!mine) mine = ld_acquire(D.order + 1 + r) >= D.n_strips;
            if (__all_sync(0xffffffffu, mine)) break;
            __nanosleep(128);
            const bool give_up = ++spins > limit || (err && *reinterpret_cast<volatile int *>(err) != 0);
            if (__any_sync(0xffffffffu, give_up)) {
                if (lane == 0) raise_error(err, kErrQueueTimeout);
                ok = false;
                break;
            }
        }
        if (!ok) break;
    }
    __syncwarp();
    return ok;
}

__device__ __forceinline__ void order_done(const LevelDesc &D, int seg, int lane)
{
    __syncwarp();
    if (lane == 0) atomicAdd(D.order + 1 + seg, 1);
}

__device__ __forceinline__ void order_ticket(const LevelDesc &D, int lane, int &next)
{
    if (lane == 0 && next < 0) next = atomicAdd(D.order, 1);  // armed by a negative value
}

// Waits (bounded) for the first `count` stages a unit has issued, so that
// no copy is still landing in the ring when the unit gives up.
template <class Pipe>
__device__ __forceinline__ void drain_issued(const Pipe &pipe, uint32_t t0, int count)
{
    for (int u = 0; u < count; ++u) pipe.wait(t0 + u);
    __syncwarp();
}

// Stage count of a 2D unit of segment `seg`: pairs k0-LAT .. k1+LAT-1, two
// per stage.
template <int NS>
__device__ __forceinline__ void unit_span(const LevelDesc &D, int seg, int &k0, int &total, int &iters)
{
    constexpr int LAT = NS / 2;
    const int npairs = (D.h + 1) >> 1;
    k0 = seg * D.seg_pairs;
    const int k1 = min(k0 + D.seg_pairs, npairs);
    total = k1 - k0 + 2 * LAT;
    iters = (total + 1) >> 1;
}

// One unit of the fused forward level: interleaved rows in, four bands out.
// Per row pair m (rows 2m, 2m+1, mirrored at the borders) the vertical
// recurrence emits output pair m - LAT; pairs k0-LAT .. k1+LAT-1 are walked
// so that the unit's outputs k0 .. k1-1 are exact.  EDGE selects the general
// path for strips touching the left or right border (mirrored columns,
// partial lanes) or unaligned outputs.  The rows are staged from column B
// on, `win` columns wide, `slot_f` floats per row slot.
template <int NS, bool EDGE, class Pipe, bool ORD = false, bool VST = true>
__device__ bool forward_unit(const LevelDesc &D, const Wavelet &W, int strip, int seg, const Pipe &pipe, int B,
                             int win, int slot_f, uint32_t &tick, int lane, int *err, int &next)
{
    constexpr int LAT = NS / 2;
    const int w = D.w, h = D.h;
    const int b = strip * kStripOut - 4;  // interleaved column held by lane 0, value 0
    int k0, total, iters;
    unit_span<NS>(D, seg, k0, total, iters);
    const int m0 = k0 - LAT;

    // staged column window [lo, hi) of every row
    const int w4 = (w + 3) & ~3;
    const int lo = max(B, 0), hi = min(B + win, w4);
    const uint32_t bytes = uint32_t(hi - lo) * 4u;
    const int dst_off = lo - B;
    const float *srow = D.in[0] + lo;
    const long long pitch = D.in_pitch[0];

    // this lane's slot offsets (mirrored at the borders)
    int off[4];
    if (EDGE) {
#pragma unroll
        for (int i = 0; i < 4; ++i) off[i] = min(max(mirror(b + 4 * lane + i, w) - B, lo - B), hi - B - 1);
    } else {
        off[0] = b - B + 4 * lane;
    }

    const uint32_t t0 = tick;
    bool issued_ok = true;
    auto issue = [&](int u) {
        const uint32_t t = t0 + u;
        if (!pipe.acquire(t)) return false;
        float *dst = pipe.slot(t) + dst_off;
        uint64_t *bar = pipe.bar(t);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, 4 * bytes);
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            int ra, rb;
            pair_rows(m0 + 2 * u + r, h, ra, rb);
            bulk_g2s(dst + (2 * r) * slot_f, srow + ra * pitch, bytes, bar);
            bulk_g2s(dst + (2 * r + 1) * slot_f, srow + rb * pitch, bytes, bar);
        }
        return true;
    };
    if (pipe.producer(lane))
        for (int u = 0; u < min(iters, Pipe::kDepth) && issued_ok; ++u) issued_ok = issue(u);
    __syncwarp();
    // ordered in-place launch: the reads are in flight; wait before storing
    if (ORD && !order_wait(D, false, LAT, seg, lane, err)) {
        drain_issued(pipe, t0, issued_ok ? min(iters, Pipe::kDepth) : 0);
        return false;
    }
    const int ticket_at = max(0, iters - Pipe::kDepth);

    // packed constants
    f2 C[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) C[k] = pk(W.c[k], W.c[k]);
    const f2 ZE = pk(W.zeta_e, W.zeta_e), ZO = pk(W.zeta_o, W.zeta_o);
    const f2 N1 = pk(W.n1_fwd, W.n1_fwd);

    // output geometry of this lane: band column q, stores of (even, odd) pairs
    const int c0 = b + 4 * lane;
    const bool lane_ok = lane >= 1 && lane <= kLanes - 2;
    const bool vL0 = lane_ok && c0 < w, vH0 = lane_ok && c0 + 1 < w;
    const bool vL1 = lane_ok && c0 + 2 < w, vH1 = lane_ok && c0 + 3 < w;
    const int q = (b >> 1) + 2 * lane;
    // LH / HH of a staged segment of an ordered in-place launch go to alt
    const bool alt = ORD && seg >= D.stage_seg;
    const long long sLH = alt ? D.alt_pitch : D.out_pitch[2], sHH = alt ? D.alt_pitch : D.out_pitch[3];
    float *pLL = D.out[0] + q + (long long)k0 * D.out_pitch[0];
    float *pHL = D.out[1] + q + (long long)k0 * D.out_pitch[1];
    float *pLH = (alt ? D.alt[0] : D.out[2]) + q + (long long)k0 * sLH;
    float *pHH = (alt ? D.alt[1] : D.out[3]) + q + (long long)k0 * sHH;
    const int last_h = (h >> 1) - 1;  // last output pair with an H row

    f2 e[2] = {0, 0}, o[2] = {0, 0}, o1[2] = {0, 0}, e1[2] = {0, 0}, o2[2] = {0, 0};

    int t = 0;  // pair counter
#pragma unroll 1
    for (int u = 0; u < iters; ++u) {
        if (!__all_sync(kFull, pipe.wait(t0 + u))) {
            if (lane == 0) raise_error(err, kErrWaitTimeout);
            return false;
        }
        const float *slot = pipe.slot(t0 + u);
        f2 E[4], O[4];  // rows 0..3 of the stage
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const float *row = slot + r * slot_f;
            if (EDGE) {
                E[r] = pk(row[off[0]], row[off[2]]);
                O[r] = pk(row[off[1]], row[off[3]]);
            } else {
                const float4 v = *reinterpret_cast<const float4 *>(row + off[0]);
                E[r] = pk(v.x, v.z);
                O[r] = pk(v.y, v.w);
            }
        }
        // the stage is read: release it, and issue the one kDepth - kLag ahead
        pipe.release(t0 + u, lane);
        if (pipe.producer(lane) && issued_ok && u >= Pipe::kLag && u - Pipe::kLag + Pipe::kDepth < iters)
            issued_ok = issue(u - Pipe::kLag + Pipe::kDepth);
        if (ORD && u == ticket_at) order_ticket(D, lane, next);
        // rows: horizontal lifting (a single-sample row is only scaled)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (w == 1) {
                E[r] = mul2(E[r], N1);
            } else {
                h_forward2<NS>(E[r], O[r], C, ZE, ZO);
            }
        }

        // columns: two steps of the vertical recurrence (two row pairs)
#pragma unroll
        for (int r = 0; r < 2; ++r, ++t) {
            f2 LE, HE, LO, HO;
            v_forward2<NS>(E[2 * r], E[2 * r + 1], e[0], o[0], o1[0], e1[0], o2[0], C, ZE, ZO, LE, HE);
            v_forward2<NS>(O[2 * r], O[2 * r + 1], e[1], o[1], o1[1], e1[1], o2[1], C, ZE, ZO, LO, HO);
            if (t >= 2 * LAT && t < total) {
                const int p = m0 + t - LAT;
                if (EDGE) {
                    if (vL0) pLL[0] = f2lo(LE);
                    if (vL1) pLL[1] = f2hi(LE);
                    if (vH0) pHL[0] = f2lo(LO);
                    if (vH1) pHL[1] = f2hi(LO);
                    if (p <= last_h) {
                        if (vL0) pLH[0] = f2lo(HE);
                        if (vL1) pLH[1] = f2hi(HE);
                        if (vH0) pHH[0] = f2lo(HO);
                        if (vH1) pHH[1] = f2hi(HO);
                    }
                } else if (lane_ok) {
                    if (VST) {
                        *reinterpret_cast<f2 *>(pLL) = LE;
                        *reinterpret_cast<f2 *>(pHL) = LO;
                        if (p <= last_h) {
                            *reinterpret_cast<f2 *>(pLH) = HE;
                            *reinterpret_cast<f2 *>(pHH) = HO;
                        }
                    } else {  // band rows not 8-byte aligned (an odd pitch): the same samples one by one
                        pLL[0] = f2lo(LE);
                        pLL[1] = f2hi(LE);
                        pHL[0] = f2lo(LO);
                        pHL[1] = f2hi(LO);
                        if (p <= last_h) {
                            pLH[0] = f2lo(HE);
                            pLH[1] = f2hi(HE);
                            pHH[0] = f2lo(HO);
                            pHH[1] = f2hi(HO);
                        }
                    }
                }
                pLL += D.out_pitch[0];
                pHL += D.out_pitch[1];
                pLH += sLH;
                pHH += sHH;
            }
        }
    }
    // a failed issue (the producer gave up waiting for a slot) fails the
    // whole warp, uniformly
    const bool ok = __all_sync(kFull, issued_ok);
    if (!ok && lane == 0) raise_error(err, kErrWaitTimeout);
    tick += iters;
    return ok;
}

// ------------------------------------------------------------------ inverse

// One band's staged window: its row 0 start rounded down to 16 bytes, the
// byte count per row and the float shift of the wanted first column.
struct BandIn {
    const float *base;  // 16-byte aligned start in row 0
    long long pitch;
    uint32_t bytes;
    int shift;
    __device__ __forceinline__ void init(const float *band, long long pit, int lo, int n)
    {
        pitch = pit;
        if (n <= 0) {
            bytes = 0;
            shift = 0;
            base = band;
            return;
        }
        const uintptr_t a = reinterpret_cast<uintptr_t>(band + lo);
        const uintptr_t a0 = a & ~uintptr_t(15);
        const uintptr_t e = (a + uintptr_t(n) * 4 + 15) & ~uintptr_t(15);
        base = reinterpret_cast<const float *>(a0);
        bytes = uint32_t(e - a0);
        shift = int((a - a0) >> 2);
    }
};

// Inverse units of single rows (one-row images and rows_only signals).
template <int NS>
__device__ bool inverse_rows_unit(const LevelDesc &D, const Wavelet &W, int strip, int seg, float *ring,
                                  uint64_t *bars, uint32_t &tick, int lane, int *err)
{
    const int w = D.w;
    const int b = strip * kStripOut - 4;
    const int bq = b >> 1;
    const int Lw = (w + 1) >> 1, Hw = w >> 1;
    const int k0 = seg * D.seg_pairs;
    const int k1 = min(k0 + D.seg_pairs, D.h);
    const int total = k1 - k0;
    const int loL = max(bq, 0), hiL = min(bq + 64, Lw);
    const int loH = loL, hiH = min(bq + 64, Hw);
    BandIn iL, iH;
    iL.init(D.in[0], D.in_pitch[0], loL, hiL - loL);
    iH.init(D.in[1], D.in_pitch[1], loH, hiH - loH);
    int off[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int bi = 0, k = 0;
        if (w != 1) {
            const int mc = mirror(b + 4 * lane + i, w);
            bi = mc >> 1;
            k = mc & 1;
        }
        const int o = bi - (k ? loH : loL) + (k ? iH.shift : iL.shift);
        off[i] = k * kSlotI + min(max(o, 0), kSlotI - 1);
    }
    const uint32_t tx = iL.bytes + iH.bytes;
    auto issue = [&](int row, const Cursor &pc) {
        float *slot = ring + pc.st * kStageFloats;
        mbar_arrive_expect_tx(&bars[pc.st], tx);
        bulk_g2s(slot, iL.base + row * iL.pitch, iL.bytes, &bars[pc.st]);
        if (iH.bytes) bulk_g2s(slot + kSlotI, iH.base + row * iH.pitch, iH.bytes, &bars[pc.st]);
    };
    if (lane == 0) {
        fence_proxy_async_smem();
        Cursor pc = cursor_at(tick);
        for (int t = 0; t < min(total, kStages); ++t) {
            issue(k0 + t, pc);
            pc.next();
        }
    }
    __syncwarp();
    const int c0 = b + 4 * lane;
    const bool lane_ok = lane >= 1 && lane <= kLanes - 2;
    bool ok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) ok[i] = lane_ok && (c0 + i < w);
    const float scale = D.rows_only ? 1.0f : W.n1_inv;
    float *orow = D.out[0] + c0 + (long long)k0 * D.out_pitch[0];

    Cursor c = cursor_at(tick);
#pragma unroll 1
    for (int t = 0; t < total; ++t) {
        if (!mbar_wait_bounded(&bars[c.st], c.par)) {
            if (lane == 0) raise_error(err, kErrWaitTimeout);
            return false;
        }
        const float *slot = ring + c.st * kStageFloats;
        float A[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) A[i] = slot[off[i]];
        if (w == 1) {
            A[0] = fmul(A[0], W.n1_inv);
        } else {
            h_inverse<NS>(A, W);
        }
        __syncwarp();
        if (lane == 0 && t + kStages < total) issue(k0 + t + kStages, c);
        c.next();
        if (!D.rows_only) {
#pragma unroll
            for (int i = 0; i < 4; ++i) A[i] = fmul(A[i], scale);
        }
        store4(orow, A, ok);
        orow += D.out_pitch[0];
    }
    tick += total;
    return true;
}

// Vertical inverse recurrence of one packed column pair (see inverse_unit).
template <int NS>
__device__ __forceinline__ void v_inverse2(f2 A, f2 B, f2 &o, f2 &e1, f2 &o1, f2 &e2, const f2 *C, f2 ZE,
                                           f2 ZO, f2 &Ev, f2 &Ov)
{
    const f2 E = mul2(A, ZO);  // pre-scale: even x (1/zeta)
    const f2 O = mul2(B, ZE);  //            odd  x zeta
    if (NS == 4) {
        const f2 e1n = lift2(E, C[0], o, O);      // e'(m)
        const f2 o1n = lift2(o, C[1], e1, e1n);   // o'(m-1)
        const f2 e2n = lift2(e1, C[2], o1, o1n);  // e''(m-1)
        const f2 o2n = lift2(o1, C[3], e2, e2n);  // o''(m-2)
        Ev = e2;                                  // e''(m-2)
        Ov = o2n;
        e1 = e1n; o1 = o1n; e2 = e2n;
    } else {
        const f2 e1n = lift2(E, C[0], o, O);      // e'(m)
        const f2 o1n = lift2(o, C[1], e1, e1n);   // o'(m-1)
        Ev = e1;                                  // e'(m-1)
        Ov = o1n;
        e1 = e1n;
    }
    o = O;
}

// One unit of the fused inverse level: four bands in, interleaved rows out.
// Per pair m the stage holds the LL and HL rows of L-row ra/2 and the LH and
// HH rows of H-row rb/2 (ra, rb the mirrored interleaved rows 2m, 2m+1); the
// horizontal inverse rebuilds both interleaved rows, the vertical recurrence
// emits output rows 2(m-LAT), 2(m-LAT)+1.  The band rows are staged from
// band column B/2 on, `band_win` columns wide.  Stage layout: band k (LL,
// HL, LH, HH) at slot + k*kBandSlotF, its row for pair r at + r*kBandRowF,
// band column c at offset c - (window start rounded down to 16 bytes).
// With tensor maps (maps: the LL band, the frame holding HL, LH, HH and, in
// an ordered in-place launch, the frame holding the in-frame LH, HH rows), an
// interior unit stages each band's two consecutive rows of a stage with one
// 68 x 2 box copy; stages with mirrored rows and edge units use one bulk copy
// per band row.
template <int NS, bool EDGE, class Pipe, bool ORD = false>
__device__ bool inverse_unit(const LevelDesc &D, const Wavelet &W, int strip, int seg, const Pipe &pipe, int B,
                             int band_win, const LevelMaps *maps, uint32_t &tick, int lane, int *err,
                             int &next)
{
    constexpr int LAT = NS / 2;
    const int w = D.w, h = D.h;
    const int b = strip * kStripOut - 4;
    const int bq = b >> 1;  // band column of lane 0's first value
    const int bqB = B >> 1;  // band column of the staged window's start
    const int Lw = (w + 1) >> 1, Hw = w >> 1;
    int k0, total, iters;
    unit_span<NS>(D, seg, k0, total, iters);
    const int m0 = k0 - LAT;

    // staged band column windows; the shift is the same for every row
    // because source pitches are multiples of 4 floats
    const int loL = max(bqB, 0), hiL = min(bqB + band_win, Lw);
    const int loH = loL, hiH = min(bqB + band_win, Hw);
    // LH / HH of a staged segment of an ordered in-place launch come from alt
    const bool alt = ORD && seg >= D.stage_seg;
    BandIn iLL, iHL, iLH, iHH;
    iLL.init(D.in[0], D.in_pitch[0], loL, hiL - loL);
    iHL.init(D.in[1], D.in_pitch[1], loH, hiH - loH);
    iLH.init(alt ? D.alt[0] : D.in[2], alt ? D.alt_pitch : D.in_pitch[2], loL, hiL - loL);
    iHH.init(alt ? D.alt[1] : D.in[3], alt ? D.alt_pitch : D.in_pitch[3], loH, hiH - loH);
    const uint32_t tx1 = 2 * (iLL.bytes + iHL.bytes + iLH.bytes + iHH.bytes);
    // box copies: interior units only (their windows start at or after
    // column 0 and the box's 16-byte aligned x is that window start)
    const bool boxes = !EDGE && maps != nullptr;
    const bool lower = ORD && !alt;  // LH / HH boxes from maps->lower
    constexpr uint32_t kBoxBytes = kBandRowF * 2 * 4;

    // this lane's offsets inside a stage: even samples from the L bands
    // (LL / LH slots), odd samples from the H bands (HL / HH slots)
    int offA[4], offB[4];
    if (EDGE) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int bi = 0, k = 0;
            if (w != 1) {
                const int mc = mirror(b + 4 * lane + i, w);
                bi = mc >> 1;
                k = mc & 1;
            }
            const int lo_k = k ? loH : loL;
            const int oa = bi - lo_k + (k ? iHL.shift : iLL.shift);
            const int ob = bi - lo_k + (k ? iHH.shift : iLH.shift);
            offA[i] = k * kBandSlotF + min(max(oa, 0), kBandRowF - 1);
            offB[i] = (2 + k) * kBandSlotF + min(max(ob, 0), kBandRowF - 1);
        }
    } else {
        const int d = bq - loL + 2 * lane;
        offA[0] = d + iLL.shift;
        offA[1] = kBandSlotF + d + iHL.shift;
        offB[0] = 2 * kBandSlotF + d + iLH.shift;
        offB[1] = 3 * kBandSlotF + d + iHH.shift;
    }

    const uint32_t t0 = tick;
    bool issued_ok = true;
    auto issue = [&](int u) {
        const uint32_t t = t0 + u;
        if (!pipe.acquire(t)) return false;
        float *slot = pipe.slot(t);
        uint64_t *bar = pipe.bar(t);
        const int m = m0 + 2 * u;  // first pair of the stage
        fence_proxy_async_smem();
        if (boxes && m >= 0 && 2 * m + 3 < h) {
            // both pairs interior: band rows m and m + 1 of every band
            mbar_arrive_expect_tx(bar, 4 * kBoxBytes);
            const CUtensorMap *mlo = lower ? &maps->lower : &maps->frame;
            tma_load_2d(slot, &maps->ll, loL - iLL.shift, m, bar);
            tma_load_2d(slot + kBandSlotF, &maps->frame, D.map_dx + loH - iHL.shift, m, bar);
            tma_load_2d(slot + 2 * kBandSlotF, mlo, loL - iLH.shift, D.map_dy + m, bar);
            tma_load_2d(slot + 3 * kBandSlotF, mlo, D.map_dx + loH - iHH.shift, D.map_dy + m, bar);
            return true;
        }
        mbar_arrive_expect_tx(bar, tx1);
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            int ra, rb;
            pair_rows(m + r, h, ra, rb);
            const int qa = ra >> 1, qb = rb >> 1;
            float *sl = slot + r * kBandRowF;
            bulk_g2s(sl, iLL.base + qa * iLL.pitch, iLL.bytes, bar);
            bulk_g2s(sl + 2 * kBandSlotF, iLH.base + qb * iLH.pitch, iLH.bytes, bar);
            if (iHL.bytes) {
                bulk_g2s(sl + kBandSlotF, iHL.base + qa * iHL.pitch, iHL.bytes, bar);
                bulk_g2s(sl + 3 * kBandSlotF, iHH.base + qb * iHH.pitch, iHH.bytes, bar);
            }
        }
        return true;
    };
    if (pipe.producer(lane))
        for (int u = 0; u < min(iters, Pipe::kDepth) && issued_ok; ++u) issued_ok = issue(u);
    __syncwarp();
    // ordered in-place launch: the reads are in flight; wait before storing
    if (ORD && !order_wait(D, true, LAT, seg, lane, err)) {
        drain_issued(pipe, t0, issued_ok ? min(iters, Pipe::kDepth) : 0);
        return false;
    }
    const int ticket_at = max(0, iters - Pipe::kDepth);

    f2 C[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) C[k] = pk(W.c[k], W.c[k]);
    const f2 ZE = pk(W.zeta_e, W.zeta_e), ZO = pk(W.zeta_o, W.zeta_o);
    const f2 N1 = pk(W.n1_inv, W.n1_inv);

    const int c0 = b + 4 * lane;
    const bool lane_ok = lane >= 1 && lane <= kLanes - 2;
    bool ok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) ok[i] = lane_ok && (c0 + i < w);
    const long long opitch = D.out_pitch[0];
    float *orow = D.out[0] + c0 + (long long)(2 * k0) * opitch;  // row 2p of output pair p
    const int last_odd = (h >> 1) - 1;

    f2 o[2] = {0, 0}, e1[2] = {0, 0}, o1[2] = {0, 0}, e2[2] = {0, 0};

    int t = 0;
#pragma unroll 1
    for (int u = 0; u < iters; ++u) {
        if (!__all_sync(kFull, pipe.wait(t0 + u))) {
            if (lane == 0) raise_error(err, kErrWaitTimeout);
            return false;
        }
        const float *slot = pipe.slot(t0 + u);
        f2 E[4], O[4];  // interleaved rows: pair 0 L-row, H-row, pair 1 L-row, H-row
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const float *sl = slot + r * kBandRowF;
            if (EDGE) {
                E[2 * r] = pk(sl[offA[0]], sl[offA[2]]);
                O[2 * r] = pk(sl[offA[1]], sl[offA[3]]);
                E[2 * r + 1] = pk(sl[offB[0]], sl[offB[2]]);
                O[2 * r + 1] = pk(sl[offB[1]], sl[offB[3]]);
            } else {
                E[2 * r] = *reinterpret_cast<const f2 *>(sl + offA[0]);
                O[2 * r] = *reinterpret_cast<const f2 *>(sl + offA[1]);
                E[2 * r + 1] = *reinterpret_cast<const f2 *>(sl + offB[0]);
                O[2 * r + 1] = *reinterpret_cast<const f2 *>(sl + offB[1]);
            }
        }
        pipe.release(t0 + u, lane);
        if (pipe.producer(lane) && issued_ok && u >= Pipe::kLag && u - Pipe::kLag + Pipe::kDepth < iters)
            issued_ok = issue(u - Pipe::kLag + Pipe::kDepth);
        if (ORD && u == ticket_at) order_ticket(D, lane, next);
        // rows first (src/libdwt.c:6706-6717), then columns
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (w == 1) {
                E[r] = mul2(E[r], N1);
            } else {
                h_inverse2<NS>(E[r], O[r], C, ZE, ZO);
            }
        }

#pragma unroll
        for (int r = 0; r < 2; ++r, ++t) {
            f2 EvE, OvE, EvO, OvO;
            v_inverse2<NS>(E[2 * r], E[2 * r + 1], o[0], e1[0], o1[0], e2[0], C, ZE, ZO, EvE, OvE);
            v_inverse2<NS>(O[2 * r], O[2 * r + 1], o[1], e1[1], o1[1], e2[1], C, ZE, ZO, EvO, OvO);
            if (t >= 2 * LAT && t < total) {
                const int p = m0 + t - LAT;
                if (EDGE) {
                    const float ev[4] = {f2lo(EvE), f2lo(EvO), f2hi(EvE), f2hi(EvO)};
                    store4(orow, ev, ok);
                    if (p <= last_odd) {
                        const float ov[4] = {f2lo(OvE), f2lo(OvO), f2hi(OvE), f2hi(OvO)};
                        store4(orow + opitch, ov, ok);
                    }
                } else if (lane_ok) {
                    *reinterpret_cast<float4 *>(orow) = make_float4(f2lo(EvE), f2lo(EvO), f2hi(EvE), f2hi(EvO));
                    if (p <= last_odd)
                        *reinterpret_cast<float4 *>(orow + opitch) =
                            make_float4(f2lo(OvE), f2lo(OvO), f2hi(OvE), f2hi(OvO));
                }
                orow += 2 * opitch;
            }
        }
    }
    const bool okw = __all_sync(kFull, issued_ok);
    if (!okw && lane == 0) raise_error(err, kErrWaitTimeout);
    tick += iters;
    return okw;
}

// Whether interior units of a launch may use vector loads and stores: every
// band pointer and pitch must keep them aligned.
template <bool INV>
__device__ __forceinline__ bool fast_ok(const LevelDesc &D)
{
    bool ok;
    if (INV) {
        ok = ((reinterpret_cast<uintptr_t>(D.out[0]) & 15) == 0) && ((D.out_pitch[0] & 3) == 0);
        for (int k = 0; k < 4; ++k) {
            // LDS.64 of band pairs needs an even float shift of every band row
            const uintptr_t a = reinterpret_cast<uintptr_t>(D.in[k]);
            ok = ok && ((a & 7) == 0) && ((D.in_pitch[k] & 3) == 0);
        }
        if (D.order)
            for (int k = 0; k < 2; ++k)
                ok = ok && ((reinterpret_cast<uintptr_t>(D.alt[k]) & 7) == 0) && ((D.alt_pitch & 3) == 0);
    } else {
        ok = true;
        for (int k = 0; k < 4; ++k)
            ok = ok && ((reinterpret_cast<uintptr_t>(D.out[k]) & 7) == 0) && ((D.out_pitch[k] & 1) == 0);
        if (D.order)
            for (int k = 0; k < 2; ++k)
                ok = ok && ((reinterpret_cast<uintptr_t>(D.alt[k]) & 7) == 0) && ((D.alt_pitch & 1) == 0);
    }
    return ok;
}

// Runs one unit (strip, seg) of the level described by D on a warp's
// private ring.
template <int NS, bool INV, bool ORD = false, bool VST = true>
__device__ __forceinline__ bool run_unit(const LevelDesc &D, const Wavelet &W, int strip, int seg, float *ring,
                                         uint64_t *bars, uint32_t &tick, int lane, int *err, bool fast_launch,
                                         const LevelMaps *maps, int &next)
{
    if (D.h == 1 || D.rows_only)
        return INV ? inverse_rows_unit<NS>(D, W, strip, seg, ring, bars, tick, lane, err)
                   : forward_rows_unit<NS>(D, W, strip, seg, ring, bars, tick, lane, err);
    const int b = strip * kStripOut - 4;
    const WarpPipe pipe{ring, bars};
    if constexpr (!INV && !VST) {
        // a forward launch whose bands are not 8-byte aligned (an odd pitch):
        // the alignment only concerns the stores (the rows come from the
        // ring), so interior strips keep the fast loads and store one by one
        if (b < 0 || b + kStripIn + 2 > D.w)
            return forward_unit<NS, true, WarpPipe, ORD>(D, W, strip, seg, pipe, b, kStripIn, kSlotF, tick, lane, err,
                                                         next);
        return forward_unit<NS, false, WarpPipe, ORD, false>(D, W, strip, seg, pipe, b, kStripIn, kSlotF, tick, lane,
                                                             err, next);
    }
    const bool edge = !fast_launch || b < 0 || b + kStripIn + 2 > D.w;
    if (INV)
        return edge ? inverse_unit<NS, true, WarpPipe, ORD>(D, W, strip, seg, pipe, b, kStripIn / 2, maps, tick, lane,
                                                            err, next)
                    : inverse_unit<NS, false, WarpPipe, ORD>(D, W, strip, seg, pipe, b, kStripIn / 2, maps, tick,
                                                             lane, err, next);
    return edge ? forward_unit<NS, true, WarpPipe, ORD>(D, W, strip, seg, pipe, b, kStripIn, kSlotF, tick, lane, err,
                                                        next)
                : forward_unit<NS, false, WarpPipe, ORD>(D, W, strip, seg, pipe, b, kStripIn, kSlotF, tick, lane,
                                                         err, next);
}

// Per-warp ring and barriers inside a CTA's dynamic shared memory.
__device__ __forceinline__ float *warp_ring(unsigned char *smem, int warp)
{
    return reinterpret_cast<float *>(smem) + warp * kStages * kStageFloats;
}
__device__ __forceinline__ uint64_t *warp_bars(unsigned char *smem, int warp, int warps_per_cta)
{
    return reinterpret_cast<uint64_t *>(smem + warps_per_cta * kStages * kStageFloats * 4) + warp * kStages;
}
__device__ __forceinline__ void init_bars(uint64_t *bars, int lane)
{
    if (lane == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncwarp();
}

}  // namespace units
}  // namespace dwt
