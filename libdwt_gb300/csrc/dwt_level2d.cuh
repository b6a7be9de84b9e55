// One decomposition level of the 2D lifting transform, fused rows + columns,
// out of place: the forward reads one interleaved image and writes the four
// bands LL, HL, LH, HH; the inverse reads the four bands and writes the
// interleaved image.  Declarations shared by the host launchers.
#pragma once

#include "dwt_common.cuh"

namespace dwt {

// Work decomposition: a warp holds kStripIn interleaved columns of a row
// (4 per lane) and produces the kStripOut middle ones; lanes 0 and 31 are the
// lifting halo.  Rows are walked as (even, odd) pairs in segments of
// seg_pairs output pairs, each segment warmed up by the lifting latency;
// one pipeline stage carries two pairs.
constexpr int kLanes = 32;
constexpr int kStripIn = 128;
constexpr int kStripOut = 120;
constexpr int kSlotF = 136;        // floats per forward row slot
constexpr int kSlotI = 68;         // floats per band-row slot of the single-row units
// Inverse 2D stages: per band (LL, HL, LH, HH) a slot of the stage's two
// band rows, kBandRowF floats each, band slots kBandSlotF floats apart so
// that every slot starts on a 128-byte boundary (the destination of a
// tensor copy of a 68 x 2 box).
constexpr int kBandRowF = 68;
constexpr int kBandSlotF = 160;
constexpr int kStageFloats = 640;  // one pipeline stage = 2 row pairs: 4 rows or 4 band slots
constexpr int kStages = 4;         // pipeline depth per warp (8 row pairs)
constexpr int kWarpsPerCta = 4;
constexpr int kSmemBytes = kWarpsPerCta * (kStages * kStageFloats * 4 + kStages * 8);

// One level of one image.  Forward: in[0] is the interleaved w x h source,
// out[0..3] receive LL, HL, LH, HH.  Inverse: in[0..3] are LL, HL, LH, HH,
// out[0] receives the interleaved w x h image.  Pitches are in floats.
// Sources must have 16-byte aligned rows (pitch % 4 == 0, 16-byte aligned
// base for out-of-band reads); destinations need 4-byte alignment only.
// rows_only: transform rows only (1D signals stored as rows), no vertical step.
struct LevelDesc {
    int w, h;
    int n_strips, seg_pairs, n_segs;
    int seg_base;  // first segment of this launch (a launch may cover a sub-range)
    int reverse;   // hand out the segments bottom-up (the previous level ended there)
    int rows_only;
    int tmap;      // inverse: the tensor maps of the launch are valid (set by launch_level)
    int map_dx, map_dy;  // with tmap: column of HL / HH and row of LH / HH in the mapped frames
    const float *in[4];
    long long in_pitch[4];
    float *out[4];
    long long out_pitch[4];
    // Ordered in-place launch (level 0 of a transform in the caller's frame;
    // null otherwise).  Units are handed out by a ticket in segment order
    // (bottom-up when reverse is set) and each one waits, before it starts,
    // for the segments that come earlier in that order and read the rows it
    // overwrites (inplace_readers).  order[0] is the ticket and order[1 + s]
    // counts the finished strips of segment s; all zero at launch.
    int *order;
    // Segments >= stage_seg write (forward) or read (inverse) their LH and
    // HH rows at alt[0] / alt[1] (pitch alt_pitch) instead of out / in.
    int stage_seg;
    int order_dy;  // frame row of the LH / HH bands' first row ((h + 1) / 2 in a dense frame)
    float *alt[2];
    long long alt_pitch;
};

__host__ __device__ inline int floordiv_i(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
__host__ __device__ inline int min_i(int a, int b) { return a < b ? a : b; }
__host__ __device__ inline int max_i(int a, int b) { return a > b ? a : b; }

// The segments of an ordered in-place level of height h (segments of S row
// pairs, nsegs of them, lifting latency lat pairs; the LH / HH bands from
// frame row dy on) that must be finished before segment s writes into the
// caller's frame: the inclusive range [a, b], empty when b < a.
//   forward: every segment whose image rows (its pairs k0 - lat .. k1 + lat,
//     mirrored) meet the LH / HH rows dy + k0 .. that s writes; a staged
//     segment (s >= stage_seg) writes those rows elsewhere and waits for
//     nothing.
//   inverse: every segment below stage_seg (the ones reading LH / HH in the
//     frame) whose LH / HH rows meet the image rows 2 k0 .. 2 k1 - 1 that s
//     writes.
// Each read range is widened by two rows of margin.  The host chooses
// stage_seg so that every segment in range comes earlier in the launch's
// order than s.
__host__ __device__ inline void inplace_readers(int h, int S, int nsegs, int lat, bool inverse, int s,
                                                int stage_seg, int dy, int &a, int &b)
{
    constexpr int mg = 2;
    const int hs = (h + 1) >> 1;
    const int k0 = s * S, k1 = min_i(k0 + S, hs);
    a = 1;
    b = 0;
    if (!inverse) {
        if (s >= stage_seg) return;
        const int lo = dy + k0, hi = dy + min_i(k1, h >> 1);
        if (hi <= lo) return;
        // segment s' reads rows [2 (s' S - lat) - mg, 2 ((s' + 1) S + lat + 1) + mg)
        a = max_i(0, floordiv_i(lo - 2 * lat - 2 - mg, 2 * S));
        b = min_i(nsegs - 1, floordiv_i(hi + 2 * lat + mg + 2 * S - 1, 2 * S) - 1);
    } else {
        const int lo = 2 * k0, hi = min_i(2 * k1, h);
        if (hi <= lo) return;
        // segment s' reads rows dy + [s' S - lat - mg, (s' + 1) S + lat + 1 + mg)
        a = max_i(0, floordiv_i(lo - dy - lat - 1 - mg, S));
        b = min_i(min_i(nsegs, stage_seg) - 1, floordiv_i(hi - dy + lat + mg + S - 1, S) - 1);
    }
}

// Tensor maps of an inverse level: the LL band (box kBandRowF x 2) and the
// coefficient frame holding HL, LH, HH (the level's w x h region, same box);
// in an ordered in-place launch `frame` is the staging frame (HL and the
// staged LH, HH rows) and `lower` the caller's frame.
struct LevelMaps {
    CUtensorMap ll;
    CUtensorMap frame;
    CUtensorMap lower;  // ordered in-place launches: the frame holding the in-frame LH, HH rows
};

// Fills n_strips / seg_pairs / n_segs for a level of size w x h (the
// segment length depends on the direction).
void plan_level(LevelDesc &d, int seg_pairs_hint, bool inverse);

// Test hook of the ordered in-place wait: counters needed (ints, zeroed by
// the caller) and the launch of one warp whose wait gives up after `limit`
// polls, raising kErrQueueTimeout into err.
int order_wait_timeout_words();
cudaError_t launch_order_wait_timeout(uint32_t limit, int *order, int *err, cudaStream_t stream);

// Launch one level on `stream`.  err: device error word (may be null).
cudaError_t launch_level(const LevelDesc &d, int wavelet, bool inverse, cudaStream_t stream,
                         int *err);

}  // namespace dwt
