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
    const float *in[4];
    long long in_pitch[4];
    float *out[4];
    long long out_pitch[4];
};

// Tensor maps of an inverse level: the LL band (box kBandRowF x 2) and the
// coefficient frame holding HL, LH, HH (the level's w x h region, same box).
struct LevelMaps {
    CUtensorMap ll;
    CUtensorMap frame;
};

// Fills n_strips / seg_pairs / n_segs for a level of size w x h (the
// segment length depends on the direction).
void plan_level(LevelDesc &d, int seg_pairs_hint, bool inverse);

// Launch one level on `stream`.  err: device error word (may be null).
cudaError_t launch_level(const LevelDesc &d, int wavelet, bool inverse, cudaStream_t stream,
                         int *err);

}  // namespace dwt
