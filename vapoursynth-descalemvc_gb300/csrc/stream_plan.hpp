// Host packing of an axis plan for the streaming kernels (stream_impl.cuh,
// tstream_impl.cuh, tstream2_impl.cuh) and the checks that admit a plan.
#pragma once

#include "planner.hpp"

#include <cstdint>
#include <string>
#include <vector>

namespace dsmvc_gb {

struct StreamPack {
    bool eligible = false;          // the plan may use the chunk-delayed streaming kernels
    bool exact = false;             // the plan may use the two-pass transposing kernels
                                    // (per-destination refill; grouped when ring_ok_transposed)
    std::string reason;             // why not chunk-delayed, when not
    int window = 0;                 // dense gather window (multiple of 4)
    int forward_stride = 0;         // floats per forward record
    int backward_stride = 0;        // floats per backward record
    // Ring capacity holds for 16-byte row loads of f32 (4 samples), u16 (8)
    // and u8 (16) rows; column loads fetch 4 rows at a time (as f32 rows).
    bool ring_ok_f32 = false;
    bool ring_ok_u16 = false;
    bool ring_ok_u8 = false;
    // The transposing 2D kernels' warp-wide block feeding fits the ring.
    bool ring_ok_transposed = false;
    double backward_transfer = 0.0; // max |carry -> state| over one chunk
    // Segments: a transposing 2D pass may split its vectors' destinations
    // into ranges of whole chunks served by different warps, each starting
    // its forward substitution from a zero history one chunk early.  Admitted
    // when that warm-up leaves a history influence below 2^-26 per slot
    // (every chunk that can serve as warm-up, computed in double).
    // Grouped forward records of the chunk-delayed transposing kernels
    // (tstream_impl.cuh, K = group_union), when the window starts of every
    // four consecutive destinations 4g..4g+3 span at most 12 (or 16) samples
    // together with the window: per group, [window start of 4g, its ring
    // offset, end of the union actually needed (the refill target), 0],
    // the four inverse diagonals, the four windows' weights each laid over
    // the union (zeros outside their own window), then the four records'
    // lower factors back to back (use order d = hb..1), padded to 4.
    int group_union = 0;            // 12 or 16; 0 when not grouped
    int group_stride = 0;           // floats per group: 8 + 4 union + round4(4 hb)
    std::vector<float> forward_groups;
    // Their backward records: per group, the four records' hb factors back
    // to back (use order), padded to 4 (round4(4 hb) floats a group).
    std::vector<float> backward_groups;
    bool segmentable = false;
    double forward_transfer = 0.0;  // max |history -> state| over one chunk
    // Segments of the two-pass transposing kernels (exact plans): forward
    // sweep from `exact_margin` chunks before a range (zero history),
    // backward sweep from as many after it (zero carry), within the vector;
    // the smallest margin of 1..4 chunks leaving below 2^-26 of a unit
    // history or carry from every chunk boundary (in double), 0 when none.
    int exact_margin = 0;
    double exact_margin_transfer = 0.0;
    // Window start of each chunk's first destination, rounded down to the
    // 16-sample feeding block: where a segment's warm-up starts its ring.
    std::vector<int> chunk_first_block;
    // Records of ceil(destination_size / chunk) * chunk destinations (zero
    // records past the end).
    std::vector<float> forward;     // * forward_stride
    std::vector<float> backward;    // * backward_stride
    // Records of the paired 2D kernels (tstream2_impl.cuh), when the window
    // is at most 16 and the transposing feed fits: every coefficient twice,
    // backward factors negated.
    bool paired = false;
    int paired_forward_stride = 0;  // 4 + 2 window + round4(2 hb)
    int paired_backward_stride = 0; // round4(2 hb)
    std::vector<float> paired_forward;
    std::vector<float> paired_backward;
};

// `chunk` destinations per register chunk, `ring` source samples held per
// thread.  A plan is eligible when its half-bandwidth has a kernel, its
// dense window fits the ring, the window starts never move backwards, and
// the zero-carry backward warm-up over one chunk leaves a carry influence
// below 2^-26 per carry slot (computed in double for every chunk of the
// plan), which keeps the warm-up error within about one float ULP.
// Records are built when either family admits the plan; the two-pass
// transposing kernels (tsolve_impl.cuh) need only the window, monotone
// window starts and the grouped ring replay.
StreamPack pack_stream_plan(const AxisPlan &plan, int chunk, int ring,
                            bool half_bandwidth_supported, bool half_bandwidth_supported_exact = false);

// Records of the Float64 two-pass transposing kernels (tsolve64_impl.cuh)
// for plans that retain Float64: window up to 16 samples, monotone window
// starts, the per-destination ring replay in blocks of 16.  Forward record
// (doubles): [s0 | count << 32 (bits), D + DBL_EPSILON, 1 / (D + DBL_EPSILON),
// window weights (count from s0), L(i, i - d) for d = hb..1]; backward
// record: L(i + d, i) for d = hb..1; both padded to an even number of
// doubles.  Strides are in floats (the staging copies floats).
struct StreamPack64 {
    bool eligible = false;
    int window = 0;
    int forward_stride = 0;
    int backward_stride = 0;
    std::vector<double> forward;
    std::vector<double> backward;
    // Segments (chunk ranges served by separate warps): a segment runs its
    // forward sweep from `margin` chunks before its range (zero history) and
    // its backward sweep from as many chunks after it (zero carry).
    // Admitted with the smallest margin of 2..4 chunks that, in double,
    // leaves an influence below 2^-60 of a unit history or carry from every
    // chunk boundary.
    bool segmentable = false;
    int margin = 0;                       // chunks
    double margin_transfer = 0.0;         // at that margin (at 4 when none)
    std::vector<int> chunk_first_block;   // window start of each chunk, rounded down to 16
};
StreamPack64 pack_stream_plan64(const AxisPlan &plan, int chunk, int ring, bool half_bandwidth_supported);

} // namespace dsmvc_gb
