// Candidate scoring of a descale sweep (score.cu): re-upscale each descaled
// plane with its plans' forward operators and reduce the mean absolute error
// against the source frame.
//
// The forward operator of an axis is A (source x destination), the matrix
// whose transpose the plan stores as a CSR by destination.  Upscaling a
// descaled plane Y (rows x cols) back to the source size is A_v * Y * A_h^T.
// One kernel computes, per column tile and segment of source rows, the row
// pass Z = Y * A_h^T for the descaled rows the segment needs (in shared
// memory), then A_v * Z, |. - frame| and one partial sum per block of 16
// rows.  Partial sums are reduced in a fixed order, so a score does not
// depend on launch shapes or on the other candidates of the sweep.
#pragma once

#include <cstdint>

namespace dsmvc_gb::dev {

// A as a CSR by source sample: entries (destination index, weight) in
// ascending destination order.
struct ForwardCsr {
    const std::uint32_t *offsets;   // source_size + 1
    const std::int32_t *indices;
    const float *weights;
};

struct ScoreJob {
    const float *descaled;          // rows x cols
    std::int64_t descaled_stride;
    std::int32_t rows, cols;
    const float *frame;             // height x width source plane
    std::int64_t frame_stride;
    std::int32_t width, height;
    ForwardCsr h, v;                // forward operators of the two axes
    float *partials;                // row blocks x column tiles
    float *score;                   // the candidate's score
    std::int32_t first_block;       // scoring blocks before this job
    std::int32_t segment_rows;      // source rows per scoring block (a multiple of kScoreRowBlock)
    std::int32_t column_tiles;      // ceil(width / kScoreThreads)
};

// Scoring fused into the columns pass of a candidate's descale (the
// chunk-delayed transposing kernel, tscore_impl.cuh): the descaled plane
// never leaves the chip.  Each CTA serves one tile of the candidate's
// descaled columns, [o_k, o_k + kScoreCtaThreads) with o_k = tile_origins[k],
// and owns the source columns s in [tile_sources[k], tile_sources[k + 1]),
// whose horizontal windows lie in those columns.  As the
// backward substitution finishes each chunk of 32 descaled rows, the
// source rows whose vertical window ends in that chunk are re-upscaled
// (vertical operator first, per descaled column, then the horizontal one
// across the tile) and compared with the frame.
//
// Operator rows are dense windows of 4 or 8 weights (zeros outside the
// CSR entries), 12 floats a row: [0] the window's first index (int bits),
// [1..3] 0, [4 .. 4 + taps) the weights in ascending index order.  A
// source row is re-upscaled after chunk q, the first chunk that holds its
// last entry and every earlier row's; its vertical window starts at
// min(first entry, 32 q + 32 - v_taps), so that it lies within the rows
// the kernel keeps (that chunk and the 6 rows before it).
struct ScoreEpilogue {
    const float *frame;             // height x width source plane
    std::int64_t frame_stride;
    std::int32_t width, height;
    const float *v_rows;            // height rows of 12 floats
    const std::int32_t *v_emit;     // per chunk q: end of the source rows emitted after it
    const float *h_cols;            // width rows of 12 floats
    const std::int32_t *tile_sources;   // tiles + 1 source column bounds
    const std::int32_t *tile_origins;   // tiles first descaled columns
    std::int32_t v_taps, h_taps;    // 4 or 8
    std::int32_t tiles;
    double *partials;               // per tile: the sum of |re-upscaled - frame|
    float *score;                   // sum of partials / (width * height)
};

} // namespace dsmvc_gb::dev

namespace dsmvc_gb {

constexpr int kScoreThreads = 256;
constexpr int kScoreRowBlock = 16;   // rows per partial sum
constexpr int kScoreSegmentEntries = 2048;   // A_v entries of a segment staged in shared memory
constexpr int kScoreMaxSegmentRows = 256;    // rows of a segment whose entry ranges are staged

// Fused re-upscale + absolute error: one block per (column tile, row
// segment); `max_span_rows` bounds the descaled rows any segment touches
// (their row-pass values are staged in shared memory).
int launch_score_tiles(const dev::ScoreJob *jobs, int job_count, int total_blocks, int max_span_rows,
                       void *stream);
// *jobs[i].score = sum of job i's partials / (width * height), one block
// per job, in a fixed order.
int launch_score_finalize(const dev::ScoreJob *jobs, int job_count, void *stream);

// Fused scoring (ScoreEpilogue): CTA size, descaled rows kept per lane (a
// chunk and the 6 rows before it), the widest vertical window this admits,
// source rows per re-upscale batch.
constexpr int kScoreCtaThreads = 128;
constexpr int kScoreRingRows = 38;
constexpr int kScoreMaxVerticalTaps = 7;
constexpr int kScoreMaxHorizontalTaps = 8;
constexpr int kScoreBatchRows = 8;
// *epilogues[i].score = its partials' sum / (width * height), in a fixed
// order; one block per epilogue.
int launch_fused_score_finalize(const dev::ScoreEpilogue *epilogues, int count, void *stream);

} // namespace dsmvc_gb
