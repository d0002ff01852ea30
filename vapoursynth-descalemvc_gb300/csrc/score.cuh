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
    std::int32_t first_block;       // scoring blocks before this job
    std::int32_t segment_rows;      // source rows per scoring block (a multiple of kScoreRowBlock)
    std::int32_t column_tiles;      // ceil(width / kScoreThreads)
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
// scores[i] = sum of job i's partials / (width * height), one block per job,
// in a fixed order.
int launch_score_finalize(const dev::ScoreJob *jobs, int job_count, float *scores, void *stream);

} // namespace dsmvc_gb
