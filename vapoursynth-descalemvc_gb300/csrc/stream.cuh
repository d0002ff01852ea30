// Packed plan records and jobs of the streaming axis kernels (stream.cu).
#pragma once

#include "kernels.cuh"

#include <cstdint>

namespace dsmvc_gb::dev {

// Per-destination records, all float-aligned to 16 bytes:
//   forward[j * forward_stride + ...]:
//     [0] window start s0 (int bits), [1] inverse diagonal,
//     [2] (s0 mod 32) * kTRingPitch (int bits), [3] 0,
//     [4 .. 4+window)  A^T weights of sources s0 .. s0+window-1 (0 where
//                      the source does not contribute),
//     [4+window ..)    forward factors -lower_ld for d = HB..1 (0 for d > j),
//                      padded to a multiple of 4;
//   backward[j * backward_stride + ...]: upper_l in use order (d = 1..3 for
//     half-bandwidth 3, d = HB..1 otherwise; 0 beyond the vector end),
//     padded to a multiple of 4.
struct StreamPlanView {
    std::int32_t source_size;
    std::int32_t destination_size;
    std::int32_t half_bandwidth;
    std::int32_t window;            // multiple of 4
    std::int32_t forward_stride;    // floats
    std::int32_t backward_stride;   // floats
    const float *forward;
    const float *backward;
};

struct StreamJob {
    StreamPlanView plan;
    const void *in;
    std::int64_t in_elem, in_vec;
    void *out;
    std::int64_t out_elem, out_vec;
    std::int32_t vectors;
    std::int32_t first_block;       // transposing kernels: the job's first warp
    Conversion conv;
    // Two-pass transposing kernels: the Float32 forward-value plane, laid
    // out like `out` (destination j of vector v at y[j * y_elem + v]).
    float *y;
    std::int64_t y_elem;
    // Chunk-delayed transposing kernels: the job's destinations are chunks
    // [chunk_begin, chunk_end) of its vectors (chunk_end 0: all of them).
    // A job starting past chunk 0 runs its forward substitution from chunk
    // chunk_begin - 1 with a zero history, its ring from sample first_sample
    // (a multiple of 16, at most that chunk's first window start), and stores
    // nothing of that chunk; one ending before the last chunk also runs the
    // forward substitution and backward warm-up of chunk chunk_end.  Every
    // warp of a CTA serves the same plan and chunk range.
    std::int32_t chunk_begin;
    std::int32_t chunk_end;
    std::int32_t first_sample;
    // Float64 two-pass kernels: a segment's forward and backward margins, in
    // chunks (StreamPack64::margin); such a segment sweeps forward from
    // `margin` chunks before its range (zero history, ring from first_sample)
    // and backward from `margin` chunks after it (zero carry), within the
    // vector, storing its forward values from its first computed chunk on
    // at y (rows of y_elem).
    std::int32_t margin;
    // Columns passes with fused candidate scoring (tscore_impl.cuh): the
    // device ScoreEpilogue (score.cuh); the pass then stores no output.
    const void *score;
    // Transposing kernels: the status word a stalled feed wait sets
    // (kStatusFeedStall).
    std::uint32_t *status;
    // Nonzero: the staged feed waits for a barrier phase nothing completes,
    // so that its bounded wait runs out (tests of the stall report).
    std::int32_t feed_stall_test;
};

} // namespace dsmvc_gb::dev

namespace dsmvc_gb {

int stream_threads();
bool stream_supports(int half_bandwidth);
constexpr int kStreamChunk = 32;     // destinations per register chunk
constexpr int kStreamRing = 32;      // source samples held per thread
// Ring row pitches (floats) of the transposing kernels, unpaired and paired;
// the host stores each destination's window offset in the ring, (s0 mod 32)
// times the pitch (in floats, resp. float2 for the paired kernels), in its
// forward record.
constexpr int kTRingPitch = 34;
constexpr int kPairedRingPitch = 66;
// `chunk` is 32 or 64; contiguous = the vector's samples are adjacent
// (rows: f32/u8/u16 in, f32 out); otherwise columns (f32 in; f32/u8/u16 out).
// Transposing 2D passes (tstream_impl.cuh): vectors with adjacent samples
// in, destination-major output with the vectors adjacent.  Every job of one
// launch has the same window when window == 8 (unrolled gather); window 12
// or 16: every job's plan view carries grouped records with that union
// (StreamPack::forward_groups).  `threads` per CTA: 32..256, a multiple of
// 32 (one warp per 32 vectors).
constexpr int kTStreamThreads = 128;   // default CTA size
constexpr int kTResidentWarps = 16;    // resident warps per SM (128 registers a thread)
constexpr int kMinSegmentChunks = 1;   // shortest segment, in chunks (StreamJob)
int launch_tstream(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads,
                   int half_bandwidth, int window, dev::Sample in, dev::Sample out, int record_floats,
                   void *stream);

// Paired transposing 2D passes (tstream2_impl.cuh): as launch_tstream with
// two vectors per thread (a CTA of `threads` covers 2 x threads vectors) and
// the plans' paired records; windows <= 16.
int launch_tstream2(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads,
                    int half_bandwidth, int window, dev::Sample in, dev::Sample out, int record_floats,
                    void *stream);

// Columns passes with fused candidate scoring (tscore_impl.cuh): as
// launch_tstream for Float32 intermediates with chunk-delayed records
// (window 0, 8, 12 or 16) and half-bandwidths 1..7, every job carrying a
// ScoreEpilogue (score.cuh) and starting on a CTA of kScoreCtaThreads
// threads, one CTA per tile; nothing is stored but the tiles' partials.
int launch_tscore(const dev::StreamJob *jobs, int job_count, int total_blocks, int half_bandwidth, int window,
                  int record_floats, void *stream);

// Two-pass transposing 2D passes (tsolve_impl.cuh): exact forward and
// backward sweeps through the jobs' forward-value planes; half-bandwidths
// 1..11 (odd).
bool tsolve_supports(int half_bandwidth);
int launch_tsolve(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads, int half_bandwidth,
                  int window, dev::Sample in, dev::Sample out, int record_floats, void *stream);

// Float64 two-pass transposing 2D passes (tsolve64_impl.cuh) for plans that
// retain Float64: the first pass reads u8/u16/f32 and writes the Float64
// intermediate, the second reads it and writes f32/u8/u16; the forward-value
// plane is Float64 (job.y as double); non-finite data sets `status` bits.
// `fused`: fused multiply-adds and the reciprocal pivot (<= 1 float32 ULP of
// the CPU route); otherwise the CPU scalar route's order, bit for bit.
int launch_tsolve64(const dev::StreamJob *jobs, int job_count, int total_blocks, int threads, int half_bandwidth,
                    dev::Sample in, dev::Sample out, int record_floats, bool fused, std::uint32_t *status,
                    void *stream);

// `record_floats`: the largest forward_stride + backward_stride of the jobs.
int launch_stream(const dev::StreamJob *jobs, int job_count, int total_blocks, int half_bandwidth,
                  int chunk, bool contiguous, dev::Sample in, dev::Sample out, int record_floats,
                  void *stream);

} // namespace dsmvc_gb
