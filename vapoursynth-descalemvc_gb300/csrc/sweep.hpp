// Batched candidate sweep: many 2D descales of one source frame (one per
// candidate geometry and kernel), each re-upscaled and scored by its mean
// absolute error against the frame, all enqueued as one CUDA graph.
//
// This is the GPU-resident form of the reference's native-resolution scan,
// where every candidate is a separate Descale call followed by a resize
// back to the source size and a PlaneStats-style average
// (docs/release-benchmark.md, "getfnative" case).  Here the candidates are
// packed into waves that fit a device-memory budget; each wave is one
// prepared batch (every descale of the wave in one launch per pass) and the
// waves share their buffers.  Each candidate is descaled to HBM and scored
// by two more launches (a re-upscale and error sum, then the reduction),
// or, with fused scoring, where its columns pass runs the chunk-delayed
// kernel and its operators fit the fused windows, scored inside that pass
// (tscore_impl.cuh: its descaled plane never leaves the chip) and reduced
// by one finalize launch.  CTA sizes of the tunable launch groups and the row segment
// of the separate scoring pass are chosen by timing the alternatives on the
// first wave (autotuning).  Scores do not depend on the chosen launch
// shapes: each candidate's arithmetic is the same whatever its wave, CTA
// size or neighbours.
#pragma once

#include "executor.hpp"
#include "planner.hpp"

#include <array>
#include <cstddef>
#include <memory>
#include <utility>
#include <vector>

namespace dsmvc_gb {

struct SweepOptions {
    std::size_t memory_budget = 0;   // bytes per wave; 0 = 32 GiB
    bool autotune = true;
    bool graph = true;
    // Score in the columns pass where the candidate allows it (the descaled
    // plane never reaches HBM: one wave where the separate scoring needs
    // several); otherwise every candidate is descaled to HBM and scored by a
    // kernel of its own (faster on a 1503-candidate 1080p sweep: the fused
    // pass couples the scoring to the substitution's 168-register warps).
    bool fused_scoring = false;
};

struct SweepInfo {
    int candidates = 0;
    int waves = 0;
    std::size_t device_bytes = 0;     // buffers owned by the sweep
    std::size_t kernel_launches = 0;  // per run()
    double tune_milliseconds = 0.0;
    int segment_rows = 0;
    int vectors_per_warp = 32;        // chosen right-hand sides per warp (32 or 64)
    int fused_candidates = 0;         // scored inside their columns pass
    BatchTuning tuning;               // chosen CTA sizes per launch group
};

class Sweep {
public:
    // `frame` is a device plane of horizontal source size x vertical source
    // size Float32 samples, `frame_stride` samples apart; every candidate's
    // plans (horizontal, vertical) must have those source sizes.  The frame
    // must outlive the sweep.
    using Candidate = std::pair<std::shared_ptr<const AxisPlan>, std::shared_ptr<const AxisPlan>>;
    Sweep(Executor &executor, const std::vector<Candidate> &candidates, const float *frame,
          std::ptrdiff_t frame_stride, const SweepOptions &options);
    ~Sweep();
    Sweep(const Sweep &) = delete;
    Sweep &operator=(const Sweep &) = delete;

    // Enqueues the whole sweep on `stream` (one graph launch with graphs on).
    void run(void *stream);
    // The same work one candidate at a time, each descale submitted as its
    // own call and waited for (the per-frame baseline).
    void run_plain(void *stream);
    // Waits for `stream` and copies the scores (candidate order) to `host`.
    void read_scores(float *host, void *stream);
    // Runs the sweep once without the graph, with CUDA events between its
    // stages, and returns their milliseconds: descale passes, re-upscale
    // with the error sums, score reduction.
    [[nodiscard]] std::array<double, 3> stage_milliseconds(void *stream);
    [[nodiscard]] const float *device_scores() const;
    [[nodiscard]] SweepInfo info() const;

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace dsmvc_gb
