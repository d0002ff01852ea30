// Transposing streaming kernels: the two passes of a 2D descale.
//
// Both passes read vectors whose samples are contiguous (rows of the input
// plane; columns of the transposed intermediate) and write their results
// transposed, destination-major with the vectors contiguous (the first pass
// writes the intermediate column-major, the second writes the output plane
// row-major).  A warp owns 32 vectors, one per lane:
//
//  * Loads: blocks of 16 source samples of all 32 vectors are fetched by the
//    whole warp with 16-byte coalesced cp.async copies (2 lanes per u16
//    vector, 4 per f32 vector, 1 per u8 vector) into the warp's staging area
//    in shared memory, completed on the warp's mbarrier; each lane then
//    converts the bytes it copied to float and scatters them into a shared
//    ring of 32 sample rows whose first 16 rows are stored again after it,
//    so that any window of up to 16 consecutive samples is contiguous (the
//    host admits windows up to 16).  Rows are 34 floats apart: the scatter of
//    every load pattern and the per-lane reads of one sample row are both
//    free of bank conflicts.  The next block is in flight while the current
//    one is consumed, in shared memory rather than in registers (on one
//    GB300: 64 YUV420P16 1080p frames to 810p, 0.796 -> 0.771 ms a batch;
//    32 4K Debicubic planes, 1.034 -> 1.023 ms).
//  * Stores: destination j of the 32 vectors is one coalesced store.
//  * Records: the CTA's warps work on the same destinations, so one
//    chunk of 32 destination records is copied (cp.async) into shared memory
//    for all of them, three chunks deep, behind a barrier per chunk.
//  * Arithmetic: as in stream_impl.cuh -- exact forward substitution in the
//    reference CUDA order, chunk-delayed backward substitution with a
//    zero-carry warm-up over the following chunk (admitted per plan by the
//    host), no forward value written to memory.  The destination loop of a
//    chunk is branch-free: samples are fetched once per four destinations
//    and destinations past the end are computed as zeros and not stored.
#pragma once

#include "kernels.cuh"
#include "smem_limit.cuh"
#include "stream.cuh"

#include <cuda_runtime.h>

#include <cstdint>

namespace dsmvc_gb {
namespace {

using dev::Conversion;
using dev::StreamJob;

constexpr int kTRing = kStreamRing;        // sample rows per ring
constexpr int kTPitch = kTRingPitch;       // floats between ring rows
constexpr int kTDup = 16;                  // leading rows stored again after the ring
constexpr int kTRingFloats = (kTRing + kTDup) * kTPitch;
constexpr int kTChunk = kStreamChunk;
constexpr int kTMaxThreads = 256;         // CTA sizes 32..256 (a multiple of 32)
constexpr int kTBlock = 16;                // samples per warp load block
// Staged feeds: per warp after the rings, up to 4 copies of 16 bytes a lane.
constexpr int kFeedWarpBytes = 4 * 32 * 16;
// try_wait rounds before a feed wait gives up, each suspending at most
// kFeedWaitSuspendNs (about 65 ms in all, far beyond any copy's latency); a
// stalled warp stops waiting and its kernel reports kStatusFeedStall.
constexpr int kFeedWaitRounds = 1 << 16;
constexpr unsigned kFeedWaitSuspendNs = 1000;

__device__ __forceinline__ int find_tjob(const StreamJob *jobs, int count, int block) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_block <= block) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void tcp_async16(float *smem, const float *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void tcp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void tcp_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <class T> __device__ __forceinline__ float tin(T v, const Conversion &c) {
    return (static_cast<float>(v) - c.in_offset) * c.in_scale;
}
template <> __device__ __forceinline__ float tin<float>(float v, const Conversion &) { return v; }

template <class T> __device__ __forceinline__ T tout(float v, const Conversion &c) {
    float s = __fadd_rn(__fmul_rn(v, c.out_scale), c.out_offset);
    s = fminf(fmaxf(s, 0.0f), static_cast<float>(c.out_max));
    return static_cast<T>(__float2uint_rn(s));
}
template <> __device__ __forceinline__ float tout<float>(float v, const Conversion &) { return v; }

__device__ __forceinline__ float4 tlds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// Predicated global stores of one output sample: no branch around the
// store, and the address is known to be global.  No memory clobber: the
// kernels never read what they store through these (outputs only), and the
// compiler stays free to move shared-memory loads across the stores.
__device__ __forceinline__ void tst(float *p, float v, bool pred) {
    asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %2, 0;\n @q st.global.f32 [%0], %1;\n}\n"
                 :: "l"(p), "f"(v), "r"(static_cast<int>(pred)));
}
__device__ __forceinline__ void tst(std::uint16_t *p, std::uint16_t v, bool pred) {
    asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %2, 0;\n @q st.global.u16 [%0], %1;\n}\n"
                 :: "l"(p), "h"(v), "r"(static_cast<int>(pred)));
}
__device__ __forceinline__ void tst(std::uint8_t *p, std::uint8_t v, bool pred) {
    asm volatile("{\n .reg .pred q;\n setp.ne.b32 q, %2, 0;\n @q st.global.u8 [%0], %1;\n}\n"
                 :: "l"(p), "r"(static_cast<unsigned>(v)), "r"(static_cast<int>(pred)));
}

// Record strides (floats).  With a compile-time window they are constants,
// so every record read is an immediate offset from the chunk's base.
// K: 0 runtime window, 8 window-8 gather, 12 and 16 grouped gather over a
// union of K samples (StreamPack::forward_groups; the stride is then a
// group's floats over 4).
template <int HB, int K> __device__ __forceinline__ int fwd_stride(const dev::StreamPlanView &p) {
    if constexpr (K > 8) return (8 + 4 * K + (4 * HB + 3) / 4 * 4) / 4;
    return K > 0 ? 4 + K + (HB + 3) / 4 * 4 : p.forward_stride;
}
// Backward records: per destination (round4(hb) floats, at least 4), or for
// grouped records (K > 8) per group of four destinations, their hb
// coefficients back to back padded to 4 (StreamPack::backward_groups).
template <int HB, int K> __device__ __forceinline__ int bwd_stride(const dev::StreamPlanView &p) {
    if constexpr (K > 8) return (4 * HB + 3) / 4;
    return K > 0 ? ((HB + 3) / 4 * 4 < 4 ? 4 : (HB + 3) / 4 * 4) : p.backward_stride;
}

// Cooperative ring feeder of one warp.  Block b covers samples
// [16 b, 16 b + 16) of the warp's 32 vectors.  STAGED: the block in flight
// waits in shared memory (cp.async, completed on the warp's mbarrier, which
// takes 32 arrivals a phase); otherwise in registers (the two-pass and
// fused scoring kernels, whose occupancy the staging area would cut).
template <class In, bool STAGED = true>
struct WarpFeeder {
    static constexpr int SPL = 16 / static_cast<int>(sizeof(In));   // samples per lane load
    static constexpr int LPV = kTBlock / SPL;                       // lanes per vector
    static constexpr int VPI = 32 / LPV;                            // vectors per load
    static constexpr int NI = 32 / VPI;                             // loads per block
    const In *base;          // vector 0 of the warp
    std::int64_t stride;     // samples between vectors
    int size;                // samples per vector
    int have;                // samples in the ring
    int vectors;             // valid vectors of the warp (>= 1)
    bool vec_ok;             // 16-byte aligned vectors
    int lane;
    float *ring;             // warp ring, ring[row * kTPitch + vector]
    Conversion conv;
    uint4 pend[STAGED ? 1 : NI];   // register feeds: the block in flight
    uint4 *stage;            // staged feeds: NI x 32 lanes x 16 bytes of this warp
    unsigned long long *mbar;   // staged feeds: this warp's completion barrier
    unsigned phase;
    bool failed;             // a wait ran out: later blocks are not waited for
    bool pend_ok;

    __device__ __forceinline__ void put(int s, int v, float x) {
        const int row = s & (kTRing - 1);
        float *r = ring + row * kTPitch + v;
        r[0] = x;
        if (row < kTDup) r[kTRing * kTPitch] = x;
    }

    __device__ __forceinline__ void issue() {
        pend_ok = vec_ok && have + kTBlock <= size;
        if (!pend_ok) return;
#pragma unroll
        for (int i = 0; i < NI; ++i) {
            int v = i * VPI + lane / LPV;
            v = v < vectors ? v : vectors - 1;
            const In *p = base + v * stride + have + (lane % LPV) * SPL;
            if constexpr (STAGED) {
                const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(stage + i * 32 + lane));
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(sa), "l"(p) : "memory");
            } else {
                pend[i] = __ldg(reinterpret_cast<const uint4 *>(p));
            }
        }
        if constexpr (STAGED) {
            // One arrival per lane once its copies have landed.
            const unsigned mb = static_cast<unsigned>(__cvta_generic_to_shared(mbar));
            asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" :: "r"(mb) : "memory");
        }
    }

    // `first`: a multiple of 16 at most the first window start.
    __device__ __forceinline__ void start(int first = 0) {
        have = first;
        issue();
    }

    // Makes samples [0, need) resident (need <= size) and visible warp-wide.
    __device__ __forceinline__ void ensure(int need) {
        if (have >= need) return;
        while (have < need) {
            if (pend_ok) {
                // A block starts on a multiple of 16, so a lane's SPL samples
                // occupy consecutive ring rows without wrapping, and all of
                // the block is in the duplicated rows or none of it is.
                const bool dup = (have & (kTRing - 1)) < kTDup;
                if constexpr (STAGED) {
                    if (!failed) {
                        const unsigned mb = static_cast<unsigned>(__cvta_generic_to_shared(mbar));
                        unsigned done = 0;
                        for (int it = 0; it < kFeedWaitRounds && !done; ++it) {
                            asm volatile("{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2, %3;\n"
                                         " selp.u32 %0, 1, 0, q;\n}\n"
                                         : "=r"(done) : "r"(mb), "r"(phase), "r"(kFeedWaitSuspendNs) : "memory");
                        }
                        failed = !done;
                    }
                    phase ^= 1u;
                }
#pragma unroll
                for (int i = 0; i < NI; ++i) {
                    const int v = i * VPI + lane / LPV;
                    uint4 staged;                               // the bytes this lane fetched
                    if constexpr (STAGED) staged = stage[i * 32 + lane];
                    else staged = pend[i];
                    const In *vals = reinterpret_cast<const In *>(&staged);
                    float *r = ring + ((have + (lane % LPV) * SPL) & (kTRing - 1)) * kTPitch + v;
#pragma unroll
                    for (int k = 0; k < SPL; ++k) {
                        const float x = tin(vals[k], conv);
                        r[k * kTPitch] = x;
                        if (dup) r[(kTRing + k) * kTPitch] = x;
                    }
                }
                have += kTBlock;
                issue();
            } else {
                // Unaligned vectors or the tail: each lane loads its own
                // vector's next sample.
                const int v = lane < vectors ? lane : vectors - 1;
                put(have, lane, tin(__ldg(base + v * stride + have), conv));
                have += 1;
            }
        }
        __syncwarp();
    }
};

__device__ __forceinline__ void tstage(float *buf, const dev::StreamPlanView &p, int chunk, int tid,
                                       int nthreads) {
    const int fs = p.forward_stride, bs = p.backward_stride;
    const float *gf = p.forward + static_cast<std::int64_t>(chunk) * kTChunk * fs;
    const float *gb = p.backward + static_cast<std::int64_t>(chunk) * kTChunk * bs;
    for (int i = tid * 4; i < kTChunk * fs; i += nthreads * 4) tcp_async16(buf + i, gf + i);
    float *bb = buf + kTChunk * fs;
    for (int i = tid * 4; i < kTChunk * bs; i += nthreads * 4) tcp_async16(bb + i, gb + i);
}

// Forward substitution of chunk destinations [j0, j0 + LC) into y[LC + t].
template <int HB, int LC, int K, class Feed>
__device__ __forceinline__ void tforward(float (&y)[2 * LC], int j0, const dev::StreamPlanView &p,
                                         const float *fwd, Feed &feed, int lane) {
    const int fs = fwd_stride<HB, K>(p);
    const int kw = K > 0 ? K : p.window;
    const int n = p.destination_size;
#pragma unroll
    for (int t = 0; t < LC; ++t) {
        if (t % 4 == 0) {
            // Window end of the group's last destination: window starts
            // never decrease, records past the end of the vector repeat the
            // last destination's start, and no window ends past the source.
            feed.ensure(__float_as_int(fwd[(t + 3) * fs]) + kw);
        }
        const float *rec = fwd + t * fs;
        const float4 hdr = tlds4(rec);
        // Record word 2: the window's ring offset, (s0 mod 32) * kTPitch.
        const float *win = feed.ring + lane + __float_as_int(hdr.z);
        // Two interleaved partial sums (even and odd taps) halve the gather's
        // dependency chain.
        float se = 0.0f, so = 0.0f;
        if constexpr (K > 0) {
#pragma unroll
            for (int k = 0; k < K; k += 4) {
                const float4 w = tlds4(rec + 4 + k);
                se = fmaf(w.x, win[(k + 0) * kTPitch], se);
                so = fmaf(w.y, win[(k + 1) * kTPitch], so);
                se = fmaf(w.z, win[(k + 2) * kTPitch], se);
                so = fmaf(w.w, win[(k + 3) * kTPitch], so);
            }
        } else {
            for (int k = 0; k < kw; k += 4) {
                const float4 w = tlds4(rec + 4 + k);
                se = fmaf(w.x, win[(k + 0) * kTPitch], se);
                so = fmaf(w.y, win[(k + 1) * kTPitch], so);
                se = fmaf(w.z, win[(k + 2) * kTPitch], se);
                so = fmaf(w.w, win[(k + 3) * kTPitch], so);
            }
        }
        float sum = se + so;
        const float *low = rec + 4 + kw;
#pragma unroll
        for (int q = 0; q < HB; q += 4) {
            const float4 l = tlds4(low + q);
            const float lv[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int d = HB - (q + e);
                if (d >= 1) sum = fmaf(lv[e], y[LC + t - d], sum);
            }
        }
        // Records past the end of the vector are zero (inverse diagonal
        // included), so their forward values are zero for finite data.
        y[LC + t] = sum * hdr.y;
    }
}

// Forward substitution of a chunk with grouped records: per group of four
// destinations the union of their windows (U = K ring rows from the first
// window's start) is read once, and each destination's weights, laid over
// the union with zeros outside its window, apply as packed float2 FMAs
// over pairs of union samples (even and odd union taps in the two halves,
// then their sum -- the zeros add nothing, so each destination's gather
// equals the per-destination one).  Rows of the union past the refill
// target hold earlier finite samples or the ring's initial zeros.
template <int HB, int LC, int U, class Feed>
__device__ __forceinline__ void tforward_grouped(float (&y)[2 * LC], const float *fwd, Feed &feed, int lane) {
    constexpr int GS = 8 + 4 * U + (4 * HB + 3) / 4 * 4;   // floats per group
#pragma unroll
    for (int t = 0; t < LC; t += 4) {
        const float *gr = fwd + (t / 4) * GS;
        const float4 h = tlds4(gr);
        feed.ensure(__float_as_int(h.z));
        const float *win = feed.ring + lane + __float_as_int(h.y);
        float x[U];
#pragma unroll
        for (int i = 0; i < U; ++i) x[i] = win[i * kTPitch];
        const float4 inv = tlds4(gr + 4);
        float g[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int i = 0; i < U; i += 4) {
                const float4 w = tlds4(gr + 8 + q * U + i);
                acc = __ffma2_rn(make_float2(w.x, w.y), make_float2(x[i], x[i + 1]), acc);
                acc = __ffma2_rn(make_float2(w.z, w.w), make_float2(x[i + 2], x[i + 3]), acc);
            }
            g[q] = acc.x + acc.y;
        }
        float lw[(4 * HB + 3) / 4 * 4];
#pragma unroll
        for (int i = 0; i < (4 * HB + 3) / 4 * 4; i += 4) {
            const float4 l = tlds4(gr + 8 + 4 * U + i);
            lw[i] = l.x;
            lw[i + 1] = l.y;
            lw[i + 2] = l.z;
            lw[i + 3] = l.w;
        }
        const float iv[4] = {inv.x, inv.y, inv.z, inv.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float sum = g[q];
#pragma unroll
            for (int e = 0; e < HB; ++e) {
                const int d = HB - e;                  // use order d = hb..1
                sum = fmaf(lw[q * HB + e], y[LC + t + q - d], sum);
            }
            // Records past the end of the vector are zero (inverse diagonal
            // included), so their forward values are zero for finite data.
            y[LC + t + q] = sum * iv[q];
        }
    }
}

// The backward coefficients (use order) of destination t of a chunk, with
// t visited in descending order: a group's are loaded at its last member.
template <int HB, int K> struct TBackCoeffs {
    static constexpr int N = K > 8 ? (4 * HB + 3) / 4 * 4 : (HB + 3) / 4 * 4;
    float v[N];
    __device__ __forceinline__ void at(const float *bwd, int bs, int t) {
        if (K > 8 && t % 4 != 3) return;
        const float *rec = K > 8 ? bwd + (t / 4) * N : bwd + t * bs;
#pragma unroll
        for (int i = 0; i < N; i += 4) {
            const float4 u = tlds4(rec + i);
            v[i] = u.x;
            v[i + 1] = u.y;
            v[i + 2] = u.z;
            v[i + 3] = u.w;
        }
    }
    __device__ __forceinline__ float operator()(int t, int pos) const { return v[K > 8 ? (t % 4) * HB + pos : pos]; }
};

// Zero-carry backward warm-up over the chunk held in y[LC, 2 LC); leaves the
// state entering the preceding chunk in `carry`.
template <int HB, int LC, int K>
__device__ __forceinline__ void twarmup(const float (&y)[2 * LC], float (&carry)[HB],
                                        const dev::StreamPlanView &p, const float *bwd) {
    const int bs = bwd_stride<HB, K>(p);
    float w[HB];
#pragma unroll
    for (int d = 0; d < HB; ++d) w[d] = 0.0f;
    TBackCoeffs<HB, K> u;
#pragma unroll
    for (int t = LC - 1; t >= 0; --t) {
        u.at(bwd, bs, t);
        float sum = 0.0f;
#pragma unroll
        for (int pos = 0; pos < HB; ++pos) {
            const int d = HB == 3 ? pos + 1 : HB - pos;
            // x_{t+d} beyond the chunk is the zero carry.
            const float xd = (t + d < LC) ? w[(t + d) % HB] : 0.0f;
            sum = fmaf(u(t, pos), xd, sum);
        }
        w[t % HB] = y[LC + t] - sum;
    }
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = w[d];
}

// Final backward substitution of the chunk held in y[B, B + LC) from
// `carry` (x after the chunk); each x is stored as soon as it is known.
// Leaves the chunk's first HB x values in `carry`.  B == 0: a chunk before
// the vector's last, every destination valid; B == LC: the last chunk,
// destinations past the vector's end not stored.
template <int HB, int LC, int K, int B, class Out>
__device__ __forceinline__ void tbackward(float (&y)[2 * LC], float (&carry)[HB], int j0,
                                          const dev::StreamPlanView &p, const float *bwd, Out *out,
                                          std::int64_t out_elem, bool active, const Conversion &conv) {
    const int bs = bwd_stride<HB, K>(p);
    const int valid = B == 0 ? LC : p.destination_size - j0;
    Out *o = out + static_cast<std::int64_t>(j0 + LC - 1) * out_elem;
    TBackCoeffs<HB, K> u;
#pragma unroll
    for (int t = LC - 1; t >= 0; --t) {
        u.at(bwd, bs, t);
        float sum = 0.0f;
#pragma unroll
        for (int pos = 0; pos < HB; ++pos) {
            const int d = HB == 3 ? pos + 1 : HB - pos;
            const float xd = (t + d < LC) ? y[B + (t + d < LC ? t + d : 0)]
                                          : carry[t + d >= LC ? t + d - LC : 0];
            sum = fmaf(u(t, pos), xd, sum);
        }
        const float x = y[B + t] - sum;
        y[B + t] = x;
        tst(o, tout<Out>(x, conv), active && (B == 0 || t < valid));
        o -= out_elem;
    }
#pragma unroll
    for (int d = 0; d < HB; ++d) carry[d] = y[B + d];
}

// At most 128 registers a thread: 16 warps per SM.
template <int HB, int LC, int K, class In, class Out>
__global__ void __launch_bounds__(kTMaxThreads, 2 * 256 / kTMaxThreads)
tstream_kernel(const StreamJob *__restrict__ jobs, int job_count, int record_floats) {
    static_assert(LC == kTChunk, "record chunks and register chunks coincide");
    extern __shared__ __align__(16) float smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthreads = static_cast<int>(blockDim.x);
    // Jobs are assigned warps; a CTA's warps share one plan and one chunk
    // range (the host rounds changes of either up to whole CTAs), whose
    // records the CTA copies once.
    const int cta_warp = static_cast<int>(blockIdx.x) * (nthreads >> 5);
    const StreamJob &job = jobs[find_tjob(jobs, job_count, cta_warp + warp)];
    const StreamJob &lead = jobs[find_tjob(jobs, job_count, cta_warp)];
    const dev::StreamPlanView p = lead.plan;
    const int n = p.destination_size;
    const int chunks = (n + LC - 1) / LC;
    // Chunks whose outputs this CTA stores: [ca, cb).  The forward
    // substitution runs over [c0, ce]: from one chunk early (zero history)
    // for a range past chunk 0, to one chunk late (the backward warm-up of
    // the last stored chunk) for a range ending before the last chunk.
    const int ca = lead.chunk_begin;
    const int cb = lead.chunk_end > 0 ? lead.chunk_end : chunks;
    const int c0 = ca > 0 ? ca - 1 : 0;
    const int ce = cb < chunks ? cb : chunks - 1;
    const int per_buffer = kTChunk * record_floats;
    float *bufs = smem;
    float *ring = smem + 3 * per_buffer + warp * kTRingFloats;
    // The warp's feed staging area (after the rings) and mbarrier.
    uint4 *stage = reinterpret_cast<uint4 *>(reinterpret_cast<char *>(smem + 3 * per_buffer
                                                                      + (nthreads >> 5) * kTRingFloats)
                                             + warp * kFeedWarpBytes);
    __shared__ unsigned long long feed_bar[kTMaxThreads / 32];
    if (lane == 0) {
        const unsigned mb = static_cast<unsigned>(__cvta_generic_to_shared(&feed_bar[warp]));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 32;\n" :: "r"(mb) : "memory");
    }
    __syncwarp();

    // The warp's vectors; a warp past its job's last vector only takes part
    // in the CTA's record copies and barriers.
    int warp_first = (cta_warp + warp - job.first_block) * 32;
    int warp_vectors = job.vectors - warp_first;
    const bool idle = warp_vectors <= 0;
    if (warp_vectors <= 0) {
        warp_first = job.vectors - 1;
        warp_vectors = 1;
    } else if (warp_vectors > 32) {
        warp_vectors = 32;
    }
    const bool active = (cta_warp + warp - job.first_block) * 32 + lane < job.vectors;

    WarpFeeder<In> feed;
    feed.base = static_cast<const In *>(job.in) + warp_first * job.in_vec;
    feed.stride = job.in_vec;
    feed.size = p.source_size;
    feed.vectors = warp_vectors;
    feed.lane = lane;
    feed.ring = ring;
    feed.stage = stage;
    feed.mbar = &feed_bar[warp];
    // A stall test waits for the phase after the one the copies complete.
    feed.phase = lead.feed_stall_test ? 1u : 0u;
    feed.failed = false;
    feed.conv = job.conv;
    feed.vec_ok = (reinterpret_cast<std::uintptr_t>(job.in) % 16 == 0)
        && (job.in_vec * static_cast<std::int64_t>(sizeof(In))) % 16 == 0;
    if constexpr (K > 8) {
        // The grouped gather reads whole unions: every ring row starts finite.
        for (int i = lane; i < kTRingFloats; i += 32) ring[i] = 0.0f;
        __syncwarp();
    }
    if (!idle) feed.start(c0 > 0 ? lead.first_sample : 0);

    Out *out = static_cast<Out *>(job.out) + (warp_first + (lane < warp_vectors ? lane : 0));

    tstage(bufs + (c0 % 3) * per_buffer, p, c0, tid, nthreads);
    tcp_commit();
    if (c0 + 1 <= ce) tstage(bufs + ((c0 + 1) % 3) * per_buffer, p, c0 + 1, tid, nthreads);
    tcp_commit();

    float y[2 * LC];
    float carry[HB];
#pragma unroll
    for (int t = 0; t < LC; ++t) y[t] = 0.0f;
    for (int c = c0;; ++c) {
        tcp_wait_one();
        __syncthreads();
        const float *cur = bufs + (c % 3) * per_buffer;
        const float *prev = bufs + ((c + 2) % 3) * per_buffer;
        if (!idle) {
            if constexpr (K > 8) tforward_grouped<HB, LC, K>(y, cur, feed, lane);
            else tforward<HB, LC, K>(y, c * LC, p, cur, feed, lane);
            const float *cur_b = cur + kTChunk * fwd_stride<HB, K>(p);
            if (c + 1 == chunks) {
                // The vector's last chunk: exact backward substitution from
                // the end, stored when the chunk is the CTA's.
#pragma unroll
                for (int d = 0; d < HB; ++d) carry[d] = 0.0f;
                tbackward<HB, LC, K, LC>(y, carry, c * LC, p, cur_b, out, job.out_elem, active && c < cb,
                                         job.conv);
            } else if (c > ca) {
                twarmup<HB, LC, K>(y, carry, p, cur_b);
            }
            if (c > ca) {
                tbackward<HB, LC, K, 0>(y, carry, (c - 1) * LC, p, prev + kTChunk * fwd_stride<HB, K>(p), out,
                                        job.out_elem, active, job.conv);
            }
        }
        if (c == ce) break;
        // Every warp is done with chunk c-1's records: fetch chunk c+2.
        __syncthreads();
        if (c + 2 <= ce) tstage(const_cast<float *>(prev), p, c + 2, tid, nthreads);
        tcp_commit();
#pragma unroll
        for (int t = 0; t < LC; ++t) y[t] = y[LC + t];
    }
    // No copy is left in flight; a stalled feed wait reports.
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (__any_sync(0xffffffffu, feed.failed) && lane == 0) atomicOr(lead.status, dev::kStatusFeedStall);
}

template <int HB, int LC, int K, class In, class Out>
int tlaunch_typed(const StreamJob *jobs, int count, int blocks, int threads, int record_floats, cudaStream_t s) {
    if (threads < 32 || threads > kTMaxThreads || threads % 32) return static_cast<int>(cudaErrorInvalidValue);
    const int smem = (3 * kTChunk * record_floats + threads / 32 * kTRingFloats) * static_cast<int>(sizeof(float))
        + threads / 32 * kFeedWarpBytes;
    auto kernel = tstream_kernel<HB, LC, K, In, Out>;
    static SmemLimit limit;
    if (const cudaError_t e = limit.ensure(kernel, smem); e != cudaSuccess) return static_cast<int>(e);
    kernel<<<blocks, threads, smem, s>>>(jobs, count, record_floats);
    return static_cast<int>(cudaGetLastError());
}

template <int HB, int LC, int K>
int tlaunch_k(const StreamJob *jobs, int count, int blocks, int threads, dev::Sample in, dev::Sample out,
              int record_floats, cudaStream_t s) {
    using dev::Sample;
    if (in == Sample::f32 && out == Sample::f32)
        return tlaunch_typed<HB, LC, K, float, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::u16 && out == Sample::f32)
        return tlaunch_typed<HB, LC, K, std::uint16_t, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::u8 && out == Sample::f32)
        return tlaunch_typed<HB, LC, K, std::uint8_t, float>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::f32 && out == Sample::u16)
        return tlaunch_typed<HB, LC, K, float, std::uint16_t>(jobs, count, blocks, threads, record_floats, s);
    if (in == Sample::f32 && out == Sample::u8)
        return tlaunch_typed<HB, LC, K, float, std::uint8_t>(jobs, count, blocks, threads, record_floats, s);
    return static_cast<int>(cudaErrorInvalidValue);
}

// window == 8 has an unrolled gather; other windows loop.
template <int HB>
int tlaunch_hb(const StreamJob *jobs, int count, int blocks, int threads, int window, dev::Sample in,
               dev::Sample out, int record_floats, cudaStream_t s) {
    if (window == 8) return tlaunch_k<HB, kTChunk, 8>(jobs, count, blocks, threads, in, out, record_floats, s);
    return tlaunch_k<HB, kTChunk, 0>(jobs, count, blocks, threads, in, out, record_floats, s);
}

// Grouped records (window 12 or 16: the union).
template <int HB>
int tlaunch_hb_grouped(const StreamJob *jobs, int count, int blocks, int threads, int window, dev::Sample in,
                       dev::Sample out, int record_floats, cudaStream_t s) {
    if (window == 12) return tlaunch_k<HB, kTChunk, 12>(jobs, count, blocks, threads, in, out, record_floats, s);
    if (window == 16) return tlaunch_k<HB, kTChunk, 16>(jobs, count, blocks, threads, in, out, record_floats, s);
    return static_cast<int>(cudaErrorInvalidValue);
}

} // namespace
} // namespace dsmvc_gb
