// ss_track.cuh — device state of the frame-to-model tracker.
#pragma once

#include "ss_internal.cuh"

namespace ss {

constexpr int kMaxLevels = 4;

// Lives in device memory for the life of a pipeline. T is the current pose
// estimate (camera -> world, FP64); pose is its float FramePose, consumed by
// integrate and raycast of the same frame.
struct TrackState {
    double T[16];
    double Tprev[16];    // pose of the model maps (previous frame)
    float Tf[12];        // float copy of T for the iteration kernel
    float Tprev_inv[12]; // world -> model camera
    FramePose pose;
    int ticket;
    int converged_level;
    int inliers[kMaxLevels];
    float rmse[kMaxLevels];
    unsigned int barrier;  // arrivals at the persistent tracker's grid barrier (0 between frames)
    int status;            // kSt* bits of the persistent tracker
    unsigned int exits;    // CTAs of the persistent tracker that have left (the last resets both counters)
    int has_start;         // one-shot: the next tracked frame starts its ICP from Tstart
    double Tstart[16];
};

// Fixed-point accumulators of the persistent tracker's cross-CTA sums: three
// buffers (iterations rotate through them) of 30 values (29 sums and an
// overflow count) x 3 chunks, one 128-byte line per word.
constexpr int kTrackAccValues = 30;
constexpr int kTrackAccChunks = 3;
constexpr int kTrackAccStride = 16;  // u64 words between accumulator words
constexpr int kTrackAccBuffers = 3;
constexpr int kTrackAccBufWords = kTrackAccValues * kTrackAccChunks * kTrackAccStride;
constexpr int kTrackAccWords = kTrackAccBuffers * kTrackAccBufWords;

struct TrackLaunch {
    const uint16_t *depth;
    int rows, cols;
    Intr in;
    const float4 *vmap, *nmap;
    TrackState *state;
    float2 *partials;
    unsigned long long *acc;  // fixed-point accumulators of the persistent tracker (kTrackAccWords, zeroed)
    int ctas;
    int levels;
    int iters[kMaxLevels];
    float dist[kMaxLevels];
    float rmin, dmax;
    bool persistent;  // one cooperative launch for all iterations (else one launch per iteration)
    // The persistent tracker's wait for the other CTAs' sums: at most wait_polls
    // polls; it waits for wait_extra contributions more than there are CTAs
    // (0; a test sets 1 to make the wait run out). On a timeout the status bit
    // is also set in *grid_status (the grid's status word, read by ss_grid_sync).
    int wait_polls = 1 << 22;
    int wait_extra = 0;
    int *grid_status = nullptr;
};

ss_status launch_track(const TrackLaunch &L, cudaStream_t s);
// CTAs of the persistent tracker on this device (co-resident, <= want_per_sm per SM).
int persistent_track_ctas(int num_sms, int want_per_sm);
ss_status launch_pose_prep(TrackState *st, cudaStream_t s);
// Stores the pose T into dst (a device address, e.g. of mapped pinned host memory).
ss_status launch_pose_out(const TrackState *st, double *dst, cudaStream_t s);

}  // namespace ss
