// ss_pipeline.cu — the per-frame reconstruction pipeline:
//   track (3-level point-to-plane GN against the last model view)
//   -> integrate at the tracked pose -> raycast the model view at that pose.
//
// All state (pose, model maps, hash table) stays in device memory; a frame
// needs no host synchronisation. With use_graph a tracked frame (4 kernels:
// the persistent tracker, then collect, fuse and raycast as programmatic
// dependent launches) is captured once per input buffer as a CUDA graph and
// replayed; a change of the grid's launch shapes re-captures it.
// The reference has no such pipeline object: its integration thread
// (src/core/integrate.cpp:47-209) calls GPUVoxelGrid::integrate with poses
// from the keypoint tracker, and raycast is called by the GUI loop
// (exe/SuperScanner.cpp:343-361).
#include <vector>

#include <cmath>

#include "ss_grid_impl.cuh"
#include "ss_track.cuh"

using namespace ss;

struct ss_pipeline {
    ss_grid *g = nullptr;
    ss_pipeline_params p{};
    TrackState *st = nullptr;
    float2 *partials = nullptr;
    unsigned long long *acc = nullptr;  // persistent tracker's fixed-point accumulators
    float4 *vmap = nullptr, *nmap = nullptr;
    // Two input buffers: a host frame is uploaded into one on the copy stream
    // while the previous frame's kernels still read the other.
    uint16_t *input = nullptr;  // inbuf[0], the buffer ss_pipeline_input hands out
    uint16_t *inbuf[2] = {nullptr, nullptr};
    int next_buf = 0;
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_done[2] = {nullptr, nullptr};    // the last frame that read inbuf[b] has finished
    cudaEvent_t ev_copied[2] = {nullptr, nullptr};  // the upload into inbuf[b] has finished
    int ctas = 0;
    int track_ctas = 0;  // co-resident CTAs of the persistent tracker
    bool have_model = false;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph[2] = {nullptr, nullptr};  // one tracked frame reading inbuf[b]
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    unsigned long long frames = 0;
    // stage profiling (non-graph frames only): 6 events per tracked frame
    bool profile = false;
    std::vector<cudaEvent_t> events;
    size_t used = 0;
    unsigned long long *rc_counters = nullptr;  // raycast traffic counters (device u64[4])
    int test_wait_polls = 0;  // one-shot test hook: the next tracked frame's tracker wait runs out
    unsigned exec_gen[2] = {0u, 0u};  // the grid's launch-config generation each graph was captured with
    unsigned lc_gen = 0;              // the generation track_ctas was computed for
};

namespace {
constexpr int kStages = 5;  // track, collect, fuse, finalize, raycast

cudaEvent_t next_event(ss_pipeline *P) {
    if (P->used == P->events.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        P->events.push_back(e);
    }
    return P->events[P->used++];
}
}  // namespace

namespace {

ss_status enqueue_fuse_raycast(ss_pipeline *P, const uint16_t *in, cudaStream_t s, bool prof = false) {
    ss_grid *g = P->g;
    FramePose dummy{};
    cudaEvent_t e1 = prof ? next_event(P) : nullptr, e2 = prof ? next_event(P) : nullptr;
    // the integrate call ends in the raycast's first thread (no finalize launch)
    ss_status st = launch_fuse(g, in, nullptr, dummy, &P->st->pose, false, false, P->p.exact_fusion != 0, s,
                               /*manage_epoch=*/false, e1, e2, /*finalize=*/false);
    if (st != SS_OK) return st;
    if (prof) SS_CUDA_TRY(cudaEventRecord(next_event(P), s));
    const bool hint = P->p.hint_margin > 0.f;
    st = launch_raycast_maps(g, dummy.E, &P->st->pose, P->p.raycast_steps, P->p.t_min, P->p.t_max, P->vmap,
                             P->nmap, s, prof ? P->rc_counters : nullptr, hint ? in : nullptr,
                             P->p.hint_margin, g->v.ctr);
    if (st != SS_OK) return st;
    if (prof) SS_CUDA_TRY(cudaEventRecord(next_event(P), s));
    return SS_OK;
}

ss_status enqueue_frame(ss_pipeline *P, const uint16_t *in, cudaStream_t s, bool prof = false, int wait_polls = 0) {
    ss_grid *g = P->g;
    if (prof) SS_CUDA_TRY(cudaEventRecord(next_event(P), s));
    TrackLaunch L{};
    L.grid_status = &g->v.ctr->status;
    if (wait_polls > 0) {
        L.wait_polls = wait_polls;
        L.wait_extra = 1;
    }
    L.depth = in;
    L.rows = g->p.resi;
    L.cols = g->p.resj;
    L.in = g->v.in;
    L.vmap = P->vmap;
    L.nmap = P->nmap;
    L.state = P->st;
    L.partials = P->partials;
    L.acc = P->acc;
    L.persistent = P->p.persistent_track != 0;
    L.ctas = L.persistent ? P->track_ctas : P->ctas;
    L.levels = P->p.levels;
    for (int l = 0; l < kMaxLevels; l++) {
        L.iters[l] = P->p.iters[l];
        L.dist[l] = P->p.dist_thresh[l];
    }
    L.rmin = g->p.rmin;
    L.dmax = P->p.t_max;
    ss_status st = launch_track(L, s);
    if (st != SS_OK) return st;
    if (prof) SS_CUDA_TRY(cudaEventRecord(next_event(P), s));
    return enqueue_fuse_raycast(P, in, s, prof);
}

// The epoch advances once per executed integrate; rebase before it wraps.
ss_status epoch_guard(ss_pipeline *P, cudaStream_t s) {
    ss_grid *g = P->g;
    if (g->host_epoch + 1 >= kEpochMax) {
        ss_status st = rebase_epoch(g, s);
        if (st != SS_OK) return st;
    }
    return SS_OK;
}

}  // namespace

extern "C" {

ss_status ss_pipeline_params_default(ss_pipeline_params *p) {
    if (!p) return SS_ERR_ARG;
    *p = ss_pipeline_params{};
    p->levels = 3;
    p->iters[0] = 10;  // 640x480
    p->iters[1] = 5;   // 320x240
    p->iters[2] = 4;   // 160x120
    p->iters[3] = 0;
    p->dist_thresh[0] = 0.06f;
    p->dist_thresh[1] = 0.10f;
    p->dist_thresh[2] = 0.15f;
    p->dist_thresh[3] = 0.20f;
    p->raycast_steps = 128;
    p->t_min = 0.2f;
    p->t_max = 10.0f;
    p->use_graph = 1;
    p->exact_fusion = 0;
    p->hint_margin = 0.f;
    p->persistent_track = 0;
    return SS_OK;
}

ss_status ss_pipeline_create(ss_grid *g, const ss_pipeline_params *params, ss_pipeline **out) {
    if (!g || !params || !out) return SS_ERR_ARG;
    *out = nullptr;
    if (params->levels < 1 || params->levels > kMaxLevels || params->raycast_steps < 1) return SS_ERR_ARG;
    if (!g->intr_set) return SS_ERR_STATE;
    ss_pipeline *P = new ss_pipeline;
    P->g = g;
    P->p = *params;
    P->ctas = g->num_sms * 2;
    P->track_ctas = persistent_track_ctas(g->num_sms, g->lc.track_ctas_per_sm);
    P->lc_gen = g->launch_gen;
    const int slot_ctas = P->ctas > 2 * g->num_sms ? P->ctas : 2 * g->num_sms;
    const size_t npix = (size_t)g->p.resi * g->p.resj;
    bool ok = cudaMalloc(&P->st, sizeof(TrackState)) == cudaSuccess &&
              cudaMalloc(&P->partials, 2 * (size_t)slot_ctas * 29 * sizeof(float2)) == cudaSuccess &&
              cudaMalloc(&P->acc, kTrackAccWords * sizeof(unsigned long long)) == cudaSuccess &&
              cudaMalloc(&P->vmap, npix * sizeof(float4)) == cudaSuccess &&
              cudaMalloc(&P->nmap, npix * sizeof(float4)) == cudaSuccess &&
              cudaMalloc(&P->inbuf[0], npix * sizeof(uint16_t)) == cudaSuccess &&
              cudaMalloc(&P->inbuf[1], npix * sizeof(uint16_t)) == cudaSuccess &&
              cudaStreamCreateWithFlags(&P->copy, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&P->ev_done[0], cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&P->ev_done[1], cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&P->ev_copied[0], cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&P->ev_copied[1], cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc(&P->rc_counters, 4 * sizeof(unsigned long long)) == cudaSuccess &&
              cudaStreamCreateWithFlags(&P->cap, cudaStreamNonBlocking) == cudaSuccess;
    P->input = P->inbuf[0];
    if (!ok) {
        cudaGetLastError();
        ss_pipeline_destroy(P);
        return SS_ERR_NOMEM;
    }
    cudaMemset(P->st, 0, sizeof(TrackState));
    cudaMemset(P->acc, 0, kTrackAccWords * sizeof(unsigned long long));
    cudaMemset(P->vmap, 0, npix * sizeof(float4));
    cudaMemset(P->nmap, 0, npix * sizeof(float4));
    double I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    cudaMemcpy(P->st->T, I, sizeof(I), cudaMemcpyHostToDevice);
    SS_CUDA_TRY(cudaDeviceSynchronize());
    *out = P;
    return SS_OK;
}

ss_status ss_pipeline_destroy(ss_pipeline *P) {
    if (!P) return SS_ERR_ARG;
    for (int b = 0; b < 2; b++) {
        if (P->exec[b]) cudaGraphExecDestroy(P->exec[b]);
        if (P->graph[b]) cudaGraphDestroy(P->graph[b]);
        if (P->ev_done[b]) cudaEventDestroy(P->ev_done[b]);
        if (P->ev_copied[b]) cudaEventDestroy(P->ev_copied[b]);
    }
    if (P->cap) cudaStreamDestroy(P->cap);
    if (P->copy) cudaStreamDestroy(P->copy);
    for (cudaEvent_t e : P->events) cudaEventDestroy(e);
    cudaFree(P->st);
    cudaFree(P->partials);
    cudaFree(P->acc);
    cudaFree(P->vmap);
    cudaFree(P->nmap);
    cudaFree(P->inbuf[0]);
    cudaFree(P->inbuf[1]);
    cudaFree(P->rc_counters);
    delete P;
    return SS_OK;
}

ss_status ss_pipeline_set_pose(ss_pipeline *P, const double T[16], ss_stream_t stream) {
    if (!P || !T) return SS_ERR_ARG;
    SS_CUDA_TRY(cudaMemcpyAsync(P->st->T, T, 16 * sizeof(double), cudaMemcpyHostToDevice, (cudaStream_t)stream));
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    return SS_OK;
}

ss_status ss_pipeline_set_start(ss_pipeline *P, const double T[16], ss_stream_t stream) {
    if (!P || !T) return SS_ERR_ARG;
    for (int k = 0; k < 16; k++)
        if (!std::isfinite(T[k])) return SS_ERR_ARG;
    static const int one = 1;
    cudaStream_t s = (cudaStream_t)stream;
    SS_CUDA_TRY(cudaMemcpyAsync(P->st->Tstart, T, 16 * sizeof(double), cudaMemcpyHostToDevice, s));
    SS_CUDA_TRY(cudaMemcpyAsync(&P->st->has_start, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    SS_CUDA_TRY(cudaStreamSynchronize(s));
    return SS_OK;
}

ss_status ss_pipeline_get_pose(ss_pipeline *P, double T[16], ss_stream_t stream) {
    if (!P || !T) return SS_ERR_ARG;
    SS_CUDA_TRY(cudaMemcpyAsync(T, P->st->T, 16 * sizeof(double), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    return SS_OK;
}

ss_status ss_pipeline_read_pose(ss_pipeline *P, double T[16], ss_stream_t stream) {
    if (!P || !T) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    // pinned host memory mapped into the device's address space: one small
    // kernel stores the pose there (a copy-engine transfer of 128 bytes
    // between two frames' kernels costs several microseconds of hand-off)
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, T) == cudaSuccess && attr.type == cudaMemoryTypeHost && attr.devicePointer)
        return launch_pose_out(P->st, (double *)attr.devicePointer, s);
    cudaGetLastError();
    SS_CUDA_TRY(cudaMemcpyAsync(T, P->st->T, 16 * sizeof(double), cudaMemcpyDefault, s));
    return SS_OK;
}

ss_status ss_pipeline_input(ss_pipeline *P, uint16_t **depth) {
    if (!P || !depth) return SS_ERR_ARG;
    *depth = P->input;
    return SS_OK;
}

ss_status ss_pipeline_maps(ss_pipeline *P, float **vertex_depth, float **normal) {
    if (!P || !vertex_depth || !normal) return SS_ERR_ARG;
    *vertex_depth = (float *)P->vmap;
    *normal = (float *)P->nmap;
    return SS_OK;
}

ss_status ss_pipeline_frame(ss_pipeline *P, const uint16_t *depth, int32_t track, ss_stream_t stream) {
    if (!P || !depth) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    ss_grid *g = P->g;
    const size_t bytes = (size_t)g->p.resi * g->p.resj * sizeof(uint16_t);
    // The input buffer of this frame. A frame already in one of them (written
    // through ss_pipeline_input) is read in place. A host frame is uploaded on
    // the copy stream into the buffer the frame before last read, as soon as
    // that frame has finished, so the upload overlaps the last frame's
    // kernels; s waits for the upload. Another device pointer is copied on s
    // (earlier work on s may be producing it).
    int b;
    if (depth == P->inbuf[0] || depth == P->inbuf[1]) {
        b = depth == P->inbuf[0] ? 0 : 1;
    } else {
        b = P->next_buf;
        P->next_buf ^= 1;
        cudaPointerAttributes attr{};
        const bool host = cudaPointerGetAttributes(&attr, depth) == cudaSuccess &&
                          (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeUnregistered);
        cudaGetLastError();
        if (host) {
            SS_CUDA_TRY(cudaStreamWaitEvent(P->copy, P->ev_done[b], 0));
            SS_CUDA_TRY(cudaMemcpyAsync(P->inbuf[b], depth, bytes, cudaMemcpyDefault, P->copy));
            SS_CUDA_TRY(cudaEventRecord(P->ev_copied[b], P->copy));
            SS_CUDA_TRY(cudaStreamWaitEvent(s, P->ev_copied[b], 0));
        } else {
            SS_CUDA_TRY(cudaMemcpyAsync(P->inbuf[b], depth, bytes, cudaMemcpyDefault, s));
        }
    }
    const uint16_t *in = P->inbuf[b];
    if (P->lc_gen != g->launch_gen) {  // launch shapes changed: new tracker grid, graphs recaptured below
        P->track_ctas = persistent_track_ctas(g->num_sms, g->lc.track_ctas_per_sm);
        P->lc_gen = g->launch_gen;
    }
    ss_status st = epoch_guard(P, s);
    if (st != SS_OK) return st;
    if (!track || !P->have_model) {
        st = launch_pose_prep(P->st, s);
        if (st == SS_OK) st = enqueue_fuse_raycast(P, in, s);
        if (st != SS_OK) return st;
        P->have_model = true;
    } else if (P->p.use_graph && P->test_wait_polls == 0) {
        if (P->exec[b] && P->exec_gen[b] != g->launch_gen) {  // launch shapes changed since the capture
            cudaGraphExecDestroy(P->exec[b]);
            cudaGraphDestroy(P->graph[b]);
            P->exec[b] = nullptr;
            P->graph[b] = nullptr;
        }
        if (!P->exec[b]) {
            SS_CUDA_TRY(cudaStreamBeginCapture(P->cap, cudaStreamCaptureModeThreadLocal));
            // collect, fuse and raycast as programmatic dependents: each launches
            // while the kernel before it drains and waits for it in-kernel
            g->pdl = true;
            st = enqueue_frame(P, in, P->cap);
            g->pdl = false;
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(P->cap, &graph);
            if (st != SS_OK) {
                if (graph) cudaGraphDestroy(graph);
                return st;
            }
            if (e != cudaSuccess) {
                set_last_error("cudaStreamEndCapture", e);
                return SS_ERR_CUDA;
            }
            P->graph[b] = graph;
            SS_CUDA_TRY(cudaGraphInstantiate(&P->exec[b], P->graph[b], 0));
            P->exec_gen[b] = g->launch_gen;
        }
        SS_CUDA_TRY(cudaGraphLaunch(P->exec[b], s));
    } else {
        st = enqueue_frame(P, in, s, P->profile, P->test_wait_polls);
        P->test_wait_polls = 0;
        if (st != SS_OK) return st;
    }
    SS_CUDA_TRY(cudaEventRecord(P->ev_done[b], s));
    g->host_epoch++;
    P->frames++;
    return SS_OK;
}

ss_status ss_pipeline_test_wait_timeout(ss_pipeline *P, int32_t polls) {
    if (!P || polls < 0) return SS_ERR_ARG;
    if (!P->p.persistent_track) return SS_ERR_STATE;
    P->test_wait_polls = polls;
    return SS_OK;
}

ss_status ss_pipeline_profile(ss_pipeline *P, int32_t enable) {
    if (!P) return SS_ERR_ARG;
    P->profile = enable != 0;
    P->used = 0;
    SS_CUDA_TRY(cudaMemset(P->rc_counters, 0, 4 * sizeof(unsigned long long)));
    return SS_OK;
}

ss_status ss_pipeline_stage_ms(ss_pipeline *P, double ms[5], int64_t *frames, int64_t counters[4],
                               ss_stream_t stream) {
    if (!P || !ms || !frames) return SS_ERR_ARG;
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    for (int k = 0; k < kStages; k++) ms[k] = 0.0;
    const size_t per = kStages + 1;
    *frames = (int64_t)(P->used / per);
    if (counters) SS_CUDA_TRY(cudaMemcpy(counters, P->rc_counters, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost));
    for (size_t f = 0; f + per <= P->used; f += per) {
        for (int k = 0; k < kStages; k++) {
            float t = 0.f;
            SS_CUDA_TRY(cudaEventElapsedTime(&t, P->events[f + k], P->events[f + k + 1]));
            ms[k] += t;
        }
    }
    return SS_OK;
}

ss_status ss_pipeline_copy_maps(ss_pipeline *P, float *vertex_depth, float *normal, ss_stream_t stream) {
    if (!P || !vertex_depth || !normal) return SS_ERR_ARG;
    const size_t bytes = (size_t)P->g->p.resi * P->g->p.resj * sizeof(float4);
    SS_CUDA_TRY(cudaMemcpyAsync(vertex_depth, P->vmap, bytes, cudaMemcpyDefault, (cudaStream_t)stream));
    SS_CUDA_TRY(cudaMemcpyAsync(normal, P->nmap, bytes, cudaMemcpyDefault, (cudaStream_t)stream));
    return SS_OK;
}

ss_status ss_pipeline_stats(ss_pipeline *P, int32_t inliers[4], float rmse[4], ss_stream_t stream) {
    if (!P || !inliers || !rmse) return SS_ERR_ARG;
    TrackState h;
    SS_CUDA_TRY(cudaMemcpyAsync(&h, P->st, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    for (int l = 0; l < 4; l++) {
        inliers[l] = h.inliers[l];
        rmse[l] = h.rmse[l];
    }
    return SS_OK;
}

}  // extern "C"
