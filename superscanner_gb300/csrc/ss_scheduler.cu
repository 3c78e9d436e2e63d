// ss_scheduler.cu — the integration thread's scheduling (re-fusion scheduler)
// of the reference, src/core/integrate.cpp:47-236, as a host-side object
// over the fusion entry points (host code only; no kernels of its own).
//
// The reference keeps three frame buffers — frames to integrate, to
// re-integrate and to deintegrate — and a list of integrated frames; each
// pass of its thread loop integrates one new frame, re-integrates one frame
// (deintegrate at the DoFs it was fused at, integrate at its current world
// DoFs) and deintegrates one frame (integrate.cpp:59-138).
// updateReintegrationBuffer (:218-236) refills the re-integration buffer with
// the integrated frames whose pose changed by diff >= treint (:205-211:
// |(d rotation DoFs, 2 d translation DoFs)|), largest change first (a stable
// sort of the integrated-frame list, so ties keep integration order).
//
// Here one step does all pending integrations, up to max_batch queued
// re-integrations as ONE batched re-fusion (ss_refuse_batch: one collection
// launch and one persistent apply launch, the volume bit for bit that of the
// sequential deintegrate + integrate pairs), then all pending
// deintegrations. Everything is stream-ordered: no host synchronisation.
// Deliberate differences, each fixing a reference race or slip:
//  * a frame deintegrated while still queued for re-integration leaves that
//    queue (the reference would re-integrate it after its deintegration);
//  * a frame removed before it was integrated is dropped from the
//    integration queue instead of being deintegrated unfused;
//  * the stop drain deintegrates the frames of the deintegration buffer (the
//    reference's drain integrates them again, integrate.cpp:185-195).
#include <algorithm>
#include <cmath>
#include <deque>
#include <map>
#include <vector>

#include "ss_grid_impl.cuh"

namespace ss {
namespace {

void dofs_to_pose(const double *x, double *T) {
    // getT (matrixutil.h:61-63) = trans(x[3..5]) Rz(x[2]) Ry(x[1]) Rx(x[0]), in closed form
    // (the product written out, as getT22, matrixutil.h:119-126)
    const double cx = std::cos(x[0]), sx = std::sin(x[0]), cy = std::cos(x[1]), sy = std::sin(x[1]);
    const double cz = std::cos(x[2]), sz = std::sin(x[2]);
    const double R[9] = {cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx,
                         sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx,
                         -sy,     sx * cy,                cx * cy};
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) T[r * 4 + c] = R[r * 3 + c];
        T[r * 4 + 3] = x[3 + r];
    }
    T[12] = T[13] = T[14] = 0.0;
    T[15] = 1.0;
}

double pose_change(const double *world, const double *integrated) {
    // diff (integrate.cpp:205-211): rotation DoF deltas, translation deltas doubled
    double s = 0.0;  // the 6-vector's squared norm, summed in element order
    for (int k = 0; k < 6; k++) {
        const double v = (k < 3 ? 1.0 : 2.0) * (world[k] - integrated[k]);
        s += v * v;
    }
    return std::sqrt(s);
}

void pose_f32(const double *dofs, float *out) {
    double T[16];
    dofs_to_pose(dofs, T);
    for (int k = 0; k < 16; k++) out[k] = (float)T[k];  // getT(...).cast<float>()
}

bool finite6(const double *d) {
    for (int k = 0; k < 6; k++)
        if (!std::isfinite(d[k])) return false;
    return true;
}

}  // namespace
}  // namespace ss

using namespace ss;

struct ss_scheduler {
    struct Frame {
        const uint16_t *depth = nullptr;
        double world[6] = {};       // current world DoFs (getWorlddofs)
        double integrated[6] = {};  // DoFs the frame is fused at (integrateddofs)
        bool integrated_flag = false;
    };
    ss_grid *g = nullptr;
    double treint = 0.04;
    int max_batch = 64;
    bool exact = false;
    std::map<int64_t, Frame> frames;
    std::vector<int64_t> integrated_order;  // integratedframes (integration order)
    std::deque<int64_t> to_integrate, to_reintegrate, to_deintegrate;
};

namespace {

void erase_id(std::deque<int64_t> &q, int64_t id) { q.erase(std::remove(q.begin(), q.end(), id), q.end()); }

ss_status run_integrations(ss_scheduler *S, cudaStream_t st, int32_t *done) {
    while (!S->to_integrate.empty()) {
        const int64_t id = S->to_integrate.front();
        ss_scheduler::Frame &f = S->frames.at(id);
        float T[16];
        pose_f32(f.world, T);
        const ss_status r = S->exact ? ss_integrate(S->g, f.depth, nullptr, T, 0, st)
                                     : ss_integrate_fast(S->g, f.depth, nullptr, T, 0, 0, st);
        if (r != SS_OK) return r;
        S->to_integrate.pop_front();
        std::copy(f.world, f.world + 6, f.integrated);
        f.integrated_flag = true;
        S->integrated_order.push_back(id);
        (*done)++;
    }
    return SS_OK;
}

ss_status run_reintegrations(ss_scheduler *S, cudaStream_t st, int limit, int32_t *done) {
    while (!S->to_reintegrate.empty() && limit > 0) {
        const int n = std::min<int>({(int)S->to_reintegrate.size(), limit, 256});
        std::vector<const uint16_t *> depths(n);
        std::vector<float> T_old(16 * (size_t)n), T_new(16 * (size_t)n);
        for (int k = 0; k < n; k++) {
            const ss_scheduler::Frame &f = S->frames.at(S->to_reintegrate[k]);
            depths[k] = f.depth;
            pose_f32(f.integrated, &T_old[16 * (size_t)k]);
            pose_f32(f.world, &T_new[16 * (size_t)k]);
        }
        const ss_status r = ss_refuse_batch(S->g, n, depths.data(), T_old.data(), T_new.data(), S->exact ? 1 : 0, st);
        if (r != SS_OK) return r;
        for (int k = 0; k < n; k++) {
            ss_scheduler::Frame &f = S->frames.at(S->to_reintegrate.front());
            std::copy(f.world, f.world + 6, f.integrated);
            S->to_reintegrate.pop_front();
        }
        *done += n;
        limit -= n;
    }
    return SS_OK;
}

ss_status run_deintegrations(ss_scheduler *S, cudaStream_t st, int32_t *done) {
    while (!S->to_deintegrate.empty()) {
        const int64_t id = S->to_deintegrate.front();
        ss_scheduler::Frame &f = S->frames.at(id);
        float T[16];
        pose_f32(f.integrated, T);
        const ss_status r = S->exact ? ss_deintegrate(S->g, f.depth, nullptr, T, 0, st)
                                     : ss_integrate_fast(S->g, f.depth, nullptr, T, 0, 1, st);
        if (r != SS_OK) return r;
        S->to_deintegrate.pop_front();
        S->integrated_order.erase(std::remove(S->integrated_order.begin(), S->integrated_order.end(), id),
                                  S->integrated_order.end());
        S->frames.erase(id);  // the frame leaves the scheduler (its depth buffer is the caller's again)
        (*done)++;
    }
    return SS_OK;
}

}  // namespace

extern "C" {

ss_status ss_dofs_to_pose(const double dofs[6], double T[16]) {
    if (!dofs || !T) return SS_ERR_ARG;
    dofs_to_pose(dofs, T);
    return SS_OK;
}

ss_status ss_pose_to_dofs(const double T[16], double dofs[6]) {
    if (!T || !dofs) return SS_ERR_ARG;
    // MattoDof (matrixutil.cpp:37-49)
    dofs[0] = std::atan2(T[9], T[10]);
    dofs[1] = -std::asin(T[8]);
    dofs[2] = std::atan2(T[4], T[0]);
    dofs[3] = T[3];
    dofs[4] = T[7];
    dofs[5] = T[11];
    return SS_OK;
}

ss_status ss_reintegration_order(int32_t n, const double *world_dofs, const double *integrated_dofs, double treint,
                                 int32_t *order, int32_t *count) {
    if (n < 0 || (n > 0 && (!world_dofs || !integrated_dofs || !order)) || !count) return SS_ERR_ARG;
    std::vector<int32_t> idx(n);
    std::vector<double> d(n);
    for (int32_t k = 0; k < n; k++) {
        idx[k] = k;
        d[k] = pose_change(world_dofs + 6 * (size_t)k, integrated_dofs + 6 * (size_t)k);
    }
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return d[a] > d[b]; });
    int32_t c = 0;
    while (c < n && !(d[idx[c]] < treint)) {
        order[c] = idx[c];
        c++;
    }
    *count = c;
    return SS_OK;
}

ss_status ss_scheduler_create(ss_grid *g, double treint, int32_t max_batch, int32_t exact, ss_scheduler **out) {
    if (!g || !out || !(treint >= 0.0) || max_batch < 1) return SS_ERR_ARG;
    ss_scheduler *S = new ss_scheduler;
    S->g = g;
    S->treint = treint;
    S->max_batch = max_batch;
    S->exact = exact != 0;
    *out = S;
    return SS_OK;
}

ss_status ss_scheduler_destroy(ss_scheduler *S) {
    delete S;
    return SS_OK;
}

ss_status ss_scheduler_push_integrate(ss_scheduler *S, int64_t id, const uint16_t *depth, const double dofs[6]) {
    if (!S || !depth || !dofs || !finite6(dofs) || S->frames.count(id)) return SS_ERR_ARG;
    ss_scheduler::Frame f;
    f.depth = depth;
    std::copy(dofs, dofs + 6, f.world);
    S->frames.emplace(id, f);
    S->to_integrate.push_back(id);
    return SS_OK;
}

ss_status ss_scheduler_set_dofs(ss_scheduler *S, int64_t id, const double dofs[6]) {
    if (!S || !dofs || !finite6(dofs)) return SS_ERR_ARG;
    auto it = S->frames.find(id);
    if (it == S->frames.end()) return SS_ERR_ARG;
    std::copy(dofs, dofs + 6, it->second.world);
    return SS_OK;
}

ss_status ss_scheduler_push_deintegrate(ss_scheduler *S, int64_t id) {
    if (!S) return SS_ERR_ARG;
    auto it = S->frames.find(id);
    if (it == S->frames.end()) return SS_ERR_ARG;
    erase_id(S->to_reintegrate, id);
    if (!it->second.integrated_flag) {  // never fused: just forget it
        erase_id(S->to_integrate, id);
        S->frames.erase(it);
        return SS_OK;
    }
    if (std::find(S->to_deintegrate.begin(), S->to_deintegrate.end(), id) == S->to_deintegrate.end())
        S->to_deintegrate.push_back(id);
    return SS_OK;
}

ss_status ss_scheduler_update(ss_scheduler *S, int32_t *queued) {
    if (!S) return SS_ERR_ARG;
    // integrated frames that are not being deintegrated, in integration order
    std::vector<int64_t> ids;
    for (int64_t id : S->integrated_order)
        if (std::find(S->to_deintegrate.begin(), S->to_deintegrate.end(), id) == S->to_deintegrate.end())
            ids.push_back(id);
    const int32_t n = (int32_t)ids.size();
    std::vector<double> w(6 * (size_t)n), in(6 * (size_t)n);
    for (int32_t k = 0; k < n; k++) {
        const ss_scheduler::Frame &f = S->frames.at(ids[k]);
        std::copy(f.world, f.world + 6, &w[6 * (size_t)k]);
        std::copy(f.integrated, f.integrated + 6, &in[6 * (size_t)k]);
    }
    std::vector<int32_t> order(n);
    int32_t c = 0;
    ss_status r = ss_reintegration_order(n, w.data(), in.data(), S->treint, order.data(), &c);
    if (r != SS_OK) return r;
    S->to_reintegrate.clear();  // reintegrationBuffer.clear() (integrate.cpp:224)
    for (int32_t k = 0; k < c; k++) S->to_reintegrate.push_back(ids[order[k]]);
    if (queued) *queued = c;
    return SS_OK;
}

ss_status ss_scheduler_queue(ss_scheduler *S, int32_t which, int32_t cap, int64_t *ids, int32_t *count) {
    if (!S || !count || which < 0 || which > 2 || cap < 0 || (cap > 0 && !ids)) return SS_ERR_ARG;
    const std::deque<int64_t> &q = which == 0 ? S->to_integrate : (which == 1 ? S->to_reintegrate : S->to_deintegrate);
    const int32_t n = (int32_t)q.size();
    for (int32_t k = 0; k < n && k < cap; k++) ids[k] = q[k];
    *count = n;
    return SS_OK;
}

ss_status ss_scheduler_step(ss_scheduler *S, ss_stream_t stream, int32_t done[3]) {
    if (!S || !done) return SS_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    done[0] = done[1] = done[2] = 0;
    ss_status r = run_integrations(S, st, &done[0]);
    if (r == SS_OK) r = run_reintegrations(S, st, S->max_batch, &done[1]);
    if (r == SS_OK) r = run_deintegrations(S, st, &done[2]);
    return r;
}

ss_status ss_scheduler_drain(ss_scheduler *S, ss_stream_t stream, int32_t done[3]) {
    if (!S || !done) return SS_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    done[0] = done[1] = done[2] = 0;
    ss_status r = run_integrations(S, st, &done[0]);
    if (r == SS_OK) r = run_reintegrations(S, st, 1 << 30, &done[1]);
    if (r == SS_OK) r = run_deintegrations(S, st, &done[2]);
    return r;
}

ss_status ss_scheduler_frame(ss_scheduler *S, int64_t id, int32_t *integrated, double integrated_dofs[6]) {
    if (!S || !integrated) return SS_ERR_ARG;
    auto it = S->frames.find(id);
    if (it == S->frames.end()) return SS_ERR_ARG;
    *integrated = it->second.integrated_flag ? 1 : 0;
    if (integrated_dofs) std::copy(it->second.integrated, it->second.integrated + 6, integrated_dofs);
    return SS_OK;
}

}  // extern "C"
