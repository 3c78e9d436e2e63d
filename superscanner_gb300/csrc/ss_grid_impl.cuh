// ss_grid_impl.cuh — host-side grid object shared by the translation units.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "ss_internal.cuh"

struct ss_grid {
    ss_params p;
    ss::GridView v;
    bool intr_set = false;
    float fx = 0, fy = 0, cx = 0, cy = 0;
    ss_launch_config lc{8, 8, 8, 8, 2};  // launch shapes (autotuner)
    unsigned launch_gen = 0;               // bumped by every ss_grid_set_launch_config
    int raycast_cap = 0;                   // test hook: ss_raycast's iteration cap (0: the default)
    uint32_t host_epoch = 1;  // mirror of Counters::epoch for wrap handling
    int device = 0;
    int num_sms = 0;
    // batched re-fusion scratch, allocated on the first ss_refuse_batch call
    uint32_t *phase_mask = nullptr;        // [buckets][kMaxPhases / 32]
    ss::FramePose *batch_poses = nullptr;  // [kMaxPhases]
    const uint16_t **batch_depths = nullptr;  // [kMaxPhases / 2] device pointers
    unsigned long long *mesh_count = nullptr;  // triangle counter of ss_grid_extract_mesh (first call)
    // launch collect, fuse and raycast as programmatic dependents of the kernel
    // before them (set by the per-frame pipeline while it captures its graph)
    bool pdl = false;
};

namespace ss {

constexpr int kMaxPhases = 512;  // 2 x keyframes of one ss_refuse_batch call
constexpr int kPhaseWords = kMaxPhases / 32;

// Last CUDA error text of this thread (ss_last_error()).
void set_last_error(const char *where, cudaError_t e);
void set_last_error_text(const std::string &s);

// Maps device status bits to the ABI status (first error wins).
ss_status status_from_bits(int bits);

#define SS_CUDA_TRY(call)                                  \
    do {                                                   \
        cudaError_t _e = (call);                           \
        if (_e != cudaSuccess) {                           \
            ::ss::set_last_error(#call, _e);               \
            return SS_ERR_CUDA;                            \
        }                                                  \
    } while (0)

#define SS_LAUNCH_CHECK()                                  \
    do {                                                   \
        cudaError_t _e = cudaGetLastError();               \
        if (_e != cudaSuccess) {                           \
            ::ss::set_last_error("kernel launch", _e);     \
            return SS_ERR_CUDA;                            \
        }                                                  \
    } while (0)

// Launches kernel<<<grid, block, smem, s>>>(args...), as a programmatic
// dependent of the previous kernel in s when pdl is set (the kernel must call
// pdl_wait() before it touches that kernel's outputs).
template <class... K, class... A>
cudaError_t launch_kernel(void (*kernel)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl,
                          A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<A &&>(args)...);
}

Mat34 mat34_from(const float E[16]);
FramePose frame_pose_from(const float extr[16]);

// The end of an integrate / deintegrate call (one thread): remembers and
// resets the block list, advances the epoch.
__device__ __forceinline__ void end_call(Counters *ctr) {
    const int n = ctr->list_count;
    ctr->last_touched = n;
    ctr->touched_total += (unsigned long long)n;
    ctr->calls += 1ull;
    ctr->list_count = 0;
    ctr->epoch = ctr->epoch + 1u;
}

// integrate / deintegrate launch sequence (collect, fuse, finalize); the pose
// comes from hp, or from device memory when dpose is not null. With
// manage_epoch the host epoch mirror is advanced here (direct calls); graph
// replays advance it in the caller instead. Without finalize the caller ends
// the call in a later kernel of the same stream (end_call) before the next
// collection.
ss_status launch_fuse(ss_grid *g, const uint16_t *depth, const uint8_t *rgb, const FramePose &hp,
                      const FramePose *dpose, bool color, bool deint, bool exact, cudaStream_t s,
                      bool manage_epoch = true, cudaEvent_t after_collect = nullptr,
                      cudaEvent_t after_fuse = nullptr, bool finalize = true);
// Clears the epoch field of every stamp and restarts the epoch at 1.
ss_status rebase_epoch(ss_grid *g, cudaStream_t s);
void inverse4_rounded(const float E[16], float out[16]);

// counters (optional, device u64[4]): hash finds, voxel loads, march steps, hits.
// end (optional): the integrate call whose end the raycast's first thread
// performs (end_call), in place of a finalize launch.
ss_status launch_raycast_maps(ss_grid *g, const Mat34 &T, const FramePose *dpose, int max_steps, float t_min,
                              float t_max, float4 *vmap, float4 *nmap, cudaStream_t s,
                              unsigned long long *counters = nullptr, const uint16_t *hint = nullptr,
                              float hint_margin = 0.f, Counters *end = nullptr);

// Blocks of persistent launches (multiple of the SM count).
int persistent_ctas(const ss_grid *g, int per_sm);

}  // namespace ss
