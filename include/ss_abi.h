/*
 * ss_abi.h — C-ABI of the GB300-native SuperScanner reconstruction hot path.
 *
 * Plain C: pointers, sizes and POD structs only. Every device buffer is a raw
 * device pointer owned by the caller; every pose is a host array copied into
 * kernel parameters at call time. All calls are stream-ordered and
 * asynchronous unless stated otherwise; a device-side status word collects
 * kernel-detected errors and is returned by ss_grid_sync().
 *
 * Reference interfaces replaced (paths inside Pandia3DPublic/SuperScanner):
 *   GPUVoxelGrid ctor                  src/VoxelGrid/GPUVoxelGrid.h:43, .cpp:10-30
 *   GPUVoxelGrid::setIntrinsic         src/VoxelGrid/GPUVoxelGrid.h:118-119, .cpp:253-266
 *   GPUVoxelGrid::integrate            src/VoxelGrid/GPUVoxelGrid.h:98-101, .cpp:41-83
 *   GPUVoxelGrid::deIntegrate          src/VoxelGrid/GPUVoxelGrid.h:102-105, .cpp:95-136
 *   GPUVoxelGrid::raycast              src/VoxelGrid/GPUVoxelGrid.h:107-108, .cpp:139-147
 *   GPUVoxelGrid::cleanMemory          src/VoxelGrid/GPUVoxelGrid.h:116-117, .cpp:185-196
 *   GPUVoxelGrid::marchingCubesHost    src/VoxelGrid/GPUVoxelGrid.cpp:200-251 (the host
 *                                       copy of the map; replaced by ss_grid_export_blocks)
 *   CreatePcdFromDepthView             src/utils/imageutil.cpp:89-111
 *   CalculateNormalsFromPCDView        src/utils/imageutil.cpp:117-157
 *   kokkosICP(View,View,tx,ty,type,r)  src/postprocessing/kokkosICP.h:19-21, .cpp:25-210
 *
 * Image layout: row-major [rows][cols] (row = i, col = j as in the reference's
 * depth(i, j)); depth is uint16 millimetres, colour is uint8 x3 interleaved,
 * point/normal maps are float x3 interleaved. Poses are 4x4 row-major.
 */
#ifndef SS_ABI_H
#define SS_ABI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same handle type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st *ss_stream_t;

typedef enum ss_status {
    SS_OK = 0,
    SS_ERR_ARG = 1,           /* null pointer, bad size, bad enum */
    SS_ERR_DIMS = 2,          /* image size differs from the grid's (GPUVoxelGrid.cpp:46-49 only printed) */
    SS_ERR_TABLE_FULL = 3,    /* no free bucket for a new block (reference: unchecked, GPUVoxelGrid.cpp:497-500) */
    SS_ERR_LIST_OVERFLOW = 4, /* touched-block list overflow (reference: unchecked, GPUVoxelGrid.cpp:506-508) */
    SS_ERR_TIMEOUT = 5,       /* a bounded device loop hit its iteration cap */
    SS_ERR_CUDA = 6,          /* a CUDA runtime call failed */
    SS_ERR_RANGE = 7,         /* a block coordinate outside the packable range (|c| > 8191 blocks) */
    SS_ERR_STATE = 8,         /* call order violated (e.g. integrate before set_intrinsic) */
    SS_ERR_NOMEM = 9          /* device allocation failed */
} ss_status;

typedef enum ss_storage {
    SS_STORAGE_F32 = 0,       /* plain form: FP32 sdf + FP32 weight (8 B/voxel) */
    SS_STORAGE_F16 = 1        /* precision form: FP16 sdf/trunc + uint16 weight (4 B/voxel), FP32 math */
} ss_storage;

typedef enum ss_icp_type {    /* src/postprocessing/kokkosICP.h:4-8 */
    SS_ICP_POINT_TO_POINT = 0,
    SS_ICP_POINT_TO_PLANE = 1
} ss_icp_type;

typedef struct ss_params {
    float voxel_length;       /* vl, metres (GPUVoxelGrid.h:48) */
    float truncation;         /* d_trunc, metres (GPUVoxelGrid.h:47) */
    int32_t resi;             /* image rows (GPUVoxelGrid.h:50) */
    int32_t resj;             /* image cols (GPUVoxelGrid.h:51) */
    uint32_t hash_buckets;    /* power of two; bucket i owns block payload i (like UnorderedMap::value_at) */
    int32_t storage;          /* ss_storage */
    int32_t with_color;       /* allocate FP32 r,g,b planes (Voxel::r,g,b, GPUVoxelGrid.h:15-17) */
    float max_weight;         /* 0 = uncapped, as the reference (GPUVoxelGrid.h:14,62) */
    float rmin;               /* minimal integrated depth, 0.2 m (GPUVoxelGrid.h:56) */
    float d_max;              /* raycast range, 10 m (GPUVoxelGrid.h:55) */
} ss_params;

typedef struct ss_grid ss_grid;

/* Launch shapes of a grid's kernels (no reference counterpart), chosen by
 * the autotuner (superscanner_gb300/autotune.py) or left at the defaults.
 * Pixel kernels run 32 x rows thread tiles (one warp per 32 pixels of a
 * row); persistent kernels run ctas_per_sm x SM-count CTAs of 256 threads. */
typedef struct ss_launch_config {
    int32_t collect_rows;       /* block collection tile rows, 1..8 (default 8) */
    int32_t raycast_rows;       /* model-view raycast tile rows, 1..16 (default 8) */
    int32_t fuse_ctas_per_sm;   /* integrate / deintegrate, 1..32 (default 8) */
    int32_t refuse_ctas_per_sm; /* batched re-fusion apply, 1..32 (default 8) */
    int32_t track_ctas_per_sm;  /* persistent tracker, 1..2, capped by occupancy (default 2) */
} ss_launch_config;

/* Fills the reference defaults of GPUVoxelGrid(c, trunc, voxlength, resi, resj)
 * (GPUVoxelGrid.cpp:10-30): buckets = next power of two >= c / 512. */
ss_status ss_params_default(ss_params *p, uint32_t capacity_voxels, float trunc,
                            float voxel_length, int32_t resi, int32_t resj);

ss_status ss_grid_create(const ss_params *p, ss_grid **out);
ss_status ss_grid_destroy(ss_grid *g);
ss_status ss_grid_get_launch_config(const ss_grid *g, ss_launch_config *c);
/* Takes effect for later launches, also of a pipeline over this grid (its
 * captured per-frame graphs are re-captured with the new shapes). */
ss_status ss_grid_set_launch_config(ss_grid *g, const ss_launch_config *c);

/* Resets the volume to empty (all buckets free, all payload zero). */
ss_status ss_grid_reset(ss_grid *g, ss_stream_t s);

/* setIntrinsic (GPUVoxelGrid.cpp:253-266): fx, fy, cx, cy of the pinhole model;
 * the grid uses ci = resi - cy, cj = cx exactly as the reference. */
ss_status ss_grid_set_intrinsic(ss_grid *g, float fx, float fy, float cx, float cy);

/* integrate / deIntegrate (GPUVoxelGrid.cpp:41-136). depth: [resi][resj] u16 mm,
 * rgb: [resi][resj][3] u8 or NULL (required when with_color != 0);
 * extr: camera->world, row-major. No host synchronisation inside. */
ss_status ss_integrate(ss_grid *g, const uint16_t *depth, const uint8_t *rgb,
                       const float extr[16], int32_t with_color, ss_stream_t s);
ss_status ss_deintegrate(ss_grid *g, const uint16_t *depth, const uint8_t *rgb,
                         const float extr[16], int32_t with_color, ss_stream_t s);

/* raycast (GPUVoxelGrid.cpp:139-147, 561-715): reference semantics — nearest
 * voxel march from 0.1 m to d_max, world-space points into ray_pcd
 * [resi][resj][3], colour/255 into ray_color (may be NULL). Misses are 0. */
ss_status ss_raycast(ss_grid *g, const float extr[16], float *ray_pcd, float *ray_color,
                     ss_stream_t s);

/* cleanMemory (GPUVoxelGrid.cpp:185-196, 785-805): frees every block whose 512
 * weights are all zero. */
ss_status ss_clean_memory(ss_grid *g, ss_stream_t s);

/* Same as ss_integrate / ss_deintegrate (deint != 0), with FMA-contracted
 * single-precision arithmetic in the voxel update and the voxel observed at
 * the pixel nearest to its projection (the reference truncates the projected
 * coordinate, GPUVoxelGrid.cpp:348-349, a half-pixel bias that makes
 * frame-to-model tracking drift); block allocation keeps the reference
 * rounding. Used by the per-frame pipeline. No reference counterpart. */
ss_status ss_integrate_fast(ss_grid *g, const uint16_t *depth, const uint8_t *rgb,
                            const float extr[16], int32_t with_color, int32_t deint,
                            ss_stream_t s);

/* Loop-closure re-fusion of n keyframes (n <= 256): for k = 0..n-1 in order,
 * deintegrate depth k at T_old[k], then integrate it at T_new[k] — the
 * reference's deIntegrate + integrate pair per re-fused frame
 * (src/core/integrate.cpp:109-113, src/postprocessing/postprocessing.cpp:64-76)
 * — as one collection launch and one persistent apply launch. depths: host
 * array of n device pointers to [resi][resj] u16 images; T_old, T_new: n x 16
 * row-major floats (host). Depth only. exact != 0 uses ss_integrate's
 * arithmetic, else ss_integrate_fast's; the volume equals the 2n sequential
 * calls bit for bit. The first call on a grid allocates the batch buffers
 * (64 bytes per hash bucket); n = 0 only allocates them, so that a caller can
 * keep allocation out of a later re-fusion. */
ss_status ss_refuse_batch(ss_grid *g, int32_t n, const uint16_t *const *depths, const float *T_old,
                          const float *T_new, int32_t exact, ss_stream_t s);

/* ---- integration scheduling (src/core/integrate.cpp:47-236) ------------ */

/* Pose (camera -> world, row-major) of six world DoFs (rx, ry, rz, tx, ty,
 * tz): trans(t) Rz(rz) Ry(ry) Rx(rx) (getT, src/utils/matrixutil.h:61-63). */
ss_status ss_dofs_to_pose(const double dofs[6], double T[16]);
/* The DoFs of a pose (MattoDof, src/utils/matrixutil.cpp:37-49). */
ss_status ss_pose_to_dofs(const double T[16], double dofs[6]);
/* updateReintegrationBuffer's order (integrate.cpp:218-236): the indices of
 * n integrated frames sorted by descending pose change (diff,
 * integrate.cpp:205-211: |(rotation DoF deltas, 2 x translation deltas)|
 * between world and integrated DoFs, n x 6 each), stable, keeping those with
 * a change >= treint; order[0..*count). Host only. */
ss_status ss_reintegration_order(int32_t n, const double *world_dofs, const double *integrated_dofs, double treint,
                                 int32_t *order, int32_t *count);

/* The integration thread's frame buffers and schedule
 * (pandia_integration::integrateThreadFunction, integrate.cpp:47-200) as a
 * host object over one grid. Frames are identified by caller ids; their
 * depth images (device, [resi][resj] u16) stay the caller's and must live
 * until the frame is deintegrated. Not thread-safe (the reference guards it
 * with integrationlock). treint: the re-integration threshold (the
 * reference's config: 0.04); max_batch: re-integrations per step, fused as
 * one ss_refuse_batch; exact != 0: ss_integrate's arithmetic. */
typedef struct ss_scheduler ss_scheduler;
ss_status ss_scheduler_create(ss_grid *g, double treint, int32_t max_batch, int32_t exact, ss_scheduler **out);
ss_status ss_scheduler_destroy(ss_scheduler *s);
/* integrationBuffer.push_back: a new frame and its world DoFs. */
ss_status ss_scheduler_push_integrate(ss_scheduler *s, int64_t id, const uint16_t *depth, const double dofs[6]);
/* The frame's world DoFs changed (pose optimisation, Frame::setWorlddofs). */
ss_status ss_scheduler_set_dofs(ss_scheduler *s, int64_t id, const double dofs[6]);
/* deintegrationBuffer.push_back; a frame not yet integrated is just dropped,
 * and the frame leaves the re-integration queue. */
ss_status ss_scheduler_push_deintegrate(ss_scheduler *s, int64_t id);
/* updateReintegrationBuffer: refills the re-integration queue (queued: its
 * length). */
ss_status ss_scheduler_update(ss_scheduler *s, int32_t *queued);
/* The ids in queue which (0 integrate, 1 re-integrate, 2 deintegrate), up to
 * cap of them; count: the queue's length. */
ss_status ss_scheduler_queue(ss_scheduler *s, int32_t which, int32_t cap, int64_t *ids, int32_t *count);
/* One pass of the thread loop: all pending integrations, up to max_batch
 * queued re-integrations (one batched re-fusion), all pending
 * deintegrations; done[3] = the counts. Stream-ordered, no host sync. */
ss_status ss_scheduler_step(ss_scheduler *s, ss_stream_t st, int32_t done[3]);
/* The stop drain (integrate.cpp:160-197): everything queued. */
ss_status ss_scheduler_drain(ss_scheduler *s, ss_stream_t st, int32_t done[3]);
/* Whether frame id is fused, and the DoFs it is fused at. */
ss_status ss_scheduler_frame(ss_scheduler *s, int64_t id, int32_t *integrated, double integrated_dofs[6]);

/* Mesh of the TSDF's zero level set, extracted on the GPU (replaces the host
 * copy into Open3D of marchingCubesHost, GPUVoxelGrid.cpp:200-251): marching
 * tetrahedra over every cell of 8 observed voxel centres (6 tetrahedra per
 * cell along its main diagonal; no cracks between cells), triangles facing
 * from negative to positive sdf, world coordinates. triangles: device float
 * [max_triangles][3][3]; count: the mesh's triangle count, which may exceed
 * max_triangles (then only the first max_triangles were written: call again
 * with a larger buffer). Synchronises s. */
ss_status ss_grid_extract_mesh(ss_grid *g, int64_t max_triangles, float *triangles, int64_t *count, ss_stream_t s);

/* The same mesh by marching cubes, in the cube conventions of the Open3D
 * extraction marchingCubesHost hands the blocks to (GPUVoxelGrid.cpp:200-251:
 * each unit's voxel (x, y, z) is the block's voxel x + 8y + 64z; a cube of 8
 * voxel centres counts when all 8 weights are non-zero; corner bit set for
 * sdf < 0; one vertex per sign-changing edge, interpolated linearly from the
 * edge's lower end). The case table is derived in code (ss_mc_table.h): its
 * polygons equal the classic table's except on cube faces with four
 * crossings (each negative corner cut off), and polygons are fanned from
 * their first vertex. Triangles face from negative to positive sdf; same
 * buffer protocol as ss_grid_extract_mesh. Synchronises s. */
ss_status ss_grid_extract_mesh_cubes(ss_grid *g, int64_t max_triangles, float *triangles, int64_t *count,
                                     ss_stream_t s);

/* Frame ingest help (src/cameras/DataCam.cpp:10-100 reads depth PNGs): undoes
 * the PNG row filters (types 0..4) of rows x (1 + row_bytes) filtered bytes
 * into rows x row_bytes (bpp: bytes per pixel). Host memory, host code. */
ss_status ss_png_unfilter(const uint8_t *filtered, int32_t rows, int32_t row_bytes, int32_t bpp, uint8_t *out);

/* Colour frames (DataCam.cpp:30-46 reads color/<NNNNNN>.jpg first, 66-69
 * resizes them with cv::resize's default, bilinear). A JPEG decoder on the GPU
 * (nvJPEG, loaded at run time: ss_jpeg_create returns SS_ERR_STATE when the
 * CUDA toolkit's libnvjpeg is absent). One decoder per host thread. */
typedef struct ss_jpeg ss_jpeg;
ss_status ss_jpeg_create(ss_jpeg **out);
ss_status ss_jpeg_destroy(ss_jpeg *j);
/* Image size of a JPEG held in host memory (1 or 3 components). */
ss_status ss_jpeg_info(ss_jpeg *j, const uint8_t *data, size_t size, int32_t *rows, int32_t *cols);
/* Decodes a JPEG (host memory) into rgb: device [rows][cols][3] u8, RGB,
 * bilinearly resized when the image's size differs (source coordinate
 * (d + 0.5) src / dst - 0.5, clamped to the border). Enqueued on s (the
 * entropy decoding runs on the calling thread). SS_ERR_ARG for a stream that
 * is not a JPEG nvJPEG supports. */
ss_status ss_jpeg_decode_rgb(ss_jpeg *j, const uint8_t *data, size_t size, uint8_t *rgb, int32_t rows, int32_t cols,
                             ss_stream_t s);
/* The same bilinear resize of a device RGB image (e.g. a PNG colour frame). */
ss_status ss_resize_rgb(const uint8_t *src, int32_t src_rows, int32_t src_cols, uint8_t *dst, int32_t rows,
                        int32_t cols, ss_stream_t s);

/* Synchronises the stream and returns (then clears) the device status word. */
ss_status ss_grid_sync(ss_grid *g, ss_stream_t s);

/* Synchronises the stream and copies the grid counters: out = {live blocks,
 * blocks touched by the last call, blocks touched by all calls, calls,
 * status bits, epoch}. No reference counterpart. */
ss_status ss_grid_counters(ss_grid *g, ss_stream_t s, int64_t out[6]);

/* Synchronises the stream and copies the work counters of ss_raycast summed
 * over all its calls on this grid: out = {hash finds, voxel reads}. They give
 * the raycast's algorithmic bytes (8 B per find, the voxel size per read).
 * No reference counterpart. */
ss_status ss_grid_raycast_counters(ss_grid *g, ss_stream_t s, int64_t out[2]);

/* Test hooks of the failure paths (no reference counterpart); they make a
 * bounded device loop run out without faulting or hanging anything.
 * ss_grid_test_raycast_cap: ss_raycast's per-ray iteration cap (default 2^20,
 * far above the longest march) becomes cap; rays that reach it end without a
 * hit and ss_grid_sync returns SS_ERR_TIMEOUT. cap = 0 restores the default.
 * ss_pipeline_test_wait_timeout: the next tracked frame's persistent tracker
 * waits for one contribution more than its CTAs make, for at most `polls`
 * polls (the default limit is 2^22, about a second): every CTA gives up, the
 * frame keeps its start pose and is fused there, and ss_grid_sync returns
 * SS_ERR_TIMEOUT. That frame runs without the captured graph. SS_ERR_STATE
 * when the pipeline's tracker is not persistent (declared with the pipeline
 * below). */
ss_status ss_grid_test_raycast_cap(ss_grid *g, int32_t cap);

/* Test hook of the exact cross-CTA sums that kokkosICP and the differentiable
 * raycast use (no reference counterpart): the n floats at values (device) are
 * added, each truncated to a multiple of 2^-48, in fixed point by integer
 * atomics from many CTAs; out[0] is the total rounded once to double, out[1]
 * and out[2] the float pair (hi, lo) kokkosICP takes from it. Synchronises s.
 * SS_ERR_ARG for n < 0 or a value of magnitude 2^47 or more. */
ss_status ss_test_fixed48_sum(const float *values, int32_t n, double out[3], ss_stream_t s);

/* Text of the last CUDA error seen by this thread (for SS_ERR_CUDA). */
const char *ss_last_error(void);

/* Number of allocated blocks (synchronises the stream). */
ss_status ss_grid_block_count(ss_grid *g, ss_stream_t s, int32_t *count);

/* Canonical dump of the map, sorted by key (the u64 prime hash), into HOST
 * buffers of room for max_blocks entries: keys, block coords [n][3],
 * sdf [n][512], weight [n][512], rgb [n][3][512] (NULL to skip any).
 * Voxel order inside a block is x + 8y + 64z (GPUVoxelGrid.h:28-31). */
ss_status ss_grid_export_blocks(ss_grid *g, ss_stream_t s, int32_t max_blocks,
                                uint64_t *keys, int32_t *coords, float *sdf,
                                float *weight, float *rgb, int32_t *n_out);

/* Bucket index of each block, in the order of ss_grid_export_blocks (key
 * order): maps payload-layout buffers such as raycast voxel gradients back to
 * blocks. No reference counterpart. */
ss_status ss_grid_export_buckets(ss_grid *g, ss_stream_t s, int32_t max_blocks, int32_t *buckets,
                                 int32_t *n_out);

/* Loads a dump written by ss_grid_export_blocks (checkpoint / resume). */
ss_status ss_grid_import_blocks(ss_grid *g, ss_stream_t s, int32_t n, const int32_t *coords,
                                const float *sdf, const float *weight, const float *rgb);

/* CreatePcdFromDepthView (imageutil.cpp:89-111): pcd [rows][cols][3]. */
ss_status ss_depth_to_pcd(const uint16_t *depth, int32_t rows, int32_t cols, float fx, float fy,
                          float cx, float cy, float *pcd, ss_stream_t s);

/* CalculateNormalsFromPCDView (imageutil.cpp:117-157): normals [rows][cols][3]. */
ss_status ss_normals_from_pcd(const float *pcd, int32_t rows, int32_t cols, float *normals,
                              ss_stream_t s);

/* kokkosICP(View d1, View d2, tx, ty, type, rmse) (kokkosICP.cpp:25-210):
 * aligns depth d1 (pose tx) to depth d2 (pose ty); returns the best relative
 * transform Txy (4x4 row-major, host) and its RMSE. Correspondence search,
 * reductions and the rotation (the polar factor of H^T, which is the SVD's
 * V U^T for a full-rank H) all run on the device; the returned rotation is
 * orthonormal to double precision. The call synchronises s once at the end to
 * return the result, which the last iteration writes into pinned host memory
 * mapped into the device's address space (no copy). Scratch memory (device,
 * and that small pinned buffer) is allocated on the first call per device and
 * reused. The result is bit-reproducible: the cross-CTA sums are exact. */
ss_status ss_kokkos_icp(const uint16_t *d1, const uint16_t *d2, int32_t rows, int32_t cols,
                        float fx, float fy, float cx, float cy, const double tx[16],
                        const double ty[16], int32_t icp_type, double txy_out[16],
                        float *rmse_out, ss_stream_t s);

/* No counterpart in the reference. Same computation, arguments and results as
 * ss_kokkos_icp, but it allocates nothing: for callers that cannot call
 * cudaMalloc while tracking (a real-time thread, or a process whose device
 * memory belongs to its own pool allocator). Its scratch is a fixed 11.1 MB
 * device array that every GPU loading the library holds until exit; rows *
 * cols above 640 x 480 return SS_ERR_DIMS. The first call on a device looks up
 * the array's address and should come before any stream capture; the address
 * is kept for the life of the process, so after a cudaDeviceReset the entry
 * point must not be called on that device again. Calls share the array:
 * calls that overlap on the GPU race and must be serialised. */
ss_status ss_kokkos_icp_noalloc(const uint16_t *d1, const uint16_t *d2, int32_t rows, int32_t cols,
                                float fx, float fy, float cx, float cy, const double tx[16],
                                const double ty[16], int32_t icp_type, double txy_out[16],
                                float *rmse_out, ss_stream_t s);

/* ------------------------------------------------------------------------
 * The per-frame method (no direct reference counterpart: the reference's
 * raycast is nearest-voxel with no normals and no step cap, GPUVoxelGrid.h:377,
 * and its ICP is the host-SVD kokkosICP above).
 */

/* Trilinear raycast: at most max_steps march steps per ray between t_min and
 * t_max (camera-frame depth). vertex_depth [resi][resj][4] = (x, y, z world,
 * depth), normal [resi][resj][4] = (nx, ny, nz, 0) world; misses are zero.
 * hint_depth (may be NULL): a u16-mm depth image taken at this pose; a ray
 * whose pixel has depth d searches only [d - hint_margin, d + hint_margin],
 * a ray without depth starts at the smallest depth of its 32-pixel row
 * segment minus hint_margin (the reference's commented-out "cheat" raycast,
 * GPUVoxelGrid.cpp:150-158, 571-582, starts at d - 0.1 m). */
ss_status ss_raycast_maps(ss_grid *g, const float extr[16], int32_t max_steps, float t_min,
                          float t_max, const uint16_t *hint_depth, float hint_margin,
                          float *vertex_depth, float *normal, ss_stream_t s);

/* Differentiable raycast (no reference counterpart). Renders the model view at
 * pose T (camera -> world, row-major doubles) with the trilinear march (at most
 * max_steps steps) refined by Newton steps to the root of the trilinear field,
 * and returns the loss against depth_obs ([resi][resj] u16 mm, device):
 *   L = sum over valid pixels of r^2 + lambda_n (r n.d)^2,  r = t* - d_obs,
 * (the second term is the squared distance of the observed point to the
 * rendered tangent plane; valid: hit, observation present, |r| < r_max,
 * surface facing the ray). valid_pixels and depth_out ([resi][resj] floats,
 * device, the rendered depth) may be NULL. Synchronises s. */
ss_status ss_raycast_loss(ss_grid *g, const double T[16], const uint16_t *depth_obs, float lambda_n,
                          float r_max, int32_t max_steps, double *loss, int64_t *valid_pixels,
                          float *depth_out, ss_stream_t s);
/* Its adjoint, recomputing the march: grad_pose = dL/d(omega, upsilon) for the
 * left increment T <- exp(xi) T; grad_voxels (device, [buckets][512] floats,
 * the TSDF payload layout, may be NULL) += dL/d(voxel TSDF value in metres).
 * The caller zeroes grad_voxels. Synchronises s. */
ss_status ss_raycast_loss_grad(ss_grid *g, const double T[16], const uint16_t *depth_obs, float lambda_n,
                               float r_max, int32_t max_steps, double *loss, double grad_pose[6],
                               float *grad_voxels, int64_t *valid_pixels, ss_stream_t s);
/* The same restricted to the pixels whose pixel_mask byte ([resi][resj] u8,
 * device) is non-zero (a pixel must also be valid as above): the loss over a
 * fixed pixel set, e.g. to compare the adjoint with finite differences
 * taken with that set frozen. */
ss_status ss_raycast_loss_grad_masked(ss_grid *g, const double T[16], const uint16_t *depth_obs,
                                      const uint8_t *pixel_mask, float lambda_n, float r_max, int32_t max_steps,
                                      double *loss, double grad_pose[6], float *grad_voxels, int64_t *valid_pixels,
                                      ss_stream_t s);

typedef struct ss_pipeline ss_pipeline;

typedef struct ss_pipeline_params {
    int32_t levels;           /* pyramid levels of the tracker (<= 4) */
    int32_t iters[4];         /* Gauss-Newton iterations per level, level 0 = full resolution */
    float dist_thresh[4];     /* correspondence distance gate per level, metres */
    int32_t raycast_steps;    /* march step cap of the model-view raycast */
    float t_min, t_max;       /* raycast depth range */
    int32_t use_graph;        /* replay each tracked frame as one captured CUDA graph */
    int32_t exact_fusion;     /* reference voxel update (rounding, truncated pixel) instead of ss_integrate_fast's */
    float hint_margin;        /* > 0: the model-view raycast starts at the fused frame's depth - hint_margin */
    int32_t persistent_track; /* all tracker iterations in one cooperative launch (else one launch each) */
} ss_pipeline_params;

ss_status ss_pipeline_params_default(ss_pipeline_params *p);
/* The pipeline fuses depth only (no colour) into g, which it borrows. */
ss_status ss_pipeline_create(ss_grid *g, const ss_pipeline_params *p, ss_pipeline **out);
ss_status ss_pipeline_destroy(ss_pipeline *p);
/* Sets the device pose (camera -> world) used by the next untracked frame and
 * as the start of tracking. Synchronises s. */
ss_status ss_pipeline_set_pose(ss_pipeline *p, const double T[16], ss_stream_t s);
/* One-shot ICP start pose (camera -> world, row-major) for the next tracked
 * frame: tracking starts from T instead of the current pose, while the model
 * maps stay those raycast at the current pose. Synchronises s. No reference
 * counterpart (the per-frame pipeline has none). */
ss_status ss_pipeline_set_start(ss_pipeline *p, const double T[16], ss_stream_t s);
/* Copies the current pose to the host. Synchronises s. */
ss_status ss_pipeline_get_pose(ss_pipeline *p, double T[16], ss_stream_t s);
/* Enqueues a copy of the current pose into T (pinned host or device memory)
 * on s without synchronising; valid once s reaches that point. */
ss_status ss_pipeline_read_pose(ss_pipeline *p, double T[16], ss_stream_t s);
/* Device input buffer [resi][resj] u16; frames written there need no copy.
 * It is also one of the two buffers host frames are uploaded into, so a
 * caller that writes frames there should pass only such frames. */
ss_status ss_pipeline_input(ss_pipeline *p, uint16_t **depth);
/* Device model maps of the last frame (layout of ss_raycast_maps). */
ss_status ss_pipeline_maps(ss_pipeline *p, float **vertex_depth, float **normal);
/* One frame: if track != 0 and a model exists, track the frame against the
 * last model view, then integrate at the pose and raycast the model view at
 * it; else integrate at the current pose and raycast. depth may be a device
 * or host pointer. A host frame (pinned for an asynchronous upload) is
 * uploaded on an internal copy stream into one of two input buffers as soon
 * as the frame before last has finished with it, overlapping the previous
 * frame's kernels; s waits for the upload, so the frame must be complete
 * when this is called and stay unchanged until s has passed it. Another
 * device pointer is copied on s. No host sync. */
ss_status ss_pipeline_frame(ss_pipeline *p, const uint16_t *depth, int32_t track, ss_stream_t s);
/* Copies the model maps into caller buffers (device or host), stream-ordered. */
ss_status ss_pipeline_copy_maps(ss_pipeline *p, float *vertex_depth, float *normal, ss_stream_t s);
/* Stage profiling of tracked frames run without the graph: when enabled,
 * events bracket track, collect, fuse, finalize and raycast of each frame;
 * ss_pipeline_stage_ms synchronises s and returns the summed milliseconds
 * per stage, the number of profiled frames and (counters, may be NULL) the
 * raycast's summed hash finds, voxel loads, march steps and hits (enabling
 * resets them all). */
ss_status ss_pipeline_profile(ss_pipeline *p, int32_t enable);
ss_status ss_pipeline_stage_ms(ss_pipeline *p, double ms[5], int64_t *frames, int64_t counters[4],
                               ss_stream_t s);
/* Tracker inliers and residual RMS per level of the last tracked frame. */
ss_status ss_pipeline_stats(ss_pipeline *p, int32_t inliers[4], float rmse[4], ss_stream_t s);
/* Test hook of the tracker's bounded wait (see ss_grid_test_raycast_cap above). */
ss_status ss_pipeline_test_wait_timeout(ss_pipeline *p, int32_t polls);

#ifdef __cplusplus
}
#endif

#endif /* SS_ABI_H */
