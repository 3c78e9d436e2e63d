// ss_gpu_voxel_grid.hpp — header-only C++ shim over ss_abi.h that keeps the
// reference's call surface, so C++ callers written against
// src/VoxelGrid/GPUVoxelGrid.h and src/postprocessing/kokkosICP.h change
// their types, not their calls:
//
//   reference                                         this shim
//   GPUVoxelGrid(c, trunc, voxlength, resi, resj)     ssgb::GPUVoxelGrid(c, trunc, voxlength, resi, resj)
//   grid.setIntrinsic(space, intr)                    grid.setIntrinsic(stream, intr)
//   grid.integrate(space, rgb, depth, extr, color)    grid.integrate(stream, rgb, depth, extr, color)
//   grid.deIntegrate(space, rgb, depth, extr, color)  grid.deIntegrate(stream, rgb, depth, extr, color)
//   grid.raycast(space, extr) -> grid.rayPcd          grid.raycast(stream, extr) -> grid.rayPcd
//   grid.cleanMemory(space)                           grid.cleanMemory(stream)
//   kokkosICP(space, d1, d2, tx, ty, type, &rmse)     ssgb::kokkosICP(stream, d1, d2, rows, cols, intr, tx, ty, type, &rmse, Txy)
//
// Kokkos::View arguments become raw device pointers in row-major [rows][cols]
// layout, the execution-space instance becomes a CUDA stream, and Eigen
// matrices become row-major float[16] / double[16] arrays. Errors throw
// ssgb::Error carrying the ss_status (the reference prints and continues).
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "ss_abi.h"

namespace ssgb {

class Error : public std::runtime_error {
   public:
    Error(ss_status s, const std::string &where)
        : std::runtime_error(where + ": ss_status " + std::to_string((int)s)), status(s) {}
    ss_status status;
};

inline void check(ss_status s, const char *where) {
    if (s != SS_OK) throw Error(s, where);
}

// open3d::camera::PinholeCameraIntrinsic as used by setIntrinsic (GPUVoxelGrid.cpp:257-262)
struct PinholeCameraIntrinsic {
    int width, height;
    float fx, fy, cx, cy;
};

// enum ICPTypes (kokkosICP.h:4-8)
enum ICPTypes { PointToPoint = SS_ICP_POINT_TO_POINT, PointToPlane = SS_ICP_POINT_TO_PLANE };

class GPUVoxelGrid {
   public:
    // GPUVoxelGrid(unsigned int c, float trunc, float voxlength, int resi_, int resj_) (GPUVoxelGrid.h:43)
    GPUVoxelGrid(unsigned int c, float trunc, float voxlength, int resi_, int resj_, int storage = SS_STORAGE_F32,
                 bool with_color = true)
        : d_trunc(trunc), vl(voxlength), vbl(8.f * voxlength), resi(resi_), resj(resj_) {
        ss_params p;
        check(ss_params_default(&p, c, trunc, voxlength, resi_, resj_), "ss_params_default");
        p.storage = storage;
        p.with_color = with_color ? 1 : 0;
        check(ss_grid_create(&p, &grid_), "ss_grid_create");
        const size_t bytes = (size_t)resi * resj * 3 * sizeof(float);
        if (cudaMalloc(&rayPcd, bytes) != cudaSuccess || cudaMalloc(&rayColorPcd, bytes) != cudaSuccess) {
            ss_grid_destroy(grid_);
            throw Error(SS_ERR_NOMEM, "GPUVoxelGrid: ray buffers");
        }
    }
    ~GPUVoxelGrid() {
        cudaFree(rayPcd);
        cudaFree(rayColorPcd);
        ss_grid_destroy(grid_);
    }
    GPUVoxelGrid(const GPUVoxelGrid &) = delete;
    GPUVoxelGrid &operator=(const GPUVoxelGrid &) = delete;

    void setIntrinsic(cudaStream_t, const PinholeCameraIntrinsic &intr) {
        check(ss_grid_set_intrinsic(grid_, intr.fx, intr.fy, intr.cx, intr.cy), "setIntrinsic");
        intrinsicSet = true;
    }
    void integrate(cudaStream_t space, const uint8_t *rgb, const uint16_t *depth, const float extr[16],
                   bool withColor = true) {
        check(ss_integrate(grid_, depth, rgb, extr, withColor ? 1 : 0, (ss_stream_t)space), "integrate");
    }
    void deIntegrate(cudaStream_t space, const uint8_t *rgb, const uint16_t *depth, const float extr[16],
                     bool withColor = true) {
        check(ss_deintegrate(grid_, depth, rgb, extr, withColor ? 1 : 0, (ss_stream_t)space), "deIntegrate");
    }
    void raycast(cudaStream_t space, const float extr[16]) {
        check(ss_raycast(grid_, extr, rayPcd, rayColorPcd, (ss_stream_t)space), "raycast");
    }
    void cleanMemory(cudaStream_t space) { check(ss_clean_memory(grid_, (ss_stream_t)space), "cleanMemory"); }
    // Device-side errors (table full, ...) surface here.
    void sync(cudaStream_t space) { check(ss_grid_sync(grid_, (ss_stream_t)space), "sync"); }
    int blockCount(cudaStream_t space) {
        int32_t n = 0;
        check(ss_grid_block_count(grid_, (ss_stream_t)space, &n), "blockCount");
        return n;
    }
    ss_grid *handle() { return grid_; }

    // members of the reference with the same meaning
    bool intrinsicSet = false;
    float d_trunc, vl, vbl;
    int resi, resj;
    float *rayPcd = nullptr;       // device [resi][resj][3], world coordinates
    float *rayColorPcd = nullptr;  // device [resi][resj][3], colour / 255

   private:
    ss_grid *grid_ = nullptr;
};

// kokkosICP(space, d1, d2, tx, ty, ICPType, rsme) (kokkosICP.cpp:25-210); Txy out, row-major.
inline void kokkosICP(cudaStream_t space, const uint16_t *d1, const uint16_t *d2, int rows, int cols,
                      const PinholeCameraIntrinsic &intr, const double tx[16], const double ty[16], ICPTypes type,
                      float *rsme, double Txy[16]) {
    check(ss_kokkos_icp(d1, d2, rows, cols, intr.fx, intr.fy, intr.cx, intr.cy, tx, ty, (int32_t)type, Txy, rsme,
                        (ss_stream_t)space),
          "kokkosICP");
}

}  // namespace ssgb
