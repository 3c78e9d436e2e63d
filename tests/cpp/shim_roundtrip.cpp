// C++ caller of the reference-shaped shim (include/ss_gpu_voxel_grid.hpp):
// integrates a synthetic fronto-parallel wall, raycasts it and runs kokkosICP,
// printing one line that tests/test_cpp_shim.py checks.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "ss_gpu_voxel_grid.hpp"

int main() {
    const int rows = 120, cols = 160;
    ssgb::PinholeCameraIntrinsic intr{cols, rows, 131.25f, 131.25f, 79.5f, 59.5f};
    std::vector<uint16_t> depth(rows * cols, 1500);  // wall at 1.5 m
    std::vector<uint8_t> rgb(rows * cols * 3, 128);
    uint16_t *d_depth = nullptr;
    uint8_t *d_rgb = nullptr;
    cudaMalloc(&d_depth, depth.size() * 2);
    cudaMalloc(&d_rgb, rgb.size());
    cudaMemcpy(d_depth, depth.data(), depth.size() * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(d_rgb, rgb.data(), rgb.size(), cudaMemcpyHostToDevice);
    const float extr[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    try {
        ssgb::GPUVoxelGrid grid(100000000u, 0.02f, 0.005f, rows, cols);
        cudaStream_t s;
        cudaStreamCreate(&s);
        grid.setIntrinsic(s, intr);
        for (int k = 0; k < 3; k++) grid.integrate(s, d_rgb, d_depth, extr);
        grid.raycast(s, extr);
        grid.sync(s);
        std::vector<float> pcd(rows * cols * 3);
        cudaMemcpy(pcd.data(), grid.rayPcd, pcd.size() * 4, cudaMemcpyDeviceToHost);
        int hits = 0;
        double zsum = 0;
        for (int p = 0; p < rows * cols; p++)
            if (pcd[p * 3 + 2] != 0) {
                hits++;
                zsum += pcd[p * 3 + 2];
            }
        const double tx[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        double Txy[16];
        float rmse = 0;
        ssgb::kokkosICP(s, d_depth, d_depth, rows, cols, intr, tx, tx, ssgb::PointToPlane, &rmse, Txy);
        double off = 0;
        for (int k = 0; k < 16; k++) off = std::fmax(off, std::fabs(Txy[k] - tx[k]));
        std::printf("blocks %d hits %d mean_z %.5f icp_offdiag %.3g\n", grid.blockCount(s), hits,
                    hits ? zsum / hits : 0.0, off);
        cudaStreamDestroy(s);
    } catch (const ssgb::Error &e) {
        std::printf("error %s\n", e.what());
        return 1;
    }
    cudaFree(d_depth);
    cudaFree(d_rgb);
    return 0;
}
