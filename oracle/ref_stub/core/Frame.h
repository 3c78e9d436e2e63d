// Stand-in for the reference's src/core/Frame.h (test infrastructure, builds
// oracle/_ref): only the members the hot-path sources touch — the device
// images (Frame.h:22-23), the id and the world pose used by kokkosICP's Frame
// overload (kokkosICP.cpp:9-13), and MovetoGPU (a no-op: frames stay resident).
#pragma once
#include "VoxelGrid/kokkosFunctions.h"

class Frame {
public:
    Kokkos::View<unsigned char **[3]> rgb;
    Kokkos::View<unsigned short **> depth;
    int unique_id = 0;
    Eigen::Matrix4d frametoworldtrans = Eigen::Matrix4d::Identity();
    void MovetoGPU() {}
    void MovetoCPU() {}
    Eigen::Matrix4d getFrametoWorldTrans() { return frametoworldtrans; }
};
