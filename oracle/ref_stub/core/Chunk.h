// Stand-in for the reference's src/core/Chunk.h (test infrastructure): the
// members kokkosICP's Chunk overload reads (kokkosICP.cpp:17-21).
#pragma once
#include <memory>
#include <vector>
#include "core/Frame.h"

class Chunk {
public:
    std::vector<std::shared_ptr<Frame>> frames;
    int unique_id = 0;
    Eigen::Matrix4d chunktoworldtrans = Eigen::Matrix4d::Identity();
};
