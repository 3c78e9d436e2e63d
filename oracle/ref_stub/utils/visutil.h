// Stand-in for the reference's src/utils/visutil.h (test infrastructure): the
// one declaration GPUVoxelGrid.cpp's debug view uses (visutil.h:30).
#pragma once
#include <memory>

std::shared_ptr<open3d::geometry::LineSet> getOrigin();
