// Stand-in for the reference's src/core/threadCom.h (test infrastructure): the
// two globals the hot-path sources use (threadCom.h:33, :99).
#pragma once
#include <atomic>

namespace threadCom {
extern std::atomic<bool> unmeshed_data;
}
extern open3d::camera::PinholeCameraIntrinsic g_intrinsic;
