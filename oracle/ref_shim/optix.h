/* Stand-in for the OptiX SDK header when the reference's device program is
 * compiled as host C++ for the oracle harness (test infrastructure only).
 * Only the handful of names src/OptiX.cu and src/ModelShared.h use exist. */
#pragma once
#include <cuda_runtime.h>
typedef unsigned long long OptixTraversableHandle;
typedef unsigned int OptixVisibilityMask;
enum OptixRayFlags { OPTIX_RAY_FLAG_NONE = 0, OPTIX_RAY_FLAG_TERMINATE_ON_FIRST_HIT = 4 };
