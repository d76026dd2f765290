/* Stand-in (oracle harness only): cudaGraphicsResource is only named by pointer. */
#pragma once
#include <cuda_runtime.h>
