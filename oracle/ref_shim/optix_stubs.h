/* Stand-in (oracle harness only): the host stubs are not needed on the CPU. */
#pragma once
#include "optix.h"
