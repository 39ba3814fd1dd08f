// Test infrastructure (oracle): the one constant the reference kernels use
// from HIP's math-constants header (random.hip.h:50-51,87,
// pathtracer.hip.cpp:107-108).  Same float value as HIP's definition.
#pragma once
#define HIP_PI_F 3.14159265358979f
