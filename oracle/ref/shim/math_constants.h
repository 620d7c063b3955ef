// Host execution shim: the CUDA math constants the reference uses.
#pragma once
#include <limits>
#define CUDART_NAN (std::numeric_limits<double>::quiet_NaN())
#define CUDART_NAN_F (std::numeric_limits<float>::quiet_NaN())
#define CUDART_INF (std::numeric_limits<double>::infinity())
#define CUDART_PI 3.1415926535897931e+0
#define CUDART_PI_F 3.141592654f
