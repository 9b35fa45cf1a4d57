// Fixed-width integer types for the device headers: <cstdint> in a normal
// build, plain typedefs when NVRTC compiles a generated network kernel (it
// has no C++ standard library).
#pragma once

#if defined(__CUDACC_RTC__)
typedef signed char int8_t;
typedef short int16_t;
typedef int int32_t;
typedef long long int64_t;
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
typedef unsigned long long uintptr_t;
#else
#include <cstddef>
#include <cstdint>
#endif
