// hc_rtc.h — what the device headers take from the C++ standard library. Under nvcc these
// are the standard headers; under NVRTC (the per-system kernels compiled at run time, which
// have no standard library) the few integer types and type traits are defined here.
#pragma once
#ifdef __CUDACC_RTC__
typedef signed char int8_t;
typedef short int16_t;
typedef int int32_t;
typedef long long int64_t;
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
namespace std {
template <bool B, class T, class F>
struct conditional {
  using type = T;
};
template <class T, class F>
struct conditional<false, T, F> {
  using type = F;
};
template <class A, class B>
struct is_same {
  static constexpr bool value = false;
};
template <class A>
struct is_same<A, A> {
  static constexpr bool value = true;
};
}  // namespace std
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#else
#include <cstdint>
#include <type_traits>
#endif
