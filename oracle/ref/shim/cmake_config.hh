// The configuration header the reference's CMake generates from
// include/cmake_config.hh.in, written out for the oracle/_ref build (test
// infrastructure): double precision always; the Orszag 3/2 convolver unless
// MF_REF_NAIVE is defined; ENABLE_PLT comes from the compiler command line as
// in the reference's CMakeLists.txt:286-288.
#pragma once

#define USE_PRECISION_DOUBLE

#ifdef __cplusplus
constexpr char CMAKE_BUILDTYPE_STR[] = "Release (oracle/_ref)";
constexpr char CMAKE_PRECISION_STR[] = "double";

#if defined(MF_REF_NAIVE)
#define USE_CONVOLVER_NAIVE
constexpr char CMAKE_CONVOLVER_STR[] = "Aliased";
#else
#define USE_CONVOLVER_ORSZAG
constexpr char CMAKE_CONVOLVER_STR[] = "Orszag3/2";
#endif

#if defined(ENABLE_PLT)
constexpr char CMAKE_PLT_STR[] = "PLT corr. on";
#else
constexpr char CMAKE_PLT_STR[] = "PLT corr. off";
#endif

extern "C" {
extern const char* GIT_TAG;
extern const char* GIT_REV;
extern const char* GIT_BRANCH;
}
#endif
