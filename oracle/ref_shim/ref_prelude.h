// Forced-include prelude for compiling the reference's SPHFunctions.cpp with
// g++ (test infrastructure, oracle/_ref only).
//
// * The reference calls std::floorf, an MSVC-ism that libstdc++ does not
//   declare in namespace std; it is forwarded to ::floorf.
// * Noise() (SPHFunctions.cpp:140-144) calls modf(double, float*), which the
//   OpenCL side maps to fract(); a C++ overload with the same meaning is given.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>

namespace std
{
	inline float floorf(float v) { return ::floorf(v); }
}

inline float modf(double value, float* intPart)
{
	double ip = 0.0;
	double frac = ::modf(value, &ip);
	*intPart = static_cast<float>(ip);
	return static_cast<float>(frac);
}
