// Stand-in for the Blaze Engine's core integer typedefs.
//
// The reference's per-particle code (SPHFluidSimulation/source/SPH/Kernels/
// SPHFunctions.cpp) includes this header through CompatibilityHeaderC++.h.
// The Blaze Engine is an un-vendored, unpinned dependency of the reference,
// so this shim restates only the names that file needs.  Test infrastructure:
// it is used to compile the reference's own CPU path into oracle/_ref.
#pragma once
#include <cstdint>
#include <cstddef>

namespace Blaze
{
	using int8 = std::int8_t;
	using int16 = std::int16_t;
	using int32 = std::int32_t;
	using int64 = std::int64_t;
	using uint8 = std::uint8_t;
	using uint16 = std::uint16_t;
	using uint32 = std::uint32_t;
	using uint64 = std::uint64_t;
	using uint = unsigned int;
	using uintMem = std::size_t;
	using intMem = std::ptrdiff_t;
}
