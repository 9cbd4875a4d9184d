// Stand-in for the Blaze Engine's small vector types (Vec3f, Vec3u, Vec4f).
//
// Test infrastructure only: compiles the reference's SPHFunctions.cpp into
// oracle/_ref.  The Blaze Engine source is absent and unpinned, so its vector
// arithmetic is restated here as plain IEEE component-wise operations:
//   * a + b, a - b, a * s, a / s  act per component (a true divide, never a
//     multiply by a reciprocal);
//   * DotProduct(a, b) = a.x*b.x + a.y*b.y + a.z*b.z, summed left to right.
// Built with -ffp-contract=off so no FMA contraction is introduced.
#pragma once
#include "BlazeEngine/Core/BlazeEngineCoreDefines.h"

namespace Blaze
{
	template<typename T>
	struct Vec3
	{
		T x, y, z;

		constexpr Vec3() : x(0), y(0), z(0) {}
		constexpr explicit Vec3(T v) : x(v), y(v), z(v) {}
		constexpr Vec3(T x, T y, T z) : x(x), y(y), z(z) {}
		template<typename U>
		constexpr explicit Vec3(const Vec3<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}

		constexpr Vec3 operator+(const Vec3& o) const { return Vec3(x + o.x, y + o.y, z + o.z); }
		constexpr Vec3 operator-(const Vec3& o) const { return Vec3(x - o.x, y - o.y, z - o.z); }
		constexpr Vec3 operator*(const Vec3& o) const { return Vec3(x * o.x, y * o.y, z * o.z); }
		constexpr Vec3 operator/(const Vec3& o) const { return Vec3(x / o.x, y / o.y, z / o.z); }
		constexpr Vec3 operator*(T s) const { return Vec3(x * s, y * s, z * s); }
		constexpr Vec3 operator/(T s) const { return Vec3(x / s, y / s, z / s); }
		constexpr Vec3 operator-() const { return Vec3(-x, -y, -z); }

		constexpr Vec3& operator+=(const Vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
		constexpr Vec3& operator-=(const Vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
		constexpr Vec3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
		constexpr Vec3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }

		constexpr T DotProduct(const Vec3& o) const { return x * o.x + y * o.y + z * o.z; }
	};

	template<typename T>
	struct Vec4
	{
		T x, y, z, w;

		constexpr Vec4() : x(0), y(0), z(0), w(0) {}
		constexpr Vec4(T x, T y, T z, T w) : x(x), y(y), z(z), w(w) {}
		constexpr Vec4(const Vec3<T>& v, T w) : x(v.x), y(v.y), z(v.z), w(w) {}

		constexpr Vec3<T> xyz() const { return Vec3<T>(x, y, z); }
	};

	using Vec3f = Vec3<float>;
	using Vec3d = Vec3<double>;
	using Vec3i = Vec3<int32>;
	using Vec3u = Vec3<uint32>;
	using Vec4f = Vec4<float>;
}
