// Declarations of the Blaze Engine names that the reference's engine headers
// (SPHFluidSimulation/include/SPH/Core/*.h) use, so the C++ adapter
// include/adapter/SimulationEngineCUDA.h can be compiled against those headers with
// `g++ -fsyntax-only` (tests/test_adapter_compiles.py).  Test
// infrastructure: declarations only, nothing here is linked or run.  The
// Blaze Engine itself is an un-vendored dependency of the reference.
#pragma once
#include <cmath>
#include <concepts>
#include <cstring>
#include "BlazeEngine/Core/BlazeEngineCoreDefines.h"
#include "BlazeEngine/Core/Math/Vector.h"

void __debugbreak();

namespace Blaze
{
	class String;
	class StringView
	{
	public:
		StringView();
		StringView(const char* text);
		StringView(const String& text);
		bool operator==(const StringView& other) const;
	};
	class String
	{
	public:
		String();
		String(StringView text);
		String(const char* text);
	};

	template<typename T>
	class Array
	{
	public:
		Array();
		explicit Array(uintMem count);
		T* Ptr();
		const T* Ptr() const;
		uintMem Count() const;
		bool Empty() const;
		void Resize(uintMem count);
		T& operator[](uintMem index);
		const T& operator[](uintMem index) const;
		T& Last();
		T* begin();
		T* end();
		const T* begin() const;
		const T* end() const;
	};

	template<typename T>
	class ArrayView
	{
	public:
		ArrayView();
		ArrayView(const Array<T>& array);
		const T* Ptr() const;
		uintMem Count() const;
		bool Empty() const;
		const T& operator[](uintMem index) const;
		const T& Last() const;
		const T* begin() const;
		const T* end() const;
	};

	template<typename K, typename V>
	class Map
	{
	public:
		struct Node { K key; V value; };
		class Iterator
		{
		public:
			bool IsNull() const;
			Node* operator->() const;
		};
		Iterator Find(StringView key) const;
	};

	class Path;
	class ReadSubStream;

	namespace Debug
	{
		class Logger
		{
		public:
			static void LogDebug(StringView source, StringView message);
			static void LogInfo(StringView source, StringView message);
			static void LogWarning(StringView source, StringView message);
			static void LogError(StringView source, StringView message);
			static void LogFatal(StringView source, StringView message);
		};
	}

	namespace Graphics
	{
		class BasicIndexedMesh
		{
		public:
			struct Triangle { Vec3f p1, p2, p3; };
			Array<Triangle> CreateTriangleArray() const;
		};
	}
}
