// ref_harness.cpp -- drives the reference's own per-particle code.
//
// TEST INFRASTRUCTURE, built only where the reference sources are present
// (never on the GPU host).  The translation unit includes the reference's
// SPHFluidSimulation/source/SPH/Kernels/SPHFunctions.cpp as it lies (the
// include path is given by oracle/Makefile) on top of the Blaze shim in
// oracle/ref_shim, and wraps the synchronous (threadCount = 0) orchestration
// of SimulationEngineCPU (SimulationEngineCPU.cpp:55-131 for init,
// :132-349 for a step) around the reference's own functions:
//   SPH::Details::ComputeDynamicParticlesHashAndPrepareHashMap  (SF:321-331)
//   SPH::Details::ReorderDynamicParticlesAndFinishHashMap       (SF:332-345)
//   SPH::Details::FillDynamicParticleMapAndFinishHashMap        (SF:346-356)
//   SPH::Details::UpdateParticlePressure                        (SF:358-501)
//   SPH::Details::UpdateParticleDynamics                        (SF:503-656)
// The static-particle sort restates SimulationEngine.h:78-114 around the
// reference's GetCell/GetHash.  Its outputs pin the C restatement in
// oracle/sph_oracle.c and generate the committed golden fixtures.
#include "SPHFunctions.cpp"

#include <cfloat>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

namespace
{
	struct RefEngine
	{
		SPH::ParticleBehaviourParameters params{};
		uint32 n = 0, s = 0, t = 0, buckets = 0;
		std::vector<SPH::DynamicParticle> buffers[3];
		uint32 current = 0;
		std::unique_ptr<std::atomic_uint32_t[]> hashMap;
		std::vector<uint32> particleMap;
		std::vector<uint32> initOrder;
		std::vector<SPH::StaticParticle> statics;
		std::unique_ptr<std::atomic_uint32_t[]> staticMap;
		std::vector<SPH::Triangle> triangles;
		float reorderInterval = FLT_MAX;
		float reorderElapsed = 0;
		double simTime = 0;
	};

	uint32 KeyOf(const Vec3f& p, float h, uint32 mod)
	{
		return SPH::Details::GetHash(SPH::Details::GetCell(p, h)) % mod;
	}
}

extern "C"
{
	__attribute__((visibility("default"))) void* sph_ref_create()
	{
		return new RefEngine();
	}

	__attribute__((visibility("default"))) void sph_ref_destroy(void* e)
	{
		delete static_cast<RefEngine*>(e);
	}

	// Same argument meaning as sph_oracle_init (oracle/sph_oracle.c).
	__attribute__((visibility("default"))) int sph_ref_init(void* handle, const float* params9,
		const float* dynPos, const float* dynVel, uint32 N,
		const float* staticPos, uint32 S, const float* tris, uint32 T, float reorderInterval)
	{
		RefEngine& e = *static_cast<RefEngine*>(handle);
		e = RefEngine();
		SPH::ParticleBehaviourParameters& P = e.params;
		P.particleMass = params9[0];
		P.gasConstant = params9[1];
		P.elasticity = params9[2];
		P.viscosity = params9[3];
		P.gravityX = params9[4];
		P.gravityY = params9[5];
		P.gravityZ = params9[6];
		P.restDensity = params9[7];
		P.maxInteractionDistance = params9[8];
		// SimulationEngineCPU.cpp:406-407
		P.smoothingKernelConstant = SPH::Details::SmoothingKernelConstant(P.maxInteractionDistance);
		P.selfDensity = P.particleMass * SPH::Details::SmoothingKernelD0(0, P.maxInteractionDistance) * P.smoothingKernelConstant;
		e.reorderInterval = reorderInterval;

		// Static particles (SimulationEngineCPU.cpp:460-477, SimulationEngine.h:78-114).
		e.s = S;
		if (S)
		{
			e.staticMap.reset(new std::atomic_uint32_t[S + 1]);
			for (uint32 k = 0; k <= S; ++k) e.staticMap[k] = 0;
			std::vector<uint32> keys(S);
			for (uint32 i = 0; i < S; ++i)
			{
				keys[i] = KeyOf(Vec3f(staticPos[3 * i], staticPos[3 * i + 1], staticPos[3 * i + 2]), P.maxInteractionDistance, S);
				++e.staticMap[keys[i]];
			}
			uint32 sum = 0;
			for (uint32 k = 0; k <= S; ++k) { sum += e.staticMap[k]; e.staticMap[k] = sum; }
			e.statics.resize(S);
			for (uint32 i = 0; i < S; ++i)
			{
				SPH::StaticParticle sp;
				sp.positionAndPressure = Vec4f(Vec3f(staticPos[3 * i], staticPos[3 * i + 1], staticPos[3 * i + 2]), 0.0f);
				e.statics[--e.staticMap[keys[i]]] = sp;
			}
		}

		// Dynamic particles (SimulationEngineCPU.cpp:478-504 and :55-131).
		e.n = N;
		if (N)
		{
			e.buckets = 2 * N;
			e.hashMap.reset(new std::atomic_uint32_t[e.buckets + 1]);
			for (uint32 k = 0; k <= e.buckets; ++k) e.hashMap[k] = 0;
			e.hashMap[e.buckets] = N;
			e.particleMap.assign(N, 0);
			e.initOrder.assign(N, 0);
			for (auto& b : e.buffers) b.assign(N, SPH::DynamicParticle{});
			auto& initial = e.buffers[0];
			for (uint32 i = 0; i < N; ++i)
			{
				initial[i].positionAndPressure = Vec4f(Vec3f(dynPos[3 * i], dynPos[3 * i + 1], dynPos[3 * i + 2]), 0.0f);
				Vec3f v = dynVel ? Vec3f(dynVel[3 * i], dynVel[3 * i + 1], dynVel[3 * i + 2]) : Vec3f(0, 0, 0);
				initial[i].velocityAndHash = Vec4f(v, 0.0f);
			}
			for (uint32 i = 0; i < N; ++i)
				SPH::Details::ComputeDynamicParticlesHashAndPrepareHashMap(i, e.hashMap.get(), e.buckets, initial.data(), P.maxInteractionDistance, N);
			uint32 valueSum = 0;
			for (uint32 k = 0; k < e.buckets; ++k) { valueSum += e.hashMap[k]; e.hashMap[k] = valueSum; }
			// The slot each input particle lands in, replayed from its key with
			// the same decrementing order the reorder below uses.
			{
				std::vector<uint32> tops(e.buckets);
				for (uint32 k = 0; k < e.buckets; ++k) tops[k] = e.hashMap[k];
				for (uint32 i = 0; i < N; ++i)
				{
					float hf = initial[i].velocityAndHash.w;
					uint32 key;
					std::memcpy(&key, &hf, 4);
					e.initOrder[--tops[key]] = i;
				}
			}
			for (uint32 i = 0; i < N; ++i)
				SPH::Details::ReorderDynamicParticlesAndFinishHashMap(i, e.particleMap.data(), e.hashMap.get(), initial.data(), e.buffers[1].data(), N);
			e.current = 1;
		}

		e.t = T;
		e.triangles.resize(T);
		for (uint32 k = 0; k < T; ++k)
		{
			e.triangles[k].p1 = Vec3f(tris[9 * k + 0], tris[9 * k + 1], tris[9 * k + 2]);
			e.triangles[k].p2 = Vec3f(tris[9 * k + 3], tris[9 * k + 4], tris[9 * k + 5]);
			e.triangles[k].p3 = Vec3f(tris[9 * k + 6], tris[9 * k + 7], tris[9 * k + 8]);
		}
		return 0;
	}

	// Update(dt, steps) with threadCount = 0 (SimulationEngineCPU.cpp:420-459
	// and SimulateParticlesTimeStep :132-349, run by one thread).
	__attribute__((visibility("default"))) int sph_ref_update(void* handle, float dt, uint32 steps)
	{
		RefEngine& e = *static_cast<RefEngine*>(handle);
		if (e.n == 0) return 0;
		const bool reorder = e.reorderElapsed > e.reorderInterval;
		const uint64 staticMapSize = e.s ? (uint64)e.s : (uint64)0 - 1;
		for (uint32 step = 0; step < steps; ++step)
		{
			SPH::DynamicParticle* in = e.buffers[e.current].data();
			e.current = (e.current + 1) % 3;
			SPH::DynamicParticle* out = e.buffers[e.current].data();
			for (uint32 i = 0; i < e.n; ++i)
				SPH::Details::UpdateParticlePressure(i, e.n, e.buckets, e.s, staticMapSize, in, out,
					e.hashMap.get(), e.particleMap.data(), e.statics.data(), e.staticMap.get(), &e.params);
			for (uint32 i = 0; i < e.n; ++i)
				SPH::Details::UpdateParticleDynamics(i, e.n, e.buckets, e.s, staticMapSize, in, out,
					e.hashMap.get(), e.particleMap.data(), e.statics.data(), e.staticMap.get(), dt, &e.params,
					e.t, e.triangles.data());
			for (uint32 k = 0; k < e.buckets; ++k) e.hashMap[k].store(0);
			for (uint32 i = 0; i < e.n; ++i)
			{
				float hf = out[i].velocityAndHash.w;
				uint32 key;
				std::memcpy(&key, &hf, 4);
				++e.hashMap[key];
			}
			uint32 valueSum = 0;
			for (uint32 k = 0; k < e.buckets; ++k) { valueSum += e.hashMap[k]; e.hashMap[k] = valueSum; }
			if (reorder)
			{
				e.current = (e.current + 1) % 3;
				SPH::DynamicParticle* ordered = e.buffers[e.current].data();
				for (uint32 i = 0; i < e.n; ++i)
					SPH::Details::ReorderDynamicParticlesAndFinishHashMap(i, e.particleMap.data(), e.hashMap.get(), out, ordered, e.n);
			}
			else
			{
				for (uint32 i = 0; i < e.n; ++i)
					SPH::Details::FillDynamicParticleMapAndFinishHashMap(i, e.particleMap.data(), e.hashMap.get(), out, e.n);
			}
		}
		e.simTime += (double)dt * steps;
		e.reorderElapsed += dt;
		if (e.reorderElapsed > e.reorderInterval) e.reorderElapsed = 0;
		return 0;
	}

	__attribute__((visibility("default"))) void sph_ref_read_raw(void* handle, void* out)
	{
		RefEngine& e = *static_cast<RefEngine*>(handle);
		if (e.n) std::memcpy(out, e.buffers[e.current].data(), sizeof(SPH::DynamicParticle) * e.n);
	}

	__attribute__((visibility("default"))) void sph_ref_read_maps(void* handle, uint32* hashMap, uint32* particleMap, uint32* initOrder)
	{
		RefEngine& e = *static_cast<RefEngine*>(handle);
		if (!e.n) return;
		if (hashMap) for (uint32 k = 0; k <= e.buckets; ++k) hashMap[k] = e.hashMap[k];
		if (particleMap) std::memcpy(particleMap, e.particleMap.data(), 4 * e.n);
		if (initOrder) std::memcpy(initOrder, e.initOrder.data(), 4 * e.n);
	}

	__attribute__((visibility("default"))) void sph_ref_read_static(void* handle, float* pos4, uint32* staticMap)
	{
		RefEngine& e = *static_cast<RefEngine*>(handle);
		if (!e.s) return;
		std::memcpy(pos4, e.statics.data(), sizeof(SPH::StaticParticle) * e.s);
		for (uint32 k = 0; k <= e.s; ++k) staticMap[k] = e.staticMap[k];
	}

	// The reference's own cell key for a position (SF:99-114 then % mod).
	__attribute__((visibility("default"))) void sph_ref_hash(const float* pos, uint32 n, float h, uint32 mod, uint32* keys)
	{
		for (uint32 i = 0; i < n; ++i)
			keys[i] = KeyOf(Vec3f(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), h, mod);
	}
}
