// SimulationEngineCUDA: the reference's engine interface (SPH::SimulationEngine,
// SPHFluidSimulation/include/SPH/Core/SimulationEngine.h:35-76) implemented over
// this library's C ABI (sph_gb300.h).  A maintainer adds this header beside
// SimulationEngineCPU in the reference tree, e.g. as
// SPHFluidSimulation/include/SPH/SimulationEngines/SimulationEngineCUDA.h, and
// links libsph_gb300.so.  It compiles against the reference's own SPH/Core
// headers (tests/test_adapter_compiles.py).
#pragma once
#include <cfloat>
#include "SPH/Core/SimulationEngine.h"
#include "SPH/Core/SceneBlueprint.h"
#include "sph_gb300.h"

namespace SPH
{
	class SimulationEngineCUDA : public SimulationEngine
	{
	public:
		explicit SimulationEngineCUDA(int device = 0)
		{
			if (sph_engine_create(&engine, device) != SPH_OK)
				Debug::Logger::LogFatal("SPH Library", sph_last_error());
		}
		~SimulationEngineCUDA() override { Clear(); sph_engine_destroy(engine); }

		void Clear() override
		{
			sph_engine_clear(engine);
			dynamicBM = staticBM = nullptr;
			simulationTime = 0;
		}

		void Initialize(SceneBlueprint& scene, ParticleBufferManager& dyn, ParticleBufferManager& stat) override
		{
			Clear();
			auto parameters = scene.GetSystemParameters();
			float reorderInterval = FLT_MAX;
			parameters.ParseParameter("reorderTimeInterval", reorderInterval);
			const ParticleBehaviourParameters& p = parameters.particleBehaviourParameters;
			sph_params params{ p.particleMass, p.gasConstant, p.elasticity, p.viscosity,
			                   p.gravityX, p.gravityY, p.gravityZ, p.restDensity, p.maxInteractionDistance };

			Array<DynamicParticle> dynamicParticles;
			Array<StaticParticle> staticParticles;
			scene.GenerateLayerParticles("dynamic", dynamicParticles);
			scene.GenerateLayerParticles("static", staticParticles);
			Array<float> dynPos = Positions(dynamicParticles), statPos = Positions(staticParticles);
			auto triangles = scene.GetMesh().CreateTriangleArray();   // 9 floats each

			sph_status st = sph_engine_initialize(engine, &params,
				dynPos.Ptr(), nullptr, (uint32_t)dynamicParticles.Count(),
				statPos.Ptr(), (uint32_t)staticParticles.Count(),
				(const float*)triangles.Ptr(), (uint32_t)triangles.Count(), reorderInterval);
			if (st != SPH_OK) { Debug::Logger::LogError("SPH Library", sph_last_error()); return; }

			// same allocations as SimulationEngineCPU.cpp:471,491 so renderers keep working
			dyn.Allocate(sizeof(DynamicParticle), dynamicParticles.Count(), nullptr, 3);
			{
				ResourceLockGuard guard = dyn.LockWrite(nullptr);
				sph_engine_read_dynamic_buffer(engine, (sph_dynamic_particle*)guard.GetResource());
				guard.Unlock({});
			}
			Array<sph_static_particle> sorted(staticParticles.Count());
			sph_engine_read_static(engine, sorted.Ptr(), nullptr);
			stat.Allocate(sizeof(StaticParticle), staticParticles.Count(), sorted.Ptr(), 1);
			dynamicBM = &dyn;
			staticBM = &stat;
		}

		void Update(float dt, uint simulationStepCount) override
		{
			if (dynamicBM == nullptr) { Debug::Logger::LogWarning("Client", "Updating a uninitialized SPHSystem"); return; }
			if (sph_engine_update(engine, dt, simulationStepCount) != SPH_OK)
				Debug::Logger::LogError("SPH Library", sph_last_error());
			simulationTime += dt * simulationStepCount;
			dynamicBM->Advance();
			ResourceLockGuard guard = dynamicBM->LockWrite(nullptr);
			// the reference's own buffer order, so renderers see what the CPU engine gives them
			sph_engine_read_dynamic_buffer(engine, (sph_dynamic_particle*)guard.GetResource());
			guard.Unlock({});
		}

		StringView SystemImplementationName() override { return "CUDA"; }
		ParticleBufferManager* GetDynamicParticlesBufferManager() override { return dynamicBM; }
		ParticleBufferManager* GetStaticParticlesBufferManager() override { return staticBM; }
		float GetSimulationTime() override { return simulationTime; }

	private:
		template<typename P>
		static Array<float> Positions(const Array<P>& particles)
		{
			Array<float> out(particles.Count() * 3);
			for (uintMem i = 0; i < particles.Count(); ++i)
			{
				out[3 * i + 0] = particles[i].position.x;
				out[3 * i + 1] = particles[i].position.y;
				out[3 * i + 2] = particles[i].position.z;
			}
			return out;
		}

		sph_engine* engine = nullptr;
		ParticleBufferManager* dynamicBM = nullptr;
		ParticleBufferManager* staticBM = nullptr;
		float simulationTime = 0;
	};
}
