// Reference-side plugin: the GB300 DFSPH time step as a SPlisHSPlasH TimeStep.
//
// These files are compiled inside the reference's build, against its own headers
// (SPlisHSPlasH 2.16.0), and link libsphgb300.so.  TimeStepDFSPH_GB300 derives from
// TimeStepDFSPH (SPlisHSPlasH/DFSPH/TimeStepDFSPH.h:24), so it keeps that class's
// parameters ("iterations", "minIterations", "maxIterations", "maxError", "iterationsV",
// "maxIterationsV", "maxErrorV", "enableDivergenceSolver", TimeStepDFSPH.cpp:77-114), its
// fields ("factor", "advected density", "p / rho^2", "p_v / rho^2", "pressure
// acceleration", :49-53) and getMethodName() == "DFSPH", so scene files are unchanged.
// step() replaces TimeStepDFSPH::step() (:117-249): it uploads the host vectors when they
// changed, runs one step on the device through the C ABI and downloads the fields back,
// so the host std::vectors stay the system of record for exporters, saveState and Python.
//
// Installation without editing the reference's files: SimulationGB300 (below) is set as the
// current Simulation before the simulator is initialised; it swaps the DFSPH time step for
// TimeStepDFSPH_GB300 and the Weiler2018 creator for Viscosity_Weiler2018_GB300 through the
// public registry (Simulation::getViscosityMethods, Simulation.h:440).  A build that may
// edit the reference selects the class at Simulation.cpp:577-583 instead.
#pragma once

#include "SPlisHSPlasH/DFSPH/TimeStepDFSPH.h"
#include "SPlisHSPlasH/Simulation.h"
#include "sphgb300.h"

namespace SPH
{
	class TimeStepDFSPH_GB300 : public TimeStepDFSPH
	{
	public:
		TimeStepDFSPH_GB300();
		~TimeStepDFSPH_GB300() override;

		void step() override;
		void reset() override;
		void resize() override;
		void performNeighborhoodSearchSort() override;
		void emittedParticles(FluidModel *model, const unsigned int startIndex) override;
		void loadState(BinaryFileReader &binReader) override;

		/** The device context, for calls of the C ABI that the plugin does not wrap. */
		sphgb_ctx *context() { return m_ctx; }
		/** The statistics of the last step (iteration counts, errors, step sizes). */
		const sphgb_stats &lastStats() const { return m_stats; }
		/** Host vectors were changed outside step(): upload them before the next step. */
		void markHostChanged() { m_dirty = true; }

	protected:
		sphgb_ctx *m_ctx = nullptr;
		sphgb_stats m_stats = {};
		bool m_dirty = true;
		void setParams();
		void upload();
		void download();
	};

	/** A Simulation that runs DFSPH ("simulationMethod": 4) and Weiler2018 ("viscosityMethod":
	 *  6) through libsphgb300.  Make it current before anything calls Simulation::getCurrent():
	 *      Simulation::setCurrent(new SimulationGB300());
	 *  then call install() after the scene's parameters are read (after
	 *  Simulation::setSimulationMethod created the time step). */
	class SimulationGB300 : public Simulation
	{
	public:
		/** Replaces the TimeStepDFSPH created by setSimulationMethod with TimeStepDFSPH_GB300
		 *  (keeping its parameter values) and points the Weiler2018 creator at the GB300
		 *  subclass; models that already hold a Weiler2018 object are switched over. */
		void install();
	};
}
