// Reference-side plugin: Weiler2018 viscosity whose solve runs on the device.
//
// "viscosityMethod": 6 keeps selecting "Weiler et al. 2018" through the creator registry
// (NonPressureForceRegistration.cpp:58).  The GB300 time step runs the whole Weiler2018 solve
// (Viscosity_Weiler2018.cpp:891-1089) inside sphgb_step, so this subclass does nothing in
// step() on the host.  It keeps the parameters ("viscosity", "viscosityBoundary",
// "viscoIterations", "viscoMaxIter", "viscoMaxError", :47-73) that the time step hands to the
// device, and its "velocity difference" field (:33), which the time step refreshes after every
// step and uploads as the warm start after a change on the host.
#pragma once

#include "SPlisHSPlasH/Viscosity/Viscosity_Weiler2018.h"

namespace SPH
{
	class Viscosity_Weiler2018_GB300 : public Viscosity_Weiler2018
	{
	public:
		explicit Viscosity_Weiler2018_GB300(FluidModel *model) : Viscosity_Weiler2018(model) {}
		static NonPressureForceBase *creator(FluidModel *model) { return new Viscosity_Weiler2018_GB300(model); }

		void step() override {}   // runs on the device inside TimeStepDFSPH_GB300::step()

		/** The CG iteration count of the device's last solve ("viscoIterations"). */
		void setIterations(const unsigned int it) { m_iterations = it; }
	};
}
