// Test infrastructure: installs the reference-side plugin (splishsplash_gb300/plugin/) into
// the reference's Simulation driven by oracle/ref_driver.cpp.
//   plugin_use_gb300_simulation()  before ref_create: SimulationGB300 becomes the current Simulation
//   plugin_install()               after ref_create: TimeStepDFSPH_GB300 and the Weiler2018 subclass
//   plugin_destroy()               instead of ref_destroy (deletes through the subclass)
#include "TimeStepDFSPH_GB300.h"
#include "Viscosity_Weiler2018_GB300.h"

using namespace SPH;

extern "C" {
int plugin_use_gb300_simulation()
{
    if (Simulation::hasCurrent()) return 1;
    Simulation::setCurrent(new SimulationGB300());
    return 0;
}
int plugin_install()
{
    SimulationGB300 *sim = dynamic_cast<SimulationGB300 *>(Simulation::getCurrent());
    if (!sim) return 1;
    sim->install();
    if (!dynamic_cast<TimeStepDFSPH_GB300 *>(sim->getTimeStep())) return 2;
    FluidModel *fm = sim->getFluidModel(0);
    if (fm->getViscosityBase() && !dynamic_cast<Viscosity_Weiler2018_GB300 *>(fm->getViscosityBase())) return 3;
    return 0;
}
void plugin_destroy()
{
    if (Simulation::hasCurrent()) delete static_cast<SimulationGB300 *>(Simulation::getCurrent());
}
}
