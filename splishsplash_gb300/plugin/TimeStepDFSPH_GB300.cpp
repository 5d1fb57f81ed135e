// Reference-side plugin: TimeStepDFSPH_GB300 over libsphgb300 (see TimeStepDFSPH_GB300.h).
#include "TimeStepDFSPH_GB300.h"
#include "Viscosity_Weiler2018_GB300.h"

#include "SPlisHSPlasH/BoundaryModel_Akinci2012.h"
#include "SPlisHSPlasH/Simulation.h"
#include "SPlisHSPlasH/TimeManager.h"
#include "SPlisHSPlasH/XSPH.h"
#include "Utilities/Counting.h"

#include <algorithm>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

using namespace SPH;

namespace
{
	void check(sphgb_ctx *c, int rc)
	{
		if (rc != SPHGB_OK)
			throw std::runtime_error(std::string("sphgb: ") + (c ? sphgb_last_error(c) : "context creation failed"));
	}

	constexpr int kDtype = sizeof(Real) == 8 ? SPHGB_DTYPE_F64 : SPHGB_DTYPE_F32;

	Viscosity_Weiler2018 *weiler(FluidModel *fm)
	{
		return dynamic_cast<Viscosity_Weiler2018 *>(fm->getViscosityBase());
	}
}

TimeStepDFSPH_GB300::TimeStepDFSPH_GB300() : TimeStepDFSPH()
{
	sphgb_config cfg = {};
	cfg.abi_version = SPHGB_ABI_VERSION;
	cfg.device = 0;
	cfg.precision = sizeof(Real) == 8 ? SPHGB_PRECISION_FP64 : SPHGB_PRECISION_FP32;
	cfg.use_graph = 1;   // the step as one CUDA graph with device-side solver loops
	check(nullptr, sphgb_create(&cfg, &m_ctx));
}

TimeStepDFSPH_GB300::~TimeStepDFSPH_GB300()
{
	sphgb_destroy(m_ctx);
}

void TimeStepDFSPH_GB300::reset()
{
	TimeStepDFSPH::reset();
	m_dirty = true;
}

void TimeStepDFSPH_GB300::resize()
{
	TimeStepDFSPH::resize();
	m_dirty = true;
}

void TimeStepDFSPH_GB300::performNeighborhoodSearchSort()
{
	TimeStepDFSPH::performNeighborhoodSearchSort();
	m_dirty = true;
}

void TimeStepDFSPH_GB300::emittedParticles(FluidModel *model, const unsigned int startIndex)
{
	TimeStepDFSPH::emittedParticles(model, startIndex);
	m_dirty = true;
}

void TimeStepDFSPH_GB300::loadState(BinaryFileReader &binReader)
{
	TimeStepDFSPH::loadState(binReader);
	m_dirty = true;
}

// Simulation, DFSPH, XSPH and Weiler2018 parameters of the scene -> sphgb_params
void TimeStepDFSPH_GB300::setParams()
{
	Simulation *sim = Simulation::getCurrent();
	FluidModel *fm = sim->getFluidModel(0);
	sphgb_params p;
	sphgb_default_params(&p);
	p.particle_radius = sim->getParticleRadius();
	p.density0 = fm->getDensity0();
	const Real *g = sim->getVecValue<Real>(Simulation::GRAVITATION);
	for (int d = 0; d < 3; d++)
		p.gravity[d] = g[d];
	p.cfl_method = sim->getValue<int>(Simulation::CFL_METHOD);
	p.cfl_factor = sim->getValue<Real>(Simulation::CFL_FACTOR);
	p.cfl_min_time_step = sim->getValue<Real>(Simulation::CFL_MIN_TIMESTEPSIZE);
	p.cfl_max_time_step = sim->getValue<Real>(Simulation::CFL_MAX_TIMESTEPSIZE);
	p.min_iterations = m_minIterations;
	p.max_iterations = m_maxIterations;
	p.max_error = m_maxError;
	p.enable_divergence_solver = m_enableDivergenceSolver ? 1 : 0;
	p.max_iterations_v = m_maxIterationsV;
	p.max_error_v = m_maxErrorV;
	if (XSPH *xs = fm->getXSPH())
	{
		p.xsph = xs->getValue<Real>(XSPH::FLUID_COEFFICIENT);
		p.xsph_boundary = xs->getValue<Real>(XSPH::BOUNDARY_COEFFICIENT);
	}
	p.viscosity_method = 0;
	if (Viscosity_Weiler2018 *w = weiler(fm))
	{
		p.viscosity_method = 6;
		p.viscosity = w->getValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT);
		p.viscosity_boundary = w->getValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT_BOUNDARY);
		p.visco_max_iter = w->getValue<unsigned int>(Viscosity_Weiler2018::MAX_ITERATIONS);
		p.visco_max_error = w->getValue<Real>(Viscosity_Weiler2018::MAX_ERROR);
	}
	check(m_ctx, sphgb_set_params(m_ctx, &p));
}

// Host vectors -> device: the static Akinci2012 boundary models concatenated, the fluid models
// concatenated in model order (their particles in index order; several models become phases of
// their own rest density), the two warm starts and Weiler2018's velocity difference.
void TimeStepDFSPH_GB300::upload()
{
	Simulation *sim = Simulation::getCurrent();
	std::vector<Real> xb;
	for (unsigned int b = 0; b < sim->numberOfBoundaryModels(); b++)
	{
		BoundaryModel_Akinci2012 *bm = static_cast<BoundaryModel_Akinci2012 *>(sim->getBoundaryModel(b));
		for (unsigned int j = 0; j < bm->numberOfParticles(); j++)
			for (int d = 0; d < 3; d++)
				xb.push_back(bm->getPosition(j)[d]);
	}
	setParams();
	std::vector<Real> x, v, kp, kpv, vd;
	std::vector<uint32_t> counts;
	std::vector<double> rho0;
	bool anyWeiler = false;
	for (unsigned int k = 0; k < sim->numberOfFluidModels(); k++)
	{
		FluidModel *fm = sim->getFluidModel(k);
		const unsigned int n = fm->numActiveParticles();
		for (unsigned int i = 0; i < n; i++)
			for (int d = 0; d < 3; d++)
			{
				x.push_back(fm->getPosition(i)[d]);
				v.push_back(fm->getVelocity(i)[d]);
			}
		for (unsigned int i = 0; i < n; i++)
		{
			kp.push_back(m_simulationData.getPressureRho2(k, i));
			kpv.push_back(m_simulationData.getPressureRho2_V(k, i));
		}
		Viscosity_Weiler2018 *w = weiler(fm);
		anyWeiler = anyWeiler || w != nullptr;
		for (unsigned int i = 0; i < n; i++)
			for (int d = 0; d < 3; d++)
				vd.push_back(w ? w->getVDiff(i)[d] : Real(0));
		counts.push_back(n);
		rho0.push_back(fm->getDensity0());
	}
	const uint32_t n = static_cast<uint32_t>(x.size() / 3);
#ifdef USE_DOUBLE
	check(m_ctx, sphgb_upload_boundary(m_ctx, xb.data(), static_cast<uint32_t>(xb.size() / 3)));
	check(m_ctx, sphgb_upload_fluid(m_ctx, x.data(), v.data(), nullptr, n));
#else
	check(m_ctx, sphgb_upload_boundary_f32(m_ctx, xb.data(), static_cast<uint32_t>(xb.size() / 3)));
	check(m_ctx, sphgb_upload_fluid_f32(m_ctx, x.data(), v.data(), nullptr, n));
#endif
	check(m_ctx, sphgb_upload_field(m_ctx, SPHGB_FIELD_PRESSURE_RHO2, kp.data(), kDtype));
	check(m_ctx, sphgb_upload_field(m_ctx, SPHGB_FIELD_PRESSURE_RHO2_V, kpv.data(), kDtype));
	if (anyWeiler)
		check(m_ctx, sphgb_upload_field(m_ctx, SPHGB_FIELD_VDIFF, vd.data(), kDtype));
	if (counts.size() > 1)
		check(m_ctx, sphgb_set_fluid_phases(m_ctx, static_cast<uint32_t>(counts.size()), counts.data(), rho0.data()));
	m_dirty = false;
}

// Device -> host vectors, model by model, in the order upload() concatenated them
void TimeStepDFSPH_GB300::download()
{
	Simulation *sim = Simulation::getCurrent();
	uint32_t n = 0;
	check(m_ctx, sphgb_num_particles(m_ctx, &n, nullptr));
	// every field in one call (one wait), then handed to the models: model by model in id order
	using Store = std::function<void(FluidModel *, unsigned int, unsigned int, const Real *)>;
	struct Column { int field; int comps; Store store; };
	std::vector<Column> cols = {
		{SPHGB_FIELD_POSITION, 3, [](FluidModel *fm, unsigned, unsigned i, const Real *s) {
			fm->getPosition(i) = Vector3r(s[0], s[1], s[2]); }},
		{SPHGB_FIELD_VELOCITY, 3, [](FluidModel *fm, unsigned, unsigned i, const Real *s) {
			fm->getVelocity(i) = Vector3r(s[0], s[1], s[2]); }},
		{SPHGB_FIELD_ACCELERATION, 3, [](FluidModel *fm, unsigned, unsigned i, const Real *s) {
			fm->getAcceleration(i) = Vector3r(s[0], s[1], s[2]); }},
		{SPHGB_FIELD_DENSITY, 1, [](FluidModel *fm, unsigned, unsigned i, const Real *s) { fm->getDensity(i) = s[0]; }},
		{SPHGB_FIELD_FACTOR, 1, [this](FluidModel *, unsigned k, unsigned i, const Real *s) {
			m_simulationData.getFactor(k, i) = s[0]; }},
		{SPHGB_FIELD_DENSITY_ADV, 1, [this](FluidModel *, unsigned k, unsigned i, const Real *s) {
			m_simulationData.getDensityAdv(k, i) = s[0]; }},
		{SPHGB_FIELD_PRESSURE_RHO2, 1, [this](FluidModel *, unsigned k, unsigned i, const Real *s) {
			m_simulationData.getPressureRho2(k, i) = s[0]; }},
		{SPHGB_FIELD_PRESSURE_RHO2_V, 1, [this](FluidModel *, unsigned k, unsigned i, const Real *s) {
			m_simulationData.getPressureRho2_V(k, i) = s[0]; }},
		{SPHGB_FIELD_PRESSURE_ACCEL, 3, [this](FluidModel *, unsigned k, unsigned i, const Real *s) {
			m_simulationData.getPressureAccel(k, i) = Vector3r(s[0], s[1], s[2]); }},
	};
	bool anyWeiler = false;
	for (unsigned int k = 0; k < sim->numberOfFluidModels(); k++)
		anyWeiler = anyWeiler || weiler(sim->getFluidModel(k)) != nullptr;
	if (anyWeiler)
		cols.push_back({SPHGB_FIELD_VDIFF, 3, [](FluidModel *fm, unsigned, unsigned i, const Real *s) {
			if (Viscosity_Weiler2018 *w = weiler(fm))
				w->getVDiff(i) = Vector3r(s[0], s[1], s[2]);
		}});
	std::vector<std::vector<Real>> bufs(cols.size());
	std::vector<int> ids(cols.size());
	std::vector<void *> dsts(cols.size());
	for (size_t c = 0; c < cols.size(); c++)
	{
		bufs[c].resize(static_cast<size_t>(n) * cols[c].comps);
		ids[c] = cols[c].field;
		dsts[c] = bufs[c].data();
	}
	check(m_ctx, sphgb_download_fields(m_ctx, static_cast<uint32_t>(cols.size()), ids.data(), dsts.data(), kDtype));
	for (size_t c = 0; c < cols.size(); c++)
	{
		size_t off = 0;
		for (unsigned int k = 0; k < sim->numberOfFluidModels(); k++)
		{
			FluidModel *fm = sim->getFluidModel(k);
			const unsigned int m = fm->numActiveParticles();
			for (unsigned int i = 0; i < m; i++)
				cols[c].store(fm, k, i, &bufs[c][off + static_cast<size_t>(i) * cols[c].comps]);
			off += static_cast<size_t>(m) * cols[c].comps;
		}
	}
}

void TimeStepDFSPH_GB300::step()
{
	Simulation *sim = Simulation::getCurrent();
	TimeManager *tm = TimeManager::getCurrent();
	if (m_dirty)
		upload();
	else
		setParams();
	check(m_ctx, sphgb_set_time_step(m_ctx, tm->getTimeStepSize()));
	check(m_ctx, sphgb_set_time(m_ctx, tm->getTime()));
	// the step is queued without a wait; the download waits for it and its fields in one go,
	// after which the step's statistics are on the host
	check(m_ctx, sphgb_step(m_ctx, nullptr));
	download();   // the host vectors stay the system of record
	check(m_ctx, sphgb_sync(m_ctx, &m_stats));
	m_iterations = m_stats.iterations;
	m_iterationsV = m_stats.iterations_v;
	INCREASE_COUNTER("DFSPH - iterations", static_cast<Real>(m_iterations));
	INCREASE_COUNTER("DFSPH - iterationsV", static_cast<Real>(m_iterationsV));
	for (unsigned int k = 0; k < sim->numberOfFluidModels(); k++)
		if (Viscosity_Weiler2018_GB300 *w = dynamic_cast<Viscosity_Weiler2018_GB300 *>(sim->getFluidModel(k)->getViscosityBase()))
			w->setIterations(m_stats.visco_iterations);
	// Simulation::updateTimeStepSize ran on the device (Simulation.cpp:395-493)
	tm->setTimeStepSize(static_cast<Real>(m_stats.dt_next));
	tm->setTime(static_cast<Real>(m_stats.time));
}

void SimulationGB300::install()
{
	// Weiler2018 creator -> GB300 subclass (NonPressureForceRegistration.cpp:58)
	for (NonPressureForceMethod &m : getViscosityMethods())
		if (m.m_name == Viscosity_Weiler2018::METHOD_NAME)
			m.m_creator = Viscosity_Weiler2018_GB300::creator;
	for (unsigned int k = 0; k < numberOfFluidModels(); k++)
	{
		FluidModel *fm = getFluidModel(k);
		if (weiler(fm) && !dynamic_cast<Viscosity_Weiler2018_GB300 *>(fm->getViscosityBase()))
		{
			// recreate the model's viscosity object through the registry, parameters kept
			Viscosity_Weiler2018 *old = weiler(fm);
			const Real nu = old->getValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT);
			const Real nub = old->getValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT_BOUNDARY);
			const unsigned int it = old->getValue<unsigned int>(Viscosity_Weiler2018::MAX_ITERATIONS);
			const Real err = old->getValue<Real>(Viscosity_Weiler2018::MAX_ERROR);
			const unsigned int method = fm->getViscosityMethod();
			fm->setViscosityMethod(0u);
			fm->setViscosityMethod(method);
			NonPressureForceBase *w = fm->getViscosityBase();
			w->setValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT, nu);
			w->setValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT_BOUNDARY, nub);
			w->setValue<unsigned int>(Viscosity_Weiler2018::MAX_ITERATIONS, it);
			w->setValue<Real>(Viscosity_Weiler2018::MAX_ERROR, err);
		}
	}
	// DFSPH -> TimeStepDFSPH_GB300 with the same parameter values (Simulation.cpp:577-583)
	if (getSimulationMethod() == static_cast<int>(SimulationMethods::DFSPH) && m_timeStep &&
		!dynamic_cast<TimeStepDFSPH_GB300 *>(m_timeStep))
	{
		TimeStep *old = m_timeStep;
		const unsigned int minIt = old->getValue<unsigned int>(TimeStepDFSPH::MIN_ITERATIONS);
		const unsigned int maxIt = old->getValue<unsigned int>(TimeStepDFSPH::MAX_ITERATIONS);
		const Real maxErr = old->getValue<Real>(TimeStepDFSPH::MAX_ERROR);
		const unsigned int maxItV = old->getValue<unsigned int>(TimeStepDFSPH::MAX_ITERATIONS_V);
		const Real maxErrV = old->getValue<Real>(TimeStepDFSPH::MAX_ERROR_V);
		const bool divOn = old->getValue<bool>(TimeStepDFSPH::USE_DIVERGENCE_SOLVER);
		m_timeStep = nullptr;
		delete old;   // removes the DFSPH fields, which the new object registers again
		TimeStepDFSPH_GB300 *ts = new TimeStepDFSPH_GB300();
		m_timeStep = ts;
		ts->init();
		ts->setValue<unsigned int>(TimeStepDFSPH::MIN_ITERATIONS, minIt);
		ts->setValue<unsigned int>(TimeStepDFSPH::MAX_ITERATIONS, maxIt);
		ts->setValue<Real>(TimeStepDFSPH::MAX_ERROR, maxErr);
		ts->setValue<unsigned int>(TimeStepDFSPH::MAX_ITERATIONS_V, maxItV);
		ts->setValue<Real>(TimeStepDFSPH::MAX_ERROR_V, maxErrV);
		ts->setValue<bool>(TimeStepDFSPH::USE_DIVERGENCE_SOLVER, divOn);
	}
}
