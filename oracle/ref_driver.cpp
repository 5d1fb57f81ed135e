// Test infrastructure: a C interface around the reference's own DFSPH time step,
// compiled from the reference's sources (SPlisHSPlasH/*.cpp, DFSPH/, Viscosity/, ...)
// against the stand-ins in oracle/shims/ by oracle/build_ref.sh.  It is the oracle
// pin: the reference's Simulation, FluidModel, BoundaryModel_Akinci2012,
// TimeStepDFSPH, XSPH and Viscosity_Weiler2018 run unchanged; this file only sets a
// scene up the way the reference's simulator does and reads fields back by particle id.
//
// Set-up order follows Simulator/SimulatorBase.cpp:432-577 (initSimulation,
// buildModel, readParameters, deferredInit) and
// Simulator/StaticBoundarySimulator.cpp:58-190 (static Akinci2012 boundary,
// updateBoundaryVolume).  The simulation method is set after the fluid model
// exists, as readParameters does (Simulation.cpp:535-602), which forces the
// precomputed kernel; `analytic_kernel` then selects the analytic cubic spline
// (setKernel(0); setGradKernel(0)), as the FP64 oracle protocol asks.
// With boundaryMethod 2 the boundary is Bender2019 volume maps: each body is a
// BoundaryModel_Bender2019 whose Discregrid::DiscreteGrid is OracleGrid below, a grid
// evaluated by the oracle's restatement of Discregrid's cubic Lagrange grid
// (oracle/vmap.c; Discregrid itself is not in the reference tree).  The reference's own
// Bender2019 code then runs on it: TimeStep::computeVolumeAndBoundaryX and the Bender2019
// branches of TimeStepDFSPH, XSPH and Viscosity_Weiler2018.
// Only tests/ and bench.py's CPU legs load the library built from this file.
#include "SPlisHSPlasH/Common.h"
#include "SPlisHSPlasH/Simulation.h"
#include "SPlisHSPlasH/TimeManager.h"
#include "SPlisHSPlasH/FluidModel.h"
#include "SPlisHSPlasH/BoundaryModel_Akinci2012.h"
#include "SPlisHSPlasH/BoundaryModel_Bender2019.h"
#include "SPlisHSPlasH/StaticRigidBody.h"
#include "SPlisHSPlasH/TimeStep.h"
#include "SPlisHSPlasH/DFSPH/TimeStepDFSPH.h"
#include "SPlisHSPlasH/XSPH.h"
#include "SPlisHSPlasH/Viscosity/Viscosity_Weiler2018.h"
#include "Utilities/Timing.h"
#include "Utilities/Counting.h"
#include "Utilities/Logger.h"

#include <chrono>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "sph_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

INIT_LOGGING
INIT_TIMING
INIT_COUNTING

using namespace SPH;

extern "C" {

struct RefParams {
    double particleRadius, density0, gravitation[3], timeStepSize;
    int cflMethod;
    double cflFactor, cflMinTimeStepSize, cflMaxTimeStepSize;
    int minIterations, maxIterations;
    double maxError;
    int enableDivergenceSolver, maxIterationsV;
    double maxErrorV;
    double xsph, xsphBoundary;
    int viscosityMethod;   // 0 none, 6 Weiler et al. 2018
    double viscosity, viscosityBoundary;
    int viscoMaxIter;
    double viscoMaxError;
    int analyticKernel;    // 1: setKernel(0); setGradKernel(0) after the parameters
    int numThreads;        // 0: OpenMP default
    int boundaryMethod;    // 0 Akinci2012 (boundary particles), 2 Bender2019 (the volume maps registered)
};

struct RefStats {
    unsigned int iterations, iterationsV, viscoIterations, pad;
    double dtOld, dt, time, stepSeconds;
};

}  // extern "C"

namespace {
StaticRigidBody *g_body = nullptr;
std::vector<Vector3r> g_x, g_v, g_xb;
std::vector<unsigned int> g_objectIds;

// A volume map as the oracle holds it: signed distance (field 0) and volume (field 1) at the
// nodes of the 32-node cubic serendipity grid over [dmin, dmax], body pose R (row-major), t.
struct MapData {
    double dmin[3], dmax[3], R[9], t[3];
    unsigned res[3];
    std::vector<double> f0, f1;
};
std::vector<MapData> g_maps;

// Several fluid models (ref_set_phases): the particles in id order form consecutive groups of
// g_phaseCount[m] particles, model m of rest density g_phaseRho0[m]; the per-model viscosity and
// XSPH coefficients default to the shared parameters where a list is empty.
std::vector<unsigned int> g_phaseCount;
std::vector<double> g_phaseRho0, g_phaseNu, g_phaseNub, g_phaseXs, g_phaseXsb;

// Akinci2012 boundary split into bodies (ref_set_bodies): body of every boundary particle, the
// bodies' reference points and dynamic flags.  A dynamic body is HeldBody: dynamic for
// BoundaryModel::addForce (forces and torques about its position accumulate), but nothing
// integrates its motion, so it stays where it is (the caller's rigid-body solver would move it).
std::vector<unsigned int> g_bodyOf;
std::vector<double> g_bodyCenter;
std::vector<int> g_bodyDynamic;
std::vector<std::vector<Vector3r>> g_bodyX;

class HeldBody : public StaticRigidBody
{
public:
    bool isDynamic() const override { return true; }
};

// The Discregrid grid interface that the reference's Bender2019 code calls, over a MapData.
// determineShapeFunctions reports whether x lies in the grid; interpolate evaluates the field
// (and its gradient) at x with the oracle's grid, so the cell, N and dN that the caller passes
// back are not needed.  Outside the grid the value is the maximum double, as Discregrid's.
class OracleGrid : public Discregrid::DiscreteGrid
{
public:
    explicit OracleGrid(const MapData &d) : m_d(d)
    {
        std::memset(&m_m, 0, sizeof(m_m));
        for (int k = 0; k < 3; k++) {
            m_m.dmin[k] = m_d.dmin[k];
            m_m.dmax[k] = m_d.dmax[k];
            m_m.res[k] = m_d.res[k];
            m_m.t[k] = m_d.t[k];
        }
        for (int k = 0; k < 9; k++) m_m.R[k] = m_d.R[k];
        m_m.field[0] = m_d.f0.data();
        m_m.field[1] = m_d.f1.data();
    }
    bool determineShapeFunctions(unsigned int field, Eigen::Vector3d const &x, std::array<unsigned int, 32> &,
                                 Eigen::Vector3d &, Eigen::Matrix<double, 32, 1> &,
                                 Eigen::Matrix<double, 32, 3> * = nullptr) const override
    {
        double v;
        return orc_vmap_interpolate(&m_m, (int)field, x.data(), &v, nullptr) != 0;
    }
    double interpolate(unsigned int field, Eigen::Vector3d const &x, const std::array<unsigned int, 32> &,
                       const Eigen::Vector3d &, const Eigen::Matrix<double, 32, 1> &, Eigen::Vector3d *gradient = nullptr,
                       Eigen::Matrix<double, 32, 3> * = nullptr) const override
    {
        return eval(field, x, gradient);
    }
    double interpolate(unsigned int field, Eigen::Vector3d const &x, Eigen::Vector3d *gradient = nullptr) const override
    {
        return eval(field, x, gradient);
    }

private:
    MapData m_d;
    orc_vmap m_m;
    double eval(unsigned int field, Eigen::Vector3d const &x, Eigen::Vector3d *gradient) const
    {
        double v, g[3];
        if (!orc_vmap_interpolate(&m_m, (int)field, x.data(), &v, g)) return std::numeric_limits<double>::max();
        if (gradient) *gradient = Eigen::Vector3d(g[0], g[1], g[2]);
        return v;
    }
};

int method_index(std::vector<Simulation::NonPressureForceMethod> &methods, const std::string &name)
{
    for (unsigned int i = 0; i < methods.size(); i++)
        if (methods[i].m_name == name) return methods[i].m_id;
    return -1;
}

FluidModel *model0() { return Simulation::getCurrent()->getFluidModel(0); }

// calls f(model, local index i, particle id) for every particle of every fluid model; ids are
// consecutive over the models in model order
template <class F> void for_particles(F f)
{
    Simulation *sim = Simulation::getCurrent();
    unsigned int off = 0;
    for (unsigned int m = 0; m < sim->numberOfFluidModels(); m++) {
        FluidModel *fm = sim->getFluidModel(m);
        const unsigned int n = fm->numActiveParticles();
        for (unsigned int i = 0; i < n; i++) f(fm, i, off + fm->getParticleId(i));
        off += n;
    }
}

// field -> (pointer getter, components); the names are the reference's field names
Real *field_ptr(FluidModel *fm, int field, unsigned int i, int &dim)
{
    dim = 1;
    switch (field) {
    case 0: dim = 3; return &fm->getPosition(i)[0];
    case 1: dim = 3; return &fm->getVelocity(i)[0];
    case 2: return &fm->getDensity(i);
    case 3: dim = 3; return &fm->getAcceleration(i)[0];
    default: break;
    }
    static const char *names[] = {"factor", "advected density", "p / rho^2", "p_v / rho^2", "pressure acceleration",
                                  "velocity difference"};
    const int k = field - 4;
    if (k < 0 || k >= 6) return nullptr;
    const FieldDescription &fd = fm->getField(names[k]);
    if (fd.name != names[k]) return nullptr;
    dim = fd.type == FieldType::Vector3 ? 3 : 1;
    return static_cast<Real *>(fd.getFct(i));
}
}  // namespace

extern "C" {

/** Builds the scene: n fluid particles (positions x, velocities v, AoS FP64, id = index)
 *  and nb static Akinci2012 boundary particles xb.  Returns 0 on success. */
int ref_create(const RefParams *p, unsigned int n, const double *x, const double *v, unsigned int nb,
               const double *xb)
{
#ifdef _OPENMP
    if (p->numThreads > 0) omp_set_num_threads(p->numThreads);
#endif
    Utilities::Timing::m_dontPrintTimes = true;
    Simulation *sim = Simulation::getCurrent();
    sim->init(static_cast<Real>(p->particleRadius), false);
    const bool maps = p->boundaryMethod == 2;
    if (maps && g_maps.empty()) return 5;
    sim->setBoundaryHandlingMethod(maps ? BoundaryHandlingMethods::Bender2019 : BoundaryHandlingMethods::Akinci2012);

    g_x.resize(n);
    g_v.resize(n);
    g_objectIds.assign(n, 0u);
    for (unsigned int i = 0; i < n; i++) {
        g_x[i] = Vector3r(static_cast<Real>(x[3 * i]), static_cast<Real>(x[3 * i + 1]), static_cast<Real>(x[3 * i + 2]));
        g_v[i] = Vector3r(static_cast<Real>(v[3 * i]), static_cast<Real>(v[3 * i + 1]), static_cast<Real>(v[3 * i + 2]));
    }
    // SimulatorBase::buildModel -> initFluidData: one fluid model per phase, no emitter reserve
    const unsigned int nmodels = g_phaseCount.size() > 1 ? (unsigned int)g_phaseCount.size() : 1u;
    {
        unsigned int off = 0;
        for (unsigned int m = 0; m < nmodels; m++) {
            const unsigned int cnt = nmodels > 1 ? g_phaseCount[m] : n;
            if (off + cnt > n) return 6;
            sim->addFluidModel(nmodels > 1 ? "Fluid" + std::to_string(m) : std::string("Fluid"), cnt,
                               g_x.data() + off, g_v.data() + off, g_objectIds.data() + off, 0u);
            off += cnt;
        }
        if (off != n) return 6;
    }
    sim->setValue(Simulation::KERNEL_METHOD, Simulation::ENUM_KERNEL_PRECOMPUTED_CUBIC);
    sim->setValue(Simulation::GRAD_KERNEL_METHOD, Simulation::ENUM_GRADKERNEL_PRECOMPUTED_CUBIC);

    // SimulatorBase::readParameters: Configuration block, then the material
    Real g[3] = {static_cast<Real>(p->gravitation[0]), static_cast<Real>(p->gravitation[1]),
                 static_cast<Real>(p->gravitation[2])};
    sim->setVecValue<Real>(Simulation::GRAVITATION, g);
    sim->setValue<int>(Simulation::CFL_METHOD, p->cflMethod);
    sim->setValue<Real>(Simulation::CFL_FACTOR, static_cast<Real>(p->cflFactor));
    sim->setValue<Real>(Simulation::CFL_MIN_TIMESTEPSIZE, static_cast<Real>(p->cflMinTimeStepSize));
    sim->setValue<Real>(Simulation::CFL_MAX_TIMESTEPSIZE, static_cast<Real>(p->cflMaxTimeStepSize));
    sim->setValue<int>(Simulation::SIMULATION_METHOD, static_cast<int>(SimulationMethods::DFSPH));
    TimeStep *ts = sim->getTimeStep();
    ts->setValue<unsigned int>(TimeStepDFSPH::MIN_ITERATIONS, static_cast<unsigned int>(p->minIterations));
    ts->setValue<unsigned int>(TimeStepDFSPH::MAX_ITERATIONS, static_cast<unsigned int>(p->maxIterations));
    ts->setValue<Real>(TimeStepDFSPH::MAX_ERROR, static_cast<Real>(p->maxError));
    ts->setValue<bool>(TimeStepDFSPH::USE_DIVERGENCE_SOLVER, p->enableDivergenceSolver != 0);
    ts->setValue<unsigned int>(TimeStepDFSPH::MAX_ITERATIONS_V, static_cast<unsigned int>(p->maxIterationsV));
    ts->setValue<Real>(TimeStepDFSPH::MAX_ERROR_V, static_cast<Real>(p->maxErrorV));

    // each model's material block: rest density, viscosity and XSPH
    auto pick = [&](const std::vector<double> &v, unsigned int m, double shared) {
        return static_cast<Real>(m < v.size() ? v[m] : shared);
    };
    for (unsigned int m = 0; m < nmodels; m++) {
        FluidModel *fm = sim->getFluidModel(m);
        fm->setValue<Real>(FluidModel::DENSITY0, pick(g_phaseRho0, m, p->density0));
        int vm = 0;
        if (p->viscosityMethod == 6) vm = method_index(sim->getViscosityMethods(), Viscosity_Weiler2018::METHOD_NAME);
        else vm = method_index(sim->getViscosityMethods(), "None");
        if (vm < 0) return 2;
        fm->setValue<int>(FluidModel::VISCOSITY_METHOD, vm);
        if (p->viscosityMethod == 6) {
            NonPressureForceBase *visc = fm->getViscosityBase();
            if (!visc) return 3;
            visc->setValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT, pick(g_phaseNu, m, p->viscosity));
            visc->setValue<Real>(Viscosity_Weiler2018::VISCOSITY_COEFFICIENT_BOUNDARY,
                                 pick(g_phaseNub, m, p->viscosityBoundary));
            visc->setValue<unsigned int>(Viscosity_Weiler2018::MAX_ITERATIONS,
                                         static_cast<unsigned int>(p->viscoMaxIter));
            visc->setValue<Real>(Viscosity_Weiler2018::MAX_ERROR, static_cast<Real>(p->viscoMaxError));
        }
        XSPH *xs = fm->getXSPH();
        if (!xs) return 4;
        xs->setValue<Real>(XSPH::FLUID_COEFFICIENT, pick(g_phaseXs, m, p->xsph));
        xs->setValue<Real>(XSPH::BOUNDARY_COEFFICIENT, pick(g_phaseXsb, m, p->xsphBoundary));
    }

    // StaticBoundarySimulator::initBoundaryData: one static body at the identity pose
    g_xb.resize(nb);
    for (unsigned int i = 0; i < nb; i++)
        g_xb[i] = Vector3r(static_cast<Real>(xb[3 * i]), static_cast<Real>(xb[3 * i + 1]),
                           static_cast<Real>(xb[3 * i + 2]));
    if (maps) {
        // StaticBoundarySimulator::initBoundaryData with Bender2019: one static body per map at
        // its pose, a BoundaryModel_Bender2019 holding the map (StaticBoundarySimulator.cpp:167-174)
        for (const MapData &d : g_maps) {
            StaticRigidBody *rb = new StaticRigidBody();
            Matrix3r R;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) R(r, c) = static_cast<Real>(d.R[3 * r + c]);
            const Vector3r t(static_cast<Real>(d.t[0]), static_cast<Real>(d.t[1]), static_cast<Real>(d.t[2]));
            rb->setPosition0(t);
            rb->setPosition(t);
            rb->setRotation0(Quaternionr(R));
            rb->setRotation(Quaternionr(R));
            BoundaryModel_Bender2019 *bm = new BoundaryModel_Bender2019();
            bm->initModel(rb);
            sim->addBoundaryModel(bm);
            bm->setMap(new OracleGrid(d));
        }
    } else if (nb > 0 && !g_bodyDynamic.empty()) {
        // one BoundaryModel_Akinci2012 per body, its particles in upload order, the body's rigid
        // body at its reference point (the torque's centre, BoundaryModel.h:38-49)
        const unsigned int nbodies = (unsigned int)g_bodyDynamic.size();
        g_bodyX.assign(nbodies, {});
        for (unsigned int i = 0; i < nb; i++) {
            if (g_bodyOf[i] >= nbodies) return 7;
            g_bodyX[g_bodyOf[i]].push_back(g_xb[i]);
        }
        for (unsigned int b = 0; b < nbodies; b++) {
            if (g_bodyX[b].empty()) return 7;
            StaticRigidBody *rb = g_bodyDynamic[b] ? new HeldBody() : new StaticRigidBody();
            const Vector3r c(static_cast<Real>(g_bodyCenter[3 * b]), static_cast<Real>(g_bodyCenter[3 * b + 1]),
                             static_cast<Real>(g_bodyCenter[3 * b + 2]));
            rb->setPosition0(c);
            rb->setPosition(c);
            rb->setRotation0(Quaternionr::Identity());
            rb->setRotation(Quaternionr::Identity());
            BoundaryModel_Akinci2012 *bm = new BoundaryModel_Akinci2012();
            bm->initModel(rb, (unsigned int)g_bodyX[b].size(), g_bodyX[b].data());
            sim->addBoundaryModel(bm);
        }
    } else if (nb > 0) {
        g_body = new StaticRigidBody();
        g_body->setPosition0(Vector3r::Zero());
        g_body->setPosition(Vector3r::Zero());
        g_body->setRotation0(Quaternionr::Identity());
        g_body->setRotation(Quaternionr::Identity());
        BoundaryModel_Akinci2012 *bm = new BoundaryModel_Akinci2012();
        bm->initModel(g_body, nb, g_xb.data());
        sim->addBoundaryModel(bm);
    }
    TimeManager::getCurrent()->setTimeStepSize(static_cast<Real>(p->timeStepSize));
    TimeManager::getCurrent()->setTime(0.0);

    // SimulatorBase::deferredInit -> Simulation::deferredInit, StaticBoundarySimulator::deferredInit
    sim->deferredInit();
    sim->performNeighborhoodSearchSort();
    if (!maps && nb > 0) sim->updateBoundaryVolume();
    sim->setSimulationInitialized(true);
    if (p->analyticKernel) {
        sim->setKernel(Simulation::ENUM_KERNEL_CUBIC);
        sim->setGradKernel(Simulation::ENUM_GRADKERNEL_CUBIC);
    }
    return 0;
}

/** One TimeStep::step() of the reference. */
int ref_step(RefStats *out)
{
    Simulation *sim = Simulation::getCurrent();
    TimeManager *tm = TimeManager::getCurrent();
    const double h0 = tm->getTimeStepSize();
    const auto t0 = std::chrono::steady_clock::now();
    sim->getTimeStep()->step();
    const auto t1 = std::chrono::steady_clock::now();
    if (out) {
        TimeStep *ts = sim->getTimeStep();
        out->iterations = ts->getValue<unsigned int>(TimeStepDFSPH::SOLVER_ITERATIONS);
        out->iterationsV = ts->getValue<unsigned int>(TimeStepDFSPH::SOLVER_ITERATIONS_V);
        out->viscoIterations = 0u;   // summed over the fluid models (one system each)
        for (unsigned int m = 0; m < sim->numberOfFluidModels(); m++) {
            NonPressureForceBase *visc = sim->getFluidModel(m)->getViscosityBase();
            if (visc) out->viscoIterations += visc->getValue<unsigned int>(Viscosity_Weiler2018::ITERATIONS);
        }
        out->dtOld = h0;
        out->dt = tm->getTimeStepSize();
        out->time = tm->getTime();
        out->stepSeconds = std::chrono::duration<double>(t1 - t0).count();
    }
    return 0;
}

/** Field of the fluid model in particle-id order (FP64, AoS).  field: 0 position,
 *  1 velocity, 2 density, 3 acceleration, 4 factor, 5 advected density, 6 p / rho^2,
 *  7 p_v / rho^2, 8 pressure acceleration, 9 velocity difference.  Returns the number
 *  of components, or a negative value for an unknown field. */
int ref_get(int field, double *out)
{
    int dim = 0;
    bool ok = true;
    for_particles([&](FluidModel *fm, unsigned int i, unsigned int id) {
        Real *p = field_ptr(fm, field, i, dim);
        if (!p) { ok = false; return; }
        for (int d = 0; d < dim; d++) out[(size_t)id * dim + d] = static_cast<double>(p[d]);
    });
    return ok ? dim : -1;
}

/** Overwrites a field in particle-id order (same numbering as ref_get). */
int ref_set(int field, const double *in)
{
    int dim = 0;
    bool ok = true;
    for_particles([&](FluidModel *fm, unsigned int i, unsigned int id) {
        Real *p = field_ptr(fm, field, i, dim);
        if (!p) { ok = false; return; }
        for (int d = 0; d < dim; d++) p[d] = static_cast<Real>(in[(size_t)id * dim + d]);
    });
    return ok ? dim : -1;
}

/** Akinci2012 boundary volumes in boundary upload order. */
int ref_boundary_volume(double *out)
{
    Simulation *sim = Simulation::getCurrent();
    if (sim->numberOfBoundaryModels() == 0) return 0;
    if (!g_bodyDynamic.empty()) {   // bodies: back to upload order
        std::vector<unsigned int> next(sim->numberOfBoundaryModels(), 0u);
        for (size_t i = 0; i < g_bodyOf.size(); i++) {
            const unsigned int b = g_bodyOf[i];
            BoundaryModel_Akinci2012 *bm = static_cast<BoundaryModel_Akinci2012 *>(sim->getBoundaryModel(b));
            out[i] = static_cast<double>(bm->getVolume(next[b]++));
        }
        return 0;
    }
    BoundaryModel_Akinci2012 *bm = static_cast<BoundaryModel_Akinci2012 *>(sim->getBoundaryModel(0));
    for (unsigned int i = 0; i < bm->numberOfParticles(); i++) out[i] = static_cast<double>(bm->getVolume(i));
    return 0;
}

/** Bodies of the Akinci2012 boundary for the next ref_create: body[i] of boundary particle i,
 *  center (3 per body: the body's position, the torque's centre) and dynamic flags.
 *  nbodies 0 returns to one static body. */
int ref_set_bodies(unsigned int nbodies, unsigned int nb, const unsigned int *body, const double *center,
                   const int *dynamic)
{
    g_bodyOf.clear();
    g_bodyCenter.clear();
    g_bodyDynamic.clear();
    if (nbodies == 0) return 0;
    g_bodyOf.assign(body, body + nb);
    g_bodyCenter.assign(center, center + 3 * (size_t)nbodies);
    g_bodyDynamic.assign(dynamic, dynamic + nbodies);
    return (int)nbodies;
}

/** Force and torque that the fluid exerted on each body since the last clear
 *  (BoundaryModel::getForceAndTorque, summed over the threads); 3 values per body each. */
int ref_body_forces(double *force, double *torque)
{
    Simulation *sim = Simulation::getCurrent();
    for (unsigned int b = 0; b < sim->numberOfBoundaryModels(); b++) {
        Vector3r f, t;
        f.setZero();
        t.setZero();
        if (sim->getBoundaryModel(b)->getRigidBodyObject()->isDynamic())
            sim->getBoundaryModel(b)->getForceAndTorque(f, t);
        for (int d = 0; d < 3; d++) {
            force[3 * b + d] = static_cast<double>(f[d]);
            torque[3 * b + d] = static_cast<double>(t[d]);
        }
    }
    return (int)sim->numberOfBoundaryModels();
}

/** Moves body b (ref_set_bodies) for the next step: rotation R (row-major), position t, linear
 *  velocity v and angular velocity w of its rigid body, then its particles as the simulator places
 *  them before every step (SimulatorBase::updateBoundaryParticles, SimulatorBase.cpp:1617-1645):
 *  x_j = R x0_j + t, v_j = w x (x_j - t) + v.  The body counts as animated from then on. */
int ref_set_body_motion(unsigned int b, const double *R, const double *t, const double *v, const double *w)
{
    Simulation *sim = Simulation::getCurrent();
    if (b >= sim->numberOfBoundaryModels()) return -1;
    BoundaryModel_Akinci2012 *bm = dynamic_cast<BoundaryModel_Akinci2012 *>(sim->getBoundaryModel(b));
    if (!bm) return -1;
    RigidBodyObject *rbo = bm->getRigidBodyObject();
    rbo->setIsAnimated(true);
    Matrix3r Rm;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) Rm(r, c) = static_cast<Real>(R[3 * r + c]);
    rbo->setRotation(Quaternionr(Rm));
    rbo->setPosition(Vector3r(static_cast<Real>(t[0]), static_cast<Real>(t[1]), static_cast<Real>(t[2])));
    rbo->setVelocity(Vector3r(static_cast<Real>(v[0]), static_cast<Real>(v[1]), static_cast<Real>(v[2])));
    rbo->setAngularVelocity(Vector3r(static_cast<Real>(w[0]), static_cast<Real>(w[1]), static_cast<Real>(w[2])));
    const Matrix3r Rq = rbo->getRotation().toRotationMatrix();
    for (unsigned int j = 0; j < bm->numberOfParticles(); j++) {
        bm->getPosition(j) = Rq * bm->getPosition0(j) + rbo->getPosition();
        bm->getVelocity(j) = rbo->getAngularVelocity().cross(bm->getPosition(j) - rbo->getPosition()) + rbo->getVelocity();
    }
    return 0;
}

/** Moves the body of volume map b (boundaryMethod 2) for the next step: its rigid body's rotation
 *  R (row-major), position t, linear velocity v and angular velocity w, the body's CFL radius
 *  max_dist, and its CFL speed bound as the simulator sets it before every step
 *  (SimulatorBase::updateVMVelocity, SimulatorBase.cpp:1670-1687): |w x (max_dist, 0, 0) + v|.
 *  The body counts as animated from then on. */
int ref_set_map_motion(unsigned int b, const double *R, const double *t, const double *v, const double *w,
                       double max_dist)
{
    Simulation *sim = Simulation::getCurrent();
    if (b >= sim->numberOfBoundaryModels()) return -1;
    BoundaryModel_Bender2019 *bm = dynamic_cast<BoundaryModel_Bender2019 *>(sim->getBoundaryModel(b));
    if (!bm) return -1;
    RigidBodyObject *rbo = bm->getRigidBodyObject();
    rbo->setIsAnimated(true);
    Matrix3r Rm;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) Rm(r, c) = static_cast<Real>(R[3 * r + c]);
    rbo->setRotation(Quaternionr(Rm));
    rbo->setPosition(Vector3r(static_cast<Real>(t[0]), static_cast<Real>(t[1]), static_cast<Real>(t[2])));
    rbo->setVelocity(Vector3r(static_cast<Real>(v[0]), static_cast<Real>(v[1]), static_cast<Real>(v[2])));
    rbo->setAngularVelocity(Vector3r(static_cast<Real>(w[0]), static_cast<Real>(w[1]), static_cast<Real>(w[2])));
    bm->setMaxDist(static_cast<Real>(max_dist));
    const Vector3r x(bm->getMaxDist(), 0.0, 0.0);
    bm->setMaxVel((rbo->getAngularVelocity().cross(x) + rbo->getVelocity()).norm());
    return 0;
}

/** BoundaryModel::clearForceAndTorque of every dynamic body. */
void ref_clear_body_forces()
{
    Simulation *sim = Simulation::getCurrent();
    for (unsigned int b = 0; b < sim->numberOfBoundaryModels(); b++)
        if (sim->getBoundaryModel(b)->getRigidBodyObject()->isDynamic()) sim->getBoundaryModel(b)->clearForceAndTorque();
}

/** Fluid and boundary neighbour counts of the last neighbourhood search, by particle id. */
int ref_neighbor_counts(unsigned int *nf, unsigned int *nb)
{
    Simulation *sim = Simulation::getCurrent();
    const unsigned int nm = sim->numberOfFluidModels();
    for (unsigned int m = 0, off = 0; m < nm; m++) {
        FluidModel *fm = sim->getFluidModel(m);
        const unsigned int n = fm->numActiveParticles();
        for (unsigned int i = 0; i < n; i++) {
            const unsigned int id = off + fm->getParticleId(i);
            nf[id] = 0;
            for (unsigned int k = 0; k < nm; k++) nf[id] += sim->numberOfNeighbors(m, k, i);
            nb[id] = 0;
            for (unsigned int k = nm; k < sim->numberOfPointSets(); k++) nb[id] += sim->numberOfNeighbors(m, k, i);
        }
        off += n;
    }
    return 0;
}

void ref_set_time_step(double dt) { TimeManager::getCurrent()->setTimeStepSize(static_cast<Real>(dt)); }

/** Total milliseconds and count of the reference's own timer `name` (START_TIMING /
 *  STOP_TIMING_AVG, e.g. "neighborhood_search", "pressureSolve") since the library loaded;
 *  returns 0 when the timer has not run. */
int ref_timing(const char *name, double *total_ms, unsigned int *count)
{
    for (const auto &kv : Utilities::Timing::m_averageTimes)
        if (kv.second.name == name) {
            *total_ms = kv.second.totalTime;
            *count = kv.second.counter;
            return 1;
        }
    *total_ms = 0.0;
    *count = 0;
    return 0;
}

int ref_precision() { return static_cast<int>(sizeof(Real)); }

/** Registers a volume map for the next ref_create with boundaryMethod 2: the grid's domain and
 *  cells per axis, the node values of the signed distance and of the volume
 *  (orc_vmap_nodes(res) each, the node order of oracle/vmap.c) and the body's pose. */
int ref_add_volume_map(const double *dmin, const double *dmax, const unsigned int *res, const double *f0,
                       const double *f1, const double *R, const double *t)
{
    MapData d;
    for (int k = 0; k < 3; k++) {
        d.dmin[k] = dmin[k];
        d.dmax[k] = dmax[k];
        d.res[k] = res[k];
        d.t[k] = t[k];
    }
    for (int k = 0; k < 9; k++) d.R[k] = R[k];
    const size_t n = orc_vmap_nodes(d.res);
    d.f0.assign(f0, f0 + n);
    d.f1.assign(f1, f1 + n);
    g_maps.push_back(std::move(d));
    return (int)g_maps.size();
}

void ref_clear_volume_maps() { g_maps.clear(); }

/** Several fluid models for the next ref_create: k consecutive groups of count[m] particles
 *  (in id order), model m of rest density rho0[m]; nu, nub (Weiler2018 viscosity and boundary
 *  viscosity) and xs, xsb (XSPH fluid and boundary coefficients) per model, or null for the
 *  shared parameters.  k <= 1 returns to one model. */
int ref_set_phases(unsigned int k, const unsigned int *count, const double *rho0, const double *nu, const double *nub,
                   const double *xs, const double *xsb)
{
    g_phaseCount.clear();
    g_phaseRho0.clear();
    g_phaseNu.clear();
    g_phaseNub.clear();
    g_phaseXs.clear();
    g_phaseXsb.clear();
    if (k <= 1) return 0;
    g_phaseCount.assign(count, count + k);
    g_phaseRho0.assign(rho0, rho0 + k);
    if (nu) g_phaseNu.assign(nu, nu + k);
    if (nub) g_phaseNub.assign(nub, nub + k);
    if (xs) g_phaseXs.assign(xs, xs + k);
    if (xsb) g_phaseXsb.assign(xsb, xsb + k);
    return (int)k;
}

void ref_destroy()
{
    if (Simulation::hasCurrent()) delete Simulation::getCurrent();
    g_body = nullptr;   // the boundary model does not own it; freed with the process
}

}  // extern "C"
