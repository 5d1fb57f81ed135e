// C++ host side of the GB300 DFSPH step: the reference's plugin interface for this path,
// restated without the reference's headers and implemented over the C ABI
// (include/sphgb300.h).
//
// Names, parameter names, field names and argument meaning follow SPlisHSPlasH 2.16.0:
//   TimeStep                   SPlisHSPlasH/TimeStep.h:13-59
//   TimeStepDFSPH parameters   SPlisHSPlasH/DFSPH/TimeStepDFSPH.h:57-64, TimeStepDFSPH.cpp:77-114
//   DFSPH fields               TimeStepDFSPH.cpp:49-53, SimulationDataDFSPH.h:55-120
//   FluidModel field layout    SPlisHSPlasH/FluidModel.h:113-124, 247-300
//   Akinci2012 boundary        SPlisHSPlasH/BoundaryModel_Akinci2012.h:32-35
//   forces on boundary bodies  SPlisHSPlasH/BoundaryModel.h:38-49, 86-87; RigidBodyObject.h
//   Bender2019 volume maps     SPlisHSPlasH/BoundaryModel_Bender2019.h, SimulatorBase.cpp:2512-2660
//   Weiler2018 viscosity       SPlisHSPlasH/Viscosity/Viscosity_Weiler2018.h:44-48, .cpp:33,47-73
//   time step size             SPlisHSPlasH/TimeManager.h
// The host vectors are the system of record, as in the reference: step() uploads them when
// they changed, advances the device copy and (with host sync on, the default) downloads the
// fields back in particle-id order.  Errors from the C ABI are thrown as sphgb_host::Error.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "sphgb300.h"

namespace sphgb_host {

#ifdef USE_DOUBLE
using Real = double;
#else
using Real = float;
#endif

// Vector3r stored as three packed Reals (the reference uses Eigen with DontAlign, Common.h:41)
struct Vector3r {
    Real v[3] = {0, 0, 0};
    Vector3r() = default;
    Vector3r(Real x, Real y, Real z) : v{x, y, z} {}
    Real &operator[](int k) { return v[k]; }
    Real operator[](int k) const { return v[k]; }
    Real x() const { return v[0]; }
    Real y() const { return v[1]; }
    Real z() const { return v[2]; }
};
static_assert(sizeof(Vector3r) == 3 * sizeof(Real), "Vector3r must be packed like the reference's");

class Error : public std::runtime_error {
public:
    Error(int code, const std::string &msg) : std::runtime_error(msg), code(code) {}
    int code;
};

// Scene-level parameters (Simulation.cpp:163-277 keys, XSPH.cpp:27-42)
struct SimulationParameters {
    Real particleRadius = Real(0.025);
    Real density0 = Real(1000);
    Vector3r gravitation{0, Real(-9.81), 0};
    int cflMethod = 1;
    Real cflFactor = Real(0.5);
    Real cflMinTimeStepSize = Real(1e-4);
    Real cflMaxTimeStepSize = Real(5e-3);
    Real xsph = Real(0.01);
    Real xsphBoundary = Real(0);
    int viscosityMethod = 0;   // 0 none, 6 "Weiler et al. 2018"
};

// Per-particle data of one fluid phase (FluidModel.h:113-124)
class FluidModel {
public:
    std::vector<Vector3r> m_x0, m_x, m_v0, m_v, m_a;
    std::vector<Real> m_density;
    std::vector<unsigned int> m_particleId;
    Real m_V = 0;
    Real m_density0 = Real(1000);
    // Per-model Weiler2018 viscosity and XSPH coefficients, as each reference FluidModel owns its
    // viscosity and XSPH objects; negative: the time step's shared settings.
    Real m_viscosity = Real(-1), m_viscosityBoundary = Real(-1), m_xsph = Real(-1), m_xsphBoundary = Real(-1);

    void initModel(const std::string &id, unsigned int nFluidParticles, const Vector3r *fluidParticles,
                   const Vector3r *fluidVelocities);
    const std::string &getId() const { return m_id; }
    unsigned int numParticles() const { return (unsigned int)m_x.size(); }
    unsigned int numActiveParticles() const { return numParticles(); }
    Vector3r &getPosition(unsigned int i) { return m_x[i]; }
    Vector3r &getVelocity(unsigned int i) { return m_v[i]; }
    Vector3r &getAcceleration(unsigned int i) { return m_a[i]; }
    Real &getDensity(unsigned int i) { return m_density[i]; }
    Real getDensity0() const { return m_density0; }
    Real getVolume(unsigned int) const { return m_V; }
    Real getMass(unsigned int) const { return m_V * m_density0; }

private:
    std::string m_id;
};

// The rigid body behind a boundary model, as far as the fluid step needs it
// (RigidBodyObject.h: getPosition, isDynamic): the reference point of the torques and
// whether the body collects the fluid's forces.
struct RigidBodyObject {
    Vector3r m_position, m_velocity, m_angularVelocity;
    Real m_rotation[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};   // row-major
    bool m_isDynamic = false, m_isAnimated = false;
    const Real *getRotation() const { return m_rotation; }
    void setRotation(const Real R[9])
    {
        for (int k = 0; k < 9; k++) m_rotation[k] = R[k];
    }
    const Vector3r &getPosition() const { return m_position; }
    void setPosition(const Vector3r &x) { m_position = x; }
    const Vector3r &getVelocity() const { return m_velocity; }
    void setVelocity(const Vector3r &v) { m_velocity = v; }
    const Vector3r &getAngularVelocity() const { return m_angularVelocity; }
    void setAngularVelocity(const Vector3r &w) { m_angularVelocity = w; }
    bool isDynamic() const { return m_isDynamic; }
    void setDynamic(bool d) { m_isDynamic = d; }
    bool isAnimated() const { return m_isAnimated; }
    void setAnimated(bool a) { m_isAnimated = a; }
};

class TimeStepDFSPH_GB300;

// Boundary of one body sampled with particles; volumes computed on the device
// (BoundaryModel_Akinci2012.cpp:48-75).  The particles of a dynamic or animated body are its rest
// shape in body coordinates (getPosition0): every step places them at R x0 + t and moves them with
// the body's velocities, as SimulatorBase::updateBoundaryParticles does (SimulatorBase.cpp:1620-1645).  The forces the fluid exerted on a dynamic body
// accumulate until clearForceAndTorque (BoundaryModel.h:86-87), as the boundary simulator
// reads them (Simulator/BoundarySimulator.cpp:8-25).
class BoundaryModel_Akinci2012 {
public:
    std::vector<Vector3r> m_x;
    std::vector<Real> m_V;
    RigidBodyObject m_rigidBody;
    void initModel(unsigned int numBoundaryParticles, const Vector3r *boundaryParticles);
    unsigned int numberOfParticles() const { return (unsigned int)m_x.size(); }
    Vector3r &getPosition(unsigned int i) { return m_x[i]; }
    Real getVolume(unsigned int i) const { return m_V[i]; }
    RigidBodyObject *getRigidBodyObject() { return &m_rigidBody; }
    // zero until the model belongs to a time step and its body is dynamic
    void getForceAndTorque(Vector3r &force, Vector3r &torque);
    void clearForceAndTorque();

private:
    friend class TimeStepDFSPH_GB300;
    TimeStepDFSPH_GB300 *m_owner = nullptr;
    unsigned int m_index = 0;
};

// TimeStep.h:13-59
class TimeStep {
public:
    virtual ~TimeStep() = default;
    virtual std::string getMethodName() = 0;
    virtual void step() = 0;
    virtual void reset() {}
    virtual void init() {}
    virtual void resize() = 0;
    virtual void emittedParticles(FluidModel *, const unsigned int) {}
    virtual void performNeighborhoodSearchSort() {}
    virtual int getNumIterations() = 0;
};

// Weiler et al. 2018 parameters and "velocity difference" field (Viscosity_Weiler2018.h:44-48)
class Viscosity_Weiler2018_GB300 {
public:
    static int VISCOSITY_COEFFICIENT;
    static int ITERATIONS;
    static int MAX_ITERATIONS;
    static int MAX_ERROR;
    static int VISCOSITY_COEFFICIENT_BOUNDARY;
    static const std::string METHOD_NAME;   // "Weiler et al. 2018"

    Real m_viscosity = Real(0.01);
    Real m_boundaryViscosity = Real(0);
    unsigned int m_maxIter = 100;
    Real m_maxError = Real(0.01);
    unsigned int m_iterations = 0;
    std::vector<Vector3r> m_vDiff;
    Vector3r &getVDiff(unsigned int i) { return m_vDiff[i]; }
};

// Static body given as a volume map (BoundaryModel_Bender2019, the reference's default boundary
// handling): its closed triangle mesh in body coordinates and the scene's map parameters
// ("mapResolution", "mapThickness", "mapInvert"); the map itself is built on the GPU.
class BoundaryModel_Bender2019 {
public:
    std::vector<Vector3r> m_vertices;
    std::vector<unsigned int> m_faces;   // 3 per triangle
    unsigned int m_mapResolution[3] = {20, 20, 20};
    Real m_mapThickness = 0;
    bool m_mapInvert = false;
    Real m_rotation[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};   // body rotation (row-major)
    RigidBodyObject m_rigidBody;                         // position: the body's translation
    void initModel(unsigned int nVertices, const Vector3r *vertices, unsigned int nFaces, const unsigned int *faces)
    {
        m_vertices.assign(vertices, vertices + nVertices);
        m_faces.assign(faces, faces + 3 * (size_t)nFaces);
    }
    RigidBodyObject *getRigidBodyObject() { return &m_rigidBody; }
    // forces of a dynamic body (BoundaryModel.h:86-87); a dynamic or animated body's pose
    // (m_rotation, position) and velocities are handed to the device before every step, as the
    // reference reads them from the rigid body
    void getForceAndTorque(Vector3r &force, Vector3r &torque);
    void clearForceAndTorque();

private:
    friend class TimeStepDFSPH_GB300;
    TimeStepDFSPH_GB300 *m_owner = nullptr;
    unsigned int m_index = 0;
};

// The DFSPH time step on the GPU (TimeStepDFSPH.cpp:117-249)
class TimeStepDFSPH_GB300 : public TimeStep {
public:
    // parameter ids (TimeStepDFSPH.h:57-64)
    static int SOLVER_ITERATIONS;
    static int MIN_ITERATIONS;
    static int MAX_ITERATIONS;
    static int MAX_ERROR;
    static int SOLVER_ITERATIONS_V;
    static int MAX_ITERATIONS_V;
    static int MAX_ERROR_V;
    static int USE_DIVERGENCE_SOLVER;
    static const std::string METHOD_NAME;   // "DFSPH"

    TimeStepDFSPH_GB300(FluidModel &model, BoundaryModel_Akinci2012 &boundary, const SimulationParameters &sim,
                        Viscosity_Weiler2018_GB300 *viscosity = nullptr, int device = 0, bool useGraph = true);
    // one boundary model per rigid body (Simulation::numberOfBoundaryModels)
    TimeStepDFSPH_GB300(FluidModel &model, const std::vector<BoundaryModel_Akinci2012 *> &boundaries,
                        const SimulationParameters &sim, Viscosity_Weiler2018_GB300 *viscosity = nullptr,
                        int device = 0, bool useGraph = true);
    // Bender2019 boundary ("boundaryHandlingMethod" 2): one volume map per static body
    TimeStepDFSPH_GB300(FluidModel &model, const std::vector<BoundaryModel_Bender2019 *> &volumeMaps,
                        const SimulationParameters &sim, Viscosity_Weiler2018_GB300 *viscosity = nullptr,
                        int device = 0, bool useGraph = true);
    ~TimeStepDFSPH_GB300() override;
    TimeStepDFSPH_GB300(const TimeStepDFSPH_GB300 &) = delete;
    TimeStepDFSPH_GB300 &operator=(const TimeStepDFSPH_GB300 &) = delete;

    std::string getMethodName() override { return METHOD_NAME; }
    void step() override;
    void reset() override;
    void init() override { m_dirty = true; }
    void resize() override;
    void emittedParticles(FluidModel *model, const unsigned int startIndex) override;
    void performNeighborhoodSearchSort() override { m_dirty = true; }
    // the boundary models' particles or rigid bodies changed: upload them before the next step
    void updateBoundary() { m_boundaryDirty = m_dirty = true; }
    int getNumIterations() override { return (int)m_iterations; }
    // a further fluid model (Simulation::numberOfFluidModels > 1), before the first step: the
    // models are phases of their own rest density (FluidModel::m_density0); the particle volume
    // is common.  getFluidModel(k) returns model k, the first being the constructor's.
    void addFluidModel(FluidModel &model);
    unsigned int numberOfFluidModels() const { return (unsigned int)m_fluids.size(); }
    FluidModel *getFluidModel(unsigned int k) { return m_fluids[k]; }

    // ParameterObject-style access by id or by the reference's parameter name
    double getValue(int id) const;
    void setValue(int id, double value);
    static int getParameterId(const std::string &name);

    // DFSPH fields by particle index (SimulationDataDFSPH.h:55-120, fields of TimeStepDFSPH.cpp:49-53);
    // with several fluid models by (model, index), as SimulationDataDFSPH holds them
    Real &getFactor(unsigned int i) { return m_factor[i]; }
    Real &getDensityAdv(unsigned int i) { return m_densityAdv[i]; }
    Real &getPressureRho2(unsigned int i) { return m_pressureRho2[i]; }
    Real &getPressureRho2_V(unsigned int i) { return m_pressureRho2V[i]; }
    Vector3r &getPressureAccel(unsigned int i) { return m_pressureAccel[i]; }
    Real &getFactor(unsigned int k, unsigned int i) { return m_factor[offset(k) + i]; }
    Real &getDensityAdv(unsigned int k, unsigned int i) { return m_densityAdv[offset(k) + i]; }
    Real &getPressureRho2(unsigned int k, unsigned int i) { return m_pressureRho2[offset(k) + i]; }
    Real &getPressureRho2_V(unsigned int k, unsigned int i) { return m_pressureRho2V[offset(k) + i]; }
    Vector3r &getPressureAccel(unsigned int k, unsigned int i) { return m_pressureAccel[offset(k) + i]; }

    // TimeManager
    Real getTimeStepSize() const { return m_dt; }
    void setTimeStepSize(Real dt);
    Real getTime() const { return m_time; }

    // download the fields after every step (default, drop-in safe) or only on syncToHost()
    void setHostSync(bool on) { m_hostSync = on; }
    void syncToHost();
    unsigned int getNumIterationsV() const { return m_iterationsV; }
    const sphgb_stats &lastStats() const { return m_stats; }
    sphgb_ctx *context() { return m_ctx; }

protected:
    friend class BoundaryModel_Akinci2012;
    friend class BoundaryModel_Bender2019;
    void check(int rc, const char *what);
    void upload();
    void applyParameters();
    void createContext(int device, bool useGraph);
    void bodyForceAndTorque(unsigned int body, Vector3r &force, Vector3r &torque);
    unsigned int numberOfBodies() const
    {
        return (unsigned int)(m_volumeMaps.empty() ? m_boundaries.size() : m_volumeMaps.size());
    }
    void pushBodyMotion();
    void clearBodyForceAndTorque(unsigned int body);
    unsigned int offset(unsigned int k) const   // first index of model k in the concatenated fields
    {
        unsigned int o = 0;
        for (unsigned int q = 0; q < k; q++) o += m_fluids[q]->numParticles();
        return o;
    }
    unsigned int totalParticles() const { return offset((unsigned int)m_fluids.size()); }

    FluidModel &m_model;
    std::vector<FluidModel *> m_fluids;   // every fluid model, the first being m_model
    std::vector<BoundaryModel_Akinci2012 *> m_boundaries;
    std::vector<BoundaryModel_Bender2019 *> m_volumeMaps;
    bool m_bodiesSet = false;
    SimulationParameters m_sim;
    Viscosity_Weiler2018_GB300 *m_visco;
    sphgb_ctx *m_ctx = nullptr;
    bool m_dirty = true, m_boundaryDirty = true, m_hostSync = true;
    // DFSPH parameters (TimeStepDFSPH.cpp:77-114 defaults)
    unsigned int m_minIterations = 2, m_maxIterations = 100, m_maxIterationsV = 100;
    Real m_maxError = Real(0.01), m_maxErrorV = Real(0.1);
    bool m_enableDivergenceSolver = true;
    unsigned int m_iterations = 0, m_iterationsV = 0;
    Real m_dt = Real(0.001), m_time = 0;
    sphgb_stats m_stats{};
    std::vector<Real> m_factor, m_densityAdv, m_pressureRho2, m_pressureRho2V;
    std::vector<Vector3r> m_pressureAccel;
};

}  // namespace sphgb_host
