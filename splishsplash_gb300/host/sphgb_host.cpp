// Implementation of the C++ host side (sphgb_host.h) over the C ABI of libsphgb300.so.
#include "sphgb_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sphgb_host {

// parameter ids: the order of TimeStepDFSPH::initParameters (TimeStepDFSPH.cpp:77-114)
int TimeStepDFSPH_GB300::SOLVER_ITERATIONS = 0;
int TimeStepDFSPH_GB300::MIN_ITERATIONS = 1;
int TimeStepDFSPH_GB300::MAX_ITERATIONS = 2;
int TimeStepDFSPH_GB300::MAX_ERROR = 3;
int TimeStepDFSPH_GB300::SOLVER_ITERATIONS_V = 4;
int TimeStepDFSPH_GB300::MAX_ITERATIONS_V = 5;
int TimeStepDFSPH_GB300::MAX_ERROR_V = 6;
int TimeStepDFSPH_GB300::USE_DIVERGENCE_SOLVER = 7;
const std::string TimeStepDFSPH_GB300::METHOD_NAME = "DFSPH";

// Viscosity_Weiler2018::initParameters order (Viscosity_Weiler2018.cpp:47-73)
int Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT = 100;
int Viscosity_Weiler2018_GB300::ITERATIONS = 101;
int Viscosity_Weiler2018_GB300::MAX_ITERATIONS = 102;
int Viscosity_Weiler2018_GB300::MAX_ERROR = 103;
int Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT_BOUNDARY = 104;
const std::string Viscosity_Weiler2018_GB300::METHOD_NAME = "Weiler et al. 2018";

namespace {

// the reference's parameter names (TimeStepDFSPH.cpp:77-114, Viscosity_Weiler2018.cpp:47-73)
struct NamedId {
    const char *name;
    int *id;
};
const NamedId kNames[] = {
    {"iterations", &TimeStepDFSPH_GB300::SOLVER_ITERATIONS},
    {"minIterations", &TimeStepDFSPH_GB300::MIN_ITERATIONS},
    {"maxIterations", &TimeStepDFSPH_GB300::MAX_ITERATIONS},
    {"maxError", &TimeStepDFSPH_GB300::MAX_ERROR},
    {"iterationsV", &TimeStepDFSPH_GB300::SOLVER_ITERATIONS_V},
    {"maxIterationsV", &TimeStepDFSPH_GB300::MAX_ITERATIONS_V},
    {"maxErrorV", &TimeStepDFSPH_GB300::MAX_ERROR_V},
    {"enableDivergenceSolver", &TimeStepDFSPH_GB300::USE_DIVERGENCE_SOLVER},
    {"viscosity", &Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT},
    {"viscoIterations", &Viscosity_Weiler2018_GB300::ITERATIONS},
    {"viscoMaxIter", &Viscosity_Weiler2018_GB300::MAX_ITERATIONS},
    {"viscoMaxError", &Viscosity_Weiler2018_GB300::MAX_ERROR},
    {"viscosityBoundary", &Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT_BOUNDARY},
};

constexpr int kDtype = sizeof(Real) == 8 ? SPHGB_DTYPE_F64 : SPHGB_DTYPE_F32;

std::vector<double> to_double(const std::vector<Vector3r> &a)
{
    std::vector<double> d(a.size() * 3);
    for (size_t i = 0; i < a.size(); i++)
        for (int k = 0; k < 3; k++) d[3 * i + k] = (double)a[i][k];
    return d;
}

}  // namespace

void FluidModel::initModel(const std::string &id, unsigned int n, const Vector3r *x, const Vector3r *v)
{
    // FluidModel::initModel (FluidModel.cpp:285-327): x0 = x, v0 = v, a = 0, id = creation index;
    // volume V = 0.8 (2r)^3 is set by the time step from the particle radius (FluidModel.cpp:234-253)
    m_id = id;
    m_x.assign(x, x + n);
    m_x0 = m_x;
    m_v.assign(v, v + n);
    m_v0 = m_v;
    m_a.assign(n, Vector3r());
    m_density.assign(n, Real(0));
    m_particleId.resize(n);
    for (unsigned int i = 0; i < n; i++) m_particleId[i] = i;
}

void BoundaryModel_Akinci2012::initModel(unsigned int n, const Vector3r *x)
{
    m_x.assign(x, x + n);
    m_V.assign(n, Real(0));
}

void BoundaryModel_Akinci2012::getForceAndTorque(Vector3r &force, Vector3r &torque)
{
    force = torque = Vector3r();
    if (m_owner && m_rigidBody.isDynamic()) m_owner->bodyForceAndTorque(m_index, force, torque);
}

void BoundaryModel_Akinci2012::clearForceAndTorque()
{
    if (m_owner && m_rigidBody.isDynamic()) m_owner->clearBodyForceAndTorque(m_index);
}

void BoundaryModel_Bender2019::getForceAndTorque(Vector3r &force, Vector3r &torque)
{
    force = torque = Vector3r();
    if (m_owner && m_rigidBody.isDynamic()) m_owner->bodyForceAndTorque(m_index, force, torque);
}

void BoundaryModel_Bender2019::clearForceAndTorque()
{
    if (m_owner && m_rigidBody.isDynamic()) m_owner->clearBodyForceAndTorque(m_index);
}

TimeStepDFSPH_GB300::TimeStepDFSPH_GB300(FluidModel &model, BoundaryModel_Akinci2012 &boundary,
                                         const SimulationParameters &sim, Viscosity_Weiler2018_GB300 *viscosity,
                                         int device, bool useGraph)
    : m_model(model), m_boundaries{&boundary}, m_sim(sim), m_visco(viscosity)
{
    createContext(device, useGraph);
}

TimeStepDFSPH_GB300::TimeStepDFSPH_GB300(FluidModel &model, const std::vector<BoundaryModel_Akinci2012 *> &boundaries,
                                         const SimulationParameters &sim, Viscosity_Weiler2018_GB300 *viscosity,
                                         int device, bool useGraph)
    : m_model(model), m_boundaries(boundaries), m_sim(sim), m_visco(viscosity)
{
    createContext(device, useGraph);
}

TimeStepDFSPH_GB300::TimeStepDFSPH_GB300(FluidModel &model, const std::vector<BoundaryModel_Bender2019 *> &volumeMaps,
                                         const SimulationParameters &sim, Viscosity_Weiler2018_GB300 *viscosity,
                                         int device, bool useGraph)
    : m_model(model), m_volumeMaps(volumeMaps), m_sim(sim), m_visco(viscosity)
{
    for (BoundaryModel_Bender2019 *b : m_volumeMaps) {
        if (!b) throw Error(SPHGB_ERR_ARGUMENT, "null boundary model");
        if (b->m_owner) throw Error(SPHGB_ERR_STATE, "boundary model already belongs to a time step");
    }
    createContext(device, useGraph);
    for (unsigned int k = 0; k < m_volumeMaps.size(); k++) {
        m_volumeMaps[k]->m_owner = this;
        m_volumeMaps[k]->m_index = k;
    }
}

void TimeStepDFSPH_GB300::createContext(int device, bool useGraph)
{
    for (unsigned int k = 0; k < m_boundaries.size(); k++) {
        if (!m_boundaries[k]) throw Error(SPHGB_ERR_ARGUMENT, "null boundary model");
        if (m_boundaries[k]->m_owner) throw Error(SPHGB_ERR_STATE, "boundary model already belongs to a time step");
    }
    sphgb_config cfg{};
    cfg.abi_version = SPHGB_ABI_VERSION;
    cfg.device = device;
    cfg.precision = sizeof(Real) == 8 ? SPHGB_PRECISION_FP64 : SPHGB_PRECISION_FP32;
    cfg.use_graph = useGraph ? 1 : 0;
    const int rc = sphgb_create(&cfg, &m_ctx);
    if (rc != SPHGB_OK) throw Error(rc, "sphgb_create failed (no CUDA device?)");
    const Real d = Real(2) * m_sim.particleRadius;
    m_model.m_V = Real(0.8) * d * d * d;
    m_model.m_density0 = m_sim.density0;
    m_fluids.assign(1, &m_model);
    applyParameters();
    for (unsigned int k = 0; k < m_boundaries.size(); k++) {
        m_boundaries[k]->m_owner = this;
        m_boundaries[k]->m_index = k;
    }
}

TimeStepDFSPH_GB300::~TimeStepDFSPH_GB300()
{
    for (BoundaryModel_Akinci2012 *b : m_boundaries) b->m_owner = nullptr;
    for (BoundaryModel_Bender2019 *b : m_volumeMaps) b->m_owner = nullptr;
    if (m_ctx) sphgb_destroy(m_ctx);
}

void TimeStepDFSPH_GB300::bodyForceAndTorque(unsigned int body, Vector3r &force, Vector3r &torque)
{
    if (!m_bodiesSet) return;
    std::vector<double> f(3 * (size_t)numberOfBodies()), t(3 * (size_t)numberOfBodies());
    check(sphgb_boundary_forces(m_ctx, f.data(), t.data()), "sphgb_boundary_forces");
    for (int d = 0; d < 3; d++) {
        force[d] = (Real)f[3 * body + d];
        torque[d] = (Real)t[3 * body + d];
    }
}

void TimeStepDFSPH_GB300::clearBodyForceAndTorque(unsigned int body)
{
    if (m_bodiesSet) check(sphgb_clear_boundary_forces(m_ctx, (int32_t)body), "sphgb_clear_boundary_forces");
}

void TimeStepDFSPH_GB300::check(int rc, const char *what)
{
    if (rc != SPHGB_OK) throw Error(rc, std::string(what) + ": " + sphgb_last_error(m_ctx));
}

void TimeStepDFSPH_GB300::applyParameters()
{
    sphgb_params p;
    sphgb_default_params(&p);
    p.particle_radius = m_sim.particleRadius;
    p.density0 = m_sim.density0;
    for (int k = 0; k < 3; k++) p.gravity[k] = m_sim.gravitation[k];
    p.cfl_method = m_sim.cflMethod;
    p.cfl_factor = m_sim.cflFactor;
    p.cfl_min_time_step = m_sim.cflMinTimeStepSize;
    p.cfl_max_time_step = m_sim.cflMaxTimeStepSize;
    p.min_iterations = m_minIterations;
    p.max_iterations = m_maxIterations;
    p.max_error = m_maxError;
    p.enable_divergence_solver = m_enableDivergenceSolver ? 1 : 0;
    p.max_iterations_v = m_maxIterationsV;
    p.max_error_v = m_maxErrorV;
    p.xsph = m_sim.xsph;
    p.xsph_boundary = m_sim.xsphBoundary;
    p.viscosity_method = (m_visco && m_sim.viscosityMethod == 6) ? 6 : 0;
    if (m_visco) {
        p.viscosity = m_visco->m_viscosity;
        p.viscosity_boundary = m_visco->m_boundaryViscosity;
        p.visco_max_iter = m_visco->m_maxIter;
        p.visco_max_error = m_visco->m_maxError;
    }
    check(sphgb_set_params(m_ctx, &p), "sphgb_set_params");
}

void TimeStepDFSPH_GB300::addFluidModel(FluidModel &model)
{
    for (FluidModel *f : m_fluids)
        if (f == &model) throw Error(SPHGB_ERR_ARGUMENT, "fluid model added twice");
    model.m_V = m_model.m_V;   // the particle volume follows the radius, common to all models
    m_fluids.push_back(&model);
    resize();
}

void TimeStepDFSPH_GB300::resize()
{
    const unsigned int n = totalParticles();
    m_factor.resize(n, Real(0));
    m_densityAdv.resize(n, Real(0));
    m_pressureRho2.resize(n, Real(0));
    m_pressureRho2V.resize(n, Real(0));
    m_pressureAccel.resize(n, Vector3r());
    if (m_visco) m_visco->m_vDiff.resize(n, Vector3r());
    m_dirty = true;
}

void TimeStepDFSPH_GB300::reset()
{
    // TimeStepDFSPH::reset (TimeStepDFSPH.cpp:709-717): warm starts and iteration counts cleared
    std::fill(m_pressureRho2.begin(), m_pressureRho2.end(), Real(0));
    std::fill(m_pressureRho2V.begin(), m_pressureRho2V.end(), Real(0));
    if (m_visco) std::fill(m_visco->m_vDiff.begin(), m_visco->m_vDiff.end(), Vector3r());
    m_iterations = m_iterationsV = 0;
    m_time = 0;
    m_dirty = true;
}

void TimeStepDFSPH_GB300::emittedParticles(FluidModel *, const unsigned int)
{
    resize();   // new particles were appended to the host vectors: upload before the next step
}

void TimeStepDFSPH_GB300::setTimeStepSize(Real dt)
{
    m_dt = dt;
    if (!m_dirty) check(sphgb_set_time_step(m_ctx, dt), "sphgb_set_time_step");
}

// Host vectors -> device (the host vectors are the system of record).  Particle ids are the
// host indices, so downloads come back in host order.
void TimeStepDFSPH_GB300::upload()
{
    const unsigned int n = totalParticles();
    if (m_factor.size() != n) resize();
    if (m_boundaryDirty && !m_volumeMaps.empty()) {
        // Bender2019: no boundary particles; one map per body, built for the current parameters
        check(sphgb_upload_boundary(m_ctx, nullptr, 0), "sphgb_upload_boundary");
        check(sphgb_clear_volume_maps(m_ctx), "sphgb_clear_volume_maps");
        for (BoundaryModel_Bender2019 *bm : m_volumeMaps) {
            const std::vector<double> v = to_double(bm->m_vertices);
            double R[9], t[3];
            for (int k = 0; k < 9; k++) R[k] = (double)bm->m_rotation[k];
            for (int k = 0; k < 3; k++) t[k] = (double)bm->m_rigidBody.getPosition()[k];
            uint32_t body;
            check(sphgb_add_volume_map(m_ctx, v.data(), (uint32_t)bm->m_vertices.size(), bm->m_faces.data(),
                                       (uint32_t)(bm->m_faces.size() / 3), bm->m_mapResolution, (double)bm->m_mapThickness,
                                       bm->m_mapInvert ? 1 : 0, R, t, 0, &body),
                  "sphgb_add_volume_map");
        }
        check(sphgb_set_boundary_method(m_ctx, 2), "sphgb_set_boundary_method");
        // map k is body k; forces only where a body is dynamic
        std::vector<double> center;
        std::vector<int> dynamic;
        bool anyDynamic = false;
        for (BoundaryModel_Bender2019 *bm : m_volumeMaps) {
            for (int d = 0; d < 3; d++) center.push_back((double)bm->m_rigidBody.getPosition()[d]);
            dynamic.push_back(bm->m_rigidBody.isDynamic() ? 1 : 0);
            anyDynamic = anyDynamic || bm->m_rigidBody.isDynamic();
        }
        check(sphgb_set_boundary_bodies(m_ctx, nullptr, anyDynamic ? (uint32_t)m_volumeMaps.size() : 0u, center.data(),
                                        dynamic.data()),
              "sphgb_set_boundary_bodies");
        m_bodiesSet = anyDynamic;
        m_boundaryDirty = false;
    }
    if (m_boundaryDirty) {
        // the boundary models' particles in model order; model k is body k
        std::vector<double> xb, center;
        std::vector<uint32_t> body;
        std::vector<int> dynamic;
        bool anyDynamic = false;
        for (unsigned int k = 0; k < m_boundaries.size(); k++) {
            const BoundaryModel_Akinci2012 &bm = *m_boundaries[k];
            const std::vector<double> x = to_double(bm.m_x);
            xb.insert(xb.end(), x.begin(), x.end());
            body.insert(body.end(), bm.numberOfParticles(), k);
            for (int d = 0; d < 3; d++) center.push_back((double)bm.m_rigidBody.getPosition()[d]);
            dynamic.push_back(bm.m_rigidBody.isDynamic() ? 1 : 0);
            // bodies where one collects forces or moves: no extra launches otherwise
            anyDynamic = anyDynamic || bm.m_rigidBody.isDynamic() || bm.m_rigidBody.isAnimated();
        }
        check(sphgb_upload_boundary(m_ctx, xb.data(), (uint32_t)body.size()), "sphgb_upload_boundary");
        check(sphgb_set_boundary_bodies(m_ctx, body.data(), anyDynamic ? (uint32_t)m_boundaries.size() : 0u,
                                        center.data(), dynamic.data()),
              "sphgb_set_boundary_bodies");
        m_bodiesSet = anyDynamic;
        m_boundaryDirty = false;
    }
    // the fluid models concatenated in model order; several models are phases of their own rest density
    std::vector<double> x, v;
    std::vector<uint32_t> counts;
    std::vector<double> rho0;
    for (FluidModel *f : m_fluids) {
        const std::vector<double> xf = to_double(f->m_x), vf = to_double(f->m_v);
        x.insert(x.end(), xf.begin(), xf.end());
        v.insert(v.end(), vf.begin(), vf.end());
        counts.push_back(f->numParticles());
        rho0.push_back((double)f->m_density0);
    }
    check(sphgb_upload_fluid(m_ctx, x.data(), v.data(), nullptr, n), "sphgb_upload_fluid");
    check(sphgb_set_fluid_phases(m_ctx, m_fluids.size() > 1 ? (uint32_t)m_fluids.size() : 0u, counts.data(),
                                 rho0.data()),
          "sphgb_set_fluid_phases");
    {   // per-model coefficients, where a model sets its own
        bool own = false;
        std::vector<double> nu, nub, xs, xsb;
        const auto pick = [&](Real mine, double shared) {
            own |= mine >= Real(0);
            return mine >= Real(0) ? (double)mine : shared;
        };
        for (FluidModel *f : m_fluids) {
            nu.push_back(pick(f->m_viscosity, m_visco ? (double)m_visco->m_viscosity : 0.0));
            nub.push_back(pick(f->m_viscosityBoundary, m_visco ? (double)m_visco->m_boundaryViscosity : 0.0));
            xs.push_back(pick(f->m_xsph, (double)m_sim.xsph));
            xsb.push_back(pick(f->m_xsphBoundary, (double)m_sim.xsphBoundary));
        }
        const uint32_t k = (own && m_fluids.size() > 1) ? (uint32_t)m_fluids.size() : 0u;
        check(sphgb_set_fluid_phase_viscosity(m_ctx, k, nu.data(), nub.data()), "sphgb_set_fluid_phase_viscosity");
        check(sphgb_set_fluid_phase_xsph(m_ctx, k, xs.data(), xsb.data()), "sphgb_set_fluid_phase_xsph");
    }
    if (n) {
        check(sphgb_upload_field(m_ctx, SPHGB_FIELD_PRESSURE_RHO2, m_pressureRho2.data(), kDtype), "upload p / rho^2");
        check(sphgb_upload_field(m_ctx, SPHGB_FIELD_PRESSURE_RHO2_V, m_pressureRho2V.data(), kDtype), "upload p_v / rho^2");
        if (m_visco)
            check(sphgb_upload_field(m_ctx, SPHGB_FIELD_VDIFF, &m_visco->m_vDiff[0][0], kDtype), "upload velocity difference");
    }
    check(sphgb_set_time_step(m_ctx, m_dt), "sphgb_set_time_step");
    check(sphgb_set_time(m_ctx, m_time), "sphgb_set_time");
    m_dirty = false;
}

// the current pose and velocities of every dynamic or animated body: boundary particles placed at
// R x0 + t (SimulatorBase.cpp:1620-1645), volume maps sampled at R^T (x - t) (TimeStep.cpp:238-240),
// both moving at w x (p - t) + v (BoundaryModel.h:78-84)
void TimeStepDFSPH_GB300::pushBodyMotion()
{
    for (unsigned int k = 0; k < m_boundaries.size() && m_bodiesSet; k++) {
        const RigidBodyObject &rb = m_boundaries[k]->m_rigidBody;
        if (!rb.isDynamic() && !rb.isAnimated()) continue;
        double R[9], t[3], v[3], w[3];
        for (int q = 0; q < 9; q++) R[q] = (double)rb.getRotation()[q];
        for (int d = 0; d < 3; d++) {
            t[d] = (double)rb.getPosition()[d];
            v[d] = (double)rb.getVelocity()[d];
            w[d] = (double)rb.getAngularVelocity()[d];
        }
        check(sphgb_set_body_motion(m_ctx, k, R, t, v, w), "sphgb_set_body_motion");
    }
    for (unsigned int k = 0; k < m_volumeMaps.size(); k++) {
        const RigidBodyObject &rb = m_volumeMaps[k]->m_rigidBody;
        if (!rb.isDynamic() && !rb.isAnimated()) continue;
        double R[9], t[3], v[3], w[3];
        for (int q = 0; q < 9; q++) R[q] = (double)m_volumeMaps[k]->m_rotation[q];
        for (int d = 0; d < 3; d++) {
            t[d] = (double)rb.getPosition()[d];
            v[d] = (double)rb.getVelocity()[d];
            w[d] = (double)rb.getAngularVelocity()[d];
        }
        check(sphgb_set_volume_map_motion(m_ctx, k, R, t, v, w), "sphgb_set_volume_map_motion");
    }
}

void TimeStepDFSPH_GB300::step()
{
    if (m_dirty) upload();
    pushBodyMotion();
    if (m_hostSync) {
        // the step is queued without a wait; the download waits for it and its fields together,
        // after which the step's statistics are on the host
        check(sphgb_step(m_ctx, nullptr), "sphgb_step");
        syncToHost();
        check(sphgb_sync(m_ctx, &m_stats), "sphgb_sync");
    } else {
        check(sphgb_step(m_ctx, &m_stats), "sphgb_step");
    }
    m_iterations = m_stats.iterations;
    m_iterationsV = m_stats.iterations_v;
    if (m_visco) m_visco->m_iterations = m_stats.visco_iterations;
    m_dt = (Real)m_stats.dt_next;   // TimeManager::setTimeStepSize of the CFL update
    m_time = (Real)m_stats.time;
}

void TimeStepDFSPH_GB300::syncToHost()
{
    const unsigned int n = totalParticles();
    if (n == 0) return;
    auto dl = [&](int field, void *dst, const char *what) { check(sphgb_download(m_ctx, field, dst, kDtype), what); };
    // the fluid fields in one call (one wait): the models' own fields of all models together,
    // handed back model by model, and the solver's fields
    std::vector<Vector3r> x(n), v(n), a(n);
    std::vector<Real> rho(n);
    std::vector<int> ids = {SPHGB_FIELD_POSITION, SPHGB_FIELD_VELOCITY, SPHGB_FIELD_ACCELERATION, SPHGB_FIELD_DENSITY,
                            SPHGB_FIELD_FACTOR, SPHGB_FIELD_DENSITY_ADV, SPHGB_FIELD_PRESSURE_RHO2,
                            SPHGB_FIELD_PRESSURE_RHO2_V, SPHGB_FIELD_PRESSURE_ACCEL};
    std::vector<void *> dsts = {&x[0][0], &v[0][0], &a[0][0], rho.data(), m_factor.data(), m_densityAdv.data(),
                                m_pressureRho2.data(), m_pressureRho2V.data(), &m_pressureAccel[0][0]};
    if (m_visco) {
        ids.push_back(SPHGB_FIELD_VDIFF);
        dsts.push_back(&m_visco->m_vDiff[0][0]);
    }
    check(sphgb_download_fields(m_ctx, static_cast<uint32_t>(ids.size()), ids.data(), dsts.data(), kDtype),
          "download fields");
    size_t off = 0;
    for (FluidModel *f : m_fluids) {
        const size_t m = f->numParticles();
        std::copy(x.begin() + off, x.begin() + off + m, f->m_x.begin());
        std::copy(v.begin() + off, v.begin() + off + m, f->m_v.begin());
        std::copy(a.begin() + off, a.begin() + off + m, f->m_a.begin());
        std::copy(rho.begin() + off, rho.begin() + off + m, f->m_density.begin());
        off += m;
    }
    // boundary volumes of all models in model order, split per model
    size_t nb = 0;
    for (const BoundaryModel_Akinci2012 *bm : m_boundaries) nb += bm->numberOfParticles();
    if (nb == 0) return;
    std::vector<Real> vol(nb);
    dl(SPHGB_FIELD_BOUNDARY_VOLUME, vol.data(), "download boundary volume");
    off = 0;
    for (BoundaryModel_Akinci2012 *bm : m_boundaries) {
        std::copy(vol.begin() + off, vol.begin() + off + bm->numberOfParticles(), bm->m_V.begin());
        off += bm->numberOfParticles();
    }
}

int TimeStepDFSPH_GB300::getParameterId(const std::string &name)
{
    for (const NamedId &p : kNames)
        if (name == p.name) return *p.id;
    return -1;
}

double TimeStepDFSPH_GB300::getValue(int id) const
{
    if (id == SOLVER_ITERATIONS) return m_iterations;
    if (id == MIN_ITERATIONS) return m_minIterations;
    if (id == MAX_ITERATIONS) return m_maxIterations;
    if (id == MAX_ERROR) return m_maxError;
    if (id == SOLVER_ITERATIONS_V) return m_iterationsV;
    if (id == MAX_ITERATIONS_V) return m_maxIterationsV;
    if (id == MAX_ERROR_V) return m_maxErrorV;
    if (id == USE_DIVERGENCE_SOLVER) return m_enableDivergenceSolver ? 1.0 : 0.0;
    if (m_visco) {
        if (id == Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT) return m_visco->m_viscosity;
        if (id == Viscosity_Weiler2018_GB300::ITERATIONS) return m_visco->m_iterations;
        if (id == Viscosity_Weiler2018_GB300::MAX_ITERATIONS) return m_visco->m_maxIter;
        if (id == Viscosity_Weiler2018_GB300::MAX_ERROR) return m_visco->m_maxError;
        if (id == Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT_BOUNDARY) return m_visco->m_boundaryViscosity;
    }
    throw Error(SPHGB_ERR_ARGUMENT, "unknown parameter id " + std::to_string(id));
}

void TimeStepDFSPH_GB300::setValue(int id, double value)
{
    // the iteration counters are read-only, as in the reference (setReadOnly(true))
    if (id == SOLVER_ITERATIONS || id == SOLVER_ITERATIONS_V ||
        (m_visco && id == Viscosity_Weiler2018_GB300::ITERATIONS))
        throw Error(SPHGB_ERR_ARGUMENT, "parameter is read-only");
    if (id == MIN_ITERATIONS) m_minIterations = (unsigned int)value;
    else if (id == MAX_ITERATIONS) m_maxIterations = (unsigned int)value;
    else if (id == MAX_ERROR) m_maxError = (Real)value;
    else if (id == MAX_ITERATIONS_V) m_maxIterationsV = (unsigned int)value;
    else if (id == MAX_ERROR_V) m_maxErrorV = (Real)value;
    else if (id == USE_DIVERGENCE_SOLVER) m_enableDivergenceSolver = value != 0.0;
    else if (m_visco && id == Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT) m_visco->m_viscosity = (Real)value;
    else if (m_visco && id == Viscosity_Weiler2018_GB300::MAX_ITERATIONS) m_visco->m_maxIter = (unsigned int)value;
    else if (m_visco && id == Viscosity_Weiler2018_GB300::MAX_ERROR) m_visco->m_maxError = (Real)value;
    else if (m_visco && id == Viscosity_Weiler2018_GB300::VISCOSITY_COEFFICIENT_BOUNDARY)
        m_visco->m_boundaryViscosity = (Real)value;
    else throw Error(SPHGB_ERR_ARGUMENT, "unknown parameter id " + std::to_string(id));
    applyParameters();
}

}  // namespace sphgb_host
