// Runs a scene through the C++ host classes (sphgb_host.h) the way a SPlisHSPlasH
// simulator drives its time step: build the models, construct the time step, call step()
// repeatedly and read the fields back from the host vectors.
//
//   sphgb_host_demo <scene.bin> <out.bin>
//
// scene.bin (little endian): uint32 n, nb, steps, lanes (0 = autotune), viscosity (0/1),
// bodies (0/1), volume map (0/1), phase0 (0: one fluid model; else the first phase0 particles are
// the first model and the rest a second one); float64 particle radius; with phase0 > 0 float64
// rest density of the second model; float64 x[n][3], v[n][3], xb[nb][3];
// with bodies: uint32 body[nb] (0: the dynamic body, 1: static walls), float64 position[3],
// velocity[3] and angular velocity[3] of the dynamic body (its pose is held, so that the run stays
// comparable; its particles are given in the scene's frame and handed over in body coordinates);
// with a volume map (then nb = 0): uint32 nv, nf, resolution[3], invert, float64 vertices[nv][3],
// uint32 faces[nf][3] of the container (Bender2019 boundary), which is then the dynamic body.
// out.bin: per step uint32 iterations, iterationsV, viscoIterations and float64 time;
// then float64 x[n][3], v[n][3], density[n], p / rho^2 [n], boundary volume[nb] (in the
// order of the boundary models: body 0's particles first), force[3], torque[3] of body 0 (the
// container with a volume map) summed over all steps (getForceAndTorque; zeros without bodies).
#include <cstdint>
#include <cstdio>
#include <memory>
#include <vector>

#include "sphgb_host.h"

using namespace sphgb_host;

namespace {

template <class T> bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <class T> void wr(FILE *f, const T *p, size_t n) { fwrite(p, sizeof(T), n, f); }

std::vector<Vector3r> to_vec(const std::vector<double> &a)
{
    std::vector<Vector3r> v(a.size() / 3);
    for (size_t i = 0; i < v.size(); i++) v[i] = Vector3r((Real)a[3 * i], (Real)a[3 * i + 1], (Real)a[3 * i + 2]);
    return v;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s scene.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t hdr[8];
    double radius, rho1 = 0;
    if (!rd(f, hdr, 8) || !rd(f, &radius, 1)) return 2;
    const uint32_t n = hdr[0], nb = hdr[1], steps = hdr[2], lanes = hdr[3], visc = hdr[4], bodies = hdr[5],
                   vmap = hdr[6], phase0 = hdr[7];
    double own1[4] = {-1, -1, -1, -1};   // the second model's nu, nu_b, xsph, xsph_b (negative: shared)
    if (phase0 && (phase0 >= n || !rd(f, &rho1, 1) || !rd(f, own1, 4))) return 2;
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), xb(3 * (size_t)nb);
    if (!rd(f, x.data(), x.size()) || !rd(f, v.data(), v.size()) || !rd(f, xb.data(), xb.size())) return 2;
    std::vector<uint32_t> body(nb, 1u);
    double pos[3] = {0, 0, 0}, bvel[6] = {0, 0, 0, 0, 0, 0};
    if (bodies && (!rd(f, body.data(), body.size()) || !rd(f, pos, 3) || !rd(f, bvel, 6))) return 2;
    uint32_t mh[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> mv;
    std::vector<uint32_t> mf;
    if (vmap) {
        if (!rd(f, mh, 6)) return 2;
        mv.resize(3 * (size_t)mh[0]);
        mf.resize(3 * (size_t)mh[1]);
        if (!rd(f, mv.data(), mv.size()) || !rd(f, mf.data(), mf.size())) return 2;
    }
    fclose(f);

    try {
        // the parameter block of the scenes (scene-file defaults of the dam-break configs)
        SimulationParameters sp;
        sp.particleRadius = (Real)radius;
        sp.cflFactor = 1;
        sp.viscosityMethod = visc ? 6 : 0;
        FluidModel model, second;
        const std::vector<Vector3r> xv = to_vec(x), vv = to_vec(v), xbv = to_vec(xb);
        const uint32_t n0 = phase0 ? phase0 : n;
        model.initModel("Fluid", n0, xv.data(), vv.data());
        if (phase0) {   // a second fluid model (a phase of its own rest density)
            second.initModel("Fluid2", n - n0, xv.data() + n0, vv.data() + n0);
            second.m_density0 = (Real)rho1;
            second.m_viscosity = (Real)own1[0];
            second.m_viscosityBoundary = (Real)own1[1];
            second.m_xsph = (Real)own1[2];
            second.m_xsphBoundary = (Real)own1[3];
        }
        // one boundary model per body: the dynamic body (body 0) and the static walls
        std::vector<Vector3r> part[2];
        for (uint32_t k = 0; k < nb; k++) {
            if (body[k] != 0) {
                part[1].push_back(xbv[k]);
            } else {   // the dynamic body's rest shape in body coordinates
                const double *p = xb.data() + 3 * (size_t)k;
                part[0].push_back(Vector3r((Real)(p[0] - pos[0]), (Real)(p[1] - pos[1]), (Real)(p[2] - pos[2])));
            }
        }
        BoundaryModel_Akinci2012 models[2];
        std::vector<BoundaryModel_Akinci2012 *> boundaries;
        for (int b = 0; b < 2; b++) {
            models[b].initModel((unsigned int)part[b].size(), part[b].data());
            if (!part[b].empty()) boundaries.push_back(&models[b]);
        }
        models[0].getRigidBodyObject()->setPosition(Vector3r((Real)pos[0], (Real)pos[1], (Real)pos[2]));
        models[0].getRigidBodyObject()->setDynamic(bodies != 0);
        models[0].getRigidBodyObject()->setVelocity(Vector3r((Real)bvel[0], (Real)bvel[1], (Real)bvel[2]));
        models[0].getRigidBodyObject()->setAngularVelocity(Vector3r((Real)bvel[3], (Real)bvel[4], (Real)bvel[5]));
        Viscosity_Weiler2018_GB300 viscosity;
        viscosity.m_maxError = Real(1e-3);
        // Bender2019: the container as a volume map instead of boundary particles
        BoundaryModel_Bender2019 container;
        if (vmap) {
            const std::vector<Vector3r> mvv = to_vec(mv);
            container.initModel(mh[0], mvv.data(), mh[1], mf.data());
            for (int k = 0; k < 3; k++) container.m_mapResolution[k] = mh[2 + k];
            container.m_mapInvert = mh[5] != 0;
            if (bodies) {
                RigidBodyObject *rb = container.getRigidBodyObject();
                rb->setPosition(Vector3r((Real)pos[0], (Real)pos[1], (Real)pos[2]));
                rb->setDynamic(true);
                rb->setVelocity(Vector3r((Real)bvel[0], (Real)bvel[1], (Real)bvel[2]));
                rb->setAngularVelocity(Vector3r((Real)bvel[3], (Real)bvel[4], (Real)bvel[5]));
            }
        }
        std::unique_ptr<TimeStepDFSPH_GB300> tsp(
            vmap ? new TimeStepDFSPH_GB300(model, std::vector<BoundaryModel_Bender2019 *>{&container}, sp,
                                           visc ? &viscosity : nullptr)
                 : new TimeStepDFSPH_GB300(model, boundaries, sp, visc ? &viscosity : nullptr));
        TimeStepDFSPH_GB300 &ts = *tsp;
        if (phase0) ts.addFluidModel(second);
        sphgb_set_lanes_per_particle(ts.context(), lanes);
        ts.resize();

        FILE *o = fopen(argv[2], "wb");
        if (!o) return 2;
        for (uint32_t k = 0; k < steps; k++) {
            ts.step();
            const uint32_t it[3] = {(uint32_t)ts.getValue(TimeStepDFSPH_GB300::SOLVER_ITERATIONS),
                                    (uint32_t)ts.getValue(TimeStepDFSPH_GB300::SOLVER_ITERATIONS_V),
                                    visc ? (uint32_t)ts.getValue(Viscosity_Weiler2018_GB300::ITERATIONS) : 0u};
            const double t = ts.getTime();
            wr(o, it, 3);
            wr(o, &t, 1);
        }
        std::vector<double> out;   // every fluid model in model order
        auto each = [&](auto fn) {
            for (unsigned int k = 0; k < ts.numberOfFluidModels(); k++)
                for (uint32_t i = 0; i < ts.getFluidModel(k)->numParticles(); i++) fn(k, i);
        };
        each([&](unsigned k, uint32_t i) { for (int c = 0; c < 3; c++) out.push_back(ts.getFluidModel(k)->getPosition(i)[c]); });
        each([&](unsigned k, uint32_t i) { for (int c = 0; c < 3; c++) out.push_back(ts.getFluidModel(k)->getVelocity(i)[c]); });
        each([&](unsigned k, uint32_t i) { out.push_back(ts.getFluidModel(k)->getDensity(i)); });
        each([&](unsigned k, uint32_t i) { out.push_back(ts.getPressureRho2(k, i)); });
        for (BoundaryModel_Akinci2012 *bm : boundaries)
            for (uint32_t i = 0; i < bm->numberOfParticles(); i++) out.push_back(bm->getVolume(i));
        Vector3r force, torque;
        if (vmap)
            container.getForceAndTorque(force, torque);
        else
            models[0].getForceAndTorque(force, torque);
        for (int c = 0; c < 3; c++) out.push_back(force[c]);
        for (int c = 0; c < 3; c++) out.push_back(torque[c]);
        wr(o, out.data(), out.size());
        fclose(o);
        printf("%s: %u steps, %u fluid + %u boundary particles, time %.6f\n", ts.getMethodName().c_str(), steps, n, nb,
               (double)ts.getTime());
    } catch (const Error &e) {
        fprintf(stderr, "error %d: %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
