// Pin driver for the CPU oracle -- TEST INFRASTRUCTURE ONLY.
//
// Compiled by oracle/build_ref.sh against the reference's OWN sources where they
// lie in the reference tree (SPlisHSPlasH/SPHKernels.{h,cpp},
// SPlisHSPlasH/Utilities/MatrixFreeSolver.h, vendored Eigen 3.4 CG).  Nothing of
// the reference is copied here; this file only calls it.  Outputs go to
// oracle/_ref/ and are turned into committed fixtures by
// tests/golden/gen_golden.py.
//
// Modes
//   kernel <support> <in.f64> <out.f64>
//       in : m x 3 float64 offset vectors r
//       out: m x 4 (W, gradW) from SPH::CubicKernel (SPHKernels.h:16-91), plus
//            with USE_AVX another m x 4 from SPH::CubicKernel_AVX (:696-792).
//   cg <in.f64> <out.f64>           (USE_DOUBLE build only)
//       Runs Eigen::ConjugateGradient<MatrixReplacement, Lower|Upper,
//       BlockJacobiPreconditioner3D> exactly as Viscosity_Weiler2018::step does
//       (Viscosity_Weiler2018.cpp:891-926), with the operator and diagonal
//       blocks supplied by the oracle's Weiler2018 restatement.
#include "SPlisHSPlasH/Common.h"
#include "SPlisHSPlasH/SPHKernels.h"
#include "SPlisHSPlasH/Utilities/MatrixFreeSolver.h"

#include <Eigen/IterativeLinearSolvers>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#ifdef USE_DOUBLE
extern "C" {
#include "sph_oracle.h"
}
#endif

using namespace SPH;

static std::vector<double> read_all(const char *path)
{
    std::vector<double> v;
    FILE *f = std::fopen(path, "rb");
    if (!f) { std::perror(path); std::exit(2); }
    double buf[4096];
    size_t k;
    while ((k = std::fread(buf, sizeof(double), 4096, f)) > 0) v.insert(v.end(), buf, buf + k);
    std::fclose(f);
    return v;
}

static void write_all(const char *path, const std::vector<double> &v)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) { std::perror(path); std::exit(2); }
    std::fwrite(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
}

static int mode_kernel(double support, const char *in, const char *out)
{
    std::vector<double> r = read_all(in);
    const size_t m = r.size() / 3;
    CubicKernel::setRadius(static_cast<Real>(support));
    std::vector<double> res;
    res.reserve(m * 8);
    for (size_t i = 0; i < m; i++) {
        const Vector3r ri(static_cast<Real>(r[3 * i]), static_cast<Real>(r[3 * i + 1]), static_cast<Real>(r[3 * i + 2]));
        const Vector3r g = CubicKernel::gradW(ri);
        res.push_back(CubicKernel::W(ri));
        res.push_back(g[0]);
        res.push_back(g[1]);
        res.push_back(g[2]);
    }
#ifdef USE_AVX
    CubicKernel_AVX::setRadius(static_cast<Real>(support));
    for (size_t i = 0; i < m; i += 8) {
        Vector3r xj[8];
        const size_t cnt = std::min<size_t>(8, m - i);
        for (size_t l = 0; l < 8; l++) {
            if (l < cnt)
                xj[l] = Vector3r(static_cast<Real>(r[3 * (i + l)]), static_cast<Real>(r[3 * (i + l) + 1]),
                                 static_cast<Real>(r[3 * (i + l) + 2]));
            else
                xj[l].setZero();
        }
        Vector3f8 x8(xj);
        Real W[8];
        CubicKernel_AVX::W(x8).store(W);
        Vector3r G[8];
        CubicKernel_AVX::gradW(x8).store(G);
        for (size_t l = 0; l < cnt; l++) {
            res.push_back(W[l]);
            res.push_back(G[l][0]);
            res.push_back(G[l][1]);
            res.push_back(G[l][2]);
        }
    }
#endif
    write_all(out, res);
    return 0;
}

#ifdef USE_DOUBLE
struct CgData {
    orc_state st;
    orc_params pp;
    double dt;
    std::vector<double> diag9;
};

static void matvec_cb(const Real *vec, Real *result, void *user)
{
    CgData *d = static_cast<CgData *>(user);
    orc_weiler_matvec(&d->st, &d->pp, d->dt, vec, result);
}

static void diag_cb(const unsigned int i, Matrix3r &res, void *user)
{
    CgData *d = static_cast<CgData *>(user);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) res(a, b) = d->diag9[9 * i + 3 * a + b];
}

// Input layout (float64): n, nb, radius, density0, viscosity, viscosityBoundary,
// dt, tol, maxIter, then x[3n], v[3n], density[n], vdiff[3n], xb[3nb], Vb[nb].
static int mode_cg(const char *in, const char *out)
{
    std::vector<double> a = read_all(in);
    size_t o = 0;
    const unsigned n = (unsigned)a[o++], nb = (unsigned)a[o++];
    CgData d;
    std::memset(&d.st, 0, sizeof(d.st));
    std::memset(&d.pp, 0, sizeof(d.pp));
    d.pp.radius = a[o++];
    d.pp.density0 = a[o++];
    d.pp.viscosity = a[o++];
    d.pp.viscosity_boundary = a[o++];
    d.dt = a[o++];
    const double tol = a[o++];
    const unsigned maxIter = (unsigned)a[o++];
    d.pp.fp32_predicate = 1;
    std::vector<double> x(a.begin() + o, a.begin() + o + 3 * n); o += 3 * n;
    std::vector<double> v(a.begin() + o, a.begin() + o + 3 * n); o += 3 * n;
    std::vector<double> rho(a.begin() + o, a.begin() + o + n); o += n;
    std::vector<double> vdiff(a.begin() + o, a.begin() + o + 3 * n); o += 3 * n;
    std::vector<double> xb(a.begin() + o, a.begin() + o + 3 * nb); o += 3 * nb;
    std::vector<double> Vb(a.begin() + o, a.begin() + o + nb); o += nb;
    d.st.n = n;
    d.st.nb = nb;
    d.st.x = x.data();
    d.st.v = v.data();
    d.st.density = rho.data();
    d.st.vdiff = vdiff.data();
    d.st.xb = xb.data();
    d.st.Vb = Vb.data();
    std::vector<double> b(3 * n), g(3 * n);
    d.diag9.resize(9 * (size_t)n);
    orc_weiler_system(&d.st, &d.pp, d.dt, b.data(), g.data(), d.diag9.data());

    typedef Eigen::ConjugateGradient<MatrixReplacement, Eigen::Lower | Eigen::Upper, BlockJacobiPreconditioner3D> Solver;
    Solver solver;
    MatrixReplacement A(3 * n, matvec_cb, (void *)&d);
    solver.preconditioner().init(n, diag_cb, (void *)&d);
    solver.setTolerance(tol);
    solver.setMaxIterations(maxIter);
    solver.compute(A);
    VectorXr bb(3 * n), gg(3 * n);
    for (size_t k = 0; k < 3 * (size_t)n; k++) { bb[k] = b[k]; gg[k] = g[k]; }
    VectorXr xs = solver.solveWithGuess(bb, gg);
    std::vector<double> res;
    res.push_back((double)solver.iterations());
    res.push_back((double)solver.error());
    for (size_t k = 0; k < 3 * (size_t)n; k++) res.push_back(xs[k]);
    write_all(out, res);
    return 0;
}
#endif

int main(int argc, char **argv)
{
    if (argc >= 5 && std::string(argv[1]) == "kernel") return mode_kernel(std::atof(argv[2]), argv[3], argv[4]);
#ifdef USE_DOUBLE
    if (argc >= 4 && std::string(argv[1]) == "cg") return mode_cg(argv[2], argv[3]);
#endif
    std::fprintf(stderr, "usage: ref_pin kernel <support> <in> <out> | cg <in> <out>\n");
    return 1;
}
