/*
 * CPU oracle for the DFSPH time-step hot path -- TEST INFRASTRUCTURE ONLY.
 * See sph_oracle.h for scope and pinning status.  Each function names the
 * reference file:line (SPlisHSPlasH 2.16.0, paths relative to the project root)
 * whose algorithm it restates.  The FP64 build follows the scalar (non-AVX)
 * code path of the reference, which is the one a USE_DOUBLE build compiles.
 *
 * Compiled with -ffp-contract=off so that x86 and Arm hosts give identical
 * results, and reductions that decide solver convergence are summed serially
 * in index order (deterministic for any thread count).
 */
#include "sph_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef orc_real real;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* Cubic spline kernel, SPHKernels.h:16-91 (CubicKernel::setRadius/W/gradW).  */
/* ------------------------------------------------------------------------ */
typedef struct {
    double h, k, l, w0;
} kern;

static kern kern_make(double h)
{
    kern K;
    const double h3 = h * h * h;
    K.h = h;
    K.k = 8.0 / (M_PI * h3);   /* SPHKernels.h:30 */
    K.l = 48.0 / (M_PI * h3);  /* SPHKernels.h:31 */
    K.w0 = K.k;                /* W(0) = k * (0 - 0 + 1) */
    return K;
}

static inline double kW(const kern *K, double r)
{
    /* SPHKernels.h:37-55 */
    const double q = r / K->h;
    if (q <= 1.0) {
        if (q <= 0.5) {
            const double q2 = q * q, q3 = q2 * q;
            return K->k * (6.0 * q3 - 6.0 * q2 + 1.0);
        }
        const double t = 1.0 - q;
        return K->k * (2.0 * t * t * t);
    }
    return 0.0;
}

static inline void kGradW(const kern *K, const double r[3], double out[3])
{
    /* SPHKernels.h:62-84 */
    const double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    const double q = rl / K->h;
    if (rl > 1.0e-9 && q <= 1.0) {
        double c;
        if (q <= 0.5)
            c = K->l * q * (3.0 * q - 2.0);
        else {
            const double f = 1.0 - q;
            c = K->l * (-f * f);
        }
        c /= (rl * K->h);
        out[0] = c * r[0];
        out[1] = c * r[1];
        out[2] = c * r[2];
    } else {
        out[0] = out[1] = out[2] = 0.0;
    }
}

double orc_kernel_W(double r, double support)
{
    kern K = kern_make(support);
    return kW(&K, r);
}

void orc_kernel_gradW(const double r[3], double support, double out[3])
{
    kern K = kern_make(support);
    kGradW(&K, r, out);
}

/* ------------------------------------------------------------------------ */
/* Neighbour search: dense cell grid (cell = support radius), counting sort.  */
/* Stands in for CompactNSearch::find_neighbors (Simulation.cpp:606-619).     */
/* ------------------------------------------------------------------------ */
typedef struct {
    double org[3], cell;
    long dim[3];
    unsigned *start;   /* ncell + 1 */
    unsigned *sorted;  /* m */
} ogrid;

static inline long clampl(long v, long lo, long hi) { return v < lo ? lo : (v > hi ? hi : v); }

static inline void cell_of(const ogrid *g, const real *p, long c[3])
{
    for (int d = 0; d < 3; d++)
        c[d] = clampl((long)floor(((double)p[d] - g->org[d]) / g->cell), 0, g->dim[d] - 1);
}

static int grid_build(ogrid *g, unsigned m, const real *y, double cell)
{
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    memset(g, 0, sizeof(*g));
    if (m > 0) {
        for (int d = 0; d < 3; d++) lo[d] = hi[d] = (double)y[d];
        for (unsigned i = 1; i < m; i++)
            for (int d = 0; d < 3; d++) {
                const double v = (double)y[3 * (size_t)i + d];
                if (v < lo[d]) lo[d] = v;
                if (v > hi[d]) hi[d] = v;
            }
    }
    g->cell = cell;
    size_t ncell = 1;
    for (int d = 0; d < 3; d++) {
        g->org[d] = lo[d] - cell;
        g->dim[d] = (long)floor((hi[d] - g->org[d]) / cell) + 2;
        if (g->dim[d] < 1) g->dim[d] = 1;
        ncell *= (size_t)g->dim[d];
    }
    if (ncell > ((size_t)1 << 31)) return -1;
    g->start = (unsigned *)calloc(ncell + 1, sizeof(unsigned));
    g->sorted = (unsigned *)malloc((m ? m : 1) * sizeof(unsigned));
    unsigned *cid = (unsigned *)malloc((m ? m : 1) * sizeof(unsigned));
    if (!g->start || !g->sorted || !cid) { free(cid); return -2; }
    for (unsigned i = 0; i < m; i++) {
        long c[3];
        cell_of(g, y + 3 * (size_t)i, c);
        cid[i] = (unsigned)((c[2] * g->dim[1] + c[1]) * g->dim[0] + c[0]);
        g->start[cid[i] + 1]++;
    }
    for (size_t c = 0; c < ncell; c++) g->start[c + 1] += g->start[c];
    unsigned *fill = (unsigned *)malloc((ncell ? ncell : 1) * sizeof(unsigned));
    if (!fill) { free(cid); return -2; }
    memcpy(fill, g->start, ncell * sizeof(unsigned));
    for (unsigned i = 0; i < m; i++) g->sorted[fill[cid[i]]++] = i;
    free(fill);
    free(cid);
    return 0;
}

static void grid_free(ogrid *g)
{
    free(g->start);
    free(g->sorted);
    g->start = g->sorted = NULL;
}

static inline int accept_pair(const real *a, const real *b, int fp32, float h2f, double h2d)
{
    if (fp32) {
        const float dx = (float)a[0] - (float)b[0];
        const float dy = (float)a[1] - (float)b[1];
        const float dz = (float)a[2] - (float)b[2];
        float d2 = dx * dx;
        d2 = d2 + dy * dy;
        d2 = d2 + dz * dz;
        return d2 < h2f;
    } else {
        const double dx = (double)a[0] - (double)b[0];
        const double dy = (double)a[1] - (double)b[1];
        const double dz = (double)a[2] - (double)b[2];
        return dx * dx + dy * dy + dz * dz < h2d;
    }
}

static int cmp_u32(const void *a, const void *b)
{
    const unsigned x = *(const unsigned *)a, y = *(const unsigned *)b;
    return (x > y) - (x < y);
}

/* Visit neighbours of query point q; mode 0 counts, mode 1 writes. */
static unsigned visit(const ogrid *g, const real *q, unsigned self, const real *y,
                      int fp32, float h2f, double h2d, unsigned *out)
{
    long c[3];
    cell_of(g, q, c);
    unsigned cnt = 0;
    for (long dz = -1; dz <= 1; dz++) {
        const long z = c[2] + dz;
        if (z < 0 || z >= g->dim[2]) continue;
        for (long dy = -1; dy <= 1; dy++) {
            const long yy = c[1] + dy;
            if (yy < 0 || yy >= g->dim[1]) continue;
            for (long dx = -1; dx <= 1; dx++) {
                const long x = c[0] + dx;
                if (x < 0 || x >= g->dim[0]) continue;
                const size_t cell = (size_t)((z * g->dim[1] + yy) * g->dim[0] + x);
                for (unsigned k = g->start[cell]; k < g->start[cell + 1]; k++) {
                    const unsigned j = g->sorted[k];
                    if (j == self) continue;
                    if (accept_pair(q, y + 3 * (size_t)j, fp32, h2f, h2d)) {
                        if (out) out[cnt] = j;
                        cnt++;
                    }
                }
            }
        }
    }
    return cnt;
}

typedef struct {
    unsigned *off, *idx;
} olist;

static int lists_build(olist *L, unsigned n, const real *x, unsigned m, const real *y,
                       double support, int same_set, int fp32)
{
    ogrid g;
    L->off = L->idx = NULL;
    if (grid_build(&g, m, y, support) != 0) return -1;
    const float h2f = (float)(support * support);
    const double h2d = support * support;
    L->off = (unsigned *)calloc((size_t)n + 1, sizeof(unsigned));
    if (!L->off) { grid_free(&g); return -2; }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; i++)
        L->off[i + 1] = (m > 0) ? visit(&g, x + 3 * (size_t)i, same_set ? (unsigned)i : 0xffffffffu,
                                         y, fp32, h2f, h2d, NULL) : 0;
    for (unsigned i = 0; i < n; i++) L->off[i + 1] += L->off[i];
    L->idx = (unsigned *)malloc(((size_t)L->off[n] + 1) * sizeof(unsigned));
    if (!L->idx) { grid_free(&g); return -2; }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; i++) {
        if (m == 0) continue;
        unsigned *o = L->idx + L->off[i];
        const unsigned c = visit(&g, x + 3 * (size_t)i, same_set ? (unsigned)i : 0xffffffffu,
                                 y, fp32, h2f, h2d, o);
        qsort(o, c, sizeof(unsigned), cmp_u32);
    }
    grid_free(&g);
    return 0;
}

static void lists_free(olist *L)
{
    free(L->off);
    free(L->idx);
    L->off = L->idx = NULL;
}

int orc_neighbors(unsigned n, const real *x, unsigned m, const real *y, double support,
                  int same_set, int fp32, unsigned *offsets, unsigned *indices, unsigned capacity)
{
    olist L;
    if (lists_build(&L, n, x, m, y, support, same_set, fp32) != 0) return -1;
    memcpy(offsets, L.off, ((size_t)n + 1) * sizeof(unsigned));
    int rc = 0;
    if (indices) {
        if (L.off[n] > capacity) rc = -3;
        else memcpy(indices, L.idx, (size_t)L.off[n] * sizeof(unsigned));
    }
    lists_free(&L);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Akinci2012 boundary volume (BoundaryModel_Akinci2012.cpp:48-75), driven by */
/* Simulation::updateBoundaryVolume (Simulation.cpp:696-756).                 */
/* ------------------------------------------------------------------------ */
int orc_boundary_volume(unsigned nb, const real *xb, double support, int fp32, real *Vb)
{
    olist L;
    kern K = kern_make(support);
    if (lists_build(&L, nb, xb, nb, xb, support, 1, fp32) != 0) return -1;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)nb; i++) {
        double delta = K.w0;
        for (unsigned k = L.off[i]; k < L.off[i + 1]; k++) {
            const unsigned j = L.idx[k];
            double r[3];
            for (int d = 0; d < 3; d++) r[d] = (double)xb[3 * i + d] - (double)xb[3 * (size_t)j + d];
            delta += kW(&K, sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]));
        }
        Vb[i] = (real)(1.0 / delta);
    }
    lists_free(&L);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Step context                                                              */
/* ------------------------------------------------------------------------ */
typedef struct {
    orc_state *s;
    const orc_params *p;
    kern K;
    olist F, B;           /* fluid-fluid, fluid-boundary */
    double V, mass, rho0, eps;
    /* several fluid phases: rest density and phase of each particle, phases, their sizes */
    double *r0;
    int *ph;
    unsigned nph;
} ctx_t;

/* rest density and mass of particle i: those of its fluid model (FluidModel::getDensity0,
 * getMass = V density0, FluidModel.cpp:234-253) */
static inline double rho0_of(const ctx_t *c, long i) { return c->r0 ? c->r0[i] : c->rho0; }
static inline double mass_of(const ctx_t *c, long i) { return c->V * rho0_of(c, i); }

static inline void diffv(const real *a, const real *b, double r[3])
{
    r[0] = (double)a[0] - (double)b[0];
    r[1] = (double)a[1] - (double)b[1];
    r[2] = (double)a[2] - (double)b[2];
}

static inline double dot3(const double a[3], const double b[3])
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

static double serial_sum(const double *v, size_t n)
{
    double s = 0.0;
    for (size_t i = 0; i < n; i++) s += v[i];
    return s;
}

/* TimeStep::computeDensities, scalar path (TimeStep.cpp:116-169). */
static void compute_densities(ctx_t *c)
{
    orc_state *s = c->s;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)s->n; i++) {
        double dens = c->V * c->K.w0;
        const real *xi = s->x + 3 * i;
        for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
            double r[3];
            diffv(xi, s->x + 3 * (size_t)c->F.idx[k], r);
            dens += c->V * kW(&c->K, sqrt(dot3(r, r)));
        }
        for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
            const unsigned j = c->B.idx[k];
            double r[3];
            diffv(xi, s->xb + 3 * (size_t)j, r);
            dens += (double)s->Vb[j] * kW(&c->K, sqrt(dot3(r, r)));
        }
        s->density[i] = (real)(dens * rho0_of(c, i));
    }
}

/* TimeStepDFSPH::computeDFSPHFactor, scalar path (TimeStepDFSPH.cpp:1106-1186). */
static void compute_factor(ctx_t *c)
{
    orc_state *s = c->s;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)s->n; i++) {
        const real *xi = s->x + 3 * i;
        double sum_grad_p_k = 0.0, gpi[3] = {0, 0, 0};
        for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
            double r[3], g[3];
            diffv(xi, s->x + 3 * (size_t)c->F.idx[k], r);
            kGradW(&c->K, r, g);
            const double gpj[3] = {-c->V * g[0], -c->V * g[1], -c->V * g[2]};
            sum_grad_p_k += dot3(gpj, gpj);
            gpi[0] -= gpj[0]; gpi[1] -= gpj[1]; gpi[2] -= gpj[2];
        }
        for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
            const unsigned j = c->B.idx[k];
            double r[3], g[3];
            diffv(xi, s->xb + 3 * (size_t)j, r);
            kGradW(&c->K, r, g);
            const double Vj = (double)s->Vb[j];
            gpi[0] += Vj * g[0]; gpi[1] += Vj * g[1]; gpi[2] += Vj * g[2];
        }
        sum_grad_p_k += dot3(gpi, gpi);
        s->factor[i] = (real)(sum_grad_p_k > c->eps ? 1.0 / sum_grad_p_k : 0.0);
        if (s->factor_raw) s->factor_raw[i] = s->factor[i];
    }
}

/* Fluid + boundary velocity divergence sum: the loops of computeDensityChange
 * (TimeStepDFSPH.cpp:1247-1295) and computeDensityAdv (:1190-1243); boundary
 * velocity is zero for static Akinci2012 walls. */
/* BoundaryModel::getPointVelocity (BoundaryModel.h:78-84): the velocity w x (p - t) + v of point p
 * of the body of boundary entry j; with volume maps the entry j = i * nbodies + b belongs to map b.
 * A boundary particle has its own velocity (s->vb; none: a static wall). */
static void boundary_point_velocity(const ctx_t *c, unsigned j, const double p[3], double out[3])
{
    const orc_state *s = c->s;
    out[0] = out[1] = out[2] = 0.0;
    if (c->p->boundary_method != 2) {   /* boundary particle j of a moving body */
        if (s->vb)
            for (int d = 0; d < 3; d++) out[d] = (double)s->vb[3 * (size_t)j + d];
        return;
    }
    if (!s->nvmaps) return;
    const orc_vmap *m = s->vmaps + (j % s->nvmaps);
    const double d[3] = {p[0] - m->t[0], p[1] - m->t[1], p[2] - m->t[2]};
    out[0] = m->w[1] * d[2] - m->w[2] * d[1] + m->v[0];
    out[1] = m->w[2] * d[0] - m->w[0] * d[2] + m->v[1];
    out[2] = m->w[0] * d[1] - m->w[1] * d[0] + m->v[2];
}

/* ... at the boundary point x_j itself */
static void boundary_velocity(const ctx_t *c, unsigned j, double out[3])
{
    const real *xb = c->s->xb + 3 * (size_t)j;
    const double p[3] = {(double)xb[0], (double)xb[1], (double)xb[2]};
    boundary_point_velocity(c, j, p, out);
}

static double velocity_divergence(const ctx_t *c, long i)
{
    const orc_state *s = c->s;
    const real *xi = s->x + 3 * i, *vi = s->v + 3 * i;
    double acc = 0.0;
    for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
        const unsigned j = c->F.idx[k];
        double r[3], g[3], dv[3];
        diffv(xi, s->x + 3 * (size_t)j, r);
        kGradW(&c->K, r, g);
        diffv(vi, s->v + 3 * (size_t)j, dv);
        acc += dot3(dv, g);
    }
    acc *= c->V;
    /* (v_i - v_b) . gradW_ib, v_b the boundary point's velocity (TimeStepDFSPH.cpp:1218-1238) */
    for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
        const unsigned j = c->B.idx[k];
        double r[3], g[3], vb[3];
        diffv(xi, s->xb + 3 * (size_t)j, r);
        kGradW(&c->K, r, g);
        boundary_velocity(c, j, vb);
        const double dv[3] = {(double)vi[0] - vb[0], (double)vi[1] - vb[1], (double)vi[2] - vb[2]};
        acc += (double)s->Vb[j] * dot3(dv, g);
    }
    return acc;
}

/* computePressureAccel, scalar path (TimeStepDFSPH.cpp:1299-1367), for the particles of one
 * phase (phase < 0: all). */
static void pressure_accel(ctx_t *c, const real *kap, int phase)
{
    orc_state *s = c->s;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)s->n; i++) {
        if (phase >= 0 && c->ph[i] != phase) continue;
        const real *xi = s->x + 3 * i;
        const double pi = (double)kap[i];
        double ai[3] = {0, 0, 0};
        for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
            const unsigned j = c->F.idx[k];
            /* kappa_i + density0_j / density0_i kappa_j (:1312) */
            const double ratio = c->r0 ? c->r0[j] / c->r0[i] : 1.0;
            const double psum = pi + ratio * (double)kap[j];
            if (fabs(psum) > c->eps) {
                double r[3], g[3];
                diffv(xi, s->x + 3 * (size_t)j, r);
                kGradW(&c->K, r, g);
                ai[0] += psum * (-c->V * g[0]);
                ai[1] += psum * (-c->V * g[1]);
                ai[2] += psum * (-c->V * g[2]);
            }
        }
        if (fabs(pi) > c->eps) {
            for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
                const unsigned j = c->B.idx[k];
                double r[3], g[3];
                diffv(xi, s->xb + 3 * (size_t)j, r);
                kGradW(&c->K, r, g);
                const double Vj = (double)s->Vb[j];
                ai[0] += pi * (-Vj * g[0]);
                ai[1] += pi * (-Vj * g[1]);
                ai[2] += pi * (-Vj * g[2]);
            }
        }
        s->pressure_accel[3 * i + 0] = (real)ai[0];
        s->pressure_accel[3 * i + 1] = (real)ai[1];
        s->pressure_accel[3 * i + 2] = (real)ai[2];
    }
}

/* Forces are collected when body_force is given and, for boundary particles, their bodies; with
 * volume maps the boundary "neighbour" j = i * nbodies + b belongs to map b. */
static inline int collects_forces(const orc_state *s, int vmaps)
{
    return s->body_force && (vmaps || s->body);
}

/* BoundaryModel::addForce (BoundaryModel.h:38-49): force f at point p on the body of boundary
 * particle j, torque (p - c) x f; only dynamic bodies collect.  Serial (deterministic). */
static void add_force_at(const ctx_t *c, unsigned j, const double p[3], const double f[3])
{
    orc_state *s = c->s;
    const int vmaps = c->p->boundary_method == 2;
    if (!collects_forces(s, vmaps)) return;
    const unsigned b = vmaps ? j % s->nvmaps : s->body[j];
    if (b >= s->nbodies || (s->body_dynamic && !s->body_dynamic[b])) return;
    const double *cen = s->body_center + 3 * (size_t)b;
    const double r[3] = {p[0] - cen[0], p[1] - cen[1], p[2] - cen[2]};
    double *F = s->body_force + 3 * (size_t)b, *T = s->body_torque + 3 * (size_t)b;
    F[0] += f[0]; F[1] += f[1]; F[2] += f[2];
    T[0] += r[1] * f[2] - r[2] * f[1];
    T[1] += r[2] * f[0] - r[0] * f[2];
    T[2] += r[0] * f[1] - r[1] * f[0];
}

/* ... at the boundary particle (or volume-map boundary point) x_j itself */
static void add_force(const ctx_t *c, unsigned j, const double f[3])
{
    const real *xb = c->s->xb + 3 * (size_t)j;
    const double p[3] = {(double)xb[0], (double)xb[1], (double)xb[2]};
    add_force_at(c, j, p, f);
}

/* The four samples that stand for a volume-map boundary point in the Weiler2018 boundary term
 * (Viscosity_Weiler2018.cpp:205-255, 383-430, 697-740, 1031-1080): x_j -+ t1 d and x_j -+ t2 d
 * with d = 0.5 h (m_tangentialDistanceFactor, :29) and t1, t2 from
 * MathFunctions::getOrthogonalVectors (MathFunctions.cpp:234-247) of n = (x_j - x_i) / |.|;
 * each carries a quarter of V_j.  0 when |x_i - x_j| <= 1e-4. */
static int vmap_samples(const real *xi, const real *xj, double h, double xs[4][3])
{
    double n[3] = {(double)xj[0] - (double)xi[0], (double)xj[1] - (double)xi[1], (double)xj[2] - (double)xi[2]};
    const double nl = sqrt(dot3(n, n));
    if (!(nl > 1.0e-4)) return 0;
    for (int d = 0; d < 3; d++) n[d] /= nl;
    double v[3] = {1.0, 0.0, 0.0};
    if (fabs(dot3(v, n)) > 0.999) { v[0] = 0.0; v[1] = 1.0; }
    double t1[3] = {n[1] * v[2] - n[2] * v[1], n[2] * v[0] - n[0] * v[2], n[0] * v[1] - n[1] * v[0]};
    double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
    const double l1 = sqrt(dot3(t1, t1)), l2 = sqrt(dot3(t2, t2));
    for (int d = 0; d < 3; d++) { t1[d] /= l1; t2[d] /= l2; }
    const double dist = 0.5 * h;
    for (int d = 0; d < 3; d++) {
        xs[0][d] = (double)xj[d] - t1[d] * dist;
        xs[1][d] = (double)xj[d] + t1[d] * dist;
        xs[2][d] = (double)xj[d] - t2[d] * dist;
        xs[3][d] = (double)xj[d] + t2[d] * dist;
    }
    return 1;
}

/* computePressureAccel with applyBoundaryForces (TimeStepDFSPH.cpp:1337-1344):
 * a = kappa_i (-V_b gradW_ib), force on the boundary -m_i a. */
static void boundary_pressure_forces(ctx_t *c, const real *kap)
{
    orc_state *s = c->s;
    if (!collects_forces(s, c->p->boundary_method == 2)) return;
    for (long i = 0; i < (long)s->n; i++) {
        const double pi = (double)kap[i];
        if (!(fabs(pi) > c->eps)) continue;
        for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
            const unsigned j = c->B.idx[k];
            double r[3], g[3], f[3];
            diffv(s->x + 3 * i, s->xb + 3 * (size_t)j, r);
            kGradW(&c->K, r, g);
            const double Vj = (double)s->Vb[j];
            for (int d = 0; d < 3; d++) f[d] = -mass_of(c, i) * (pi * (-Vj * g[d]));
            add_force(c, j, f);
        }
    }
}

/* compute_aij_pj, scalar path (TimeStepDFSPH.cpp:1370-1420). */
static double aij_pj(const ctx_t *c, long i)
{
    const orc_state *s = c->s;
    const real *xi = s->x + 3 * i;
    const real *ai = s->pressure_accel + 3 * i;
    double acc = 0.0;
    for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
        const unsigned j = c->F.idx[k];
        double r[3], g[3], da[3];
        diffv(xi, s->x + 3 * (size_t)j, r);
        kGradW(&c->K, r, g);
        diffv(ai, s->pressure_accel + 3 * (size_t)j, da);
        acc += dot3(da, g);
    }
    acc *= c->V;
    const double a[3] = {(double)ai[0], (double)ai[1], (double)ai[2]};
    for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
        const unsigned j = c->B.idx[k];
        double r[3], g[3];
        diffv(xi, s->xb + 3 * (size_t)j, r);
        kGradW(&c->K, r, g);
        acc += (double)s->Vb[j] * dot3(a, g);
    }
    return acc;
}

/* neighbours of all point sets (TimeStepDFSPH.cpp:421-423); volume maps are no point set */
static inline unsigned num_neighbors(const ctx_t *c, long i)
{
    const unsigned nb = c->p->boundary_method == 2 ? 0u : (c->B.off[i + 1] - c->B.off[i]);
    return (c->F.off[i + 1] - c->F.off[i]) + nb;
}

/* TimeStepDFSPH::divergenceSolve (TimeStepDFSPH.cpp:386-541) with
 * divergenceSolveIteration (:621-706); USE_WARMSTART_V (TimeStepDFSPH.h:10). */
static void divergence_solve(ctx_t *c, double h, double *err_buf)
{
    orc_state *s = c->s;
    const double invH = 1.0 / h;
    const long n = (long)s->n;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        const double dadv_stored = velocity_divergence(c, i);   /* computeDensityChange */
        s->density_adv[i] = (real)dadv_stored;
        if (s->density_adv_v) s->density_adv_v[i] = (real)dadv_stored;
        double densityAdv = dadv_stored > 0.0 ? dadv_stored : 0.0;
        if (num_neighbors(c, i) < 20) densityAdv = 0.0;      /* 3D deficiency */
        s->factor[i] = (real)((double)s->factor[i] * invH);
        if (densityAdv > 0.0) {
            const double kv = (double)s->kappa_v[i];
            s->kappa_v[i] = (real)(0.5 * (kv < 0.5 ? kv : 0.5) * invH);
        } else {
            s->kappa_v[i] = 0;
        }
    }
    unsigned it = 0;
    double avg = 0.0;
    int chk = 0;
    /* one iteration visits the fluid models in turn, each with its own tolerance (:476-495) */
    const int nph = c->r0 ? (int)c->nph : 1;
    while ((!chk || it < 1) && it < c->p->max_iterations_v) {
        chk = 1;
        for (int k = 0; k < nph; k++) {
            const int phase = c->r0 ? k : -1;
            pressure_accel(c, s->kappa_v, phase);
#pragma omp parallel for schedule(static)
            for (long i = 0; i < n; i++) {
                if (phase >= 0 && c->ph[i] != phase) { err_buf[i] = 0.0; continue; }
                const double apj = aij_pj(c, i) * h;
                const double si = -(double)s->density_adv[i];
                double residuum = si - apj < 0.0 ? si - apj : 0.0;
                if (num_neighbors(c, i) < 20) residuum = 0.0;
                double kv = (double)s->kappa_v[i] - 0.5 * (si - apj) * (double)s->factor[i];
                s->kappa_v[i] = (real)(kv > 0.0 ? kv : 0.0);
                err_buf[i] = -rho0_of(c, i) * residuum;
            }
            const double cnt = phase >= 0 ? (double)s->phase_count[k] : (double)n;
            const double rho0k = phase >= 0 ? s->phase_density0[k] : c->rho0;
            avg = serial_sum(err_buf, (size_t)n) / cnt;
            chk = chk && avg <= invH * c->p->max_error_v * 0.01 * rho0k;
        }
        it++;
    }
    s->iterations_v = it;
    s->avg_density_err_v = avg;
    pressure_accel(c, s->kappa_v, -1);
    boundary_pressure_forces(c, s->kappa_v);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        for (int d = 0; d < 3; d++)
            s->v[3 * i + d] = (real)((double)s->v[3 * i + d] + h * (double)s->pressure_accel[3 * i + d]);
        s->factor[i] = (real)((double)s->factor[i] * h);
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) s->kappa_v[i] = (real)((double)s->kappa_v[i] * h);
}

/* TimeStepDFSPH::pressureSolve (TimeStepDFSPH.cpp:252-384) with
 * pressureSolveIteration (:544-619); USE_WARMSTART (TimeStepDFSPH.h:9). */
static void pressure_solve(ctx_t *c, double h, double *err_buf)
{
    orc_state *s = c->s;
    const double h2 = h * h, invH2 = 1.0 / h2;
    const long n = (long)s->n;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        /* computeDensityAdv (:1190-1243) */
        const double delta = velocity_divergence(c, i);
        s->density_adv[i] = (real)((double)s->density[i] / rho0_of(c, i) + h * delta);
        s->factor[i] = (real)((double)s->factor[i] * invH2);
        if ((double)s->density_adv[i] > 1.0) {
            const double k = (double)s->kappa[i];
            s->kappa[i] = (real)(0.5 * (k < 0.00025 ? k : 0.00025) * invH2);
        } else {
            s->kappa[i] = 0;
        }
    }
    unsigned it = 0;
    double avg = 0.0;
    int chk = 0;
    /* one iteration visits the fluid models in turn, each with its own tolerance (:322-339) */
    const int nph = c->r0 ? (int)c->nph : 1;
    while ((!chk || it < c->p->min_iterations) && it < c->p->max_iterations) {
        chk = 1;
        for (int m = 0; m < nph; m++) {
            const int phase = c->r0 ? m : -1;
            pressure_accel(c, s->kappa, phase);
#pragma omp parallel for schedule(static)
            for (long i = 0; i < n; i++) {
                if (phase >= 0 && c->ph[i] != phase) { err_buf[i] = 0.0; continue; }
                const double apj = aij_pj(c, i) * h * h;
                const double si = 1.0 - (double)s->density_adv[i];
                const double residuum = si - apj < 0.0 ? si - apj : 0.0;
                const double k = (double)s->kappa[i] - 0.5 * (si - apj) * (double)s->factor[i];
                s->kappa[i] = (real)(k > 0.0 ? k : 0.0);
                err_buf[i] = -rho0_of(c, i) * residuum;
            }
            const double cnt = phase >= 0 ? (double)s->phase_count[m] : (double)n;
            const double rho0m = phase >= 0 ? s->phase_density0[m] : c->rho0;
            avg = serial_sum(err_buf, (size_t)n) / cnt;
            chk = chk && avg <= c->p->max_error * 0.01 * rho0m;
        }
        it++;
    }
    s->iterations = it;
    s->avg_density_err = avg;
    pressure_accel(c, s->kappa, -1);
    boundary_pressure_forces(c, s->kappa);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
            s->v[3 * i + d] = (real)((double)s->v[3 * i + d] + h * (double)s->pressure_accel[3 * i + d]);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) s->kappa[i] = (real)((double)s->kappa[i] * h2);
}

/* XSPH::step, scalar path (XSPH.cpp:138-211); static boundary => v_b = 0. */
/* XSPH coefficients of particle i's model (each FluidModel's XSPH has its own, XSPH.cpp:19-39) */
static double xsph_cf(const ctx_t *c, long i)
{
    return (c->r0 && c->s->phase_xsph) ? c->s->phase_xsph[c->ph[i]] : c->p->xsph_fluid;
}
static double xsph_cb(const ctx_t *c, long i)
{
    return (c->r0 && c->s->phase_xsph_boundary) ? c->s->phase_xsph_boundary[c->ph[i]] : c->p->xsph_boundary;
}

static void xsph(ctx_t *c, double h)
{
    orc_state *s = c->s;
    const double invH = 1.0 / h;
    int any_cb = 0;
    for (long i = 0; i < (long)s->n; i++) any_cb |= xsph_cb(c, i) != 0.0;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)s->n; i++) {
        const real *xi = s->x + 3 * i, *vi = s->v + 3 * i;
        const double cf = xsph_cf(c, i), cb = xsph_cb(c, i);
        double ai[3] = {0, 0, 0};
        for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
            const unsigned j = c->F.idx[k];
            double r[3], dv[3];
            diffv(xi, s->x + 3 * (size_t)j, r);
            diffv(vi, s->v + 3 * (size_t)j, dv);
            const double w = invH * cf * (mass_of(c, j) / (double)s->density[j]) * kW(&c->K, sqrt(dot3(r, r)));
            ai[0] -= w * dv[0]; ai[1] -= w * dv[1]; ai[2] -= w * dv[2];
        }
        if (cb != 0.0) {
            const double rhoi = (double)s->density[i];
            for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
                const unsigned j = c->B.idx[k];
                double r[3];
                diffv(xi, s->xb + 3 * (size_t)j, r);
                const double w = invH * cb * (rho0_of(c, i) * (double)s->Vb[j] / rhoi) * kW(&c->K, sqrt(dot3(r, r)));
                double vb[3];
                boundary_velocity(c, j, vb);
                for (int d = 0; d < 3; d++) ai[d] -= w * ((double)vi[d] - vb[d]);
            }
        }
        for (int d = 0; d < 3; d++) s->a[3 * i + d] = (real)((double)s->a[3 * i + d] + ai[d]);
    }
    /* boundary feedback of the XSPH boundary term (XSPH.cpp:183-203): force -m_i a_ib */
    if (any_cb && collects_forces(s, c->p->boundary_method == 2))
        for (long i = 0; i < (long)s->n; i++) {
            const real *xi = s->x + 3 * i, *vi = s->v + 3 * i;
            const double rhoi = (double)s->density[i], cb = xsph_cb(c, i);
            for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
                const unsigned j = c->B.idx[k];
                double r[3], f[3];
                diffv(xi, s->xb + 3 * (size_t)j, r);
                const double w = invH * cb * (rho0_of(c, i) * (double)s->Vb[j] / rhoi) * kW(&c->K, sqrt(dot3(r, r)));
                double vb[3];
                boundary_velocity(c, j, vb);
                for (int d = 0; d < 3; d++) f[d] = -mass_of(c, i) * (-w * ((double)vi[d] - vb[d]));
                add_force(c, j, f);
            }
        }
}

/* ------------------------------------------------------------------------ */
/* Weiler et al. 2018 implicit viscosity (Viscosity_Weiler2018.cpp).          */
/* ------------------------------------------------------------------------ */
/* One system per fluid model (Viscosity_Weiler2018 is a per-model NonPressureForceBase, its
 * sums run over forall_fluid_neighbors_in_same_phase): the particles [lo, hi) of phase ph
 * (-1: the one model), its rest density rho0 and mu = nu rho0, mub = nu_b rho0. */
typedef struct {
    ctx_t *c;
    double dt, mu, mub, h2, d, rho0;
    long lo, hi;
    int ph;
} visc_t;

/* nu and nu_b of phase ph (-1: the one model) */
static double phase_nu(const ctx_t *c, int ph)
{
    return (ph >= 0 && c->s->phase_viscosity) ? c->s->phase_viscosity[ph] : c->p->viscosity;
}
static double phase_nub(const ctx_t *c, int ph)
{
    return (ph >= 0 && c->s->phase_viscosity_boundary) ? c->s->phase_viscosity_boundary[ph] : c->p->viscosity_boundary;
}

static visc_t visc_make(ctx_t *c, double dt, int ph, long lo, long hi)
{
    visc_t w;
    w.c = c;
    w.dt = dt;
    w.rho0 = ph >= 0 ? c->s->phase_density0[ph] : c->rho0;
    w.mu = phase_nu(c, ph) * w.rho0;             /* :288 */
    w.mub = phase_nub(c, ph) * w.rho0;           /* :289 */
    w.h2 = c->K.h * c->K.h;
    w.d = 10.0;                                  /* 3D, :292-294 */
    w.lo = lo;
    w.hi = hi;
    w.ph = ph;
    return w;
}

/* a fluid neighbour of another phase takes no part in the phase's system */
static inline int visc_skip(const visc_t *w, unsigned j) { return w->ph >= 0 && w->c->ph[j] != w->ph; }

/* matrixVecProd, scalar path (Viscosity_Weiler2018.cpp:271-443). */
static void visc_matvec(const visc_t *w, const real *vec, real *result)
{
    const ctx_t *c = w->c;
    const orc_state *s = c->s;
#pragma omp parallel for schedule(static)
    for (long i = w->lo; i < w->hi; i++) {
        const real *xi = s->x + 3 * i;
        const double rhoi = (double)s->density[i];
        const real *vi = vec + 3 * i;
        double ai[3] = {0, 0, 0};
        for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
            const unsigned j = c->F.idx[k];
            if (visc_skip(w, j)) continue;
            double r[3], g[3], dv[3];
            diffv(xi, s->x + 3 * (size_t)j, r);
            kGradW(&c->K, r, g);
            diffv(vi, vec + 3 * (size_t)j, dv);
            const double f = w->d * w->mu * (mass_of(c, j) / (double)s->density[j]) * dot3(dv, r) / (dot3(r, r) + 0.01 * w->h2);
            ai[0] += f * g[0]; ai[1] += f * g[1]; ai[2] += f * g[2];
        }
        if (w->mub != 0.0) {
            const double v3[3] = {(double)vi[0], (double)vi[1], (double)vi[2]};
            for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
                const unsigned j = c->B.idx[k];
                if (c->p->boundary_method == 2) {   /* four samples, a quarter of V_j each, no rho0 / rho_i */
                    double xs[4][3];
                    if (!vmap_samples(xi, s->xb + 3 * (size_t)j, c->K.h, xs)) continue;
                    const double vol = 0.25 * (double)s->Vb[j];
                    for (int q = 0; q < 4; q++) {
                        double r[3], g[3];
                        for (int d = 0; d < 3; d++) r[d] = (double)xi[d] - xs[q][d];
                        kGradW(&c->K, r, g);
                        const double f = w->d * w->mub * vol * dot3(v3, r) / (dot3(r, r) + 0.01 * w->h2);
                        ai[0] += f * g[0]; ai[1] += f * g[1]; ai[2] += f * g[2];
                    }
                    continue;
                }
                double r[3], g[3];
                diffv(xi, s->xb + 3 * (size_t)j, r);
                kGradW(&c->K, r, g);
                const double f = w->d * w->mub * (w->rho0 * (double)s->Vb[j] / rhoi) * dot3(v3, r) / (dot3(r, r) + 0.01 * w->h2);
                ai[0] += f * g[0]; ai[1] += f * g[1]; ai[2] += f * g[2];
            }
        }
        for (int d = 0; d < 3; d++)
            result[3 * i + d] = (real)((double)vec[3 * i + d] - w->dt / rhoi * ai[d]);
    }
}

/* diagonalMatrixElement with USE_BLOCKDIAGONAL_PRECONDITIONER, scalar path
 * (Viscosity_Weiler2018.cpp:605-742), followed by the 3x3 inverse taken in
 * BlockJacobiPreconditioner3D::compute (MatrixFreeSolver.h:231-244).
 * Writes the inverse block row-major into inv9. */
static void visc_diag_inverse(const visc_t *w, real *diag9, real *inv9)
{
    const ctx_t *c = w->c;
    const orc_state *s = c->s;
#pragma omp parallel for schedule(static)
    for (long i = w->lo; i < w->hi; i++) {
        const real *xi = s->x + 3 * i;
        const double rhoi = (double)s->density[i];
        double R[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (unsigned k = c->F.off[i]; k < c->F.off[i + 1]; k++) {
            const unsigned j = c->F.idx[k];
            if (visc_skip(w, j)) continue;
            double r[3], g[3];
            diffv(xi, s->x + 3 * (size_t)j, r);
            kGradW(&c->K, r, g);
            const double f = w->d * w->mu * (mass_of(c, j) / (double)s->density[j]) / (dot3(r, r) + 0.01 * w->h2);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) R[3 * a + b] += f * g[a] * r[b];
        }
        if (w->mub != 0.0) {
            for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
                const unsigned j = c->B.idx[k];
                if (c->p->boundary_method == 2) {
                    double xs[4][3];
                    if (!vmap_samples(xi, s->xb + 3 * (size_t)j, c->K.h, xs)) continue;
                    const double vol = 0.25 * (double)s->Vb[j];
                    for (int q = 0; q < 4; q++) {
                        double r[3], g[3];
                        for (int d = 0; d < 3; d++) r[d] = (double)xi[d] - xs[q][d];
                        kGradW(&c->K, r, g);
                        const double f = w->d * w->mub * vol / (dot3(r, r) + 0.01 * w->h2);
                        for (int a = 0; a < 3; a++)
                            for (int b = 0; b < 3; b++) R[3 * a + b] += f * g[a] * r[b];
                    }
                    continue;
                }
                double r[3], g[3];
                diffv(xi, s->xb + 3 * (size_t)j, r);
                kGradW(&c->K, r, g);
                const double f = w->d * w->mub * (w->rho0 * (double)s->Vb[j] / rhoi) / (dot3(r, r) + 0.01 * w->h2);
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) R[3 * a + b] += f * g[a] * r[b];
            }
        }
        double M[9];
        for (int a = 0; a < 9; a++) M[a] = ((a % 4) == 0 ? 1.0 : 0.0) - (w->dt / rhoi) * R[a];
        if (diag9)
            for (int a = 0; a < 9; a++) diag9[9 * i + a] = (real)M[a];
        if (inv9) {
            /* adjugate / determinant */
            const double c00 = M[4] * M[8] - M[5] * M[7];
            const double c01 = M[5] * M[6] - M[3] * M[8];
            const double c02 = M[3] * M[7] - M[4] * M[6];
            const double det = M[0] * c00 + M[1] * c01 + M[2] * c02;
            const double id = 1.0 / det;
            double I[9];
            I[0] = c00 * id;
            I[1] = (M[2] * M[7] - M[1] * M[8]) * id;
            I[2] = (M[1] * M[5] - M[2] * M[4]) * id;
            I[3] = c01 * id;
            I[4] = (M[0] * M[8] - M[2] * M[6]) * id;
            I[5] = (M[2] * M[3] - M[0] * M[5]) * id;
            I[6] = c02 * id;
            I[7] = (M[1] * M[6] - M[0] * M[7]) * id;
            I[8] = (M[0] * M[4] - M[1] * M[3]) * id;
            for (int a = 0; a < 9; a++) inv9[9 * i + a] = (real)I[a];
        }
    }
}

/* computeRHS (Viscosity_Weiler2018.cpp:1091-1254): b = v - dt / rho_i sum_b (boundary term of
 * the boundary's velocity), warm start g = v + vDiff.  Boundary particles are static walls (the
 * term vanishes); a moving volume-map body contributes at its four samples per boundary point
 * (:1191-1243). */
static void visc_rhs(const visc_t *w, real *b, real *g)
{
    const ctx_t *c = w->c;
    const orc_state *s = c->s;
    for (size_t i = 3 * (size_t)w->lo; i < 3 * (size_t)w->hi; i++) {
        b[i] = s->v[i];
        g[i] = (real)((double)s->v[i] + (double)s->vdiff[i]);
    }
    if (w->mub == 0.0) return;
    if (c->p->boundary_method != 2) {   /* moving boundary particles (:1130-1138) */
        if (!s->vb) return;
        for (long i = w->lo; i < w->hi; i++) {
            const real *xi = s->x + 3 * i;
            const double rhoi = (double)s->density[i];
            double bi[3] = {0, 0, 0};
            for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
                const unsigned j = c->B.idx[k];
                double r[3], gw[3], vj[3];
                diffv(xi, s->xb + 3 * (size_t)j, r);
                kGradW(&c->K, r, gw);
                boundary_velocity(c, j, vj);
                const double f = w->d * w->mub * (w->rho0 * (double)s->Vb[j] / rhoi) * dot3(vj, r) / (dot3(r, r) + 0.01 * w->h2);
                for (int d = 0; d < 3; d++) bi[d] += f * gw[d];
            }
            for (int d = 0; d < 3; d++) b[3 * i + d] = (real)((double)s->v[3 * i + d] - w->dt / rhoi * bi[d]);
        }
        return;
    }
    for (long i = w->lo; i < w->hi; i++) {
        const real *xi = s->x + 3 * i;
        double bi[3] = {0, 0, 0};
        for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
            const unsigned j = c->B.idx[k];
            double xs[4][3];
            if (!vmap_samples(xi, s->xb + 3 * (size_t)j, c->K.h, xs)) continue;
            const double vol = 0.25 * (double)s->Vb[j];
            for (int q = 0; q < 4; q++) {
                double r[3], gw[3], vk[3];
                for (int d = 0; d < 3; d++) r[d] = (double)xi[d] - xs[q][d];
                kGradW(&c->K, r, gw);
                boundary_point_velocity(c, j, xs[q], vk);
                const double f = w->d * w->mub * vol * dot3(vk, r) / (dot3(r, r) + 0.01 * w->h2);
                for (int d = 0; d < 3; d++) bi[d] += f * gw[d];
            }
        }
        const double rhoi = (double)s->density[i];
        for (int d = 0; d < 3; d++) b[3 * i + d] = (real)((double)s->v[3 * i + d] - w->dt / rhoi * bi[d]);
    }
}

static double vdot(const real *a, const real *b, size_t n)
{
    double s = 0.0;
    for (size_t i = 0; i < n; i++) s += (double)a[i] * (double)b[i];
    return s;
}

static void precond_apply(const real *inv9, const real *r, real *z, long lo, long hi)
{
#pragma omp parallel for schedule(static)
    for (long i = lo; i < hi; i++)
        for (int a = 0; a < 3; a++)
            z[3 * i + a] = (real)((double)inv9[9 * i + 3 * a + 0] * (double)r[3 * i + 0] +
                                  (double)inv9[9 * i + 3 * a + 1] * (double)r[3 * i + 1] +
                                  (double)inv9[9 * i + 3 * a + 2] * (double)r[3 * i + 2]);
}

/* Eigen::internal::conjugate_gradient (extern/eigen/Eigen/src/IterativeLinearSolvers/
 * ConjugateGradient.h:29-90) on the matrix-free operator, as driven by
 * Viscosity_Weiler2018::step (Viscosity_Weiler2018.cpp:891-926). */
static int visc_cg(const visc_t *w, const real *b, real *x, const real *inv9,
                   unsigned max_iters, double tol, unsigned *iters_out, double *err_out)
{
    const unsigned n = w->c->s->n;
    const size_t N = 3 * (size_t)n;
    const size_t k0 = 3 * (size_t)w->lo, k1 = 3 * (size_t)w->hi, M = k1 - k0;   /* the phase's rows */
    real *r = (real *)malloc(N * sizeof(real));
    real *p = (real *)malloc(N * sizeof(real));
    real *z = (real *)malloc(N * sizeof(real));
    real *t = (real *)malloc(N * sizeof(real));
    if (!r || !p || !z || !t) { free(r); free(p); free(z); free(t); return -2; }
    visc_matvec(w, x, t);
    for (size_t k = k0; k < k1; k++) r[k] = (real)((double)b[k] - (double)t[k]);
    const double rhsNorm2 = vdot(b + k0, b + k0, M);
    if (rhsNorm2 == 0.0) {
        for (size_t k = k0; k < k1; k++) x[k] = 0;
        *iters_out = 0;
        *err_out = 0.0;
        free(r); free(p); free(z); free(t);
        return 0;
    }
    const double considerAsZero = (sizeof(real) == sizeof(double)) ? DBL_MIN : (double)FLT_MIN;
    double threshold = tol * tol * rhsNorm2;
    if (threshold < considerAsZero) threshold = considerAsZero;
    double resNorm2 = vdot(r + k0, r + k0, M);
    if (resNorm2 < threshold) {
        *iters_out = 0;
        *err_out = sqrt(resNorm2 / rhsNorm2);
        free(r); free(p); free(z); free(t);
        return 0;
    }
    precond_apply(inv9, r, p, w->lo, w->hi);
    double absNew = vdot(r + k0, p + k0, M);
    unsigned i = 0;
    while (i < max_iters) {
        visc_matvec(w, p, t);
        const double alpha = absNew / vdot(p + k0, t + k0, M);
        for (size_t k = k0; k < k1; k++) {
            x[k] = (real)((double)x[k] + alpha * (double)p[k]);
            r[k] = (real)((double)r[k] - alpha * (double)t[k]);
        }
        resNorm2 = vdot(r + k0, r + k0, M);
        if (resNorm2 < threshold) break;
        precond_apply(inv9, r, z, w->lo, w->hi);
        const double absOld = absNew;
        absNew = vdot(r + k0, z + k0, M);
        const double beta = absNew / absOld;
        for (size_t k = k0; k < k1; k++) p[k] = (real)((double)z[k] + beta * (double)p[k]);
        i++;
    }
    *iters_out = i;
    *err_out = sqrt(resNorm2 / rhsNorm2);
    free(r); free(p); free(z); free(t);
    return 0;
}

/* Viscosity_Weiler2018::step + applyForces (Viscosity_Weiler2018.cpp:891-936), once per fluid
 * model in model order (TimeStepDFSPH.cpp:172-173 runs each model's non-pressure forces); the
 * reported iterations are the models' sum, the error their largest. */
static int viscosity_weiler(ctx_t *c, double dt)
{
    orc_state *s = c->s;
    const size_t N = 3 * (size_t)s->n;
    if (s->n == 0) return 0;
    real *b = (real *)malloc(N * sizeof(real));
    real *x = (real *)malloc(N * sizeof(real));
    real *inv9 = (real *)malloc(3 * N * sizeof(real));
    if (!b || !x || !inv9) { free(b); free(x); free(inv9); return -2; }
    const int nph = c->r0 ? (int)c->nph : 1;
    int rc = 0;
    long lo = 0;
    s->visco_iterations = 0;
    s->visco_error = 0.0;
    for (int ph = 0; ph < nph && rc == 0; ph++) {
        const long hi = c->r0 ? lo + (long)s->phase_count[ph] : (long)s->n;
        visc_t w = visc_make(c, dt, c->r0 ? ph : -1, lo, hi);
        visc_diag_inverse(&w, NULL, inv9);
        visc_rhs(&w, b, x);
        unsigned it = 0;
        double err = 0.0;
        rc = visc_cg(&w, b, x, inv9, c->p->visco_max_iter, c->p->visco_max_error, &it, &err);
        s->visco_iterations += it;
        if (err > s->visco_error) s->visco_error = err;
        lo = hi;
    }
    for (size_t k = 0; k < N; k++) {
        const double dv = (double)x[k] - (double)s->v[k];
        s->a[k] = (real)((double)s->a[k] + (1.0 / dt) * dv);
        s->vdiff[k] = (real)dv;
    }
    /* boundary feedback of applyForces (Viscosity_Weiler2018.cpp:960-975), static v_b = 0:
     * a = d mub (rho0 V_b / rho_i) (v_i'.x_ib) / (|x_ib|^2 + 0.01 h^2) gradW_ib, force -m_i / rho_i a,
     * rho0, mub and m_i those of the particle's model */
    int any_mub = 0;
    for (int ph = 0; ph < nph; ph++) any_mub |= phase_nub(c, c->r0 ? ph : -1) != 0.0;
    if (any_mub && collects_forces(s, c->p->boundary_method == 2)) {
        const double h2 = c->K.h * c->K.h;
        for (long i = 0; i < (long)s->n; i++) {
            const double rhoi = (double)s->density[i];
            const double r0 = rho0_of(c, i), mub = phase_nub(c, c->r0 ? c->ph[i] : -1) * r0, mi = mass_of(c, i);
            const double nv[3] = {(double)x[3 * i], (double)x[3 * i + 1], (double)x[3 * i + 2]};
            for (unsigned k = c->B.off[i]; k < c->B.off[i + 1]; k++) {
                const unsigned j = c->B.idx[k];
                if (c->p->boundary_method == 2) {   /* at the four samples (:1031-1080) */
                    double xs[4][3];
                    if (!vmap_samples(s->x + 3 * i, s->xb + 3 * (size_t)j, c->K.h, xs)) continue;
                    const double vol = 0.25 * (double)s->Vb[j];
                    for (int q = 0; q < 4; q++) {
                        double r[3], g[3], f[3], vk[3];
                        for (int d = 0; d < 3; d++) r[d] = (double)s->x[3 * i + d] - xs[q][d];
                        kGradW(&c->K, r, g);
                        boundary_point_velocity(c, j, xs[q], vk);
                        const double dv[3] = {nv[0] - vk[0], nv[1] - vk[1], nv[2] - vk[2]};
                        const double coef = 10.0 * mub * vol * dot3(dv, r) / (dot3(r, r) + 0.01 * h2);
                        for (int d = 0; d < 3; d++) f[d] = -mi / rhoi * (coef * g[d]);
                        add_force_at(c, j, xs[q], f);
                    }
                    continue;
                }
                double r[3], g[3], f[3], vj[3];
                diffv(s->x + 3 * i, s->xb + 3 * (size_t)j, r);
                kGradW(&c->K, r, g);
                boundary_velocity(c, j, vj);
                const double dv[3] = {nv[0] - vj[0], nv[1] - vj[1], nv[2] - vj[2]};
                const double coef = 10.0 * mub * (r0 * (double)s->Vb[j] / rhoi) * dot3(dv, r) / (dot3(r, r) + 0.01 * h2);
                for (int d = 0; d < 3; d++) f[d] = -mi / rhoi * (coef * g[d]);
                add_force(c, j, f);
            }
        }
    }
    free(b); free(x); free(inv9);
    return rc;
}

/* Simulation::updateTimeStepSize / updateTimeStepSizeCFL (Simulation.cpp:395-493);
 * static Akinci2012 boundaries do not contribute. */
static double update_time_step(const ctx_t *c, double h)
{
    const orc_state *s = c->s;
    const orc_params *p = c->p;
    if (p->cfl_method == 0) return h;
    double maxVel = 0.0;
    for (unsigned i = 0; i < s->n; i++) {
        double m = 0.0;
        for (int d = 0; d < 3; d++) {
            const double vv = (double)s->v[3 * i + d] + (double)s->a[3 * i + d] * h;
            m += vv * vv;
        }
        if (m > maxVel) maxVel = m;
    }
    /* the boundary particles of moving bodies (Simulation.cpp:442-458) */
    if (p->boundary_method != 2 && s->vb)
        for (unsigned j = 0; j < s->nb; j++) {
            double m = 0.0;
            for (int d = 0; d < 3; d++) m += (double)s->vb[3 * (size_t)j + d] * (double)s->vb[3 * (size_t)j + d];
            if (m > maxVel) maxVel = m;
        }
    /* a moving volume-map body: |w x (maxDist, 0, 0) + v| (SimulatorBase::updateVMVelocity,
     * SimulatorBase.cpp:1670-1687), taken into the maximum of the squared fluid speeds as it is
     * (Simulation.cpp:466-476) */
    if (p->boundary_method == 2)
        for (unsigned b = 0; b < s->nvmaps; b++) {
            const orc_vmap *m = s->vmaps + b;
            const double vel[3] = {m->v[0], m->v[1] + m->w[2] * m->max_dist, m->v[2] - m->w[1] * m->max_dist};
            const double speed = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
            if (speed > maxVel) maxVel = speed;
        }
    if (maxVel < 1.0e-9) maxVel = 1.0e-9;
    double hn = p->cfl_factor * 0.4 * (2.0 * p->radius / sqrt(maxVel));
    if (hn > p->cfl_max) hn = p->cfl_max;
    if (hn < p->cfl_min) hn = p->cfl_min;
    if (p->cfl_method == 2) {
        /* :399-412, uses the pressure iterations of the previous step */
        const unsigned iters = s->iterations;
        if (iters == 0) return hn;
        double hh = h;
        if (iters > 10) hh *= 0.9;
        else if (iters < 5) hh *= 1.1;
        return hh < hn ? hh : hn;
    }
    return hn;
}

/* TimeStep::computeVolumeAndBoundaryX (TimeStep.cpp:219-340) for static bodies (v_b = 0): for
 * every particle and body (in body order, so a particle moved by one body is seen moved by the
 * next, as in the reference), the boundary point x_j = x_i - max(phi + r / 2, 2 r) n and volume
 * V_j of the particle's volume-map sample, and, for a particle inside a body (phi <= 0), its move
 * of min(2 r - phi, r / 10) along n with v_i = 0.  The samples with V_j > 0 become the
 * particle's boundary "neighbours" i * nbodies + b, so the Akinci2012 sums of the step apply to
 * them unchanged, as forall_volume_maps does (Simulation.h:79-89). */
static int volume_maps_boundary(ctx_t *c, real **xb_out, real **Vb_out)
{
    orc_state *s = c->s;
    const unsigned nbod = s->nvmaps;
    const long n = (long)s->n;
    const double r = c->p->radius, hs = c->K.h;
    real *xb = (real *)calloc(3 * (size_t)n * nbod + 1, sizeof(real));
    real *Vb = (real *)calloc((size_t)n * nbod + 1, sizeof(real));
    c->B.off = (unsigned *)calloc((size_t)n + 1, sizeof(unsigned));
    c->B.idx = (unsigned *)malloc(((size_t)n * nbod + 1) * sizeof(unsigned));
    if (!xb || !Vb || !c->B.off || !c->B.idx) { free(xb); free(Vb); return -2; }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        unsigned cnt = 0;
        for (unsigned b = 0; b < nbod; b++) {
            const orc_vmap *m = s->vmaps + b;
            real *xr = s->x + 3 * i;
            const double xi[3] = {(double)xr[0], (double)xr[1], (double)xr[2]};
            double dx[3], local[3], gl[3] = {0, 0, 0}, nrm[3];
            for (int d = 0; d < 3; d++) dx[d] = xi[d] - m->t[d];
            for (int k = 0; k < 3; k++) local[k] = m->R[k] * dx[0] + m->R[3 + k] * dx[1] + m->R[6 + k] * dx[2];
            double dist = DBL_MAX;
            orc_vmap_interpolate(m, 0, local, &dist, gl);
            for (int k = 0; k < 3; k++) nrm[k] = m->R[3 * k] * gl[0] + m->R[3 * k + 1] * gl[1] + m->R[3 * k + 2] * gl[2];
            const double nl = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
            double V = 0.0, xj[3] = {0, 0, 0};
            if (dist > 0.0 && dist < hs) {
                double vol = DBL_MAX;
                if (orc_vmap_interpolate(m, 1, local, &vol, NULL) && vol > 0.0 && vol != DBL_MAX && nl > 1.0e-9) {
                    const double dd = fmax(dist + 0.5 * r, 2.0 * r);
                    for (int d = 0; d < 3; d++) xj[d] = xi[d] - dd * (nrm[d] / nl);
                    V = vol;
                }
            } else if (dist <= 0.0 && nl > 1.0e-5) {
                const double delta = fmin(2.0 * r - dist, 0.1 * r);
                for (int d = 0; d < 3; d++) {
                    xr[d] = (real)(xi[d] + delta * (nrm[d] / nl));
                    s->v[3 * i + d] = 0;
                }
            }
            const size_t e = (size_t)i * nbod + b;
            for (int d = 0; d < 3; d++) xb[3 * e + d] = (real)xj[d];
            Vb[e] = (real)V;
            if (Vb[e] > 0) cnt++;
        }
        c->B.off[i + 1] = cnt;
    }
    for (long i = 0; i < n; i++) c->B.off[i + 1] += c->B.off[i];
    for (long i = 0; i < n; i++) {
        unsigned k = c->B.off[i];
        for (unsigned b = 0; b < nbod; b++)
            if (Vb[(size_t)i * nbod + b] > 0) c->B.idx[k++] = (unsigned)((size_t)i * nbod + b);
    }
    *xb_out = xb;
    *Vb_out = Vb;
    return 0;
}

int orc_step(orc_state *s, const orc_params *p)
{
#ifdef _OPENMP
    if (p->num_threads > 0) omp_set_num_threads(p->num_threads);
#endif
    ctx_t c;
    memset(&c, 0, sizeof(c));
    c.s = s;
    c.p = p;
    c.K = kern_make(4.0 * p->radius);
    const double diam = 2.0 * p->radius;
    c.V = 0.8 * diam * diam * diam;           /* FluidModel.cpp:234-253 */
    c.rho0 = p->density0;
    c.mass = c.V * c.rho0;
    c.eps = 1.0e-5;                           /* TimeStepDFSPH.h:28 */
    const double h = s->dt;                   /* TimeStepDFSPH.cpp:121 */
    const long n = (long)s->n;
    int rc = 0;

    /* Bender2019: the bodies are the maps (no body array) */
    const int vmaps = p->boundary_method == 2;
    if (vmaps && s->body) return -5;
    /* several fluid phases: each particle's rest density */
    if (s->nphase > 1) {
        unsigned total = 0;
        for (unsigned k = 0; k < s->nphase; k++) total += s->phase_count[k];
        if (total != s->n) return -6;
        c.r0 = (double *)malloc(((size_t)n + 1) * sizeof(double));
        c.ph = (int *)malloc(((size_t)n + 1) * sizeof(int));
        if (!c.r0 || !c.ph) { free(c.r0); free(c.ph); return -2; }
        c.nph = s->nphase;
        long i = 0;
        for (unsigned k = 0; k < s->nphase; k++)
            for (unsigned q = 0; q < s->phase_count[k]; q++, i++) {
                c.r0[i] = s->phase_density0[k];
                c.ph[i] = (int)k;
            }
    }
    real *xb_saved = s->xb, *Vb_saved = s->Vb, *vxb = NULL, *vVb = NULL;
    const unsigned nb_saved = s->nb;
    if (lists_build(&c.F, s->n, s->x, s->n, s->x, c.K.h, 1, p->fp32_predicate) != 0) {
        free(c.r0); free(c.ph);
        return -1;
    }
    if (vmaps) {
        /* after the neighbourhood search, before the densities (TimeStepDFSPH.cpp:141-142) */
        if (volume_maps_boundary(&c, &vxb, &vVb) != 0) {
            lists_free(&c.F); lists_free(&c.B); free(c.r0); free(c.ph);
            return -2;
        }
        s->xb = vxb;
        s->Vb = vVb;
        s->nb = s->n * s->nvmaps;
    } else if (lists_build(&c.B, s->n, s->x, s->nb, s->xb, c.K.h, 0, p->fp32_predicate) != 0) {
        lists_free(&c.F);
        free(c.r0); free(c.ph);
        return -1;
    }
    if (s->num_fluid_neighbors)
        for (long i = 0; i < n; i++) s->num_fluid_neighbors[i] = c.F.off[i + 1] - c.F.off[i];
    if (s->num_boundary_neighbors)
        for (long i = 0; i < n; i++) s->num_boundary_neighbors[i] = vmaps ? 0u : c.B.off[i + 1] - c.B.off[i];
    double *err_buf = (double *)malloc(((size_t)n + 1) * sizeof(double));
    if (!err_buf) {
        lists_free(&c.F);
        lists_free(&c.B);
        s->xb = xb_saved;
        s->Vb = Vb_saved;
        s->nb = nb_saved;
        free(vxb);
        free(vVb);
        free(c.r0); free(c.ph);
        return -2;
    }

    compute_densities(&c);
    compute_factor(&c);
    if (p->enable_divergence_solver) divergence_solve(&c, h, err_buf);
    else { s->iterations_v = 0; s->avg_density_err_v = 0.0; }

    /* clearAccelerations (TimeStep.cpp:35-50): every particle has mass != 0 */
    for (long i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) s->a[3 * i + d] = (real)p->gravity[d];

    /* computeNonPressureForces (Simulation.cpp:495-509): viscosity, then XSPH */
    s->visco_iterations = 0;
    s->visco_error = 0.0;
    if (p->viscosity_method == 6) rc = viscosity_weiler(&c, h);
    if (p->xsph_fluid != 0.0 || p->xsph_boundary != 0.0 || (c.r0 && (s->phase_xsph || s->phase_xsph_boundary)))
        xsph(&c, h);

    const double hnew = update_time_step(&c, h);

    /* v += h * a with the old step size (TimeStepDFSPH.cpp:192-208) */
    for (size_t k = 0; k < 3 * (size_t)n; k++) s->v[k] = (real)((double)s->v[k] + h * (double)s->a[k]);

    pressure_solve(&c, hnew, err_buf);

    /* x += h * v with the old step size (TimeStepDFSPH.cpp:220-237) */
    for (size_t k = 0; k < 3 * (size_t)n; k++) s->x[k] = (real)((double)s->x[k] + h * (double)s->v[k]);

    s->dt_old = h;
    s->dt = hnew;
    s->time += h;                             /* :248 */
    free(err_buf);
    lists_free(&c.F);
    lists_free(&c.B);
    s->xb = xb_saved;
    s->Vb = Vb_saved;
    s->nb = nb_saved;
    free(vxb);
    free(vVb);
    free(c.r0);
    free(c.ph);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Weiler operator entry points for the CG pin                               */
/* ------------------------------------------------------------------------ */
static int ctx_for_state(ctx_t *c, const orc_state *s, const orc_params *p)
{
    memset(c, 0, sizeof(*c));
    c->s = (orc_state *)s;
    c->p = p;
    c->K = kern_make(4.0 * p->radius);
    const double diam = 2.0 * p->radius;
    c->V = 0.8 * diam * diam * diam;
    c->rho0 = p->density0;
    c->mass = c->V * c->rho0;
    c->eps = 1.0e-5;
    if (lists_build(&c->F, s->n, s->x, s->n, s->x, c->K.h, 1, p->fp32_predicate) != 0) return -1;
    if (lists_build(&c->B, s->n, s->x, s->nb, s->xb, c->K.h, 0, p->fp32_predicate) != 0) return -1;
    return 0;
}

int orc_weiler_system(const orc_state *s, const orc_params *p, double dt, real *b, real *g, real *diag9)
{
    ctx_t c;
    if (ctx_for_state(&c, s, p) != 0) return -1;
    visc_t w = visc_make(&c, dt, -1, 0, (long)s->n);
    visc_diag_inverse(&w, diag9, NULL);
    visc_rhs(&w, b, g);
    lists_free(&c.F);
    lists_free(&c.B);
    return 0;
}

int orc_weiler_matvec(const orc_state *s, const orc_params *p, double dt, const real *vec, real *result)
{
    ctx_t c;
    if (ctx_for_state(&c, s, p) != 0) return -1;
    visc_t w = visc_make(&c, dt, -1, 0, (long)s->n);
    visc_matvec(&w, vec, result);
    lists_free(&c.F);
    lists_free(&c.B);
    return 0;
}

int orc_weiler_solve(const orc_state *s, const orc_params *p, double dt, real *x_out, unsigned *iters, double *err)
{
    ctx_t c;
    if (ctx_for_state(&c, s, p) != 0) return -1;
    visc_t w = visc_make(&c, dt, -1, 0, (long)s->n);
    const size_t N = 3 * (size_t)s->n;
    real *b = (real *)malloc(N * sizeof(real));
    real *inv9 = (real *)malloc(3 * N * sizeof(real));
    int rc = -2;
    if (b && inv9) {
        visc_diag_inverse(&w, NULL, inv9);
        visc_rhs(&w, b, x_out);
        rc = visc_cg(&w, b, x_out, inv9, p->visco_max_iter, p->visco_max_error, iters, err);
    }
    free(b);
    free(inv9);
    lists_free(&c.F);
    lists_free(&c.B);
    return rc;
}
