/*
 * Bender2019 volume maps for the CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, without the Discregrid library (an external project absent from the reference
 * tree, so parity with the reference is unpinned here):
 *   - Discregrid::CubicLagrangeDiscreteGrid: a regular grid whose cells are interpolated with
 *     the 32-node cubic serendipity element (the 8 vertices and 2 nodes at 1/3 and 2/3 of each
 *     of the 12 edges, shared between neighbouring cells), as BoundaryModel_Bender2019 samples
 *     it (TimeStep.cpp:219-340);
 *   - Discregrid::TriangleMeshDistance: the distance to a triangle mesh, signed by the
 *     angle-weighted pseudo-normal of the closest feature (Baerentzen and Aanaes, "Signed
 *     distance computation using the angle weighted pseudonormal", 2005);
 *   - the volume function of SimulatorBase::initVolumeMap (SimulatorBase.cpp:2512-2660),
 *     integrated with the tensor Gauss-Legendre rule of GaussQuadrature::integrate
 *     (GaussQuadrature.cpp:5930-5962; order p uses p / 2 + 1 points per axis).
 */
#include "sph_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---- grid layout --------------------------------------------------------- */
typedef struct {
    size_t nx, ny, nz;
    size_t nv, ex, ey, ez;   /* vertices, x-, y- and z-edge nodes (two per edge) */
} layout;

static layout layout_of(const unsigned res[3])
{
    layout L;
    L.nx = res[0];
    L.ny = res[1];
    L.nz = res[2];
    L.nv = (L.nx + 1) * (L.ny + 1) * (L.nz + 1);
    L.ex = 2 * L.nx * (L.ny + 1) * (L.nz + 1);
    L.ey = 2 * (L.nx + 1) * L.ny * (L.nz + 1);
    L.ez = 2 * (L.nx + 1) * (L.ny + 1) * L.nz;
    return L;
}

size_t orc_vmap_nodes(const unsigned res[3])
{
    const layout L = layout_of(res);
    return L.nv + L.ex + L.ey + L.ez;
}

static void cell_size(const orc_vmap *m, double cs[3])
{
    for (int d = 0; d < 3; d++) cs[d] = (m->dmax[d] - m->dmin[d]) / (double)m->res[d];
}

/* Node numbering: vertex (i, j, k) at ((k (ny+1) + j) (nx+1) + i); x-edge node a (at 1/3, 2/3)
 * of the edge from vertex (i, j, k) at nv + 2 ((k (ny+1) + j) nx + i) + a; y-edge node at
 * nv + ex + 2 ((k ny + j) (nx+1) + i) + a; z-edge node at nv + ex + ey + 2 ((k (ny+1) + j) (nx+1)
 * + i) + a. */
void orc_vmap_node_position(const orc_vmap *m, size_t node, double p[3])
{
    const layout L = layout_of(m->res);
    double cs[3], g[3];
    cell_size(m, cs);
    if (node < L.nv) {
        const size_t i = node % (L.nx + 1), t = node / (L.nx + 1);
        g[0] = (double)i;
        g[1] = (double)(t % (L.ny + 1));
        g[2] = (double)(t / (L.ny + 1));
    } else if ((node -= L.nv) < L.ex) {
        const size_t a = node % 2, e = node / 2, i = e % L.nx, t = e / L.nx;
        g[0] = (double)i + (double)(a + 1) / 3.0;
        g[1] = (double)(t % (L.ny + 1));
        g[2] = (double)(t / (L.ny + 1));
    } else if ((node -= L.ex) < L.ey) {
        const size_t a = node % 2, e = node / 2, i = e % (L.nx + 1), t = e / (L.nx + 1);
        g[0] = (double)i;
        g[1] = (double)(t % L.ny) + (double)(a + 1) / 3.0;
        g[2] = (double)(t / L.ny);
    } else {
        node -= L.ey;
        const size_t a = node % 2, e = node / 2, i = e % (L.nx + 1), t = e / (L.nx + 1);
        g[0] = (double)i;
        g[1] = (double)(t % (L.ny + 1));
        g[2] = (double)(t / (L.ny + 1)) + (double)(a + 1) / 3.0;
    }
    for (int d = 0; d < 3; d++) p[d] = m->dmin[d] + g[d] * cs[d];
}

/* The 32 nodes of cell (i, j, k) in the order of shape(): corners c = sx + 2 sy + 4 sz; x-edges
 * 8 + 2 (sy + 2 sz) + a; y-edges 16 + 2 (sx + 2 sz) + a; z-edges 24 + 2 (sx + 2 sy) + a. */
static void cell_nodes(const layout *L, size_t i, size_t j, size_t k, size_t nd[32])
{
    for (int c = 0; c < 8; c++) {
        const size_t sx = c & 1, sy = (c >> 1) & 1, sz = c >> 2;
        nd[c] = ((k + sz) * (L->ny + 1) + (j + sy)) * (L->nx + 1) + (i + sx);
    }
    for (int q = 0; q < 4; q++)
        for (int a = 0; a < 2; a++) {
            const size_t u = q & 1, v = q >> 1;
            nd[8 + 2 * q + a] = L->nv + 2 * (((k + v) * (L->ny + 1) + (j + u)) * L->nx + i) + a;
            nd[16 + 2 * q + a] = L->nv + L->ex + 2 * (((k + v) * L->ny + j) * (L->nx + 1) + (i + u)) + a;
            nd[24 + 2 * q + a] = L->nv + L->ex + L->ey + 2 * ((k * (L->ny + 1) + (j + v)) * (L->nx + 1) + (i + u)) + a;
        }
}

/* Cubic serendipity shape functions on [-1, 1]^3 and their derivatives:
 *   corner (xc, yc, zc) in {-1, 1}^3:  (1 + x xc)(1 + y yc)(1 + z zc)(9 (x^2 + y^2 + z^2) - 19) / 64
 *   x-edge node (e, yc, zc), e = -1/3 or 1/3:  9 (1 - x^2)(1 + 9 x e)(1 + y yc)(1 + z zc) / 64
 *   and likewise for the y- and z-edge nodes. */
static void shape(const double xi[3], double N[32], double dN[32][3])
{
    const double x = xi[0], y = xi[1], z = xi[2];
    const double f = 9.0 * (x * x + y * y + z * z) - 19.0;
    for (int c = 0; c < 8; c++) {
        const double xc = (c & 1) ? 1.0 : -1.0, yc = ((c >> 1) & 1) ? 1.0 : -1.0, zc = (c >> 2) ? 1.0 : -1.0;
        const double a = 1.0 + x * xc, b = 1.0 + y * yc, d = 1.0 + z * zc;
        N[c] = a * b * d * f / 64.0;
        dN[c][0] = (xc * b * d * f + a * b * d * 18.0 * x) / 64.0;
        dN[c][1] = (a * yc * d * f + a * b * d * 18.0 * y) / 64.0;
        dN[c][2] = (a * b * zc * f + a * b * d * 18.0 * z) / 64.0;
    }
    /* edge nodes: w = the coordinate along the edge, p and q the other two */
    for (int axis = 0; axis < 3; axis++)
        for (int q = 0; q < 4; q++)
            for (int a = 0; a < 2; a++) {
                const double e = a ? 1.0 / 3.0 : -1.0 / 3.0;
                const double uc = (q & 1) ? 1.0 : -1.0, vc = (q >> 1) ? 1.0 : -1.0;
                /* the edge's axis and the two others in increasing order */
                const int o1 = axis == 0 ? 1 : 0, o2 = axis == 2 ? 1 : 2;
                const double w = xi[axis], pu = xi[o1], pv = xi[o2];
                const double s = 1.0 - w * w, t = 1.0 + 9.0 * w * e;
                const double bu = 1.0 + pu * uc, bv = 1.0 + pv * vc;
                const int k = 8 + 8 * axis + 2 * q + a;
                N[k] = 9.0 / 64.0 * s * t * bu * bv;
                dN[k][axis] = 9.0 / 64.0 * bu * bv * (-2.0 * w * t + s * 9.0 * e);
                dN[k][o1] = 9.0 / 64.0 * s * t * uc * bv;
                dN[k][o2] = 9.0 / 64.0 * s * t * bu * vc;
            }
}

int orc_vmap_interpolate(const orc_vmap *m, int field, const double xl[3], double *value, double grad[3])
{
    double cs[3], xi[3];
    size_t c[3];
    for (int d = 0; d < 3; d++)
        if (!(xl[d] >= m->dmin[d] && xl[d] <= m->dmax[d])) return 0;
    cell_size(m, cs);
    for (int d = 0; d < 3; d++) {
        size_t ci = (size_t)((xl[d] - m->dmin[d]) / cs[d]);
        if (ci >= m->res[d]) ci = m->res[d] - 1;
        c[d] = ci;
        const double lo = m->dmin[d] + (double)ci * cs[d], hi = lo + cs[d];
        xi[d] = (2.0 * xl[d] - (lo + hi)) / cs[d];
    }
    const layout L = layout_of(m->res);
    size_t nd[32];
    double N[32], dN[32][3];
    cell_nodes(&L, c[0], c[1], c[2], nd);
    shape(xi, N, dN);
    const double *f = m->field[field];
    double v = 0.0, g[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 32; k++) {
        const double fk = f[nd[k]];
        v += N[k] * fk;
        for (int d = 0; d < 3; d++) g[d] += dN[k][d] * fk;
    }
    *value = v;
    if (grad)
        for (int d = 0; d < 3; d++) grad[d] = g[d] * (2.0 / cs[d]);
    return 1;
}

/* ---- signed distance to a triangle mesh ----------------------------------- */
static inline void sub3(const double *a, const double *b, double *r)
{
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
static inline double dot3v(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void cross3(const double *a, const double *b, double *r)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
static inline void normalize3(double *a)
{
    const double l = sqrt(dot3v(a, a));
    if (l > 0.0) {
        a[0] /= l;
        a[1] /= l;
        a[2] /= l;
    }
}

/* Closest point q of triangle (a, b, c) to p by the Voronoi regions of its features; feature:
 * 0..2 vertex a, b, c; 3 edge ab, 4 edge bc, 5 edge ca; 6 the face. */
static void closest_on_triangle(const double *p, const double *a, const double *b, const double *c, double *q,
                                int *feature)
{
    double ab[3], ac[3], ap[3], bp[3], cp[3];
    sub3(b, a, ab);
    sub3(c, a, ac);
    sub3(p, a, ap);
    const double d1 = dot3v(ab, ap), d2 = dot3v(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) { memcpy(q, a, 3 * sizeof(double)); *feature = 0; return; }
    sub3(p, b, bp);
    const double d3 = dot3v(ab, bp), d4 = dot3v(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) { memcpy(q, b, 3 * sizeof(double)); *feature = 1; return; }
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        const double v = d1 / (d1 - d3);
        for (int d = 0; d < 3; d++) q[d] = a[d] + v * ab[d];
        *feature = 3;
        return;
    }
    sub3(p, c, cp);
    const double d5 = dot3v(ab, cp), d6 = dot3v(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) { memcpy(q, c, 3 * sizeof(double)); *feature = 2; return; }
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        const double w = d2 / (d2 - d6);
        for (int d = 0; d < 3; d++) q[d] = a[d] + w * ac[d];
        *feature = 5;
        return;
    }
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        for (int d = 0; d < 3; d++) q[d] = b[d] + w * (c[d] - b[d]);
        *feature = 4;
        return;
    }
    const double denom = 1.0 / (va + vb + vc);
    const double v = vb * denom, w = vc * denom;
    for (int d = 0; d < 3; d++) q[d] = a[d] + ab[d] * v + ac[d] * w;
    *feature = 6;
}

typedef struct {
    unsigned a, b, face;
} edge_rec;

static int cmp_edge(const void *x, const void *y)
{
    const edge_rec *e = (const edge_rec *)x, *f = (const edge_rec *)y;
    if (e->a != f->a) return e->a < f->a ? -1 : 1;
    if (e->b != f->b) return e->b < f->b ? -1 : 1;
    return (e->face > f->face) - (e->face < f->face);
}

typedef struct {
    const double *vert;
    const unsigned *tri;
    unsigned nt;
    double *fn;          /* 3 nt face normals */
    double *vn;          /* 3 nv angle-weighted vertex pseudo-normals */
    double *en;          /* 9 nt: the pseudo-normal of edge e (ab, bc, ca) of face f at 9 f + 3 e */
} mesh_normals;

static int normals_build(mesh_normals *M, const double *vert, unsigned nv, const unsigned *tri, unsigned nt)
{
    M->vert = vert;
    M->tri = tri;
    M->nt = nt;
    M->fn = (double *)calloc(3 * (size_t)nt + 1, sizeof(double));
    M->vn = (double *)calloc(3 * (size_t)nv + 1, sizeof(double));
    M->en = (double *)calloc(9 * (size_t)nt + 1, sizeof(double));
    edge_rec *E = (edge_rec *)malloc((3 * (size_t)nt + 1) * sizeof(edge_rec));
    if (!M->fn || !M->vn || !M->en || !E) { free(E); return -2; }
    for (unsigned f = 0; f < nt; f++) {
        const double *p[3] = {vert + 3 * (size_t)tri[3 * f], vert + 3 * (size_t)tri[3 * f + 1], vert + 3 * (size_t)tri[3 * f + 2]};
        double e1[3], e2[3], n[3];
        sub3(p[1], p[0], e1);
        sub3(p[2], p[0], e2);
        cross3(e1, e2, n);
        normalize3(n);
        memcpy(M->fn + 3 * (size_t)f, n, sizeof(n));
        for (int k = 0; k < 3; k++) {
            /* the angle of the face at its vertex k */
            double u[3], w[3];
            sub3(p[(k + 1) % 3], p[k], u);
            sub3(p[(k + 2) % 3], p[k], w);
            normalize3(u);
            normalize3(w);
            double cosang = dot3v(u, w);
            if (cosang > 1.0) cosang = 1.0;
            if (cosang < -1.0) cosang = -1.0;
            const double ang = acos(cosang);
            double *vn = M->vn + 3 * (size_t)tri[3 * f + k];
            for (int d = 0; d < 3; d++) vn[d] += ang * n[d];
            const unsigned va = tri[3 * f + k], vb = tri[3 * f + (k + 1) % 3];
            E[3 * (size_t)f + k].a = va < vb ? va : vb;
            E[3 * (size_t)f + k].b = va < vb ? vb : va;
            E[3 * (size_t)f + k].face = f;
        }
    }
    /* edge pseudo-normal: the sum of the normals of the faces sharing the edge */
    qsort(E, 3 * (size_t)nt, sizeof(edge_rec), cmp_edge);
    for (size_t s = 0; s < 3 * (size_t)nt;) {
        size_t e = s;
        double sum[3] = {0.0, 0.0, 0.0};
        while (e < 3 * (size_t)nt && E[e].a == E[s].a && E[e].b == E[s].b) {
            for (int d = 0; d < 3; d++) sum[d] += M->fn[3 * (size_t)E[e].face + d];
            e++;
        }
        for (size_t r = s; r < e; r++) {
            const unsigned f = E[r].face;
            for (int k = 0; k < 3; k++) {
                const unsigned va = tri[3 * f + k], vb = tri[3 * f + (k + 1) % 3];
                if ((va < vb ? va : vb) == E[s].a && (va < vb ? vb : va) == E[s].b)
                    memcpy(M->en + 9 * (size_t)f + 3 * k, sum, sizeof(sum));
            }
        }
        s = e;
    }
    free(E);
    return 0;
}

static void normals_free(mesh_normals *M)
{
    free(M->fn);
    free(M->vn);
    free(M->en);
}

/* signed distance from p to the mesh: positive outside (pseudo-normal of the closest feature) */
static double mesh_signed_distance(const mesh_normals *M, const double *p)
{
    double best = DBL_MAX, q_best[3] = {0, 0, 0};
    unsigned f_best = 0;
    int feat_best = 6;
    for (unsigned f = 0; f < M->nt; f++) {
        const unsigned *t = M->tri + 3 * (size_t)f;
        double q[3], r[3];
        int feat;
        closest_on_triangle(p, M->vert + 3 * (size_t)t[0], M->vert + 3 * (size_t)t[1], M->vert + 3 * (size_t)t[2], q,
                            &feat);
        sub3(p, q, r);
        const double d2 = dot3v(r, r);
        if (d2 < best) {
            best = d2;
            memcpy(q_best, q, sizeof(q));
            f_best = f;
            feat_best = feat;
        }
    }
    const double *n;
    if (feat_best <= 2) n = M->vn + 3 * (size_t)M->tri[3 * (size_t)f_best + feat_best];
    else if (feat_best <= 5) n = M->en + 9 * (size_t)f_best + 3 * (feat_best - 3);
    else n = M->fn + 3 * (size_t)f_best;
    double r[3];
    sub3(p, q_best, r);
    const double d = sqrt(best);
    return dot3v(r, n) >= 0.0 ? d : -d;
}

/* ---- volume map construction ----------------------------------------------- */
void orc_vmap_domain(const double *vert, unsigned nv, double support, double thickness, double dmin[3],
                     double dmax[3])
{
    for (int d = 0; d < 3; d++) dmin[d] = dmax[d] = nv ? vert[d] : 0.0;
    for (unsigned i = 1; i < nv; i++)
        for (int d = 0; d < 3; d++) {
            const double v = vert[3 * (size_t)i + d];
            if (v < dmin[d]) dmin[d] = v;
            if (v > dmax[d]) dmax[d] = v;
        }
    for (int d = 0; d < 3; d++) {
        dmax[d] += 8.0 * support + thickness;
        dmin[d] -= 8.0 * support + thickness;
    }
}

/* Gauss-Legendre points and weights on [-1, 1]: Newton's method on P_n from the three-term
 * recurrence, started at cos(pi (i + 3/4) / (n + 1/2)). */
static void gauss_legendre(unsigned n, double *x, double *w)
{
    for (unsigned i = 0; i < n; i++) {
        double z = cos(M_PI * ((double)i + 0.75) / ((double)n + 0.5)), pp = 1.0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1.0, p2 = 0.0;
            for (unsigned j = 1; j <= n; j++) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-15) break;
        }
        x[i] = -z;   /* ascending */
        w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

int orc_vmap_build(orc_vmap *m, const double *vert, unsigned nv, const unsigned *tri, unsigned nt,
                   double support, double thickness, int invert, unsigned order)
{
    if (!m || !vert || !tri || nt == 0 || !m->field[0] || !m->field[1]) return -1;
    orc_vmap_domain(vert, nv, support, thickness, m->dmin, m->dmax);
    mesh_normals M;
    if (normals_build(&M, vert, nv, tri, nt) != 0) { normals_free(&M); return -2; }
    const size_t N = orc_vmap_nodes(m->res);
    const double sign = invert ? -1.0 : 1.0;
#pragma omp parallel for schedule(dynamic, 64)
    for (long k = 0; k < (long)N; k++) {
        double p[3];
        orc_vmap_node_position(m, (size_t)k, p);
        m->field[0][k] = sign * (mesh_signed_distance(&M, p) - thickness);
    }
    normals_free(&M);

    const unsigned np = order < 1 ? 1u : order / 2 + 1;
    double gx[64], gw[64];
    if (np > 64) return -1;
    gauss_legendre(np, gx, gw);
    const double h = support, w0 = orc_kernel_W(0.0, support);
#pragma omp parallel for schedule(dynamic, 16)
    for (long k = 0; k < (long)N; k++) {
        double p[3], dist_x = DBL_MAX;
        orc_vmap_node_position(m, (size_t)k, p);
        orc_vmap_interpolate(m, 0, p, &dist_x, NULL);
        double res = 0.0;
        if (!(dist_x > 2.0 * h)) {
            for (unsigned a = 0; a < np; a++)
                for (unsigned b = 0; b < np; b++)
                    for (unsigned c = 0; c < np; c++) {
                        const double y[3] = {h * gx[a], h * gx[b], h * gx[c]};
                        double g = 0.0;
                        if (!(y[0] * y[0] + y[1] * y[1] + y[2] * y[2] > h * h)) {
                            const double q[3] = {p[0] + y[0], p[1] + y[1], p[2] + y[2]};
                            double dist = DBL_MAX;
                            orc_vmap_interpolate(m, 0, q, &dist, NULL);
                            if (dist <= 0.0) g = 1.0;
                            else if (dist < h) g = orc_kernel_W(dist, support) / w0;
                        }
                        res += gw[a] * gw[b] * gw[c] * g;
                    }
            res *= h * h * h;
        }
        m->field[1][k] = 0.8 * res;
    }
    return 0;
}
