// Construction of Bender2019 volume maps on the device (FP64), as SimulatorBase::initVolumeMap
// builds them (SimulatorBase.cpp:2512-2660) with the Discregrid library:
//   field 0: sign (d - thickness) at every node, d the distance to the body's triangle mesh,
//            signed by the angle-weighted pseudo-normal of the closest feature (positive
//            outside), sign = -1 for an inverted map (a container);
//   field 1: 0 where field 0 > 2 h, else 0.8 x the tensor Gauss-Legendre integral over
//            [-h, h]^3 (order p: p / 2 + 1 points per axis, GaussQuadrature.cpp:5930-5962) of
//            gamma(phi(x + y)) for |y| <= h, with gamma = 1 for phi <= 0, W(phi) / W(0) for
//            phi < h, 0 beyond, phi interpolated from field 0 (0 outside the grid).
// The grid covers the mesh's bounding box grown by 8 h + thickness.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sph_ctx.h"
#include "vmap.cuh"

namespace sphgb {

namespace {

__device__ __forceinline__ void sub3(const double *a, const double *b, double *r)
{
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
__device__ __forceinline__ double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Closest point q of triangle (a, b, c) to p, found by the Voronoi region of p (vertex, edge or
// face); feature: 0..2 vertex a, b, c; 3 edge ab, 4 edge bc, 5 edge ca; 6 the face.
__device__ void closest_on_triangle(const double *p, const double *a, const double *b, const double *c, double *q,
                                    int &feature)
{
    double ab[3], ac[3], ap[3], bp[3], cp[3];
    sub3(b, a, ab);
    sub3(c, a, ac);
    sub3(p, a, ap);
    const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) {
        q[0] = a[0]; q[1] = a[1]; q[2] = a[2];
        feature = 0;
        return;
    }
    sub3(p, b, bp);
    const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) {
        q[0] = b[0]; q[1] = b[1]; q[2] = b[2];
        feature = 1;
        return;
    }
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        const double v = d1 / (d1 - d3);
        for (int d = 0; d < 3; d++) q[d] = a[d] + v * ab[d];
        feature = 3;
        return;
    }
    sub3(p, c, cp);
    const double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) {
        q[0] = c[0]; q[1] = c[1]; q[2] = c[2];
        feature = 2;
        return;
    }
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        const double w = d2 / (d2 - d6);
        for (int d = 0; d < 3; d++) q[d] = a[d] + w * ac[d];
        feature = 5;
        return;
    }
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        for (int d = 0; d < 3; d++) q[d] = b[d] + w * (c[d] - b[d]);
        feature = 4;
        return;
    }
    const double denom = 1.0 / (va + vb + vc);
    const double v = vb * denom, w = vc * denom;
    for (int d = 0; d < 3; d++) q[d] = a[d] + ab[d] * v + ac[d] * w;
    feature = 6;
}

struct GridGeom {
    double dmin[3], dmax[3], cs[3];
    uint32_t res[3];
};

__device__ __forceinline__ void node_position(const VMapLayout &L, const GridGeom &G, uint64_t node, double p[3])
{
    double g[3];
    L.node_coords(node, g);
    for (int d = 0; d < 3; d++) p[d] = G.dmin[d] + g[d] * G.cs[d];
}

// field f (node values) at x; false outside the grid
__device__ bool interp_nodes(const VMapLayout &L, const GridGeom &G, const double *f, const double x[3], double &val)
{
    uint32_t c[3];
    double xi[3];
    if (!vmap_locate<double>(G.dmin, G.dmax, G.cs, G.res, x, c, xi)) return false;
    uint64_t nd[32];
    L.cell_nodes(c[0], c[1], c[2], nd);
    double s = 0.0;
    vmap_shape<double>(xi, [&](int k, double N, double, double, double) { s += N * f[nd[k]]; });
    val = s;
    return true;
}

// field 0: signed distance to the mesh at every node (brute force over the triangles)
__global__ void k_vmap_sdf(VMapLayout L, GridGeom G, const double *__restrict__ vert, const uint32_t *__restrict__ tri,
                           uint32_t nt, const double *__restrict__ fn, const double *__restrict__ vn,
                           const double *__restrict__ en, double sign, double thickness, double *__restrict__ f0)
{
    const uint64_t node = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= L.nodes()) return;
    double p[3];
    node_position(L, G, node, p);
    double best = 1.0e300, qb[3] = {0, 0, 0};
    uint32_t fb = 0;
    int featb = 6;
    for (uint32_t f = 0; f < nt; f++) {
        const uint32_t *t = tri + 3 * (size_t)f;
        double q[3], r[3];
        int feat;
        closest_on_triangle(p, vert + 3 * (size_t)t[0], vert + 3 * (size_t)t[1], vert + 3 * (size_t)t[2], q, feat);
        sub3(p, q, r);
        const double d2 = dot3(r, r);
        if (d2 < best) {
            best = d2;
            qb[0] = q[0]; qb[1] = q[1]; qb[2] = q[2];
            fb = f;
            featb = feat;
        }
    }
    const double *n;
    if (featb <= 2) n = vn + 3 * (size_t)tri[3 * (size_t)fb + featb];
    else if (featb <= 5) n = en + 9 * (size_t)fb + 3 * (featb - 3);
    else n = fn + 3 * (size_t)fb;
    double r[3];
    sub3(p, qb, r);
    const double d = sqrt(best);
    f0[node] = sign * ((dot3(r, n) >= 0.0 ? d : -d) - thickness);
}

constexpr int kVolThreads = 128;

// field 1: one block per node, the quadrature points dealt to its threads, summed in a fixed order
__global__ void __launch_bounds__(kVolThreads) k_vmap_volume(VMapLayout L, GridGeom G, const double *__restrict__ f0,
                                                             const double *__restrict__ gx, const double *__restrict__ gw,
                                                             uint32_t np, Kernel<double> K, double *__restrict__ f1)
{
    const uint64_t node = blockIdx.x;
    const double h = K.h;
    double p[3], dist_x = 1.0e300;
    node_position(L, G, node, p);
    interp_nodes(L, G, f0, p, dist_x);
    if (dist_x > 2.0 * h) {   // block uniform
        if (threadIdx.x == 0) f1[node] = 0.0;
        return;
    }
    const uint32_t total = np * np * np;
    double acc = 0.0;
    for (uint32_t q = threadIdx.x; q < total; q += kVolThreads) {
        const uint32_t a = q / (np * np), b = (q / np) % np, c = q % np;
        const double y[3] = {h * gx[a], h * gx[b], h * gx[c]};
        double g = 0.0;
        if (!(y[0] * y[0] + y[1] * y[1] + y[2] * y[2] > h * h)) {
            const double x[3] = {p[0] + y[0], p[1] + y[1], p[2] + y[2]};
            double dist = 1.0e300;
            interp_nodes(L, G, f0, x, dist);
            if (dist <= 0.0) g = 1.0;
            else if (dist < h) g = kernel_W(K, dist) / K.w0;
        }
        acc += gw[a] * gw[b] * gw[c] * g;
    }
    __shared__ double part[kVolThreads];
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kVolThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) f1[node] = 0.8 * part[0] * h * h * h;
}

// the 32 (distance, volume) coefficients of every cell, stored together in T
template <class T>
__global__ void k_vmap_expand(VMapLayout L, const double *__restrict__ f0, const double *__restrict__ f1,
                              T *__restrict__ coef)
{
    const uint64_t cell = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= L.cells()) return;
    const uint64_t i = cell % L.nx, t = cell / L.nx, j = t % L.ny, k = t / L.ny;
    uint64_t nd[32];
    L.cell_nodes(i, j, k, nd);
    for (int n = 0; n < 32; n++) {
        coef[cell * 64 + 2 * n] = (T)f0[nd[n]];
        coef[cell * 64 + 2 * n + 1] = (T)f1[nd[n]];
    }
}

}  // namespace

namespace {

// Face normals, angle-weighted vertex pseudo-normals and edge pseudo-normals (the sum of the
// normals of the faces sharing the edge; edge e = (k, k+1) of face f at 9 f + 3 e).
void pseudo_normals(const double *v, uint32_t nv, const uint32_t *t, uint32_t nt, std::vector<double> &fn,
                    std::vector<double> &vn, std::vector<double> &en)
{
    fn.assign(3 * (size_t)nt, 0.0);
    vn.assign(3 * (size_t)nv, 0.0);
    en.assign(9 * (size_t)nt, 0.0);
    auto norm = [](double *a) {
        const double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        if (l > 0.0) { a[0] /= l; a[1] /= l; a[2] /= l; }
    };
    struct Edge { uint32_t a, b, face, k; };
    std::vector<Edge> edges(3 * (size_t)nt);
    for (uint32_t f = 0; f < nt; f++) {
        const double *p[3] = {v + 3 * (size_t)t[3 * (size_t)f], v + 3 * (size_t)t[3 * (size_t)f + 1],
                              v + 3 * (size_t)t[3 * (size_t)f + 2]};
        double e1[3], e2[3], n[3];
        for (int d = 0; d < 3; d++) { e1[d] = p[1][d] - p[0][d]; e2[d] = p[2][d] - p[0][d]; }
        n[0] = e1[1] * e2[2] - e1[2] * e2[1];
        n[1] = e1[2] * e2[0] - e1[0] * e2[2];
        n[2] = e1[0] * e2[1] - e1[1] * e2[0];
        norm(n);
        for (int d = 0; d < 3; d++) fn[3 * (size_t)f + d] = n[d];
        for (int k = 0; k < 3; k++) {
            double u[3], w[3];
            for (int d = 0; d < 3; d++) {
                u[d] = p[(k + 1) % 3][d] - p[k][d];
                w[d] = p[(k + 2) % 3][d] - p[k][d];
            }
            norm(u);
            norm(w);
            const double ang = std::acos(std::max(-1.0, std::min(1.0, u[0] * w[0] + u[1] * w[1] + u[2] * w[2])));
            for (int d = 0; d < 3; d++) vn[3 * (size_t)t[3 * (size_t)f + k] + d] += ang * n[d];
            const uint32_t a = t[3 * (size_t)f + k], b = t[3 * (size_t)f + (k + 1) % 3];
            edges[3 * (size_t)f + k] = Edge{std::min(a, b), std::max(a, b), f, (uint32_t)k};
        }
    }
    std::sort(edges.begin(), edges.end(), [](const Edge &x, const Edge &y) {
        return x.a != y.a ? x.a < y.a : (x.b != y.b ? x.b < y.b : x.face < y.face);
    });
    for (size_t s = 0; s < edges.size();) {
        size_t e = s;
        double sum[3] = {0.0, 0.0, 0.0};
        while (e < edges.size() && edges[e].a == edges[s].a && edges[e].b == edges[s].b) {
            for (int d = 0; d < 3; d++) sum[d] += fn[3 * (size_t)edges[e].face + d];
            e++;
        }
        for (size_t r = s; r < e; r++)
            for (int d = 0; d < 3; d++) en[9 * (size_t)edges[r].face + 3 * edges[r].k + d] = sum[d];
        s = e;
    }
}

// Gauss-Legendre points (ascending) and weights on [-1, 1]: Newton's method on P_n evaluated by
// its three-term recurrence, started at cos(pi (i + 3/4) / (n + 1/2)).
void gauss_legendre(unsigned n, double *x, double *w)
{
    for (unsigned i = 0; i < n; i++) {
        double z = std::cos(M_PI * ((double)i + 0.75) / ((double)n + 0.5)), pp = 1.0;
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
            if (std::fabs(z - z1) < 1e-15) break;
        }
        x[i] = -z;
        w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

template <class P> cudaError_t upload(P **d, const P *h, size_t n, std::vector<void *> &tmp)
{
    cudaError_t e = cudaMalloc(d, std::max<size_t>(n, 1) * sizeof(P));
    if (e != cudaSuccess) return e;
    tmp.push_back(*d);
    return n ? cudaMemcpy(*d, h, n * sizeof(P), cudaMemcpyHostToDevice) : cudaSuccess;
}

}  // namespace

void vmap_domain(const double *vert, uint32_t nv, double support, double thickness, double dmin[3], double dmax[3])
{
    for (int d = 0; d < 3; d++) dmin[d] = dmax[d] = nv ? vert[d] : 0.0;
    for (uint32_t i = 1; i < nv; i++)
        for (int d = 0; d < 3; d++) {
            dmin[d] = std::min(dmin[d], vert[3 * (size_t)i + d]);
            dmax[d] = std::max(dmax[d], vert[3 * (size_t)i + d]);
        }
    for (int d = 0; d < 3; d++) {
        dmax[d] += 8.0 * support + thickness;
        dmin[d] -= 8.0 * support + thickness;
    }
}

cudaError_t vmap_build_device(const double *vert, uint32_t nv, const uint32_t *tri, uint32_t nt, const uint32_t res[3],
                              double support, double thickness, int invert, uint32_t order, double *f0, double *f1,
                              const double dmin[3], const double dmax[3], cudaStream_t s)
{
    const VMapLayout L(res[0], res[1], res[2]);
    GridGeom G;
    for (int d = 0; d < 3; d++) {
        G.dmin[d] = dmin[d];
        G.dmax[d] = dmax[d];
        G.res[d] = res[d];
        G.cs[d] = (dmax[d] - dmin[d]) / (double)res[d];
    }
    std::vector<double> fn, vn, en;
    pseudo_normals(vert, nv, tri, nt, fn, vn, en);
    const unsigned np = order < 1 ? 1u : order / 2 + 1;
    std::vector<double> gx(np), gw(np);
    gauss_legendre(np, gx.data(), gw.data());
    std::vector<void *> tmp;
    double *dv = nullptr, *dfn = nullptr, *dvn = nullptr, *den = nullptr, *dgx = nullptr, *dgw = nullptr;
    uint32_t *dt = nullptr;
    cudaError_t e = upload(&dv, vert, 3 * (size_t)nv, tmp);
    if (e == cudaSuccess) e = upload(&dt, tri, 3 * (size_t)nt, tmp);
    if (e == cudaSuccess) e = upload(&dfn, fn.data(), fn.size(), tmp);
    if (e == cudaSuccess) e = upload(&dvn, vn.data(), vn.size(), tmp);
    if (e == cudaSuccess) e = upload(&den, en.data(), en.size(), tmp);
    if (e == cudaSuccess) e = upload(&dgx, gx.data(), gx.size(), tmp);
    if (e == cudaSuccess) e = upload(&dgw, gw.data(), gw.size(), tmp);
    if (e == cudaSuccess) {
        const uint64_t nodes = L.nodes();
        k_vmap_sdf<<<(unsigned)((nodes + 127) / 128), 128, 0, s>>>(L, G, dv, dt, nt, dfn, dvn, den,
                                                                  invert ? -1.0 : 1.0, thickness, f0);
        Kernel<double> K;
        K.h = support;
        K.invh = 1.0 / support;
        K.invh2 = 1.0 / (support * support);
        K.k = 8.0 / (M_PI * support * support * support);
        K.l = 48.0 / (M_PI * support * support * support);
        K.w0 = K.k;
        K.h2 = support * support;
        k_vmap_volume<<<(unsigned)nodes, kVolThreads, 0, s>>>(L, G, f0, dgx, dgw, np, K, f1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    for (void *p : tmp) cudaFree(p);
    return e;
}

template <class T>
cudaError_t vmap_expand_device(const uint32_t res[3], const double *f0, const double *f1, T *coef, cudaStream_t s)
{
    const VMapLayout L(res[0], res[1], res[2]);
    const uint64_t cells = L.cells();
    k_vmap_expand<T><<<(unsigned)((cells + 127) / 128), 128, 0, s>>>(L, f0, f1, coef);
    return cudaGetLastError();
}
template cudaError_t vmap_expand_device<float>(const uint32_t[3], const double *, const double *, float *, cudaStream_t);
template cudaError_t vmap_expand_device<double>(const uint32_t[3], const double *, const double *, double *, cudaStream_t);

}  // namespace sphgb
