// Bender2019 volume maps on the device: Discregrid's CubicLagrangeDiscreteGrid restated (the
// 32-node cubic serendipity element per cell: 8 vertices and 2 nodes at 1/3 and 2/3 of each edge,
// shared between neighbouring cells), as BoundaryModel_Bender2019 samples it
// (SPlisHSPlasH/TimeStep.cpp:219-340).  Two fields per node: 0 signed distance, 1 volume.
#pragma once

#include "sph_common.cuh"

namespace sphgb {

// Node numbering of a grid of (nx, ny, nz) cells: vertex (i, j, k) at (k (ny+1) + j) (nx+1) + i;
// then the x-edge nodes (two per edge, at 1/3 and 2/3 from the lower vertex) at
// nv + 2 ((k (ny+1) + j) nx + i) + a, the y-edge nodes at nv + ex + 2 ((k ny + j) (nx+1) + i) + a
// and the z-edge nodes at nv + ex + ey + 2 ((k (ny+1) + j) (nx+1) + i) + a.
struct VMapLayout {
    uint64_t nx, ny, nz, nv, ex, ey, ez;
    __host__ __device__ VMapLayout(uint32_t rx, uint32_t ry, uint32_t rz)
        : nx(rx), ny(ry), nz(rz), nv((nx + 1) * (ny + 1) * (nz + 1)), ex(2 * nx * (ny + 1) * (nz + 1)),
          ey(2 * (nx + 1) * ny * (nz + 1)), ez(2 * (nx + 1) * (ny + 1) * nz)
    {
    }
    __host__ __device__ uint64_t nodes() const { return nv + ex + ey + ez; }
    __host__ __device__ uint64_t cells() const { return nx * ny * nz; }
    // grid coordinates (in cells) of a node
    __host__ __device__ void node_coords(uint64_t node, double g[3]) const
    {
        if (node < nv) {
            g[0] = (double)(node % (nx + 1));
            const uint64_t t = node / (nx + 1);
            g[1] = (double)(t % (ny + 1));
            g[2] = (double)(t / (ny + 1));
        } else if ((node -= nv) < ex) {
            const uint64_t a = node % 2, e = node / 2, t = e / nx;
            g[0] = (double)(e % nx) + (double)(a + 1) / 3.0;
            g[1] = (double)(t % (ny + 1));
            g[2] = (double)(t / (ny + 1));
        } else if ((node -= ex) < ey) {
            const uint64_t a = node % 2, e = node / 2, t = e / (nx + 1);
            g[0] = (double)(e % (nx + 1));
            g[1] = (double)(t % ny) + (double)(a + 1) / 3.0;
            g[2] = (double)(t / ny);
        } else {
            node -= ey;
            const uint64_t a = node % 2, e = node / 2, t = e / (nx + 1);
            g[0] = (double)(e % (nx + 1));
            g[1] = (double)(t % (ny + 1));
            g[2] = (double)(t / (ny + 1)) + (double)(a + 1) / 3.0;
        }
    }
    // the 32 nodes of cell (i, j, k) in the order of vmap_shape: corners c = sx + 2 sy + 4 sz;
    // x-edges 8 + 2 (sy + 2 sz) + a; y-edges 16 + 2 (sx + 2 sz) + a; z-edges 24 + 2 (sx + 2 sy) + a
    __host__ __device__ void cell_nodes(uint64_t i, uint64_t j, uint64_t k, uint64_t nd[32]) const
    {
        for (int c = 0; c < 8; c++) {
            const uint64_t sx = c & 1, sy = (c >> 1) & 1, sz = c >> 2;
            nd[c] = ((k + sz) * (ny + 1) + (j + sy)) * (nx + 1) + (i + sx);
        }
        for (int q = 0; q < 4; q++)
            for (int a = 0; a < 2; a++) {
                const uint64_t u = q & 1, v = q >> 1;
                nd[8 + 2 * q + a] = nv + 2 * (((k + v) * (ny + 1) + (j + u)) * nx + i) + a;
                nd[16 + 2 * q + a] = nv + ex + 2 * (((k + v) * ny + j) * (nx + 1) + (i + u)) + a;
                nd[24 + 2 * q + a] = nv + ex + ey + 2 * ((k * (ny + 1) + (j + v)) * (nx + 1) + (i + u)) + a;
            }
    }
};

// Cubic serendipity shape functions on [-1, 1]^3 and their derivatives, handed node by node to
// visit(k, N_k, dN_k/dx, dN_k/dy, dN_k/dz) in the order of cell_nodes:
//   corner (xc, yc, zc) in {-1, 1}^3:  (1 + x xc)(1 + y yc)(1 + z zc)(9 (x^2 + y^2 + z^2) - 19) / 64
//   edge node along axis w at w = e (+-1/3), the others at (uc, vc) in {-1, 1}^2:
//                                     9 (1 - w^2)(1 + 9 w e)(1 + u uc)(1 + v vc) / 64
template <class T, class V> __host__ __device__ __forceinline__ void vmap_shape(const T xi[3], V visit)
{
    const T x = xi[0], y = xi[1], z = xi[2];
    const T f = T(9) * (x * x + y * y + z * z) - T(19);
    const T r64 = T(1) / T(64), n64 = T(9) / T(64);
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const T xc = (c & 1) ? T(1) : T(-1), yc = ((c >> 1) & 1) ? T(1) : T(-1), zc = (c >> 2) ? T(1) : T(-1);
        const T a = T(1) + x * xc, b = T(1) + y * yc, d = T(1) + z * zc;
        visit(c, a * b * d * f * r64, (xc * b * d * f + a * b * d * T(18) * x) * r64,
              (a * yc * d * f + a * b * d * T(18) * y) * r64, (a * b * zc * f + a * b * d * T(18) * z) * r64);
    }
#pragma unroll
    for (int axis = 0; axis < 3; axis++)
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int a = 0; a < 2; a++) {
                const T e = a ? T(1) / T(3) : T(-1) / T(3);
                const T uc = (q & 1) ? T(1) : T(-1), vc = (q >> 1) ? T(1) : T(-1);
                const int o1 = axis == 0 ? 1 : 0, o2 = axis == 2 ? 1 : 2;
                const T w = xi[axis], pu = xi[o1], pv = xi[o2];
                const T s = T(1) - w * w, t = T(1) + T(9) * w * e;
                const T bu = T(1) + pu * uc, bv = T(1) + pv * vc;
                T d[3];
                d[axis] = n64 * bu * bv * (T(-2) * w * t + s * T(9) * e);
                d[o1] = n64 * s * t * uc * bv;
                d[o2] = n64 * s * t * bu * vc;
                visit(8 + 8 * axis + 2 * q + a, n64 * s * t * bu * bv, d[0], d[1], d[2]);
            }
}

// Cell and local coordinates of the body-local point xl (DiscreteGrid::determineShapeFunctions):
// false outside [dmin, dmax]; the last cell takes the upper face.
template <class T>
__host__ __device__ __forceinline__ bool vmap_locate(const T dmin[3], const T dmax[3], const T cs[3], const uint32_t res[3],
                                                     const T xl[3], uint32_t c[3], T xi[3])
{
#pragma unroll
    for (int d = 0; d < 3; d++)
        if (!(xl[d] >= dmin[d] && xl[d] <= dmax[d])) return false;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        uint32_t ci = (uint32_t)((xl[d] - dmin[d]) / cs[d]);
        if (ci >= res[d]) ci = res[d] - 1;
        c[d] = ci;
        const T lo = dmin[d] + (T)ci * cs[d], hi = lo + cs[d];
        xi[d] = (T(2) * xl[d] - (lo + hi)) / cs[d];
    }
    return true;
}

// Volume map of one body as the per-step kernel reads it: the 32 (distance, volume)
// coefficients of each cell stored together.
template <class T> struct VMapDev {
    T dmin[3], dmax[3], cs[3];   // body-local grid box and cell size
    T R[9], t[3];                // rotation (row-major) and position: x_local = R^T (x - t)
    T v[3], w[3];                // linear and angular velocity of the body: point p moves at w x (p - t) + v
    T max_dist;                  // largest distance of a mesh vertex from the vertices' mean (CFL bound)
    uint32_t res[3];
    uint32_t pad;
    const T *coef;               // [cells][32][2]
};

// signed distance, its gradient and the volume at body-local xl; false outside the grid
template <class T>
__device__ __forceinline__ bool vmap_sample(const VMapDev<T> &m, const T xl[3], T &sdf, T g[3], T &vol)
{
    uint32_t c[3];
    T xi[3];
    if (!vmap_locate<T>(m.dmin, m.dmax, m.cs, m.res, xl, c, xi)) return false;
    const T *cf = m.coef + ((((uint64_t)c[2] * m.res[1] + c[1]) * m.res[0] + c[0]) * 64u);
    T s = T(0), v = T(0), gx = T(0), gy = T(0), gz = T(0);
    vmap_shape<T>(xi, [&](int k, T N, T dx, T dy, T dz) {
        const T fk = cf[2 * k], vk = cf[2 * k + 1];
        s += N * fk;
        v += N * vk;
        gx += dx * fk;
        gy += dy * fk;
        gz += dz * fk;
    });
    sdf = s;
    vol = v;
    g[0] = gx * (T(2) / m.cs[0]);
    g[1] = gy * (T(2) / m.cs[1]);
    g[2] = gz * (T(2) / m.cs[2]);
    return true;
}

}  // namespace sphgb
