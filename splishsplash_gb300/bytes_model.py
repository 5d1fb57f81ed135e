"""Algorithmic HBM bytes of the step's kernels (FP32 layout).

Counted per fluid particle: every per-particle array the kernel must read or
write once, plus its neighbour-list entries (4-byte indices, written once by the
list build and read once by every later neighbour pass).  Re-reads of
neighbour data (x_j, v_j, kappa_j, a_j, boundary x_b) are not counted: after the
per-step cell sort those are cache hits, and any DRAM traffic they cause is
waste that the ncu dram counters expose.

Layout: position/velocity/acceleration/vDiff and CG vectors are float4 (16 B);
scalars (density, alpha, advected density, kappa, kappa_v) 4 B; neighbour counts
2 x 4 B; cell id 4 B.  nf, nb = mean fluid / boundary neighbour counts.
"""
from __future__ import annotations

V4 = 16
S = 4
IDX = 4


def per_particle(kernel: str, nf: float, nb: float, visc_boundary: bool = False) -> float:
    """Algorithmic bytes per fluid particle for one launch of `kernel`."""
    lists = IDX * (nf + nb)
    lists_f = IDX * nf + (IDX * nb if visc_boundary else 0)
    counts = 2 * IDX
    table = {
        # x_i, v_i, cell id; writes lists + counts, density, alpha, advected density; kappa_v r/w
        "build_lists_density_alpha": 2 * V4 + IDX + lists + counts + 3 * S + 2 * S,
        # x_i, kappa_i, counts, lists; writes a_i
        "pressure_accel": V4 + S + counts + lists + V4,
        # x_i, a_i, counts, lists, alpha_i, advected density_i, kappa_i r/w
        "jacobi_update": 2 * V4 + counts + lists + 2 * S + 2 * S,
        # pressure_accel + v_i r/w
        "solver_finalize": V4 + S + counts + lists + V4 + 2 * V4,
        # x_i, v_i, density_i, counts, lists (fluid); writes a_i; kappa_v r/w; with viscosity
        # also reads vDiff_i and writes the CG warm start
        "xsph_gravity": 2 * V4 + S + counts + IDX * nf + V4 + 2 * S + 2 * V4,
        # x_i, warm start g_i (+ weight), v_i, density_i, counts, lists; writes 2 symmetric
        # inverse rows, r, p
        "visc_setup": 3 * V4 + S + counts + lists_f + 2 * V4 + 2 * V4,
        # the two passes above fused (one fluid phase with viscosity): x_i, v_i, vDiff_i (rho_i
        # in w), density_i, counts, one walk of the lists; writes a_i, kappa_v r/w, the warm
        # start, 2 symmetric inverse rows, r, p
        "xsph_visc_setup": 3 * V4 + S + counts + lists_f + V4 + 2 * S + V4 + 2 * V4 + 2 * V4,
        # x_i, p_i, density_i, counts, lists; writes t_i
        "cg_matvec": 2 * V4 + S + counts + lists_f + V4,
        # p, t, x, r, 2 inverse rows; writes x, r, z
        "cg_update": 6 * V4 + 3 * V4,
        # z, p; writes p
        "cg_p": 3 * V4,
        # a, v, cg x; writes v, a, vdiff
        "kick_cfl": 3 * V4 + 3 * V4,
        # x_i, v_i, density_i, kappa_i r/w, counts, lists; writes advected density
        "press_init": 2 * V4 + S + 2 * S + counts + lists + S,
        # x hi/lo r/w, v, kappa r/w
        "integrate": 4 * V4 + V4 + 2 * S,
        # x_i; writes key, value, cell id
        "keys": V4 + 3 * IDX,
        # 3 passes x (read key+value, write key+value) + histograms (small)
        "radix_sort": 3 * 4 * IDX,
        # state gather: x, xlo, v, vdiff, kappa, kappa_v, id, cell id read + write
        "gather": 2 * (4 * V4 + 4 * S),
        "cell_ranges": IDX * 3,
    }
    return float(table.get(kernel, 0.0))


def per_launch(kernel: str, n: int, nf: float, nb: float, visc_boundary: bool = False) -> float:
    return per_particle(kernel, nf, nb, visc_boundary) * n
