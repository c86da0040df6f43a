"""CPU check of the algebra behind the box-specialised FP64 kernels
(kernels.cu: k_pg_residual_box, k_forces_box).

Box shape functions are products of 1D factors, so the kernels replace Gauss-point
sums by 1D passes:
* the SUPG element residual (pg_shape_fn + element_residual, Advection_diffusion.c:
  448-727): values at the 2x2x2 Gauss points by three 1D interpolation passes,
  gradients as face differences interpolated in the other two axes, and the test
  sums as the transposed passes;
* the element force (get_elt_f, Element_calculations.c:989-1075): the assembled
  consistent mass matrix as a tensor product of 1D weights.
Here both are restated in numpy, in the kernels' index order (q = x + 2y + 4z), and
compared with the direct Gauss-point sums over the reference's shape functions on
random data.  The GPU kernels themselves are checked against the oracle and the
reference by the -m gpu parity tests."""
import numpy as np

BETA = 0.57735026918962576451
P, Q = 0.5 * (1.0 + BETA), 0.5 * (1.0 - BETA)


def loc(a, d):
    """local node / Gauss point a -> 0/1 offset along axis d (level.h cg_loc)"""
    return int([(a & 3) in (1, 2), (a & 3) >= 2, a >= 4][d])


def shape_tables(h):
    N = np.zeros((8, 8))
    gnx = np.zeros((8, 8, 3))
    for k in range(8):
        for a in range(8):
            f = [0.5 * (1 + (1 if loc(a, d) else -1) * (BETA if loc(k, d) else -BETA)) for d in range(3)]
            N[k, a] = np.prod(f)
            for d in range(3):
                gnx[k, a, d] = (1 if loc(a, d) else -1) / h[d] * np.prod([f[e] for e in range(3) if e != d])
    return N, gnx


def pass1d(f, strides):
    f = f.copy()
    for s in strides:
        for q in range(len(f)):
            if not q & s:
                a, b = f[q], f[q + s]
                f[q], f[q + s] = P * a + Q * b, Q * a + P * b
    return f


def q_of(d, lo, hi, side):
    a1 = 1 if d == 0 else 0
    a2 = 1 if d == 2 else 2
    return (side << d) | (lo << a1) | (hi << a2)


def test_supg_residual_sum_factorised():
    rng = np.random.default_rng(11)
    for _ in range(5):
        h = rng.uniform(0.1, 1.0, 3)
        J = np.prod(h) / 8.0
        N, gnx = shape_tables(h)
        tn, dtn, vn = rng.random(8), rng.random(8), rng.normal(0, 30, (8, 3))
        Q0, adiff = rng.random(), rng.random()
        # direct Gauss-point sums, local node order a
        er = np.zeros(8)
        for k in range(8):
            dT, v, t = dtn @ N[k], vn.T @ N[k], gnx[k].T @ tn
            adv = dT - Q0 + v @ t
            for a in range(8):
                pg = N[k, a] + adiff * (v @ gnx[k, a])
                er[a] -= pg * J * adv + J * (gnx[k, a] @ t)
        # sum-factorised, index q = x + 2y + 4z
        qa = [loc(a, 0) + 2 * loc(a, 1) + 4 * loc(a, 2) for a in range(8)]
        T, D, V = np.zeros(8), np.zeros(8), np.zeros((3, 8))
        for a in range(8):
            T[qa[a]], D[qa[a]], V[:, qa[a]] = tn[a], dtn[a], vn[a]
        gt = np.zeros((3, 4))
        for d in range(3):
            for m in range(4):
                gt[d, m] = (T[q_of(d, m & 1, m >> 1, 1)] - T[q_of(d, m & 1, m >> 1, 0)]) / h[d]
            gt[d] = pass1d(gt[d], (1, 2))
        A = pass1d(D, (1, 2, 4))
        vk = np.array([pass1d(V[d], (1, 2, 4)) for d in range(3)])
        sb = np.zeros((3, 4))
        for q in range(8):
            x, y, z = q & 1, (q >> 1) & 1, q >> 2
            g = (gt[0, y + 2 * z], gt[1, x + 2 * z], gt[2, x + 2 * y])
            A[q] = A[q] - Q0 + sum(vk[d, q] * g[d] for d in range(3))
            sb[0, y + 2 * z] += adiff * A[q] * vk[0, q] + g[0]
            sb[1, x + 2 * z] += adiff * A[q] * vk[1, q] + g[1]
            sb[2, x + 2 * y] += adiff * A[q] * vk[2, q] + g[2]
        A = pass1d(A, (1, 2, 4))
        sb = np.array([pass1d(sb[d], (1, 2)) for d in range(3)])
        ef = np.zeros(8)
        for q in range(8):
            x, y, z = q & 1, (q >> 1) & 1, q >> 2
            f = [sb[0, y + 2 * z] * (1 if x else -1), sb[1, x + 2 * z] * (1 if y else -1),
                 sb[2, x + 2 * y] * (1 if z else -1)]
            ef[q] = -J * (A[q] + sum(f[d] / h[d] for d in range(3)))
        assert np.max(np.abs(er - ef[qa])) <= 1e-13 * np.max(np.abs(er))


def test_force_mass_weights():
    rng = np.random.default_rng(12)
    nox, noy, noz = 4, 3, 5
    h = (0.2, 0.3, 0.25)
    J = np.prod(h) / 8.0
    N, _ = shape_tables(h)
    b = rng.random((noy, nox, noz))
    direct = np.zeros_like(b)
    for y in range(noy):
        for x in range(nox):
            for z in range(noz):
                for a in range(8):
                    ex, ey, ez = x - loc(a, 0), y - loc(a, 1), z - loc(a, 2)
                    if not (0 <= ex < nox - 1 and 0 <= ey < noy - 1 and 0 <= ez < noz - 1):
                        continue
                    bb = np.array([b[ey + loc(c, 1), ex + loc(c, 0), ez + loc(c, 2)] for c in range(8)])
                    direct[y, x, z] += J * sum((bb @ N[k]) * N[k, a] for k in range(8))
    c0, c1 = P * P + Q * Q, 2.0 * P * Q

    def w1(i, n, d):
        if d < 0:
            return c1 if i > 0 else 0.0
        if d > 0:
            return c1 if i < n - 1 else 0.0
        return (c0 if i > 0 else 0.0) + (c0 if i < n - 1 else 0.0)

    weights = np.zeros_like(b)
    for y in range(noy):
        for x in range(nox):
            for z in range(noz):
                s = 0.0
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        for dz in (-1, 0, 1):
                            w = w1(y, noy, dy) * w1(x, nox, dx) * w1(z, noz, dz)
                            if w:
                                s += w * b[y + dy, x + dx, z + dz]
                weights[y, x, z] = J * s
    assert np.max(np.abs(direct - weights)) <= 1e-13 * np.max(np.abs(direct))
