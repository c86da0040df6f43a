"""CPU check of the spherical element geometry (citcomcu_gb300/csrc/geometry.cu,
compiled here for the host) against the unchanged reference's own spherical
run (tests/golden/sphere_tdep.npz): the stiffness, 1/diag K, divergence and
gradient assembled in numpy from the geometry tables reproduce the reference's
operator probes on every level, the TWW-weighted projection its
project_vector, the size-weighted interpolation its interp_vector, the face
weights its horizontal averages (thermal_buoyancy) and the radial-force
projection its assemble_forces."""
import math
import os
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LOC = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
FIELDS = [("Mk", (8, 8, 8, 9)), ("g", (24,)), ("gnx", (8, 8, 3)), ("N", (8, 8)), ("gda", (8,)), ("tww", (8,)),
          ("size", (3,)), ("area", ()), ("cr", (8, 8, 3)), ("rinv", (8,)), ("rsin", (8,)), ("wface", (4,)),
          ("gnxc", (8, 3)), ("rinvc", ()), ("thetac", ())]
MGUNIT = (2, 3, 2)
SPHERE = (45.0, 135.0, 0.0, 90.0, 0.55, 1.0)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def dump():
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "geometry_dump")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I/usr/local/cuda/include", "-x", "c++",
                    os.path.join(ROOT, "citcomcu_gb300", "csrc", "geometry.cu"), "-x", "c++",
                    os.path.join(HERE, "geometry_dump.cpp"), "-o", exe], check=True)

    def level(l):
        el = [m * 2 ** l for m in MGUNIT]
        rad = math.pi / 180
        h = [(SPHERE[1] - SPHERE[0]) * rad / el[0], (SPHERE[3] - SPHERE[2]) * rad / el[1],
             (SPHERE[5] - SPHERE[4]) / el[2]]
        out = os.path.join(d, f"geo{l}.bin")
        subprocess.run([exe] + [str(e) for e in el] + [repr(SPHERE[0] * rad), repr(SPHERE[2] * rad), repr(SPHERE[4])] +
                       [repr(x) for x in h] + [out], check=True, capture_output=True)
        raw = np.fromfile(out, dtype=np.float64)
        raw = raw.reshape(-1, sum(int(np.prod(s)) for _, s in FIELDS))
        G, o = {}, 0
        for nm, s in FIELDS:
            k = int(np.prod(s))
            G[nm] = raw[:, o:o + k].reshape((raw.shape[0],) + s)
            o += k
        return el, G
    return level


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "golden", "sphere_tdep.npz")))


def mesh(el):
    """Element node lists (nel x 8), element column index, constrained-dof mask."""
    no = [e + 1 for e in el]
    ey, ex, ez = np.meshgrid(np.arange(el[1]), np.arange(el[0]), np.arange(el[2]), indexing="ij")
    ex, ey, ez = ex.reshape(-1), ey.reshape(-1), ez.reshape(-1)
    nodes = np.stack([(ez + LOC[a, 2]) + no[2] * ((ex + LOC[a, 0]) + no[0] * (ey + LOC[a, 1])) for a in range(8)], 1)
    col = ex * el[2] + ez
    y, x, z = np.meshgrid(np.arange(no[1]), np.arange(no[0]), np.arange(no[2]), indexing="ij")
    cons = np.stack([(x == 0) | (x == no[0] - 1), (y == 0) | (y == no[1] - 1), (z == 0) | (z == no[2] - 1)], -1)
    return nodes, col, cons.reshape(-1)


@pytest.mark.parametrize("lev", [0, 1, 2])
def test_operators_from_geometry_match_reference(dump, gold, lev):
    el, G = dump(lev)
    nodes, col, cons = mesh(el)
    neq = cons.size
    eta = gold[f"EVI_{lev}"].reshape(-1, 8)
    g = G["g"][col].reshape(-1, 8, 3)
    Ke = np.einsum("ek,ekabq->eabq", eta, G["Mk"][col]).reshape(-1, 8, 8, 3, 3)
    Ke += 1e3 * eta.mean(1)[:, None, None, None, None] * np.einsum("eai,ebj->eabij", g, g)
    dof = (3 * nodes[:, :, None] + np.arange(3)).reshape(-1, 24)
    Kf = Ke.transpose(0, 1, 3, 2, 4).reshape(-1, 24, 24)
    u = gold[f"u_{lev}"][:neq]
    um = np.where(cons, 0.0, u)
    Ku = np.zeros(neq)
    np.add.at(Ku, dof, np.einsum("epq,eq->ep", Kf, um[dof]))
    Ku[cons] = 0.0
    diag = np.zeros(neq)
    np.add.at(diag, dof, np.einsum("epp->ep", Kf))
    divu = np.einsum("ep,ep->e", g.reshape(-1, 24), u[dof])
    grad = np.zeros(neq)
    np.add.at(grad, dof, g.reshape(-1, 24) * gold[f"p_{lev}"][:, None])
    grad[cons] = 0.0
    assert rel(Ku, gold[f"Ku_{lev}"][:neq]) < 1e-13
    assert rel(1.0 / diag, gold[f"BI_{lev}"][:neq]) < 1e-13
    assert rel(divu, gold[f"divu_{lev}"]) < 1e-13
    assert rel(grad, gold[f"gradp_{lev}"][:neq]) < 1e-13


@pytest.mark.parametrize("lev", [1, 2])
def test_projection_weights_match_reference(dump, gold, lev):
    elf, _ = dump(lev)
    elc, Gc = dump(lev - 1)
    nof = [e + 1 for e in elf]
    nodes_c, col_c, cons_c = mesh(elc)
    i = np.arange(3 * nof[0] * nof[1] * nof[2], dtype=np.float64)
    u = (np.sin(0.29 * i + 0.3) + 0.25 * np.cos(0.013 * i * i)).reshape(-1, 3)
    ey, ex, ez = np.meshgrid(np.arange(elc[1]), np.arange(elc[0]), np.arange(elc[2]), indexing="ij")
    ex, ey, ez = ex.reshape(-1), ey.reshape(-1), ez.reshape(-1)
    AD = np.zeros((cons_c.size // 3, 3))
    M = np.zeros(cons_c.size // 3)
    for a in range(8):
        sx, sy, sz = 2 * ex + LOC[a, 0], 2 * ey + LOC[a, 1], 2 * ez + LOC[a, 2]
        avg = sum(u[(sz + LOC[b, 2]) + nof[2] * ((sx + LOC[b, 0]) + nof[0] * (sy + LOC[b, 1]))] for b in range(8))
        w = Gc["tww"][col_c, a]
        np.add.at(AD, nodes_c[:, a], w[:, None] * avg)
        np.add.at(M, nodes_c[:, a], w)
    AD = (AD / M[:, None]).reshape(-1)
    assert rel(AD, gold[f"proj_{lev}"][:AD.size]) < 1e-13


def test_forces_match_reference(dump, gold):
    el, G = dump(2)
    nodes, col, cons = mesh(el)
    b = gold["buoyancy0"][nodes]                     # nel x 8
    fg = np.einsum("eka,ea->ek", G["N"][col], b)     # force at the Gauss points
    fe = np.einsum("ek,eka,ek,ekai->eai", fg, G["N"][col], G["gda"][col], G["cr"][col])
    F = np.zeros(cons.size)
    np.add.at(F, (3 * nodes[:, :, None] + np.arange(3)).reshape(-1), fe.reshape(-1))
    F[cons] = 0.0
    assert rel(F, gold["s0_F"][:F.size]) < 1e-13


@pytest.mark.parametrize("lev", [1, 2])
def test_interpolation_weights_match_reference(dump, gold, lev):
    """interp_vector (Solver_multigrid.c:173-298): fills along x, z, y with
    weights x2/(x1+x2) from the sizes of the neighbours' first elements."""
    elf, Gf = dump(lev)
    elc, _ = dump(lev - 1)
    nof, noc = [e + 1 for e in elf], [e + 1 for e in elc]
    i = np.arange(3 * noc[0] * noc[1] * noc[2], dtype=np.float64)
    ad = (np.sin(0.43 * i + 0.9) + 0.25 * np.cos(0.013 * i * i)).reshape(noc[1], noc[0], noc[2], 3)
    au = np.zeros((nof[1], nof[0], nof[2], 3))
    au[::2, ::2, ::2] = ad
    size = Gf["size"]

    def col(x, z):
        return max(x, 0) * elf[2] + max(z, 0)
    for y in range(0, nof[1], 2):
        for z in range(0, nof[2], 2):
            for x in range(1, nof[0] - 1, 2):
                x1, x2 = size[col(x - 2, z - 1), 0], size[col(x, z - 1), 0]
                au[y, x, z] = x2 / (x1 + x2) * au[y, x - 1, z] + x1 / (x1 + x2) * au[y, x + 1, z]
    for y in range(0, nof[1], 2):
        for x in range(nof[0]):
            for z in range(1, nof[2] - 1, 2):
                x1, x2 = size[col(x - 1, z - 2), 2], size[col(x - 1, z), 2]
                au[y, x, z] = x2 / (x1 + x2) * au[y, x, z - 1] + x1 / (x1 + x2) * au[y, x, z + 1]
    for y in range(1, nof[1] - 1, 2):
        au[y] = 0.5 * au[y - 1] + 0.5 * au[y + 1]
    assert rel(au.reshape(-1), gold[f"interp_{lev}"][:au.size]) < 1e-13


def test_horizontal_average_weights_match_reference(dump, gold):
    """thermal_buoyancy: Ra T minus its layer mean, the mean weighted by the
    lower faces of each layer's elements (return_horiz_ave)."""
    el, G = dump(2)
    no = [e + 1 for e in el]
    T = gold["T0"].reshape(no[1], no[0], no[2])
    Ra = 1e4
    buoy = np.empty_like(T)
    for z in range(no[2]):
        ez = min(z, el[2] - 1)
        s = w = 0.0
        for y in range(el[1]):
            for x in range(el[0]):
                wf = G["wface"][x * el[2] + ez]
                s += Ra * (T[y, x, z] * wf[0] + T[y, x + 1, z] * wf[1] + T[y + 1, x + 1, z] * wf[2] + T[y + 1, x, z] * wf[3])
                w += wf.sum()
        buoy[:, :, z] = Ra * T[:, :, z] - s / w
    assert rel(buoy.reshape(-1), gold["buoyancy0"]) < 1e-12
