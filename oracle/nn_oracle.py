"""CPU oracle of the warm-start network (numpy).  Test infrastructure only:
it checks the library's tensor-core forward pass and gradients, and is never
called by the product path.

The network has no counterpart in the reference (CitcomCU starts every Stokes
solve from the previous step's solution, Stokes_flow_Incomp.c:295); this file
restates the library's own definition in plain array code, in float64, with
the values that the GPU stores in BF16 rounded to BF16 at the same points
(round to nearest even), so that the two agree to the accumulation-order
differences of FP32 versus float64.

Arrays are (ny, nx, nz, channels): flattening gives the solver's node order
v = z + nz (x + nx y).  Tap k of a 3x3x3 kernel is 9 (dy + 1) + 3 (dx + 1) +
(dz + 1).  Parameters are one flat float32 vector: per layer W[cout][cin][27]
then b[cout].
"""
from __future__ import annotations

import numpy as np

# (resolution, cin, cout, relu); resolution r has (n - 1) / 2^r + 1 nodes per axis
LAYERS = [(0, 2, 16, 1), (0, 16, 16, 1), (1, 16, 32, 1), (1, 32, 32, 1), (2, 32, 64, 1),
          (2, 64, 64, 1), (1, 64, 32, 1), (0, 32, 16, 1), (0, 16, 4, 0)]


def param_count() -> int:
    return sum(27 * ci * co + co for _, ci, co, _ in LAYERS)


def _bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(p):
    out, o = [], 0
    for _, ci, co, _ in LAYERS:
        w = np.asarray(p[o:o + 27 * ci * co], dtype=np.float64).reshape(co, ci, 27)
        o += 27 * ci * co
        b = np.asarray(p[o:o + co], dtype=np.float64)
        o += co
        out.append((w, b))
    return out


def pack(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([w.reshape(-1), b.reshape(-1)]) for w, b in layers]).astype(np.float64)


def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ls = []
    for _, ci, co, _ in LAYERS:
        a = np.sqrt(6.0 / (27.0 * ci))
        ls.append((rng.uniform(-a, a, size=(co, ci, 27)), rng.uniform(-0.1, 0.1, size=co)))
    return pack(ls)


def _taps():
    for k in range(27):
        yield k, k // 9 - 1, (k // 3) % 3 - 1, k % 3 - 1


def _shift(xp, dy, dx, dz, shape):
    ny, nx, nz = shape
    return xp[1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx, 1 + dz:1 + dz + nz]


def conv(x, w):
    """sum_k sum_i x[v + off_k][i] w[o][i][k] (zero padding)."""
    shape = x.shape[:3]
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros(shape + (w.shape[0],))
    for k, dy, dx, dz in _taps():
        out += _shift(xp, dy, dx, dz, shape) @ w[:, :, k].T
    return out


def conv_data_grad(g, w):
    """Transpose of conv with respect to x."""
    shape = g.shape[:3]
    dxp = np.zeros((shape[0] + 2, shape[1] + 2, shape[2] + 2, w.shape[1]))
    for k, dy, dx, dz in _taps():
        dxp[1 + dy:1 + dy + shape[0], 1 + dx:1 + dx + shape[1], 1 + dz:1 + dz + shape[2]] += g @ w[:, :, k]
    return dxp[1:-1, 1:-1, 1:-1]


def conv_weight_grad(x, g):
    shape = x.shape[:3]
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    gw = np.zeros((g.shape[-1], x.shape[-1], 27))
    g2 = g.reshape(-1, g.shape[-1])
    for k, dy, dx, dz in _taps():
        gw[:, :, k] = g2.T @ _shift(xp, dy, dx, dz, shape).reshape(-1, x.shape[-1])
    return gw


def prolong(c):
    """Trilinear prolongation of a node grid to 2n - 1 nodes per axis."""
    f = c
    for ax in range(3):
        n = f.shape[ax]
        shape = list(f.shape)
        shape[ax] = 2 * n - 1
        g = np.zeros(shape)
        idx = [slice(None)] * 4
        idx[ax] = slice(0, None, 2)
        g[tuple(idx)] = f
        a = [slice(None)] * 4
        b = [slice(None)] * 4
        a[ax] = slice(0, n - 1)
        b[ax] = slice(1, n)
        idx[ax] = slice(1, None, 2)
        g[tuple(idx)] = 0.5 * (f[tuple(a)] + f[tuple(b)])
        f = g
    return f


def prolong_t(f):
    """Transpose of prolong."""
    c = f
    for ax in range(3):
        nf = c.shape[ax]
        nc = (nf + 1) // 2
        sl = lambda s: tuple(s if i == ax else slice(None) for i in range(4))  # noqa: E731
        g = c[sl(slice(0, None, 2))].copy()
        odd = c[sl(slice(1, None, 2))]
        g[sl(slice(0, nc - 1))] += 0.5 * odd
        g[sl(slice(1, nc))] += 0.5 * odd
        c = g
    return c


def norm(shape):
    """Per coarse node: the sum of the prolongation weights onto the fine grid."""
    ws = []
    for n in shape:
        w = np.ones(n)
        w[1:] += 0.5
        w[:-1] += 0.5
        ws.append(w)
    return (ws[0][:, None, None] * ws[1][None, :, None] * ws[2][None, None, :])[..., None]


def restrict(f):
    c = prolong_t(f)
    return c / norm(c.shape[:3])


def restrict_t(c):
    return prolong(c / norm(c.shape[:3]))


def forward(p, x, exact: bool = False):
    """x: (ny, nx, nz, 2) -> (y (ny, nx, nz, 4), saved activations).  exact:
    no BF16 rounding (float64 throughout, for finite-difference checks)."""
    bf16 = (lambda a: np.asarray(a, dtype=np.float64)) if exact else _bf16
    L = unpack(p)
    W = [bf16(w) for w, _ in L]
    B = [b if exact else b.astype(np.float32).astype(np.float64) for _, b in L]
    relu = lambda a: np.maximum(a, 0.0)  # noqa: E731
    s = {}
    s["x0"] = bf16(x)
    s["a1"] = bf16(relu(conv(s["x0"], W[0]) + B[0]))
    s["a2"] = bf16(relu(conv(s["a1"], W[1]) + B[1]))
    s["b0"] = bf16(restrict(s["a2"]))
    s["b1"] = bf16(relu(conv(s["b0"], W[2]) + B[2]))
    s["b2"] = bf16(relu(conv(s["b1"], W[3]) + B[3]))
    s["c0"] = bf16(restrict(s["b2"]))
    s["c1"] = bf16(relu(conv(s["c0"], W[4]) + B[4]))
    s["c2"] = bf16(relu(conv(s["c1"], W[5]) + B[5]))
    s["d0"] = bf16(prolong(s["c2"]))
    s["d1"] = bf16(relu(conv(s["d0"], W[6]) + B[6] + s["b2"]))
    s["e0"] = bf16(prolong(s["d1"]))
    s["e1"] = bf16(relu(conv(s["e0"], W[7]) + B[7] + s["a2"]))
    y = conv(s["e1"], W[8]) + B[8]
    return y, (W, s)


def loss_grad(p, x, t, exact: bool = False):
    """loss = mean (y - t)^2 and its gradient (flat parameter layout)."""
    bf16 = (lambda a: np.asarray(a, dtype=np.float64)) if exact else _bf16
    y, (W, s) = forward(p, x, exact)
    scale = 1.0 / y.size
    loss = scale * float(np.sum((y - t) ** 2))
    pos = lambda a: (a > 0.0).astype(np.float64)  # noqa: E731
    gW, gB = [None] * 9, [None] * 9

    def wb(l, xin, g):
        gW[l] = conv_weight_grad(xin, g)
        gB[l] = g.reshape(-1, g.shape[-1]).sum(axis=0)

    gy = bf16(2.0 * scale * (y - t))
    wb(8, s["e1"], gy)
    ge1 = bf16(conv_data_grad(gy, W[8]) * pos(s["e1"]))
    wb(7, s["e0"], ge1)
    ge0 = bf16(conv_data_grad(ge1, W[7]))
    gd1 = bf16(prolong_t(ge0) * pos(s["d1"]))
    wb(6, s["d0"], gd1)
    gd0 = bf16(conv_data_grad(gd1, W[6]))
    gc2 = bf16(prolong_t(gd0) * pos(s["c2"]))
    wb(5, s["c1"], gc2)
    gc1 = bf16(conv_data_grad(gc2, W[5]) * pos(s["c1"]))
    wb(4, s["c0"], gc1)
    gc0 = bf16(conv_data_grad(gc1, W[4]))
    gb2 = bf16((restrict_t(gc0) + gd1) * pos(s["b2"]))
    wb(3, s["b1"], gb2)
    gb1 = bf16(conv_data_grad(gb2, W[3]) * pos(s["b1"]))
    wb(2, s["b0"], gb1)
    gb0 = bf16(conv_data_grad(gb1, W[2]))
    ga2 = bf16((restrict_t(gb0) + ge1) * pos(s["a2"]))
    wb(1, s["a1"], ga2)
    ga1 = bf16(conv_data_grad(ga2, W[1]) * pos(s["a1"]))
    wb(0, s["x0"], ga1)
    return loss, pack(list(zip(gW, gB)))


bf16 = _bf16
