"""CPU oracle of the fields of an output step, for a Cartesian box with uniform
element sizes (numpy).  Test infrastructure only: it is checked against the
reference's own values in the golden fixtures and is never called by the
product path.

Restated from
  heat_flux          Process_buoyancy.c:63-203 (Have.T, the element integrals
                     of u_z T - dT/dz, u_z T' and u_z |T'|, their TWW-weighted
                     nodal values, the surface extrapolation shflux / bhflux,
                     Nut / Nub, and the layer means Have.Rho / F / f)
  averages           Process_velocity.c:179-224 (Have.Vi from
                     visc_from_gint_to_nodes, Nodal_mesh.c:583-615, and
                     Have.vrms), without its composition part
  return_horiz_ave   Global_operations.c:133-240 (area-weighted layer mean)

Node arrays are in the reference's order, node = z + noz (x + nox y); element
e = ez + elz (ex + elx ey).  With uniform elements every Gauss weight, TWW
entry and surface-element area is the same, so the weighted means reduce to
plain means.
"""
from __future__ import annotations

import numpy as np

_G = 1.0 / np.sqrt(3.0)


def _grid(a, nox, noy, noz):
    return np.asarray(a, dtype=np.float64).reshape(noy, nox, noz)


def horiz_ave(a, nox, noy, noz):
    """Layer means: the mean over surface elements of the 4-corner average."""
    g = _grid(a, nox, noy, noz)
    c = 0.25 * (g[:-1, :-1] + g[:-1, 1:] + g[1:, :-1] + g[1:, 1:])
    return c.mean(axis=(0, 1))


def _corners(g):
    """(ely, elx, elz, 8) corner values, corner index 4 dy + 2 dx + dz."""
    out = []
    for dy in (0, 1):
        for dx in (0, 1):
            for dz in (0, 1):
                out.append(g[dy:g.shape[0] - 1 + dy, dx:g.shape[1] - 1 + dx, dz:g.shape[2] - 1 + dz])
    return np.stack(out, axis=-1)


def _shape(hz):
    """N (8 Gauss points x 8 corners) and dN/dz."""
    N = np.zeros((8, 8))
    Nz = np.zeros((8, 8))
    k = 0
    for gy in (-_G, _G):
        for gx in (-_G, _G):
            for gz in (-_G, _G):
                a = 0
                for dy in (0, 1):
                    for dx in (0, 1):
                        for dz in (0, 1):
                            sy, sx, sz = 2 * dy - 1, 2 * dx - 1, 2 * dz - 1
                            fy, fx, fz = (1 + sy * gy) / 2, (1 + sx * gx) / 2, (1 + sz * gz) / 2
                            N[k, a] = fy * fx * fz
                            Nz[k, a] = fy * fx * (sz / 2) * (2.0 / hz)
                            a += 1
                k += 1
    return N, Nz


def _to_nodes(ev):
    """Nodal mean of the adjacent elements' values (uniform TWW)."""
    ely, elx, elz = ev.shape
    s = np.zeros((ely + 1, elx + 1, elz + 1))
    m = np.zeros_like(s)
    for dy in (0, 1):
        for dx in (0, 1):
            for dz in (0, 1):
                s[dy:dy + ely, dx:dx + elx, dz:dz + elz] += ev
                m[dy:dy + ely, dx:dx + elx, dz:dz + elz] += 1.0
    return (s / m).reshape(-1)


def output_fields(T, V, evi, nox, noy, noz, dimen):
    """T (nno), V (3 nno: V[1], V[2], V[3]), evi (nel x 8 Gauss-point
    viscosities) -> dict of Have (6 noz: T, vrms, Vi, Rho, F, f), surf
    (shflux, bhflux), heatflux (as heat_flux leaves it), heatflux_adv, Nut, Nub."""
    nno = nox * noy * noz
    elx, ely, elz = nox - 1, noy - 1, noz - 1
    hz = dimen[2] / elz
    HT = horiz_ave(T, nox, noy, noz)
    Tg = _grid(T, nox, noy, noz)
    Vz = _grid(V[2 * nno:3 * nno], nox, noy, noz)
    N, Nz = _shape(hz)
    ct, cv = _corners(Tg), _corners(Vz)
    ca = _corners(Tg - HT[None, None, :])
    u = cv @ N.T
    t = ct @ N.T
    t1 = ca @ N.T
    dz = ct @ Nz.T
    ue = [np.mean(u * t - dz, axis=-1), np.mean(u * t1, axis=-1), np.mean(u * np.abs(t1), axis=-1)]
    hf, hfadv, flux = (_to_nodes(x) for x in ue)
    g = hf.reshape(noy, nox, noz).copy()
    sh = (2.0 * g[:, :, -1] - g[:, :, -2]).reshape(-1)
    bh = (2.0 * g[:, :, 0] - g[:, :, 1]).reshape(-1)
    g[:, :, -1] = sh.reshape(noy, nox)
    g[:, :, 0] = bh.reshape(noy, nox)

    def surf_mean(s):
        s = s.reshape(noy, nox)
        return float((s[:-1, :-1] + s[:-1, 1:] + s[1:, :-1] + s[1:, 1:]).mean() / 4.0)

    v2 = V[:nno] ** 2 + V[nno:2 * nno] ** 2 + V[2 * nno:] ** 2
    vn = _to_nodes(np.asarray(evi, dtype=np.float64).reshape(ely, elx, elz, 8).mean(axis=-1))
    Have = np.concatenate([HT, np.sqrt(horiz_ave(v2, nox, noy, noz)), horiz_ave(vn, nox, noy, noz),
                           horiz_ave(g.reshape(-1), nox, noy, noz), horiz_ave(hfadv, nox, noy, noz),
                           horiz_ave(flux, nox, noy, noz)])
    return dict(Have=Have, surf=np.concatenate([sh, bh]), heatflux=flux, heatflux_adv=hfadv,
                Nut=surf_mean(sh), Nub=surf_mean(bh))
