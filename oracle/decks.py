"""Input decks for running the reference CitcomCU build (test infrastructure).

The keys and their meaning follow the reference's own example decks
(examples/Busse1993/case1a.input, examples/input1) and the reader in
Instructions.c:690-1060 / Convection.c:114-300 / Viscosity_structures.c:57-330.
The solver knobs (aug_lagr, precond, mg_cycle, down_heavy, up_heavy, vlowstep,
vhighstep, piterations) default to examples/input1:176-199.

`Case` also carries everything the GPU library needs to build the same problem
(mesh, boundary conditions, rheology, solver controls), so one object drives
the reference, the oracle restatement and the CUDA path alike.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional


@dataclasses.dataclass
class Case:
    name: str = "case"
    mgunit: tuple = (4, 4, 4)          # (x, y, z) elements of the coarsest level
    levels: int = 3
    dimen: tuple = (1.0, 1.0, 1.0)     # (x, y, z) box size
    rayleigh: float = 1e4
    Q0: float = 0.0
    # rheology: tdepv False -> eta = visc0[mat]; True -> rheol=3,
    # eta = visc0[mat] * exp(viscE[mat] * (viscT[mat] - T)) (Viscosity_structures.c:617-646)
    tdepv: bool = False
    visc0: tuple = (1.0,)
    viscE: tuple = (0.0,)
    viscT: tuple = (0.0,)
    z_layer: tuple = ()                # material interfaces, top down (num_mat-1 values)
    vmin: Optional[float] = None
    vmax: Optional[float] = None
    # initial temperature (Convection.c:344-350) when no T0 array is given
    perturbmag: float = 0.01
    perturbk: float = 1.0
    # solver controls
    aug_lagr: bool = True
    aug_number: float = 1.0e3
    precond: bool = True
    mg_cycle: int = 1
    down_heavy: int = 3
    up_heavy: int = 3
    vlowstep: int = 20
    vhighstep: int = 3
    piterations: int = 375
    accuracy: float = 1.0e-6
    # Uzawa stopping rule: 0 the reference's (dv/v, dp/p); 1 the residual rule
    # (GPU library and oracle only; the reference build has no such rule)
    stop_rule: int = 0
    # energy equation
    adv_sub_iterations: int = 2
    finetunedt: float = 0.75
    fixed_timestep: float = 0.0
    maxstep: int = 10
    # regional spherical shell segment (Geometry=Rsphere): theta_north,
    # theta_south, fi_west, fi_east in degrees, radius_inner, radius_outer;
    # None is the Cartesian box.  x, y, z of the mesh are then theta, phi, r.
    sphere: Optional[tuple] = None
    # stress-dependent viscosity (Viscosity_structures.c:155-162, 286, 303-307)
    sdepv: bool = False
    sdepv_rheology: int = 2
    sdepv_expt: tuple = (3.0,)
    sdepv_trns: tuple = (1.0,)
    sdepv_misfit: float = 0.001
    max_sdep_visc_iter: int = 50
    sdepv_iter_damp: float = 1.0

    @property
    def nox(self):
        return self.mgunit[0] * 2 ** (self.levels - 1) + 1

    @property
    def noy(self):
        return self.mgunit[1] * 2 ** (self.levels - 1) + 1

    @property
    def noz(self):
        return self.mgunit[2] * 2 ** (self.levels - 1) + 1

    @property
    def nno(self):
        return self.nox * self.noy * self.noz

    @property
    def nel(self):
        return (self.nox - 1) * (self.noy - 1) * (self.noz - 1)

    def num_mat(self):
        return len(self.visc0)


def _vec(v) -> str:
    return ",".join(repr(float(x)) for x in v)


def make_deck(c: Case, datafile: str) -> str:
    nm = c.num_mat()
    lines: List[str] = [
        f'datafile="{datafile}"',
        'use_scratch="local"',
        f'oldfile="{datafile}"',
        "restart=0", "restart_timesteps=0", "stokes_flow_only=0",
        f"maxstep={c.maxstep}", "storage_spacing=1",
        "Solver=multigrid node_assemble=1",
        f"rayleigh={c.rayleigh!r}", "rayleigh_comp=0", "composition=0",
        f"Q0={c.Q0!r}", "Q0_enriched=0", "markers_per_ele=0", "comp_depth=0.605",
        "visc_heating=0", "adi_heating=0",
        "nprocx=1", "nprocz=1", "nprocy=1",
        f"nodex={c.nox} nodez={c.noz} nodey={c.noy}",
        f"mgunitx={c.mgunit[0]}", f"mgunitz={c.mgunit[2]}", f"mgunity={c.mgunit[1]}",
        f"levels={c.levels}",
    ] + (_geometry_cart(c) if c.sphere is None else _geometry_sphere(c)) + [
        "z_lmantle=0.76655052", "z_410=0.857143", "z_lith=0.9651568",
        "rheol=3",
        f"TDEPV={'on' if c.tdepv else 'off'}",
        f"VISC_UPDATE={'on' if (c.tdepv or c.sdepv) else 'off'}",
        "update_every_steps=1",
        f"num_mat={nm}",
        f"visc0={_vec(c.visc0)}", f"viscE={_vec(c.viscE)}", f"viscT={_vec(c.viscT)}",
        f"viscZ={_vec([0.0] * nm)}",
        f"SDEPV={'on' if c.sdepv else 'off'}", f"sdepv_rheology={c.sdepv_rheology}",
        f"sdepv_misfit={c.sdepv_misfit!r}", f"max_sdep_visc_iter={c.max_sdep_visc_iter}",
        f"sdepv_iter_damp={c.sdepv_iter_damp!r}",
        f"sdepv_expt={_vec((list(c.sdepv_expt) * nm)[:nm])}", f"sdepv_trns={_vec((list(c.sdepv_trns) * nm)[:nm])}",
        f"VMIN={'on' if c.vmin is not None else 'off'} visc_min={c.vmin if c.vmin is not None else 1e-3!r}",
        f"VMAX={'on' if c.vmax is not None else 'off'} visc_max={c.vmax if c.vmax is not None else 1e3!r}",
        "visc_smooth_cycles=1", "Viscosity=system",
        "layerd=2870000.0", "radius=6370000.0", "ReferenceT=3800.0", "refvisc=1.0e20",
        "density=3300.0", "thermdiff=1.0e-6", "gravacc=9.8", "thermexp=5e-5", "cp=1250",
        "wdensity=0.0", "visc_factor=1.0", "thermexp_factor=1.0", "thermdiff_factor=1.00",
        "dissipation_number=0.0", "surf_temp=0.078947",
        "Ra_410=0.0", "Ra_670=0.0", "clapeyron410=3.0e6", "clapeyron670=-3.0e6",
        "width410=3.5e4", "width670=3.5e4",
        "topvbc=0", "topvbxval=0.0", "topvbyval=0.0",
        "botvbc=0", "botvbxval=0.0", "botvbyval=0.0",
        "toptbc=1 bottbc=1", "toptbcval=0.0 bottbcval=1.0",
        "periodicx=off", "periodicy=off", "flowthroughx=off", "flowthroughy=off",
        "num_perturbations=1", f"perturbmag={c.perturbmag!r}", f"perturbk={c.perturbk!r}",
        "perturbl=1.0", "perturbm=0.0",
        "Problem=convection",
        f"aug_lagr={'on' if c.aug_lagr else 'off'}", f"aug_number={c.aug_number!r}",
        f"precond={'on' if c.precond else 'off'}", "orthogonal=off", "maxsub=1",
        "viterations=2", f"mg_cycle={c.mg_cycle}", f"down_heavy={c.down_heavy}",
        f"up_heavy={c.up_heavy}", f"vlowstep={c.vlowstep}", f"vhighstep={c.vhighstep}",
        f"piterations={c.piterations}", f"accuracy={c.accuracy!r}",
        "tole_compressibility=1e-7",
        f"adv_sub_iterations={c.adv_sub_iterations}", f"finetunedt={c.finetunedt!r}",
        f"fixed_timestep={c.fixed_timestep!r}",
        "ll_max=20", "nlong=180", "nlati=90",
        "DESCRIBE=off", "BEGINNER=off", "VERBOSE=off", "verbose=off", "see_convergence=1",
    ]
    # Viscosity_structures.c:120-135 wants num_mat values of z_layer (r_layer
    # in the sphere): material l+1 where the element centroid z (r) >=
    # z_layer[l], scanned top down
    zl = list(c.z_layer) + [0.0] * (nm - len(c.z_layer))
    lines.append(f"{'z' if c.sphere is None else 'r'}_layer={_vec(zl)}")
    return "\n".join(lines) + "\n"


def _geometry_cart(c: Case) -> List[str]:
    return ["Geometry=cart3d",
            f"dimenx={c.dimen[0]!r}", f"dimenz={c.dimen[2]!r}", f"dimeny={c.dimen[1]!r}",
            "z_grid_layers=2", f"zz=0.0,{c.dimen[2]!r}", f"nz=1,{c.noz}",
            "x_grid_layers=2", f"xx=0.0,{c.dimen[0]!r}", f"nx=1,{c.nox}",
            "y_grid_layers=2", f"yy=0.0,{c.dimen[1]!r}", f"ny=1,{c.noy}"]


def _geometry_sphere(c: Case) -> List[str]:
    # Instructions.c:1018-1029 (corners), Nodal_mesh.c:87-133 (t/f/r grid layers)
    tn, ts, fw, fe, ri, ro = c.sphere
    return ["Geometry=Rsphere",
            f"theta_north={tn!r}", f"theta_south={ts!r}", f"fi_west={fw!r}", f"fi_east={fe!r}",
            f"radius_inner={ri!r}", f"radius_outer={ro!r}",
            "r_grid_layers=2", f"rr={ri!r},{ro!r}", f"nr=1,{c.noz}",
            "t_grid_layers=2", f"tt={tn!r},{ts!r}", f"nt=1,{c.nox}",
            "f_grid_layers=2", f"ff={fw!r},{fe!r}", f"nf=1,{c.noy}",
            "r_lmantle=0.7", "r_410=0.9", "r_lith=0.98"]


def conductive_T0(c: Case, amp: float = 0.01, seed: int = 0):
    """Seeded initial temperature: 1 - z plus uniform noise of +-amp on interior
    nodes (Dirichlet rows at z=0/z=dimenz are reset to the boundary values).
    Node order is z fastest, then x, then y (Construct_arrays.c:78-81)."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    z = np.linspace(0.0, c.dimen[2], c.noz)
    T = np.empty((c.noy, c.nox, c.noz))
    T[:] = 1.0 - z / c.dimen[2]
    T += rng.uniform(-amp, amp, size=T.shape)
    T[:, :, 0] = 1.0
    T[:, :, -1] = 0.0
    return T.reshape(-1)


def sinusoid_T0(c: Case):
    """T = 1 - z + A sin(pi z) cos(k pi x) cos(k pi y) (Convection.c:344-350)."""
    import numpy as np
    x = np.linspace(0.0, c.dimen[0], c.nox)
    y = np.linspace(0.0, c.dimen[1], c.noy)
    z = np.linspace(0.0, c.dimen[2], c.noz)
    Y, X, Z = np.meshgrid(y, x, z, indexing="ij")
    T = 1.0 - Z + c.perturbmag * np.sin(math.pi * (1.0 - Z)) * np.cos(c.perturbk * math.pi * X) * \
        np.cos(c.perturbk * math.pi * Y)
    return T.reshape(-1)
