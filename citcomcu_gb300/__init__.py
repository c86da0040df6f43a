"""GB300 (sm_103a) implementation of CitcomCU's per-timestep hot path.

The compute lives in the in-tree C-ABI library libcitcom_gb300.so
(include/citcom_gb300.h).  This module is a thin ctypes front end whose method
names and argument meanings follow the reference routines they replace
(solve_Ahat_p_fhat, solve_constrained_flow_iterative, general_stokes_solver,
PG_timestep, construct_stiffness_B_matrix, ...).  There is no CPU fallback: if
the library is missing or no CUDA device is present, construction raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Optional, Tuple

import numpy as np

from .build import LIB as LIB_PATH
from .build import build as _build_lib

__all__ = ["Config", "Solver", "WarmStart", "CitcomGPUError", "load_library", "build", "heat_flux_noalloc", "FP64",
           "MIXED", "STOP_REFERENCE", "STOP_RESIDUAL"]

FP64 = 0
MIXED = 1
STOP_REFERENCE = 0
STOP_RESIDUAL = 1

_ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "invalid state", -4: "no convergence"}


class CitcomGPUError(RuntimeError):
    pass


@dataclasses.dataclass
class Config:
    """Problem and solver controls (field names follow the reference's
    input deck keys, Instructions.c:690-1060)."""
    mgunit: tuple = (4, 4, 4)
    levels: int = 3
    dimen: tuple = (1.0, 1.0, 1.0)
    rayleigh: float = 1e4
    Q0: float = 0.0
    tdepv: bool = False
    visc0: tuple = (1.0,)
    viscE: tuple = (0.0,)
    viscT: tuple = (0.0,)
    z_layer: tuple = ()
    vmin: Optional[float] = None
    vmax: Optional[float] = None
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
    adv_sub_iterations: int = 2
    finetunedt: float = 0.75
    fixed_timestep: float = 0.0
    precision: int = FP64
    # Geometry=Rsphere: (theta_north, theta_south, fi_west, fi_east) in degrees,
    # (radius_inner, radius_outer); x, y, z of the mesh are then theta, phi, r
    # and dimen is unused.  None: the Cartesian box.
    sphere: Optional[tuple] = None
    # stress-dependent viscosity (SDEPV) and the viscosity iteration of
    # general_stokes_solver; sdepv_expt / sdepv_trns per material
    sdepv: bool = False
    sdepv_rheology: int = 2
    sdepv_expt: tuple = (3.0,)
    sdepv_trns: tuple = (1.0,)
    sdepv_misfit: float = 0.001
    max_sdep_visc_iter: int = 50
    sdepv_iter_damp: float = 1.0
    # Uzawa stopping rule: STOP_REFERENCE (dv/v and dp/p below accuracy) or
    # STOP_RESIDUAL (both FP64 residuals of the solution at most accuracy)
    stop_rule: int = 0

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

    @classmethod
    def like(cls, other, **overrides) -> "Config":
        """Copy the matching attributes of any parameter object."""
        kw = {f.name: getattr(other, f.name) for f in dataclasses.fields(cls) if hasattr(other, f.name)}
        kw.update(overrides)
        return cls(**kw)


class _CConfig(ctypes.Structure):
    _fields_ = [
        ("levels", ctypes.c_int),
        ("mgunit", ctypes.c_int * 3),
        ("dimen", ctypes.c_double * 3),
        ("rayleigh", ctypes.c_double),
        ("Q0", ctypes.c_double),
        ("tdepv", ctypes.c_int),
        ("num_mat", ctypes.c_int),
        ("visc0", ctypes.c_double * 8),
        ("viscE", ctypes.c_double * 8),
        ("viscT", ctypes.c_double * 8),
        ("z_layer", ctypes.c_double * 8),
        ("vmin_on", ctypes.c_int),
        ("vmax_on", ctypes.c_int),
        ("vmin", ctypes.c_double),
        ("vmax", ctypes.c_double),
        ("aug_lagr", ctypes.c_int),
        ("aug_number", ctypes.c_double),
        ("precond", ctypes.c_int),
        ("mg_cycle", ctypes.c_int),
        ("down_heavy", ctypes.c_int),
        ("up_heavy", ctypes.c_int),
        ("vlowstep", ctypes.c_int),
        ("vhighstep", ctypes.c_int),
        ("piterations", ctypes.c_int),
        ("accuracy", ctypes.c_double),
        ("adv_sub_iterations", ctypes.c_int),
        ("finetunedt", ctypes.c_double),
        ("fixed_timestep", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("sphere", ctypes.c_int),
        ("theta", ctypes.c_double * 2),
        ("fi", ctypes.c_double * 2),
        ("radius", ctypes.c_double * 2),
        ("sdepv", ctypes.c_int),
        ("sdepv_rheology", ctypes.c_int),
        ("sdepv_expt", ctypes.c_double * 8),
        ("sdepv_trns", ctypes.c_double * 8),
        ("sdepv_misfit", ctypes.c_double),
        ("sdepv_iter_damp", ctypes.c_double),
        ("max_sdep_visc_iter", ctypes.c_int),
        ("stop_rule", ctypes.c_int),
    ]


class _CAdvection(ctypes.Structure):
    _fields_ = [("timestep", ctypes.c_double), ("elapsed_time", ctypes.c_double),
                ("T_interior", ctypes.c_double), ("last_sub_iterations", ctypes.c_int)]


class _CStats(ctypes.Structure):
    _fields_ = [("uzawa_iterations", ctypes.c_int), ("del2_calls", ctypes.c_int), ("mg_passes", ctypes.c_int),
                ("initial_residual", ctypes.c_double), ("stokes_ms", ctypes.c_double), ("energy_ms", ctypes.c_double),
                ("smoother_ms", ctypes.c_double), ("smoother_sweeps", ctypes.c_int),
                ("kernel_launches", ctypes.c_ulonglong), ("visc_iterations", ctypes.c_int),
                ("visc_misfit", ctypes.c_double), ("warm_start", ctypes.c_int),
                ("warm_residual", ctypes.c_double), ("base_residual", ctypes.c_double),
                ("pass_ms", ctypes.c_double), ("final_momentum", ctypes.c_double),
                ("final_continuity", ctypes.c_double), ("corrections", ctypes.c_int),
                ("warm_compared", ctypes.c_int), ("assembly_ms", ctypes.c_double)]


# every symbol of include/citcom_gb300.h with its argument types
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_H = ctypes.c_void_p

# fields of an output step, in the order of citcom_gpu_output; count per field
# in units of (nno, nel, noz, nsf)
OUTPUT_FIELDS = (("T", (1, 0, 0, 0)), ("V", (3, 0, 0, 0)), ("P", (0, 1, 0, 0)), ("heatflux", (1, 0, 0, 0)),
                 ("heatflux_adv", (1, 0, 0, 0)), ("Have", (0, 0, 6, 0)), ("surf", (0, 0, 0, 2)), ("scalars", None))
HAVE_COLUMNS = ("T", "vrms", "Vi", "Rho", "F", "f")


class _COutput(ctypes.Structure):
    _fields_ = [(name, _D) for name, _ in OUTPUT_FIELDS]
_F = ctypes.POINTER(ctypes.c_float)
_SIGNATURES = {
    "citcom_gpu_create": (ctypes.c_int, [ctypes.POINTER(_CConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "citcom_gpu_destroy": (None, [_H]),
    "citcom_gpu_error_string": (ctypes.c_char_p, [_H]),
    "citcom_gpu_level_dims": (ctypes.c_int, [_H, ctypes.c_int, _I]),
    "citcom_gpu_get_system_viscosity": (ctypes.c_int, [_H, _D]),
    "citcom_gpu_set_viscosity": (ctypes.c_int, [_H, ctypes.c_int, _D]),
    "citcom_gpu_get_viscosity": (ctypes.c_int, [_H, ctypes.c_int, _D]),
    "citcom_gpu_construct_stiffness_B_matrix": (ctypes.c_int, [_H]),
    "citcom_gpu_assemble_forces": (ctypes.c_int, [_H, _D, _D, _D]),
    "citcom_gpu_solve_Ahat_p_fhat": (ctypes.c_int, [_H, _D, _D, _D, ctypes.c_double, _I, _D]),
    "citcom_gpu_solve_Ahat_p_fhat_device": (ctypes.c_int, [_H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                           ctypes.c_double, _I, _D]),
    "citcom_gpu_solve_constrained_flow_iterative": (ctypes.c_int, [_H, _D, _D, _D, _D]),
    "citcom_gpu_general_stokes_solver": (ctypes.c_int, [_H, _D, _D, _D, _D]),
    "citcom_gpu_PG_timestep": (ctypes.c_int, [_H, _D, _D, _D, ctypes.POINTER(_CAdvection)]),
    "citcom_gpu_heat_flux": (ctypes.c_int, [_H, _D, _D, _D, _D]),
    "citcom_gpu_vrms": (ctypes.c_int, [_H, _D, _D]),
    "citcom_gpu_load_state": (ctypes.c_int, [_H, _D, _D, _D, _D]),
    "citcom_gpu_store_state": (ctypes.c_int, [_H, _D, _D, _D, _D, _D]),
    "citcom_gpu_stokes_resident": (ctypes.c_int, [_H]),
    "citcom_gpu_step_resident": (ctypes.c_int, [_H, ctypes.POINTER(_CAdvection)]),
    "citcom_gpu_last_stats": (ctypes.c_int, [_H, ctypes.POINTER(_CStats)]),
    "citcom_gpu_stokes_residuals": (ctypes.c_int, [_H, _D]),
    "citcom_gpu_output_async": (ctypes.c_int, [_H, ctypes.POINTER(_COutput)]),
    "citcom_gpu_output_wait": (ctypes.c_int, [_H]),
    "citcom_gpu_op_kmul": (ctypes.c_int, [_H, ctypes.c_int, _D, _D]),
    "citcom_gpu_op_gauss_seidel": (ctypes.c_int, [_H, ctypes.c_int, _D, _D, _D, ctypes.c_int, ctypes.c_int]),
    "citcom_gpu_op_project": (ctypes.c_int, [_H, ctypes.c_int, _D, _D]),
    "citcom_gpu_op_interp": (ctypes.c_int, [_H, ctypes.c_int, _D, _D]),
    "citcom_gpu_op_div": (ctypes.c_int, [_H, ctypes.c_int, _D, _D]),
    "citcom_gpu_op_grad": (ctypes.c_int, [_H, ctypes.c_int, _D, _D]),
    "citcom_gpu_op_multi_grid": (ctypes.c_int, [_H, _D, _D, _D]),
    "citcom_gpu_op_solve_del2_u": (ctypes.c_int, [_H, _D, _D, ctypes.c_double, _I]),
    "citcom_gpu_op_diagonals": (ctypes.c_int, [_H, ctypes.c_int, _D, _D]),
    "citcom_gpu_test_hold_tile_copy": (ctypes.c_int, []),
    "citcom_gpu_heat_flux_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, ctypes.c_void_p,
                                                    ctypes.c_void_p, _D, _D]),
    "citcom_nn_create": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_uint, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "citcom_nn_destroy": (None, [_H]),
    "citcom_nn_error_string": (ctypes.c_char_p, [_H]),
    "citcom_nn_info": (ctypes.c_int, [_H, _I]),
    "citcom_nn_get_params": (ctypes.c_int, [_H, _F]),
    "citcom_nn_set_params": (ctypes.c_int, [_H, _F]),
    "citcom_nn_get_scales": (ctypes.c_int, [_H, _D]),
    "citcom_nn_set_scales": (ctypes.c_int, [_H, _D]),
    "citcom_nn_record": (ctypes.c_int, [_H]),
    "citcom_nn_train": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, ctypes.c_double, _D]),
    "citcom_nn_attach": (ctypes.c_int, [_H, ctypes.c_int]),
    "citcom_nn_set_mode": (ctypes.c_int, [_H, ctypes.c_int]),
    "citcom_nn_set_check_interval": (ctypes.c_int, [_H, ctypes.c_int]),
    "citcom_nn_predict": (ctypes.c_int, [_H, _D, _D]),
    "citcom_nn_forward": (ctypes.c_int, [_H, _F, _F]),
    "citcom_nn_loss_grad": (ctypes.c_int, [_H, _F, _F, _D, _F]),
}

_lib = None


def build(force: bool = False) -> str:
    return _build_lib(force=force)


def load_library(path: str = LIB_PATH):
    """Load the in-tree CUDA library.  Fails loudly when it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise CitcomGPUError(f"{path} is missing: build it with citcomcu_gb300.build() (nvcc, sm_103a)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


NOALLOC_MAX_NODES = 274625
NOALLOC_MAX_ELEMENTS = 262144


def heat_flux_noalloc(nox: int, noy: int, noz: int, dimen, dT: int, dV: int):
    """Nusselt numbers (top, bottom) from device-resident T (nno) and V
    (3*nno) given as raw device addresses, without any device allocation:
    for callers that cannot allocate (see include/citcom_gb300.h).  Raises
    for meshes above NOALLOC_MAX_NODES / NOALLOC_MAX_ELEMENTS."""
    lib = load_library()
    dim = (ctypes.c_double * 3)(*[float(x) for x in dimen])
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib.citcom_gpu_heat_flux_noalloc(nox, noy, noz, dim, ctypes.c_void_p(dT), ctypes.c_void_p(dV),
                                          ctypes.byref(a), ctypes.byref(b))
    if rc != 0:
        raise CitcomGPUError(f"citcom_gpu_heat_flux_noalloc failed ({_ERRORS.get(rc, rc)})")
    return a.value, b.value


def _dp(a: np.ndarray):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("arrays passed to the library must be C-contiguous float64")
    return a.ctypes.data_as(_D)


class Solver:
    """One problem on the current CUDA device (a `citcom_gpu` handle)."""

    def __init__(self, cfg):
        if not isinstance(cfg, Config):
            cfg = Config.like(cfg)
        self.cfg = cfg
        self.lib = load_library()
        c = _CConfig()
        c.levels = cfg.levels
        for i in range(3):
            c.mgunit[i] = cfg.mgunit[i]
            c.dimen[i] = cfg.dimen[i]
        c.rayleigh = cfg.rayleigh
        c.Q0 = cfg.Q0
        c.tdepv = int(cfg.tdepv)
        c.num_mat = len(cfg.visc0)
        zl = list(cfg.z_layer) + [0.0] * (8 - len(cfg.z_layer))
        for i in range(c.num_mat):
            c.visc0[i] = cfg.visc0[i]
            c.viscE[i] = cfg.viscE[i] if i < len(cfg.viscE) else 0.0
            c.viscT[i] = cfg.viscT[i] if i < len(cfg.viscT) else 0.0
        for i in range(8):
            c.z_layer[i] = zl[i]
        c.vmin_on = int(cfg.vmin is not None)
        c.vmax_on = int(cfg.vmax is not None)
        c.vmin = cfg.vmin or 0.0
        c.vmax = cfg.vmax or 0.0
        c.aug_lagr = int(cfg.aug_lagr)
        c.aug_number = cfg.aug_number
        c.precond = int(cfg.precond)
        c.mg_cycle = cfg.mg_cycle
        c.down_heavy = cfg.down_heavy
        c.up_heavy = cfg.up_heavy
        c.vlowstep = cfg.vlowstep
        c.vhighstep = cfg.vhighstep
        c.piterations = cfg.piterations
        c.accuracy = cfg.accuracy
        c.adv_sub_iterations = cfg.adv_sub_iterations
        c.finetunedt = cfg.finetunedt
        c.fixed_timestep = cfg.fixed_timestep
        c.precision = cfg.precision
        c.sdepv = int(cfg.sdepv)
        c.sdepv_rheology = cfg.sdepv_rheology
        for i in range(8):
            c.sdepv_expt[i] = cfg.sdepv_expt[min(i, len(cfg.sdepv_expt) - 1)]
            c.sdepv_trns[i] = cfg.sdepv_trns[min(i, len(cfg.sdepv_trns) - 1)]
        c.sdepv_misfit = cfg.sdepv_misfit
        c.sdepv_iter_damp = cfg.sdepv_iter_damp
        c.max_sdep_visc_iter = cfg.max_sdep_visc_iter
        c.stop_rule = int(cfg.stop_rule)
        if cfg.sphere is not None:
            tn, ts, fw, fe, ri, ro = cfg.sphere
            c.sphere = 1
            c.theta[0], c.theta[1] = tn, ts
            c.fi[0], c.fi[1] = fw, fe
            c.radius[0], c.radius[1] = ri, ro
        self._c = c
        h = ctypes.c_void_p()
        rc = self.lib.citcom_gpu_create(ctypes.byref(c), ctypes.byref(h))
        if rc != 0:
            raise CitcomGPUError(f"citcom_gpu_create failed ({_ERRORS.get(rc, rc)}); a CUDA device is required")
        self.h = h
        self.dims = []
        for l in range(cfg.levels):
            d = (ctypes.c_int * 6)()
            self._check(self.lib.citcom_gpu_level_dims(self.h, l, d))
            self.dims.append(dict(nox=d[0], noy=d[1], noz=d[2], nno=d[3], nel=d[4], neq=d[5]))

    # ---------------------------------------------------------------- admin
    def close(self):
        if getattr(self, "h", None):
            self.lib.citcom_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.citcom_gpu_error_string(self.h)
            raise CitcomGPUError(f"{_ERRORS.get(rc, rc)}: {msg.decode() if msg else ''}")

    @property
    def fine(self):
        return self.dims[-1]

    def stats(self) -> dict:
        s = _CStats()
        self._check(self.lib.citcom_gpu_last_stats(self.h, ctypes.byref(s)))
        return dict(uzawa=s.uzawa_iterations, del2_calls=s.del2_calls, mg_passes=s.mg_passes,
                    initial_residual=s.initial_residual, stokes_ms=s.stokes_ms, energy_ms=s.energy_ms,
                    smoother_ms=s.smoother_ms, smoother_sweeps=s.smoother_sweeps, kernel_launches=s.kernel_launches,
                    warm_start=s.warm_start, warm_residual=s.warm_residual, base_residual=s.base_residual,
                    visc_iterations=s.visc_iterations, visc_misfit=s.visc_misfit, pass_ms=s.pass_ms,
                    final_momentum=s.final_momentum, final_continuity=s.final_continuity,
                    corrections=s.corrections, warm_compared=s.warm_compared, assembly_ms=s.assembly_ms)

    def stokes_residuals(self):
        """(|F - K U - G P| / |F|, |div U| / (|U| sqrt(npno/neq))) of the resident solution."""
        out = np.zeros(2)
        self._check(self.lib.citcom_gpu_stokes_residuals(self.h, _dp(out)))
        return float(out[0]), float(out[1])

    # --------------------------------------------------------- set-up steps
    def get_system_viscosity(self, T):
        self._check(self.lib.citcom_gpu_get_system_viscosity(self.h, _dp(np.ascontiguousarray(T, dtype=np.float64))))

    def set_viscosity(self, lev, evi):
        self._check(self.lib.citcom_gpu_set_viscosity(self.h, lev, _dp(np.ascontiguousarray(evi, dtype=np.float64))))

    def get_viscosity(self, lev):
        out = np.zeros(self.dims[lev]["nel"] * 8)
        self._check(self.lib.citcom_gpu_get_viscosity(self.h, lev, _dp(out)))
        return out

    def construct_stiffness_B_matrix(self):
        self._check(self.lib.citcom_gpu_construct_stiffness_B_matrix(self.h))

    def assemble_forces(self, T) -> Tuple[np.ndarray, np.ndarray]:
        F = np.zeros(self.fine["neq"])
        b = np.zeros(self.fine["nno"])
        self._check(self.lib.citcom_gpu_assemble_forces(self.h, _dp(np.ascontiguousarray(T, dtype=np.float64)),
                                                        _dp(F), _dp(b)))
        return F, b

    # ---------------------------------------------------------------- solves
    def solve_Ahat_p_fhat(self, V, P, F, imp, steps_max):
        """V (neq) and P (npno) are updated in place; returns (initial
        residual, iterations) like the reference (return value, *steps_max)."""
        steps = ctypes.c_int(steps_max)
        r0 = ctypes.c_double(0.0)
        self._check(self.lib.citcom_gpu_solve_Ahat_p_fhat(self.h, _dp(V), _dp(P),
                                                          _dp(np.ascontiguousarray(F, dtype=np.float64)),
                                                          imp, ctypes.byref(steps), ctypes.byref(r0)))
        return r0.value, steps.value

    def solve_Ahat_p_fhat_device(self, dV: int, dP: int, dF: int, imp, steps_max):
        """Device-pointer variant (integers from e.g. torch.Tensor.data_ptr())."""
        steps = ctypes.c_int(steps_max)
        r0 = ctypes.c_double(0.0)
        self._check(self.lib.citcom_gpu_solve_Ahat_p_fhat_device(self.h, ctypes.c_void_p(dV), ctypes.c_void_p(dP),
                                                                 ctypes.c_void_p(dF), imp, ctypes.byref(steps),
                                                                 ctypes.byref(r0)))
        return r0.value, steps.value

    def _out_V(self, V):
        """The nodal velocity output (3 nno): the caller's buffer (e.g. pinned
        host memory, written in place like the reference's E->V) or a new one."""
        n = 3 * self.fine["nno"]
        if V is None:
            return np.zeros(n)
        if V.shape != (n,):
            raise ValueError(f"V must have shape ({n},)")
        return V

    def solve_constrained_flow_iterative(self, U, P, F, V=None):
        V = self._out_V(V)
        self._check(self.lib.citcom_gpu_solve_constrained_flow_iterative(
            self.h, _dp(U), _dp(P), _dp(np.ascontiguousarray(F, dtype=np.float64)), _dp(V)))
        return V

    def general_stokes_solver(self, T, U, P, V=None):
        V = self._out_V(V)
        self._check(self.lib.citcom_gpu_general_stokes_solver(self.h, _dp(np.ascontiguousarray(T, dtype=np.float64)),
                                                              _dp(U), _dp(P), _dp(V)))
        return V

    def PG_timestep(self, T, Tdot, V, elapsed_time=0.0) -> dict:
        adv = _CAdvection()
        adv.elapsed_time = elapsed_time
        self._check(self.lib.citcom_gpu_PG_timestep(self.h, _dp(T), _dp(Tdot),
                                                    _dp(np.ascontiguousarray(V, dtype=np.float64)), ctypes.byref(adv)))
        return dict(timestep=adv.timestep, elapsed_time=adv.elapsed_time, T_interior=adv.T_interior)

    def heat_flux(self, T=None, V=None):
        a, b = ctypes.c_double(), ctypes.c_double()
        Tp = _dp(np.ascontiguousarray(T, dtype=np.float64)) if T is not None else None
        Vp = _dp(np.ascontiguousarray(V, dtype=np.float64)) if V is not None else None
        self._check(self.lib.citcom_gpu_heat_flux(self.h, Tp, Vp, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def vrms(self, V=None):
        r = ctypes.c_double()
        Vp = _dp(np.ascontiguousarray(V, dtype=np.float64)) if V is not None else None
        self._check(self.lib.citcom_gpu_vrms(self.h, Vp, ctypes.byref(r)))
        return r.value

    # ------------------------------------------------------ resident state
    def load_state(self, T=None, Tdot=None, U=None, P=None):
        conv = lambda a: _dp(np.ascontiguousarray(a, dtype=np.float64)) if a is not None else None  # noqa: E731
        self._check(self.lib.citcom_gpu_load_state(self.h, conv(T), conv(Tdot), conv(U), conv(P)))

    def store_state(self):
        f = self.fine
        T, Tdot, U, P, V = np.zeros(f["nno"]), np.zeros(f["nno"]), np.zeros(f["neq"]), np.zeros(f["nel"]), \
            np.zeros(3 * f["nno"])
        self._check(self.lib.citcom_gpu_store_state(self.h, _dp(T), _dp(Tdot), _dp(U), _dp(P), _dp(V)))
        return dict(T=T, Tdot=Tdot, U=U, P=P, V=V)

    def stokes_resident(self):
        self._check(self.lib.citcom_gpu_stokes_resident(self.h))

    def step_resident(self, elapsed_time=0.0):
        adv = _CAdvection()
        adv.elapsed_time = elapsed_time
        self._check(self.lib.citcom_gpu_step_resident(self.h, ctypes.byref(adv)))
        return dict(timestep=adv.timestep, elapsed_time=adv.elapsed_time, T_interior=adv.T_interior)

    # ---------------------------------------------------------- output step
    def output_sizes(self) -> dict:
        f = self.fine
        nsf = f["nox"] * f["noy"]
        out = {}
        for name, k in OUTPUT_FIELDS:
            out[name] = 3 if k is None else k[0] * f["nno"] + k[1] * f["nel"] + k[2] * f["noz"] + k[3] * nsf
        return out

    def output_buffers(self, pinned: bool = True) -> dict:
        """Host buffers for output_async, page-locked when torch is available
        (the copy to the host then overlaps the next step)."""
        out = {}
        for name, n in self.output_sizes().items():
            if pinned:
                try:
                    import torch
                    out[name] = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
                    continue
                except Exception:  # noqa: BLE001 - plain memory still works, only without the overlap
                    pass
            out[name] = np.empty(n)
        return out

    def output_async(self, bufs: dict):
        """Start an output step into `bufs` (name -> float64 array, any subset
        of OUTPUT_FIELDS); the arrays are complete after output_wait()."""
        sizes = self.output_sizes()
        o = _COutput()
        for name, n in sizes.items():
            a = bufs.get(name)
            if a is None:
                continue
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size < n:
                raise CitcomGPUError(f"output buffer {name}: need {n} contiguous float64")
            setattr(o, name, _dp(a))
        self._out_bufs = bufs  # kept alive until the copies complete
        self._check(self.lib.citcom_gpu_output_async(self.h, ctypes.byref(o)))

    def output_wait(self):
        self._check(self.lib.citcom_gpu_output_wait(self.h))
        self._out_bufs = None

    def output(self) -> dict:
        """One output step, synchronously: the fields as a dict of arrays,
        Have split into its six layer profiles."""
        bufs = self.output_buffers(pinned=False)
        self.output_async(bufs)
        self.output_wait()
        noz, nsf = self.fine["noz"], self.fine["nox"] * self.fine["noy"]
        out = {k: bufs[k] for k in ("T", "V", "P", "heatflux", "heatflux_adv")}
        for i, c in enumerate(HAVE_COLUMNS):
            out["Have_" + c] = bufs["Have"][i * noz:(i + 1) * noz]
        out["shflux"], out["bhflux"] = bufs["surf"][:nsf], bufs["surf"][nsf:]
        out["Nut"], out["Nub"], out["vrms"] = (float(x) for x in bufs["scalars"])
        return out

    # ---------------------------------------------------- single operators
    def op_kmul(self, lev, u):
        out = np.zeros(self.dims[lev]["neq"])
        self._check(self.lib.citcom_gpu_op_kmul(self.h, lev, _dp(np.ascontiguousarray(u, dtype=np.float64)), _dp(out)))
        return out

    def op_gauss_seidel(self, lev, F, cycles, d0=None):
        n = self.dims[lev]["neq"]
        d = np.zeros(n) if d0 is None else np.array(d0, dtype=np.float64)
        ad = np.zeros(n)
        self._check(self.lib.citcom_gpu_op_gauss_seidel(self.h, lev, _dp(d), _dp(np.ascontiguousarray(F, dtype=np.float64)),
                                                        _dp(ad), cycles, int(d0 is not None)))
        return d, ad

    def op_project(self, fine_lev, AU):
        out = np.zeros(self.dims[fine_lev - 1]["neq"])
        self._check(self.lib.citcom_gpu_op_project(self.h, fine_lev, _dp(np.ascontiguousarray(AU, dtype=np.float64)),
                                                   _dp(out)))
        return out

    def op_interp(self, coarse_lev, AD):
        out = np.zeros(self.dims[coarse_lev + 1]["neq"])
        self._check(self.lib.citcom_gpu_op_interp(self.h, coarse_lev, _dp(np.ascontiguousarray(AD, dtype=np.float64)),
                                                  _dp(out)))
        return out

    def op_div(self, lev, U):
        out = np.zeros(self.dims[lev]["nel"])
        self._check(self.lib.citcom_gpu_op_div(self.h, lev, _dp(np.ascontiguousarray(U, dtype=np.float64)), _dp(out)))
        return out

    def op_grad(self, lev, P):
        out = np.zeros(self.dims[lev]["neq"])
        self._check(self.lib.citcom_gpu_op_grad(self.h, lev, _dp(np.ascontiguousarray(P, dtype=np.float64)), _dp(out)))
        return out

    def op_multi_grid(self, F):
        f = np.array(F, dtype=np.float64)
        d1 = np.zeros_like(f)
        r = ctypes.c_double()
        self._check(self.lib.citcom_gpu_op_multi_grid(self.h, _dp(d1), _dp(f), ctypes.byref(r)))
        return d1, f, r.value

    def op_solve_del2_u(self, F, acc):
        d0 = np.zeros(self.fine["neq"])
        v = ctypes.c_int()
        self._check(self.lib.citcom_gpu_op_solve_del2_u(self.h, _dp(d0), _dp(np.ascontiguousarray(F, dtype=np.float64)),
                                                        acc, ctypes.byref(v)))
        return d0, v.value

    def op_diagonals(self, lev):
        bi = np.zeros(self.dims[lev]["neq"])
        bpi = np.zeros(self.dims[lev]["nel"]) if lev == len(self.dims) - 1 else None
        self._check(self.lib.citcom_gpu_op_diagonals(self.h, lev, _dp(bi), _dp(bpi) if bpi is not None else None))
        return bi, bpi


def _fp(a: np.ndarray):
    if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("arrays passed to the network must be C-contiguous float32")
    return a.ctypes.data_as(_F)


class WarmStart:
    """Learned warm start of a Solver's Stokes solves (a `citcom_nn` handle).

    A 3D convolutional encoder-decoder on the node grid of multigrid level
    `level` (-1: the second finest) maps (T, log10 viscosity) to (u, v, w, p).
    `record()` adds the solver's converged state to the training set,
    `train()` runs Adam steps on it, `attach()` makes every Stokes solve of the
    solver start from the network's guess when that guess has the smaller
    Uzawa initial residual.  With mode=INCREMENT the network instead predicts
    the change of U and P from the change of T since the last solve, and the
    solve starts from the previous solution plus that change scaled by the
    step minimising the momentum residual.  Destroy (close) it before its
    solver."""

    ABSOLUTE = 0
    INCREMENT = 1

    def __init__(self, solver: Solver, level: int = -1, seed: int = 0, capacity: int = 64, mode: int = 0):
        self.solver = solver
        self.lib = solver.lib
        h = ctypes.c_void_p()
        solver._check(self.lib.citcom_nn_create(solver.h, level, seed, capacity, ctypes.byref(h)))
        self.h = h
        self.mode = mode
        if mode:
            self._check(self.lib.citcom_nn_set_mode(self.h, mode))
        info = (ctypes.c_int * 6)()
        self._check(self.lib.citcom_nn_info(self.h, info))
        self.grid = (info[0], info[1], info[2])
        self.n_params = info[3]
        self.level = info[5]
        self.voxels = info[0] * info[1] * info[2]

    def close(self):
        if getattr(self, "h", None):
            self.lib.citcom_nn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.citcom_nn_error_string(self.h)
            raise CitcomGPUError(f"{_ERRORS.get(rc, rc)}: {msg.decode() if msg else ''}")

    @property
    def recorded(self) -> int:
        info = (ctypes.c_int * 6)()
        self._check(self.lib.citcom_nn_info(self.h, info))
        return info[4]

    def get_params(self) -> np.ndarray:
        w = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.lib.citcom_nn_get_params(self.h, _fp(w)))
        return w

    def set_params(self, w):
        self._check(self.lib.citcom_nn_set_params(self.h, _fp(np.ascontiguousarray(w, dtype=np.float32))))

    def get_scales(self):
        s = np.zeros(3)
        self._check(self.lib.citcom_nn_get_scales(self.h, _dp(s)))
        return tuple(float(x) for x in s)

    def set_scales(self, s):
        self._check(self.lib.citcom_nn_set_scales(self.h, _dp(np.ascontiguousarray(s, dtype=np.float64))))

    def record(self):
        self._check(self.lib.citcom_nn_record(self.h))

    def train(self, steps: int, batch: int = 4, lr: float = 1e-3) -> float:
        loss = ctypes.c_double()
        self._check(self.lib.citcom_nn_train(self.h, steps, batch, lr, ctypes.byref(loss)))
        return loss.value

    def set_check_interval(self, every: int):
        """Compare the network's start with the resident one on every
        `every`-th solve (1: always; see citcom_nn_set_check_interval)."""
        self._check(self.lib.citcom_nn_set_check_interval(self.h, int(every)))

    def attach(self, on: bool = True):
        self._check(self.lib.citcom_nn_attach(self.h, int(on)))

    def predict(self):
        f = self.solver.fine
        U, P = np.zeros(f["neq"]), np.zeros(f["nel"])
        self._check(self.lib.citcom_nn_predict(self.h, _dp(U), _dp(P)))
        return U, P

    def forward(self, x: np.ndarray) -> np.ndarray:
        """x: (V, 2) float32 scaled inputs -> (V, 4) scaled outputs."""
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(self.voxels, 2)
        y = np.zeros((self.voxels, 4), dtype=np.float32)
        self._check(self.lib.citcom_nn_forward(self.h, _fp(x), _fp(y)))
        return y

    def loss_grad(self, x: np.ndarray, t: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(self.voxels, 2)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(self.voxels, 4)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.citcom_nn_loss_grad(self.h, _fp(x), _fp(t), ctypes.byref(loss), _fp(g)))
        return loss.value, g
