"""ctypes front end of the CPU restatement (liboracle.so) and a reader for the
records written by the reference driver (oracle/ref/oracle_main.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker or the timed CPU baseline,
never as part of the product path.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

MAXL = 12
MAXM = 8


class _Params(ctypes.Structure):
    _fields_ = [
        ("levels", ctypes.c_int),
        ("mgunit", ctypes.c_int * 3),
        ("dimen", ctypes.c_double * 3),
        ("rayleigh", ctypes.c_double),
        ("Q0", ctypes.c_double),
        ("tdepv", ctypes.c_int),
        ("num_mat", ctypes.c_int),
        ("visc0", ctypes.c_double * MAXM),
        ("viscE", ctypes.c_double * MAXM),
        ("viscT", ctypes.c_double * MAXM),
        ("z_layer", ctypes.c_double * MAXM),
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
        ("gs_colored", ctypes.c_int),
        ("sdepv", ctypes.c_int),
        ("sdepv_rheology", ctypes.c_int),
        ("sdepv_expt", ctypes.c_double * MAXM),
        ("sdepv_trns", ctypes.c_double * MAXM),
        ("sdepv_misfit", ctypes.c_double),
        ("sdepv_iter_damp", ctypes.c_double),
        ("max_sdep_visc_iter", ctypes.c_int),
        ("stop_rule", ctypes.c_int),
    ]


def build(quiet: bool = True) -> str:
    """Compile liboracle.so in place (plain gcc, no reference sources)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


# the unchanged reference's sources, where they exist: $CITCOM_REF_SRC, else
# the reference tree beside the repository (../reference/src); absent on hosts
# that only run the GPU library
REF_SRC = os.environ.get("CITCOM_REF_SRC") or os.path.normpath(os.path.join(HERE, "..", "..", "reference", "src"))


def build_reference(quiet: bool = True) -> bool:
    """Compile the unchanged reference into oracle/_ref when its sources are
    present (this container); returns False where they are absent."""
    if not os.path.isdir(REF_SRC):
        return False
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"), f"REF={REF_SRC}"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None,
                   stderr=subprocess.DEVNULL if quiet else None)
    return True


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        I = ctypes.POINTER(ctypes.c_int)
        L.oracle_create.restype = P
        L.oracle_create.argtypes = [ctypes.POINTER(_Params)]
        L.oracle_destroy.argtypes = [P]
        L.oracle_level_dims.argtypes = [P, ctypes.c_int, I]
        for nm in ["oracle_T", "oracle_Tdot", "oracle_U", "oracle_P", "oracle_F", "oracle_buoyancy"]:
            getattr(L, nm).restype = D
            getattr(L, nm).argtypes = [P]
        L.oracle_V.restype = D
        L.oracle_V.argtypes = [P, ctypes.c_int]
        for nm in ["oracle_EVI", "oracle_BI", "oracle_BPI", "oracle_stencil"]:
            getattr(L, nm).restype = D
            getattr(L, nm).argtypes = [P, ctypes.c_int]
        L.oracle_vflags.restype = ctypes.POINTER(ctypes.c_uint)
        L.oracle_vflags.argtypes = [P, ctypes.c_int]
        for nm in ["oracle_timestep", "oracle_elapsed_time", "oracle_T_interior"]:
            getattr(L, nm).restype = ctypes.c_double
            getattr(L, nm).argtypes = [P]
        L.oracle_set_timestep.argtypes = [P, ctypes.c_double]
        for nm in ["oracle_thermal_buoyancy", "oracle_assemble_forces", "oracle_get_system_viscosity",
                   "oracle_project_viscosity", "oracle_construct_stiffness", "oracle_pg_timestep"]:
            getattr(L, nm).argtypes = [P]
        L.oracle_kmul.argtypes = [P, ctypes.c_int, D, D, ctypes.c_int]
        L.oracle_strip_bcs.argtypes = [P, ctypes.c_int, D]
        L.oracle_gauss_seidel.argtypes = [P, ctypes.c_int, D, D, D, ctypes.c_int, ctypes.c_int]
        L.oracle_project_vector.argtypes = [P, ctypes.c_int, D, D]
        L.oracle_interp_vector.argtypes = [P, ctypes.c_int, D, D]
        L.oracle_div_u.argtypes = [P, ctypes.c_int, D, D]
        L.oracle_grad_p.argtypes = [P, ctypes.c_int, D, D]
        L.oracle_multi_grid.restype = ctypes.c_double
        L.oracle_multi_grid.argtypes = [P, D, D, ctypes.c_double]
        L.oracle_solve_del2_u.restype = ctypes.c_int
        L.oracle_solve_del2_u.argtypes = [P, D, D, ctypes.c_double, I]
        L.oracle_solve_Ahat_p_fhat.restype = ctypes.c_double
        L.oracle_solve_Ahat_p_fhat.argtypes = [P, D, D, D, ctypes.c_double, I, I, I]
        L.oracle_last_residuals.argtypes = [P, D]
        L.oracle_stokes.restype = ctypes.c_double
        L.oracle_stokes.argtypes = [P, I, I, I]
        L.oracle_heat_flux.argtypes = [P, D, D]
        L.oracle_vrms.restype = ctypes.c_double
        L.oracle_vrms.argtypes = [P]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def params_from_case(case, gs_colored: bool = False) -> _Params:
    p = _Params()
    p.levels = case.levels
    for i in range(3):
        p.mgunit[i] = case.mgunit[i]
        p.dimen[i] = case.dimen[i]
    p.rayleigh = case.rayleigh
    p.Q0 = case.Q0
    p.tdepv = int(case.tdepv)
    p.num_mat = len(case.visc0)
    for i in range(p.num_mat):
        p.visc0[i] = case.visc0[i]
        p.viscE[i] = case.viscE[i] if i < len(case.viscE) else 0.0
        p.viscT[i] = case.viscT[i] if i < len(case.viscT) else 0.0
    zl = list(case.z_layer) + [0.0] * (p.num_mat - len(case.z_layer))
    for i in range(p.num_mat):
        p.z_layer[i] = zl[i]
    p.vmin_on = int(case.vmin is not None)
    p.vmax_on = int(case.vmax is not None)
    p.vmin = case.vmin or 0.0
    p.vmax = case.vmax or 0.0
    p.aug_lagr = int(case.aug_lagr)
    p.aug_number = case.aug_number
    p.precond = int(case.precond)
    p.mg_cycle = case.mg_cycle
    p.down_heavy = case.down_heavy
    p.up_heavy = case.up_heavy
    p.vlowstep = case.vlowstep
    p.vhighstep = case.vhighstep
    p.piterations = case.piterations
    p.accuracy = case.accuracy
    p.adv_sub_iterations = case.adv_sub_iterations
    p.finetunedt = case.finetunedt
    p.fixed_timestep = case.fixed_timestep
    p.gs_colored = int(gs_colored)
    p.stop_rule = int(getattr(case, "stop_rule", 0))
    p.sdepv = int(getattr(case, "sdepv", False))
    if p.sdepv:
        p.sdepv_rheology = case.sdepv_rheology
        ex = (list(case.sdepv_expt) * p.num_mat)[:p.num_mat]
        tr = (list(case.sdepv_trns) * p.num_mat)[:p.num_mat]
        for i in range(p.num_mat):
            p.sdepv_expt[i] = ex[i]
            p.sdepv_trns[i] = tr[i]
        p.sdepv_misfit = case.sdepv_misfit
        p.sdepv_iter_damp = case.sdepv_iter_damp
        p.max_sdep_visc_iter = case.max_sdep_visc_iter
    return p


class Oracle:
    """One problem instance of the CPU restatement."""

    def __init__(self, case, gs_colored: bool = False):
        self.case = case
        self._p = params_from_case(case, gs_colored)
        self.h = lib().oracle_create(ctypes.byref(self._p))
        self.L = case.levels
        self.dims = []
        for l in range(self.L):
            d = (ctypes.c_int * 6)()
            lib().oracle_level_dims(self.h, l, d)
            self.dims.append(dict(nox=d[0], noy=d[1], noz=d[2], nno=d[3], nel=d[4], neq=d[5]))

    def __del__(self):
        try:
            if self.h:
                lib().oracle_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def _view(self, ptr, n):
        return np.ctypeslib.as_array(ptr, shape=(n,))

    @property
    def fine(self):
        return self.dims[-1]

    def T(self):
        return self._view(lib().oracle_T(self.h), self.fine["nno"])

    def Tdot(self):
        return self._view(lib().oracle_Tdot(self.h), self.fine["nno"])

    def U(self):
        return self._view(lib().oracle_U(self.h), self.fine["neq"] + 2)

    def P(self):
        return self._view(lib().oracle_P(self.h), self.fine["nel"])

    def F(self):
        return self._view(lib().oracle_F(self.h), self.fine["neq"] + 2)

    def V(self, d):
        return self._view(lib().oracle_V(self.h, d), self.fine["nno"])

    def buoyancy(self):
        return self._view(lib().oracle_buoyancy(self.h), self.fine["nno"])

    def EVI(self, lev):
        return self._view(lib().oracle_EVI(self.h, lev), self.dims[lev]["nel"] * 8)

    def BI(self, lev):
        return self._view(lib().oracle_BI(self.h, lev), self.dims[lev]["neq"])

    def BPI(self, lev):
        return self._view(lib().oracle_BPI(self.h, lev), self.dims[lev]["nel"])

    def vflags(self, lev):
        return np.ctypeslib.as_array(lib().oracle_vflags(self.h, lev), shape=(self.dims[lev]["nno"],))

    def stencil(self, lev):
        return self._view(lib().oracle_stencil(self.h, lev), self.dims[lev]["nno"] * 243)

    def set_T(self, T):
        self.T()[:] = T

    def thermal_buoyancy(self):
        lib().oracle_thermal_buoyancy(self.h)

    def assemble_forces(self):
        lib().oracle_assemble_forces(self.h)

    def viscosity(self):
        lib().oracle_get_system_viscosity(self.h)
        lib().oracle_project_viscosity(self.h)

    def construct_stiffness(self):
        lib().oracle_construct_stiffness(self.h)

    def setup_operators(self):
        """buoyancy, forces, viscosity on all levels, stiffness: everything
        general_stokes_solver prepares before the Uzawa solve."""
        self.thermal_buoyancy()
        self.assemble_forces()
        if self.case.tdepv:
            lib().oracle_get_system_viscosity(self.h)
        lib().oracle_project_viscosity(self.h)
        self.construct_stiffness()

    def kmul(self, lev, u, strip=True):
        neq = self.dims[lev]["neq"]
        uu = np.zeros(neq + 2)
        uu[:neq] = u[:neq]
        au = np.zeros(neq + 2)
        lib().oracle_kmul(self.h, lev, _dp(uu), _dp(au), int(strip))
        return au[:neq]

    def strip(self, lev, r):
        r = np.ascontiguousarray(r, dtype=np.float64).copy()
        lib().oracle_strip_bcs(self.h, lev, _dp(r))
        return r

    def gauss_seidel(self, lev, F, cycles, d0=None):
        neq = self.dims[lev]["neq"]
        f = np.zeros(neq + 2)
        f[:neq] = F[:neq]
        d = np.zeros(neq + 2)
        guess = 0
        if d0 is not None:
            d[:neq] = d0[:neq]
            guess = 1
        ad = np.zeros(neq + 2)
        lib().oracle_gauss_seidel(self.h, lev, _dp(d), _dp(f), _dp(ad), cycles, guess)
        return d[:neq], ad[:neq]

    def project(self, fine_lev, AU):
        neqc = self.dims[fine_lev - 1]["neq"]
        au = np.ascontiguousarray(AU, dtype=np.float64)
        ad = np.zeros(neqc + 2)
        lib().oracle_project_vector(self.h, fine_lev, _dp(au), _dp(ad))
        return ad[:neqc]

    def interp(self, coarse_lev, AD):
        neqf = self.dims[coarse_lev + 1]["neq"]
        ad = np.ascontiguousarray(AD, dtype=np.float64)
        au = np.zeros(neqf + 2)
        lib().oracle_interp_vector(self.h, coarse_lev, _dp(ad), _dp(au))
        return au[:neqf]

    def div(self, lev, U):
        u = np.ascontiguousarray(U, dtype=np.float64)
        out = np.zeros(self.dims[lev]["nel"])
        lib().oracle_div_u(self.h, lev, _dp(u), _dp(out))
        return out

    def grad(self, lev, P):
        p = np.ascontiguousarray(P, dtype=np.float64)
        out = np.zeros(self.dims[lev]["neq"] + 2)
        lib().oracle_grad_p(self.h, lev, _dp(p), _dp(out))
        return out[: self.dims[lev]["neq"]]

    def multi_grid(self, F, acc=1e-3):
        neq = self.fine["neq"]
        f = np.zeros(neq + 2)
        f[:neq] = F[:neq]
        d1 = np.zeros(neq + 2)
        r = lib().oracle_multi_grid(self.h, _dp(d1), _dp(f), acc)
        return d1[:neq], f[:neq], r

    def solve_del2_u(self, F, acc):
        neq = self.fine["neq"]
        f = np.zeros(neq + 2)
        f[:neq] = F[:neq]
        d0 = np.zeros(neq + 2)
        calls = ctypes.c_int(0)
        v = lib().oracle_solve_del2_u(self.h, _dp(d0), _dp(f), acc, ctypes.byref(calls))
        return d0[:neq], v, calls.value

    def solve_Ahat_p_fhat(self, imp, steps):
        """solve_Ahat_p_fhat on the oracle's own U, P, F (after setup_operators)."""
        st, c, m = ctypes.c_int(steps), ctypes.c_int(0), ctypes.c_int(0)
        r = lib().oracle_solve_Ahat_p_fhat(self.h, lib().oracle_U(self.h), lib().oracle_P(self.h),
                                           lib().oracle_F(self.h), imp, ctypes.byref(st), ctypes.byref(c),
                                           ctypes.byref(m))
        return dict(residual=r, uzawa=st.value, del2_calls=c.value, mg_calls=m.value, **self.last_residuals())

    def last_residuals(self):
        """The residual rule's final momentum and continuity residuals and
        velocity corrections of the last solve (zeros under the reference rule)."""
        out = np.zeros(3)
        lib().oracle_last_residuals(self.h, _dp(out))
        return dict(momentum=float(out[0]), continuity=float(out[1]), corrections=int(out[2]))

    def stokes(self):
        s, c, m = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        r = lib().oracle_stokes(self.h, ctypes.byref(s), ctypes.byref(c), ctypes.byref(m))
        return dict(residual=r, uzawa=s.value, del2_calls=c.value, mg_calls=m.value, **self.last_residuals())

    def pg_timestep(self):
        lib().oracle_pg_timestep(self.h)

    def heat_flux(self):
        a, b = ctypes.c_double(0), ctypes.c_double(0)
        lib().oracle_heat_flux(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def vrms(self):
        return lib().oracle_vrms(self.h)

    def timestep(self):
        return lib().oracle_timestep(self.h)

    def elapsed_time(self):
        return lib().oracle_elapsed_time(self.h)


def read_records(path: str) -> dict:
    """Records of oracle_main.c: 32-byte name, int64 count, count doubles."""
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    while off < len(data):
        name = data[off:off + 32].split(b"\0", 1)[0].decode()
        (n,) = struct.unpack_from("<q", data, off + 32)
        off += 40
        out[name] = np.frombuffer(data, dtype="<f8", count=n, offset=off).copy()
        off += 8 * n
    return out


def run_reference(case, workdir: str, nsteps: int, T0=None, probe: bool = False,
                  precision: str = "f64") -> dict:
    """Run the reference build (oracle/_ref/citcom_ref_<precision>) on `case`."""
    from .decks import make_deck
    os.makedirs(workdir, exist_ok=True)
    deck = os.path.join(workdir, "deck")
    with open(deck, "w") as f:
        f.write(make_deck(case, os.path.join(workdir, "case")))
    t0 = "-"
    if T0 is not None:
        t0 = os.path.join(workdir, "T0.bin")
        np.ascontiguousarray(T0, dtype="<f8").tofile(t0)
    out = os.path.join(workdir, "out.bin")
    exe = os.path.join(REF_DIR, f"citcom_ref_{precision}")
    cmd = [exe, deck, t0, str(nsteps), out] + (["probe"] if probe else [])
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return read_records(out)
