"""CPU oracle for the lattice-Boltzmann step -- TEST INFRASTRUCTURE ONLY.

This module is the checker used by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline arm of ``bench.py``.  The product (``muphfasa_gb300``) never
imports it.

Two interchangeable back ends share the C interface of ``oracle_api.h``:

* ``liboracle.so`` -- ``lbm_oracle.cpp``, a C++ restatement of the reference's
  CPU path (src/LBM/Collision.cpp:18-143, BoundaryConditions.H:124-189,
  BCTypes/*.H, Macroscopic.cpp, Equilibrium.cpp, Units.cpp, SimulationSetup.cpp
  :120-299) with the reference's operation order, built with
  ``-ffp-contract=off`` so that it is bit-identical to the reference.
* ``_ref/libmphref{2,3}d.so`` -- the reference's own LBM sources compiled
  against a project-written AMReX stand-in (``build_ref.sh``); only available
  where the reference sources are.  Used to pin the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

BC = {"MovingWall": 0, "NoSlip": 1, "Inflow": 2, "Outflow": 3, "PressureOutlet": 4, "Periodic": 5}
LATTICE_DQ = {"D2Q9": (2, 9), "D3Q15": (3, 15), "D3Q19": (3, 19), "D3Q27": (3, 27)}


class OrcDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("q", C.c_int), ("n", C.c_int * 3), ("omega", C.c_double),
        ("forced", C.c_int), ("F", C.c_double * 3), ("face_type", C.c_int * 6),
        ("face_rho", C.c_double * 6), ("face_U", (C.c_double * 3) * 6),
    ]


class OrcUnitsIn(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("ncells", C.c_int * 3), ("prob_lo", C.c_double * 3),
        ("prob_hi", C.c_double * 3), ("ref_length", C.c_double), ("ref_velocity", C.c_double),
        ("ref_density", C.c_double), ("has_Re", C.c_int), ("Re", C.c_double),
        ("has_nu", C.c_int), ("nu_phys", C.c_double), ("has_u_lat", C.c_int),
        ("u_lat", C.c_double), ("has_tau", C.c_int), ("tau", C.c_double),
    ]


class OrcUnitsOut(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("dx", "dt", "u_lat", "nu_lat", "tau", "omega", "Re", "nu_phys")]


def build(verbose: bool = False) -> str:
    """Compiles lbm_oracle.cpp into _build/liboracle.so (host compiler, OpenMP)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "lbm_oracle.cpp")
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle_api.h"))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", tmp, src]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


# Root of a reference checkout: the MPH_REFERENCE_ROOT environment variable,
# else the default of build_ref.sh.  Hosts without a checkout build the copy
# of its src/LBM that build_ref.sh stages under baseline/_ref/.
REFERENCE_ROOT = os.environ.get("MPH_REFERENCE_ROOT") or "/root/reference"
STAGED_SRC = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "src")


def build_ref() -> bool:
    """Builds oracle/_ref from the reference sources (the checkout, else the
    staged copy) when either is present; True when the libraries exist."""
    srcs = [os.path.join(REFERENCE_ROOT, "src", "LBM", "Collision.cpp"),
            os.path.join(STAGED_SRC, "LBM", "Collision.cpp")]
    if not any(os.path.exists(p) for p in srcs):
        return ref_available()
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT], check=True, capture_output=True)
    return ref_available()


def ref_available() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, f"libmphref{d}d.so")) for d in (2, 3))


def _bind(lib):
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    lib.orc_create.restype = P
    lib.orc_create.argtypes = [C.POINTER(OrcDesc)]
    lib.orc_destroy.argtypes = [P]
    lib.orc_ncells.restype = C.c_longlong
    lib.orc_ncells.argtypes = [P]
    lib.orc_nghost_cells.restype = C.c_longlong
    lib.orc_nghost_cells.argtypes = [P]
    for name in ("orc_set_f", "orc_get_f", "orc_set_f_ghost", "orc_get_f_ghost"):
        getattr(lib, name).argtypes = [P, dp]
    lib.orc_fill_ghosts.argtypes = [P]
    lib.orc_step.argtypes = [P, C.c_int, C.c_int]
    lib.orc_init_fields.argtypes = [P, dp, dp]
    lib.orc_moments.argtypes = [P, dp, dp]
    if hasattr(lib, "orc_set_obstacles"):  # the restatement only (no reference counterpart)
        lib.orc_set_obstacles.argtypes = [P, C.c_void_p]
    lib.orc_units.argtypes = [C.POINTER(OrcUnitsIn), C.POINTER(OrcUnitsOut), C.c_int, dp, dp,
                              C.c_int, dp, dp, C.c_int, dp, dp]
    lib.orc_resolve_bc.argtypes = [C.POINTER(OrcDesc), C.POINTER(C.c_int), dp, dp]
    return lib


_LIBS: dict = {}


def load(kind: str = "port", dim: int = 3):
    """kind 'port' -> restated oracle; 'ref' -> reference build for `dim`."""
    key = (kind, dim if kind == "ref" else 0)
    if key not in _LIBS:
        if kind == "port":
            path = build()
        else:
            path = os.path.join(REF_DIR, f"libmphref{dim}d.so")
        _LIBS[key] = _bind(C.CDLL(path))
    return _LIBS[key]


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class Config:
    """Lattice-unit description of one domain (what the reference derives in
    SimulationImpl's constructor, SimulationSetup.cpp:32-89)."""
    lattice: str
    n: tuple
    omega: float
    faces: list = field(default_factory=lambda: ["Periodic"] * 6)  # xlo,xhi,ylo,yhi,zlo,zhi
    face_rho: list = field(default_factory=lambda: [1.0] * 6)
    face_U: list = field(default_factory=lambda: [[0.0, 0.0, 0.0] for _ in range(6)])
    force: tuple | None = None

    @property
    def dim(self):
        return LATTICE_DQ[self.lattice][0]

    @property
    def q(self):
        return LATTICE_DQ[self.lattice][1]

    @property
    def ncells(self):
        n = list(self.n) + [1] * (3 - len(self.n))
        return n[0] * n[1] * n[2]

    def desc(self) -> OrcDesc:
        d = OrcDesc()
        d.dim, d.q = self.dim, self.q
        n = list(self.n) + [1] * (3 - len(self.n))
        for i in range(3):
            d.n[i] = int(n[i])
        d.omega = float(self.omega)
        d.forced = 1 if self.force is not None else 0
        F = list(self.force or (0.0, 0.0, 0.0)) + [0.0] * 3
        for i in range(3):
            d.F[i] = float(F[i])
        for i in range(6):
            d.face_type[i] = BC[self.faces[i]] if isinstance(self.faces[i], str) else int(self.faces[i])
            d.face_rho[i] = float(self.face_rho[i])
            for c in range(3):
                d.face_U[i][c] = float(self.face_U[i][c])
        return d


class OracleSim:
    """One domain advanced by the oracle (or the reference build)."""

    def __init__(self, cfg: Config, kind: str = "port"):
        self.cfg = cfg
        self.lib = load(kind, cfg.dim)
        self._desc = cfg.desc()
        self.h = self.lib.orc_create(C.byref(self._desc))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        self.N = int(self.lib.orc_ncells(self.h))
        self.G = int(self.lib.orc_nghost_cells(self.h))

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_f(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        assert f.size == self.cfg.q * self.N
        self.lib.orc_set_f(self.h, _dptr(f))

    def get_f(self) -> np.ndarray:
        out = np.empty(self.cfg.q * self.N, dtype=np.float64)
        self.lib.orc_get_f(self.h, _dptr(out))
        return out

    def get_f_ghost(self) -> np.ndarray:
        out = np.empty(self.cfg.q * self.G, dtype=np.float64)
        self.lib.orc_get_f_ghost(self.h, _dptr(out))
        return out

    def set_f_ghost(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        assert f.size == self.cfg.q * self.G
        self.lib.orc_set_f_ghost(self.h, _dptr(f))

    def fill_ghosts(self):
        if self.lib.orc_fill_ghosts(self.h) != 0:
            raise RuntimeError("oracle ghost fill failed")

    def step(self, nsteps: int, nthreads: int = 1):
        if self.lib.orc_step(self.h, int(nsteps), int(nthreads)) != 0:
            raise RuntimeError("oracle step failed")

    def init_fields(self, rho: np.ndarray, u: np.ndarray):
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1).copy()
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1).copy()
        assert rho.size == self.N and u.size == self.cfg.dim * self.N
        if self.lib.orc_init_fields(self.h, _dptr(rho), _dptr(u)) != 0:
            raise RuntimeError("oracle init failed")
        return rho, u

    def set_obstacles(self, mask):
        """Interior obstacles (project-defined rule, restatement only): mask
        is N booleans, x fastest; None removes them."""
        if mask is None:
            self.lib.orc_set_obstacles(self.h, None)
            return
        m = np.ascontiguousarray(np.asarray(mask, dtype=np.uint8).ravel())
        assert m.size == self.N
        self.lib.orc_set_obstacles(self.h, m.ctypes.data)

    def moments(self):
        rho = np.empty(self.N, dtype=np.float64)
        u = np.empty(self.cfg.dim * self.N, dtype=np.float64)
        if self.lib.orc_moments(self.h, _dptr(rho), _dptr(u)) != 0:
            raise RuntimeError("oracle moments failed")
        return rho, u


def resolve_bc(cfg: Config, kind: str = "port"):
    lib = load(kind, cfg.dim)
    d = cfg.desc()
    t = (C.c_int * 27)()
    r = np.zeros(27)
    U = np.zeros(81)
    rc = lib.orc_resolve_bc(C.byref(d), t, _dptr(r), _dptr(U))
    return rc, np.array(list(t), dtype=np.int32), r, U.reshape(27, 3)


def units(dim, ncells, prob_lo, prob_hi, ref_length=1.0, ref_velocity=1.0, ref_density=1.0,
          Re=None, nu_phys=None, u_lat=None, tau=None, accel=(), vel=(), rho=(), kind="port"):
    lib = load(kind, dim)
    ui = OrcUnitsIn()
    ui.dim = dim
    for i in range(dim):
        ui.ncells[i] = int(ncells[i])
        ui.prob_lo[i] = float(prob_lo[i])
        ui.prob_hi[i] = float(prob_hi[i])
    ui.ref_length, ui.ref_velocity, ui.ref_density = ref_length, ref_velocity, ref_density
    for name, val in (("Re", Re), ("nu", nu_phys), ("u_lat", u_lat), ("tau", tau)):
        if val is not None:
            setattr(ui, "has_" + name, 1)
            setattr(ui, {"nu": "nu_phys"}.get(name, name), float(val))
    uo = OrcUnitsOut()
    a_in = np.ascontiguousarray(accel, dtype=np.float64).reshape(-1)
    v_in = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
    r_in = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
    a_out, v_out, r_out = np.zeros_like(a_in), np.zeros_like(v_in), np.zeros_like(r_in)
    if a_in.size == 0:
        a_in = a_out = np.zeros(1)
        na = 0
    else:
        na = a_in.size
    if v_in.size == 0:
        v_in = v_out = np.zeros(1)
        nv = 0
    else:
        nv = v_in.size
    if r_in.size == 0:
        r_in = r_out = np.zeros(1)
        nr = 0
    else:
        nr = r_in.size
    rc = lib.orc_units(C.byref(ui), C.byref(uo), na, _dptr(a_in), _dptr(a_out), nv, _dptr(v_in),
                       _dptr(v_out), nr, _dptr(r_in), _dptr(r_out))
    res = {k: getattr(uo, k) for k, _ in OrcUnitsOut._fields_}
    res["accel_lat"] = a_out[:na].copy()
    res["vel_lat"] = v_out[:nv].copy()
    res["rho_lat"] = r_out[:nr].copy()
    return rc, res
