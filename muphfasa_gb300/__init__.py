"""muphfasa_gb300 -- GB300-native lattice-Boltzmann time step.

Python binding of the C ABI in ``include/mph.h`` (the library itself is C++
and sm_103a CUDA, built in-tree into ``muphfasa_gb300/_build/libmph.so``).
The classes mirror the reference solver's host interface:

* :class:`InputParser` -- the inputs file (ParmParse format, ``key=value``
  overrides; reference src/IO/InputParser.cpp).
* :func:`make_simulation` -- ``makeSimulation`` (SimulationFactory.cpp:36-60).
* :class:`Simulation` -- ``ISimulation`` (ISimulation.H:16-44): ``initialize``,
  ``advance``, ``update_macroscopic``, ``f``, ``rho``, ``vel``, ``time``,
  ``omega``.

There is no CPU fallback: if the compiled library is missing or no CUDA
device is present the calls raise.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libmph.so")

MPH_OK = 0
ERRORS = {1: "MPH_ERR_ARG", 2: "MPH_ERR_CONFIG", 3: "MPH_ERR_CUDA", 4: "MPH_ERR_UNSUPPORTED",
          5: "MPH_ERR_PARSE", 6: "MPH_ERR_NONFINITE", 7: "MPH_ERR_STATE"}
BC = {"MovingWall": 0, "NoSlip": 1, "Inflow": 2, "Outflow": 3, "PressureOutlet": 4, "Periodic": 5}
PRECISION = {"f64": 0, "f64_fast": 1, "f32": 2, "f16s": 3, "bf16s": 4, "f64x": 5, "f16c": 6, "f16w": 7}
LATTICE_DQ = {"D2Q9": (2, 9), "D3Q15": (3, 15), "D3Q19": (3, 19), "D3Q27": (3, 27)}

# Exported entry points (the declarations of include/mph.h).
EXPORTS = [
    "mph_last_error", "mph_abi_version", "mph_set_device", "mph_inputs_load", "mph_inputs_parse_string", "mph_inputs_free",
    "mph_inputs_get", "mph_inputs_derive", "mph_resolve_bc", "mph_create", "mph_destroy", "mph_set_f",
    "mph_get_f", "mph_init_fields", "mph_advance", "mph_update_macroscopic", "mph_reduce", "mph_time",
    "mph_launches_per_step", "mph_advance_timed", "mph_step_host", "mph_pull_collide_fused_arr",
    "mph_periodic_fill_arr", "mph_bc_fill_arr", "mph_reduce_f64_noalloc", "mph_pull_copy_timed", "mph_pipe_rate", "mph_batch_create",
    "mph_batch_destroy", "mph_batch_init_fields", "mph_batch_advance", "mph_batch_advance_timed",
    "mph_batch_advance_looped_timed", "mph_batch_get_f", "mph_batch_set_f", "mph_batch_moments", "mph_batch_info",
    "mph_residual", "mph_batch_residual", "mph_batch_range_flags", "mph_lattice", "mph_set_obstacles", "mph_batch_set_obstacles",
    "mph_init_fields_neq", "mph_batch_init_fields_neq", "mph_set_time", "mph_state_bytes", "mph_get_state",
    "mph_set_state", "mph_host_alloc", "mph_host_free", "mph_nn_alloc", "mph_nn_free", "mph_nn_copy", "mph_nn_sync", "mph_nn_gemm", "mph_nn_im2col3", "mph_nn_col2im3",
    "mph_nn_bias_act", "mph_nn_act_bwd", "mph_nn_colsum", "mph_nn_pool", "mph_nn_pool_bwd", "mph_nn_up",
    "mph_nn_up_bwd", "mph_nn_slice", "mph_nn_mse", "mph_nn_adam", "mph_nn_cast", "mph_nn_fill",
    "mph_nn_gemm_mode", "mph_nn_status", "mph_nn_sumsq", "mph_nn_transpose", "mph_nn_wflip", "mph_nn_conv3",
]


class MphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Desc(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("q", C.c_int), ("n", C.c_int * 3), ("omega", C.c_double), ("forced", C.c_int),
        ("force", C.c_double * 3), ("face_type", C.c_int * 6), ("face_rho", C.c_double * 6),
        ("face_U", (C.c_double * 3) * 6), ("precision", C.c_int),
    ]


class ResolvedBC(C.Structure):
    _fields_ = [("type", C.c_int), ("rho", C.c_double), ("U", C.c_double * 3)]


class RunInfo(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("dx", "dt", "u_lat", "nu_lat", "tau", "omega", "Re", "nu_phys",
                                           "ref_length", "ref_velocity", "ref_density")] + [
        ("max_step", C.c_int), ("stop_time", C.c_double), ("plot_int", C.c_int), ("chk_int", C.c_int)]


class Array4(C.Structure):
    _fields_ = [("p", C.c_void_p), ("jstride", C.c_longlong), ("kstride", C.c_longlong),
                ("nstride", C.c_longlong), ("begin", C.c_int * 3), ("end", C.c_int * 3), ("ncomp", C.c_int)]


_lib = None


def lib():
    """Loads libmph.so (building it first if only the sources are present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    L = C.CDLL(LIB_PATH)
    P, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.mph_last_error.restype = C.c_char_p
    L.mph_abi_version.restype = C.c_int
    L.mph_set_device.argtypes = [C.c_int]
    L.mph_inputs_load.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(P)]
    L.mph_inputs_parse_string.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(P)]
    L.mph_inputs_free.argtypes = [P]
    L.mph_inputs_free.restype = None
    L.mph_inputs_get.argtypes = [P, C.c_char_p, C.c_char_p, C.c_size_t]
    L.mph_inputs_derive.argtypes = [P, C.c_int, C.POINTER(Desc), C.POINTER(RunInfo)]
    L.mph_resolve_bc.argtypes = [C.POINTER(Desc), C.POINTER(ResolvedBC)]
    L.mph_create.argtypes = [C.POINTER(Desc), C.POINTER(P)]
    L.mph_destroy.argtypes = [P]
    L.mph_set_f.argtypes = [P, dp]
    L.mph_get_f.argtypes = [P, dp]
    L.mph_init_fields.argtypes = [P, dp, dp]
    L.mph_advance.argtypes = [P, C.c_int]
    L.mph_update_macroscopic.argtypes = [P, dp, dp]
    L.mph_reduce.argtypes = [P, dp]
    L.mph_residual.argtypes = [P, dp]
    L.mph_set_time.argtypes = [P, C.c_double]
    L.mph_host_alloc.argtypes = [C.c_longlong, C.POINTER(C.c_void_p)]
    L.mph_host_free.argtypes = [C.c_void_p]
    L.mph_state_bytes.argtypes = [P, C.POINTER(C.c_longlong)]
    L.mph_get_state.argtypes = [P, C.c_void_p, C.c_longlong]
    L.mph_set_state.argtypes = [P, C.c_void_p, C.c_longlong]
    L.mph_init_fields_neq.argtypes = [P, dp, dp]
    L.mph_batch_init_fields_neq.argtypes = [P, C.c_int, dp, dp]
    L.mph_set_obstacles.argtypes = [P, C.c_void_p]
    L.mph_batch_set_obstacles.argtypes = [P, C.c_int, C.c_void_p]
    L.mph_lattice.argtypes = [C.c_int, C.POINTER(C.c_int), dp, C.POINTER(C.c_int)]
    L.mph_batch_residual.argtypes = [P, dp]
    L.mph_time.argtypes = [P, dp]
    L.mph_launches_per_step.argtypes = [P, ip]
    L.mph_advance_timed.argtypes = [P, C.c_int, C.POINTER(C.c_float)]
    L.mph_step_host.argtypes = [P, dp, dp, C.c_int]
    L.mph_pull_collide_fused_arr.argtypes = [C.c_int, C.c_int, ip, ip, C.POINTER(Array4), C.POINTER(Array4),
                                             C.c_double, dp, P]
    L.mph_periodic_fill_arr.argtypes = [C.c_int, C.c_int, ip, ip, ip, C.POINTER(Array4), P]
    L.mph_bc_fill_arr.argtypes = [C.c_int, C.c_int, ip, ip, ip, C.POINTER(ResolvedBC), C.POINTER(Array4), P]
    L.mph_reduce_f64_noalloc.argtypes = [C.c_int, C.c_int, P, C.c_longlong, P, P]
    L.mph_pull_copy_timed.argtypes = [C.c_int] * 7 + [C.POINTER(C.c_float)]
    L.mph_pipe_rate.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.mph_batch_range_flags.argtypes = [P, C.POINTER(C.c_int)]
    L.mph_batch_create.argtypes = [C.c_int, C.POINTER(Desc), C.POINTER(P)]
    L.mph_batch_destroy.argtypes = [P]
    L.mph_batch_init_fields.argtypes = [P, C.c_int, dp, dp]
    L.mph_batch_advance.argtypes = [P, C.c_int]
    L.mph_batch_advance_timed.argtypes = [P, C.c_int, C.POINTER(C.c_float)]
    L.mph_batch_advance_looped_timed.argtypes = [P, C.c_int, C.POINTER(C.c_float)]
    L.mph_batch_get_f.argtypes = [P, C.c_int, dp]
    L.mph_batch_set_f.argtypes = [P, C.c_int, dp]
    L.mph_batch_moments.argtypes = [P, C.c_int, dp, dp]
    L.mph_batch_info.argtypes = [P, C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int)]
    _lib = L
    return L


def check(rc: int):
    if rc != MPH_OK:
        raise MphError(rc, lib().mph_last_error().decode(errors="replace"))


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def lattice_tables(lattice: str):
    """(c [q, 3] int, w [q] float64, opp [q] int) of a velocity set, from the library."""
    q = LATTICE_DQ[lattice][1]
    c = (C.c_int * (3 * q))()
    w = np.zeros(q)
    opp = (C.c_int * q)()
    check(lib().mph_lattice(q, c, _dp(w), opp))
    return np.array(list(c), dtype=np.int64).reshape(q, 3), w, np.array(list(opp), dtype=np.int64)


class PinnedArray:
    """A float64 NumPy array in page-locked host memory (mph_host_alloc)."""

    def __init__(self, n: int):
        self._p = C.c_void_p()
        check(lib().mph_host_alloc(C.c_longlong(8 * int(n)), C.byref(self._p)))
        self.array = np.ctypeslib.as_array((C.c_double * int(n)).from_address(self._p.value))

    def close(self):
        if getattr(self, "_p", None) is not None and self._p.value:
            self.array = None
            lib().mph_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pull_copy_ms(elem_bytes, mode, q, n, reps=20):
    """Mean milliseconds of one pull-stencil copy pass (the step's memory
    pattern without its arithmetic) on an n = (nx, ny[, nz]) periodic grid."""
    nn = list(n) + [1] * (3 - len(n))
    ms = C.c_float()
    check(lib().mph_pull_copy_timed(int(elem_bytes), int(mode), int(q), int(nn[0]), int(nn[1]), int(nn[2]), int(reps),
                                    C.byref(ms)))
    return float(ms.value)


def pipe_rate(op):
    """Operations per second of one arithmetic pipe (mph_pipe_rate): 0 DFMA,
    1 FFMA, 2 IMAD, 3 64-bit high multiply + add, 4 int64 -> FP64 + add."""
    r = C.c_double()
    check(lib().mph_pipe_rate(int(op), C.byref(r)))
    return float(r.value)


def make_desc(lattice: str, n, omega: float, faces=None, face_rho=None, face_U=None, force=None,
              precision: str = "f64") -> Desc:
    """A lattice-unit domain description (what SimulationImpl's constructor derives)."""
    dim, q = LATTICE_DQ[lattice]
    d = Desc()
    d.dim, d.q = dim, q
    nn = list(n) + [1] * (3 - len(n))
    for i in range(3):
        d.n[i] = int(nn[i])
    d.omega = float(omega)
    d.forced = 1 if force is not None else 0
    F = list(force or (0.0, 0.0, 0.0)) + [0.0] * 3
    for i in range(3):
        d.force[i] = float(F[i])
    faces = faces or ["Periodic"] * 6
    face_rho = face_rho or [1.0] * 6
    face_U = face_U or [[0.0, 0.0, 0.0]] * 6
    for i in range(6):
        d.face_type[i] = BC[faces[i]] if isinstance(faces[i], str) else int(faces[i])
        d.face_rho[i] = float(face_rho[i])
        for c in range(3):
            d.face_U[i][c] = float(face_U[i][c])
    d.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
    return d


def set_device(device: int):
    """Device for handles created afterwards on this thread (one per rank)."""
    check(lib().mph_set_device(int(device)))


def resolve_bc(desc: Desc):
    tab = (ResolvedBC * 27)()
    check(lib().mph_resolve_bc(C.byref(desc), tab))
    return [(t.type, t.rho, tuple(t.U)) for t in tab]


class InputParser:
    """An inputs file plus ``key=value`` overrides (amrex::Initialize(argc, argv))."""

    def __init__(self, path: str | None = None, overrides=(), text: str | None = None):
        L = lib()
        arr = (C.c_char_p * max(1, len(overrides)))(*[o.encode() for o in overrides])
        h = C.c_void_p()
        if text is not None:
            check(L.mph_inputs_parse_string(text.encode(), len(overrides), arr, C.byref(h)))
        else:
            check(L.mph_inputs_load(path.encode() if path else None, len(overrides), arr, C.byref(h)))
        self._h = h

    def __del__(self):
        try:
            if self._h:
                lib().mph_inputs_free(self._h)
                self._h = None
        except Exception:
            pass

    def get(self, key: str) -> str | None:
        buf = C.create_string_buffer(4096)
        rc = lib().mph_inputs_get(self._h, key.encode(), buf, 4096)
        return buf.value.decode() if rc == MPH_OK else None

    def derive(self, precision: str = "f64"):
        d, info = Desc(), RunInfo()
        p = PRECISION[precision] if isinstance(precision, str) else int(precision)
        check(lib().mph_inputs_derive(self._h, p, C.byref(d), C.byref(info)))
        return d, info


class Simulation:
    """Device-resident domain advanced by the sm_103a kernels (the ISimulation surface)."""

    def __init__(self, desc: Desc, info: RunInfo | None = None):
        self.desc = desc
        self.info = info
        self.dim, self.q = desc.dim, desc.q
        self.shape = (desc.n[2], desc.n[1], desc.n[0]) if desc.dim == 3 else (desc.n[1], desc.n[0])
        self.ncell = int(np.prod(self.shape))
        h = C.c_void_p()
        check(lib().mph_create(C.byref(desc), C.byref(h)))
        self._h = h
        self._rho = np.ones(self.ncell)
        self._vel = np.zeros(self.dim * self.ncell)

    def close(self):
        if getattr(self, "_h", None):
            lib().mph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- lifecycle ---------------------------------------------------------
    def initialize(self, rho=None, u=None):
        """setInitialConditions from (rho, u) (quiescent by default, InitData.cpp:8-15)."""
        rho = np.ones(self.ncell) if rho is None else np.ascontiguousarray(rho, dtype=np.float64).reshape(-1).copy()
        u = np.zeros(self.dim * self.ncell) if u is None else np.ascontiguousarray(u, dtype=np.float64).reshape(-1).copy()
        assert rho.size == self.ncell and u.size == self.dim * self.ncell
        check(lib().mph_init_fields(self._h, _dp(rho), _dp(u)))
        self._rho, self._vel = rho, u
        return rho, u

    def initialize_neq(self, rho, u):
        """Warm start: f = feq(rho, u) + the first-order non-equilibrium part
        from grad u (unforced domains)."""
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        assert rho.size == self.ncell and u.size == self.dim * self.ncell
        check(lib().mph_init_fields_neq(self._h, _dp(rho), _dp(u)))

    def advance(self, nsteps: int = 1):
        check(lib().mph_advance(self._h, int(nsteps)))

    def advance_timed(self, nsteps: int) -> float:
        ms = C.c_float()
        check(lib().mph_advance_timed(self._h, int(nsteps), C.byref(ms)))
        return float(ms.value)

    def step_host(self, f_in: np.ndarray, f_out: np.ndarray, nsteps: int = 1):
        check(lib().mph_step_host(self._h, _dp(f_in), _dp(f_out), int(nsteps)))

    def update_macroscopic(self):
        rho = np.empty(self.ncell)
        u = np.empty(self.dim * self.ncell)
        check(lib().mph_update_macroscopic(self._h, _dp(rho), _dp(u)))
        self._rho, self._vel = rho, u
        return rho, u

    # -- state -------------------------------------------------------------
    def set_f(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        assert f.size == self.q * self.ncell
        check(lib().mph_set_f(self._h, _dp(f)))

    def f(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.q * self.ncell)
        assert out.size == self.q * self.ncell
        check(lib().mph_get_f(self._h, _dp(out)))
        return out

    def rho(self):
        return self._rho

    def vel(self):
        return self._vel

    def reduce(self):
        out = np.zeros(4)
        check(lib().mph_reduce(self._h, _dp(out)))
        return out

    def set_obstacles(self, mask):
        """Interior obstacles: mask of N cells (x fastest), nonzero = solid;
        None removes them."""
        if mask is None:
            check(lib().mph_set_obstacles(self._h, None))
            return
        m = np.ascontiguousarray(np.asarray(mask, dtype=np.uint8).ravel())
        if m.size != self.ncell:
            raise ValueError(f"mask has {m.size} cells, the domain {self.ncell}")
        check(lib().mph_set_obstacles(self._h, m.ctypes.data))

    def residual(self):
        """(||u - u_prev|| / ||u||, ||u||) of the stored-population velocity
        against the previous call (inf on the first call after an init)."""
        out = np.zeros(2)
        check(lib().mph_residual(self._h, _dp(out)))
        return float(out[0]), float(out[1])

    def time(self) -> float:
        t = C.c_double()
        check(lib().mph_time(self._h, C.byref(t)))
        return t.value

    def omega(self) -> float:
        return self.desc.omega

    def launches_per_step(self) -> int:
        n = C.c_int()
        check(lib().mph_launches_per_step(self._h, C.byref(n)))
        return n.value


class Batch:
    """Independent domains of uneven sizes advanced together (mph_batch_*)."""

    def __init__(self, descs):
        self.descs = list(descs)
        arr = (Desc * len(self.descs))(*self.descs)
        h = C.c_void_p()
        check(lib().mph_batch_create(len(self.descs), arr, C.byref(h)))
        self._h = h
        self.ncells = [int(d.n[0] * d.n[1] * (d.n[2] if d.dim == 3 else 1)) for d in self.descs]

    def close(self):
        if getattr(self, "_h", None):
            lib().mph_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self, domain, rho=None, u=None):
        d, N = self.descs[domain], self.ncells[domain]
        rho = np.ones(N) if rho is None else np.ascontiguousarray(rho, dtype=np.float64).reshape(-1).copy()
        u = np.zeros(d.dim * N) if u is None else np.ascontiguousarray(u, dtype=np.float64).reshape(-1).copy()
        check(lib().mph_batch_init_fields(self._h, int(domain), _dp(rho), _dp(u)))
        return rho, u

    def initialize_neq(self, domain, rho, u):
        """Warm start of one domain, as Simulation.initialize_neq."""
        d, N = self.descs[domain], self.ncells[domain]
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        assert rho.size == N and u.size == d.dim * N
        check(lib().mph_batch_init_fields_neq(self._h, int(domain), _dp(rho), _dp(u)))

    def advance(self, nsteps=1):
        check(lib().mph_batch_advance(self._h, int(nsteps)))

    def advance_timed(self, nsteps):
        ms = C.c_float()
        check(lib().mph_batch_advance_timed(self._h, int(nsteps), C.byref(ms)))
        return float(ms.value)

    def advance_looped_timed(self, nsteps):
        ms = C.c_float()
        check(lib().mph_batch_advance_looped_timed(self._h, int(nsteps), C.byref(ms)))
        return float(ms.value)

    def f(self, domain):
        out = np.empty(self.descs[domain].q * self.ncells[domain])
        check(lib().mph_batch_get_f(self._h, int(domain), _dp(out)))
        return out

    def set_f(self, domain, f):
        """Replaces one domain's populations (FP64, valid-cell SoA)."""
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        assert f.size == self.descs[domain].q * self.ncells[domain]
        check(lib().mph_batch_set_f(self._h, int(domain), _dp(f)))

    def moments(self, domain):
        N, dim = self.ncells[domain], self.descs[domain].dim
        rho, u = np.empty(N), np.empty(dim * N)
        check(lib().mph_batch_moments(self._h, int(domain), _dp(rho), _dp(u)))
        return rho, u

    def set_obstacles(self, domain, mask):
        """Obstacles of one domain, as Simulation.set_obstacles."""
        if mask is None:
            check(lib().mph_batch_set_obstacles(self._h, int(domain), None))
            return
        m = np.ascontiguousarray(np.asarray(mask, dtype=np.uint8).ravel())
        if m.size != self.ncells[domain]:
            raise ValueError(f"mask has {m.size} cells, domain {domain} {self.ncells[domain]}")
        check(lib().mph_batch_set_obstacles(self._h, int(domain), m.ctypes.data))

    def residual(self):
        """Per-domain (relative change, norm) arrays, as Simulation.residual."""
        out = np.zeros(2 * len(self.descs))
        check(lib().mph_batch_residual(self._h, _dp(out)))
        return out[0::2].copy(), out[1::2].copy()

    def range_flags(self):
        """Per-domain flags of a fixed-point batch: True where the domain's
        populations left the representable range (mph_batch_range_flags)."""
        out = (C.c_int * len(self.descs))()
        check(lib().mph_batch_range_flags(self._h, out))
        return np.array(out[:], dtype=bool)

    def info(self):
        """(total cells, cells per thread, chunks per step, persistent grid) of
        the launch the autotuner chose (zeros before the first advance)."""
        tc, tw, nt, pe = C.c_longlong(), C.c_int(), C.c_int(), C.c_int()
        check(lib().mph_batch_info(self._h, C.byref(tc), C.byref(tw), C.byref(nt), C.byref(pe)))
        return int(tc.value), int(tw.value), int(nt.value), bool(pe.value)


def cavity_batch_descs(n_domains=512, seed=20261203, lattice="D2Q9", precision="f32", lid=0.1,
                       side=(64, 512), re=(100.0, 5000.0)):
    """The uneven lid-driven-cavity ensemble: side and Reynolds number drawn
    log-uniformly (seeded), tau = 0.5 + 3 lid side / Re; draws with tau
    outside (0.5, 2) are redrawn.  MovingWall lid at y = hi, NoSlip elsewhere."""
    rng = np.random.default_rng(seed)
    descs = []
    while len(descs) < n_domains:
        n = int(round(math.exp(rng.uniform(math.log(side[0]), math.log(side[1])))))
        Re = math.exp(rng.uniform(math.log(re[0]), math.log(re[1])))
        tau = 0.5 + 3.0 * lid * n / Re
        if not (0.5 < tau < 2.0):
            continue
        U = [[0.0] * 3 for _ in range(6)]
        U[3] = [lid, 0.0, 0.0]
        descs.append(make_desc(lattice, (n, n), 1.0 / tau,
                               faces=["NoSlip", "NoSlip", "NoSlip", "MovingWall", "Periodic", "Periodic"],
                               face_U=U, precision=precision))
    return descs


def make_simulation(inputs: InputParser, precision: str = "f64") -> Simulation:
    """makeSimulation (SimulationFactory.cpp:36-60): lattice/collision dispatch from the inputs."""
    d, info = inputs.derive(precision)
    return Simulation(d, info)
