"""ctypes bindings to the oracle libraries — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this module, and only to check results against. Two libraries:

* ``RefSolver``   — oracle/_ref/libmifref.so: the reference's own sources
  compiled here against single-rank MPI / FFTW stand-ins (oracle/Makefile,
  target ``ref``). Exists only where the reference sources were present.
* ``OracleSolver`` — oracle/libmif_oracle.so: the plain-C restatement of the
  same algorithm (oracle/mif_oracle.c), buildable anywhere.

Both expose the reference's state (velocity, velocity_buffer,
velocity_buffer_2, pressure, pressure_buffer) as numpy arrays in the
reference's own layout: shape (Ez, Ey, Ex), x fastest (include/Tensor.h:237).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libmifref.so")
ORACLE_LIB = os.path.join(HERE, "libmif_oracle.so")
ORACLE_FAST_LIB = os.path.join(HERE, "libmif_oracle_fast.so")

FIELD_NAMES = ["u", "v", "w", "u1", "v1", "w1", "u2", "v2", "w2", "p", "phi"]
FIELD_ID = {n: i for i, n in enumerate(FIELD_NAMES)}

KIND_ZERO, KIND_SINCOS, KIND_ETHIER = 0, 1, 2


class Params(C.Structure):
    """Layout shared by mifref_params and mif_oracle_params."""

    _fields_ = [
        ("n_global", C.c_long * 3),
        ("size", C.c_double * 3),
        ("origin", C.c_double * 3),
        ("Re", C.c_double),
        ("dt", C.c_double),
        ("periodic", C.c_int * 3),
        ("exact_kind", C.c_int),
    ]


@dataclass
class Case:
    """Grid and physics of one run, in the reference's conventions.

    n_global follows include/Constants.h:14-16: for a periodic axis with N
    unique points it is N + 1; for a Dirichlet axis it counts every node
    including both walls.
    """

    n_global: tuple
    size: tuple = (1.0, 1.0, 1.0)
    origin: tuple = (0.0, 0.0, 0.0)
    Re: float = 1000.0
    dt: float = 1e-4
    periodic: tuple = (False, False, False)
    exact_kind: int = KIND_ZERO
    forcing: int = 0  # oracle restatement only: 0 none, 1 velocity forcing, 2 with grad p

    def params(self) -> Params:
        p = Params()
        for d in range(3):
            p.n_global[d] = int(self.n_global[d])
            p.size[d] = float(self.size[d])
            p.origin[d] = float(self.origin[d])
            p.periodic[d] = 1 if self.periodic[d] else 0
        p.Re = float(self.Re)
        p.dt = float(self.dt)
        p.exact_kind = int(self.exact_kind)
        return p

    def extents(self, name: str) -> tuple:
        """(Ex, Ey, Ez) of a field, src/Constants.cpp:80-88 and src/StaggeredTensor.cpp:6-9.

        With one rank the y and z staggered extents always gain a point
        (Ny_staggered = Ny + 1 even on a periodic axis); x only when not periodic.
        """
        base = [self.n_global[d] + 1 if self.periodic[d] else self.n_global[d] for d in range(3)]
        stag = {"u": 0, "v": 1, "w": 2}.get(name.rstrip("12"), None)
        if stag is not None and (stag > 0 or not self.periodic[stag]):
            base[stag] += 1
        return tuple(base)

    def cells(self) -> int:
        """Cells counted for throughput: intervals per axis."""
        return int(np.prod([n - 1 for n in self.n_global]))


def _load(path: str) -> C.CDLL:
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library not built: {path}")
    return C.CDLL(path)


class _Solver:
    prefix = ""
    lib_path = ""

    def __init__(self, case: Case):
        self.case = case
        self.lib = _load(self.lib_path)
        pre = self.prefix
        f = getattr(self.lib, pre + "create")
        f.restype = C.c_void_p
        f.argtypes = [C.POINTER(Params)]
        self._params = case.params()
        self.h = f(C.byref(self._params))
        if not self.h:
            raise RuntimeError("oracle create failed")
        for name in ("timestep", "timestep_nhn", "timestep_velocity", "adjust_pressure"):
            fn = getattr(self.lib, pre + name)
            fn.argtypes = [C.c_void_p, C.c_double]
            fn.restype = C.c_int
        for name in ("solve_pressure", "apply_bc", "project"):
            fn = getattr(self.lib, pre + name)
            fn.argtypes = [C.c_void_p, C.c_int, C.c_double]
            fn.restype = C.c_int
        getattr(self.lib, pre + "solve_pressure_nhn").argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double]
        getattr(self.lib, pre + "set").argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        getattr(self.lib, pre + "get").argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        getattr(self.lib, pre + "set_exact_velocity").argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int]
        getattr(self.lib, pre + "set_exact_pressure").argtypes = [C.c_void_p, C.c_double]
        getattr(self.lib, pre + "error_norms").argtypes = [C.c_void_p, C.c_double, C.c_void_p]
        getattr(self.lib, pre + "destroy").argtypes = [C.c_void_p]

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def close(self):
        if self.h:
            self._fn("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, name: str) -> tuple:
        ext = (C.c_long * 3)()
        fn = self._fn("extent")
        fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        assert fn(self.h, FIELD_ID[name], ext) == 0
        assert tuple(ext) == self.case.extents(name), (name, tuple(ext), self.case.extents(name))
        return (ext[2], ext[1], ext[0])

    def get(self, name: str) -> np.ndarray:
        out = np.empty(self.shape(name), dtype=np.float64)
        rc = self._fn("get")(self.h, FIELD_ID[name], out.ctypes.data)
        assert rc == 0
        return out

    def set(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == self.shape(name), (a.shape, self.shape(name))
        rc = self._fn("set")(self.h, FIELD_ID[name], a.ctypes.data)
        assert rc == 0

    def set_exact_velocity(self, vset: int, t: float, include_border: bool = True):
        self._fn("set_exact_velocity")(self.h, vset, t, 1 if include_border else 0)

    def set_exact_pressure(self, t: float):
        self._fn("set_exact_pressure")(self.h, t)

    def timestep(self, t_n: float):
        assert self._fn("timestep")(self.h, t_n) == 0

    def timestep_nhn(self, t_n: float):
        assert self._fn("timestep_nhn")(self.h, t_n) == 0

    def timestep_velocity(self, t_n: float):
        assert self._fn("timestep_velocity")(self.h, t_n) == 0

    def solve_pressure(self, vset: int, dt: float):
        assert self._fn("solve_pressure")(self.h, vset, dt) == 0

    def solve_pressure_nhn(self, vset: int, dt: float, t_new: float, t_old: float):
        assert self._fn("solve_pressure_nhn")(self.h, vset, dt, t_new, t_old) == 0

    def apply_bc(self, vset: int, t: float):
        assert self._fn("apply_bc")(self.h, vset, t) == 0

    def project(self, vset: int, dt: float):
        assert self._fn("project")(self.h, vset, dt) == 0

    def adjust_pressure(self, t: float):
        assert self._fn("adjust_pressure")(self.h, t) == 0

    def error_norms(self, t: float) -> np.ndarray:
        out = np.zeros(9)
        self._fn("error_norms")(self.h, t, out.ctypes.data)
        return out

    def state(self) -> dict:
        return {n: self.get(n) for n in FIELD_NAMES}

    def load_state(self, st: dict) -> None:
        for n, a in st.items():
            self.set(n, a)


class RefSolver(_Solver):
    """The reference's own code (oracle/_ref/libmifref.so)."""

    prefix = "mifref_"
    lib_path = REF_LIB

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_LIB)

    # The reference's exporters (include/VTKDatExport.h:10-29) on velocity
    # set 0 and the pressure.
    def write_vtk(self, filename: str) -> None:
        fn = self._fn("write_vtk")
        fn.argtypes = [C.c_void_p, C.c_char_p]
        fn(self.h, filename.encode())

    def write_dat(self, filename: str, direction: int, x: float, y: float, z: float) -> None:
        fn = self._fn("write_dat")
        fn.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_double, C.c_double, C.c_double]
        fn(self.h, filename.encode(), int(direction), float(x), float(y), float(z))

    def write_vtk_full_mesh(self, filename: str) -> None:
        fn = self._fn("write_vtk_full_mesh")
        fn.argtypes = [C.c_void_p, C.c_char_p]
        fn(self.h, filename.encode())


class OracleSolver(_Solver):
    """The plain-C restatement (oracle/libmif_oracle.so)."""

    prefix = "mif_oracle_"
    lib_path = ORACLE_LIB

    def __init__(self, case: Case):
        super().__init__(case)
        self._fn("set_forcing").argtypes = [C.c_void_p, C.c_int]
        self._fn("set_forcing")(self.h, int(case.forcing))

    def set_forcing_noise(self, rel: float, seed: int = 1) -> None:
        """Sensitivity probe (not reference behaviour): every forcing value is
        scaled by 1 + rel * r, r in [-1, 1) hashed per point from `seed`;
        rel = 0 restores the reference's arithmetic."""
        fn = self._fn("set_forcing_noise")
        fn.argtypes = [C.c_void_p, C.c_double, C.c_uint]
        fn(self.h, float(rel), int(seed))

    @staticmethod
    def available() -> bool:
        return os.path.exists(ORACLE_LIB)


class OracleFastSolver(OracleSolver):
    """The same restatement built with the reference's optimisation flags
    (oracle/libmif_oracle_fast.so): the CPU baseline's timing build only, never
    a checker."""

    lib_path = ORACLE_FAST_LIB

    @staticmethod
    def available() -> bool:
        return os.path.exists(ORACLE_FAST_LIB)


def pressure_gradient_value(kind: int, comp: int, t: float, x: float, y: float, z: float, Re: float) -> float:
    """Component `comp` of the analytic family's pressure gradient at (t, x,
    y, z) (oracle/manufactured.h, the functions the reference build uses)."""
    lib = _load(ORACLE_LIB)
    fn = lib.mif_oracle_pressure_gradient_value
    fn.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
    fn.restype = C.c_double
    return fn(int(kind), int(comp), float(t), float(x), float(y), float(z), float(Re))


def gradient_faces(case: Case, t_new: float, t_old: float) -> list:
    """The data apply_non_homogeneous_neumann adds (src/PressureEquation.cpp:10-56)
    for the family's gradient difference over time, get_difference_over_time(t_new,
    t_old) = grad p(t_old) - grad p(t_new): its normal component at the pressure
    nodes of the faces x_min, x_max, y_min, y_max, z_min, z_max, each of numpy
    shape (slow axis, fast axis) = the face's two other axes in reverse order."""
    E = case.extents("p")
    h = [case.size[d] / (case.n_global[d] - 1) for d in range(3)]
    base = [-1 if case.periodic[d] else 0 for d in range(3)]

    def pos(d, i):  # include/StaggeredTensor.h:113-119
        return case.origin[d] + h[d] * (base[d] + i)

    faces = []
    for d in range(3):
        a, b = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))
        for side in (0, 1):
            arr = np.empty((E[b], E[a]))
            for pb in range(E[b]):
                for pa in range(E[a]):
                    idx = [0, 0, 0]
                    idx[d] = 0 if side == 0 else E[d] - 1
                    idx[a], idx[b] = pa, pb
                    x, y, z = (pos(q, idx[q]) for q in range(3))
                    arr[pb, pa] = (pressure_gradient_value(case.exact_kind, d, t_old, x, y, z, case.Re) -
                                   pressure_gradient_value(case.exact_kind, d, t_new, x, y, z, case.Re))
            faces.append(arr)
    return faces


def r2r(kind: int, x: np.ndarray, direct: bool = False) -> np.ndarray:
    """oracle/r2r.c on one line (kind: 0 R2HC, 1 HC2R, 3 REDFT00)."""
    lib = _load(ORACLE_LIB)
    fn = lib.oracle_r2r_1d_direct if direct else lib.oracle_r2r_1d
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    a = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(a)
    rc = fn(len(a), kind, a.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise ValueError("r2r failed")
    return out


def reference_dir(ref_dir: str | None = None) -> str | None:
    """Where the reference's sources are: `ref_dir`, else MIF_REFERENCE_DIR,
    else a `reference` checkout beside this repository; None if none exists."""
    cands = [ref_dir, os.environ.get("MIF_REFERENCE_DIR"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "src")):
            return c
    return None


def build(ref_dir: str | None = None, with_ref: bool = True, fast: bool = False) -> None:
    """Compile the restatement (and its timing build when `fast`) and, when
    the reference sources exist, the reference library."""
    import subprocess

    subprocess.run(["make", "-s", "-C", HERE, "libmif_oracle.so"], check=True)
    if fast:
        subprocess.run(["make", "-s", "-C", HERE, "libmif_oracle_fast.so"], check=True)
    ref = reference_dir(ref_dir)
    if with_ref and ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True)
