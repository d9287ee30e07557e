"""Python host binding of the mifgpu C ABI (include/mifgpu.h) over ctypes.

It mirrors the reference's operator interface for the time step
(include/Timestep.h:16-27, include/TimestepVelocity.h:15-16,
include/PressureEquation.h:10-25, include/Norms.h): one ``Solver`` holds what
the reference passes as Constants, PressureSolverStructures and the six
tensors, and exposes ``timestep``, ``timestep_nhn``, ``timestep_velocity``,
``solve_pressure_equation_homogeneous_periodic``, ``apply_bc``,
``adjust_pressure`` and the error norms. Fields travel as numpy arrays in the
reference's layout: shape (Ez, Ey, Ex), x fastest.

There is no CPU path: if libmifgpu.so is missing or no CUDA device is present,
constructing a Solver raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmifgpu.so")

FIELDS = {"u": 0, "v": 1, "w": 2, "u1": 3, "v1": 4, "w1": 5, "u2": 6, "v2": 7, "w2": 8, "p": 9, "phi": 10}
FP64, MIXED, MIXED_COMPENSATED = 0, 1, 2
FIELD_ZERO, FIELD_SINCOS, FIELD_ETHIER, FIELD_CALLER = 0, 1, 2, 3
FORCING_NONE, FORCING_VELOCITY, FORCING_NAVIER_STOKES, FORCING_TAYLOR_GREEN = 0, 1, 2, 3

EXPORTED = [
    "mifgpu_create", "mifgpu_destroy", "mifgpu_set_stream", "mifgpu_synchronize", "mifgpu_last_error",
    "mifgpu_field_extent", "mifgpu_upload", "mifgpu_download", "mifgpu_set_exact_velocity",
    "mifgpu_set_exact_pressure", "mifgpu_timestep", "mifgpu_run", "mifgpu_timestep_host", "mifgpu_timestep_nhn",
    "mifgpu_timestep_velocity", "mifgpu_apply_bc", "mifgpu_solve_pressure", "mifgpu_divergence", "mifgpu_project",
    "mifgpu_adjust_pressure", "mifgpu_error_norms", "mifgpu_profile_step", "mifgpu_launch_count",
    "mifgpu_device_bytes", "mifgpu_gradient_ke", "mifgpu_backward", "mifgpu_download_adjoint",
    "mifgpu_set_forcing_amplitude", "mifgpu_velocity_error_norms_noalloc", "mifgpu_write_vtk",
    "mifgpu_write_dat", "mifgpu_write_vtk_full_mesh", "mifgpu_probe_fp64_fma", "mifgpu_set_boundary_values",
    "mifgpu_set_pressure_gradient_faces", "mifgpu_solve_pressure_nhn", "mifgpu_run_velocity",
]
PROFILE_CLASSES = ["stage", "boundary", "divergence", "x_forward", "y_forward", "z_fused", "y_inverse",
                   "x_inverse", "periodic", "project"]


class MifGpuError(RuntimeError):
    pass


class Params(C.Structure):
    _fields_ = [
        ("n_global", C.c_long * 3),
        ("size", C.c_double * 3),
        ("origin", C.c_double * 3),
        ("Re", C.c_double),
        ("dt", C.c_double),
        ("periodic", C.c_int * 3),
        ("precision", C.c_int),
        ("boundary_kind", C.c_int),
        ("forcing", C.c_int),
        ("forcing_amplitude", C.c_double),
    ]


_LIB = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libmifgpu.so (built by build.py) and declare its signatures."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise MifGpuError(f"mifgpu CUDA library not built: {path} (run build.py)")
    lib = C.CDLL(path)
    vp, i, d, dp = C.c_void_p, C.c_int, C.c_double, C.c_void_p
    sig = {
        "mifgpu_create": [C.POINTER(Params), C.POINTER(C.c_void_p)],
        "mifgpu_destroy": [vp],
        "mifgpu_set_stream": [vp, vp],
        "mifgpu_synchronize": [vp],
        "mifgpu_field_extent": [vp, i, dp],
        "mifgpu_upload": [vp, i, dp],
        "mifgpu_download": [vp, i, dp],
        "mifgpu_set_exact_velocity": [vp, i, d],
        "mifgpu_set_exact_pressure": [vp, d],
        "mifgpu_timestep": [vp, d],
        "mifgpu_run": [vp, d, i],
        "mifgpu_timestep_host": [vp, d, dp, dp, dp, dp],
        "mifgpu_timestep_nhn": [vp, d],
        "mifgpu_timestep_velocity": [vp, d],
        "mifgpu_run_velocity": [vp, d, i],
        "mifgpu_apply_bc": [vp, i, d],
        "mifgpu_solve_pressure": [vp, i, d],
        "mifgpu_divergence": [vp, i, d],
        "mifgpu_project": [vp, i, d],
        "mifgpu_adjust_pressure": [vp, d],
        "mifgpu_error_norms": [vp, d, dp],
        "mifgpu_profile_step": [vp, d, i, dp],
        "mifgpu_launch_count": [vp, dp],
        "mifgpu_device_bytes": [vp, dp],
        "mifgpu_gradient_ke": [vp, d, i, i, dp, dp, dp, dp],
        "mifgpu_backward": [vp, d, i, i, dp, dp, dp, dp, dp, dp],
        "mifgpu_download_adjoint": [vp, i, dp],
        "mifgpu_set_forcing_amplitude": [vp, d],
        "mifgpu_velocity_error_norms_noalloc": [vp, d, dp],
        "mifgpu_write_vtk": [vp, C.c_char_p],
        "mifgpu_write_dat": [vp, C.c_char_p, i, d, d, d],
        "mifgpu_write_vtk_full_mesh": [vp, C.c_char_p],
        "mifgpu_probe_fp64_fma": [dp],
        "mifgpu_set_boundary_values": [vp, i, dp, dp, dp],
        "mifgpu_set_pressure_gradient_faces": [vp, i, C.POINTER(C.c_void_p)],
        "mifgpu_solve_pressure_nhn": [vp, i, d, C.POINTER(C.c_void_p)],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.mifgpu_last_error.argtypes = [vp]
    lib.mifgpu_last_error.restype = C.c_char_p
    _LIB = lib
    return lib


def probe_fp64_fma() -> float:
    """FP64 fused multiply-add rate of the current device, TFLOP/s (instrumentation)."""
    lib = load_library()
    out = C.c_double(0.0)
    rc = lib.mifgpu_probe_fp64_fma(C.byref(out))
    if rc != 0:
        raise MifGpuError(f"mifgpu_probe_fp64_fma failed ({rc})")
    return out.value


class Solver:
    """One device-resident solver state (the reference's Constants + tensors)."""

    def __init__(self, n_global, size=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), Re=1000.0, dt=1e-4,
                 periodic=(False, False, False), precision=FP64, boundary_kind=FIELD_ZERO, forcing=FORCING_NONE,
                 forcing_amplitude=0.0):
        self.lib = load_library()
        p = Params()
        for k in range(3):
            p.n_global[k] = int(n_global[k])
            p.size[k] = float(size[k])
            p.origin[k] = float(origin[k])
            p.periodic[k] = 1 if periodic[k] else 0
        p.Re, p.dt = float(Re), float(dt)
        p.precision, p.boundary_kind, p.forcing = int(precision), int(boundary_kind), int(forcing)
        p.forcing_amplitude = float(forcing_amplitude)
        self.params = p
        self.dt = float(dt)
        h = C.c_void_p()
        rc = self.lib.mifgpu_create(C.byref(p), C.byref(h))
        self.h = h
        if rc != 0:
            msg = self.lib.mifgpu_last_error(h).decode() if h.value else "no context"
            if h.value:
                self.lib.mifgpu_destroy(h)
            self.h = None
            raise MifGpuError(f"mifgpu_create failed ({rc}): {msg}")

    # -- plumbing --
    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise MifGpuError(f"{what} failed ({rc}): {self.lib.mifgpu_last_error(self.h).decode()}")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mifgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int) -> None:
        self._check(self.lib.mifgpu_set_stream(self.h, C.c_void_p(stream_ptr)), "set_stream")

    def synchronize(self) -> None:
        self._check(self.lib.mifgpu_synchronize(self.h), "synchronize")

    def launch_count(self) -> int:
        out = C.c_longlong(0)
        self._check(self.lib.mifgpu_launch_count(self.h, C.byref(out)), "launch_count")
        return out.value

    def device_bytes(self) -> int:
        out = C.c_size_t(0)
        self._check(self.lib.mifgpu_device_bytes(self.h, C.byref(out)), "device_bytes")
        return out.value

    # -- fields --
    def extent(self, name: str) -> tuple:
        out = (C.c_long * 3)()
        self._check(self.lib.mifgpu_field_extent(self.h, FIELDS[name], out), "field_extent")
        return tuple(out)

    def shape(self, name: str) -> tuple:
        ex, ey, ez = self.extent(name)
        return (ez, ey, ex)

    def upload(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.shape != self.shape(name):
            raise MifGpuError(f"field {name}: shape {a.shape} != {self.shape(name)}")
        self._check(self.lib.mifgpu_upload(self.h, FIELDS[name], a.ctypes.data), "upload")
        self.synchronize()

    def download(self, name: str) -> np.ndarray:
        out = np.empty(self.shape(name), dtype=np.float64)
        self._check(self.lib.mifgpu_download(self.h, FIELDS[name], out.ctypes.data), "download")
        return out

    def set_exact_velocity(self, vset: int, t: float) -> None:
        self._check(self.lib.mifgpu_set_exact_velocity(self.h, vset, t), "set_exact_velocity")

    def set_exact_pressure(self, t: float) -> None:
        self._check(self.lib.mifgpu_set_exact_pressure(self.h, t), "set_exact_pressure")

    def load_state(self, st: dict) -> None:
        for n, a in st.items():
            self.upload(n, a)

    def state(self, names=tuple(FIELDS)) -> dict:
        return {n: self.download(n) for n in names}

    # -- the reference's operators --
    def timestep(self, t_n: float) -> None:
        self._check(self.lib.mifgpu_timestep(self.h, t_n), "timestep")

    def run(self, t0: float, nsteps: int) -> None:
        self._check(self.lib.mifgpu_run(self.h, t0, nsteps), "run")

    def timestep_host(self, t_n: float, u: np.ndarray, v: np.ndarray, w: np.ndarray, p: np.ndarray) -> None:
        for a in (u, v, w, p):
            if not (a.flags.c_contiguous and a.dtype == np.float64):
                raise MifGpuError("timestep_host needs C-contiguous float64 arrays")
        self._check(self.lib.mifgpu_timestep_host(self.h, t_n, u.ctypes.data, v.ctypes.data, w.ctypes.data,
                                                  p.ctypes.data), "timestep_host")

    def timestep_nhn(self, t_n: float) -> None:
        self._check(self.lib.mifgpu_timestep_nhn(self.h, t_n), "timestep_nhn")

    def timestep_velocity(self, t_n: float) -> None:
        self._check(self.lib.mifgpu_timestep_velocity(self.h, t_n), "timestep_velocity")

    def run_velocity(self, t0: float, nsteps: int) -> None:
        """`nsteps` velocity-only steps from graph replays (test/benchmark.cpp's loop)."""
        self._check(self.lib.mifgpu_run_velocity(self.h, t0, int(nsteps)), "run_velocity")

    def apply_bc(self, vset: int, t: float) -> None:
        self._check(self.lib.mifgpu_apply_bc(self.h, vset, t), "apply_bc")

    def solve_pressure_equation_homogeneous_periodic(self, vset: int, dt: float) -> None:
        self._check(self.lib.mifgpu_solve_pressure(self.h, vset, dt), "solve_pressure")

    solve_pressure = solve_pressure_equation_homogeneous_periodic

    # -- caller boundary data (boundary_kind FIELD_CALLER) --
    def set_boundary_values(self, slot: int, u: np.ndarray, v: np.ndarray, w: np.ndarray) -> None:
        """The Dirichlet face planes of u, v, w (reference layout; only the
        faces are read) for time slot `slot`: 0 for apply_bc, 1..3 for the
        stage times of the next step."""
        arrs = []
        for n, a in zip(("u", "v", "w"), (u, v, w)):
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != self.shape(n):
                raise MifGpuError(f"boundary values {n}: shape {a.shape} != {self.shape(n)}")
            arrs.append(a)
        self._check(self.lib.mifgpu_set_boundary_values(self.h, int(slot), *(a.ctypes.data for a in arrs)),
                    "set_boundary_values")

    def face_shapes(self) -> list:
        """Shapes of the six pressure-gradient face arrays (x_min, x_max,
        y_min, y_max, z_min, z_max), numpy order (slow axis first)."""
        ex, ey, ez = self.extent("p")
        return [(ez, ey), (ez, ey), (ez, ex), (ez, ex), (ey, ex), (ey, ex)]

    def _faces(self, faces):
        arrs = []
        for f, (a, shp) in enumerate(zip(faces, self.face_shapes())):
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != shp:
                raise MifGpuError(f"face {f}: shape {a.shape} != {shp}")
            arrs.append(a)
        ptrs = (C.c_void_p * 6)(*(a.ctypes.data for a in arrs))
        return arrs, ptrs

    def set_pressure_gradient_faces(self, slot: int, faces) -> None:
        """Normal pressure-gradient data (grad p(t_{k-1}) - grad p(t_k)) of
        stage `slot` of the next non-homogeneous Neumann step."""
        arrs, ptrs = self._faces(faces)
        self._check(self.lib.mifgpu_set_pressure_gradient_faces(self.h, int(slot), ptrs),
                    "set_pressure_gradient_faces")

    def solve_pressure_equation_non_homogeneous_neumann(self, vset: int, dt: float, faces) -> None:
        """phi from div(set)/dt and the caller's normal pressure-gradient faces
        (src/PressureEquation.cpp:276-286)."""
        arrs, ptrs = self._faces(faces)
        self._check(self.lib.mifgpu_solve_pressure_nhn(self.h, int(vset), float(dt), ptrs), "solve_pressure_nhn")

    solve_pressure_nhn = solve_pressure_equation_non_homogeneous_neumann

    def divergence(self, vset: int, dt: float) -> None:
        self._check(self.lib.mifgpu_divergence(self.h, vset, dt), "divergence")

    def project(self, vset: int, dt: float) -> None:
        self._check(self.lib.mifgpu_project(self.h, vset, dt), "project")

    def adjust_pressure(self, t: float) -> None:
        self._check(self.lib.mifgpu_adjust_pressure(self.h, t), "adjust_pressure")

    def profile_step(self, t_n: float, reps: int = 1) -> dict:
        """Mean ms per step of each kernel class (runs `reps` real steps)."""
        out = np.zeros(len(PROFILE_CLASSES))
        self._check(self.lib.mifgpu_profile_step(self.h, t_n, reps, out.ctypes.data), "profile_step")
        return dict(zip(PROFILE_CLASSES, out.tolist()))

    def error_norms(self, t: float) -> np.ndarray:
        out = np.zeros(9)
        self._check(self.lib.mifgpu_error_norms(self.h, t, out.ctypes.data), "error_norms")
        return out

    # -- the reference's writers (include/VTKDatExport.h) --
    def write_vtk(self, filename: str) -> None:
        self._check(self.lib.mifgpu_write_vtk(self.h, filename.encode()), "write_vtk")

    def write_dat(self, filename: str, direction: int, x: float, y: float, z: float) -> None:
        self._check(self.lib.mifgpu_write_dat(self.h, filename.encode(), int(direction), float(x), float(y), float(z)),
                    "write_dat")

    def write_vtk_full_mesh(self, filename: str) -> None:
        self._check(self.lib.mifgpu_write_vtk_full_mesh(self.h, filename.encode()), "write_vtk_full_mesh")

    def velocity_error_norms_noalloc(self, t: float) -> np.ndarray:
        """L1, L2, Linf of the velocity error (error_norms()[0:3]) from a static
        device scratch: no allocation, bitwise reproducible (see include/mifgpu.h)."""
        out = np.zeros(3)
        self._check(self.lib.mifgpu_velocity_error_norms_noalloc(self.h, t, out.ctypes.data),
                    "velocity_error_norms_noalloc")
        return out

    # -- reverse mode (no counterpart in the reference) --
    def set_forcing_amplitude(self, alpha: float) -> None:
        self._check(self.lib.mifgpu_set_forcing_amplitude(self.h, float(alpha)), "set_forcing_amplitude")
        self.params.forcing_amplitude = float(alpha)

    def gradient_ke(self, t0: float, nsteps: int, checkpoint_every: int, box) -> dict:
        """Kinetic energy in `box` (x0, x1, y0, y1, z0, z1) after `nsteps` steps from the
        current state and its gradient; the state advances to the final time.

        Returns loss, dloss_dalpha and the milliseconds of the forward pass,
        the whole backward pass (segment recomputes overlapped with reverse
        sweeps) and the reverse sweeps alone; the gradients with respect to
        the initial u, v, w, p come from ``adjoint(name)``."""
        b = np.ascontiguousarray(box, dtype=np.float64)
        loss, da = C.c_double(), C.c_double()
        ms = np.zeros(3)
        self._check(self.lib.mifgpu_gradient_ke(self.h, t0, int(nsteps), int(checkpoint_every), b.ctypes.data,
                                                C.addressof(loss), C.addressof(da), ms.ctypes.data),
                    "gradient_ke")
        return {"loss": loss.value, "dloss_dalpha": da.value, "forward_ms": ms[0], "backward_ms": ms[1],
                "reverse_ms": ms[2]}

    def backward(self, t0: float, nsteps: int, checkpoint_every: int, seeds: dict) -> dict:
        """Back-propagates d loss / d (final u, v, w, p) (``seeds``, reference-layout arrays,
        missing = 0) through `nsteps` steps from the current state."""
        bufs = []
        ptrs = []
        for n in ("u", "v", "w", "p"):
            if seeds.get(n) is None:
                ptrs.append(None)
                continue
            a = np.ascontiguousarray(seeds[n], dtype=np.float64)
            if a.shape != self.shape(n):
                raise MifGpuError(f"seed {n}: shape {a.shape} != {self.shape(n)}")
            bufs.append(a)
            ptrs.append(a.ctypes.data)
        da = C.c_double()
        ms = np.zeros(3)
        self._check(self.lib.mifgpu_backward(self.h, t0, int(nsteps), int(checkpoint_every), *ptrs,
                                             C.addressof(da), ms.ctypes.data), "backward")
        return {"dloss_dalpha": da.value, "forward_ms": ms[0], "backward_ms": ms[1], "reverse_ms": ms[2]}

    def adjoint(self, name: str) -> np.ndarray:
        """d loss / d (initial field) of the last gradient_ke / backward call (u, v, w or p)."""
        if name not in ("u", "v", "w", "p"):
            raise MifGpuError(f"no adjoint field {name}")
        out = np.empty(self.shape(name), dtype=np.float64)
        self._check(self.lib.mifgpu_download_adjoint(self.h, FIELDS[name], out.ctypes.data), "download_adjoint")
        return out
