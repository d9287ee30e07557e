"""Generate the golden fixtures from the reference's own code.

Runs oracle/_ref/libmifref.so — the reference's src/*.cpp and
deps/2Decomp_C/*.cpp compiled by oracle/Makefile (target `ref`) against the
single-rank MPI / FFTW stand-ins — on small seeded cases and stores inputs
and outputs as .npz files next to this script. Needs the reference sources
(only present where the fixtures are generated); the fixtures themselves are
committed and travel everywhere.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from cases import CASES  # noqa: E402


def run_case(name, spec):
    case = O.Case(**spec["case"])
    ref = O.RefSolver(case)
    rng = np.random.default_rng(spec.get("seed", 0))
    init = spec["init"]
    if init == "exact":
        ref.set_exact_velocity(0, spec.get("t0", 0.0), True)
        ref.set_exact_pressure(spec.get("t0", 0.0))
    elif init == "random":
        for n in ("u", "v", "w", "p"):
            ref.set(n, rng.standard_normal(ref.shape(n)) * spec.get("amp", 0.1))
    inputs = {n: ref.get(n) for n in O.FIELD_NAMES}
    op = spec["op"]
    dt = case.dt
    t0 = spec.get("t0", 0.0)
    for s in range(spec.get("steps", 1)):
        t = t0 + s * dt
        if op == "timestep":
            ref.timestep(t)
        elif op == "timestep_nhn":
            ref.timestep_nhn(t)
        elif op == "timestep_velocity":
            ref.timestep_velocity(t)
        elif op == "solve_pressure":
            ref.solve_pressure(0, spec.get("solve_dt", 1.0))
        elif op == "apply_bc":
            ref.apply_bc(0, spec.get("bc_t", 0.3))
        elif op == "solve_pressure_nhn":
            ref.solve_pressure_nhn(0, spec.get("solve_dt", 1.0), spec["t_new"], spec["t_old"])
        else:
            raise ValueError(op)
    outputs = {n: ref.get(n) for n in O.FIELD_NAMES}
    norms = ref.error_norms(t0 + spec.get("steps", 1) * dt) if case.exact_kind else np.zeros(9)
    arrays = {f"in_{k}": v for k, v in inputs.items()}
    arrays.update({f"out_{k}": v for k, v in outputs.items()})
    arrays["norms"] = norms
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
    print(f"{name}: {[a.shape for a in inputs.values()][:3]} ... norms {norms[:3]}")


# The reference's writers (src/VTKDatExport.cpp) on the state after one step:
# the state and the bytes of every file they write.
EXPORT_CASES = {
    "export_dirichlet": dict(case=dict(n_global=(9, 10, 11), size=(1.0, 1.0, 2.0), origin=(0.0, 0.0, -1.0),
                                       Re=1000.0, dt=1e-4, exact_kind=O.KIND_ETHIER), init="exact",
                             # (direction, x, y, z): y midway / z on planes; x on a plane; x midway (the y line
                             # that reads v where u is meant)
                             lines=[(0, 0.5, 0.5, 0.0), (1, 0.5, 0.5, 0.0), (2, 0.5, 0.5, 0.0), (1, 0.0625, 0.5, 0.0)]),
    "export_channel": dict(case=dict(n_global=(9, 8, 10), size=(6.283185307179586, 2.0, 3.141592653589793),
                                     origin=(0.0, -1.0, 0.0), Re=500.0, dt=1e-3, periodic=(True, False, True)),
                           init="random", seed=5,
                           lines=[(0, 0.0, 0.0, 0.0), (1, 0.0, 0.0, 0.0), (2, 0.0, 0.0, 0.0), (2, 0.3926990816987241, 0.0, 0.0)]),
}


def run_export_case(name, spec, tmpdir):
    case = O.Case(**spec["case"])
    ref = O.RefSolver(case)
    if spec["init"] == "exact":
        ref.set_exact_velocity(0, 0.0, True)
        ref.set_exact_pressure(0.0)
    else:
        rng = np.random.default_rng(spec["seed"])
        for n in ("u", "v", "w", "p"):
            ref.set(n, rng.standard_normal(ref.shape(n)) * 0.1)
    ref.timestep(0.0)
    arrays = {f"state_{n}": ref.get(n) for n in ("u", "v", "w", "p")}
    f = os.path.join(tmpdir, f"{name}.vtk")
    ref.write_vtk(f)
    arrays["vtk"] = np.frombuffer(open(f, "rb").read(), dtype=np.uint8)
    f = os.path.join(tmpdir, f"{name}_full.vtk")
    ref.write_vtk_full_mesh(f)
    arrays["vtk_full"] = np.frombuffer(open(f, "rb").read(), dtype=np.uint8)
    for q, (d, x, y, z) in enumerate(spec["lines"]):
        f = os.path.join(tmpdir, f"{name}_{q}.dat")
        ref.write_dat(f, d, x, y, z)
        arrays[f"dat{q}"] = np.frombuffer(open(f, "rb").read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
    print(f"{name}: vtk {arrays['vtk'].size} B, full {arrays['vtk_full'].size} B, "
          f"dat {[arrays[f'dat{q}'].size for q in range(len(spec['lines']))]} B")


if __name__ == "__main__":
    import tempfile

    if not O.RefSolver.available():
        O.build()
    for name, spec in CASES.items():
        run_case(name, spec)
    with tempfile.TemporaryDirectory() as tmp:
        for name, spec in EXPORT_CASES.items():
            run_export_case(name, spec, tmp)
