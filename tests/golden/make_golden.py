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
        else:
            raise ValueError(op)
    outputs = {n: ref.get(n) for n in O.FIELD_NAMES}
    norms = ref.error_norms(t0 + spec.get("steps", 1) * dt) if case.exact_kind else np.zeros(9)
    arrays = {f"in_{k}": v for k, v in inputs.items()}
    arrays.update({f"out_{k}": v for k, v in outputs.items()})
    arrays["norms"] = norms
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
    print(f"{name}: {[a.shape for a in inputs.values()][:3]} ... norms {norms[:3]}")


if __name__ == "__main__":
    if not O.RefSolver.available():
        O.build()
    for name, spec in CASES.items():
        run_case(name, spec)
