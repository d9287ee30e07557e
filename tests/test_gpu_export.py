"""The VTK and DAT writers (mifgpu_write_vtk / _dat / _vtk_full_mesh) against
the reference's own writers: on the same state an FP64 context must write the
same bytes as src/VTKDatExport.cpp (golden fixtures made from the reference,
tests/golden/make_golden.py); a mixed context writes the reference's float
layout with values equal to the FP64 ones to float rounding."""
import os
import struct
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)

pytestmark = pytest.mark.gpu

NAMES = ("export_dirichlet", "export_channel")


def solver_for(mg, name, precision):
    import make_golden as M

    c = M.EXPORT_CASES[name]["case"]
    return mg.Solver(n_global=c["n_global"], size=c["size"], origin=c["origin"], Re=c["Re"], dt=c["dt"],
                     periodic=c.get("periodic", (False, False, False)), precision=precision,
                     boundary_kind=c.get("exact_kind", 0))


@pytest.mark.parametrize("name", NAMES)
def test_fp64_writers_match_reference_bytes(mifgpu_lib, cuda_device, tmp_path, name):
    import make_golden as M

    want = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s = solver_for(mifgpu_lib, name, mifgpu_lib.FP64)
    s.load_state({n: want[f"state_{n}"] for n in ("u", "v", "w", "p")})
    s.write_vtk(str(tmp_path / "a.vtk"))
    assert (tmp_path / "a.vtk").read_bytes() == want["vtk"].tobytes()
    s.write_vtk_full_mesh(str(tmp_path / "f.vtk"))
    assert (tmp_path / "f.vtk").read_bytes() == want["vtk_full"].tobytes()
    for q, (d, x, y, z) in enumerate(M.EXPORT_CASES[name]["lines"]):
        s.write_dat(str(tmp_path / f"{q}.dat"), d, x, y, z)
        assert (tmp_path / f"{q}.dat").read_bytes() == want[f"dat{q}"].tobytes(), (name, q)
    s.close()


def _vtk_scalars(blob, real):
    """Coordinates and the four scalar arrays of a binary VTK written by writeVTK."""
    size = 8 if real == "double" else 4
    fmt = ">" + ("d" if size == 8 else "f")
    head = blob.index(b"POINTS ")
    line_end = blob.index(b"\n", head)
    n = int(blob[head:line_end].split()[1])
    pos = line_end + 1
    coords = np.array(struct.unpack(fmt[0] + fmt[1] * (3 * n), blob[pos:pos + 3 * n * size]))
    pos += 3 * n * size
    cols = []
    for _ in range(4):
        pos = blob.index(b"LOOKUP_TABLE default\n", pos) + len(b"LOOKUP_TABLE default\n")
        cols.append(np.array(struct.unpack(fmt[0] + fmt[1] * n, blob[pos:pos + n * size])))
        pos += n * size
    return coords, cols


def test_mixed_writer_uses_float_layout(mifgpu_lib, cuda_device, tmp_path):
    name = "export_dirichlet"
    want = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s = solver_for(mifgpu_lib, name, mifgpu_lib.MIXED)
    s.load_state({n: want[f"state_{n}"] for n in ("u", "v", "w", "p")})
    s.write_vtk(str(tmp_path / "m.vtk"))
    blob = (tmp_path / "m.vtk").read_bytes()
    assert b"POINTS 299 float\n" in blob
    c32, v32 = _vtk_scalars(blob, "float")
    c64, v64 = _vtk_scalars(want["vtk"].tobytes(), "double")
    np.testing.assert_allclose(c32, c64, rtol=0, atol=1e-6)
    for a, b in zip(v32, v64):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-6 * max(1.0, np.abs(b).max()))
    s.close()


def test_writer_rejects_bad_line(mifgpu_lib, cuda_device, tmp_path):
    s = solver_for(mifgpu_lib, "export_dirichlet", mifgpu_lib.FP64)
    with pytest.raises(mifgpu_lib.MifGpuError, match="pressure planes"):
        s.write_dat(str(tmp_path / "bad.dat"), 0, 0.5, 0.3, 0.0)
    with pytest.raises(mifgpu_lib.MifGpuError, match="direction"):
        s.write_dat(str(tmp_path / "bad.dat"), 3, 0.5, 0.5, 0.0)
    s.close()
