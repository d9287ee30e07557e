"""The reference-side binding, integration/Timestep_gb300.cpp (the
single-GPU `src/Timestep.cpp` that INTEGRATION.md quotes), compiles against
the reference's own headers.

The build uses the single-rank MPI stand-in and `-DMIF_GB300
-Werror=missing-declarations`, so `timestep` and `timestep_nhn` must match
the declarations of include/Timestep.h:16-27. The object then links against
libmifgpu.so with no undefined symbol. Nothing runs, so no GPU is needed.

The compile test skips where the reference's headers are absent."""
import os
import re
import subprocess

import pytest

from conftest import ORACLE, REPO

BINDING = os.path.join(REPO, "integration", "Timestep_gb300.cpp")
SECTION = "## The binding a maintainer adds to `src/Timestep.cpp`"


def test_integration_md_quotes_the_binding_file():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    assert SECTION in text
    block = re.search(r"```cpp\n(.*?)```", text.split(SECTION, 1)[1], re.S)
    assert block, "no C++ block under the binding section"
    assert block.group(1) == open(BINDING).read()


def test_timestep_binding_compiles_against_the_reference_and_links(tmp_path, mifgpu_lib):
    import oracle

    ref = oracle.reference_dir()
    if ref is None:
        pytest.skip("reference headers not present on this machine")
    r = subprocess.run(["make", "-s", "-C", ORACLE, "adapter", f"REF={ref}", f"ADAPTER={BINDING}",
                        f"ADAPTER_OUT={tmp_path}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "libadapter.so").exists()
    nm = subprocess.run(["nm", "-C", str(tmp_path / "adapter.o")], capture_output=True, text=True,
                        check=True).stdout
    for fn in ("mif::timestep(", "mif::timestep_nhn("):
        assert re.search(r"\bT " + re.escape(fn), nm), fn
    for sym in ("mifgpu_create", "mifgpu_timestep_host", "mifgpu_upload", "mifgpu_timestep_nhn",
                "mifgpu_download", "mifgpu_set_boundary_values", "mifgpu_set_pressure_gradient_faces"):
        assert re.search(r"\bU " + sym + r"\b", nm), sym
