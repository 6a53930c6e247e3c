"""The package's VTK writer (io_utils.write_vtk, native lbm_write_vtk) writes
byte for byte the files of the reference's io_utils/vtk_writer.py: hashes in
tests/golden/vtk_sha256.json, made by tests/golden/make_golden_vtk.py from the
reference itself.  Host only (no GPU)."""
import json
import os

import pytest

from make_golden_vtk import HERE, sha256_file, vtk_cases


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "vtk_sha256.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", sorted(vtk_cases()))
def test_vtk_bytes_match_reference(name, golden, tmp_path, built_lib):
    from io_utils import write_vtk
    rho, u, solid, dx, step, t = vtk_cases()[name]
    path = tmp_path / "sub" / (name + ".vtk")
    write_vtk(str(path), rho, u, solid=solid, dx=dx, step=step, t=t)
    h, n = sha256_file(path)
    assert n == golden[name]["bytes"]
    assert h == golden[name]["sha256"]


def test_vtk_torch_inputs(tmp_path, built_lib):
    """torch tensors are accepted and give the same file as numpy arrays."""
    torch = pytest.importorskip("torch")
    from io_utils import write_vtk
    rho, u, solid, dx, step, t = vtk_cases()["f32_3d"]
    a, b = tmp_path / "a.vtk", tmp_path / "b.vtk"
    write_vtk(str(a), rho, u, solid=solid, dx=dx, step=step, t=t)
    write_vtk(str(b), torch.from_numpy(rho), torch.from_numpy(u), solid=torch.from_numpy(solid), dx=dx,
              step=step, t=t)
    assert a.read_bytes() == b.read_bytes()


def test_vtk_unwritable_path_raises(tmp_path, built_lib):
    from io_utils import write_vtk
    rho, u, solid, dx, step, t = vtk_cases()["f32_3d"]
    blocker = tmp_path / "file"
    blocker.write_text("x")
    with pytest.raises(OSError):
        write_vtk(str(blocker / "sub" / "a.vtk"), rho, u)  # a directory under a regular file


def test_native_vtk_rejects_null_arguments(tmp_path, built_lib):
    lib = built_lib
    assert lib.lbm_write_vtk(str(tmp_path / "a.vtk").encode(), b"", 1, None, None, None, None, None) == -1
