"""Checkpoints (state_dict / load_state_dict, save_checkpoint / load_checkpoint)
and snapshots, through the C ABI.

A run resumed from a checkpoint must continue bit-identically: the state
blob carries the library's own pull-form populations, both phi buffers, the
mass-correction factors and the step sequencing flags."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from _cases import CASES, config, inputs  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return built_lib


def _solver(name, dtype, init=True):
    from lbm.fe_ac_solver import AllenCahnSolver
    case = CASES[name]
    solid, frac, C, u = inputs(case)
    s = AllenCahnSolver(config(case, "cuda"), dtype=dtype, **case["kw"])
    s.set_solid(solid, frac)
    if init:
        s.init_fields(C, u)
    return s


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64, torch.float16])
@pytest.mark.parametrize("at", [0, 1, 7])
def test_resume_is_bit_identical(dtype, at):
    """Checkpoint after `at` steps (0: right after init_fields), continue both
    the original and a fresh solver restored from the checkpoint."""
    a = _solver("ridge_l162", dtype)
    a.run(at)
    sd = a.state_dict()
    a.run(9)
    b = _solver("ridge_l162", dtype, init=False)
    b.load_state_dict(sd)
    assert b.step_count == at
    b.run(9)
    for fa, fb in zip(a.fields("phi", "u", "P", "mu_phi"), b.fields("phi", "u", "P", "mu_phi")):
        assert torch.equal(fa, fb)
    assert a.scalars() == b.scalars()
    assert b.step_count == a.step_count


def test_fields_after_restore_match():
    """Fields read right after a restore are those of the saved solver."""
    a = _solver("flat_q120", torch.float32)
    a.run(4)
    b = _solver("flat_q120", torch.float32, init=False)
    b.load_state_dict(a.state_dict())
    for k in ("phi", "rho", "u", "P", "p", "mu_phi"):
        assert torch.equal(getattr(a, k), getattr(b, k)), k
    assert torch.equal(a.f, b.f) and torch.equal(a.g, b.g)


def test_checkpoint_file_roundtrip(tmp_path):
    a = _solver("flat_q120", torch.float32)
    a.run(3)
    path = tmp_path / "ck.npz"
    a.save_checkpoint(path)
    a.run(5)
    b = _solver("flat_q120", torch.float32, init=False)
    b.load_checkpoint(path)
    b.run(5)
    assert torch.equal(a.phi, b.phi) and torch.equal(a.u, b.u)


def test_checkpoint_rejects_other_geometry_and_grid():
    from lbm import _native as nat
    a = _solver("ridge_l162", torch.float32)
    a.run(2)
    sd = a.state_dict()
    # same grid, other geometry (discrete-normal ridge: another node-class table)
    other = _solver("discrete_l162", torch.float32, init=False)
    with pytest.raises(nat.LbmError):
        other.load_state_dict(sd)
    # other precision
    with pytest.raises(nat.LbmError):
        _solver("ridge_l162", torch.float64, init=False).load_state_dict(sd)
    # not a state blob
    bad = dict(sd, state=np.zeros_like(sd["state"]))
    with pytest.raises(nat.LbmError):
        _solver("ridge_l162", torch.float32, init=False).load_state_dict(bad)


def test_snapshot_layout(tmp_path):
    """save_snapshot writes the key layout of the reference's sweep driver."""
    a = _solver("flat_q120", torch.float32)
    a.run(2)
    path = tmp_path / "snap.npz"
    a.save_snapshot(path)
    z = np.load(path)
    nx, ny, nz = a.shape
    phi = a.phi.cpu().numpy()
    assert np.array_equal(z["phi_3d"], phi)
    assert np.array_equal(z["u_3d"], a.u.cpu().numpy())
    assert np.array_equal(z["solid_3d"], a.solid.cpu().numpy())
    assert np.array_equal(z["xz_slice"], phi[:, ny // 2, :])
    assert np.array_equal(z["yz_slice"], phi[nx // 2, :, :])
    assert int(z["step"]) == 2 and (int(z["nx"]), int(z["ny"]), int(z["nz"])) == (nx, ny, nz)
