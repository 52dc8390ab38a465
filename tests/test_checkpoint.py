"""Checkpoint output and restart against the reference's own ``save_npz`` / ``load_restart_host`` /
``infer_restart_step`` (fixture ``golden/checkpoint.npz``, made by ``golden/make_golden.py`` running
those functions): file name, keys and every array bit for bit, alpha1 clipping, missing keys and
shape errors. The restart uses the reference's constants (water 6.12 / 3.43e8, gas 1.4 / 0)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from wavemp import SolverParams  # noqa: E402
from wavemp.checkpoint import infer_restart_step, load_restart, save_npz  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ("ar1", "ar2", "ru", "rv", "E", "al", "u_p", "v_p", "p_p")
REF_EOS = SolverParams(dx=1.0, dy=1.0, gamma1=6.12, pinf1=3.43e8, gamma2=1.4, pinf2=0.0)


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(HERE, "golden", "checkpoint.npz"))


def state_from(gold, device="cpu"):
    q = {k: torch.from_numpy(gold["in_" + k].copy()).to(device) for k in NAMES}
    q["al_prim"] = q["al"].clone()
    return q


def check_restart(q, gold, prefix):
    for k in NAMES:
        got = q[k].to("cpu").numpy()
        assert np.array_equal(got, gold[prefix + k]), f"{prefix}{k}"
    assert not q["al_prim"].any()


@pytest.mark.parametrize("device", ["cpu", pytest.param("cuda", marks=pytest.mark.gpu)])
def test_save_matches_reference(gold, tmp_path, device):
    if device == "cuda" and not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = state_from(gold, device)
    path = save_npz(q, gold["in_x"], gold["in_y"], int(gold["in_step"]), float(gold["in_time"]),
                    directory=str(tmp_path))
    assert os.path.basename(path) == "mp5_000137.npz"
    with np.load(path) as f:
        keys = sorted(f.files)
        assert keys == sorted(k[len("saved_"):] for k in gold.files if k.startswith("saved_"))
        for k in keys:
            assert f[k].dtype == gold["saved_" + k].dtype
            assert np.array_equal(f[k], gold["saved_" + k]), k


@pytest.mark.parametrize("device", ["cpu", pytest.param("cuda", marks=pytest.mark.gpu)])
def test_restart_matches_reference(gold, tmp_path, device):
    if device == "cuda" and not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    nx, ny = gold["saved_ar1"].shape
    path = tmp_path / "mp5_000137.npz"
    np.savez_compressed(path, **{k[len("saved_"):]: gold[k] for k in gold.files if k.startswith("saved_")})
    q, t, step = load_restart(str(path), REF_EOS, nx, ny, device=device)
    check_restart(q, gold, "restart_")
    assert t == float(gold["restart_time"]) and step == int(gold["restart_step"])
    edge = tmp_path / "edge.npz"
    np.savez(edge, **{k[len("edge_in_"):]: gold[k] for k in gold.files if k.startswith("edge_in_")})
    q, t, step = load_restart(str(edge), REF_EOS, nx, ny, device=device)
    check_restart(q, gold, "edge_restart_")
    assert t == float(gold["edge_restart_time"]) == 0.0 and step == 0
    _, t, step = load_restart(str(path), REF_EOS, nx, ny, device=device, time=3.0, step=9)
    assert (t, step) == (3.0, 9)


def test_restart_errors(gold, tmp_path):
    nx, ny = gold["saved_ar1"].shape
    bad = tmp_path / "bad_7.npz"
    np.savez(bad, **{k: gold["saved_" + k] for k in ("ar1", "ar2", "u", "v", "p")})
    with pytest.raises(KeyError):
        load_restart(str(bad), REF_EOS, nx, ny, device="cpu")
    full = tmp_path / "full.npz"
    np.savez(full, **{k: gold["saved_" + k] for k in ("ar1", "ar2", "u", "v", "p", "alpha1")})
    with pytest.raises(ValueError):
        load_restart(str(full), REF_EOS, nx + 1, ny, device="cpu")
    assert infer_restart_step("out/mp5_000042.npz") == 42
    assert infer_restart_step("final.npz") == 0
