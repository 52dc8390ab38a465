"""Schlieren post-processing on the device against the reference's own figure arithmetic
(numpy.gradient on the cell centres and the gradient magnitude, SC:1734-1739), bit for bit, on
coordinates with round-off-unequal spacings (the reference's cell centres) and with exactly equal
ones (numpy's uniform branch); and the headless image's layout."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from wavemp import ic  # noqa: E402
from wavemp.checkpoint import cell_centres  # noqa: E402
from wavemp.post import save_schlieren, schlieren  # noqa: E402

G = 5


def reference_grad(q, x, y, nx, ny):
    rho = (q["ar1"] + q["ar2"]).cpu().numpy()[G:G + nx, G:G + ny]
    xg, yg = x[G:G + nx], y[G:G + ny]
    drhodx = np.gradient(rho, xg, axis=0)
    drhody = np.gradient(rho, yg, axis=1)
    return np.sqrt(drhodx ** 2 + drhody ** 2)


@pytest.mark.parametrize("nx,ny,coords", [(96, 48, "centres"), (37, 19, "centres"), (64, 32, "uniform"),
                                          (2, 2, "centres")])
def test_schlieren_equals_numpy_gradient(nx, ny, coords):
    q = ic.random_valid(nx, ny, np.random.default_rng(3))
    if coords == "centres":
        x, y = cell_centres(nx, 0.0, 1.0, G), cell_centres(ny, 0.0, 0.5, G)
        assert not (np.diff(x[G:G + nx]) == np.diff(x[G:G + nx])[0]).all() or nx <= 3
    else:
        x, y = 0.25 * np.arange(nx + 2 * G, dtype=np.float64), 0.5 * np.arange(ny + 2 * G, dtype=np.float64)
    grad, rgb = schlieren(q, x, y, G)
    ref = reference_grad(q, x, y, nx, ny)
    assert np.array_equal(grad.cpu().numpy(), ref)
    assert tuple(rgb.shape) == (ny, 2 * nx, 3)


def test_image_panels(tmp_path):
    nx, ny = 128, 64
    q = ic.shock_droplet(nx, ny, 1.0, 0.5, mach=2.4)
    x, y = cell_centres(nx, 0.0, 1.0, G), cell_centres(ny, 0.0, 0.5, G)
    _, rgb = schlieren(q, x, y, G)
    img = rgb.cpu().numpy()
    al = q["al"].cpu().numpy()[G:G + nx, G:G + ny]
    red = (img[:, :nx, 0] == 255) & (img[:, :nx, 1] == 0) & (img[:, :nx, 2] == 0)
    assert red.any()  # the droplet outline
    # right panel: inverted grey of alpha1 (water = dark)
    grey = img[:, nx:, 0].T
    assert np.all(np.abs(grey.astype(float) - 255.0 * (1.0 - np.clip(al, 0, 1))) <= 0.5 + 1e-9)
    npz, ppm = save_schlieren(q, x, y, 7, 1.0e-6, directory=str(tmp_path))
    with np.load(npz) as f:
        assert f["grad"].shape == (nx, ny) and float(f["time"]) == 1.0e-6
    head = open(ppm, "rb").read(20)
    assert head.startswith(b"P6\n256 64\n255\n")
