"""CPU oracle of the learned gate: the network's gradients against finite differences, the
bfloat16 rounding, and the features / labels of smooth and discontinuous states."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import gate_oracle as go  # noqa: E402
from hos_gb300 import cases  # noqa: E402
from oracle_lib import gate_cells  # noqa: E402


def test_mlp_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, go.NPARAM)
    X = rng.random((96, 16))
    y = rng.random(96) > 0.4
    _, g = go.loss_grad(p, X, y, quantize=False)
    idx = rng.choice(go.NPARAM, 64, replace=False)
    fd = go.finite_difference(p, X, y, idx)
    assert np.abs(fd - g[idx]).max() <= 1e-7 * max(1.0, np.abs(g).max())


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5e-3], np.float32)
    out = go.bf16(x)
    assert out[0] == 1.0 and out[1] == 1.0 and out[2] == 1.0 + 2.0 ** -6 and out[3] == 1.0
    assert abs(out[4] - x[4]) <= 2.0 ** -9 * abs(x[4])


def test_gate_labels_smooth_and_discontinuous_states():
    pb, con, _ = cases.sinwave2d(32, order=9)
    f, d = gate_cells(pb, con)
    ok = d >= 0
    assert (d[ok] <= 0.02).all()                    # a resolved sine wave: weights stay linear
    pb, con, _ = cases.isentropic_vortex(64, order=5)
    f, d = gate_cells(pb, con)
    ok = d >= 0
    assert (d[ok] <= 0.02).mean() > 0.9             # the vortex core on 64^2 cells
    assert f.min() >= 0.0 and f.max() <= 1.0
    pb, con, _ = cases.riemann2d(32, order=7)
    f, d = gate_cells(pb, con)
    ok = d >= 0
    assert (d[ok] > 0.02).sum() > 50                # the quadrant interfaces are not smooth
    assert (d[ok] <= 0.02).mean() > 0.5             # but most of the domain is piecewise constant
