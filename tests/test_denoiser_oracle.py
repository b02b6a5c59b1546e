"""CPU tests of the denoiser oracle: its backward pass against central
differences of its forward pass (float64, no rounding), the BF16 rounding
helper, and the parameter layout shared with the C ABI."""
import numpy as np

import helios_gb300 as hx
from oracle import denoiser_ref as dr


def test_backward_matches_finite_differences():
    assert dr.finite_difference_check(seed=0, probes=40) < 1e-3
    assert dr.finite_difference_check(seed=1, probes=24, loss="l2lin") < 1e-3


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-39], np.float32)
    r = dr.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even
    assert r[2] == 1.0 + 2 ** -7
    assert r[3] == 1.0 + 2 ** -6  # tie -> even (up)
    assert r[4] == -2.5


def test_parameter_layout():
    shapes = dr.layer_shapes()
    assert len(shapes) == 13
    assert shapes[0] == (32, 32) and shapes[7] == (224, 96) and shapes[-1] == (32, 3)
    assert dr.num_params() == sum(9 * ci * co + co for ci, co in shapes)
    flat = np.arange(dr.num_params(), dtype=np.float64)
    parts = dr.split_params(flat)
    assert parts[0][0].shape == (9, 32, 32) and parts[0][1][0] == 9 * 32 * 32
    names = [t[0] for t in hx.DENOISER_TENSORS]
    assert names[:3] == ["x", "a0", "a0b"] and names[-1] == "gy"
    for name, c, lev in hx.DENOISER_TENSORS[1:-1]:
        assert c % 32 == 0 and 0 <= lev <= 4


def test_forward_shapes_and_loss():
    rng = np.random.default_rng(1)
    p = dr.init_params(2)
    f = rng.uniform(0, 1, (1, 32, 32, dr.FEATURES)).astype(np.float32)
    t = rng.uniform(0, 1, (1, 32, 32, 4)).astype(np.float32)
    loss, g, acts = dr.loss_and_grad(p, f, t)
    assert acts["y"].shape == (1, 32, 32, 3)
    assert acts["a4b"].shape == (1, 2, 2, 128)
    assert np.isfinite(loss) and loss > 0 and g.shape == (dr.num_params(),)
