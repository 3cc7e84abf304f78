"""The FP64 restatement of the warm-start U-Net: analytic gradients against central finite
differences (CPU, no GPU). This pins the reference that the GPU tensor-core backward is checked
against."""
import numpy as np

from oracle import unet as U


def test_unet_layout_and_size():
    spec = U.layer_specs()
    assert len(spec) == 15
    assert U.num_params() == 1_466_320
    theta = U.init_params(0)
    assert theta.size == U.num_params()


def test_unet_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    dims = (8, 8, 8)
    x0 = np.zeros(dims[::-1] + (U.IN_C,))
    x0[..., :3] = rng.standard_normal(dims[::-1] + (3,))
    target = rng.standard_normal(dims[::-1])
    dom = (7, 8, 6)
    theta = U.init_params(3)
    # make every layer's output matter: give the head's channel 0 and the biases some weight
    theta += 0.01 * rng.standard_normal(theta.size)
    loss, grad = U.loss_and_grad(theta, x0, target, dom)
    assert np.isfinite(loss) and grad.shape == theta.shape
    # sample parameters from every layer (weights and biases)
    offs, idx = 0, []
    for nin, c0, c1, co, t in U.layer_specs():
        nw = t * co * (c0 + c1)
        idx += list(offs + rng.integers(0, nw, 3)) + [offs + nw + int(rng.integers(0, co))]
        offs += nw + co
    eps = 1e-5
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        fd = (U.loss_and_grad(tp, x0, target, dom)[0] - U.loss_and_grad(tm, x0, target, dom)[0]) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-6 * abs(grad[i]) + 1e-10, (i, fd, grad[i])
