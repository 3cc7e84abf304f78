"""Learned warm start on the GPU: the tensor-core U-Net's loss and gradients against the FP64
restatement (itself pinned by finite differences in test_oracle_unet.py), training progress, and
the warm-started nodal solve (used / bypassed) converging to the same phi as the zero start."""
import numpy as np
import pytest
import torch

from incflo_gb300 import Geometry, NodalProjector, make_options, synth
from incflo_gb300.surrogate import Surrogate
from oracle import unet as U

pytestmark = pytest.mark.gpu


def bf16(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.bfloat16).double().numpy()


def padded_input(x0):
    """[Z, Y, X, 16] -> zero-haloed rows [R, 16] bf16 on the GPU."""
    z, y, x, c = x0.shape
    p = torch.zeros(z + 2, y + 2, x + 2, c, dtype=torch.bfloat16, device="cuda")
    p[1:-1, 1:-1, 1:-1] = torch.from_numpy(x0).to(torch.bfloat16).cuda()
    return p.reshape(-1, c).contiguous()


def padded_target(t):
    z, y, x = t.shape
    p = torch.zeros(z + 2, y + 2, x + 2, dtype=torch.float32, device="cuda")
    p[1:-1, 1:-1, 1:-1] = torch.from_numpy(t).float().cuda()
    return p.reshape(-1).contiguous()


def weight_mask():
    m = []
    for nin, c0, c1, co, t in U.layer_specs():
        m += [np.ones(t * co * (c0 + c1), bool), np.zeros(co, bool)]
    return np.concatenate(m)


def layer_slices():
    out, off = [], 0
    for nin, c0, c1, co, t in U.layer_specs():
        nw = t * co * (c0 + c1)
        out.append((slice(off, off + nw), slice(off + nw, off + nw + co)))
        off += nw + co
    return out


def test_surrogate_loss_and_gradients_match_fp64_oracle(gpu_lib):
    """BF16 activations, weights and gradients with FP32 accumulation against FP64: the loss within
    2 % and every layer's weight / bias gradient within 5 % (relative L2), overall cosine > 0.999."""
    s = Surrogate(seed=5)
    assert s.num_params == U.num_params()
    theta = s.params().astype(np.float64)
    wm = weight_mask()
    theta_bf = theta.copy()
    theta_bf[wm] = bf16(theta[wm])
    rng = np.random.default_rng(11)
    dims, dom = (16, 16, 16), (15, 16, 13)
    x0 = np.zeros((16, 16, 16, 16))
    x0[..., :3] = bf16(rng.standard_normal((16, 16, 16, 3)))
    target = rng.standard_normal((16, 16, 16)).astype(np.float32).astype(np.float64)
    xp, tp = padded_input(x0), padded_target(target)
    loss_gpu = s.train_pair(xp, tp, dims, dom, lr=0.0)
    g_gpu = s.grads().astype(np.float64)
    loss_cpu, g_cpu = U.loss_and_grad(theta_bf, x0, target, dom)
    assert abs(loss_gpu - loss_cpu) <= 0.02 * loss_cpu, (loss_gpu, loss_cpu)
    for i, (sw, sb) in enumerate(layer_slices()):
        for sl, what in ((sw, "w"), (sb, "b")):
            ref = g_cpu[sl]
            err = np.linalg.norm(g_gpu[sl] - ref) / max(np.linalg.norm(ref), 1e-30)
            if i == len(U.layer_specs()) - 1:
                # head: only output channel 0 carries gradient; the rest must be exactly zero
                assert np.all(g_gpu[sl][np.abs(ref) == 0] == 0)
            assert err <= 0.05, (i, what, err)
    cos = g_gpu @ g_cpu / (np.linalg.norm(g_gpu) * np.linalg.norm(g_cpu))
    assert cos > 0.999, cos


def test_surrogate_adam_fits_one_pair(gpu_lib):
    s = Surrogate(seed=1)
    rng = np.random.default_rng(2)
    dims, dom = (16, 16, 8), (16, 16, 8)
    x0 = np.zeros((8, 16, 16, 16))
    x0[..., :3] = rng.standard_normal((8, 16, 16, 3))
    # a smooth target the network can represent
    z, y, x = np.meshgrid(*[np.linspace(0, 1, d) for d in (8, 16, 16)], indexing="ij")
    target = np.sin(2 * np.pi * x) * np.cos(np.pi * z) + 0.5 * y
    xp, tp = padded_input(x0), padded_target(target)
    first = s.train_pair(xp, tp, dims, dom, lr=2e-3)
    for _ in range(60):
        last = s.train_pair(xp, tp, dims, dom, lr=2e-3)
    assert last < 0.3 * first, (first, last)


def _projector(n, seed, surrogate=None, level=1):
    case = synth.variable_density_rt(n, seed_h=seed, seed_u=seed + 100)
    geom = Geometry(case["n"], case["lo"], case["hi"])
    vel = torch.from_numpy(synth.with_ghosts(case["vel"])).cuda()
    sigma = torch.from_numpy(1.0 / case["rho"]).cuda()
    opts = make_options(0, precision="mixed", mg_rtol=1e-10, mg_atol=0.0)
    p = NodalProjector(vel, sigma, geom, options=opts)
    p.setDomainBC(["Periodic", "Periodic", "Neumann"], ["Periodic", "Periodic", "Neumann"])
    if surrogate is not None:
        p.setSurrogate(surrogate, level)
    return p


def test_warm_started_solve_converges_to_the_same_phi(gpu_lib):
    n = 32
    s = Surrogate(seed=3)
    for seed in range(4):
        p = _projector(n, seed)
        st = p.project()
        assert st["status"] == 0
        s.add_sample(p)
    assert s.num_samples == 4
    losses = s.train(60, lr=1e-3)
    assert np.isfinite(losses).all()
    ref = _projector(n, 9)
    st0 = ref.project()
    warm = _projector(n, 9, s, level=1)
    st1 = warm.project()
    assert st0["warm_start"] == 0
    assert st1["warm_start"] in (1, 2)
    assert st1["status"] == 0 and st1["final_rel_resid"] <= 1e-10
    a, b = warm.getPhi().cpu().numpy(), ref.getPhi().cpu().numpy()
    assert np.linalg.norm(a - b) <= 1e-7 * np.linalg.norm(b)


def test_zero_network_is_bypassed(gpu_lib):
    s = Surrogate(seed=4)
    s.set_params(np.zeros(s.num_params, np.float32))
    p = _projector(32, 5, s, level=1)
    st = p.project()
    assert st["warm_start"] == 2 and st["status"] == 0 and st["final_rel_resid"] <= 1e-10


def _sequence_projector(case, initial_guess, surrogate=None, level=1):
    geom = Geometry(case["n"], case["lo"], case["hi"])
    opts = make_options(0, precision="mixed", mg_rtol=1e-10, mg_atol=0.0, initial_guess=initial_guess)
    p = NodalProjector(torch.from_numpy(synth.with_ghosts(case["vel"])).cuda(),
                       torch.from_numpy(1.0 / case["rho"]).cuda(), geom, options=opts)
    p.setDomainBC(["Periodic", "Periodic", "Neumann"], ["Periodic", "Periodic", "Neumann"])
    if surrogate is not None:
        p.setSurrogate(surrogate, level)
    return p


def _run_sequence(n, initial_guess, surrogate=None, steps=4, seed=31):
    """successive projections of a slowly displaced interface on one plan; returns stats and phis"""
    from incflo_gb300.projection import NodalProjector as NP
    NP._plans.clear()  # a fresh plan: no last solution from other tests
    out = []
    for case in synth.rt_sequence(n, seed=seed, steps=steps):
        p = _sequence_projector(case, initial_guess, surrogate)
        st = p.project()
        assert st["status"] == 0 and st["final_rel_resid"] <= 1e-10
        out.append((st, p.getPhi().cpu().numpy().copy()))
    NP._plans.clear()
    return out


def test_previous_phi_start_saves_vcycles_on_a_sequence(gpu_lib):
    """initial_guess = previous: each projection of a time sequence starts from the plan's last phi, reaches
    the same tolerance in fewer V-cycles, and gives the same phi as the zero start (to the tolerance)."""
    zero = _run_sequence(64, "zero")
    prev = _run_sequence(64, "previous")
    assert prev[0][0]["prev_rel_resid"] == 0.0  # nothing before the first step
    for (sz, pz), (sp, pp) in zip(zero[1:], prev[1:]):
        assert 0.0 < sp["prev_rel_resid"] < 0.2
        assert sp["vcycles"] < sz["vcycles"]
        assert np.linalg.norm(pp - pz) <= 1e-8 * np.linalg.norm(pz)


def test_learned_increment_is_taken_only_when_it_beats_the_previous_phi(gpu_lib):
    """The warm start on top of the previous solution: the network predicts the increment, the Galerkin-
    scaled candidate is taken only when its residual is below the previous-phi start's, and the solve
    reaches the same phi either way. A network with zero weights predicts nothing and is bypassed; a
    briefly trained one is used or bypassed by that rule."""
    s0 = Surrogate(seed=4)
    s0.set_params(np.zeros(s0.num_params, np.float32))
    seq = _run_sequence(64, "previous", surrogate=s0, steps=3)
    # bypassed (2) on the first attempts; after two bypasses in a row the plan skips (3) the next ones
    assert seq[0][0]["warm_start"] == 2 and seq[1][0]["warm_start"] == 2
    assert all(st["warm_start"] in (2, 3) and st["status"] == 0 for st, _ in seq)
    # a few streamed training steps on sequence pairs (increments), then the rule on a held-out sequence
    from incflo_gb300.projection import NodalProjector as NP
    s = Surrogate(seed=5)
    NP._plans.clear()
    prev = None
    losses = []
    for case in synth.rt_sequence(64, seed=7, steps=6):
        p = _sequence_projector(case, "zero")
        assert p.project()["status"] == 0
        losses.append(s.train_step(p, prev, lr=1e-3))
        prev = p.getPhi().clone()
    assert np.isfinite(losses).all()
    ref = _run_sequence(64, "previous", steps=3)
    got = _run_sequence(64, "previous", surrogate=s, steps=3)
    for (sr, pr), (sg, pg) in zip(ref[1:], got[1:]):
        assert sg["warm_start"] in (1, 2, 3)
        if sg["warm_start"] == 1:
            assert sg["warm_rel_resid"] < sg["prev_rel_resid"]
        assert np.linalg.norm(pg - pr) <= 1e-8 * np.linalg.norm(pr)
