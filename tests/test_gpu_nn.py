"""Tensor-core (tcgen05) BF16 convolutions of the warm-start network against PyTorch FP32.

Inputs and weights are rounded to BF16 first, so both sides multiply the same numbers; the
kernels accumulate in FP32 and round the output to BF16, hence the tolerance of a few BF16
ulps of the output magnitude."""
import ctypes

import numpy as np
import pytest
import torch
import torch.nn.functional as F

pytestmark = pytest.mark.gpu

GELU, ACCUM, DGELU = 1, 2, 4


def pad_cl(x):
    """[C, Z, Y, X] -> zero-haloed channels-last BF16 rows [R, C]."""
    c, z, y, xx = x.shape
    p = torch.zeros(z + 2, y + 2, xx + 2, c, dtype=torch.bfloat16, device="cuda")
    p[1:-1, 1:-1, 1:-1, :] = x.permute(1, 2, 3, 0).to(torch.bfloat16)
    return p.reshape(-1, c).contiguous()


def unpad(p, c, dims):
    xx, y, z = dims
    return p.reshape(z + 2, y + 2, xx + 2, c)[1:-1, 1:-1, 1:-1].permute(3, 0, 1, 2).float()


def halo(p, c, dims):
    xx, y, z = dims
    v = p.reshape(z + 2, y + 2, xx + 2, c).float().clone()
    v[1:-1, 1:-1, 1:-1] = 0
    return v


def taps_fwd(w):
    """torch [co][ci][3][3][3] (or 1x1x1) -> [taps][co][ci] BF16."""
    co, ci = w.shape[:2]
    return w.permute(2, 3, 4, 0, 1).reshape(-1, co, ci).to(torch.bfloat16).contiguous()


def bf(x):
    return x.to(torch.bfloat16).float()


def gelu_ref(x):
    return 0.5 * x * (1.0 + torch.tanh(0.7978845608028654 * (x + 0.044715 * x ** 3)))


def dgelu_ref(x):
    t = torch.tanh(0.7978845608028654 * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * 0.7978845608028654 * (1 + 3 * 0.044715 * x * x)


def ptrs(ts):
    return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])


def ints(v):
    return (ctypes.c_int * len(v))(*v)


def conv(lib, dims, ins, cins, w, ntaps, cout, bias=None, segs=None, aux=None, flags=0, flip=0):
    segs = segs or [cout]
    rows = (dims[0] + 2) * (dims[1] + 2) * (dims[2] + 2)
    outs = [torch.full((rows, c), 7.0, dtype=torch.bfloat16, device="cuda") for c in segs]
    return outs, _run(lib, dims, ins, cins, w, ntaps, cout, bias, segs, outs, aux, flags, flip)


def _run(lib, dims, ins, cins, w, ntaps, cout, bias, segs, outs, aux, flags, flip):
    rc = lib.gbp_nn_conv3d(ints(dims), len(ins), ptrs(ins), ints(cins), ctypes.c_void_p(w.data_ptr()), ntaps, flip,
                           cout, ctypes.c_void_p(bias.data_ptr() if bias is not None else None), len(segs), ptrs(outs),
                           ptrs(aux) if aux else None, ints(segs), flags,
                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.gbp_last_error().decode()
    return rc


def close(a, ref, ulps=4):
    scale = ref.abs().max().item()
    err = (a - ref).abs().max().item()
    assert err <= ulps * 2.0 ** -8 * scale + 1e-6, (err, scale)


CASES = [
    # dims (X, Y, Z), input channels, cout, taps
    ((8, 8, 8), [16], 16, 1),
    ((8, 8, 8), [16], 16, 27),
    ((16, 12, 10), [16], 32, 27),
    ((12, 10, 9), [32], 64, 27),
    ((10, 8, 8), [64], 64, 27),
    ((8, 8, 6), [128], 128, 27),
    ((9, 7, 8), [32, 16], 48, 27),
    ((8, 8, 8), [128, 64], 64, 27),
    ((40, 36, 34), [16], 16, 27),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}-{c[2]}-{c[3]}" for c in CASES])
def test_conv_forward_matches_torch(gpu_lib, case):
    dims, cins, cout, ntaps = case
    torch.manual_seed(0)
    xs = [bf(torch.randn(c, dims[2], dims[1], dims[0], device="cuda")) for c in cins]
    k = 3 if ntaps == 27 else 1
    w = bf(torch.randn(cout, sum(cins), k, k, k, device="cuda") / np.sqrt(ntaps * sum(cins)))
    bias = torch.randn(cout, device="cuda") * 0.1
    ref = F.conv3d(torch.cat(xs)[None], w, bias, padding=k // 2)[0]
    (out,), _ = conv(gpu_lib, dims, [pad_cl(x) for x in xs], cins, taps_fwd(w), ntaps, cout, bias)
    torch.cuda.synchronize()
    close(unpad(out, cout, dims), ref)
    assert halo(out, cout, dims).abs().max().item() == 0.0


def test_conv_forward_gelu_pre_and_segments(gpu_lib):
    dims, cins, cout = (10, 9, 8), [32, 16], 48
    torch.manual_seed(1)
    xs = [bf(torch.randn(c, dims[2], dims[1], dims[0], device="cuda")) for c in cins]
    w = bf(torch.randn(cout, sum(cins), 3, 3, 3, device="cuda") / np.sqrt(27 * sum(cins)))
    bias = torch.randn(cout, device="cuda") * 0.1
    pre_ref = F.conv3d(torch.cat(xs)[None], w, bias, padding=1)[0]
    rows = (dims[0] + 2) * (dims[1] + 2) * (dims[2] + 2)
    aux = [torch.full((rows, c), 3.0, dtype=torch.bfloat16, device="cuda") for c in (32, 16)]
    outs, _ = conv(gpu_lib, dims, [pad_cl(x) for x in xs], cins, taps_fwd(w), 27, cout, bias, segs=[32, 16],
                   aux=aux, flags=GELU)
    torch.cuda.synchronize()
    pre = torch.cat([unpad(aux[0], 32, dims), unpad(aux[1], 16, dims)])
    post = torch.cat([unpad(outs[0], 32, dims), unpad(outs[1], 16, dims)])
    close(pre, pre_ref)
    close(post, gelu_ref(pre_ref), ulps=6)
    for t, c in ((outs[0], 32), (outs[1], 16), (aux[0], 32), (aux[1], 16)):
        assert halo(t, c, dims).abs().max().item() == 0.0


@pytest.mark.parametrize("cin,cout", [(16, 16), (48, 32), (64, 128)])
def test_conv_data_gradient_matches_torch(gpu_lib, cin, cout):
    """dL/dx of y = conv(x, w): the flipped-tap kernel with transposed weights, accumulated onto an
    existing gradient and multiplied by gelu'(pre) of the layer that produced x."""
    dims = (10, 8, 9)
    torch.manual_seed(2)
    w = bf(torch.randn(cout, cin, 3, 3, 3, device="cuda") / np.sqrt(27 * cin))
    g = bf(torch.randn(cout, dims[2], dims[1], dims[0], device="cuda"))
    pre = bf(torch.randn(cin, dims[2], dims[1], dims[0], device="cuda"))
    prev = bf(torch.randn(cin, dims[2], dims[1], dims[0], device="cuda"))
    dx = torch.nn.grad.conv3d_input((1, cin) + tuple(g.shape[1:]), w, g[None], padding=1)[0]
    ref = (dx + prev) * dgelu_ref(pre)
    wt = w.permute(2, 3, 4, 1, 0).reshape(27, cin, cout).to(torch.bfloat16).contiguous()
    segs = [cin] if cin != 48 else [32, 16]
    outs = []
    auxs = []
    c0 = 0
    for c in segs:
        outs.append(pad_cl(prev[c0:c0 + c]))
        auxs.append(pad_cl(pre[c0:c0 + c]))
        c0 += c
    _run(gpu_lib, dims, [pad_cl(g)], [cout], wt, 27, cin, None, segs, outs, auxs, ACCUM | DGELU, 1)
    torch.cuda.synchronize()
    got = torch.cat([unpad(o, c, dims) for o, c in zip(outs, segs)])
    close(got, ref, ulps=6)


@pytest.mark.parametrize("cin,cout,ntaps", [(16, 16, 27), (32, 16, 27), (64, 32, 27), (128, 64, 27), (16, 32, 1)])
def test_conv_weight_gradient_matches_torch(gpu_lib, cin, cout, ntaps):
    dims = (12, 10, 11)
    torch.manual_seed(3)
    x = bf(torch.randn(cin, dims[2], dims[1], dims[0], device="cuda"))
    g = bf(torch.randn(cout, dims[2], dims[1], dims[0], device="cuda"))
    k = 3 if ntaps == 27 else 1
    ref = torch.nn.grad.conv3d_weight(x[None], (cout, cin, k, k, k), g[None], padding=k // 2)
    ref = ref.permute(2, 3, 4, 0, 1).reshape(ntaps, cout, cin)
    # write into the second half of a wider dw (channel offset ci0 = cin of a concatenated input)
    dw = torch.zeros(ntaps, cout, 2 * cin, device="cuda")
    xp, gp = pad_cl(x), pad_cl(g)  # keep both alive across the call
    rc = gpu_lib.gbp_nn_conv3d_wgrad(ints(dims), ctypes.c_void_p(xp.data_ptr()), cin, cin, 2 * cin,
                                     ctypes.c_void_p(gp.data_ptr()), cout, ntaps,
                                     ctypes.c_void_p(dw.data_ptr()),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, gpu_lib.gbp_last_error().decode()
    torch.cuda.synchronize()
    assert dw[:, :, :cin].abs().max().item() == 0.0
    got = dw[:, :, cin:]
    err = (got - ref).abs().max().item()
    assert err <= 1e-4 * ref.abs().max().item() + 1e-4, err
