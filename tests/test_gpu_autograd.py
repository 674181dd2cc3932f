"""Differentiable CP layer: forward vs torch, backward vs torch autograd, central
finite differences (h = 1e-3, FP64) and the reference's gradient (GaussNewton.py:401-427)."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden, split_x

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")
torch = pytest.importorskip("torch")


def torch_cp(factors):
    L = len(factors)
    letters = "abcdefghijkl"[:L]
    return torch.einsum(",".join(c + "z" for c in letters) + "->" + letters, *factors)


def c3(dtype=torch.float64, seed=0, shape=(256, 256, 3, 3), R=64):
    g = torch.Generator(device="cpu").manual_seed(seed)
    W = [(torch.randn(d, R, generator=g, dtype=torch.float64) / np.sqrt(R)).to("cuda", dtype) for d in shape]
    T = torch.randn(*shape, generator=g, dtype=torch.float64).to("cuda", dtype)
    return T, W


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 2e-5)])
def test_reconstruct_forward_backward(dtype, tol):
    T, W = c3(dtype, shape=(40, 30, 3, 5), R=16)
    W = [w.clone().requires_grad_(True) for w in W]
    out = tfx.cp_reconstruct(W)
    W32 = [w.detach().clone().requires_grad_(True) for w in W]
    ref = torch_cp(W32)
    np.testing.assert_allclose(out.detach().cpu().numpy(), ref.detach().cpu().numpy(), rtol=tol, atol=tol)
    G = torch.randn_like(out)
    (out * G).sum().backward()
    (ref * G).sum().backward()
    for a, b in zip(W, W32):
        np.testing.assert_allclose(a.grad.cpu().numpy(), b.grad.cpu().numpy(), rtol=tol * 10, atol=tol * 10)


def test_fit_loss_gradient_finite_differences_c3():
    """c3: 256x256x3x3 weight, rank 64, factors N(0, 1/sqrt(R)); central FD, h = 1e-3, FP64."""
    T, W = c3(torch.float64)
    W = [w.clone().requires_grad_(True) for w in W]
    loss = tfx.cp_fit_loss(T, W)
    loss.backward()
    ref = ((torch_cp([w.detach() for w in W]) - T) ** 2).sum()
    assert abs(loss.item() - ref.item()) <= 1e-10 * ref.item()
    rng = np.random.default_rng(1)
    h = 1e-3
    for _ in range(4):
        dirs = [torch.from_numpy(rng.standard_normal(tuple(w.shape))).to("cuda") for w in W]
        nrm = float(torch.sqrt(sum((d * d).sum() for d in dirs)))
        dirs = [d / nrm for d in dirs]      # unit direction: h is the step length
        with torch.no_grad():
            lp = tfx.cp_fit_loss(T, [w + h * d for w, d in zip(W, dirs)]).item()
            lm = tfx.cp_fit_loss(T, [w - h * d for w, d in zip(W, dirs)]).item()
        fd = (lp - lm) / (2 * h)
        an = sum((w.grad * d).sum().item() for w, d in zip(W, dirs))
        assert abs(fd - an) <= 1e-5 * abs(an) + 1e-7


@pytest.mark.parametrize("name", ["units_L3", "units_L4", "units_L5"])
def test_fit_loss_gradient_is_twice_the_reference_gradient(name):
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    Wn = split_x(g["x"], dims, R)
    T = torch.from_numpy(g["T"]).cuda()
    W = [torch.from_numpy(w).cuda().requires_grad_(True) for w in Wn]
    tfx.cp_fit_loss(T, W).backward()
    got = np.concatenate([w.grad.cpu().numpy().flatten('F') for w in W])
    # the reference's compute_grad returns g with grad = -g inside cg (golden "grad" = g)
    np.testing.assert_allclose(got, 2 * g["grad"], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_mttkrp_all_modes_vs_oracle(dtype):
    rng = np.random.default_rng(3)
    dims, R = (23, 17, 9, 5), 11
    T = rng.standard_normal(dims)
    W = [rng.standard_normal((d, R)) for d in dims]
    Tl = [orc.unfold(T, l + 1) for l in range(4)]
    Td = torch.from_numpy(T).to("cuda", dtype)
    Wd = [torch.from_numpy(w).to("cuda", dtype) for w in W]
    tol = 1e-11 if dtype == torch.float64 else 1e-5
    for l in range(4):
        got = tfx.mttkrp(Td, Wd, l).double().cpu().numpy()
        ref = orc.mttkrp(Tl, W, l)
        np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * np.abs(ref).max())
