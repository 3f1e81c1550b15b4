"""The adjoint (gradient of a band-limited harmonic yield with respect to the field).

* against central finite differences (h = 1e-6 a.u.) of the FP64 forward path:
  |grad_adjoint - grad_fd| <= 1e-5 max|grad| on random samples (the form's target);
* against torch autograd through a small dense restatement of the same step
  (psi' = Phi (A^{-1} 2 M2 psi - psi), 1DTDSE/sources/prop.c:137-205): relative 1e-9;
* through the torch.autograd.Function wrapper.
"""
import numpy as np
import pytest
import torch

from tests.tdse_cases import OMEGA0, sin2_pulse

pytestmark = pytest.mark.gpu


def _setup(num_r=300, dx=0.4, a=1.0, n_cycles=1.5, E0s=(0.06, 0.045), skip_first=True):
    from mma_gb300.tdse_batch import TDSEGrids

    t, base = sin2_pulse(n_cycles, E0=1.0, skip_first=skip_first)
    dtf = t[1] - t[0]
    grids = TDSEGrids([dict(num_r=num_r, dx=dx, trg_a=a)], dt=dtf, adjoint=True)
    fields = torch.tensor(np.stack([e0 * base for e0 in E0s]), device="cuda")
    return grids, fields, t, dtf


def test_adjoint_matches_finite_differences(gpu_lib):
    from mma_gb300.tdse_adjoint import yield_and_grad

    grids, fields, t, dtf = _setup()
    band = (3 * OMEGA0, 9 * OMEGA0)
    L, g = yield_and_grad(grids, fields, dtf, band, ckpt_every=32)
    torch.cuda.synchronize()
    rng = np.random.default_rng(0)
    h = 1e-6
    for i in range(fields.shape[0]):
        gi = g[i].cpu().numpy()
        idx = rng.choice(np.arange(2, fields.shape[1] - 2), size=8, replace=False)
        for n in idx:
            fp = fields.clone()
            fm = fields.clone()
            fp[i, n] += h
            fm[i, n] -= h
            Lp, _ = yield_and_grad(grids, fp, dtf, band, want_grad=False)
            Lm, _ = yield_and_grad(grids, fm, dtf, band, want_grad=False)
            fd = (Lp[i] - Lm[i]).item() / (2 * h)
            err = abs(gi[n] - fd) / np.abs(gi).max()
            assert err < 1e-5, (i, n, gi[n], fd, err)
    assert torch.all(L > 0)


def _torch_reference(grids, E, dtf, band):
    """Dense complex128 restatement of the FP64 step and the band loss, for autograd."""
    g = 0
    n = int(grids.n[g])
    dx, a = grids.params[g]["dx"], grids.params[g]["trg_a"]
    x = grids.x(g).cpu().to(torch.float64)
    psi0 = grids.psi0(g).cpu().to(torch.complex128)
    V = -1.0 / torch.sqrt(a * a + x * x)
    gv = x * (a * a + x * x) ** -1.5
    dt = dtf
    h = 0.5 * dt
    w = h * (-0.5 / dx ** 2) + h / 12.0 * V
    d = h / dx ** 2 + h * 10.0 / 12.0 * V
    A = torch.zeros(n, n, dtype=torch.complex128)
    M2 = torch.zeros(n, n, dtype=torch.float64)
    idx = torch.arange(n)
    A[idx, idx] = torch.complex(torch.full((n,), 10.0 / 12.0, dtype=torch.float64), d)
    A[idx[1:], idx[:-1]] = torch.complex(torch.full((n - 1,), 1.0 / 12.0, dtype=torch.float64), w[:-1])
    A[idx[:-1], idx[1:]] = torch.complex(torch.full((n - 1,), 1.0 / 12.0, dtype=torch.float64), w[1:])
    M2[idx, idx] = 10.0 / 12.0
    M2[idx[1:], idx[:-1]] = 1.0 / 12.0
    M2[idx[:-1], idx[1:]] = 1.0 / 12.0
    Ainv2M2 = torch.linalg.solve(A, 2 * M2.to(torch.complex128))
    nf = E.shape[0]
    S = nf + 2
    psi = psi0
    s = [torch.zeros((), dtype=torch.float64)]
    gate_open = False
    for k in range(S):
        fk = E[k] if k < nf else torch.zeros((), dtype=torch.float64)
        fk1 = E[k + 1] if k + 1 < nf else torch.zeros((), dtype=torch.float64)
        if not gate_open:
            if float(fk.detach()) * float(fk1.detach()) <= 0.0:  # the gate is not differentiated
                gate_open = True
            F = torch.zeros((), dtype=torch.float64)
        else:
            F = fk
        psi = torch.exp(1j * F * dt * x) * (Ainv2M2 @ psi - psi)
        s.append(-(psi.abs() ** 2 * gv).sum() + F)
    s = torch.stack(s[:S])
    tmax = (nf - 1) * dtf
    q = torch.arange(S // 2 + 1)
    om = 2 * np.pi * q / tmax
    sel = q[(om >= band[0]) & (om <= band[1]) & (q >= 1)]
    nn = torch.arange(S)
    ang = -2 * np.pi * ((sel[:, None] * nn[None, :]) % S).to(torch.float64) / S
    D = (torch.cos(ang) * s[None, :]).sum(1) + 1j * (torch.sin(ang) * s[None, :]).sum(1)
    return dt * dt / (2 * np.pi) * (D.abs() ** 2).sum()


def test_adjoint_matches_torch_autograd(gpu_lib):
    from mma_gb300.tdse_adjoint import yield_and_grad

    grids, fields, t, dtf = _setup(num_r=60, dx=0.5, n_cycles=0.75, E0s=(0.08,), skip_first=False)
    band = (2 * OMEGA0, 12 * OMEGA0)
    L, g = yield_and_grad(grids, fields, dtf, band, ckpt_every=16)
    E = fields[0].cpu().clone().requires_grad_(True)
    Lr = _torch_reference(grids, E, dtf, band)
    (gr,) = torch.autograd.grad(Lr, E)
    assert abs(L[0].item() - Lr.item()) < 1e-9 * abs(Lr.item())
    gk = g[0].cpu()
    assert torch.linalg.norm(gk - gr) / torch.linalg.norm(gr) < 1e-9


def test_autograd_function(gpu_lib):
    from mma_gb300.tdse_adjoint import TDSEYield, yield_and_grad

    grids, fields, t, dtf = _setup()
    band = (3 * OMEGA0, 9 * OMEGA0)
    f = fields.clone().requires_grad_(True)
    loss = TDSEYield.apply(f, grids, dtf, band, 64)
    (2.0 * loss[0] + loss[1]).backward()
    _, g = yield_and_grad(grids, fields, dtf, band, ckpt_every=64)
    assert torch.allclose(f.grad[0], 2.0 * g[0], rtol=1e-12, atol=0)
    assert torch.allclose(f.grad[1], g[1], rtol=1e-12, atol=0)
