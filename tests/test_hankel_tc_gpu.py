"""Tensor-core form of the per-plane far-field transforms (split-precision FP16, FP32 accumulation).

* the tcgen05 building blocks against a float32 matrix product of the same FP16 operands
  (operands staged by threads, and B by TMA);
* every plane against the plain FP64 form on a problem with ragged sizes (n_r, n_z, n_rho not
  multiples of the tile sizes): per-harmonic relative L2 error over rho <= 2e-5, the bound
  stated for the fast form;
* the cumulative results of Hankel_long through the tensor-core planes against the reference's
  own fixtures (Hankel_transform.py run on the same inputs).
"""
import ctypes
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 2e-5


def per_harmonic(a, b):
    """max over omega of ||a[:, w] - b[:, w]|| / ||b[:, w]|| (arrays [rho, omega])."""
    return float(np.max(np.linalg.norm(a - b, axis=0) / np.linalg.norm(b, axis=0)))


@pytest.mark.parametrize("use_tma", [0, 1])
def test_tcgen05_tile(gpu_lib, use_tma):
    from mma_gb300._lib import load

    lib = load()
    lib.mma_tc_selftest.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.mma_tc_selftest.restype = ctypes.c_int
    g = torch.Generator().manual_seed(3)
    A = torch.randn(128, 32, generator=g).half().cuda()
    B = torch.randn(256, 32, generator=g).half().cuda()
    D = torch.full((128, 256), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.mma_tc_selftest(A.data_ptr(), B.data_ptr(), D.data_ptr(), use_tma, status.data_ptr(), st) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    ref = A.float() @ B.float().T
    assert torch.isfinite(D).all()
    assert (D - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()


def test_tcgen05_bounded_wait_runs_out(gpu_lib):
    """A bounded mbarrier wait that nothing satisfies gives up, the kernel reports the timeout in
    its status word and returns; the next tensor-core launch in the same context still works."""
    from mma_gb300._lib import load

    lib = load()
    lib.mma_tc_selftest.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.mma_tc_selftest.restype = ctypes.c_int
    A = torch.ones(128, 32, dtype=torch.float16, device="cuda")
    B = torch.ones(256, 32, dtype=torch.float16, device="cuda")
    D = torch.full((128, 256), -7.0, dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.mma_tc_selftest(A.data_ptr(), B.data_ptr(), D.data_ptr(), 2, status.data_ptr(), st) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 1  # the first bounded wait gave up
    assert bool((D == -7.0).all())  # nothing was written
    assert lib.mma_tc_selftest(A.data_ptr(), B.data_ptr(), D.data_ptr(), 1, status.data_ptr(), st) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert bool((D == 32.0).all())


def test_tf32_tile_layout(gpu_lib):
    """One tcgen05.mma kind::tf32 (M 128, N 16, K 8) from K-major core-matrix tiles without
    swizzle, the operand layout of the tensor-core stage 1: integer operands are exact in TF32, so
    D = A B^T is exact."""
    lib = gpu_lib
    lib.mma_s1tc_selftest.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_void_p]
    lib.mma_s1tc_selftest.restype = ctypes.c_int
    rng = np.random.default_rng(7)
    A = rng.integers(-8, 9, (128, 8)).astype(np.float32)
    B = rng.integers(-8, 9, (16, 8)).astype(np.float32)
    dA, dB = torch.tensor(A, device="cuda"), torch.tensor(B, device="cuda")
    dD = torch.full((128, 16), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.mma_s1tc_selftest(dA.data_ptr(), dB.data_ptr(), dD.data_ptr(), status.data_ptr(), st) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert np.array_equal(dD.cpu().numpy(), A @ B.T)


def _problem(n_omega=24, n_r=200, n_z=40, n_rho=50, seed=0, rho_max=5e-3):
    omega0 = 0.057 / 2.4188843265857e-17
    rgrid = np.linspace(0.0, 200e-6, n_r)
    zgrid = np.linspace(-5e-3, 5e-3, n_z)
    ogrid = np.linspace(10 * omega0, 42 * omega0, n_omega)
    rho = np.linspace(0.0, rho_max, n_rho)
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0, 2 * np.pi, size=(n_z, n_omega))
    S = np.exp(-(rgrid / 50e-6) ** 2)[None, None, :] * np.exp(1j * ph)[:, :, None]
    return zgrid, rgrid, ogrid, rho, torch.tensor(S, dtype=torch.complex64, device="cuda")


@pytest.mark.parametrize("tol,rho_max,terms", [(1e-9, 5e-3, 16), (1e-6, 1e-3, 8), (1e-13, 5e-3, 32)],
                         ids=["16 terms", "8 terms", "32 terms"])
def test_all_planes_vs_plain(gpu_lib, tol, rho_max, terms):
    from mma_gb300 import hankel as H

    zg, rg, og, rho, S = _problem(rho_max=rho_max)
    planes = list(range(len(zg)))
    pre = np.exp(1j * np.linspace(0, 1, len(zg)))[:, None] * np.ones((1, len(og)))
    _, p64, _ = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=planes, form="plain")
    _, ptc, plan = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=planes, form="fast", tol=tol,
                               planes_via="tc")
    assert plan["planes_via"] == "tc"
    assert {8: 8, 12: 16, 16: 16, 20: 32, 24: 32, 32: 32}[int(plan["n_terms"])] == terms
    worst = max(per_harmonic(ptc[k].cpu().numpy(), p64[k].cpu().numpy()) for k in planes)
    print("tensor-core planes, %d terms: worst per-harmonic error %.2e" % (plan["n_terms"], worst))
    assert worst < TOL


def test_ring_fed_b_operand_matches_direct_loads(gpu_lib):
    """A complex64 source with an even number of radii goes through the ring-fed B preparation
    (bulk copies into shared memory, packed pair arithmetic); the same values as complex128 go
    through the preparation that loads each value itself.  Both compute the same operations in the
    same order, so the planes agree bit for bit."""
    from mma_gb300 import hankel as H

    zg, rg, og, rho, S = _problem(n_omega=16, n_z=40)
    planes = list(range(len(zg)))
    pre = np.exp(1j * np.linspace(0, 1, len(zg)))[:, None] * np.ones((1, len(og)))
    _, p64, _ = H.far_field(og, rg, zg, rho, S, 1.0, pre, True, planes=planes, form="fast", planes_via="tc")
    _, p128, _ = H.far_field(og, rg, zg, rho, S.to(torch.complex128), 1.0, pre, True, planes=planes, form="fast",
                             planes_via="tc")
    for k in planes:
        assert torch.equal(p64[k], p128[k]), k


@pytest.mark.parametrize("nz,nrho,no", [(40, 50, 24), (600, 3, 37)], ids=["40 planes", "600 planes, ragged"])
def test_z_trapezoid_of_planes(gpu_lib, nz, nrho, no):
    """mma_hankel_ff_from_planes (FF_integrated from every plane, Hankel_transform.py:661) against
    the trapezoid in numpy: planes stored in a permuted slot order, a non-uniform z grid, more
    planes than one staged chunk (512) and element counts that leave a ragged last CTA."""
    import ctypes

    from mma_gb300 import hankel as H

    lib = H._sig()
    rng = np.random.default_rng(nz)
    z = np.sort(rng.uniform(-5e-3, 5e-3, nz))
    slot = rng.permutation(nz).astype(np.int64)
    planes = rng.standard_normal((nz, nrho, no)) + 1j * rng.standard_normal((nz, nrho, no))
    w = np.zeros(nz)
    w[:-1] += 0.5 * np.diff(z)
    w[1:] += 0.5 * np.diff(z)
    ref = np.einsum("k,kab->ab", w, planes[slot])  # plane k is stored at slot[k]
    prob = H.HankelProblem(no, 2, nz, nrho, 1.0, 1, 0, no * 2, 2, 0)
    dz = torch.tensor(z, device="cuda")
    ds = torch.tensor(slot, device="cuda")
    dp = torch.tensor(planes, dtype=torch.complex128, device="cuda")
    ff = torch.full((nrho, no), complex("nan"), dtype=torch.complex128, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.mma_hankel_ff_from_planes(ctypes.byref(prob), dz.data_ptr(), ds.data_ptr(), dp.data_ptr(),
                                         ff.data_ptr(), st) == 0
    torch.cuda.synchronize()
    got = ff.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_selected_planes_only(gpu_lib):
    """Planes not requested are not written; requested ones match the direct FP32 form."""
    from mma_gb300 import hankel as H

    zg, rg, og, rho, S = _problem(n_omega=8, n_z=20)
    want = [0, 3, 19]
    _, pd, _ = H.far_field(og, rg, zg, rho, S, 1.0, None, True, planes=want, form="fast", planes_via="direct")
    _, pt, plan = H.far_field(og, rg, zg, rho, S, 1.0, None, True, planes=want, form="fast", planes_via="tc")
    assert plan["planes_via"] == "tc" and sorted(pt) == want
    for k in want:
        assert per_harmonic(pt[k].cpu().numpy(), pd[k].cpu().numpy()) < TOL


def test_cumulative_vs_reference_fixture(gpu_lib):
    from mma_gb300 import hankel as H

    g = np.load(os.path.join(GOLDEN, "hankel_config3_slice.npz"))
    H.XUV_index.set_constant_index(complex(g["n_xuv"][0], g["n_xuv"][1]))
    target = H.FSources_provider(g["zgrid"], g["rgrid"], g["ogrid"], data_source="static", FSource=g["S"])
    gas = g["gas"].item().decode() if isinstance(g["gas"].item(), bytes) else str(g["gas"])
    h = H.Hankel_long(target, float(g["distance"]), g["rho"], preset_gas=gas, pressure=1.0,
                      near_field_factor=bool(g["near_field"]), store_cumulative_result=True, form="fast")
    assert h.fast_plan["planes_via"] == "tc"
    ref = g["cumulative"]
    for k in range(ref.shape[0]):
        assert per_harmonic(h.cumulative_field[k], ref[k]) < TOL, k
    assert per_harmonic(h.entry_plane_transform, g["entry"]) < TOL
    assert per_harmonic(h.exit_plane_transform, g["exit"]) < TOL
